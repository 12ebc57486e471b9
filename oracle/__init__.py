"""CPU oracle for the subspace normal-operator path of MRISubspaceRecon.jl.

TEST INFRASTRUCTURE ONLY.  This package is the checker: a float64 CPU
restatement of the reference algorithm, written with NumPy/SciPy (and one
small C file for the bit-exact GROG grid indices).  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product (the CUDA library and its
Python mirror) never imports, links or calls anything in here.

Modules and the reference code they restate (paths inside the reference
project):

* ``trajectories`` -- ``src/Trajectories.jl:81-173``
* ``nudft``        -- exact non-uniform DFTs used as the forward model of the
  reference tests (``test/reconstruct_radial.jl:62-74``) and as the exact
  replacement of the NonuniformFFTs.jl type-1 transform, plus a float64
  spreading type-1 NUFFT (~1e-7) for benchmark-sized trajectories
* ``normalop``     -- ``src/NFFTNormalOp.jl:106-267`` (kmask, Toeplitz kernel
  for complex and real bases, apply) and ``src/FFTNormalOp.jl:81-149``
* ``backprojection`` -- ``src/BackProjection.jl:23-203``
* ``grog``         -- ``src/GROG.jl:14-102``
* ``cg``           -- IterativeSolvers.jl 0.9 ``cg`` as called from the
  reference tests (``test/reconstruct_radial.jl:83``)
* ``cpu_apply``    -- float32 structure-faithful restatement of the CPU apply
  ``src/NFFTNormalOp.jl:227-267`` used only as the timed CPU baseline

Parity pinning: the reference is Julia and cannot run in this build
environment, and none of its tests hold element-wise golden vectors for this
path.  The oracle is pinned against the known-answer and invariance tests of
the reference test suite, re-expressed on seeded synthetic inputs in
``tests/test_oracle_pins.py`` (Cartesian backprojection reproduces the
phantom, Hermitian kernel blocks, GROG repeat invariance and spoke shift,
recon-vs-truth tolerances).  The NonuniformFFTs.jl kernel and its kmask
footprint are third-party code absent from the reference tree; the oracle
uses the exact sums they approximate, so Toeplitz-kernel parity against the
reference itself is unpinned at that boundary.
"""
