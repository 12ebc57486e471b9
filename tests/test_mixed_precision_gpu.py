"""Reduced-precision reconstructions against the float64 oracle.

The reference reconstructs with cg(A, b; maxiter) from x0 = 0
(test/reconstruct_radial.jl:83, 20 iterations).  On the kmask-truncated Toeplitz
operator (src/NFFTNormalOp.jl:227-267) that iteration count is what defines the image:
CG does not converge to a unique solution at float32 or float64 (the residual stalls
near 1e-4 and iterates hundreds of steps apart differ by ~10%), so the float64 oracle
here is the same 20-iteration CG in float64 on the same right-hand side.

A reduced-precision operator (apply error a few 1e-4) moves a plain 20-iteration CG
iterate by ~1e-2: CG amplifies product errors, most of all those taken while the
residual is large.  ``cg_relaxed`` takes the products on the float32 operator until
||r|| <= 0.05 ||b|| and on the reduced-precision operator after that, on one recurrence;
its image is within 1e-3 of the float64 CG image.  Checked here with the tensor-core
operator (fp16-tc, 256^2), the fp16-storage operator at the 64^2, 4-coil, K = 4
configuration's exact shape, and the fp16-storage operator on a 3D koosh-ball problem
(32^3; the 128^3 configuration's operator is the same code on longer lines, and its
float64 CG is out of reach of the CPU oracle in a test).
"""
import numpy as np
import pytest
import torch

from oracle import cg as ocg
from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-4     # float32 CG-20 vs float64 CG-20
TOL_MIXED = 1e-3    # reduced-precision reconstruction vs float64 (the mixed-precision bar)


def _problem(mr, img, Nr, Nt, K, Nc, lo_precision):
    if len(img) == 2:
        trj = otraj.traj_2d_radial_goldenratio(Nr, 1, Nt)
    else:  # 16 spokes per frame: 2400 spokes for 32^3 (with 2 coils or 600 spokes even the
        # float32 CG-20 is 3e-4 .. 6e-4 from the float64 one: too ill-conditioned to measure)
        trj = otraj.traj_kooshball_goldenratio(Nr, 16, Nt).astype(np.float32)
    D = mr.synthetic.dictionary(Nt)
    U = mr.synthetic.basis(D, K)
    x = mr.synthetic.phantom(img, D, U)
    cm = mr.synthetic.coil_maps(img, Nc)
    cmd = mr.to_jl(cm, torch.complex64)
    data = mr.synthetic.add_noise(mr.forward_model(mr.to_jl(x, torch.complex64), trj, U, cmaps=cmd), 0.01)
    A32 = mr.NFFTNormalOp(img, trj, U, cmaps=cm)
    Alo = A32.share(cmaps=cm, precision=lo_precision)
    b = mr.calculate_backprojection(data, trj, cm, U=U)
    return trj, U, cm, A32, Alo, b


def _oracle_cg(img, trj, U, cm, b, iters):
    G = tuple(2 * n for n in img)
    Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U, fast=True)
    K = U.shape[1]
    cml = [cm[..., c] for c in range(cm.shape[-1])]

    def apply(v):
        return onormal.nfft_normalop_apply(v.reshape(img + (K,), order="F"), Lam, km, img, cmaps=cml).ravel(order="F")

    x, _, _ = ocg.cg(apply, b.ravel(order="F"), maxiter=iters, reltol=0.0)
    return x.reshape(img + (K,), order="F")


# switch: the relative residual below which products go to the reduced operator.  The 3D
# koosh ball is worse conditioned (CG-20 amplifies an apply error more), so its products
# stay float32 a little longer (0.05: 7e-4 .. 8e-4 from float64; 0.02: ~1e-4).
@pytest.mark.parametrize("img,Nr,Nt,K,Nc,lo,switch", [
    ((256, 256), 512, 200, 4, 4, "fp16-tc", 0.05),
    ((64, 64), 128, 200, 4, 4, "fp16", 0.05),
    ((32, 32, 32), 64, 150, 3, 4, "fp16", 0.02),
])
def test_relaxed_mixed_precision_cg_matches_float64(mr, cuda, img, Nr, Nt, K, Nc, lo, switch):
    trj, U, cm, A32, Alo, b = _problem(mr, img, Nr, Nt, K, Nc, lo)
    x64 = _oracle_cg(img, trj, U, cm, mr.to_host(b).astype(np.complex128), 20)
    x32 = mr.to_host(mr.cg(A32, b, maxiter=20, reltol=0.0))
    xlo = mr.to_host(mr.cg(Alo, b, maxiter=20, reltol=0.0))
    rel = mr.cg_relaxed(Alo, A32, b, maxiter=20, reltol=0.0, switch=switch, log=True)
    e32, elo, erel = rel_l2(x32, x64), rel_l2(xlo, x64), rel_l2(mr.to_host(rel.x), x64)
    print(f"{img} {lo}: cg-20 vs float64: float32 {e32:.2e}, {lo} {elo:.2e}, relaxed {erel:.2e} "
          f"({rel.hi_iters} of {rel.iters} products float32)")
    assert rel.iters == 20 and 0 < rel.hi_iters < 20
    assert e32 < TOL_FP32
    assert erel < TOL_MIXED


def test_relaxed_switch_extremes_are_the_plain_solves(mr, cuda):
    """switch = 0 runs every product on the float32 operator (= cg on it), switch >= 1 every
    product on the reduced-precision one; a tolerance stops the solve as cg does."""
    trj, U, cm, A32, Alo, b = _problem(mr, (64, 64), 128, 60, 3, 2, "fp16")
    x32 = mr.to_host(mr.cg(A32, b, maxiter=12, reltol=0.0))
    xlo = mr.to_host(mr.cg(Alo, b, maxiter=12, reltol=0.0))
    r0 = mr.cg_relaxed(Alo, A32, b, maxiter=12, reltol=0.0, switch=0.0, log=True)
    r1 = mr.cg_relaxed(Alo, A32, b, maxiter=12, reltol=0.0, switch=1.0, log=True)
    assert r0.hi_iters == 12 and r1.hi_iters == 0
    assert rel_l2(mr.to_host(r0.x), x32) < 1e-6
    assert rel_l2(mr.to_host(r1.x), xlo) < 1e-6
    t = mr.cg(A32, b, maxiter=200, reltol=1e-2, log=True)
    rt = mr.cg_relaxed(Alo, A32, b, maxiter=200, reltol=1e-2, switch=0.05, log=True)
    assert rt.iters < 200 and abs(rt.iters - t.iters) <= 2
    with pytest.raises(ValueError):
        mr.cg_relaxed(A32, A32, b, maxiter=5)
