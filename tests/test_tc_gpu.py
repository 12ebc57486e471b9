"""The tensor-core operator (precision "fp16-tc"): every 64-point DFT stage of the Λ
pass and of the inverse row pass is a tcgen05 MMA with fp16 operands, per-tile
power-of-two scales and float32 accumulation; the DFT-8 stages, twiddles, coil maps,
K x K kernel and coil sums run in float32, and the stack between the passes is float32.
The forward row pass is the float32 four-step kernel.

Four fp16 roundings of the operands (one per DFT-64) and the fp16 DFT matrix set the
error: relative L2 vs the float64 oracle of ``mul!`` (src/NFFTNormalOp.jl:227-267) a few
1e-4; the bound written here is the mixed-precision target, 1e-3.
"""
import numpy as np
import pytest
import torch

from oracle import cg as ocg
from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

TOL = 1e-3
pytestmark = pytest.mark.gpu


def _problem(seed, img, K, Nc, density=0.8, complex_lam=True):
    rng = np.random.default_rng(seed)
    G = tuple(2 * n for n in img)
    cells = np.flatnonzero(rng.random(int(np.prod(G))) < density) + 1
    P = K * (K + 1) // 2
    lam = rand_c(rng, (P, cells.size)) if complex_lam else rng.standard_normal((P, cells.size)).astype(np.float32)
    cm = rand_c(rng, img + (Nc,))
    x = rand_c(rng, img + (K,))
    return lam, cells, cm, x


@pytest.mark.parametrize("K,Nc,cplx", [(1, 2, True), (3, 2, False), (5, 3, False), (5, 2, True), (8, 2, True),
                                       (5, 20, False), (2, 5, True)])
def test_tc_apply_matches_oracle(mr, cuda, K, Nc, cplx):
    img = (256, 256)
    lam, cells, cm, x = _problem(20 + K, img, K, Nc, complex_lam=cplx)
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml, precision="fp16-tc")
    assert A.precision == 3
    y = mr.to_host(A @ x)
    ref = onormal.nfft_normalop_apply(x, onormal.unpack_lambda(lam.astype(np.complex128), K), cells, img, cmaps=cml)
    err = rel_l2(y, ref)
    y32 = mr.to_host(mr.NFFTNormalOp(img, lam, cells, cmaps=cml) @ x)
    print(f"fp16-tc apply K={K} Nc={Nc} cplx={cplx}: rel L2 {err:.2e} (float32 {rel_l2(y32, ref):.2e})")
    assert err < TOL


def test_tc_without_coil_maps(mr, cuda):
    img, K = (256, 256), 3
    lam, cells, _, x = _problem(41, img, K, 1)
    A = mr.NFFTNormalOp(img, lam, cells, precision="fp16-tc")
    ref = onormal.nfft_normalop_apply(x, onormal.unpack_lambda(lam.astype(np.complex128), K), cells, img)
    assert rel_l2(mr.to_host(A @ x), ref) < TOL


def test_tc_scale_invariant(mr, cuda):
    """Per-tile scales follow the data: tiny and huge inputs keep their accuracy, a zero
    coil map gives exact zeros."""
    img, K, Nc = (256, 256), 4, 3
    lam, cells, cm, x = _problem(31, img, K, Nc)
    cm[..., 1] = 0
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml, precision="fp16-tc")
    L64 = onormal.unpack_lambda(lam.astype(np.complex128), K)
    for s in (1e-20, 1e15):
        xs = (x * s).astype(np.complex64)
        y = mr.to_host(A @ xs)
        assert np.all(np.isfinite(y))
        assert rel_l2(y, onormal.nfft_normalop_apply(xs.astype(np.complex128), L64, cells, img, cmaps=cml)) < TOL


def test_tc_from_trajectory_and_cg(mr, cuda):
    """Operator from a radial trajectory (real basis, packed real kernel); cg(A, b; maxiter=20)
    against the float64 CG on the oracle operator."""
    rng = np.random.default_rng(5)
    N, K, Nt, Nc = 256, 4, 40, 2
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 8, Nt)
    U = np.linalg.svd(rng.standard_normal((Nt, K)), full_matrices=False)[0].astype(np.float32)
    cm = rand_c(rng, (N, N, Nc))
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp((N, N), trj, U, cmaps=cml, precision="fp16-tc")
    A32 = mr.NFFTNormalOp((N, N), A.Λ, A.kmask_indcs, cmaps=cml)
    b = rand_c(rng, (N, N, K))
    L64 = onormal.unpack_lambda(mr.to_host(A.Λ).astype(np.complex128), K)
    km = mr.to_host(A.kmask_indcs)
    assert rel_l2(mr.to_host(A @ b), onormal.nfft_normalop_apply(b, L64, km, (N, N), cmaps=cml)) < TOL
    bt = mr.to_jl(b, torch.complex64)
    x16 = mr.to_host(mr.cg(A, bt, maxiter=20, reltol=0.0)).ravel(order="F")
    x32 = mr.to_host(mr.cg(A32, bt, maxiter=20, reltol=0.0)).ravel(order="F")
    print(f"cg-20 fp16-tc vs float32: {rel_l2(x16, x32):.2e}")
    assert rel_l2(x16, x32) < 2e-3


def test_tc_rejects_other_grids(mr, cuda):
    lam, cells, cm, _ = _problem(8, (128, 128), 3, 1)
    with pytest.raises(NotImplementedError):
        mr.NFFTNormalOp((128, 128), lam, cells, cmaps=[cm[..., 0]], precision="fp16-tc")


def _radial_tc(seed=6, N=256, K=4, Nt=40, Nc=2):
    rng = np.random.default_rng(seed)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 8, Nt)
    U = np.linalg.svd(rng.standard_normal((Nt, K)), full_matrices=False)[0].astype(np.float32)
    cm = rand_c(rng, (N, N, Nc))
    return rng, trj, U, [cm[..., c] for c in range(Nc)]


def test_tc_refinement_reaches_float32_residual(mr, cuda):
    """Refinement with the tensor-core operator inside, float32 outer residual, on a
    well-determined problem (32 spokes x 20 frames, 8 coils, K=3).  The operator is shared
    from a float32 one whose Λ tiles are 8 columns wide (K=3)."""
    rng = np.random.default_rng(6)
    N, K, Nt, Nc = 256, 3, 20, 8
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 32, Nt)
    U = np.linalg.svd(rng.standard_normal((Nt, K)), full_matrices=False)[0].astype(np.float32)
    cm = rand_c(rng, (N, N, Nc))
    cml = [cm[..., c] for c in range(Nc)]
    A32 = mr.NFFTNormalOp((N, N), trj, U, cmaps=cml)
    At = A32.share(cmaps=cml, precision="fp16-tc")
    x_true = mr.to_jl(rand_c(rng, (N, N, K)), torch.complex64)
    assert rel_l2(mr.to_host(At @ x_true), mr.to_host(A32 @ x_true)) < TOL
    bt = A32 @ x_true
    res = mr.cg_refined(At, A32, bt, inner_iters=30, max_outer=20, tol=1e-4, log=True)
    print(f"fp16-tc refined: outer {res.iters}, residual {res.resnorm:.2e}")
    assert res.resnorm <= 1e-4


def test_tc_in_cg_batch_graph(mr, cuda):
    """The tensor-core passes inside a captured CUDA graph (the serving path): each branch
    equals cg on the same operator."""
    rng, trj, U, cml = _radial_tc(seed=7, K=3)
    N, K = 256, U.shape[1]
    base = mr.NFFTNormalOp((N, N), trj, U, cmaps=cml, precision="fp16-tc")
    ops = [base, base.share(cmaps=cml)]
    bs = [mr.to_jl(rand_c(rng, (N, N, K)), torch.complex64) for _ in ops]
    refs = [mr.to_host(mr.cg(A, b, maxiter=5, reltol=0.0)) for A, b in zip(ops, bs)]
    xs = [mr.jl_empty(b.shape, torch.complex64) for b in bs]
    batch = mr.CgBatch(ops, bs, xs, 5)
    batch.launch()
    torch.cuda.synchronize()
    for x, r in zip(xs, refs):
        assert rel_l2(mr.to_host(x), r) < 1e-6


def test_tc_3d_operator(mr, cuda):
    """3D: the tensor-core row and Λ passes (512-point lines along dims 1 and 3) around the
    float32 middle pass along dim 2."""
    img, K, Nc = (256, 8, 256), 3, 2
    lam, cells, cm, x = _problem(51, img, K, Nc, density=0.6, complex_lam=False)
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml, precision="fp16-tc")
    ref = onormal.nfft_normalop_apply(x, onormal.unpack_lambda(lam.astype(np.complex128), K), cells, img, cmaps=cml)
    err = rel_l2(mr.to_host(A @ x), ref)
    print(f"fp16-tc 3D apply: rel L2 {err:.2e}")
    assert err < TOL
