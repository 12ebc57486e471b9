"""Mixed-precision (fp16-storage) normal operator and the refinement solver.

``precision="fp16"`` keeps the oversampled K-stack and the Toeplitz kernel in
half precision with one float32 scale per tile; every FFT butterfly, the K x K
product and the coil sums run in float32.  Half precision carries 11
significant bits (unit roundoff 2^-11 = 4.9e-4), so one apply agrees with the
float64 oracle of ``mul!`` (src/NFFTNormalOp.jl:227-267) to a relative L2
error of a few 1e-4; the bound written here is 2e-3.  A fixed-iteration CG
solve (the reference's ``cg(A, b, maxiter=20)``, test/reconstruct_radial.jl:83)
on the fp16 operator stays within 1e-3 of the same solve in float64, and the
refinement loop (fp16 inner CG, float32 residuals) reaches residuals below
what fp16 alone can.
"""
import numpy as np
import pytest
import torch

from oracle import cg as ocg
from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

TOL_APPLY = 2e-3
TOL_CG = 1e-3
pytestmark = pytest.mark.gpu


def _problem(seed, img, K, Nc, density=0.8, complex_lam=True, xscale=1.0):
    rng = np.random.default_rng(seed)
    G = tuple(2 * n for n in img)
    cells = np.flatnonzero(rng.random(int(np.prod(G))) < density) + 1
    P = K * (K + 1) // 2
    lam = rand_c(rng, (P, cells.size)) if complex_lam else rng.standard_normal((P, cells.size)).astype(np.float32)
    cm = rand_c(rng, img + (Nc,)) if Nc else None
    x = (rand_c(rng, img + (K,)) * xscale).astype(np.complex64)
    return lam, cells, cm, x


@pytest.mark.parametrize("img,K,Nc,cplx", [
    ((32, 32), 3, 2, True),       # 64 = 8 x 8
    ((64, 64), 5, 4, False),      # 128 = 8 x 16
    ((128, 128), 4, 3, True),     # 256 = 16 x 16
    ((256, 64), 4, 2, False),     # 512 = 16 x 32 and 128
    ((192, 192), 3, 2, True),     # 384 = 12 x 32
    ((32, 32), 1, 0, True),       # one basis function, cmaps=(1,)
    ((64, 64), 8, 2, True),       # largest K of the register product
    ((32, 32, 32), 5, 2, False),  # 3D: 64^3
    ((32, 64, 32), 3, 2, True),   # 3D mixed 64 / 128
])
def test_half_apply_matches_oracle(mr, cuda, img, K, Nc, cplx):
    lam, cells, cm, x = _problem(5, img, K, Nc, complex_lam=cplx)
    cml = None if cm is None else [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml, precision="fp16")
    assert A.precision == 1
    y = mr.to_host(A @ x)
    ref = onormal.nfft_normalop_apply(x, onormal.unpack_lambda(lam.astype(np.complex128), K), cells, img, cmaps=cml)
    err = rel_l2(y, ref)
    print(f"fp16 apply {img} K={K} Nc={Nc}: rel L2 {err:.2e}")
    assert err < TOL_APPLY


@pytest.mark.parametrize("xscale", [1e-12, 1e9])
def test_half_apply_scale_invariant(mr, cuda, xscale):
    """Per-tile scales follow the data: inputs far outside fp16's range keep their accuracy,
    and a coil whose map is zero (every tile maximum 0) yields exact zeros, not NaNs."""
    img, K, Nc = (64, 64), 4, 3
    lam, cells, cm, x = _problem(6, img, K, Nc, xscale=xscale)
    cm[..., 1] = 0
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml, precision="fp16")
    y = mr.to_host(A @ x)
    assert np.all(np.isfinite(y))
    ref = onormal.nfft_normalop_apply(x.astype(np.complex128), onormal.unpack_lambda(lam.astype(np.complex128), K),
                                      cells, img, cmaps=cml)
    assert rel_l2(y, ref) < TOL_APPLY


def test_half_fft_normalop(mr, cuda):
    """The Cartesian operator (src/FFTNormalOp.jl:111-149) in fp16 storage."""
    rng = np.random.default_rng(7)
    img, K, Nt, Nc = (64, 64), 4, 12, 2
    M = (rng.random(img + (Nt,)) < 0.3)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    cm = rand_c(rng, img + (Nc,))
    cml = [cm[..., c] for c in range(Nc)]
    A16 = mr.FFTNormalOp(M, U, cmaps=cml, precision="fp16")
    A32 = mr.FFTNormalOp(M, U, cmaps=cml)
    x = rand_c(rng, img + (K,))
    y16 = mr.to_host(A16 @ x)
    y32 = mr.to_host(A32 @ x)
    assert rel_l2(y16, y32) < TOL_APPLY


def test_half_rejects_generic_lengths(mr, cuda):
    lam, cells, cm, _ = _problem(8, (24, 40), 3, 1)
    with pytest.raises(NotImplementedError):
        mr.NFFTNormalOp((24, 40), lam, cells, cmaps=[cm[..., 0]], precision="fp16")


def _radial_problem(N=32, K=4, Nc=3, Ncyc=4, Nt=20, seed=9):
    rng = np.random.default_rng(seed)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, Ncyc, Nt)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    cm = rand_c(rng, (N, N, Nc))
    Lam, km = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    b = rand_c(rng, (N, N, K))
    return Lam, km, [cm[..., c] for c in range(Nc)], b


def test_half_cg_fixed_iterations_vs_float64(mr, cuda):
    """cg(A, b, maxiter=20) on the fp16 operator against the same 20 iterations in float64."""
    N, K = 32, 4
    Lam, km, cml, b = _radial_problem(N=N, K=K)
    packed = onormal.pack_lambda(Lam).astype(np.complex64)
    A16 = mr.NFFTNormalOp((N, N), packed, km, cmaps=cml, precision="fp16")
    A32 = mr.NFFTNormalOp((N, N), packed, km, cmaps=cml)
    Lam64 = onormal.unpack_lambda(packed.astype(np.complex128), K)

    def apply64(v):
        return onormal.nfft_normalop_apply(v.reshape((N, N, K), order="F"), Lam64, km, (N, N), cmaps=cml).ravel(order="F")

    x64, _, _ = ocg.cg(apply64, b.ravel(order="F"), maxiter=20, reltol=0.0)
    bt = mr.to_jl(b, torch.complex64)
    x16 = mr.to_host(mr.cg(A16, bt, maxiter=20, reltol=0.0)).ravel(order="F")
    x32 = mr.to_host(mr.cg(A32, bt, maxiter=20, reltol=0.0)).ravel(order="F")
    e16, e32 = rel_l2(x16, x64), rel_l2(x32, x64)
    print(f"cg-20 vs float64: fp16 {e16:.2e}, fp32 {e32:.2e}")
    assert e32 < 1e-4
    assert e16 < TOL_CG


def test_cg_refined_reaches_float32_residual(mr, cuda):
    """Refinement: fp16 inner CG, residual b - A x in float32, stops at ||r|| <= tol ||b||."""
    N, K = 32, 4
    Lam, km, cml, b = _radial_problem(N=N, K=K, Ncyc=8)
    packed = onormal.pack_lambda(Lam).astype(np.complex64)
    A16 = mr.NFFTNormalOp((N, N), packed, km, cmaps=cml, precision="fp16")
    A32 = mr.NFFTNormalOp((N, N), packed, km, cmaps=cml)
    # a right-hand side in the well-resolved range of the operator: b = A x_true
    x_true = mr.to_jl(b, torch.complex64)
    bt = A32 @ x_true
    tol = 1e-4
    res = mr.cg_refined(A16, A32, bt, inner_iters=30, max_outer=20, tol=tol, log=True)
    Lam64 = onormal.unpack_lambda(packed.astype(np.complex128), K)
    x = mr.to_host(res.x).astype(np.complex128)
    r = mr.to_host(bt).astype(np.complex128) - onormal.nfft_normalop_apply(x, Lam64, km, (N, N), cmaps=cml)
    rel = np.linalg.norm(r) / np.linalg.norm(mr.to_host(bt))
    print(f"cg_refined: outer {res.iters}, reported {res.resnorm:.2e}, float64 check {rel:.2e}")
    assert res.resnorm <= tol
    assert rel < 2 * tol
