"""CG and the Cartesian (FFTNormalOp / integer-trajectory) paths against the oracle."""
import numpy as np
import pytest
import torch

from oracle import backprojection as obp
from oracle import normalop as onormal
from oracle import trajectories as otraj
from oracle.cg import cg as ocg
from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


def _cart_problem(seed, N, Nt, K, Nc, density=0.3, nrep=1, cplx=True):
    rng = np.random.default_rng(seed)
    img = (N, N)
    trj = otraj.traj_cartesian(N, N, 1, Nt, T=np.int32)[:2]
    mask = rng.random(trj.shape[1:]) < density
    U = rand_c(rng, (Nt, K)) if cplx else rng.standard_normal((Nt, K)).astype(np.float32)
    U = np.linalg.svd(U, full_matrices=False)[0].astype(U.dtype)
    if nrep > 1:
        U = np.repeat(U[:, :, None], nrep, axis=2)
    cm = rand_c(rng, img + (Nc,))
    return rng, img, trj, mask, U, cm


@pytest.mark.parametrize("N,cplx,nrep", [(16, True, 1), (24, False, 1), (16, True, 3)])
def test_fft_normalop_from_trajectory(mr, cuda, N, cplx, nrep):
    rng, img, trj, mask, U, cm = _cart_problem(0, N, 6, 3, 2, cplx=cplx, nrep=nrep)
    cml = [cm[..., c] for c in range(2)]
    A = mr.FFTNormalOp(img, trj, U, cmaps=cml, sample_mask=mask)
    lam_full = onormal.calculate_kernel_cartesian(img, trj, U, sample_mask=mask)
    lam_c, km, _ = onormal.fft_normalop_from_lambda(lam_full)
    np.testing.assert_array_equal(mr.to_host(A.kmask_indcs), km)
    L = mr.to_host(A.Λ)
    assert rel_l2(L, lam_c) < 1e-6
    # every K x K block Hermitian (test/reconstruct_cart_trj.jl:68-73)
    assert np.abs(L - np.conj(np.transpose(L, (1, 0, 2)))).max() <= 1e-6 * np.abs(L).max()
    x = rand_c(rng, img + (3,))
    assert rel_l2(mr.to_host(A @ x), onormal.fft_normalop_apply(x, lam_c, km, img, cmaps=cml)) < 1e-5


def test_fft_normalop_from_mask(mr, cuda):
    rng = np.random.default_rng(1)
    N, Nt, K = 16, 8, 3
    M = rng.random((N, N, Nt)) < 0.2
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    cm = rand_c(rng, (N, N, 2))
    A = mr.FFTNormalOp(M, U, cmaps=[cm[..., 0], cm[..., 1]])
    lam_c, km, _ = onormal.fft_normalop_from_lambda(onormal.calculate_kernel_cartesian_mask(M, U))
    np.testing.assert_array_equal(mr.to_host(A.kmask_indcs), km)
    assert rel_l2(mr.to_host(A.Λ), lam_c) < 1e-6


@pytest.mark.parametrize("coilwise,nrep", [(False, 1), (True, 1), (False, 2)])
def test_cartesian_backprojection(mr, cuda, coilwise, nrep):
    rng, img, trj, mask, U, cm = _cart_problem(2, 16, 5, 3, 3, nrep=nrep)
    data = rand_c(rng, trj.shape[1:] + (3,) + ((nrep,) if nrep > 1 else ()))
    cml = [cm[..., c] for c in range(3)]
    b = mr.to_host(mr.calculate_backprojection(data, trj, img if coilwise else cml, U=U, sample_mask=mask))
    ref = obp.calculate_backprojection_cartesian(data, trj, cmaps=None if coilwise else cml, img_shape=img, U=U,
                                                 sample_mask=mask)
    assert rel_l2(b, ref) < 1e-5


def test_cartesian_backprojection_known_answer(mr, cuda):
    """test/backprojection_cart.jl: a fully sampled Cartesian trajectory backprojects to the phantom."""
    N, Nc = 32, 4
    rng = np.random.default_rng(3)
    x = np.zeros((N, N))
    x[8:24, 10:20] = 1.0
    x[12:16, 4:28] += 0.5
    cm = rand_c(rng, (N, N, Nc)).astype(np.complex128)
    cm /= np.sqrt(np.sum(np.abs(cm) ** 2, axis=2, keepdims=True))
    # data = centred DFT of each coil image on the Cartesian grid (exact forward model)
    trj_f = otraj.traj_cartesian(N, N, 1, 1, T=np.float64)[:2]
    from oracle import nudft
    data = np.stack([nudft.forward(cm[..., c] * x, trj_f[:, :, 0]) for c in range(Nc)], axis=1)[:, None, :]
    trj_i = otraj.traj_cartesian(N, N, 1, 1, T=np.int32)[:2]
    U = np.ones((1, 1), dtype=np.complex64)
    reco = mr.to_host(mr.calculate_backprojection(data.astype(np.complex64), trj_i,
                                                  [cm[..., c].astype(np.complex64) for c in range(Nc)], U=U))[..., 0]
    assert np.abs(reco - x).max() < 4e-5  # atol of test/backprojection_cart.jl:66


@pytest.mark.parametrize("maxiter", [1, 5, 20])
def test_cg_matches_oracle_iterations(mr, cuda, maxiter):
    rng = np.random.default_rng(4)
    N, K, Nc = 16, 3, 2
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 4, 12)
    U = np.linalg.svd(rand_c(rng, (12, K)), full_matrices=False)[0].astype(np.complex64)
    cm = rand_c(rng, (N, N, Nc))
    cml = [cm[..., c] for c in range(Nc)]
    Lam, km = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    A = mr.NFFTNormalOp((N, N), onormal.pack_lambda(Lam).astype(np.complex64), km, cmaps=cml)
    b = rand_c(rng, (N, N, K))
    res = mr.cg(A, b, maxiter=maxiter, reltol=0.0, log=True)
    xo, it, hist = ocg(lambda v: onormal.nfft_normalop_apply(v, Lam, km, (N, N), cmaps=cml).ravel(order="F"),
                       b, maxiter=maxiter, reltol=0.0)
    assert res.iters == it == maxiter
    assert rel_l2(mr.to_host(res.x).ravel(order="F"), xo) < 1e-4
    assert abs(res.resnorm - hist[-1]) / hist[0] < 1e-4


def test_cg_default_tolerance_stops_early(mr, cuda):
    """reltol = sqrt(eps(Float32)) stops once |r| <= reltol |b| (IterativeSolvers default)."""
    rng = np.random.default_rng(5)
    N, K = 8, 2
    lamf = np.zeros((K, K, N, N), dtype=np.complex64)
    lamf[0, 0] = lamf[1, 1] = 2.0  # A = 2 I: CG converges in one iteration
    A = mr.FFTNormalOp(lamf)
    b = rand_c(rng, (N, N, K))
    res = mr.cg(A, b, maxiter=50, log=True)
    assert res.iters == 1
    assert rel_l2(mr.to_host(res.x), b / 2) < 1e-6
