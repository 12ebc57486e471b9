"""CUDA NUFFT paths against the float64 oracle (exact non-uniform sums).

* forward model (type 2) vs the exact NUDFT forward of the reference tests
* calculate_backprojection (type 1 + coil combination, masks, density
  compensation) vs src/BackProjection.jl restated with exact sums
* NFFTNormalOp(img_shape, trj, U): kmask bit-exact and Toeplitz kernel Λ
  vs calculate_kernel_noncartesian with exact point-spread sums.
The ES kernel (w = 8, sigma = 2) approximates the exact sums to ~1e-7; the
float32 tolerance for every result here is 1e-5 relative L2.
"""
import numpy as np
import pytest
import torch

from oracle import backprojection as obp
from oracle import normalop as onormal
from oracle import nudft, trajectories as otraj
from tests.helpers import rand_c, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _setup(seed, N, d, Nr, Ncyc, Nt, K, Nc, cplx_u=True):
    rng = np.random.default_rng(seed)
    if d == 2:
        trj = otraj.traj_2d_radial_goldenratio(Nr, Ncyc, Nt)
    else:
        trj = otraj.traj_kooshball_goldenratio(Nr, Ncyc, Nt, thetaRot=0.3, phiRot=0.1).astype(np.float32)
    img = (N,) * d
    U = rand_c(rng, (Nt, K)) if cplx_u else rng.standard_normal((Nt, K)).astype(np.float32)
    U = np.linalg.svd(U, full_matrices=False)[0].astype(U.dtype)
    cm = rand_c(rng, img + (Nc,))
    x = rand_c(rng, img + (K,))
    return rng, trj, img, U, cm, x


def _oracle_forward(x, trj, U, cm):
    Ns, Nt = trj.shape[1:]
    K = x.shape[-1]
    pts = trj.reshape(trj.shape[0], -1, order="F").astype(np.float64)
    t_of = np.repeat(np.arange(Nt), Ns)
    out = np.zeros((Ns, Nt, cm.shape[-1]), dtype=np.complex128)
    for c in range(cm.shape[-1]):
        acc = np.zeros(Ns * Nt, dtype=np.complex128)
        for k in range(K):
            acc += U[t_of, k] * nudft.forward(cm[..., c] * x[..., k], pts)
        out[:, :, c] = acc.reshape(Ns, Nt, order="F")
    return out


@pytest.mark.parametrize("d,N,cplx", [(2, 16, True), (2, 24, False), (3, 8, True)])
def test_forward_model_matches_exact_nudft(mr, cuda, d, N, cplx):
    rng, trj, img, U, cm, x = _setup(0, N, d, 2 * N, 2, 5, 3, 2, cplx)
    y = mr.to_host(mr.forward_model(x, trj, U, cmaps=cm))
    ref = _oracle_forward(x, trj, U, cm)
    assert rel_l2(y, ref) < TOL


@pytest.mark.parametrize("d,N,cplx,dcf,masked,coilwise", [
    (2, 16, True, "none", False, False),
    (2, 16, False, "radial_2D", True, False),
    (2, 20, True, "none", True, True),
    (3, 8, True, "radial_3D", False, False),
    (3, 8, False, "none", True, True),
])
def test_backprojection_matches_oracle(mr, cuda, d, N, cplx, dcf, masked, coilwise):
    rng, trj, img, U, cm, x = _setup(1, N, d, 2 * N, 3, 4, 3, 3, cplx)
    data = rand_c(rng, trj.shape[1:] + (3,))
    mask = None
    if masked:
        mask = np.ones(trj.shape[1:], dtype=bool)
        mask[: 2 * N, 0] = False  # remove one spoke of the first frame (test/data_removal.jl:72-77)
    cml = [cm[..., c] for c in range(3)]
    arg = img if coilwise else cml
    b = mr.to_host(mr.calculate_backprojection(data, trj, arg, U=U, sample_mask=mask, density_compensation=dcf))
    ref = obp.calculate_backprojection(data, trj, cmaps=None if coilwise else cml, img_shape=img, U=U,
                                       sample_mask=mask, density_compensation=dcf)
    assert b.shape == ref.shape
    assert rel_l2(b, ref) < TOL


def test_backprojection_identity_basis_and_errors(mr, cuda):
    rng, trj, img, U, cm, x = _setup(2, 16, 2, 32, 2, 3, 3, 2)
    data = rand_c(rng, trj.shape[1:] + (2,))
    cml = [cm[..., c] for c in range(2)]
    b = mr.to_host(mr.calculate_backprojection(data, trj, cml))  # U = I(Nt)
    ref = obp.calculate_backprojection(data, trj, cmaps=cml)
    assert b.shape == (16, 16, 3) and rel_l2(b, ref) < TOL
    with pytest.raises(ValueError):  # test_dimension: coil count mismatch
        mr.calculate_backprojection(data, trj, cml[:1], U=U)
    with pytest.raises(ValueError):
        mr.calculate_backprojection(data, trj, cml, U=U, density_compensation="bogus")
    with pytest.raises(AssertionError):
        mr.calculate_backprojection(data, trj, cml, U=U, sample_mask=np.zeros(trj.shape[1:], dtype=bool))


@pytest.mark.parametrize("d,N,cplx,masked", [(2, 16, True, False), (2, 16, False, True), (2, 24, True, True),
                                             (3, 8, False, False)])
def test_nfft_normalop_kernel_matches_oracle(mr, cuda, d, N, cplx, masked):
    rng, trj, img, U, cm, x = _setup(3, N, d, 2 * N, 3, 6, 3, 2, cplx)
    mask = None
    if masked:
        mask = np.ones(trj.shape[1:], dtype=bool)
        mask[5:2 * N, 1] = False
    cml = [cm[..., c] for c in range(2)]
    A = mr.NFFTNormalOp(img, trj, U, cmaps=cml, sample_mask=mask)
    G = tuple(2 * n for n in img)
    Lam_o, km_o = onormal.calculate_kernel_noncartesian(G, trj, U, sample_mask=mask)
    np.testing.assert_array_equal(mr.to_host(A.kmask_indcs), km_o)
    Lp = mr.to_host(A.Λ)
    assert np.iscomplexobj(Lp) == cplx  # isreal(A.prod!.A.Λ) for a real basis (test/reconstruct_radial_gpu_real.jl)
    Lp_o = onormal.pack_lambda(Lam_o, real=not cplx)
    assert rel_l2(Lp, Lp_o) < TOL
    y = mr.to_host(A @ x)
    ref = onormal.nfft_normalop_apply(x, Lam_o, km_o, img, cmaps=cml)
    assert rel_l2(y, ref) < TOL


def test_nfft_normalop_rejects_empty_mask_and_odd_grids(mr, cuda):
    rng, trj, img, U, cm, x = _setup(4, 16, 2, 32, 2, 3, 2, 1)
    with pytest.raises(AssertionError):
        mr.NFFTNormalOp(img, trj, U, sample_mask=np.zeros(trj.shape[1:], dtype=bool))
    with pytest.raises(AssertionError):
        mr.NFFTNormalOp((7, 16), trj, U)  # 14 is not 2,3,5-smooth
