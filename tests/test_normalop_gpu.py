"""Parity of the CUDA Toeplitz normal operator against the float64 oracle.

Given the same kernel Λ and kmask, the float32 operator must agree with the
oracle's restatement of ``mul!`` (src/NFFTNormalOp.jl:227-267,
src/FFTNormalOp.jl:111-149) to a relative L2 error of 1e-5.
"""
import numpy as np
import pytest
import torch

from oracle import normalop as onormal
from tests.helpers import rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _rand_c(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _problem(seed, img, K, Nc, density=0.8, complex_lam=True):
    rng = np.random.default_rng(seed)
    G = tuple(2 * n for n in img)
    ng = int(np.prod(G))
    cells = np.flatnonzero(rng.random(ng) < density) + 1
    P = K * (K + 1) // 2
    if complex_lam:
        lam = _rand_c(rng, (P, cells.size))
    else:
        lam = rng.standard_normal((P, cells.size)).astype(np.float32)
    cm = _rand_c(rng, img + (Nc,)) if Nc else None
    x = _rand_c(rng, img + (K,))
    return lam, cells, cm, x


@pytest.mark.parametrize("img,K,Nc,cplx", [
    ((16, 16), 3, 2, True),
    ((32, 32), 5, 4, False),
    ((24, 40), 4, 3, True),      # 2,3,5-smooth, non-square
    ((30, 20), 2, 1, False),     # radix 3 and 5
    ((64, 64), 6, 5, True),
    ((16, 16), 1, 0, True),      # cmaps=(1,)
    ((8, 12, 16), 3, 2, True),   # 3D
    ((16, 16, 8), 4, 3, False),  # 3D real kernel
    ((128, 128), 5, 3, False),   # four-step kernels: 256 = 16 x 16
    ((256, 64), 4, 2, True),     # 512 = 16 x 32 and 128 = 8 x 16
    ((192, 96), 3, 2, True),     # 384 = 12 x 32 and 192 (generic)
    ((32, 32, 32), 5, 2, False), # 3D four-step: 64 = 8 x 8
    ((32, 64, 32), 3, 2, True),  # 3D mixed: 64 / 128
    ((256, 256), 5, 3, False),   # K = 5 on 512-point columns (the benchmark's Λ pass)
    ((128, 256), 5, 2, True),    # the same with a complex kernel
    ((64, 128), 3, 2, True),     # three-step Λ pass at 256 points (4 x 8 x 8), 8-column tiles
    ((10, 128), 4, 2, True),     # the same with 4-column tiles (plane width 20)
    ((64, 256), 2, 2, False),    # 512 points with 8-column tiles (K = 2)
    ((96, 128), 6, 2, False),    # K = 6, the largest the three-step kernel takes
    ((16, 16, 128), 3, 2, True), # 3D with a 256-point last axis
    ((256, 24), 3, 20, True),    # three-step row passes at 512 points, 20 coils (five groups of 4)
    ((128, 10), 4, 13, False),   # 256-point rows, 13 coils (a partial group), 10 rows (a partial row block)
    ((128, 64), 2, 0, True),     # 256-point rows without coil maps
    ((128, 12, 8), 2, 3, True),  # 3D with 256-point rows
    ((32, 256), 6, 2, False),    # K = 6 on 512-point columns (4-column tiles, one CTA per SM)
    ((16, 256), 1, 3, True),     # K = 1 on 512-point columns (8-column tiles)
    ((256, 256), 3, 40, False),  # two coil groups of 20 (the stack of one group kept L2-sized)
])
def test_nfft_apply_matches_oracle(mr, cuda, img, K, Nc, cplx):
    lam, cells, cm, x = _problem(1, img, K, Nc, complex_lam=cplx)
    cml = None if cm is None else [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml)
    y = mr.to_host(A @ x)
    full = onormal.unpack_lambda(lam.astype(np.complex128), K)
    ref = onormal.nfft_normalop_apply(x, full, cells, img, cmaps=cml)
    assert rel_l2(y, ref) < TOL


def test_alpha_beta_semantics(mr, cuda):
    img, K, Nc = (16, 16), 3, 2
    lam, cells, cm, x = _problem(2, img, K, Nc)
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml)
    rng = np.random.default_rng(3)
    y0 = _rand_c(rng, img + (K,))
    full = onormal.unpack_lambda(lam.astype(np.complex128), K)
    alpha, beta = 0.5 - 0.25j, 1.5 + 0.5j
    yt = mr.to_jl(y0, torch.complex64)
    A.mul(yt, mr.to_jl(x, torch.complex64), alpha, beta)
    ref = onormal.nfft_normalop_apply(x, full, cells, img, cmaps=cml, alpha=alpha, beta=beta, xout=y0)
    assert rel_l2(mr.to_host(yt), ref) < TOL
    # beta == 0 overwrites NaNs (src/NFFTNormalOp.jl:232-236)
    yn = mr.to_jl(np.full(img + (K,), np.nan, dtype=np.complex64), torch.complex64)
    A.mul(yn, mr.to_jl(x, torch.complex64), 1.0, 0.0)
    assert np.all(np.isfinite(mr.to_host(yn)))


def test_vec_interface_and_lambda_roundtrip(mr, cuda):
    img, K, Nc = (20, 20), 4, 3
    lam, cells, cm, x = _problem(4, img, K, Nc)
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=[cm[..., c] for c in range(Nc)])
    assert A.shape == (20 * 20 * K, 20 * 20 * K)
    xv = torch.from_numpy(x.ravel(order="F")).cuda()
    yv = A @ xv
    assert yv.shape == (20 * 20 * K,)
    y = (A @ x)
    assert np.allclose(mr.to_host(yv), mr.to_host(y).ravel(order="F"))
    # A.prod.A.Λ / kmask_indcs hand back the reference's packed layout
    np.testing.assert_array_equal(mr.to_host(A.prod.A.kmask_indcs), cells)
    np.testing.assert_array_equal(mr.to_host(A.prod.A.Λ), lam)


def test_kmask_out_of_range_raises(mr, cuda):
    img = (8, 8)
    lam = np.ones((3, 2), dtype=np.complex64)
    with pytest.raises(AssertionError):
        mr.NFFTNormalOp(img, lam, np.array([1, 16 * 16 + 1]))
    with pytest.raises(AssertionError):
        mr.NFFTNormalOp(img, lam, np.array([0, 5]))


def test_hermitian_operator(mr, cuda):
    """<y, A x> == <A y, x> for the Hermitian packed kernel (LinearOperator hermitian=true)."""
    img, K, Nc = (16, 24), 3, 2
    lam, cells, cm, x = _problem(5, img, K, Nc)
    rng = np.random.default_rng(6)
    # make the diagonal blocks real so Λ(f) is Hermitian at every voxel
    for k in range(K):
        lam[onormal.packed_index(k, k)] = lam[onormal.packed_index(k, k)].real
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=[cm[..., c] for c in range(Nc)])
    y = _rand_c(rng, img + (K,))
    lhs = np.vdot(y, mr.to_host(A @ x))
    rhs = np.vdot(mr.to_host(A @ y), x)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


@pytest.mark.parametrize("img,K,Nc", [((16, 16), 3, 2), ((30, 24), 4, 3), ((8, 8, 12), 2, 2)])
def test_fft_normalop_from_full_lambda(mr, cuda, img, K, Nc):
    rng = np.random.default_rng(7)
    lamf = _rand_c(rng, (K, K) + img)
    lamf[:, :, rng.random(img) < 0.3] = 0  # kmask = Λ[1,1,:] .!= 0
    cm = _rand_c(rng, img + (Nc,))
    x = _rand_c(rng, img + (K,))
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.FFTNormalOp(lamf, cmaps=cml)
    y = mr.to_host(A @ x)
    lam_c, kmask, shp = onormal.fft_normalop_from_lambda(lamf)
    ref = onormal.fft_normalop_apply(x, lam_c, kmask, shp, cmaps=cml)
    assert rel_l2(y, ref) < TOL
    np.testing.assert_array_equal(mr.to_host(A.kmask_indcs), kmask)
    np.testing.assert_array_equal(mr.to_host(A.Λ), lam_c.astype(np.complex64))
