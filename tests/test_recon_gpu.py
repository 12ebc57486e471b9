"""End-to-end subspace reconstructions, in the shape of the reference's own integration tests.

Each test builds a seeded coefficient phantom, coil maps, a golden-angle radial
trajectory and a basis; synthesises k-space data; and reconstructs with
backprojection, NFFTNormalOp and cg(A, b; maxiter=20), the way
test/reconstruct_radial.jl:62-96 and its siblings do. Two checks follow:
* against the float64 oracle reconstruction on the same data, within 1e-2
  (the reference's CPU-vs-GPU tolerance, test/reconstruct_radial_gpu.jl:103);
* against the phantom cropped to the sampled k-space disk, within 1e-1
  (test/reconstruct_radial.jl:96).
The oracle uses exact non-uniform sums; the GPU path uses its ES-kernel NUFFT.
"""
import numpy as np
import pytest
import torch

from oracle import backprojection as obp
from oracle import cg as ocg
from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


def _phantom(rng, img, K):
    """Piecewise-constant complex coefficient images: random ellipses with random values per coefficient."""
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in img], indexing="ij")
    x = np.zeros(img + (K,), dtype=np.complex128)
    for _ in range(6):
        c = rng.uniform(-0.4, 0.4, len(img))
        ax = rng.uniform(0.15, 0.45, len(img))
        m = sum(((g - ci) / ai) ** 2 for g, ci, ai in zip(grids, c, ax)) <= 1.0
        x[m] += rand_c(rng, (K,)).astype(np.complex128)
    return x.astype(np.complex64)


def _coil_maps(img, Nc):
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in img], indexing="ij")
    maps = np.empty(img + (Nc,), dtype=np.complex128)
    for c in range(Nc):
        a = 2 * np.pi * c / Nc
        mag = np.exp(-((grids[0] - 1.2 * np.cos(a)) ** 2 + (grids[1] - 1.2 * np.sin(a)) ** 2) / (2 * 0.9 ** 2))
        maps[..., c] = mag * np.exp(1j * np.pi * (0.3 * c * grids[0] - 0.2 * grids[1]))
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=-1, keepdims=True))
    return maps.astype(np.complex64)


def _disk_crop(x):
    """x with its k-space support limited to the disk |k| <= N/2 that radial spokes sample."""
    N = x.shape[0]
    f = np.fft.fftshift(np.fft.fft2(x, axes=(0, 1)), axes=(0, 1))
    ky, kx = np.meshgrid(np.arange(N) - N // 2, np.arange(N) - N // 2, indexing="ij")
    f[np.sqrt(kx ** 2 + ky ** 2) > N / 2] = 0
    return np.fft.ifft2(np.fft.ifftshift(f, axes=(0, 1)), axes=(0, 1))


def _problem(seed, N=24, Nt=30, Ncyc=4, K=3, Nc=4, cplx=True):
    rng = np.random.default_rng(seed)
    img = (N, N)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, Ncyc, Nt)
    U = rand_c(rng, (Nt, K)) if cplx else rng.standard_normal((Nt, K)).astype(np.float32)
    U = np.linalg.svd(U, full_matrices=False)[0].astype(U.dtype)
    return rng, img, trj, U, _phantom(rng, img, K), _coil_maps(img, Nc)


def _gpu_recon(mr, img, trj, U, cm, data, mask=None, iters=20):
    cml = [cm[..., c] for c in range(cm.shape[-1])]
    A = mr.NFFTNormalOp(img, trj, U, cmaps=cml, sample_mask=mask)
    b = mr.calculate_backprojection(data, trj, cml, U=U, sample_mask=mask)
    return mr.to_host(mr.cg(A, b, maxiter=iters, reltol=0.0))


def _oracle_recon(img, trj, U, cm, data, mask=None, iters=20):
    cml = [cm[..., c] for c in range(cm.shape[-1])]
    G = tuple(2 * n for n in img)
    Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U, sample_mask=mask)
    K = U.shape[1]
    b = obp.calculate_backprojection(data, trj, cmaps=cml, U=U, sample_mask=mask)

    def apply(v):
        return onormal.nfft_normalop_apply(v.reshape(img + (K,), order="F"), Lam, km, img, cmaps=cml).ravel(order="F")

    x, _, _ = ocg.cg(apply, np.asarray(b).ravel(order="F"), maxiter=iters, reltol=0.0)
    return x.reshape(img + (K,), order="F")


def _data(mr, x, trj, U, cm):
    xt = mr.to_jl(x, torch.complex64)
    return mr.to_host(mr.forward_model(xt, trj, U, cmaps=mr.to_jl(cm, torch.complex64)))


@pytest.mark.parametrize("cplx", [True, False])
def test_radial_reconstruction(mr, cuda, cplx):
    """test/reconstruct_radial.jl (complex U) and reconstruct_radial_gpu_real.jl (real U, real Λ)."""
    rng, img, trj, U, x, cm = _problem(1 if cplx else 2, cplx=cplx)
    data = _data(mr, x, trj, U, cm)
    xg = _gpu_recon(mr, img, trj, U, cm, data)
    xo = _oracle_recon(img, trj, U, cm, data)
    assert rel_l2(xg, xo) < 1e-2
    truth = np.stack([_disk_crop(x[..., k]) for k in range(x.shape[-1])], axis=-1)
    assert rel_l2(xg, truth) < 1e-1


def test_asymmetric_half_spokes(mr, cuda):
    """test/reconstruct_radial_asym.jl: half spokes (centre outwards) with a real basis; the
    point-spread function is complex although the basis is real."""
    rng, img, trj, U, x, cm = _problem(3, cplx=False, Ncyc=8)
    half = np.ascontiguousarray(trj[:, trj.shape[1] // 2:, :])
    data = _data(mr, x, half, U, cm)
    xg = _gpu_recon(mr, img, half, U, cm, data)
    xo = _oracle_recon(img, half, U, cm, data)
    assert rel_l2(xg, xo) < 1e-2


def test_sample_mask_removes_a_spoke(mr, cuda):
    """test/data_removal.jl: a sample mask drops one spoke, so frames have unequal sample counts."""
    rng, img, trj, U, x, cm = _problem(4)
    mask = np.ones(trj.shape[1:], dtype=bool)
    Nr = 2 * img[0]
    mask[Nr:2 * Nr, 5] = False  # the second spoke of frame 6
    data = _data(mr, x, trj, U, cm)
    xg = _gpu_recon(mr, img, trj, U, cm, data, mask=mask)
    xo = _oracle_recon(img, trj, U, cm, data, mask=mask)
    assert rel_l2(xg, xo) < 1e-2
    full = _gpu_recon(mr, img, trj, U, cm, data)
    assert rel_l2(xg, full) > 1e-6  # the mask changes the result


def test_4d_wrappers_match_3d(mr, cuda):
    """test/wrapper_gpu.jl: trajectory (d, Nr, Ncyc, Nt) and data (Nr, Ncyc, Nt, Nc) give the
    same operator and backprojection as their (d, Nr*Ncyc, Nt) / (Nr*Ncyc, Nt, Nc) reshapes."""
    rng, img, trj, U, x, cm = _problem(5)
    Nr, Ncyc = 2 * img[0], 4
    data = _data(mr, x, trj, U, cm)
    trj4 = trj.reshape(2, Nr, Ncyc, trj.shape[2], order="F")
    data4 = data.reshape(Nr, Ncyc, data.shape[1], data.shape[2], order="F")
    cml = [cm[..., c] for c in range(cm.shape[-1])]
    A3 = mr.NFFTNormalOp(img, trj, U, cmaps=cml)
    A4 = mr.NFFTNormalOp(img, trj4, U, cmaps=cml)
    v = mr.to_jl(rand_c(rng, img + (U.shape[1],)), torch.complex64)
    assert rel_l2(mr.to_host(A4 @ v), mr.to_host(A3 @ v)) < 1e-6
    b3 = mr.to_host(mr.calculate_backprojection(data, trj, cml, U=U))
    b4 = mr.to_host(mr.calculate_backprojection(data4, trj4, cml, U=U))
    assert rel_l2(b4, b3) < 1e-5
