"""The coil-map calibration caller (src/CoilMaps.jl): calibration masks on the CPU,
coil-wise reconstructions on the GPU against the float64 oracle.

``reconstruct_coilwise`` solves one K=1 system per receive channel on a single
operator (src/CoilMaps.jl:118-162).  Checks:
* the Nc solves on the operator stacked over the coils equal Nc sequential ``cg`` calls
  on the same operator (1e-6);
* the coil images agree with the float64 oracle's 20-iteration CG on the exact-PSF
  operator within 1e-2 (the reference's CPU-vs-GPU tolerance,
  test/reconstruct_radial_gpu.jl:103; the GPU NUFFT uses the ES kernel).  Two operators
  built from the same inputs differ in the last bits (Λ is spread with float atomics),
  and 20 float32 CG iterations that fit the 1% noise amplify that to 1e-4 .. 1e-3, so
  runs are compared through the oracle, not with each other;
* the Cartesian form (5 tolerance-checked iterations) against the oracle's.
"""
import importlib

import numpy as np
import pytest
import torch

from oracle import backprojection as obp
from oracle import cg as ocg
from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2


def _radial(seed=0, N=24, Nt=10, Ncyc=6, Nc=4):
    rng = np.random.default_rng(seed)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, Ncyc, Nt)
    data = rand_c(rng, trj.shape[1:] + (Nc,))
    return rng, trj, data


def _consistent_data(mr, seed=0, N=24, Nt=10, Ncyc=6, Nc=4):
    """Samples of a smooth object seen through Nc smooth coil maps (K=1, U = ones):
    a well-posed calibration problem, as the reference's calibration region is."""
    rng = np.random.default_rng(seed)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, Ncyc, Nt)
    g = np.meshgrid(np.linspace(-1, 1, N), np.linspace(-1, 1, N), indexing="ij")
    obj = (np.exp(-(g[0] ** 2 + 1.5 * g[1] ** 2) / 0.4) * (1 + 0.3j * g[0])).astype(np.complex64)[..., None]
    cm = np.stack([np.exp(-((g[0] - np.cos(a)) ** 2 + (g[1] - np.sin(a)) ** 2)) * np.exp(1j * a * g[1])
                   for a in 2 * np.pi * np.arange(Nc) / Nc], -1).astype(np.complex64)
    U1 = np.ones((Nt, 1), np.float32)
    data = mr.to_host(mr.forward_model(mr.to_jl(obj, torch.complex64), trj, U1, cmaps=mr.to_jl(cm, torch.complex64)))
    data = data + 0.01 * rand_c(rng, data.shape) * np.sqrt(np.mean(np.abs(data) ** 2))
    return rng, trj, data.astype(np.complex64)


# ------------------------------------------------------------------ CPU ---
def test_calibration_mask_noncartesian(mr):
    rng, trj, _ = _radial(N=64)
    sm = rng.random(trj.shape[1:]) < 0.9
    mask, trj_c, cs = mr.calibration_mask(trj, (64, 64), sample_mask=sm)
    assert cs == (32, 32)  # nextprod((2,3,5), 64 ÷ (64 ÷ 32))
    ref = np.all(np.abs(trj) * np.float32(2.0) < 0.5, axis=0) & sm
    np.testing.assert_array_equal(mask, ref)
    np.testing.assert_array_equal(trj_c, trj * np.float32(2.0))
    assert mr.calibration_mask(trj, (256, 256))[2] == (32, 32)
    assert mr.calibration_mask(trj, (240, 256))[2] == (30, 32)
    with pytest.raises(AssertionError):
        mr.calibration_mask(trj, (64, 64), calib_size=(28, 28))


def test_calibration_mask_cartesian(mr):
    trj = otraj.traj_cartesian(64, 64, 1, 4, T=np.int32)[:2]
    mask, trj_c, cs = mr.calibration_mask(trj, (64, 64))
    assert cs == (32, 32) and trj_c is trj
    lo = int(np.ceil((64 - 32) / 2))
    ref = np.all(trj > lo, axis=0) & np.all(trj < lo + 33, axis=0)
    np.testing.assert_array_equal(mask, ref)


# ------------------------------------------------------------------ GPU ---
coilmaps = None


@pytest.fixture(autouse=True)
def _coilmaps_module(mr):
    global coilmaps
    coilmaps = importlib.import_module(mr.__name__ + ".coilmaps")

def _oracle_coilwise(data, trj, img, U1, mask, iters):
    G = tuple(2 * n for n in img)
    Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U1, sample_mask=mask)
    b = obp.calculate_backprojection(data, trj, img_shape=img, U=U1, sample_mask=mask)  # (img, 1, Nc)
    out = []
    for c in range(data.shape[2]):
        def apply(v):
            return onormal.nfft_normalop_apply(v.reshape(img + (1,), order="F"), Lam, km, img).ravel(order="F")
        x, _, _ = ocg.cg(apply, np.asarray(b)[..., 0, c].ravel(order="F"), maxiter=iters, reltol=0.0)
        out.append(x.reshape(img, order="F"))
    return np.stack(out, -1)


@pytest.mark.gpu
@pytest.mark.parametrize("cplx_u,masked", [(False, False), (True, True)])
def test_reconstruct_coilwise_noncartesian(mr, cuda, cplx_u, masked):
    rng, trj, data = _consistent_data(mr, seed=1)
    img, Nt = (24, 24), trj.shape[2]
    U = rand_c(rng, (Nt, 3)) if cplx_u else rng.standard_normal((Nt, 3)).astype(np.float32)
    U[:, 0] = 1.0  # the calibration uses the first basis column
    mask = (rng.random(trj.shape[1:]) < 0.85) if masked else None
    x = mr.to_host(mr.reconstruct_coilwise(data, trj, img, U=U, sample_mask=mask, Niter_cg=20))
    assert x.shape == img + (4,)
    U1 = U[:, :1]
    ref = _oracle_coilwise(data, trj, img, U1, mask, 20)
    assert rel_l2(x, ref) < 1e-2
    # the stacked per-coil solves against the sequential entry point on the same operator
    A = mr.NFFTNormalOp(img, trj, U1, sample_mask=mask)
    b = mr.calculate_backprojection(data, trj, img, U=U1, sample_mask=mask)
    xb = mr.to_host(coilmaps._coilwise_solve(A, b, 20))
    for c in range(4):
        xc = mr.to_host(mr.cg(A, b[..., 0, c], maxiter=20, reltol=0.0))[..., 0]
        assert rel_l2(xb[..., c], xc) < 1e-6, c


@pytest.mark.gpu
def test_reconstruct_coilwise_default_basis_is_ones(mr, cuda):
    rng, trj, data = _consistent_data(mr, seed=2, Nc=3)
    img = (24, 24)
    x0 = mr.to_host(mr.reconstruct_coilwise(data, trj, img, Niter_cg=10))
    U1 = np.ones((trj.shape[2], 1), np.float32)
    ref = _oracle_coilwise(data, trj, img, U1, None, 10)
    assert rel_l2(x0, ref) < 1e-2


@pytest.mark.gpu
def test_reconstruct_coilwise_cartesian(mr, cuda):
    rng = np.random.default_rng(3)
    N, Nt, Nc = 16, 6, 3
    trj = otraj.traj_cartesian(N, N, 1, Nt, T=np.int32)[:2]
    mask = rng.random(trj.shape[1:]) < 0.4
    data = rand_c(rng, trj.shape[1:] + (Nc,))
    U1 = np.ones((Nt, 1), np.float32)
    x = mr.to_host(mr.reconstruct_coilwise(data, trj, (N, N), sample_mask=mask))
    lam_c, km, _ = onormal.fft_normalop_from_lambda(onormal.calculate_kernel_cartesian((N, N), trj, U1, mask))
    b = obp.calculate_backprojection_cartesian(data, trj, img_shape=(N, N), U=U1, sample_mask=mask)
    for c in range(Nc):
        def apply(v):
            return onormal.fft_normalop_apply(v.reshape((N, N, 1), order="F"), lam_c, km, (N, N)).ravel(order="F")
        xr, _, _ = ocg.cg(apply, np.asarray(b)[..., 0, c].ravel(order="F"), maxiter=5)
        assert rel_l2(x[..., c], xr.reshape((N, N), order="F")) < 1e-4, c


@pytest.mark.gpu
def test_calibration_kspace(mr, cuda):
    """calculate_coil_maps up to ESPIRiT: the centred FFT of the coil-wise images of the
    calibration region (the samples with |k| * N / n < 1/2, coordinates scaled by N / n)."""
    rng, trj, data = _consistent_data(mr, seed=4, N=64, Nt=8, Ncyc=12)
    k = mr.calculate_calibration_kspace(data, trj, (64, 64), Niter_cg=15)
    assert k.shape == (32, 32, 4)
    mask, trj_c, cs = mr.calibration_mask(trj, (64, 64))
    x = _oracle_coilwise(data, trj_c, cs, np.ones((trj.shape[2], 1), np.float32), mask, 15)
    ref = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(x, axes=(0, 1)), axes=(0, 1)), axes=(0, 1))
    assert rel_l2(k, ref) < 1e-2
    # 4D wrapper: readout lines on their own axis
    Nr = 128
    trj4 = trj.reshape(2, Nr, -1, trj.shape[2], order="F")
    data4 = data.reshape(Nr, -1, data.shape[1], data.shape[2], order="F")
    k4 = mr.calculate_calibration_kspace(data4, trj4, (64, 64), Niter_cg=15)
    assert rel_l2(k4, ref) < 1e-2
