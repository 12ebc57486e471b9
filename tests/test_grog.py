"""GROG (src/GROG.jl): oracle pins on the CPU, CUDA parity on the GPU.

Grid indices are integer work: bit-exact against the C and NumPy
restatements of src/GROG.jl:89-94.  lnG and the gridded data are compared
with the float64 oracle (lstsq + scipy logm/expm) at 1e-4 relative L2 (the
reference itself computes in float32).
"""
import numpy as np
import pytest
import scipy.linalg as sla

from oracle import cbuild, grog as ogrog, nudft, trajectories as otraj
from tests.helpers import rand_c, rel_l2, shepp_logan


def _grog_data(N=16, Ncyc=3, Nt=40, Nc=8, seed=0):
    rng = np.random.default_rng(seed)
    Nr = 2 * N
    trj = otraj.traj_2d_radial_goldenratio(Nr, Ncyc, Nt)
    g = np.meshgrid(np.linspace(-1, 1, N), np.linspace(-1, 1, N), indexing="ij")
    # asymmetric object and jittered coil positions: symmetric data makes the spoke Gram matrices singular
    x = ((g[0] ** 2 + 1.5 * g[1] ** 2) < 0.6).astype(float) + 0.5 * ((g[0] - 0.2) ** 2 + (g[1] - 0.3) ** 2 < 0.05)
    x = x * (1.0 + 0.3 * g[0] + 0.2 * g[1] ** 2)
    maps = []
    for c in range(Nc):
        a = 2 * np.pi * c / Nc + rng.uniform(-0.2, 0.2)
        maps.append(np.exp(-((g[0] - 1.2 * np.cos(a)) ** 2 + (g[1] - 1.2 * np.sin(a)) ** 2) / 1.5)
                    * np.exp(1j * np.pi * 0.2 * (g[0] * np.cos(a) + g[1] * np.sin(a))))
    maps = np.stack(maps, -1)
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, -1, keepdims=True))
    pts = trj.reshape(2, -1, order="F").astype(np.float64)
    data = np.stack([nudft.forward(maps[..., c] * x, pts).reshape(trj.shape[1:], order="F") for c in range(Nc)], -1)
    # 1% complex Gaussian noise, as in the synthetic benchmark data
    sigma = 0.01 * np.sqrt(np.mean(np.abs(data) ** 2))
    data = data + sigma * (rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape)) / np.sqrt(2)
    return trj, data.astype(np.complex64), Nr, (N, N), maps.astype(np.complex64), x


# ------------------------------------------------------------ CPU pins ---
def test_grog_index_c_and_numpy_agree_bitwise():
    rng = np.random.default_rng(1)
    trj = otraj.traj_2d_radial_goldenratio(64, 3, 20)
    trj = np.concatenate([trj, rng.uniform(-0.5, 0.5, (2, 64, 20)).astype(np.float32)], axis=1)
    ic, sc = cbuild.grog_index_c(trj, (32, 32), 64)
    inp, snp = ogrog.grog_index(trj, (32, 32), 64)
    np.testing.assert_array_equal(ic, inp)
    np.testing.assert_array_equal(sc, snp)


def test_grog_index_ties_round_to_even():
    """The first golden-angle spoke has ky = 0 -> t = 0.5 -> k = 0 (src/GROG.jl:91-92)."""
    N = 16
    trj = np.array([[[0.0], [1.0 / N], [-0.5], [0.5]], [[0.0], [0.0], [0.0], [0.0]]], dtype=np.float32)
    idx, shift = ogrog.grog_index(trj, (N, N), 2 * N)
    assert idx[0, 0, 0] == 0 + N // 2          # round(0.5) = 0
    assert idx[0, 1, 0] == 2 + N // 2          # round(1.5) = 2
    assert idx[0, 2, 0] == -8 + N // 2         # round(-7.5) = -8
    assert idx[0, 3, 0] == 8 + N // 2          # round(8.5) = 8
    assert shift[0, 0, 0] == (0 - 0.5) * 2 * N / N


def test_grog_calibration_repeat_invariance_and_spoke_shift():
    """test/grog_precalc_shift.jl:64-67 and test/grog_spoke_shift.jl:60-73 on synthetic data."""
    trj, data, Nr, img, _, _ = _grog_data()
    lnG = ogrog.grog_calib(data, trj, Nr)
    lnG2 = ogrog.grog_calib(np.repeat(data[..., None], 3, axis=3), trj, Nr)
    for a, b in zip(lnG, lnG2):
        assert rel_l2(b, a) < 1e-6
    dr = data.reshape((Nr, -1, data.shape[2]), order="F")
    tr = trj.reshape((2, Nr, -1), order="F")
    for sp in range(0, dr.shape[1], 7):
        nm = (tr[:, 1, sp] - tr[:, 0, sp]) * Nr
        E = sla.expm(nm[0] * lnG[0]) @ sla.expm(nm[1] * lnG[1])
        d1 = (E @ dr[:-1, sp, :].T).T
        assert rel_l2(d1, dr[1:, sp, :]) < 3e-1


# ---------------------------------------------------------- GPU parity ---
@pytest.mark.gpu
def test_grog_calib_matches_oracle(mr, cuda):
    trj, data, Nr, img, _, _ = _grog_data()
    lnG = [mr.to_host(m) for m in mr.grog_calib(data, trj, Nr)]
    ref = ogrog.grog_calib(data, trj, Nr)
    for a, b in zip(lnG, ref):
        assert rel_l2(a, b) < 1e-4


@pytest.mark.gpu
def test_grog_calib_repeat_invariance(mr, cuda):
    trj, data, Nr, img, _, _ = _grog_data(seed=2)
    l1 = [mr.to_host(m) for m in mr.grog_calib(data, trj, Nr)]
    l2 = [mr.to_host(m) for m in mr.grog_calib(np.repeat(data[..., None], 3, axis=3), trj, Nr)]
    for a, b in zip(l1, l2):
        assert rel_l2(b, a) < 1e-6  # test/grog_precalc_shift.jl:67


@pytest.mark.gpu
@pytest.mark.parametrize("nrep", [1, 2])
def test_grog_gridding_matches_oracle(mr, cuda, nrep):
    import torch
    trj, data, Nr, img, _, _ = _grog_data(seed=3)
    if nrep > 1:
        data = np.repeat(data[..., None], nrep, axis=3)
    lnG = ogrog.grog_calib(data, trj, Nr)
    lnG32 = [m.astype(np.complex64) for m in lnG]
    d = mr.to_jl(data, torch.complex64)
    idx = mr.to_host(mr.grog_gridding(d, trj, lnG32, Nr, img))
    ref_idx, ref_data = ogrog.grog_gridding(data, trj, lnG32, Nr, img)
    np.testing.assert_array_equal(idx, ref_idx)                       # bit-exact indices
    np.testing.assert_array_equal(idx, cbuild.grog_index_c(trj, img, Nr)[0])
    got = mr.to_host(d)
    if nrep == 1:
        ref_data = ref_data[..., 0]
    assert rel_l2(got, ref_data) < 1e-4
    if nrep > 1:  # the repetitions grid identically (test/grog_precalc_shift.jl:81-82)
        assert rel_l2(got[..., 1], got[..., 0]) < 1e-5


@pytest.mark.gpu
def test_radial_grog_then_fft_normalop_recon(mr, cuda):
    """test/grog_recon.jl at its own sizes: 64^2, Nr = 128, rank 4 (two non-zero coefficient
    images: the modified Shepp-Logan phantom), Nt = 100 frames x 200 golden-angle spokes, 9 Gaussian coil maps.  Both the NUFFT
    reconstruction (NFFTNormalOp + cg, 20 iterations) and the GROG reconstruction (radial_grog!
    + FFTNormalOp + cg, 20 iterations, global phase slope removed as in :91-92) match the
    phantom cropped to the sampled k-space disk within the reference's rtol = 5e-2 (:95-96)."""
    import torch
    Nx, Nr, K, Nt, Ncyc, Ncoil = 64, 128, 4, 100, 200, 9
    img = (Nx, Nx)
    rng = np.random.default_rng(42)
    x = np.zeros((Nx, Nx, K), dtype=np.complex64)
    sl = shepp_logan(Nx, oversample=4)  # the modified Shepp-Logan phantom, anti-aliased
    x[:, :, 0] = sl.T
    x[: Nx // 2, :, 0] *= np.exp(1j * np.pi / 3)
    x[:, :, 1] = sl
    # Gaussian coil maps centred on a 3 x 3 grid (gauss2 at Nx/8, Nx/2, 7Nx/8, width Nx/1.5)
    ii, jj = np.meshgrid(np.arange(1, Nx + 1), np.arange(1, Nx + 1), indexing="ij")
    cm = np.empty((Nx, Nx, Ncoil), dtype=np.complex64)
    centres = [Nx // 8, Nx // 2, 7 * Nx // 8]
    for a, ca in enumerate(centres):
        for b, cb in enumerate(centres):
            w = Nx // 1.5
            cm[:, :, 3 * a + b] = np.exp(-4 * np.log(2) * (((ii - ca) / w) ** 2 + ((jj - cb) / w) ** 2))
    cm /= np.sqrt(np.sum(np.abs(cm) ** 2, axis=-1, keepdims=True))
    # traj_kooshball(Nr, theta = pi/2, phi = golden angle) restricted to its first two dimensions
    ag = 2 * np.pi / (1 + np.sqrt(5))
    phi = (ag * np.arange(Nt * Ncyc)).astype(np.float32).reshape(Ncyc, Nt, order="F")
    theta = np.full_like(phi, np.float32(np.pi / 2))
    trj = np.ascontiguousarray(otraj.traj_kooshball(Nr, theta, phi)[:2]).astype(np.float32)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    cmd = mr.to_jl(cm, torch.complex64)
    d = mr.forward_model(mr.to_jl(x, torch.complex64), trj, U, cmaps=cmd)
    cml = [cm[..., c] for c in range(Ncoil)]
    # ground truth: x cropped to the disk |k| <= Nx/2
    xc = np.fft.fftshift(np.fft.fft2(x, axes=(0, 1)), axes=(0, 1))
    xc[(ii - 1 - Nx / 2) ** 2 + (jj - 1 - Nx / 2) ** 2 > (Nx / 2) ** 2] = 0
    xc = np.fft.ifft2(np.fft.ifftshift(xc, axes=(0, 1)), axes=(0, 1))
    # NUFFT reconstruction
    A = mr.NFFTNormalOp(img, trj, U, cmaps=cml)
    b = mr.calculate_backprojection(d, trj, cml, U=U)
    xr = mr.to_host(mr.cg(A, b, maxiter=20))
    # GROG reconstruction
    trj_cart = mr.radial_grog(d, trj, Nr, img)
    Ac = mr.FFTNormalOp(img, trj_cart, U, cmaps=cml)
    bc = mr.calculate_backprojection(d, trj_cart, cml, U=U)
    xg = mr.to_host(mr.cg(Ac, bc, maxiter=20))
    xg = xg * -np.exp(1j * np.pi * ((ii - 1) + (jj - 1)) / Nx)[..., None]

    def isapprox(a, b, rtol):  # Julia's norm-wise isapprox
        return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))

    er, eg = rel_l2(xr, xc), rel_l2(xg, xc)
    print(f"grog_recon: NUFFT recon vs crop {er:.3e}, GROG recon vs crop {eg:.3e}")
    assert isapprox(xc, xr, 5e-2)
    assert isapprox(xc, xg, 5e-2)
