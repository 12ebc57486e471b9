"""Pins of the float64 oracle (CPU only).

The reference cannot run here and its tests hold no element-wise golden
vectors, so the oracle is pinned by (a) exact identities the reference's
algorithm must satisfy and (b) the reference tests' own known answers and
invariances, re-expressed on seeded synthetic inputs.
"""
import numpy as np
import pytest

from oracle import backprojection as obp
from oracle import cbuild, grog as ogrog, normalop as onormal, nudft, trajectories as otraj
from oracle.cg import cg as ocg
from tests.helpers import rand_c, rel_l2


def _radial(N, Ncyc, Nt, Nr=None):
    return otraj.traj_2d_radial_goldenratio(Nr or 2 * N, Ncyc, Nt)


# ----------------------------------------------------------------- trajectories
def test_golden_angle_trajectory_layout():
    """src/Trajectories.jl:81-93: phi starts at 0, sample index ir + Nr*icyc, frames consecutive angles."""
    Nr, Ncyc, Nt = 8, 2, 3
    k = otraj.traj_2d_radial_goldenratio(Nr, Ncyc, Nt)
    assert k.shape == (2, Nr * Ncyc, Nt) and k.dtype == np.float32
    kr = (np.arange(Nr) - (Nr - 1) / 2) / Nr
    # frame 0, cycle 0: phi = 0 -> kx = -kr, ky = 0
    np.testing.assert_allclose(k[0, :Nr, 0], -kr, rtol=0, atol=1e-7)
    np.testing.assert_array_equal(k[1, :Nr, 0], 0)
    # frame 1, cycle 0 has angle index 1; cycle 1 of frame 0 has index Nt
    ang = np.float32(np.pi / ((np.sqrt(5) + 1) / 2))
    for (s0, t, i) in ((0, 1, 1), (Nr, 0, Nt)):
        phi = np.float32(i * np.float64(ang))
        np.testing.assert_allclose(k[1, s0:s0 + Nr, t], np.sin(np.float64(phi)) * kr, atol=1e-6)
    assert np.all(np.abs(k) <= 0.5)


def test_golden_means():
    g1, g2 = otraj.calculate_golden_means()
    lam = 1 / g2
    assert abs(lam ** 3 - lam ** 2 - 1) < 1e-12 and abs(g1 - g2 ** 2) < 1e-12


def test_kooshball_and_cartesian_shapes():
    k = otraj.traj_kooshball_goldenratio(16, 3, 5, thetaRot=0.3, phiRot=0.2)
    assert k.shape == (3, 48, 5) and np.all(np.abs(k) <= 0.5)
    kc = otraj.traj_cartesian(4, 3, 2, 2, T=np.int32)
    assert kc.shape == (3, 24, 2)
    np.testing.assert_array_equal(kc[:, :5, 0].T, [[1, 1, 1], [2, 1, 1], [3, 1, 1], [4, 1, 1], [1, 2, 1]])


# ------------------------------------------------------- Toeplitz identities
@pytest.mark.parametrize("cplx", [True, False])
def test_toeplitz_embedding_equals_direct_normal_operator_2d(cplx):
    """With every cell kept, crop F^-1 Λ F pad equals Aᴴ A built from exact NUDFTs."""
    rng = np.random.default_rng(0)
    N, K, Nt, Ncyc = 8, 3, 6, 2
    img = (N, N)
    trj = _radial(N, Ncyc, Nt)
    U = np.linalg.svd(rand_c(rng, (Nt, K)) if cplx else rng.standard_normal((Nt, K)), full_matrices=False)[0]
    U = U.astype(np.complex64 if cplx else np.float32)
    Lam, kmask = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    all_cells = np.arange(1, 4 * N * N + 1)
    mask = np.ones(trj.shape[1:], dtype=bool)
    pts = onormal.masked_points(trj, mask)
    t_of = onormal.frame_of_sample(mask)
    # Λ on every cell
    Lfull = np.zeros((K, K, 4 * N * N), dtype=np.complex128)
    for k2 in range(K):
        for k1 in range(k2 + 1):
            w = np.conj(U[t_of, k1].astype(np.complex128)) * U[t_of, k2]
            c = onormal.psf((2 * N, 2 * N), pts, w)
            lam = np.fft.fftn(c).ravel(order="F")
            Lfull[k2, k1] = np.conj(lam)
            Lfull[k1, k2] = lam
    cm = [rand_c(rng, img).astype(np.complex128) for _ in range(2)]
    x = rand_c(rng, img + (K,)).astype(np.complex128)
    y = onormal.nfft_normalop_apply(x, Lfull, all_cells, img, cmaps=cm)
    # direct: sum_c S_c^H A_t^H A_t S_c with the subspace basis
    ref = np.zeros_like(y)
    for c in range(2):
        for k2 in range(K):
            f = nudft.forward(cm[c] * x[..., k2], pts)
            for k1 in range(K):
                v = f * np.conj(U[t_of, k1]) * U[t_of, k2]
                ref[..., k1] += np.conj(cm[c]) * nudft.adjoint(v, pts, img)
    # the adjoint/forward pair of the oracle uses centred coordinates; the phase cancels in AᴴA
    assert rel_l2(y, ref) < 1e-10


def test_kmask_is_union_of_footprints():
    trj = np.zeros((2, 1, 1), dtype=np.float32)
    km = onormal.kmask_indcs((16, 16), trj)
    assert km.size == 64
    cells = km - 1
    p1, p2 = cells % 16, cells // 16
    assert set(p1) == set(range(-3, 5)) - set() or set(p1) == {(i % 16) for i in range(-3, 5)}
    assert set(p2) == {(i % 16) for i in range(-3, 5)}
    # full radial coverage keeps most of the grid
    km2 = onormal.kmask_indcs((64, 64), _radial(32, 16, 20))
    assert 0.6 < km2.size / 64 ** 2 < 1.0


def test_real_and_complex_kernels_agree_on_the_operator():
    """A real basis stored as real or complex gives the same operator (ext:89 vs ext:140)."""
    rng = np.random.default_rng(1)
    N, K, Nt = 8, 2, 5
    trj = _radial(N, 2, Nt)
    U = np.linalg.svd(rng.standard_normal((Nt, K)), full_matrices=False)[0].astype(np.float32)
    Lr, km = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    Lc, km2 = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U.astype(np.complex64))
    np.testing.assert_array_equal(km, km2)
    x = rand_c(rng, (N, N, K))
    yr = onormal.nfft_normalop_apply(x, Lr, km, (N, N))
    yc = onormal.nfft_normalop_apply(x, Lc, km, (N, N))
    assert rel_l2(yr, yc) < 5e-3  # differ only through the grid-edge convention of the two PSFs


def test_kernel_diagonal_keeps_lambda():
    """The diagonal blocks are λ itself, not its conjugate (src/NFFTNormalOp.jl:161-162 order)."""
    rng = np.random.default_rng(5)
    N, K, Nt = 8, 2, 4
    trj = _radial(N, 2, Nt)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    Lam, km = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    mask = np.ones(trj.shape[1:], dtype=bool)
    pts = onormal.masked_points(trj, mask)
    t_of = onormal.frame_of_sample(mask)
    w = np.abs(U[t_of, 0].astype(np.complex128)) ** 2
    lam = np.fft.fftn(onormal.psf((2 * N, 2 * N), pts, w)).ravel(order="F")[km - 1]
    np.testing.assert_allclose(Lam[0, 0], lam, rtol=1e-12, atol=1e-9)
    assert np.abs(lam.imag).max() > 1e-6  # the grid-edge PSF entry makes the diagonal slightly complex


def test_packing_roundtrip():
    rng = np.random.default_rng(2)
    K = 4
    L = rand_c(rng, (K, K, 7)).astype(np.complex128)
    L = (L + np.conj(np.transpose(L, (1, 0, 2)))) / 2
    np.testing.assert_allclose(onormal.unpack_lambda(onormal.pack_lambda(L), K), L)


def test_cpu_baseline_apply_matches_oracle():
    """The float32 CPU restatement timed as the baseline computes the same operator."""
    from oracle.cpu_apply import CpuNFFTNormalOp
    rng = np.random.default_rng(7)
    for img in ((12, 16), (8, 6, 10)):
        K, Nc = 3, 2
        G = tuple(2 * n for n in img)
        km = np.flatnonzero(rng.random(int(np.prod(G))) < 0.7) + 1
        P = K * (K + 1) // 2
        Lp = rand_c(rng, (P, km.size)).astype(np.complex128)
        Lam = onormal.unpack_lambda(Lp, K)
        cm = rand_c(rng, img + (Nc,))
        x = rand_c(rng, img + (K,))
        y = CpuNFFTNormalOp(img, Lam, km, cm, workers=2).apply(x)
        ref = onormal.nfft_normalop_apply(x, Lam, km, img, cmaps=[cm[..., c] for c in range(Nc)])
        assert rel_l2(y, ref) < 1e-5


def test_package_trajectories_match_oracle(mr):
    """The package's input generators reproduce the oracle restatement of src/Trajectories.jl."""
    from importlib import import_module
    tr = import_module("mrsr_gb300.trajectories")
    np.testing.assert_array_equal(tr.traj_2d_radial_goldenratio(64, 2, 7), otraj.traj_2d_radial_goldenratio(64, 2, 7))
    np.testing.assert_array_equal(tr.traj_kooshball_goldenratio(32, 3, 4, thetaRot=0.2, phiRot=0.1),
                                  otraj.traj_kooshball_goldenratio(32, 3, 4, thetaRot=0.2, phiRot=0.1))
    np.testing.assert_array_equal(tr.traj_cartesian(4, 3, 2, 2, T=np.int32), otraj.traj_cartesian(4, 3, 2, 2, T=np.int32))
    g1, g2 = tr.calculate_golden_means()
    o1, o2 = otraj.calculate_golden_means()
    assert abs(g1 - o1) < 1e-14 and abs(g2 - o2) < 1e-14


def _espirit_consistent_calibration(N=64, Nc=8, calib=24, seed=0):
    """Calibration k-space of smooth coil maps times an object, and the true maps."""
    g = np.meshgrid(np.linspace(-1, 1, N), np.linspace(-1, 1, N), indexing="ij")
    m = ((g[0] / 0.7) ** 2 + (g[1] / 0.85) ** 2 <= 1).astype(float) * (1 + 0.3 * g[0])
    S = np.empty((N, N, Nc), complex)
    for c in range(Nc):
        a = 2 * np.pi * c / Nc
        S[..., c] = (np.exp(-((g[0] - 1.3 * np.cos(a)) ** 2 + (g[1] - 1.3 * np.sin(a)) ** 2) / 2.0)
                     * np.exp(1j * np.pi * 0.3 * (np.cos(a) * g[0] + np.sin(a) * g[1])))
    S /= np.sqrt(np.sum(np.abs(S) ** 2, -1, keepdims=True))
    X = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(S * m[..., None], axes=(0, 1)), axes=(0, 1)), axes=(0, 1))
    c0 = N // 2 - calib // 2
    return X[c0:c0 + calib, c0:c0 + calib], S, m


def test_espirit_oracle_recovers_known_maps():
    """ESPIRiT's defining property (Uecker et al. 2014): on consistent calibration data the
    true sensitivities, normalised to unit root-sum-of-squares, are eigenvalue-1
    eigenvectors of the image-space operator, so the maps reproduce them (up to a
    per-pixel phase, fixed here by coil 1)."""
    from oracle import espirit as oesp
    kbp, S, m = _espirit_consistent_calibration()
    maps, lam = oesp.espirit(kbp, (64, 64), (6, 6))
    obj = m > 0
    assert lam[obj, 0].min() > 0.99
    Sn = S * (np.conj(S[..., 0:1]) / np.abs(S[..., 0:1]))
    err = np.linalg.norm((maps[..., 0] - Sn)[obj]) / np.linalg.norm(Sn[obj])
    assert err < 1e-2
