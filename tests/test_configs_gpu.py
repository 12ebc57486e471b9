"""Parity at the benchmark configurations' own sizes.

The other GPU tests run on small cases the exact-sum oracle finishes in
seconds.  These run the CUDA path on the configuration shapes themselves:

* 64^2, Nt = 200 x 1 spoke x 128 samples, 4 coils, K = 4 (the CPU-runnable
  configuration at its exact shape): operator from the trajectory, backprojection
  and cg(A, b; maxiter = 20) against the float64 oracle with exact sums
  (test/reconstruct_radial.jl:62-96 is the reference's version of this pipeline);
* 256^2, Nt = 1000 x 1 x 512 (512k samples), K = 5: the trajectory-built kernel Λ
  and kmask against the float64 oracle (spreading NUFFT point-spread sums,
  ~1e-7), every k-space centre cell summing ~10^4 samples, and bitwise
  reproducibility of Λ and of the 20-coil backprojection run to run (the grids
  accumulate in 64-bit fixed point, so the sums do not depend on the order in
  which the samples land);
* 128^3 (256^3 grid): the apply from a given Λ against the oracle
  (ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218);
* 256^2 GROG with 32 coils and 1000 spokes of 512 samples: grid indices bit-exact
  on all 512k samples, lnG and gridded data against the oracle
  (src/GROG.jl:14-102; 1000 spokes < 32^2 is the regime where the reference
  warns that the calibration is ill-posed, src/GROG.jl:26-27).
"""
import numpy as np
import pytest
import torch

from oracle import backprojection as obp
from oracle import cbuild
from oracle import cg as ocg
from oracle import grog as ogrog
from oracle import normalop as onormal
from oracle import nudft
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


def _synthetic(mr, img, Nt, K, Nc, seed=42):
    D = mr.synthetic.dictionary(Nt, seed=seed)
    U = mr.synthetic.basis(D, K)
    x = mr.synthetic.phantom(img, D, U, seed=seed)
    cm = mr.synthetic.coil_maps(img, Nc, seed=seed)
    return U, x, cm


def _data(mr, x, trj, U, cm):
    d = mr.forward_model(mr.to_jl(x, torch.complex64), trj, U, cmaps=mr.to_jl(cm, torch.complex64))
    return mr.to_host(mr.synthetic.add_noise(d, 0.01))


def test_cfg_64_nt200_nc4_k4_pipeline_matches_oracle(mr, cuda):
    img, Nr, Nt, K, Nc = (64, 64), 128, 200, 4, 4
    trj = otraj.traj_2d_radial_goldenratio(Nr, 1, Nt)
    U, x, cm = _synthetic(mr, img, Nt, K, Nc)
    data = _data(mr, x, trj, U, cm)
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, trj, U, cmaps=cml)
    b = mr.calculate_backprojection(data, trj, cml, U=U)
    xr = mr.to_host(mr.cg(A, b, maxiter=20, reltol=0.0))

    G = tuple(2 * n for n in img)
    Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U)
    np.testing.assert_array_equal(mr.to_host(A.kmask_indcs), km)
    assert rel_l2(mr.to_host(A.Λ), onormal.pack_lambda(Lam, real=True)) < 1e-5
    bo = obp.calculate_backprojection(data, trj, cmaps=cml, U=U)
    assert rel_l2(mr.to_host(b), bo) < 1e-5

    def apply(v):
        return onormal.nfft_normalop_apply(v.reshape(img + (K,), order="F"), Lam, km, img, cmaps=cml).ravel(order="F")

    xo, _, _ = ocg.cg(apply, bo.ravel(order="F"), maxiter=20, reltol=0.0)
    err = rel_l2(xr, xo.reshape(img + (K,), order="F"))
    print(f"64^2 cg-20 vs float64 oracle: {err:.2e}")
    assert err < 1e-4


def test_cfg_256_nt1000_lambda_matches_oracle_and_is_reproducible(mr, cuda):
    img, Nr, Nt, K = (256, 256), 512, 1000, 5
    trj = otraj.traj_2d_radial_goldenratio(Nr, 1, Nt)
    D = mr.synthetic.dictionary(Nt)
    U = mr.synthetic.basis(D, K)
    A1 = mr.NFFTNormalOp(img, trj, U)
    A2 = mr.NFFTNormalOp(img, trj, U)
    L1, L2 = mr.to_host(A1.Λ), mr.to_host(A2.Λ)
    np.testing.assert_array_equal(L1, L2)  # bitwise: fixed-point sums do not depend on sample order
    G = tuple(2 * n for n in img)
    Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U, fast=True)
    np.testing.assert_array_equal(mr.to_host(A1.kmask_indcs), km)
    Lo = onormal.pack_lambda(Lam, real=True)
    err = rel_l2(L1, Lo)
    # the centre cells sum every spoke: compare them on their own as well
    cen = np.argsort(-np.abs(Lo[0]))[:2000]
    err_c = rel_l2(L1[:, cen], Lo[:, cen])
    print(f"256^2 / 512k samples: Λ rel L2 {err:.2e}, 2000 largest cells {err_c:.2e}")
    assert err < 1e-5 and err_c < 1e-5


def test_cfg_256_nt1000_nc20_backprojection_reproducible_and_matches_oracle(mr, cuda):
    img, Nr, Nt, K, Nc = (256, 256), 512, 1000, 5, 20
    trj = otraj.traj_2d_radial_goldenratio(Nr, 1, Nt)
    U, x, cm = _synthetic(mr, img, Nt, K, Nc)
    data = _data(mr, x, trj, U, cm)
    cml = [cm[..., c] for c in range(Nc)]
    b1 = mr.to_host(mr.calculate_backprojection(data, trj, cml, U=U))
    b2 = mr.to_host(mr.calculate_backprojection(data, trj, cml, U=U))
    np.testing.assert_array_equal(b1, b2)
    # per-coil backprojection of two coils against the oracle's float64 spreading NUFFT
    sub = np.ascontiguousarray(data[..., :2])
    bc = mr.to_host(mr.calculate_backprojection(sub, trj, img, U=U))  # (img..., K, 2)
    pts = trj.reshape(2, -1, order="F").astype(np.float64)
    t_of = np.repeat(np.arange(Nt), Nr)
    plan = nudft.Nufft1Plan(pts, [np.arange(n) - n // 2 for n in img], +1.0)
    ref = np.zeros(img + (K, 2), dtype=np.complex128)
    for c in range(2):
        y = sub[..., c].ravel(order="F").astype(np.complex128)
        for k in range(K):
            ref[..., k, c] = plan(y * U[t_of, k])
    err = rel_l2(bc, ref)
    print(f"256^2 / 512k samples: per-coil backprojection rel L2 {err:.2e}")
    assert err < 1e-5


def test_cfg_128cubed_apply_matches_oracle(mr, cuda):
    rng = np.random.default_rng(7)
    img, K, Nc = (128, 128, 128), 2, 2
    G = tuple(2 * n for n in img)
    cells = np.flatnonzero(rng.random(int(np.prod(G))) < 0.5) + 1
    P = K * (K + 1) // 2
    lam = rng.standard_normal((P, cells.size)).astype(np.float32)  # real kernel, as for a real basis
    cm = rand_c(rng, img + (Nc,))
    x = rand_c(rng, img + (K,))
    cml = [cm[..., c] for c in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml)
    y = mr.to_host(A @ mr.to_jl(x, torch.complex64))
    ref = onormal.nfft_normalop_apply(x, onormal.unpack_lambda(lam.astype(np.complex128), K), cells, img, cmaps=cml)
    err = rel_l2(y, ref)
    print(f"128^3 apply rel L2 {err:.2e}")
    assert err < 1e-5


def test_cfg_grog_256_nc32_1000_spokes(mr, cuda):
    img, Nr, Nt, spf, Nc = (256, 256), 512, 500, 2, 32
    trj = otraj.traj_2d_radial_goldenratio(Nr, spf, Nt)
    D = mr.synthetic.dictionary(Nt)
    U1 = np.ones((Nt, 1), dtype=np.float32)  # one image for every frame
    x = mr.synthetic.phantom(img, D, mr.synthetic.basis(D, 1))
    cm = mr.synthetic.coil_maps(img, Nc)
    data = _data(mr, x, trj, U1, cm)
    with pytest.warns(UserWarning):  # 1000 spokes < 32^2: src/GROG.jl:26-27 warns
        lnG = [mr.to_host(m) for m in mr.grog_calib(data, trj, Nr)]
    # the oracle's batched eigendecomposition logarithm, pinned against scipy's Schur-form
    # logm on the first 40 spokes
    sub = (np.ascontiguousarray(data[:, :20]), np.ascontiguousarray(trj[:, :, :20]))
    for a, b in zip(ogrog.grog_calib(*sub, Nr), ogrog.grog_calib(*sub, Nr, log_method="eig")):
        assert rel_l2(b, a) < 1e-9
    ref = ogrog.grog_calib(data, trj, Nr, log_method="eig")
    errs = [rel_l2(a, b) for a, b in zip(lnG, ref)]
    print(f"GROG 32 coils / 1000 spokes: lnG rel L2 {errs}")
    assert max(errs) < 1e-3
    # gridding: indices bit-exact on every sample; data against the oracle on 8 frames
    lnG32 = [m.astype(np.complex64) for m in lnG]
    d = mr.to_jl(data, torch.complex64)
    idx = mr.to_host(mr.grog_gridding(d, trj, lnG32, Nr, img))
    np.testing.assert_array_equal(idx, cbuild.grog_index_c(trj, img, Nr)[0])
    fr = slice(0, 8)
    ref_idx, ref_data = ogrog.grog_gridding(np.ascontiguousarray(data[:, fr]), np.ascontiguousarray(trj[:, :, fr]),
                                            lnG32, Nr, img)
    np.testing.assert_array_equal(idx[:, :, fr], ref_idx)
    got = mr.to_host(d)[:, fr]
    err = rel_l2(got, ref_data[..., 0] if ref_data.ndim == 4 else ref_data)
    print(f"GROG gridded data (8 frames) rel L2 {err:.2e}")
    assert err < 1e-4
