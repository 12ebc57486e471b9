"""The reconstruction server and its device pieces on the GPU.

* mrsr_normalop_share: an operator on a shared kernel applies exactly like a
  fresh operator with the same kernel and coil maps, also after the operator
  it was made from is destroyed.
* CgBatch: each branch of the graph equals ``cg(A, b; maxiter, reltol=0)``.
* The server: every request's image equals the same request served alone and
  the direct API calls (backprojection + cg) bit for bit: the kernel and the
  backprojection accumulate in 64-bit fixed point, and every reduction of the
  solve has a fixed order, so nothing depends on what else is on the GPU.
"""
import importlib

import numpy as np
import pytest
import torch

from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sv(mr):
    return importlib.import_module(mr.__name__ + ".serving")


def _op_problem(mr, seed=0, N=32, K=3, Nc=3, Nt=12):
    rng = np.random.default_rng(seed)
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 2, Nt)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].real.astype(np.float32)
    cm = rand_c(rng, (N, N, Nc))
    return trj, U, cm


def test_share_matches_fresh_operator(mr, cuda):
    trj, U, cm = _op_problem(mr)
    N, K = 32, 3
    base = mr.NFFTNormalOp((N, N), trj, U)
    lam, km = base.Λ, base.kmask_indcs
    cml = [cm[..., c] for c in range(cm.shape[-1])]
    fresh = mr.NFFTNormalOp((N, N), lam, km, cmaps=cml)
    shared = base.share(cmaps=cml)
    assert shared.ncoils == cm.shape[-1] and shared.nk == base.nk
    x = mr.to_jl(rand_c(np.random.default_rng(1), (N, N, K)), torch.complex64)
    y1 = mr.to_host(fresh @ x)
    base.close()                  # the kernel stays alive while `shared` uses it
    y2 = mr.to_host(shared @ x)
    assert np.array_equal(y1, y2)
    half = shared.share(cmaps=cml, precision="fp16")
    assert half.precision == 1
    assert rel_l2(mr.to_host(half @ x), y1) < 2e-3


def test_cg_batch_branches_equal_cg(mr, cuda):
    rng = np.random.default_rng(2)
    ops, bs, refs = [], [], []
    for i, (N, K, Nc) in enumerate(((32, 3, 2), (48, 2, 3), (32, 4, 1))):
        trj, U, cm = _op_problem(mr, seed=10 + i, N=N, K=K, Nc=Nc)
        A = mr.NFFTNormalOp((N, N), trj, U, cmaps=[cm[..., c] for c in range(Nc)])
        b = mr.to_jl(rand_c(rng, (N, N, K)), torch.complex64)
        ops.append(A)
        bs.append(b)
        refs.append(mr.to_host(mr.cg(A, b, maxiter=7, reltol=0.0)))
    xs = [mr.jl_empty(b.shape, torch.complex64) for b in bs]
    batch = mr.CgBatch(ops, bs, xs, 7)
    for rep in range(2):          # the graph relaunches with the same result
        batch.launch()
        torch.cuda.synchronize()
        for i in range(3):
            assert rel_l2(mr.to_host(xs[i]), refs[i]) < 1e-6, (rep, i)
            it, rn = batch.result(i)
            assert it == 7 and np.isfinite(rn)
    with pytest.raises(ValueError):
        mr.CgBatch([ops[0], ops[0]], [bs[0], bs[0]], [xs[0], mr.jl_empty(bs[0].shape, torch.complex64)], 3)


def _serve_problem(mr, sv):
    protos = []
    for i, (N, K, Nt) in enumerate(((32, 3, 40), (64, 2, 30), (32, 4, 24))):
        trj = mr.trajectories.traj_2d_radial_goldenratio(2 * N, 2, Nt, thetaRot=0.3 * i)
        U = mr.synthetic.basis(mr.synthetic.dictionary(Nt, natoms=200, seed=i), K)
        protos.append(sv.Protocol(name=f"p{i}", img=(N, N), trj=mr.to_jl(trj, torch.float32),
                                  U=mr.to_jl(U, torch.float32), K=K))
    scans = [sv.make_scans(mr, p, 4, seed=i) for i, p in enumerate(protos)]
    torch.cuda.synchronize()
    return protos, scans


def test_server_results_equal_alone_and_direct(mr, cuda, sv):
    protos, scans = _serve_problem(mr, sv)
    iters = 8
    reqs = sv.make_request_stream(protos, scans, 12, rate_hz=2000.0, coil_range=(2, 4), seed=3)
    ex = sv.GpuExecutor(mr, iters=iters)
    srv = sv.ReconServer(ex, 8 << 30, slots=3, max_batch=3)
    st = srv.run(reqs)
    assert st.completed == 12 and st.kernel_builds == 3
    mix = {r.rid: mr.to_host(r.x) for r in reqs}
    for r in reqs:
        # alone: a fresh server, one slot, one request
        alone = sv.Request(rid=r.rid, protocol=r.protocol, data=r.data, cmaps=r.cmaps, arrival=0.0)
        srv1 = sv.ReconServer(sv.GpuExecutor(mr, iters=iters), 8 << 30, slots=1, max_batch=1)
        srv1.run([alone])
        srv1.close()
        np.testing.assert_array_equal(mr.to_host(alone.x), mix[r.rid], err_msg=str(r.rid))
        # the direct calls of the package API
        p = r.protocol
        A = mr.NFFTNormalOp(p.img, p.trj, p.U, cmaps=r.cmaps)
        b = mr.calculate_backprojection(r.data, p.trj, r.cmaps, U=p.U)
        x = mr.to_host(mr.cg(A, b, maxiter=iters, reltol=0.0))
        np.testing.assert_array_equal(x, mix[r.rid], err_msg=str(r.rid))
    srv.close()


def test_server_refined_precision(mr, cuda, sv):
    protos, scans = _serve_problem(mr, sv)
    reqs = sv.make_request_stream(protos, scans, 6, rate_hz=0.0, coil_range=(3, 4), seed=4)
    res = {}
    for outer in (1, 3):
        rq = [sv.Request(rid=r.rid, protocol=r.protocol, data=r.data, cmaps=r.cmaps) for r in reqs]
        srv = sv.ReconServer(sv.GpuExecutor(mr, iters=10, precision="refined", outer=outer), 8 << 30, slots=2,
                             max_batch=2)
        srv.run(rq)
        srv.close()
        res[outer] = [r.resnorm for r in rq]
    assert all(np.isfinite(v) for v in res[1] + res[3])
    assert all(a3 < a1 for a1, a3 in zip(res[1], res[3]))


def test_server_tensor_core_precision(mr, cuda, sv):
    """fp16-tc serving: the 256^2 protocol runs the tensor-core operator and equals the direct
    API calls with it; the 32^2 protocol falls back to float32.  The direct calls rebuild the
    kernel and the backprojection, which are reproducible, so both agree bit for bit."""
    protos = []
    for i, (N, K, Nt) in enumerate(((256, 3, 24), (32, 3, 24))):
        trj = mr.trajectories.traj_2d_radial_goldenratio(2 * N, 2, Nt, thetaRot=0.2 * i)
        U = mr.synthetic.basis(mr.synthetic.dictionary(Nt, natoms=200, seed=i), K)
        protos.append(sv.Protocol(name=f"p{i}", img=(N, N), trj=mr.to_jl(trj, torch.float32),
                                  U=mr.to_jl(U, torch.float32), K=K))
    scans = [sv.make_scans(mr, p, 3, seed=20 + i) for i, p in enumerate(protos)]
    torch.cuda.synchronize()
    reqs = sv.make_request_stream(protos, scans, 4, rate_hz=0.0, coil_range=(2, 3), seed=5)
    iters = 6
    srv = sv.ReconServer(sv.GpuExecutor(mr, iters=iters, precision="fp16-tc"), 8 << 30, slots=2, max_batch=2)
    srv.run(reqs)
    srv.close()
    for r in reqs:
        p = r.protocol
        prec = "fp16-tc" if p.img[0] == 256 else "fp32"
        A = mr.NFFTNormalOp(p.img, p.trj, p.U, cmaps=r.cmaps, precision=prec)
        b = mr.calculate_backprojection(r.data, p.trj, r.cmaps, U=p.U)
        x = mr.to_host(mr.cg(A, b, maxiter=iters, reltol=0.0))
        np.testing.assert_array_equal(x, mr.to_host(r.x), err_msg=f"{r.rid} {prec}")


def test_cg_batch_relaxed_schedule(mr, cuda):
    """The relaxed batch (one recurrence, float32 products first) is the float32 CG when every
    product is float32 and the reduced-precision CG when none is, bit for bit (its accuracy
    against float64 is checked on a reconstruction below; on this random right-hand side the
    mixed schedules only have to stay near both)."""
    N, K, Nc, it = 256, 3, 2, 8
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 2, 24)
    rng = np.random.default_rng(7)
    U = np.linalg.svd(rand_c(rng, (24, K)), full_matrices=False)[0].real.astype(np.float32)
    cml = [rand_c(rng, (N, N)) for _ in range(Nc)]
    A32 = mr.NFFTNormalOp((N, N), trj, U, cmaps=cml)
    Atc = A32.share(cmaps=cml, precision="fp16-tc")
    b = mr.to_jl(rand_c(rng, (N, N, K)), torch.complex64)
    x32 = mr.to_host(mr.cg(A32, b, maxiter=it, reltol=0.0))
    xtc = mr.to_host(mr.cg(Atc, b, maxiter=it, reltol=0.0))
    out = {}
    for hi in (it, 0, 3):
        lo_op = A32.share(cmaps=cml, precision="fp16-tc")
        hi_op = A32.share(cmaps=cml)
        x = mr.jl_empty(b.shape, torch.complex64)
        bt = mr.CgBatch([lo_op], [b], [x], it, ops_hi=[hi_op], hi_iters=hi)
        bt.launch()
        n_it, rn = bt.result(0)
        assert n_it == it and np.isfinite(rn)
        out[hi] = mr.to_host(x)
        bt.close()
    np.testing.assert_array_equal(out[it], x32)
    np.testing.assert_array_equal(out[0], xtc)
    assert rel_l2(out[3], x32) < 1e-2 and rel_l2(out[3], xtc) < 1e-2
    with pytest.raises(ValueError):
        mr.CgBatch([Atc], [b], [mr.jl_empty(b.shape, torch.complex64)], it, hi_iters=2)


def test_server_relaxed_precision_equal_alone_and_within_float64_bar(mr, cuda, sv):
    """relaxed-tc serving: bit-identical alone and in a mix; the 256^2 protocol's image is
    within 1e-3 of the float64 oracle's CG on the same backprojection."""
    from oracle import cg as ocg
    from oracle import normalop as onormal
    protos = []
    for i, (N, K, Nt) in enumerate(((256, 3, 200), (32, 3, 24))):
        trj = mr.trajectories.traj_2d_radial_goldenratio(2 * N, 2, Nt, thetaRot=0.2 * i)
        U = mr.synthetic.basis(mr.synthetic.dictionary(Nt, natoms=200, seed=i), K)
        protos.append(sv.Protocol(name=f"p{i}", img=(N, N), trj=mr.to_jl(trj, torch.float32),
                                  U=mr.to_jl(U, torch.float32), K=K))
    scans = [sv.make_scans(mr, p, 4, seed=30 + i) for i, p in enumerate(protos)]
    torch.cuda.synchronize()
    iters = 20
    reqs = sv.make_request_stream(protos, scans, 5, rate_hz=0.0, coil_range=(3, 4), seed=6)
    srv = sv.ReconServer(sv.GpuExecutor(mr, iters=iters, precision="relaxed-tc"), 8 << 30, slots=2, max_batch=2)
    srv.run(reqs)
    srv.close()
    checked = False
    for r in reqs:
        alone = sv.Request(rid=r.rid, protocol=r.protocol, data=r.data, cmaps=r.cmaps, arrival=0.0)
        srv1 = sv.ReconServer(sv.GpuExecutor(mr, iters=iters, precision="relaxed-tc"), 8 << 30, slots=1,
                              max_batch=1)
        srv1.run([alone])
        srv1.close()
        np.testing.assert_array_equal(mr.to_host(alone.x), mr.to_host(r.x), err_msg=str(r.rid))
        p = r.protocol
        if p.img[0] != 256 or checked:
            continue
        checked = True
        trj, U = mr.to_host(p.trj), mr.to_host(p.U)
        cm = mr.to_host(r.cmaps)
        cml = [cm[..., c] for c in range(cm.shape[-1])]
        b = mr.to_host(mr.calculate_backprojection(r.data, p.trj, r.cmaps, U=p.U)).astype(np.complex128)
        G = tuple(2 * n for n in p.img)
        Lam, km = onormal.calculate_kernel_noncartesian(G, trj, U, fast=True)

        def apply(v):
            return onormal.nfft_normalop_apply(v.reshape(p.img + (p.K,), order="F"), Lam, km, p.img,
                                               cmaps=cml).ravel(order="F")

        x64, _, _ = ocg.cg(apply, b.ravel(order="F"), maxiter=iters, reltol=0.0)
        err = rel_l2(mr.to_host(r.x), x64.reshape(p.img + (p.K,), order="F"))
        print(f"served relaxed-tc 256^2 cg-20 vs float64: {err:.2e}")
        assert err < 1e-3
    assert checked
