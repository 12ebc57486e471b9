"""Scheduling logic of the reconstruction server, on the CPU with a simulated executor.

The executor models device work by a duration per batch on a simulated
clock; the tests check continuous admission, same-protocol batching, the
HBM budget (admission and kernel eviction), the kernel cache and that every
request completes.
"""
import importlib
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def sv(mr):
    return importlib.import_module(mr.__name__ + ".serving")


class SimClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def tick(self, dt=1e-4):
        self.t += dt


class SimExecutor:
    """Batches take `per_req` seconds per request (run in parallel branches: max, not sum)."""

    def __init__(self, clock, per_req=2e-3, req_bytes=100, kern_bytes=1000):
        self.clock = clock
        self.per_req = per_req
        self.req_bytes = req_bytes
        self.kern_bytes = kern_bytes
        self.built, self.dropped, self.batches = [], [], []
        self.live = 0
        self.max_live = 0

    def kernel_bytes(self, proto):
        return self.kern_bytes

    def request_bytes(self, r):
        return self.req_bytes * r.ncoils

    def build_kernel(self, proto, si):
        self.built.append(proto.key)
        return ("kernel", proto.key)

    def drop_kernel(self, kern):
        self.dropped.append(kern[1])

    def start(self, si, batch, kern):
        assert kern == ("kernel", batch[0].protocol.key)
        self.batches.append([r.rid for r in batch])
        self.live += 1
        self.max_live = max(self.max_live, self.live)
        return {"end": self.clock() + self.per_req * (1 + 0.25 * (len(batch) - 1))}

    def poll(self, h):
        return self.clock() >= h["end"]

    def finish(self, h, batch):
        self.live -= 1
        for r in batch:
            r.x = r.rid


class _Cm:
    def __init__(self, nc):
        self.shape = (4, 4, nc)


def _protocols(sv, n):
    return [sv.Protocol(name=f"p{i}", img=(16, 16), trj=None, U=None, K=3, key=f"key{i}") for i in range(n)]


def _requests(sv, protos, n, rate, seed=0, nc=4):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        out.append(sv.Request(rid=i, protocol=protos[int(rng.integers(len(protos)))], data=None, cmaps=_Cm(nc),
                              arrival=t))
    return out


def _server(sv, ex, clk, budget, slots=3, max_batch=4):
    return sv.ReconServer(ex, budget, slots=slots, max_batch=max_batch, clock=clk, idle=clk.tick)


def test_all_requests_complete_with_continuous_admission(sv):
    clk = SimClock()
    ex = SimExecutor(clk)
    protos = _protocols(sv, 3)
    reqs = _requests(sv, protos, 60, rate=800.0)
    st = _server(sv, ex, clk, budget=10 ** 9).run(reqs)
    assert st.completed == 60
    assert all(r.x == r.rid for r in reqs)
    assert all(r.t_start >= r.arrival - 1e-12 and r.t_done > r.t_start for r in reqs)
    assert ex.max_live <= 3
    assert sum(len(b) for b in ex.batches) == 60
    # every batch is one protocol, at most max_batch requests
    by_id = {r.rid: r for r in reqs}
    for b in ex.batches:
        assert len(b) <= 4
        assert len({by_id[i].protocol.key for i in b}) == 1
    assert st.max_batch_seen > 1  # the arrival rate exceeds one slot's service rate: batching happens
    assert st.kernel_builds == 3  # one kernel per protocol, cached afterwards
    assert st.p99_ms >= st.p50_ms > 0


def test_head_of_queue_is_always_in_the_started_batch(sv):
    clk = SimClock()
    ex = SimExecutor(clk)
    protos = _protocols(sv, 4)
    reqs = _requests(sv, protos, 40, rate=2000.0, seed=3)
    _server(sv, ex, clk, budget=10 ** 9, slots=2).run(reqs)
    by_id = {r.rid: r for r in reqs}
    started = set()
    for b in ex.batches:
        waiting = [r for r in reqs if r.rid not in started and r.arrival <= by_id[b[0]].t_start]
        assert b[0] == min(r.rid for r in waiting)  # FIFO head leads every batch
        started.update(b)


def test_budget_limits_admission_and_evicts_idle_kernels(sv):
    clk = SimClock()
    ex = SimExecutor(clk, req_bytes=100, kern_bytes=1000)
    protos = _protocols(sv, 5)
    reqs = _requests(sv, protos, 50, rate=1000.0, seed=5, nc=4)   # 400 bytes per request
    budget = 2 * 1000 + 2 * 400                                     # two kernels and two requests
    srv = _server(sv, ex, clk, budget=budget, slots=4, max_batch=4)
    st = srv.run(reqs)
    assert st.completed == 50
    assert st.peak_reserved_bytes <= budget
    assert st.evictions > 0 and len(ex.dropped) == st.evictions
    assert st.kernel_builds > 5  # protocols come back after eviction
    srv.close()
    assert len(ex.dropped) == len(ex.built)


def test_request_larger_than_budget_raises(sv):
    clk = SimClock()
    ex = SimExecutor(clk, req_bytes=1000, kern_bytes=10)
    reqs = _requests(sv, _protocols(sv, 1), 2, rate=100.0, nc=8)
    with pytest.raises(MemoryError):
        _server(sv, ex, clk, budget=5000).run(reqs)


def test_request_bytes_and_kernel_bytes_scale(sv):
    a = sv.request_bytes((128, 128), 4, 8)
    b = sv.request_bytes((256, 256), 4, 8)
    c = sv.request_bytes((256, 256), 4, 32)
    assert 3 * a < b < c
    assert sv.request_bytes((256, 256), 4, 8, "fp16") < b
    assert sv.request_bytes((256, 256), 4, 8, "fp16", refine=True) > sv.request_bytes((256, 256), 4, 8, "fp16")
    assert sv.kernel_bytes((256, 256), 5) < sv.kernel_bytes((256, 256), 5, fp16=True)
    assert sv.kernel_bytes((256, 256), 5) < sv.kernel_bytes((256, 256), 5, complex_kernel=True)


def test_protocol_key_depends_on_trajectory_basis_and_size(sv):
    rng = np.random.default_rng(0)
    trj = rng.standard_normal((2, 8, 5)).astype(np.float32)
    U = rng.standard_normal((5, 2)).astype(np.float32)
    k = sv.protocol_key(trj, U, (8, 8))
    assert k == sv.protocol_key(trj.copy(), U.copy(), (8, 8))
    trj2 = trj.copy()
    trj2[0, 0, 0] += 1e-6
    assert k != sv.protocol_key(trj2, U, (8, 8))
    assert k != sv.protocol_key(trj, U, (8, 16))
    assert k != sv.protocol_key(trj, U * 2, (8, 8))
    assert not math.isnan(sv.Request(rid=0, protocol=None, data=None, cmaps=_Cm(3), arrival=1.0).arrival)


def test_tensor_core_sizes_and_bytes(sv, mr):
    assert sv.tc_grid((256, 256)) and sv.tc_grid((256, 64, 256))
    assert not sv.tc_grid((128, 128)) and not sv.tc_grid((256, 128))
    assert sv.kernel_bytes((256, 256), 5, tc=True) > sv.kernel_bytes((256, 256), 5)
    with pytest.raises(ValueError):
        sv.GpuExecutor(mr, precision="bf16")
    assert set(sv.GpuExecutor.PRECISIONS) >= {"fp16-tc", "refined-tc"}
