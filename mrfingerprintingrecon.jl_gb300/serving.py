"""Continuous-batching reconstruction server on one GPU.

A request is one subspace reconstruction: the k-space data of one scan
``(ns_per_frame, Nt, Nc)``, its coil maps ``(img..., Nc)`` and its protocol --
the trajectory and temporal basis the scan was acquired with (matrix size,
Nt, K, trajectory).  Scans of one protocol share the Toeplitz kernel Λ and
its kmask; they differ in coils and data.

The server

* keeps every protocol's kernel device-resident, cached by a hash of the
  trajectory, basis and matrix size (:class:`KernelCache`);
* admits queued requests into free slots while the HBM budget allows,
  evicting idle cached kernels first; a request that does not fit waits, and
  requests behind it wait with it (arrival order is kept);
* groups queued requests of the same protocol into one batch of up to
  ``max_batch``: their backprojections run on the slot's stream, then one
  CUDA-graph launch runs all their CG solves as parallel graph branches
  (``CgBatch``: fixed iteration count, graph-captured iterations);
* runs up to ``slots`` batches at once on separate CUDA streams, so work
  admitted while other batches are on the GPU overlaps theirs;
* records arrival, start and completion times of every request and reports
  throughput and latency percentiles.

Each request's arithmetic depends only on its own inputs (its own operator,
work vectors and CG state; fixed-order reductions; backprojection grids summed in
64-bit fixed point), so its image is bit-identical alone and in any mix.

The scheduling core (:class:`ReconServer`) is separate from the device work
(:class:`GpuExecutor`) so that admission, batching and eviction can be tested
on the CPU with a simulated executor.
"""
from __future__ import annotations

import collections
import dataclasses
import hashlib
import math
import time
from typing import Any, Dict, List, Optional

import numpy as np


# ---------------------------------------------------------------- data ---
@dataclasses.dataclass
class Protocol:
    """Trajectory + basis + matrix size shared by many scans."""
    name: str
    img: tuple
    trj: Any            # (d, ns_per_frame, Nt) float32, device
    U: Any              # (Nt, K) float32 or complex64, device
    K: int
    key: str = ""

    def __post_init__(self):
        if not self.key:
            self.key = protocol_key(self.trj, self.U, self.img)


@dataclasses.dataclass
class Request:
    rid: int
    protocol: Protocol
    data: Any           # (ns_per_frame, Nt, Nc) complex64, device
    cmaps: Any          # (img..., Nc) complex64, device
    arrival: float = 0.0  # seconds after the start of the stream
    # filled in by the server
    t_start: float = math.nan
    t_done: float = math.nan
    batch_size: int = 0
    x: Any = None
    resnorm: float = math.nan

    @property
    def ncoils(self):
        return int(self.cmaps.shape[-1])

    @property
    def latency(self):
        return self.t_done - self.arrival


def protocol_key(trj, U, img):
    """Hash of the trajectory, the basis and the matrix size (the inputs of Λ and kmask)."""
    h = hashlib.sha1()
    for a in (trj, U):
        arr = a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
        h.update(str(arr.dtype).encode())
        h.update(str(arr.shape).encode())
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(str(tuple(img)).encode())
    return h.hexdigest()


# ------------------------------------------------------------- memory ---
def _prod(t):
    return int(np.prod([int(v) for v in t]))


def tc_grid(img):
    """The tensor-core operator needs 512-point lines along dims 1 and the last one."""
    return len(img) in (2, 3) and 2 * img[0] == 512 and 2 * img[-1] == 512


def kernel_bytes(img, K, nk=None, complex_kernel=False, fp16=False, tc=False):
    """Device bytes of one cached kernel: Λ over the 2x grid (+ fp16 copy, + the tensor-core
    layout) and the kmask."""
    G = _prod(2 * int(n) for n in img)
    P = K * (K + 1) // 2
    lam = P * G * (8 if complex_kernel else 4)
    half = P * G * (4 if complex_kernel else 2) if fp16 else 0
    tcl = lam + 36864 if tc else 0  # rearranged copy + DFT-64 operand and twiddles
    nk = G if nk is None else nk
    base_stack = K * 2 * _prod(img) * 8  # the cache's own one-coil operator
    return lam + half + tcl + 8 * nk + base_stack


def request_bytes(img, K, nc, precision="fp32", refine=False):
    """Device bytes one admitted request holds while it runs (estimate, rounded up)."""
    img = tuple(int(v) for v in img)
    nimg = _prod(img)
    G = _prod(2 * n for n in img)
    vec = nimg * K * 8
    esz = 4 if precision == "fp16" else 8
    per_coil = K * 2 * img[0] * _prod(img[1:]) * esz
    cg = min(nc, max(1, (112 << 20) // per_coil)) if len(img) == 2 else 1
    stacks = per_coil * cg
    if len(img) == 3:
        stacks += K * 4 * img[0] * img[1] * img[2] * esz * cg
    ops = stacks + nimg * nc * 8
    if refine:
        ops *= 2
    # backprojection: float2 grid plus its 64-bit fixed-point accumulator (re, im) per coil batch
    bp_grid = 3 * K * G * 8 * min(nc, max(1, (2 << 30) // (K * G * 8)))
    cgwork = 3 * vec + 32 * 1024
    return int(1.1 * (ops + bp_grid + cgwork + 2 * vec + (2 * vec if refine else 0))) + (1 << 20)


class KernelCache:
    """Protocol kernels by key, least recently used first; entries in use are never evicted."""

    def __init__(self):
        self.entries: "collections.OrderedDict[str, list]" = collections.OrderedDict()  # key -> [kernel, bytes, users]

    def bytes(self):
        return sum(e[1] for e in self.entries.values())

    def get(self, key):
        e = self.entries.get(key)
        if e is not None:
            self.entries.move_to_end(key)
        return e

    def put(self, key, kernel, nbytes):
        self.entries[key] = [kernel, nbytes, 0]

    def acquire(self, key):
        self.entries[key][2] += 1

    def release(self, key):
        self.entries[key][2] -= 1

    def evict_idle(self, need, drop):
        """Drop idle entries, least recently used first, until `need` bytes are freed; returns the bytes freed."""
        freed = 0
        for key in list(self.entries):
            if freed >= need:
                break
            kern, nb, users = self.entries[key]
            if users == 0:
                del self.entries[key]
                drop(kern)
                freed += nb
        return freed


# --------------------------------------------------------- scheduling ---
@dataclasses.dataclass
class ServeStats:
    completed: int
    wall_s: float
    recons_per_s: float
    p50_ms: float
    p99_ms: float
    mean_ms: float
    max_batch_seen: int
    kernel_builds: int
    evictions: int
    peak_reserved_bytes: int

    def as_dict(self):
        return dataclasses.asdict(self)


class ReconServer:
    """Continuous batching over ``slots`` concurrent batches under an HBM budget."""

    def __init__(self, executor, hbm_budget_bytes, slots=4, max_batch=4, clock=None, idle=None):
        if slots < 1 or max_batch < 1:
            raise ValueError("slots and max_batch must be >= 1")
        self.ex = executor
        self.budget = int(hbm_budget_bytes)
        self.slots: List[Optional[dict]] = [None] * slots
        self.max_batch = max_batch
        self.cache = KernelCache()
        self.reserved = 0           # bytes held by running batches
        self.peak = 0
        self.kernel_builds = 0
        self.evictions = 0
        self.clock = clock or time.perf_counter
        self.idle = idle or (lambda: time.sleep(50e-6))

    # -- memory -----------------------------------------------------------
    def _used(self):
        return self.reserved + self.cache.bytes()

    def _make_room(self, need):
        over = self._used() + need - self.budget
        if over > 0:
            n0 = len(self.cache.entries)
            self.cache.evict_idle(over, self.ex.drop_kernel)
            self.evictions += n0 - len(self.cache.entries)
        return self._used() + need <= self.budget

    # -- admission --------------------------------------------------------
    def _pick_batch(self, queue):
        head = queue[0]
        batch = [head]
        for r in queue[1:]:
            if len(batch) >= self.max_batch:
                break
            if r.protocol.key == head.protocol.key:
                batch.append(r)
        return batch

    def _admit(self, queue, now):
        started = False
        for si in range(len(self.slots)):
            if self.slots[si] is not None or not queue:
                continue
            batch = self._pick_batch(queue)
            proto = batch[0].protocol
            cached = self.cache.get(proto.key)
            if cached is not None:
                self.cache.acquire(proto.key)  # pinned: room is never made by evicting it
            kb = 0 if cached is not None else self.ex.kernel_bytes(proto)
            # shrink the batch until it fits (a single request that cannot fit waits)
            while batch:
                need = kb + sum(self.ex.request_bytes(r) for r in batch)
                if self._make_room(need):
                    break
                batch.pop()
            if not batch:
                if cached is not None:
                    self.cache.release(proto.key)
                if not any(self.slots):
                    req = queue[0]
                    raise MemoryError(f"request {req.rid} needs more than the HBM budget of {self.budget} bytes")
                return started
            if cached is None:
                kern = self.ex.build_kernel(proto, si)
                self.kernel_builds += 1
                self.cache.put(proto.key, kern, self.ex.kernel_bytes(proto))
                self.cache.acquire(proto.key)
            for r in batch:
                queue.remove(r)
                r.t_start = now
                r.batch_size = len(batch)
            rb = sum(self.ex.request_bytes(r) for r in batch)
            self.reserved += rb
            self.peak = max(self.peak, self._used())
            handle = self.ex.start(si, batch, self.cache.get(proto.key)[0])
            self.slots[si] = {"batch": batch, "handle": handle, "bytes": rb, "key": proto.key}
            started = True
        return started

    def _reap(self, now_fn):
        done = False
        for si, s in enumerate(self.slots):
            if s is None or not self.ex.poll(s["handle"]):
                continue
            t = now_fn()
            self.ex.finish(s["handle"], s["batch"])
            for r in s["batch"]:
                r.t_done = t
            self.reserved -= s["bytes"]
            self.cache.release(s["key"])
            self.slots[si] = None
            done = True
        return done

    def run(self, requests):
        """Serve `requests` (arrival times relative to the call); returns ServeStats."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue: List[Request] = []
        finished: List[Request] = []
        t0 = self.clock()
        now = lambda: self.clock() - t0  # noqa: E731
        max_batch_seen = 0
        total = len(pending)
        while len(finished) < total:
            t = now()
            while pending and pending[0].arrival <= t:
                queue.append(pending.popleft())
            progressed = self._reap(now)
            if progressed:
                finished = [r for r in requests if not math.isnan(r.t_done)]
            if queue:
                progressed |= self._admit(queue, now())
                max_batch_seen = max([max_batch_seen] + [len(s["batch"]) for s in self.slots if s])
            if not progressed:
                self.idle()
        wall = max(r.t_done for r in requests) if requests else 0.0
        lat = np.array([r.latency for r in requests]) * 1e3 if requests else np.zeros(1)
        return ServeStats(completed=total, wall_s=wall, recons_per_s=total / wall if wall > 0 else 0.0,
                          p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                          mean_ms=float(lat.mean()), max_batch_seen=max_batch_seen,
                          kernel_builds=self.kernel_builds, evictions=self.evictions,
                          peak_reserved_bytes=self.peak)

    def close(self):
        for e in list(self.cache.entries.values()):
            self.ex.drop_kernel(e[0])
        self.cache.entries.clear()


# ------------------------------------------------------ device executor ---
# grid lengths with register four-step FFT kernels (the fp16-storage operator needs them)
FOUR_STEP_LENGTHS = (64, 128, 256, 384, 512, 768, 1024)


class GpuExecutor:
    """Device work of the server: kernels, backprojections and graph-captured CG batches.

    ``precision``: "fp32" (cg on the float32 operator), "fp16" (cg on the
    fp16-storage operator), "refined" (fp16 inner CG with ``outer`` float32
    residual corrections, all inside one graph), "fp16-tc" / "refined-tc" (the
    same with the tensor-core operator), "relaxed-tc" (one CG recurrence whose
    first ``relaxed_hi`` products use the float32 operator and the rest the
    tensor-core one: the fixed-schedule relaxed CG, within 1e-3 of float64).
    Matrix sizes without the reduced form (fp16: a four-step 2x grid; fp16-tc:
    512-point lines, i.e. 256 samples along dims 1 and last) run the float32
    operator in every mode.
    """
    PRECISIONS = ("fp32", "fp16", "refined", "fp16-tc", "refined-tc", "relaxed-tc")

    def __init__(self, mr, iters=20, precision="fp32", outer=2, keep_results=True, relaxed_hi=5):
        import torch
        if precision not in self.PRECISIONS:
            raise ValueError("precision must be one of " + ", ".join(self.PRECISIONS))
        self.mr = mr
        self.torch = torch
        self.iters = iters
        self.precision = precision
        self.outer = outer
        self.relaxed_hi = relaxed_hi
        self.keep_results = keep_results
        self.streams: Dict[int, Any] = {}

    def _stream(self, si):
        if si not in self.streams:
            self.streams[si] = self.torch.cuda.Stream()
        return self.streams[si]

    def _tc(self):
        return self.precision in ("fp16-tc", "refined-tc", "relaxed-tc")

    def kernel_bytes(self, proto):
        return kernel_bytes(proto.img, proto.K, complex_kernel=self.torch.is_complex(proto.U),
                            fp16=self.precision in ("fp16", "refined"), tc=self._tc() and tc_grid(proto.img))

    def request_bytes(self, r):
        return request_bytes(r.protocol.img, r.protocol.K, r.ncoils,
                             "fp16" if self.precision in ("fp16", "refined") else "fp32",
                             refine=self.precision in ("refined", "refined-tc", "relaxed-tc"))

    def build_kernel(self, proto, si):
        s = self._stream(si)
        with self.torch.cuda.stream(s):
            return self.mr.NFFTNormalOp(proto.img, proto.trj, proto.U, stream=s)

    def drop_kernel(self, kern):
        kern.close()

    def start(self, si, batch, kern):
        torch, mr = self.torch, self.mr
        s = self._stream(si)
        # the reduced forms exist for some matrix sizes only; the others run float32
        img = batch[0].protocol.img
        if self._tc():
            mixed, lo_prec = tc_grid(img), "fp16-tc"
        else:
            mixed, lo_prec = self.precision != "fp32" and all(2 * n in FOUR_STEP_LENGTHS for n in img), "fp16"
        lo_prec = lo_prec if mixed else "fp32"
        refined = mixed and self.precision in ("refined", "refined-tc")
        relaxed = mixed and self.precision == "relaxed-tc"
        with torch.cuda.stream(s):
            ops, ops_hi, bs, xs = [], [], [], []
            for r in batch:
                p = r.protocol
                if not r.data.is_cuda:  # scanner data in (pinned) host memory: copy on the slot's stream
                    d = mr.jl_empty(r.data.shape, torch.complex64)
                    d.copy_(r.data, non_blocking=True)
                    r.data = d
                ops.append(kern.share(cmaps=r.cmaps, precision=lo_prec, stream=s))
                if refined or relaxed:
                    ops_hi.append(kern.share(cmaps=r.cmaps, precision="fp32", stream=s))
                bs.append(mr.calculate_backprojection(r.data, p.trj, r.cmaps, U=p.U, stream=s))
                xs.append(mr.jl_empty(bs[-1].shape, torch.complex64))
            cgb = mr.CgBatch(ops, bs, xs, self.iters, ops_hi=ops_hi or None, outer=self.outer, stream=s,
                             hi_iters=min(self.relaxed_hi, self.iters) if relaxed else None)
            cgb.launch(stream=s)
            ev = torch.cuda.Event()
            ev.record(s)
        return {"ev": ev, "ops": ops + ops_hi, "bs": bs, "xs": xs, "cgb": cgb}

    def poll(self, h):
        return h["ev"].query()

    def finish(self, h, batch):
        for i, r in enumerate(batch):
            _, r.resnorm = h["cgb"].result(i)
            r.x = h["xs"][i] if self.keep_results else None
        h["cgb"].close()
        for op in h["ops"]:
            op.close()
        h.clear()


# -------------------------------------------------------- request stream ---
SERVE_MATRICES = (128, 192, 256, 384)


def make_protocols(mr, n=8, seed=42, matrices=SERVE_MATRICES, K_range=(3, 6), Nt_range=(300, 1500),
                   spokes_per_frame=1):
    """`n` protocols from seeded draws: matrix size, K, Nt and a trajectory rotation per seed.

    The trajectory is the golden-ratio radial one (2x oversampled readout of
    2N samples, ``spokes_per_frame`` spokes per frame) rotated by a seeded
    angle; the basis is the top-K SVD of the synthetic dictionary for Nt frames.
    """
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(rng.choice(matrices))
        K = int(rng.integers(K_range[0], K_range[1] + 1))
        Nt = int(rng.integers(Nt_range[0], Nt_range[1] + 1))
        rot = float(rng.uniform(0, np.pi))
        trj = mr.trajectories.traj_2d_radial_goldenratio(2 * N, spokes_per_frame, Nt, thetaRot=rot)
        D = mr.synthetic.dictionary(Nt, seed=seed + i)
        U = mr.synthetic.basis(D, K)
        out.append(Protocol(name=f"p{i}_N{N}_K{K}_Nt{Nt}", img=(N, N),
                            trj=mr.to_jl(trj, torch.float32), U=mr.to_jl(U, torch.float32), K=K))
    return out


def make_scans(mr, proto, max_coils, seed=0, noise=0.01):
    """One synthetic scan of a protocol with `max_coils` coils: (data, cmaps, phantom x).

    Requests take the first Nc coils of it (data and maps are contiguous in
    the coil dimension)."""
    import torch
    N = proto.img
    Uh = mr.to_host(proto.U)
    D = mr.synthetic.dictionary(Uh.shape[0], seed=seed)
    x = mr.synthetic.phantom(N, D, Uh, seed=seed)
    cm = mr.synthetic.coil_maps(N, max_coils, seed=seed)
    cmt = mr.to_jl(cm, torch.complex64)
    xt = mr.to_jl(x, torch.complex64)
    data = mr.forward_model(xt, proto.trj, proto.U, cmaps=cmt)
    data = mr.synthetic.add_noise(data, noise, seed=seed)
    return data, cmt, xt


def make_request_stream(protocols, scans, n_requests, rate_hz, coil_range=(8, 32), seed=7):
    """Poisson arrivals at `rate_hz`; each request draws a protocol and a coil count."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += float(rng.exponential(1.0 / rate_hz)) if rate_hz > 0 else 0.0
        p = int(rng.integers(len(protocols)))
        data, cm = scans[p][0], scans[p][1]
        nc = int(rng.integers(coil_range[0], min(coil_range[1], cm.shape[-1]) + 1))
        reqs.append(Request(rid=i, protocol=protocols[p], data=data[..., :nc], cmaps=cm[..., :nc], arrival=t))
    return reqs
