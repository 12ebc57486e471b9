"""Solvers on a :class:`NormalOperator`, run on the device by ``libmrsr.so``.

``cg`` mirrors IterativeSolvers.jl 0.9 ``cg(A, b; maxiter, reltol, abstol)``
as the reference calls it (``test/reconstruct_radial.jl:83``, x0 = 0).
``cg_relaxed`` is the same CG with its operator products switched from the
float32 operator to a reduced-precision one once the residual is small, and
``cg_refined`` the restarted mixed-precision iterative refinement (inner CG on a
reduced-precision operator, outer residual with the float32 operator); neither
has a counterpart in the reference.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .arrays import jl_empty, ptr, stream_handle

DEFAULT_RELTOL = float(np.sqrt(np.finfo(np.float32).eps))


class CgResult:
    def __init__(self, x, iters, resnorm):
        self.x, self.iters, self.resnorm = x, iters, resnorm


def cg(A, b, maxiter=None, reltol=DEFAULT_RELTOL, abstol=0.0, log=False, stream=None):
    """``cg(A, vec(b); maxiter, reltol, abstol)``; returns x with b's shape
    (``log=True`` also returns iterations and the final residual norm)."""
    lib = _lib.load()
    bi = A._as_image(b)
    x = jl_empty(bi.shape, torch.complex64)
    if maxiter is None:
        maxiter = A.shape[1]  # IterativeSolvers default: size(A, 2)
    it = C.c_int(0)
    rn = C.c_double(0.0)
    _lib.check(lib.mrsr_cg(A.handle, ptr(bi), ptr(x), int(maxiter), float(reltol), float(abstol), C.byref(it),
                           C.byref(rn), stream_handle(stream)))
    out = x
    if isinstance(b, torch.Tensor) and b.dim() == 1:
        out = x.permute(*reversed(range(x.dim()))).reshape(-1)
    if log:
        return CgResult(out, it.value, rn.value)
    return out


def cg_stacked(A, b, maxiter=None, reltol=DEFAULT_RELTOL, abstol=0.0, log=False, stream=None):
    """One ``cg(A1, b[..., i]; maxiter, reltol, abstol)`` per plane i of ``b`` (img..., nrhs),
    where ``A = A1.stack(nrhs)``; the solves run together (one launch per step for all
    planes) but each keeps its own iteration.  ``log=True`` also returns per-plane
    iteration counts and residual norms (lists)."""
    lib = _lib.load()
    bi = A._as_image(b)
    x = jl_empty(bi.shape, torch.complex64)
    nrhs = A.Ncoeff
    if maxiter is None:
        maxiter = int(np.prod(A.shape_img))  # size(A1, 2) of the rank-1 operator
    its = (C.c_int * nrhs)()
    rns = (C.c_double * nrhs)()
    _lib.check(lib.mrsr_cg_stacked(A.handle, ptr(bi), ptr(x), int(maxiter), float(reltol), float(abstol), its, rns,
                                   stream_handle(stream)))
    if log:
        return CgResult(x, list(its), list(rns))
    return x


class RelaxedResult(CgResult):
    def __init__(self, x, iters, hi_iters, resnorm):
        super().__init__(x, iters, resnorm)
        self.hi_iters = hi_iters


def cg_relaxed(A_lo, A_hi, b, maxiter=None, reltol=DEFAULT_RELTOL, abstol=0.0, switch=0.05, log=False, stream=None):
    """``cg(A, vec(b); maxiter, reltol, abstol)`` with the products on the float32 ``A_hi``
    while ||r|| > switch ||b|| and on the reduced-precision ``A_lo`` after that (one
    recurrence, no restart).  ``log=True`` also returns the iterations, how many of them
    ran on ``A_hi``, and the final residual norm."""
    lib = _lib.load()
    bi = A_hi._as_image(b)
    x = jl_empty(bi.shape, torch.complex64)
    if maxiter is None:
        maxiter = A_hi.shape[1]
    it = C.c_int(0)
    hi = C.c_int(0)
    rn = C.c_double(0.0)
    _lib.check(lib.mrsr_cg_relaxed(A_lo.handle, A_hi.handle, ptr(bi), ptr(x), int(maxiter), float(reltol),
                                   float(abstol), float(switch), C.byref(it), C.byref(hi), C.byref(rn),
                                   stream_handle(stream)))
    out = x
    if isinstance(b, torch.Tensor) and b.dim() == 1:
        out = x.permute(*reversed(range(x.dim()))).reshape(-1)
    if log:
        return RelaxedResult(out, it.value, hi.value, rn.value)
    return out


def cg_refined(A_lo, A_hi, b, inner_iters=20, max_outer=10, tol=1e-4, log=False, stream=None):
    """Mixed-precision iterative refinement: x <- x + CG_lo(b - A_hi x) until
    ||b - A_hi x|| <= tol ||b|| (A_lo a reduced-precision operator, A_hi float32),
    or until a step more than doubles that residual (the step is undone)."""
    lib = _lib.load()
    bi = A_hi._as_image(b)
    x = jl_empty(bi.shape, torch.complex64)
    outer = C.c_int(0)
    rel = C.c_double(0.0)
    _lib.check(lib.mrsr_cg_refined(A_lo.handle, A_hi.handle, ptr(bi), ptr(x), int(inner_iters), int(max_outer),
                                   float(tol), C.byref(outer), C.byref(rel), stream_handle(stream)))
    if log:
        return CgResult(x, outer.value, rel.value)
    return x


class CgBatch:
    """Fixed-iteration solves of independent systems recorded into one CUDA graph.

    Entry i solves ``ops[i] x[i] = b[i]`` with ``cg(A, b; maxiter=iters,
    reltol=0)`` from x0 = 0, or, when ``ops_hi`` is given, by mixed-precision
    refinement with ``outer`` fixed steps (inner CG on ``ops[i]``, residual with
    ``ops_hi[i]``), or, when ``ops_hi`` and ``hi_iters`` are given, by the relaxed
    schedule (one CG recurrence, the first ``hi_iters`` products on ``ops_hi[i]``,
    the rest on ``ops[i]``; the fixed-schedule form of :func:`cg_relaxed`).  Each
    entry is a branch of the graph, so the solves overlap on the device;
    :meth:`launch` re-solves with the current contents of the ``b`` tensors
    (their storage is baked into the graph).
    """

    def __init__(self, ops, bs, xs, iters, ops_hi=None, outer=1, stream=None, hi_iters=None):
        lib = _lib.load()
        n = len(ops)
        if not (len(bs) == len(xs) == n) or n == 0:
            raise ValueError("ops, bs and xs must have the same nonzero length")
        self._ops, self._ops_hi = list(ops), (list(ops_hi) if ops_hi is not None else None)
        self._b = [ops[i]._as_image(bs[i]) for i in range(n)]
        self._x = [ops[i]._as_image(xs[i]) for i in range(n)]
        for i in range(n):
            if self._b[i].data_ptr() != bs[i].data_ptr() or self._x[i].data_ptr() != xs[i].data_ptr():
                raise ValueError("b and x must be column-major complex64 CUDA tensors of the operator's size")
        P = C.c_void_p * n
        lo = P(*[o.handle.value for o in ops])
        hi = P(*[o.handle.value for o in ops_hi]) if ops_hi is not None else None
        bp = P(*[t.data_ptr() for t in self._b])
        xp = P(*[t.data_ptr() for t in self._x])
        h = C.c_void_p()
        if hi_iters is not None:
            if hi is None:
                raise ValueError("the relaxed schedule needs ops_hi")
            _lib.check(lib.mrsr_cg_batch_create_relaxed(lo, hi, bp, xp, n, int(iters), int(hi_iters),
                                                        stream_handle(stream), C.byref(h)))
        else:
            _lib.check(lib.mrsr_cg_batch_create(lo, hi, bp, xp, n, int(iters), int(outer), stream_handle(stream),
                                                C.byref(h)))
        self._h = h
        self.n = n

    def launch(self, stream=None):
        _lib.check(_lib.load().mrsr_cg_batch_launch(self._h, stream_handle(stream)))

    def result(self, i):
        """(iterations or outer steps, residual norm) of entry i; waits for the last launch."""
        it = C.c_int(0)
        rn = C.c_double(0.0)
        _lib.check(_lib.load().mrsr_cg_batch_result(self._h, int(i), C.byref(it), C.byref(rn)))
        return it.value, rn.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().mrsr_cg_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
