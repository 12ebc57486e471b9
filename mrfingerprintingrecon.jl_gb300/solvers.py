"""Solvers on a :class:`NormalOperator`, run on the device by ``libmrsr.so``.

``cg`` mirrors IterativeSolvers.jl 0.9 ``cg(A, b; maxiter, reltol, abstol)``
as the reference calls it (``test/reconstruct_radial.jl:83``, x0 = 0).
``cg_refined`` is the mixed-precision iterative refinement (no counterpart in
the reference): inner CG on an fp16-storage operator, outer residual with the
float32 operator.
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


def cg_refined(A_lo, A_hi, b, inner_iters=20, max_outer=10, tol=1e-4, log=False, stream=None):
    """Mixed-precision iterative refinement: x <- x + CG_lo(b - A_hi x) until
    ||b - A_hi x|| <= tol ||b|| (A_lo the fp16-storage operator, A_hi float32)."""
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
