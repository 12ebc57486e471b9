"""Python mirror of the reference's ``NFFTNormalOp`` / ``FFTNormalOp`` constructors.

Each constructor returns a :class:`NormalOperator`, the counterpart of the
``LinearOperator`` the reference builds (``src/NFFTNormalOp.jl:76-85``,
``ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:59-69``): square, Hermitian,
``mul(res, x, alpha, beta)`` is the reference's 5-argument ``prod!``, and
``A.prod.A.Λ`` / ``A.prod.A.kmask_indcs`` reach the kernel like the
reference tests' ``A.prod!.A.Λ`` (``test/reconstruct_cart_mask.jl:65``).
All work runs in ``libmrsr.so`` on the current CUDA device and stream.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .arrays import (is_complex_array, jl_empty, jl_reshape, mask_u8, ptr, stack_cmaps, stream_handle, to_jl)

_PREC = {"fp32": _lib.PREC_FP32, "fp16": _lib.PREC_FP16, "fp16-tc": _lib.PREC_FP16_TC}


def _prec(precision):
    if isinstance(precision, int):
        return precision
    return _PREC[precision]


class _Prod:
    """Callable ``prod`` with an ``A`` attribute, so ``op.prod.A.Λ`` works."""

    def __init__(self, op):
        self.A = op

    def __call__(self, res, x, alpha=1.0, beta=0.0):
        return self.A.mul(res, x, alpha, beta)


class NormalOperator:
    def __init__(self, handle):
        self._h = C.c_void_p(handle)
        info = (C.c_int64 * 12)()
        _lib.check(_lib.load().mrsr_normalop_info(self._h, info))
        (kind, ndims, n1, n2, n3, K, ncoils, nk, lc, prec, P, launches) = list(info)
        self.kind = int(kind)
        self.shape_img = (int(n1), int(n2)) if ndims == 2 else (int(n1), int(n2), int(n3))
        self.Ncoeff = int(K)
        self.ncoils = int(ncoils)
        self.nk = int(nk)
        self.lambda_is_complex = bool(lc)
        self.precision = int(prec)
        self.P = int(P)
        self.launches_per_apply = int(launches)
        n = int(np.prod(self.shape_img)) * self.Ncoeff
        self.shape = (n, n)
        self.dtype = torch.complex64
        self.symmetric = True
        self.hermitian = True
        self.prod = _Prod(self)

    # -- lifetime -------------------------------------------------------
    def close(self):
        if self._h is not None and self._h.value:
            _lib.load().mrsr_normalop_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- products -------------------------------------------------------
    def _as_image(self, v):
        shp = self.shape_img + (self.Ncoeff,)
        t = to_jl(v, torch.complex64)
        if tuple(t.shape) != shp:
            if t.numel() != int(np.prod(shp)):
                raise ValueError(f"vector of length {t.numel()} does not match operator size {self.shape[0]}")
            # a Julia vec(): column-major flatten
            flat = t.permute(*reversed(range(t.dim()))).reshape(-1) if t.dim() > 1 else t
            t = flat.reshape(shp[::-1]).permute(*reversed(range(len(shp))))
        return t

    def mul(self, res, x, alpha=1.0, beta=0.0, stream=None):
        """``mul!(res, A, x, alpha, beta)``: res <- beta*res + alpha*A*x (device tensors)."""
        xi = self._as_image(x)
        ri = self._as_image(res)
        if ri.data_ptr() != res.data_ptr() or not res.is_cuda:
            raise ValueError("res must be a column-major complex64 CUDA tensor")
        a = complex(alpha)
        b = complex(beta)
        _lib.check(_lib.load().mrsr_normalop_apply(self._h, ptr(xi), ptr(ri), a.real, a.imag, b.real, b.imag,
                                                  stream_handle(stream)))
        return res

    def mul_host(self, res, x, alpha=1.0, beta=0.0, stream=None):
        """``mul!(res, A, x, alpha, beta)`` on host arrays: res and x are complex64 CPU tensors
        holding the column-major (img..., K) data (a flat vector, or a column-major view).  x is
        copied to the device; with one coil group and res page-locked, the inverse row pass
        stores res straight into host memory (``mrsr_normalop_apply_host``), else res returns by
        a copy.  Enqueued on ``stream``; res is final once the stream has synchronised."""
        n = self.shape[0]
        for name, t in (("x", x), ("res", res)):
            if not isinstance(t, torch.Tensor) or t.is_cuda or t.dtype != torch.complex64 or t.numel() != n:
                raise ValueError(f"{name} must be a complex64 CPU tensor of {n} elements")
            if not t.permute(*reversed(range(t.dim()))).is_contiguous():
                raise ValueError(f"{name} must be dense (column-major (img..., K) data)")
        if x.data_ptr() == res.data_ptr():
            raise ValueError("x and res must not alias")
        a = complex(alpha)
        b = complex(beta)
        _lib.check(_lib.load().mrsr_normalop_apply_host(self._h, ptr(x), ptr(res), a.real, a.imag, b.real, b.imag,
                                                       stream_handle(stream)))
        return res

    def __matmul__(self, x):
        xi = self._as_image(x)
        out = jl_empty(xi.shape, torch.complex64)
        self.mul(out, xi, 1.0, 0.0)
        if isinstance(x, torch.Tensor) and x.dim() == 1:
            return out.permute(*reversed(range(out.dim()))).reshape(-1)
        return out

    __mul__ = __matmul__

    # -- kernel access (A.prod!.A.Λ / .kmask_indcs) ------------------------
    @property
    def kmask_indcs(self):
        out = torch.empty(self.nk, dtype=torch.int64, device="cuda")
        _lib.check(_lib.load().mrsr_normalop_get_kmask(self._h, ptr(out), stream_handle()))
        return out

    @property
    def Λ(self):
        if self.kind == _lib.KIND_FFT:
            out = jl_empty((self.Ncoeff, self.Ncoeff, self.nk), torch.complex64)
        else:
            dt = torch.complex64 if self.lambda_is_complex else torch.float32
            out = jl_empty((self.P, self.nk), dt)
        _lib.check(_lib.load().mrsr_normalop_get_lambda(self._h, ptr(out), stream_handle()))
        return out

    Lambda = Λ

    def share(self, cmaps=None, precision=None, stream=None):
        """A new operator on this operator's Toeplitz kernel and kmask (shared, not copied)
        with its own coil maps; ``precision`` defaults to this operator's."""
        S = stack_cmaps(cmaps)
        nc = 1 if S is None else int(S.shape[-1])
        prec = self.precision if precision is None else _prec(precision)
        op = _new_handle(_lib.load().mrsr_normalop_share, self._h, ptr(S), nc, prec, stream_handle(stream))
        op._cmaps_ref = S
        return op

    def stack(self, nrhs, stream=None):
        """An operator on ``nrhs`` stacked images (img..., nrhs) that applies this rank-1
        float32 operator to each plane independently (for :func:`cg_stacked`)."""
        op = _new_handle(_lib.load().mrsr_normalop_stack, self._h, int(nrhs), stream_handle(stream))
        op._stack_source = self
        return op

    def profile(self, x, y, iters=10, stream=None):
        """Per-pass device milliseconds of one apply (CUDA events between launches)."""
        xi, yi = self._as_image(x), self._as_image(y)
        ms = (C.c_float * self.launches_per_apply)()
        _lib.check(_lib.load().mrsr_normalop_profile(self._h, ptr(xi), ptr(yi), int(iters), ms,
                                                    stream_handle(stream)))
        return list(ms)

    def check(self, stream=None):
        """Synchronise and raise ``MrsrError`` if an apply since the last check hit a
        bounded device wait that gave up (its outputs are not valid); clears the flag.
        The CG solvers make the same check when they finish."""
        _lib.check(_lib.load().mrsr_normalop_check(self._h, stream_handle(stream)))


def _new_handle(fn, *args):
    h = C.c_void_p()
    _lib.check(fn(*args, C.byref(h)))
    return NormalOperator(h.value)


def _img(img_shape):
    img_shape = tuple(int(s) for s in img_shape)
    if len(img_shape) not in (2, 3):
        raise ValueError("img_shape must have 2 or 3 entries")
    return img_shape


def NFFTNormalOp(img_shape, trj_or_lambda, U_or_kmask, cmaps=None, sample_mask=None, precision="fp32",
                 stream=None):
    """``NFFTNormalOp(img_shape, trj, U; cmaps, sample_mask)`` or
    ``NFFTNormalOp(img_shape, Λ, kmask_indcs; cmaps)`` (packed GPU Λ).

    trj: (d, Ns, Nt) float32 in [-0.5, 0.5]; U: (Nt, K) real or complex.
    Λ: packed (K(K+1)/2, Nk) float32 or complex64; kmask_indcs: 1-based int64.
    """
    lib = _lib.load()
    img_shape = _img(img_shape)
    d = len(img_shape)
    S = stack_cmaps(cmaps, img_shape)
    nc = 1 if S is None else int(S.shape[-1])
    arr = trj_or_lambda
    is_traj = (getattr(arr, "ndim", None) or getattr(arr, "dim", lambda: 0)()) in (3, 4) and arr.shape[0] == d
    if is_traj:
        trj = to_jl(arr, torch.float32)
        if trj.dim() == 4:  # 4D wrapper (src/NFFTNormalOp.jl:45-49)
            trj = to_jl(trj.reshape(trj.shape[0], -1, trj.shape[3]), torch.float32)
            if isinstance(sample_mask, torch.Tensor):
                sample_mask = jl_reshape(mask_u8(sample_mask), (-1, sample_mask.shape[-1]))
            elif sample_mask is not None:
                sample_mask = np.asarray(sample_mask).reshape(-1, np.asarray(sample_mask).shape[-1], order="F")
        U = U_or_kmask
        ucplx = is_complex_array(U)
        Ut = to_jl(U, torch.complex64 if ucplx else torch.float32)
        K = int(Ut.shape[1])
        m = mask_u8(sample_mask)
        return _new_handle(lib.mrsr_nfft_normalop_create, d, _lib.int64_array(img_shape), int(trj.shape[1]),
                           int(trj.shape[2]), ptr(trj), ptr(m), ptr(Ut), int(ucplx), K, ptr(S), nc,
                           _prec(precision), stream_handle(stream))
    lam = arr
    lc = is_complex_array(lam)
    L = to_jl(lam, torch.complex64 if lc else torch.float32)
    P = int(L.shape[0])
    K = (int(np.sqrt(8 * P + 1)) - 1) // 2  # ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:33
    km = to_jl(np.asarray(U_or_kmask, dtype=np.int64) if not isinstance(U_or_kmask, torch.Tensor) else U_or_kmask,
               torch.int64)
    if km.numel() != L.shape[1]:
        raise AssertionError("AssertionError: length(kmask_indcs) == size(Λ, 2)")
    return _new_handle(lib.mrsr_nfft_normalop_from_lambda, d, _lib.int64_array(img_shape), K, ptr(L), int(lc),
                       ptr(km), int(km.numel()), ptr(S), nc, _prec(precision), stream_handle(stream))


def FFTNormalOp(*args, cmaps=None, sample_mask=None, precision="fp32", stream=None):
    """``FFTNormalOp(img_shape, trj::Integer, U; cmaps, sample_mask)``,
    ``FFTNormalOp(M, U; cmaps)`` or ``FFTNormalOp(Λ; cmaps)``."""
    lib = _lib.load()
    S = stack_cmaps(cmaps)
    nc = 1 if S is None else int(S.shape[-1])
    if len(args) == 1:
        lam = to_jl(args[0], torch.complex64)
        K = int(lam.shape[0])
        img_shape = _img(lam.shape[2:])
        return _new_handle(lib.mrsr_fft_normalop_from_lambda, len(img_shape), _lib.int64_array(img_shape), K,
                           ptr(lam), ptr(S), nc, _prec(precision), stream_handle(stream))
    if len(args) == 2:
        M, U = args
        Mt = to_jl(np.asarray(M, dtype=np.uint8) if not isinstance(M, torch.Tensor) else M.to(torch.uint8),
                   torch.uint8)
        img_shape = _img(Mt.shape[:-1])
        ucplx = is_complex_array(U)
        Ut = to_jl(U, torch.complex64 if ucplx else torch.float32)
        return _new_handle(lib.mrsr_fft_normalop_create_from_mask, len(img_shape), _lib.int64_array(img_shape),
                           int(Mt.shape[-1]), ptr(Mt), ptr(Ut), int(ucplx), int(Ut.shape[1]), ptr(S), nc,
                           _prec(precision), stream_handle(stream))
    img_shape, trj, U = args
    img_shape = _img(img_shape)
    t = to_jl(trj, torch.int32)
    ucplx = is_complex_array(U)
    Ut = to_jl(U, torch.complex64 if ucplx else torch.float32)
    nrep = int(Ut.shape[2]) if Ut.dim() == 3 else 1
    m = mask_u8(sample_mask)
    return _new_handle(lib.mrsr_fft_normalop_create, len(img_shape), _lib.int64_array(img_shape), int(t.shape[1]),
                       int(t.shape[2]), ptr(t), ptr(m), ptr(Ut), int(ucplx), int(Ut.shape[1]), nrep, ptr(S), nc,
                       _prec(precision), stream_handle(stream))
