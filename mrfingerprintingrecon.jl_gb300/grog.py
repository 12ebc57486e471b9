"""Python mirror of ``grog_calib``, ``grog_gridding!`` and ``radial_grog!``
(src/GROG.jl), backed by ``libmrsr.so``."""
import numpy as np
import torch

from . import _lib
from .arrays import jl_empty, ptr, stream_handle, to_jl


def _data4(data):
    d = to_jl(data, torch.complex64)
    nrep = int(d.shape[3]) if d.dim() == 4 else 1
    return d, nrep


def grog_calib(data, trj, Nr, stream=None):
    """``grog_calib(data, trj, Nr)``: list of Nd ComplexF32 (Nc, Nc) device matrices lnG[d]."""
    lib = _lib.load()
    d, nrep = _data4(data)
    t = to_jl(trj, torch.float32)
    Nd = int(t.shape[0])
    ns, nt, nc = int(d.shape[0]), int(d.shape[1]), int(d.shape[2])
    if Nr < nc:
        import warnings
        warnings.warn("Ncoil < Nr, problem is ill posed")  # src/GROG.jl:26
    if (ns // Nr) * nt * nrep < nc * nc:
        import warnings
        warnings.warn("Number of spokes < Ncoil^2, problem is ill posed")  # src/GROG.jl:27
    out = jl_empty((Nd, nc, nc), torch.complex64)
    _lib.check(lib.mrsr_grog_calib(Nd, int(Nr), ns, nt, nc, nrep, ptr(d), ptr(t), ptr(out), stream_handle(stream)))
    return [out[i] for i in range(Nd)]


def grog_gridding(data, trj, lnG, Nr, img_shape, stream=None):
    """``grog_gridding!(data, trj, lnG, Nr, img_shape)``: grids ``data`` in place
    when it is a column-major complex64 CUDA tensor and returns the Int32
    Cartesian trajectory; for other inputs returns ``(trj_cart, gridded_data)``."""
    lib = _lib.load()
    inplace = isinstance(data, torch.Tensor) and data.is_cuda and data.dtype == torch.complex64
    d, nrep = _data4(data)
    if inplace and d.data_ptr() != data.data_ptr():
        inplace = False
    t = to_jl(trj, torch.float32)
    Nd = int(t.shape[0])
    L = jl_empty((Nd,) + tuple(lnG[0].shape), torch.complex64)
    for i in range(Nd):
        L[i].copy_(to_jl(lnG[i], torch.complex64))
    img_shape = tuple(int(v) for v in img_shape)
    out = jl_empty(tuple(t.shape), torch.int32)
    _lib.check(lib.mrsr_grog_gridding(Nd, _lib.int64_array(img_shape), int(Nr), int(d.shape[0]), int(d.shape[1]),
                                      int(d.shape[2]), nrep, ptr(d), ptr(t), ptr(L), ptr(out), stream_handle(stream)))
    return out if inplace else (out, d)


def radial_grog(data, trj, Nr, img_shape, stream=None):
    """``radial_grog!(data, trj, Nr, img_shape)``: calibration + gridding."""
    lnG = grog_calib(data, trj, Nr, stream=stream)
    return grog_gridding(data, trj, lnG, Nr, img_shape, stream=stream)
