"""Device arrays in Julia's column-major layout.

The C ABI takes pointers to column-major arrays with the reference's index
order.  Here such an array is a CUDA ``torch.Tensor`` whose *shape* is the
Julia shape and whose strides are Fortran strides (a permuted view of a
C-contiguous buffer).  Host ``numpy`` inputs are copied to the device once.
"""
import numpy as np
import torch

_NP2T = {
    np.dtype(np.float32): torch.float32,
    np.dtype(np.complex64): torch.complex64,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.bool_): torch.bool,
    np.dtype(np.uint8): torch.uint8,
}


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required (this package has no CPU implementation)")
    return torch.device("cuda", torch.cuda.current_device())


def jl_empty(shape, dtype, dev=None):
    """Uninitialised column-major device tensor with Julia shape ``shape``."""
    shape = tuple(int(s) for s in shape)
    dev = dev or device()
    t = torch.empty(shape[::-1], dtype=dtype, device=dev)
    return t.permute(*reversed(range(len(shape))))


def jl_zeros(shape, dtype, dev=None):
    t = jl_empty(shape, dtype, dev)
    t.zero_()
    return t


def is_jl_contiguous(t):
    return t.permute(*reversed(range(t.dim()))).is_contiguous()


def to_jl(a, dtype):
    """Column-major CUDA tensor of ``dtype`` holding ``a`` (numpy array or tensor)."""
    if isinstance(a, torch.Tensor):
        if a.is_cuda and a.dtype == dtype and is_jl_contiguous(a):
            return a
        out = jl_empty(a.shape, dtype, a.device if a.is_cuda else None)
        out.copy_(a.to(dtype) if a.dtype != dtype else a)
        return out
    arr = np.asarray(a)
    src = torch.from_numpy(np.ascontiguousarray(arr))
    out = jl_empty(arr.shape, dtype)
    out.copy_(src.to(dtype) if src.dtype != dtype else src)
    return out


def mask_u8(m):
    """Column-major uint8 CUDA tensor of a sample mask (numpy array or tensor, bool or
    integer), or None."""
    if m is None:
        return None
    if isinstance(m, torch.Tensor):
        return to_jl(m if m.dtype == torch.uint8 else m.to(torch.uint8), torch.uint8)
    return to_jl(np.asarray(m, dtype=np.uint8), torch.uint8)


def jl_reshape(t, shape):
    """Julia ``reshape`` (column-major) of a column-major tensor; shares memory."""
    shape = list(shape)
    if -1 in shape:
        i = shape.index(-1)
        rest = int(np.prod([s for j, s in enumerate(shape) if j != i]))
        shape[i] = t.numel() // rest
    c = t.permute(*reversed(range(t.dim())))
    return c.reshape(tuple(shape[::-1])).permute(*reversed(range(len(shape))))


def to_host(t):
    """numpy copy of a device tensor, keeping the Julia index order."""
    return t.detach().cpu().numpy()


def ptr(t):
    return None if t is None else t.data_ptr()


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def is_complex_array(a):
    if isinstance(a, torch.Tensor):
        return a.is_complex()
    return np.iscomplexobj(a)


def stack_cmaps(cmaps, img_shape=None):
    """The reference passes ``cmaps`` as a vector of per-coil arrays; the C ABI
    takes one (img..., Nc) array.  Accepts a list or an already stacked array."""
    if cmaps is None:
        return None
    if isinstance(cmaps, (list, tuple)):
        if len(cmaps) == 1 and not isinstance(cmaps[0], (np.ndarray, torch.Tensor)):
            return None  # cmaps=(1,): the reference's default single unit coil
        parts = [to_jl(c, torch.complex64) for c in cmaps]
        shape = tuple(parts[0].shape) + (len(parts),)
        out = jl_empty(shape, torch.complex64)
        for i, c in enumerate(parts):
            out[..., i].copy_(c)
        return out
    return to_jl(cmaps, torch.complex64)
