"""Python mirror of ``calculate_backprojection`` (src/BackProjection.jl:1-164,
ext/MRISubspaceReconCUDAExt/BackProjection.jl:1-79) and of the tests'
forward model, backed by ``libmrsr.so``."""
import numpy as np
import torch

from . import _lib
from .arrays import is_complex_array, jl_empty, jl_reshape, mask_u8, ptr, stack_cmaps, stream_handle, to_jl

_DCF = {"none": _lib.DCF_NONE, "radial_2D": _lib.DCF_RADIAL_2D, "radial_3D": _lib.DCF_RADIAL_3D}


def _is_int_traj(trj):
    if isinstance(trj, torch.Tensor):
        return not trj.is_floating_point()
    return np.issubdtype(np.asarray(trj).dtype, np.integer)


def test_dimension(data, trj, U, cmaps_list_len, img_ndim, nt_u):
    """``src/BackProjection.jl:183-203`` (ValueError plays ArgumentError)."""
    if nt_u != data.shape[1]:
        raise ValueError(f"The second dimension of data ({data.shape[1]}) and the first one of U ({nt_u}) do not match. "
                         "Both should be number of time points.")
    if trj.shape[0] != img_ndim:
        raise ValueError(f"`cmaps` contains {img_ndim} image plus one coil dimension, yet the 1st dimension of each "
                         f"trj is of length {trj.shape[0]}.")
    if trj.shape[1] != data.shape[0]:
        raise ValueError(f"The 2nd dimension of each `trj` is {trj.shape[1]} and the 1st dimension of `data` is "
                         f"{data.shape[0]}. They should match and reflect the number of k-space samples.")
    if trj.shape[2] != data.shape[1]:
        raise ValueError(f"`trj` contains {trj.shape[2]} time frames, while data consists of {data.shape[1]}.")
    if cmaps_list_len != data.shape[2]:
        raise ValueError(f"The last dimension of `cmaps` is {cmaps_list_len} and the 3rd dimension of data is "
                         f"{data.shape[2]}.")


def calculate_backprojection(data, trj, cmaps_or_img_shape, U=None, sample_mask=None, density_compensation="none",
                             verbose=False, stream=None):
    """``calculate_backprojection(data, trj, cmaps | img_shape; U, sample_mask, density_compensation)``.

    With coil maps the result is ``(img..., K)`` (coil-combined); with an image
    shape it is ``(img..., K, Ncoil)``.  A float trajectory uses the NUFFT
    adjoint, an integer trajectory the binned Cartesian path.  4D ``data`` /
    ``trj`` (readout samples on a separate axis) are reshaped like the
    reference's wrapper (src/BackProjection.jl:159-164).
    """
    lib = _lib.load()
    if isinstance(cmaps_or_img_shape, (tuple, list)) and len(cmaps_or_img_shape) in (2, 3) and all(
            isinstance(v, (int, np.integer)) for v in cmaps_or_img_shape):
        img_shape = tuple(int(v) for v in cmaps_or_img_shape)
        S = None
        ncm = None
    else:
        S = stack_cmaps(cmaps_or_img_shape)
        img_shape = tuple(int(v) for v in S.shape[:-1])
        ncm = int(S.shape[-1])
    d = len(img_shape)
    int_traj = _is_int_traj(trj)
    t = to_jl(trj, torch.int32 if int_traj else torch.float32)
    dt = to_jl(data, torch.complex64)
    if t.dim() == 4 and dt.dim() == 4:  # wrapper for (Nr, Ncyc, ...) sample axes (src/BackProjection.jl:159-164)
        dt = jl_reshape(dt, (-1, dt.shape[2], dt.shape[3]))
        t = jl_reshape(t, (t.shape[0], -1, t.shape[3]))
        if isinstance(sample_mask, torch.Tensor):
            sample_mask = jl_reshape(mask_u8(sample_mask), (-1, sample_mask.shape[-1]))
        elif sample_mask is not None:
            m = np.asarray(sample_mask)
            sample_mask = m.reshape((-1, m.shape[-1]), order="F")
    nrep = int(dt.shape[3]) if dt.dim() == 4 else 1
    nt = int(t.shape[2])
    if U is None:
        Ut, ucplx, K, nt_u = None, 0, nt, nt
    else:
        ucplx = int(is_complex_array(U))
        Ut = to_jl(U, torch.complex64 if ucplx else torch.float32)
        K, nt_u = int(Ut.shape[1]), int(Ut.shape[0])
    ncoils = int(dt.shape[2])
    if S is not None and not int_traj:
        test_dimension(dt, t, Ut, ncm, d, nt_u)
    m = mask_u8(sample_mask)
    out = jl_empty(img_shape + ((K,) if S is not None else (K, ncoils)), torch.complex64)
    if int_traj:
        _lib.check(lib.mrsr_backprojection_cartesian(d, _lib.int64_array(img_shape), int(t.shape[1]), nt, ncoils, nrep,
                                                     ptr(dt), ptr(t), ptr(m), ptr(Ut), ucplx, K, ptr(S), ptr(out),
                                                     stream_handle(stream)))
        return out
    dcf_arr = None
    if isinstance(density_compensation, str):
        key = density_compensation.lstrip(":")
        if key not in _DCF:
            raise ValueError("`density_compensation` can only be `:radial_3D`, `:radial_2D`, `:none`, or of type "
                             "`AbstractArray`")
        kind = _DCF[key]
    else:
        kind = _lib.DCF_ARRAY
        dcf_arr = to_jl(np.asarray(density_compensation, dtype=np.float32).ravel(order="F"), torch.float32)
    _lib.check(lib.mrsr_backprojection(d, _lib.int64_array(img_shape), int(t.shape[1]), nt, ncoils, ptr(dt), ptr(t),
                                       ptr(m), ptr(Ut), ucplx, K, ptr(S), kind, ptr(dcf_arr), ptr(out),
                                       stream_handle(stream)))
    return out


def forward_model(x, trj, U, cmaps=None, stream=None):
    """Synthesise k-space data with the reference tests' forward model
    (``exec_type2!`` with fftshift=true, test/reconstruct_radial.jl:62-74):
    data[s, t, c] = sum_r S_c(r) sum_k U[t,k] x_k(r) exp(-2 pi i k_{s,t}.(r - N/2))."""
    lib = _lib.load()
    xt = to_jl(x, torch.complex64)
    t = to_jl(trj, torch.float32)
    img_shape = tuple(int(v) for v in xt.shape[:-1])
    K = int(xt.shape[-1])
    ucplx = int(is_complex_array(U))
    Ut = to_jl(U, torch.complex64 if ucplx else torch.float32)
    S = stack_cmaps(cmaps)
    nc = 1 if S is None else int(S.shape[-1])
    out = jl_empty((int(t.shape[1]), int(t.shape[2]), nc), torch.complex64)
    _lib.check(lib.mrsr_forward_model(len(img_shape), _lib.int64_array(img_shape), int(t.shape[1]), int(t.shape[2]), nc,
                                      ptr(xt), ptr(t), ptr(Ut), ucplx, K, ptr(S), ptr(out), stream_handle(stream)))
    return out
