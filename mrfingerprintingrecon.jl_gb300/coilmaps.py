"""Coil-wise calibration reconstructions: the caller of the normal operator inside
``calculate_coil_maps`` (src/CoilMaps.jl:1-116; GPU ext/MRISubspaceReconCUDAExt/CoilMaps.jl:1-55).

``reconstruct_coilwise`` (src/CoilMaps.jl:118-162, ext/.../CoilMaps.jl:57-77) builds
one K=1 operator without coil maps and solves Nc independent systems on it, one per
receive channel: non-Cartesian with a fixed iteration count
(``cg!(x_c, AᴴA, b_c; maxiter=Niter_cg, reltol=0)``), Cartesian with IterativeSolvers'
default tolerance (src/CoilMaps.jl:159).  Here the Nc systems run together on the
operator stacked over the coils (``NormalOperator.stack``, ``cg_stacked``): every pass
and CG step is one launch for all coils, while each coil keeps its own CG iteration.

``calculate_calibration_kspace`` is ``calculate_coil_maps`` up to the ESPIRiT call:
the calibration mask and the rescaled trajectory, the coil-wise reconstruction and
``fftshift(fft(fftshift(x)))``.  ``espirit`` runs ESPIRiT (MRICoilSensitivities'
``espirit``, which the reference's GPU extension calls on the host,
``espirit(Array(kbp), ...)``, ext/.../CoilMaps.jl:30) on the device, and
``calculate_coil_maps`` chains the two without leaving the device.
"""
import numpy as np
import torch

import ctypes as C

from . import _lib
from .arrays import jl_empty, jl_reshape, jl_zeros, mask_u8, ptr, stream_handle, to_host, to_jl
from .backprojection import _is_int_traj, calculate_backprojection
from .normalop import FFTNormalOp, NFFTNormalOp
from .solvers import DEFAULT_RELTOL, CgBatch, cg, cg_stacked


def _first_basis_column(U, nt):
    """``U[:, 1]`` as an (Nt, 1) basis; the GPU extension's default U is ``ones(Nt)``."""
    if U is None:
        return np.ones((nt, 1), dtype=np.float32)
    if isinstance(U, torch.Tensor):
        u = U if U.dim() == 1 else U[:, 0]
        return u.reshape(-1, 1)
    u = np.asarray(U)
    u = u if u.ndim == 1 else u[:, 0]
    return u.reshape(-1, 1)


def reconstruct_coilwise(data, trj, img_shape, U=None, sample_mask=None, Niter_cg=None, stream=None):
    """One image per receive channel: (img_shape..., Nc) column-major device tensor."""
    img_shape = tuple(int(s) for s in img_shape)
    cart = _is_int_traj(trj)
    U1 = _first_basis_column(U, int(trj.shape[-1]))
    if Niter_cg is None:
        Niter_cg = 5 if cart else 100  # the reference's defaults
    # the operator and the backprojection read the same trajectory and mask: upload once
    if trj.ndim == 3:
        trj = to_jl(trj, torch.int32 if cart else torch.float32)
        sample_mask = mask_u8(sample_mask)
    if cart:
        A = FFTNormalOp(img_shape, trj, U1, sample_mask=sample_mask, stream=stream)
    else:
        A = NFFTNormalOp(img_shape, trj, U1, sample_mask=sample_mask, stream=stream)
    b = calculate_backprojection(data, trj, img_shape, U=U1, sample_mask=sample_mask, stream=stream)
    x = _coilwise_solve(A, b, Niter_cg, tolerance_checked=cart, stream=stream)
    A.close()
    return x


def _coilwise_solve(A, b, iters, tolerance_checked=False, stream=None):
    """x[..., c] = cg(A, b[..., 1, c]) for every coil c of the (img..., 1, Nc) backprojection.

    The Nc solves run together on A stacked over the coils (``A.stack(Nc)``, one launch
    per pass and CG step for all coils), each with its own CG iteration: fixed
    iterations (reltol = 0), or with ``tolerance_checked`` IterativeSolvers' default
    reltol, coil by coil.  Where the stacked planes do not fit one block's shared memory
    (very long lines), the fixed solves run as the branches of one CUDA graph on operators
    sharing A's kernel and the tolerance-checked ones one after another."""
    img_shape = tuple(int(s) for s in b.shape[:-2])
    nc = int(b.shape[-1])
    try:
        S = A.stack(nc, stream=stream)
    except NotImplementedError:
        S = None
    if S is not None:
        reltol = DEFAULT_RELTOL if tolerance_checked else 0.0
        x = cg_stacked(S, b[..., 0, :], maxiter=int(iters), reltol=reltol, stream=stream)
        S.close()
        return x
    x = jl_zeros(img_shape + (nc,), torch.complex64)
    if tolerance_checked:
        for c in range(nc):
            x[..., c] = cg(A, b[..., 0, c], maxiter=iters, stream=stream)[..., 0]
        return x
    shares = [A.share(stream=stream) for _ in range(nc - 1)]
    batch = CgBatch([A] + shares, [b[..., 0, c] for c in range(nc)], [x[..., c] for c in range(nc)], int(iters),
                    stream=stream)
    batch.launch(stream=stream)
    (stream or torch.cuda.current_stream()).synchronize()
    batch.close()
    for op in shares:
        op.close()
    return x


def _calib_size_noncartesian(img_shape):
    """nextprod((2, 3, 5), N_i ÷ (maximum(img_shape) ÷ 32)) (src/CoilMaps.jl:37)."""
    def nextprod235(n):
        m = max(int(n), 1)
        while True:
            r = m
            for p in (2, 3, 5):
                while r % p == 0:
                    r //= p
            if r == 1:
                return m
            m += 1
    q = max(img_shape) // 32
    return tuple(nextprod235(n // q) for n in img_shape)


def calibration_mask(trj, img_shape, calib_size=None, sample_mask=None):
    """Calibration-region mask and trajectory of ``calculate_coil_maps``.

    Non-Cartesian (src/CoilMaps.jl:44-48, ext/.../CoilMaps.jl:17-20): keep samples with
    |k_d| * N_d / n_d < 1/2 in every dimension (products in float32, as the GPU
    extension's ``cu`` scale vector gives); the trajectory is scaled by N_d / n_d.
    Cartesian (src/CoilMaps.jl:80-84): keep lower < k_d < lower + n_d + 1 with
    lower = ceil((N_d - n_d) / 2); the trajectory is unchanged.
    Returns (mask (Ns, Nt) bool numpy, trajectory, calib_size)."""
    img_shape = tuple(int(s) for s in img_shape)
    t = to_host(trj) if isinstance(trj, torch.Tensor) else np.asarray(trj)
    d = t.shape[0]
    if np.issubdtype(t.dtype, np.integer):
        if calib_size is None:
            calib_size = tuple(n // (img_shape[0] // 32) for n in img_shape)
        lower = np.array([int(np.ceil((n - c) / 2)) for n, c in zip(img_shape, calib_size)]).reshape(d, 1, 1)
        upper = lower + np.array(calib_size).reshape(d, 1, 1) + 1
        mask = np.all(t > lower, axis=0) & np.all(t < upper, axis=0)
        trj_c = trj
    else:
        if calib_size is None:
            calib_size = _calib_size_noncartesian(img_shape)
        for c in calib_size:
            r = c
            for p in (2, 3, 5):
                while r % p == 0:
                    r //= p
            if r != 1:
                raise AssertionError("calib_size has to be composed of the prime factors 2, 3, and 5 "
                                     "(cf. NonuniformFFTs.jl documentation).")
        scale = np.array([n / c for n, c in zip(img_shape, calib_size)], dtype=np.float32).reshape(d, 1, 1)
        t32 = t.astype(np.float32)
        mask = np.all(np.abs(t32) * scale < np.float32(0.5), axis=0)
        trj_c = (t32 * scale).astype(np.float32)
    mask = mask.reshape(t.shape[1], -1)
    if sample_mask is not None:
        sm = to_host(sample_mask) if isinstance(sample_mask, torch.Tensor) else np.asarray(sample_mask)
        mask &= sm.reshape(mask.shape).astype(bool)
    return mask, trj_c, tuple(int(c) for c in calib_size)


def calculate_calibration_kspace(data, trj, img_shape, U=None, sample_mask=None, calib_size=None, Niter_cg=None,
                                 stream=None):
    """``calculate_coil_maps`` up to ESPIRiT: the centred calibration k-space
    ``fftshift(fft(fftshift(x)))`` of the coil-wise images, (calib_size..., Nc) complex64
    on the host.  4D data / trajectories (readout lines on their own axis) are
    reshaped as in src/CoilMaps.jl:99-111."""
    if getattr(data, "ndim", None) == 4 or (isinstance(data, torch.Tensor) and data.dim() == 4):
        data = to_jl(data, torch.complex64)
        data = jl_reshape(data, (-1, data.shape[2], data.shape[3]))
        t = to_host(trj) if isinstance(trj, torch.Tensor) else np.asarray(trj)
        trj = t.reshape(t.shape[0], -1, t.shape[3], order="F")
        if sample_mask is not None:
            sm = to_host(sample_mask) if isinstance(sample_mask, torch.Tensor) else np.asarray(sample_mask)
            sample_mask = sm.reshape(-1, sm.shape[-1], order="F")
    mask, trj_c, calib_size = calibration_mask(trj, img_shape, calib_size, sample_mask)
    x = to_host(reconstruct_coilwise(data, trj_c, calib_size, U=U, sample_mask=mask, Niter_cg=Niter_cg,
                                     stream=stream))
    axes = tuple(range(len(calib_size)))
    k = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(x, axes=axes), axes=axes), axes=axes)
    return k.astype(np.complex64)


def _centred_fft(x, ndim):
    """fftshift(fft(fftshift(x, 1:d), 1:d), 1:d) of a (calib..., Nc) device tensor."""
    axes = tuple(range(ndim))
    return torch.fft.fftshift(torch.fft.fftn(torch.fft.fftshift(x, dim=axes), dim=axes), dim=axes)


def calibration_kspace_device(data, trj, img_shape, U=None, sample_mask=None, calib_size=None, Niter_cg=None,
                              stream=None):
    """``calculate_calibration_kspace`` without leaving the device: (calib..., Nc) complex64."""
    if getattr(data, "ndim", None) == 4 or (isinstance(data, torch.Tensor) and data.dim() == 4):
        data = to_jl(data, torch.complex64)
        data = jl_reshape(data, (-1, data.shape[2], data.shape[3]))
        t = to_host(trj) if isinstance(trj, torch.Tensor) else np.asarray(trj)
        trj = t.reshape(t.shape[0], -1, t.shape[3], order="F")
        if sample_mask is not None:
            sm = to_host(sample_mask) if isinstance(sample_mask, torch.Tensor) else np.asarray(sample_mask)
            sample_mask = sm.reshape(-1, sm.shape[-1], order="F")
    mask, trj_c, calib_size = calibration_mask(trj, img_shape, calib_size, sample_mask)
    x = reconstruct_coilwise(data, trj_c, calib_size, U=U, sample_mask=mask, Niter_cg=Niter_cg, stream=stream)
    k = _centred_fft(x, len(calib_size))
    return to_jl(k, torch.complex64)


def espirit(kbp, img_shape, kernel_size=None, eigThresh_1=0.01, eigThresh_2=0.9, nmaps=1, eigenvalues=False,
            stream=None):
    """ESPIRiT maps (img..., Nc, nmaps) on the device from the centred calibration k-space
    ``kbp`` (calib..., Nc); ``eigenvalues=True`` also returns the (img..., nmaps) eigenvalues."""
    lib = _lib.load()
    k = to_jl(kbp, torch.complex64)
    img_shape = tuple(int(s) for s in img_shape)
    d = len(img_shape)
    calib = tuple(int(s) for s in k.shape[:d])
    nc = int(k.shape[d])
    if kernel_size is None:
        kernel_size = (6,) * d
    maps = jl_empty(img_shape + (nc, int(nmaps)), torch.complex64)
    eig = jl_empty(img_shape + (int(nmaps),), torch.float32)
    shp = (C.c_int64 * d)(*img_shape)
    cal = (C.c_int64 * d)(*calib)
    ks = (C.c_int64 * d)(*[int(v) for v in kernel_size])
    _lib.check(lib.mrsr_espirit(d, shp, cal, nc, ptr(k), ks, float(eigThresh_1), float(eigThresh_2), int(nmaps),
                                ptr(maps), ptr(eig), stream_handle(stream)))
    return (maps, eig) if eigenvalues else maps


def calculate_coil_maps(data, trj, img_shape, U=None, sample_mask=None, kernel_size=None, calib_size=None,
                        eigThresh_1=0.01, eigThresh_2=0.9, nmaps=1, Niter_cg=None, stream=None):
    """``calculate_coil_maps`` (src/CoilMaps.jl:32-63, :66-96; GPU ext/.../CoilMaps.jl:1-34) on
    the device: calibration region, coil-wise reconstruction, centred FFT, ESPIRiT.  Returns
    the reference's ``Vector`` of maps: one (img...) device array per coil (nmaps == 1) or
    per (coil, map)."""
    img_shape = tuple(int(s) for s in img_shape)
    kbp = calibration_kspace_device(data, trj, img_shape, U=U, sample_mask=sample_mask, calib_size=calib_size,
                                    Niter_cg=Niter_cg, stream=stream)
    maps = espirit(kbp, img_shape, kernel_size=kernel_size, eigThresh_1=eigThresh_1, eigThresh_2=eigThresh_2,
                   nmaps=nmaps, stream=stream)
    nc = int(maps.shape[len(img_shape)])
    if nmaps == 1:
        return [maps[..., c, 0] for c in range(nc)]
    return [maps[..., c, m] for c in range(nc) for m in range(int(nmaps))]
