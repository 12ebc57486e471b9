"""Float64 restatement of ``src/BackProjection.jl``."""
import numpy as np

from . import nudft
from .normalop import masked_points, frame_of_sample


def test_dimension(data, trj, U, cmaps):
    """``src/BackProjection.jl:183-203``: the same ArgumentError checks (ValueError here)."""
    Nt = U.shape[0]
    img_shape = np.asarray(cmaps[0]).shape
    Ncoil = len(cmaps)
    if Nt != data.shape[1]:
        raise ValueError("second dimension of data and first of U do not match")
    if trj.shape[0] != len(img_shape):
        raise ValueError("trj dimensionality does not match cmaps")
    if trj.shape[1] != data.shape[0]:
        raise ValueError("number of k-space samples of trj and data do not match")
    if trj.shape[2] != data.shape[1]:
        raise ValueError("number of time frames of trj and data do not match")
    if Ncoil != data.shape[2]:
        raise ValueError("number of coils of cmaps and data do not match")


def density_compensation_weights(pts, density_compensation):
    """``src/BackProjection.jl:169-181`` (evaluated in float32 like the reference)."""
    if isinstance(density_compensation, str):
        p32 = pts.astype(np.float32)
        if density_compensation == "radial_3D":
            return np.sum(p32 * p32, axis=0, dtype=np.float32)
        if density_compensation == "radial_2D":
            return np.sqrt(np.sum(p32 * p32, axis=0, dtype=np.float32))
        if density_compensation == "none":
            return None
        raise ValueError("density_compensation can only be radial_3D, radial_2D, none, or an array")
    return np.asarray(density_compensation)


def calculate_backprojection(data, trj, cmaps=None, img_shape=None, U=None, sample_mask=None,
                             density_compensation="none"):
    """Non-Cartesian backprojection (``src/BackProjection.jl:23-102``).

    With ``cmaps`` the coils are combined (``:62-102``) and the result has shape
    ``img_shape + (K,)``; with ``img_shape`` only it is ``img_shape + (K, Ncoil)``
    (``:23-60``).
    """
    data = np.asarray(data)
    trj = np.asarray(trj, dtype=np.float32)
    if U is None:
        U = np.eye(trj.shape[2], dtype=np.complex64)
    U = np.asarray(U)
    if sample_mask is None:
        sample_mask = np.ones(trj.shape[1:], dtype=bool)
    sample_mask = np.asarray(sample_mask, dtype=bool)
    if cmaps is not None:
        test_dimension(data, trj, U, cmaps)
        img_shape = np.asarray(cmaps[0]).shape
    img_shape = tuple(img_shape)
    pts = masked_points(trj, sample_mask)
    t_of = frame_of_sample(sample_mask)
    if len(t_of) == 0:
        raise AssertionError("Sample mask removes all samples, cannot compute backprojection.")
    dcf = density_compensation_weights(pts, density_compensation)
    K = U.shape[1]
    Nc = data.shape[2]
    dm = np.stack([data[:, :, c].T[sample_mask.T] for c in range(Nc)], axis=1).astype(np.complex128)
    if cmaps is not None:
        out = np.zeros(img_shape + (K,), dtype=np.complex128)
    else:
        out = np.zeros(img_shape + (K, Nc), dtype=np.complex128)
    for k in range(K):
        uk = np.conj(U[t_of, k].astype(np.complex128))
        for c in range(Nc):
            v = dm[:, c] * uk
            if dcf is not None:
                v = v * dcf
            b = nudft.adjoint(v, pts, img_shape)
            if cmaps is not None:
                out[..., k] += np.conj(np.asarray(cmaps[c], dtype=np.complex128)) * b
            else:
                out[..., k, c] = b
    return out


def calculate_backprojection_cartesian(data, trj, cmaps=None, img_shape=None, U=None, sample_mask=None):
    """Integer-trajectory backprojection (``src/BackProjection.jl:104-156``).

    data is (Ns, Nt, Nc) or (Ns, Nt, Nc, Nrep); U is (Nt, K) or (Nt, K, Nrep).
    """
    data = np.asarray(data)
    if data.ndim == 3:
        data = data[..., None]
    trj = np.asarray(trj)
    if U is None:
        U = np.eye(trj.shape[2], dtype=np.complex64)
    U = np.asarray(U)
    if U.ndim == 2:
        U = U[:, :, None]
    if sample_mask is None:
        sample_mask = np.ones(trj.shape[1:], dtype=bool)
    if cmaps is not None:
        img_shape = np.asarray(cmaps[0]).shape
    img_shape = tuple(img_shape)
    d = len(img_shape)
    K = U.shape[1]
    Nc = data.shape[2]
    s_idx, t_idx = np.nonzero(np.asarray(sample_mask, dtype=bool))
    cells = tuple(np.mod(trj[i, s_idx, t_idx].astype(np.int64) - img_shape[i] // 2 - 1, img_shape[i]) for i in range(d))
    if cmaps is not None:
        out = np.zeros(img_shape + (K,), dtype=np.complex128)
    else:
        out = np.zeros(img_shape + (K, Nc), dtype=np.complex128)
    Uc = U.astype(np.complex128)
    for k in range(K):
        for c in range(Nc):
            g = np.zeros(img_shape, dtype=np.complex128)
            v = np.sum(data[s_idx, t_idx, c, :].astype(np.complex128) * np.conj(Uc[t_idx, k, :]), axis=1)
            np.add.at(g, cells, v)
            g = np.fft.fftshift(np.fft.ifftn(g))
            if cmaps is not None:
                out[..., k] += np.conj(np.asarray(cmaps[c], dtype=np.complex128)) * g
            else:
                out[..., k, c] = g
    return out
