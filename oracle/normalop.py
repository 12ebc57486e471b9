"""Float64 restatement of the Toeplitz normal operators of MRISubspaceRecon.jl.

Index order follows the reference: images ``x[r1, r2(, r3), k]``, kernels
``Lam[k1, k2, i]`` (CPU layout, ``src/NFFTNormalOp.jl:137``) or packed
``Lp[ind, i]`` with ``ind = k1 + k2 (k2+1)/2`` for 0-based ``k1 <= k2`` (GPU
layout, ``ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:239``), linear grid
indices are 1-based and column-major like Julia's ``findall``.
"""
import numpy as np
import scipy.fft as sfft

from . import nudft

KMASK_HALF_SUPPORT = 4  # NonuniformFFTs.jl default HalfSupport(4): 2*4 cells per dimension


def packed_index(k1, k2):
    """0-based packed upper-triangle index (column-major, k1 <= k2)."""
    if k1 > k2:
        k1, k2 = k2, k1
    return k1 + k2 * (k2 + 1) // 2


def frame_of_sample(sample_mask):
    """Frame index of each masked sample in the order ``trj[:, sample_mask]`` takes them."""
    m = np.asarray(sample_mask, dtype=bool)
    t = np.broadcast_to(np.arange(m.shape[1])[None, :], m.shape)
    return t.T[m.T]


def masked_points(trj, sample_mask):
    """``trj[:, sample_mask]`` with Julia's column-major (frame-major) order."""
    trj = np.asarray(trj)
    m = np.asarray(sample_mask, dtype=bool)
    d = trj.shape[0]
    pts = np.stack([trj[i].T[m.T] for i in range(d)])
    return pts


def kmask_indcs(img_shape_os, trj, sample_mask=None):
    """Kept cells of the oversampled grid (``src/NFFTNormalOp.jl:106-118``).

    The reference keeps every grid cell in the footprint of a σ=1 Gaussian
    spreading kernel of half-support 4 (NonuniformFFTs.jl).  For a sample k_d
    the footprint covers cells i0-3 .. i0+4 (mod G_d) with
    i0 = floor(fl32(-k_d * G_d)): the cell holding the point -2 pi k_d on the
    grid of spacing 2 pi / G_d.  Returns sorted 1-based column-major indices.
    """
    trj = np.asarray(trj, dtype=np.float32)
    if sample_mask is None:
        sample_mask = np.ones(trj.shape[1:], dtype=bool)
    G = tuple(int(g) for g in img_shape_os)
    for g in G:
        r = g
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        assert r == 1, "img_shape_os has to be composed of the prime factors 2, 3, and 5"
    pts = masked_points(trj, sample_mask)
    d = len(G)
    hit = np.zeros(G, dtype=bool)
    m = KMASK_HALF_SUPPORT
    i0 = [np.floor((np.float32(-1.0) * pts[i]) * np.float32(G[i])).astype(np.int64) for i in range(d)]
    offs = np.arange(-m + 1, m + 1)
    if d == 2:
        for a in offs:
            c1 = (i0[0] + a) % G[0]
            for b in offs:
                hit[c1, (i0[1] + b) % G[1]] = True
    else:
        for a in offs:
            c1 = (i0[0] + a) % G[0]
            for b in offs:
                c2 = (i0[1] + b) % G[1]
                for c in offs:
                    hit[c1, c2, (i0[2] + c) % G[2]] = True
    return np.flatnonzero(hit.ravel(order="F")) + 1


def _fft_order(n):
    return np.concatenate([np.arange(0, n // 2), np.arange(-(n // 2), 0)])


def _psf_sets(G, half_first):
    sets = [np.arange(0, G[0] // 2 + 1) if half_first else _fft_order(G[0])]
    return sets + [_fft_order(g) for g in G[1:]]


def psf(img_shape_os, pts, w, half_first=False):
    """Exact point-spread sums c[j] = sum_n w_n exp(+2 pi i j.k_n) on the grid in FFT order.

    With ``half_first`` the first dimension holds j1 = 0..G1/2 (the half
    spectrum a real-input type-1 transform returns), the others FFT order.
    """
    return nudft.nudft_sum(w, pts, _psf_sets(img_shape_os, half_first), +1.0)


def calculate_kernel_noncartesian(img_shape_os, trj, U, sample_mask=None, fast=False):
    """``src/NFFTNormalOp.jl:121-225`` with exact PSFs. Returns (Lam[K,K,Nk], kmask).

    ``fast``: the point-spread sums come from the float64 spreading NUFFT
    (``nudft.Nufft1Plan``, ~1e-7 relative) instead of exact sums, for
    trajectories too large for O(modes x samples).
    """
    trj = np.asarray(trj, dtype=np.float32)
    if sample_mask is None:
        sample_mask = np.ones(trj.shape[1:], dtype=bool)
    kmask = kmask_indcs(img_shape_os, trj, sample_mask)
    pts = masked_points(trj, sample_mask)
    t_of = frame_of_sample(sample_mask)
    assert len(t_of) > 0, "Mask removes all samples, cannot compute kernel."
    U = np.asarray(U)
    K = U.shape[1]
    G = tuple(img_shape_os)
    Lam = np.zeros((K, K, len(kmask)), dtype=np.complex128)
    real_u = not np.iscomplexobj(U)
    if fast:
        plan = nudft.Nufft1Plan(pts, _psf_sets(G, real_u), +1.0)
        psf_of = lambda w, half_first=False: plan(w)  # noqa: E731
    else:
        psf_of = lambda w, half_first=False: psf(G, pts, w, half_first=half_first)  # noqa: E731
    for k2 in range(K):
        for k1 in range(k2 + 1):
            if real_u:
                w = (U[t_of, k1].astype(np.float64) * U[t_of, k2].astype(np.float64))
                ch = psf_of(w, half_first=True)
                axes = tuple(range(1, len(G))) + (0,)
                s = tuple(G[1:]) + (G[0],)
                lam = np.fft.irfftn(np.conj(ch), s=s, axes=axes) * np.prod(G)
                v = lam.ravel(order="F")[kmask - 1]
                Lam[k1, k2] = v
                Lam[k2, k1] = v
            else:
                w = np.conj(U[t_of, k1].astype(np.complex128)) * U[t_of, k2].astype(np.complex128)
                c = psf_of(w)
                lam = np.fft.fftn(c)
                v = lam.ravel(order="F")[kmask - 1]
                # statement order of src/NFFTNormalOp.jl:161-162: the mirror first, so the diagonal keeps λ
                Lam[k2, k1] = np.conj(v)
                Lam[k1, k2] = v
    if real_u:
        Lam = Lam.real.astype(np.float64) + 0j
    return Lam, kmask


def pack_lambda(Lam, real=False):
    """(K,K,Nk) -> packed (P, Nk) upper triangle (GPU extension layout)."""
    K = Lam.shape[0]
    P = K * (K + 1) // 2
    out = np.zeros((P, Lam.shape[2]), dtype=np.float64 if real else np.complex128)
    for k2 in range(K):
        for k1 in range(k2 + 1):
            v = Lam[k1, k2]
            out[packed_index(k1, k2)] = v.real if real else v
    return out


def unpack_lambda(Lp, K):
    """Packed (P, Nk) -> full Hermitian (K, K, Nk) (``kernel_mul!`` semantics)."""
    out = np.zeros((K, K, Lp.shape[1]), dtype=np.complex128)
    for k2 in range(K):
        for k1 in range(K):
            if k1 <= k2:
                out[k1, k2] = Lp[packed_index(k1, k2)]
            else:
                out[k1, k2] = np.conj(Lp[packed_index(k2, k1)])
    return out


def _stack_cmaps(cmaps, img_shape):
    if cmaps is None:
        return np.ones((1,) + tuple(img_shape), dtype=np.complex128)
    return np.stack([np.asarray(c, dtype=np.complex128) for c in cmaps])


def nfft_normalop_apply(x, Lam, kmask, img_shape, cmaps=None, alpha=1.0, beta=0.0, xout=None):
    """``src/NFFTNormalOp.jl:227-267``: x_out <- beta x_out + alpha sum_c S_c^H crop F^-1 Lam F pad S_c x."""
    img_shape = tuple(img_shape)
    d = len(img_shape)
    K = Lam.shape[0]
    x = np.asarray(x, dtype=np.complex128).reshape(img_shape + (K,), order="F")
    G = tuple(2 * n for n in img_shape)
    S = _stack_cmaps(cmaps, img_shape)
    out = np.zeros(img_shape + (K,), dtype=np.complex128)
    if xout is not None and beta != 0:
        out = beta * np.asarray(xout, dtype=np.complex128).reshape(img_shape + (K,), order="F")
    idx = tuple(slice(0, n) for n in img_shape)
    kidx = np.asarray(kmask) - 1
    for c in range(S.shape[0]):
        kL1 = np.zeros(G + (K,), dtype=np.complex128)
        kL1[idx] = S[c][..., None] * x
        kL1 = sfft.fftn(kL1, axes=tuple(range(d)), workers=-1)
        k1r = kL1.reshape(-1, K, order="F")
        k2r = np.zeros_like(k1r)
        k2r[kidx] = np.einsum("jki,ik->ij", Lam, k1r[kidx])
        kL2 = k2r.reshape(G + (K,), order="F")
        kL2 = sfft.ifftn(kL2, axes=tuple(range(d)), workers=-1)
        out += alpha * np.conj(S[c])[..., None] * kL2[idx]
    return out


def calculate_kernel_cartesian(img_shape, trj, U, sample_mask=None):
    """``src/FFTNormalOp.jl:81-97``: binned Uᴴ diag(count) U on the ifftshifted grid."""
    img_shape = tuple(img_shape)
    trj = np.asarray(trj)
    if sample_mask is None:
        sample_mask = np.ones(trj.shape[1:], dtype=bool)
    U = np.asarray(U)
    if U.ndim == 2:
        U = U[:, :, None]
    K = U.shape[1]
    d = len(img_shape)
    Lam = np.zeros((K, K) + img_shape, dtype=np.complex128)
    m = np.asarray(sample_mask, dtype=bool)
    s_idx, t_idx = np.nonzero(m)
    cells = tuple(np.mod(trj[i, s_idx, t_idx].astype(np.int64) - img_shape[i] // 2 - 1, img_shape[i]) for i in range(d))
    Uc = U.astype(np.complex128)
    for k1 in range(K):
        for k2 in range(K):
            w = np.sum(np.conj(Uc[t_idx, k1, :]) * Uc[t_idx, k2, :], axis=1)
            np.add.at(Lam[k1, k2], cells, w)
    return Lam


def calculate_kernel_cartesian_mask(M, U):
    """``src/FFTNormalOp.jl:99-109``: Lam[:,:,i] = U' * (M[i,:] .* U) on the ifftshifted mask."""
    M = np.asarray(M)
    d = M.ndim - 1
    Ms = np.fft.ifftshift(M, axes=tuple(range(d))).astype(np.float64)
    Uc = np.asarray(U).astype(np.complex128)
    return np.einsum("tk,...t,tl->kl...", np.conj(Uc), Ms, Uc)


def fft_normalop_from_lambda(Lam):
    """``src/FFTNormalOp.jl:38-64``: kmask = Lam[1,1,:] != 0 and the compacted kernel."""
    K = Lam.shape[0]
    img_shape = Lam.shape[2:]
    flat = Lam.reshape(K, K, -1, order="F")
    kmask = np.flatnonzero(flat[0, 0] != 0) + 1
    return flat[:, :, kmask - 1], kmask, tuple(img_shape)


def fft_normalop_apply(x, Lam_c, kmask, img_shape, cmaps=None, alpha=1.0, beta=0.0, xout=None):
    """``src/FFTNormalOp.jl:111-149``."""
    img_shape = tuple(img_shape)
    d = len(img_shape)
    K = Lam_c.shape[0]
    x = np.asarray(x, dtype=np.complex128).reshape(img_shape + (K,), order="F")
    S = _stack_cmaps(cmaps, img_shape)
    out = np.zeros(img_shape + (K,), dtype=np.complex128)
    if xout is not None and beta != 0:
        out = beta * np.asarray(xout, dtype=np.complex128).reshape(img_shape + (K,), order="F")
    kidx = np.asarray(kmask) - 1
    for c in range(S.shape[0]):
        kL1 = np.fft.fftn(S[c][..., None] * x, axes=tuple(range(d)))
        k1r = kL1.reshape(-1, K, order="F")
        k2r = np.zeros_like(k1r)
        k2r[kidx] = np.einsum("jki,ik->ij", Lam_c, k1r[kidx])
        kL2 = np.fft.ifftn(k2r.reshape(img_shape + (K,), order="F"), axes=tuple(range(d)))
        out += alpha * np.conj(S[c])[..., None] * kL2
    return out
