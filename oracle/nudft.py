"""Exact non-uniform DFTs (float64), separable per dimension.

Sign conventions are the ones the reference fixes through
``NonuniformFFTs._transform_point_convention`` (comment at
``src/BackProjection.jl:35``) and the forward model of its tests
(``exec_type2!`` with ``fftshift=true``, ``test/reconstruct_radial.jl:62-74``):

* forward (type 2):  y_n = sum_r x[r] exp(-2 pi i k_n . (r - N/2))
* adjoint (type 1):  b[r] = sum_n v_n exp(+2 pi i k_n . (r - N/2))
* point-spread sums: c[j] = sum_n w_n exp(+2 pi i j . k_n)

Array index order follows the reference (``trj[d, n]``, images ``x[r1, r2(, r3)]``).
"""
import numpy as np


def _phase(freqs, kd, sign):
    """E[f, n] = exp(sign * 2 pi i * f * k_n) in float64."""
    return np.exp(sign * 2j * np.pi * np.outer(np.asarray(freqs, dtype=np.float64),
                                              np.asarray(kd, dtype=np.float64)))


def nudft_sum(v, k, freq_sets, sign):
    """out[j1, j2(, j3)] = sum_n v_n exp(sign 2 pi i sum_d j_d k_dn) for j_d in freq_sets[d]."""
    k = np.asarray(k, dtype=np.float64)
    v = np.asarray(v, dtype=np.complex128)
    d = k.shape[0]
    E = [_phase(freq_sets[i], k[i], sign) for i in range(d)]
    if d == 2:
        return (E[0] * v[None, :]) @ E[1].T
    if d == 3:
        out = np.empty((len(freq_sets[0]), len(freq_sets[1]), len(freq_sets[2])), dtype=np.complex128)
        for i3 in range(len(freq_sets[2])):
            out[:, :, i3] = (E[0] * (v * E[2][i3])[None, :]) @ E[1].T
        return out
    if d == 1:
        return E[0] @ v
    raise ValueError("1 <= d <= 3")


def forward(x, k):
    """Type-2 exact: y_n = sum_r x[r] exp(-2 pi i k_n . (r - N/2)). x shape img_shape."""
    x = np.asarray(x, dtype=np.complex128)
    k = np.asarray(k, dtype=np.float64)
    d = k.shape[0]
    E = [_phase(np.arange(n) - n // 2, k[i], -1.0) for i, n in enumerate(x.shape)]
    if d == 2:
        return np.einsum("an,an->n", E[0], x @ E[1])
    if d == 3:
        t = np.einsum("abc,cn->abn", x, E[2])
        t = np.einsum("abn,bn->an", t, E[1])
        return np.einsum("an,an->n", t, E[0])
    raise ValueError("d must be 2 or 3")


def adjoint(v, k, img_shape):
    """Type-1 exact with centred output: b[r] = sum_n v_n exp(+2 pi i k_n . (r - N/2))."""
    return nudft_sum(v, k, [np.arange(n) - n // 2 for n in img_shape], +1.0)


# ---------------------------------------------------------------------------
# Fast float64 type-1 transform for large sample counts (test infrastructure).
#
# The exact sums above cost O(modes x samples); for the benchmark-sized
# trajectories (512k samples on a 512^2 mode grid) they take hours.  This is
# the standard spreading NUFFT with the exponential-of-semicircle kernel
# phi(z) = exp(beta (sqrt(1 - z^2) - 1)), w = 8 cells, beta = 2.30 w, on a
# grid oversampled by 2 (Barnett, Magland, af Klinteberg, SIAM J. Sci.
# Comput. 41, 2019), evaluated entirely in float64: relative error ~1e-7
# against ``nudft_sum``.
# ---------------------------------------------------------------------------
ES_W = 8
ES_BETA = 2.30 * ES_W


def _es_phi(z):
    out = np.zeros_like(z)
    m = np.abs(z) < 1.0
    out[m] = np.exp(ES_BETA * (np.sqrt(1.0 - z[m] * z[m]) - 1.0))
    return out


def _es_psi_hat(j, M):
    """psi_hat(j) = (w/2) int_{-1}^{1} phi(z) cos(pi j w z / M) dz by 200-point Gauss-Legendre."""
    x, wq = np.polynomial.legendre.leggauss(200)
    ph = _es_phi(x)
    j = np.asarray(j, dtype=np.float64)
    return 0.5 * ES_W * (np.cos(np.pi * np.outer(j, x) * ES_W / M) @ (wq * ph))


class Nufft1Plan:
    """Type-1 spreading plan of fixed points: approximates ``nudft_sum(v, k, freq_sets, sign)``
    for many weight vectors v (|j| <= M/4 per dimension)."""

    def __init__(self, k, freq_sets, sign=+1.0):
        k = np.asarray(k, dtype=np.float64)
        d = k.shape[0]
        self.freq_sets = [np.asarray(s) for s in freq_sets]
        M = []
        for s in self.freq_sets:  # grid of at least 4 max|j| cells with a 2,3,5-smooth length
            m = max(16, 4 * int(np.max(np.abs(s))) + 4)
            while not _smooth(m):
                m += 2
            M.append(m)
        self.M = M
        hw = ES_W / 2
        taps = []
        for i in range(d):
            u = sign * k[i] * M[i]
            l0 = np.ceil(u - hw).astype(np.int64)
            l = l0[:, None] + np.arange(ES_W)[None, :]                    # (n, w)
            taps.append((np.mod(l, M[i]), _es_phi((l - u[:, None]) / hw)))
        # flattened C-order cell index and weight of every (sample, tap) pair
        idx, wt = taps[0]
        for i in range(1, d):
            shp = (taps[i][0].shape[0],) + (1,) * i + (ES_W,)
            idx = idx[..., None] * M[i] + taps[i][0].reshape(shp)
            wt = wt[..., None] * taps[i][1].reshape(shp)
        self.n = k.shape[1]
        self.idx = idx.reshape(-1)
        self.wt = wt.reshape(self.n, -1)
        self.ncell = int(np.prod(M))
        self.inv_psi = []
        for i, s in enumerate(self.freq_sets):
            shape = [1] * d
            shape[i] = len(s)
            self.inv_psi.append((1.0 / _es_psi_hat(s, M[i])).reshape(shape))

    def __call__(self, v):
        v = np.asarray(v)
        if np.iscomplexobj(v):
            g = (np.bincount(self.idx, (self.wt * v.real[:, None]).reshape(-1), minlength=self.ncell)
                 + 1j * np.bincount(self.idx, (self.wt * v.imag[:, None]).reshape(-1), minlength=self.ncell))
        else:
            g = np.bincount(self.idx, (self.wt * np.asarray(v, dtype=np.float64)[:, None]).reshape(-1),
                            minlength=self.ncell) + 0j
        F = np.fft.ifftn(g.reshape(self.M)) * self.ncell              # sum_l g[l] exp(+2 pi i j l / M)
        out = F[np.ix_(*[np.mod(s, self.M[i]) for i, s in enumerate(self.freq_sets)])]
        for f in self.inv_psi:
            out = out * f
        return out


def nufft1_es(v, k, freq_sets, sign=+1.0):
    """One-shot ``Nufft1Plan(k, freq_sets, sign)(v)``."""
    return Nufft1Plan(k, freq_sets, sign)(v)


def _smooth(m):
    for p in (2, 3, 5):
        while m % p == 0:
            m //= p
    return m == 1
