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
