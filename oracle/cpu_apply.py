"""Float32 CPU restatement of the reference's CPU apply, used only as the timed
CPU baseline (test infrastructure; see ``oracle/__init__.py``).

Follows ``mul!(x, ::_NFFTNormalOp, b, α, β)`` of ``src/NFFTNormalOp.jl:227-267``
step by step: per coil, zero the 2x oversampled K-stack, copy ``cmap .* b``
into the low corner, K full FFTs, a per-voxel K x K product on the kmask
voxels (kL2 zero elsewhere), K inverse FFTs, crop and accumulate
``α conj(cmap) .* kL2``.  FFTs run through ``scipy.fft`` with all host threads
(the reference runs its K FFTs on Julia threads); the per-voxel K x K products
are batched matmuls over voxel chunks on a thread pool of all host cores, as the
reference's ``@tasks`` loop over voxels (``src/NFFTNormalOp.jl:253-255``).
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as sfft


class CpuNFFTNormalOp:
    def __init__(self, img_shape, Lam, kmask, cmaps, workers=None):
        """Lam: (K, K, Nk) complex; kmask: 1-based indices into the 2x grid; cmaps: (img..., Nc)."""
        self.img = tuple(img_shape)
        self.G = tuple(2 * n for n in self.img)
        self.K = Lam.shape[0]
        self.kidx = np.asarray(kmask, dtype=np.int64) - 1
        self.lamT = np.ascontiguousarray(np.transpose(Lam, (2, 0, 1)).astype(np.complex64))  # (Nk, K, K)
        self.cmaps = np.asarray(cmaps, dtype=np.complex64)
        self.workers = workers or os.cpu_count()
        self.kL1 = np.zeros((self.K,) + self.G[::-1], dtype=np.complex64)  # C-order (K, G_d, ..., G_1)
        self.kL2 = np.zeros_like(self.kL1)
        self.pool = ThreadPoolExecutor(self.workers)
        nch = 4 * self.workers
        bounds = np.linspace(0, self.kidx.size, nch + 1).astype(np.int64)
        self.chunks = [(int(a), int(b)) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]

    def apply(self, b, coils=None, alpha=1.0):
        """x = alpha * A b for the coils in ``coils`` (default: all); b (img..., K)."""
        d = len(self.img)
        bT = np.ascontiguousarray(np.moveaxis(np.asarray(b, dtype=np.complex64), -1, 0).transpose(
            (0,) + tuple(range(d, 0, -1))))  # (K, N_d, ..., N_1)
        cT = np.moveaxis(self.cmaps, -1, 0).transpose((0,) + tuple(range(d, 0, -1)))
        x = np.zeros_like(bT)
        sl = (slice(None),) + tuple(slice(0, n) for n in self.img[::-1])
        axes = tuple(range(1, d + 1))
        for c in (range(cT.shape[0]) if coils is None else coils):
            self.kL1.fill(0)
            self.kL1[sl] = cT[c][None] * bT
            self._fft(self.kL1, axes, -1)
            k1 = self.kL1.reshape(self.K, -1)
            k2 = self.kL2.reshape(self.K, -1)
            k2.fill(0)
            # kmask indices are column-major over the 2x grid = row-major over the reversed C-order axes
            def voxels(ab, k1=k1, k2=k2):
                a, b = ab
                ix = self.kidx[a:b]
                X = k1[:, ix].T[:, :, None]                     # (n, K, 1)
                k2[:, ix] = np.matmul(self.lamT[a:b], X)[:, :, 0].T
            list(self.pool.map(voxels, self.chunks))
            self._fft(self.kL2, axes, +1)
            x += alpha * np.conj(cT[c])[None] * self.kL2[sl]
        return np.moveaxis(x.transpose((0,) + tuple(range(d, 0, -1))), 0, -1)

    def _fft(self, a, axes, sign):
        if sign < 0:
            a[...] = sfft.fftn(a, axes=axes, workers=self.workers)
        else:
            a[...] = sfft.ifftn(a, axes=axes, workers=self.workers)
        return a
