"""Float64 restatement of ESPIRiT coil-sensitivity estimation (test infrastructure).

The reference calls ``espirit(kbp, img_shape, kernel_size; eigThresh_1, eigThresh_2,
nmaps)`` of MRICoilSensitivities.jl 0.1.1 (``Project.toml:9,21``; call sites
``src/CoilMaps.jl:57``, ``:91`` and ``ext/MRISubspaceReconCUDAExt/CoilMaps.jl:30``, which
copies the calibration k-space to the host).  That package is a dependency absent from
the reference tree, so this module restates the published algorithm (Uecker, Lai,
Murphy, Virtue, Elad, Pauly, Vasanawala, Lustig, "ESPIRiT -- an eigenvalue approach to
autocalibrating parallel MRI", Magn. Reson. Med. 71, 2014) with the conventions below;
element-wise parity with the Julia package is unpinned.  It is pinned instead by the
method's defining property: on consistent calibration data the true sensitivities are
eigenvalue-1 eigenvectors of the image-space ESPIRiT operator (tests/test_oracle_pins.py).

Conventions:

* ``kbp`` (calib..., Nc) is the centred calibration k-space, DC at index calib // 2
  (``fftshift(fft(fftshift(x)))`` of the coil-wise calibration images).
* Calibration matrix A: one row per kernel position p (every p with p + [0, k) inside the
  calibration region), columns (kappa, c) with kappa column-major over the kernel and the
  coil index outermost: A[p, (kappa, c)] = kbp[p + kappa, c].
* Signal subspace: the right singular vectors V of A with sigma >= eigThresh_1 sigma_max.
  A patch R_p x (a row of A, as a column vector) lies in the span of conj(V), so the
  projector onto the patch signal space is P = conj(V) V^T.
* ESPIRiT operator, k-space: W = (1/M) sum_p R_p^H P R_p (M = prod(kernel) patches
  cover each point).  Image space, pixel r of the N^d image (centre at N // 2):
  W(r)_{cc'} = (1/M) sum_delta Q_{cc'}(delta) exp(-2 pi i delta . (r - N//2) / N) with
  Q_{cc'}(delta) = sum_kappa P[(kappa, c), (kappa + delta, c')].
* Maps: the nmaps leading eigenvectors of W(r), set to zero where their eigenvalue is
  below eigThresh_2, each rotated so that its coil-1 entry is real and non-negative.
"""
import numpy as np


def calibration_matrix(kbp, kernel_size):
    kbp = np.asarray(kbp, dtype=np.complex128)
    calib = kbp.shape[:-1]
    nc = kbp.shape[-1]
    d = len(calib)
    k = tuple(int(v) for v in kernel_size)
    npos = tuple(c - kk + 1 for c, kk in zip(calib, k))
    assert all(n >= 1 for n in npos), "kernel larger than the calibration region"
    cols = []
    for c in range(nc):
        for kap in np.ndindex(*k[::-1]):
            kap = kap[::-1]  # column-major over the kernel
            sl = tuple(slice(kap[i], kap[i] + npos[i]) for i in range(d))
            cols.append(kbp[sl + (c,)].ravel(order="F"))
    return np.stack(cols, axis=1)  # (prod(npos), prod(k) * nc)


def signal_subspace(A, eig_thresh_1):
    _, s, vh = np.linalg.svd(A, full_matrices=False)
    n = int(np.sum(s >= eig_thresh_1 * s[0]))
    return vh[:n].conj().T, s


def espirit_operator(V, kernel_size, nc, img_shape):
    """W(r) for every pixel: (img..., Nc, Nc)."""
    k = tuple(int(v) for v in kernel_size)
    d = len(k)
    M = int(np.prod(k))
    P = V.conj() @ V.T
    P = P.reshape((nc, M, nc, M))  # [c, kappa, c', kappa'] with kappa linear (column-major)
    kaps = [np.array(np.unravel_index(i, k, order="F")) for i in range(M)]
    img_shape = tuple(img_shape)
    W = np.zeros(img_shape + (nc, nc), dtype=np.complex128)
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in img_shape], indexing="ij")
    Q = {}
    for a in range(M):
        for b in range(M):
            delta = tuple(kaps[b] - kaps[a])
            Q[delta] = Q.get(delta, 0) + P[:, a, :, b]
    for delta, q in Q.items():
        ph = np.exp(-2j * np.pi * sum(delta[i] * grids[i] / img_shape[i] for i in range(d)))
        W += ph[..., None, None] * q[(None,) * d]
    return W / M


def espirit(kbp, img_shape, kernel_size, eig_thresh_1=0.01, eig_thresh_2=0.9, nmaps=1):
    """Returns (maps (img..., Nc, nmaps), eigenvalues (img..., nmaps))."""
    kbp = np.asarray(kbp)
    nc = kbp.shape[-1]
    A = calibration_matrix(kbp, kernel_size)
    V, _ = signal_subspace(A, eig_thresh_1)
    W = espirit_operator(V, kernel_size, nc, img_shape)
    lam, vec = np.linalg.eigh(W)                     # ascending
    lam = lam[..., ::-1][..., :nmaps]
    vec = vec[..., :, ::-1][..., :, :nmaps]          # (img..., Nc, nmaps)
    ph = vec[..., 0:1, :]
    mag = np.abs(ph)
    rot = np.where(mag > 0, np.conj(ph) / np.where(mag > 0, mag, 1.0), 1.0)
    maps = vec * rot
    maps = np.where((lam >= eig_thresh_2)[..., None, :], maps, 0.0)
    return maps, lam
