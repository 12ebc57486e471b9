"""Float64 restatement of ``src/GROG.jl`` (GROG calibration and gridding).

The grid indices are integer work and must be bit-exact: ``grog_index`` follows
``src/GROG.jl:89-94`` operation by operation with Julia's promotion rules
(Float32 * Int -> Float32, Float32 + 1/2 -> Float64, ``round`` ties to even,
Float64 shift).  ``oracle/grog_index.c`` is the same restatement in C and is
cross-checked against this one in the tests.
"""
import numpy as np
import scipy.linalg as sla


def grog_index(trj, img_shape, Nr):
    """Returns (idx int32 (d, Ns, Nt), shift float64 (d, Ns, Nt))."""
    trj = np.asarray(trj, dtype=np.float32)
    d = trj.shape[0]
    idx = np.empty(trj.shape, dtype=np.int32)
    shift = np.empty(trj.shape, dtype=np.float64)
    for i in range(d):
        n = int(img_shape[i])
        p = trj[i] * np.float32(n)                   # Float32 * Int -> Float32
        t = p.astype(np.float64) + 0.5               # Float32 + Float64(1/2) -> Float64
        k = np.rint(t)                               # round(): ties to even
        shift[i] = ((k - t) * np.float64(Nr)) / np.float64(n)
        idx[i] = (k.astype(np.int64) + n // 2).astype(np.int32)
    return idx, shift


def _logm_eig(X):
    """Principal logarithm of a batch of diagonalisable matrices, V diag(log lambda) V^-1."""
    lam, V = np.linalg.eig(X)
    return np.einsum("pij,pj,pjk->pik", V, np.log(lam), np.linalg.inv(V))


def grog_calib(data, trj, Nr, log_method="schur"):
    """``src/GROG.jl:14-51``. data (Ns, Nt, Nc[, Nrep]); returns [lnG_d (Nc, Nc)] * Nd.

    ``log_method``: "schur" takes each spoke's principal logarithm with scipy's
    inverse scaling and squaring (Schur form); "eig" with a batched
    eigendecomposition, ~50x faster for many coils and exact for diagonalisable
    spoke operators (tests pin it against "schur" on a subset of spokes).
    """
    data = np.asarray(data)
    if data.ndim == 3:
        data = data[..., None]
    Ns, Nt, Nc, Nrep = data.shape
    Nd = trj.shape[0]
    # permutedims(data, (1,2,4,3)) then reshape(data, Nr, :, Ncoil) in column-major order
    dp = np.transpose(data, (0, 1, 3, 2))                       # (Ns, Nt, Nrep, Nc)
    drs = dp.reshape((Nr, -1, Nc), order="F").astype(np.complex128)
    nspk = drs.shape[1]
    trs = np.asarray(trj, dtype=np.float32).reshape((Nd, Nr, -1), order="F")
    nm = ((trs[:, 1, :] - trs[:, 0, :]).T * np.float32(Nr)).astype(np.float64)   # (nspk/Nrep, Nd)
    nm = np.tile(nm, (Nrep, 1))
    vth = np.empty((nspk, Nc, Nc), dtype=np.complex128)
    Xt = np.empty((nspk, Nc, Nc), dtype=np.complex128)
    for ip in range(nspk):
        D = drs[:, ip, :]
        Xt[ip] = np.linalg.lstsq(D[:-1], D[1:], rcond=None)[0].T   # (D1 \ D2)^T
    if log_method == "eig":
        vth[:] = _logm_eig(Xt)
    else:
        for ip in range(nspk):
            vth[ip] = sla.logm(Xt[ip])
    lnG = np.linalg.lstsq(nm, vth.reshape(nspk, Nc * Nc), rcond=None)[0]   # (Nd, Nc*Nc)
    return [lnG[i].reshape(Nc, Nc) for i in range(Nd)]


def grog_gridding(data, trj, lnG, Nr, img_shape):
    """``src/GROG.jl:73-102``. Returns (trj_cart int32 (d,Ns,Nt), gridded data copy)."""
    data = np.array(data, dtype=np.complex128)
    if data.ndim == 3:
        data = data[..., None]
    idx, shift = grog_index(trj, img_shape, Nr)
    Ns, Nt = data.shape[:2]
    d = len(img_shape)
    L = [np.asarray(l, dtype=np.complex64) for l in lnG]
    for it in range(Nt):
        for s in range(Ns):
            for i in range(d):
                A = (shift[i, s, it] * L[i].astype(np.complex128)).astype(np.complex64).astype(np.complex128)
                data[s, it] = sla.expm(A) @ data[s, it]
    return idx, data
