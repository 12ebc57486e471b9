"""Trajectory generators restated from ``src/Trajectories.jl`` (oracle copy).

Arrays use the reference's index order (``k[d, sample, frame]``); values are
float32 like the reference's default ``T=Float32``.  Float32 sin/cos are
evaluated in float64 and rounded once, which is how Julia evaluates
``sin(::Float32)``.
"""
import numpy as np


def calculate_golden_means():
    """``src/Trajectories.jl:168-174``: real eigenvector of [0 1 0; 0 0 1; 1 0 1].

    The eigenvector for the real eigenvalue l (l^3 = l^2 + 1) is (1, l, l^2),
    so gm1 = 1/l^2 and gm2 = 1/l.
    """
    M = np.array([[0, 1, 0], [0, 0, 1], [1, 0, 1]], dtype=np.float64)
    w, v = np.linalg.eig(M)
    i = int(np.argmax(w.real))
    vec = v[:, i].real
    return vec[0] / vec[2], vec[1] / vec[2]


def traj_kooshball(Nr, theta, phi, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0)):
    """``src/Trajectories.jl:108-154``. ``theta``/``phi`` have shape (Ncyc, Nt)."""
    theta = np.asarray(theta)
    phi = np.asarray(phi)
    assert theta.dtype == phi.dtype
    T = theta.dtype
    Ncyc, Nt = theta.shape
    kr = (np.arange(Nr, dtype=np.float64) - (Nr - 1) / 2) / Nr
    if T == np.float32:
        trig = lambda f, a: f(a.astype(np.float64)).astype(np.float32)
    else:
        trig = lambda f, a: f(a)
    st, ct, sp, cp = trig(np.sin, theta), trig(np.cos, theta), trig(np.sin, phi), trig(np.cos, phi)
    # k[d, ic, ir, it]; the flattened sample index is ir + Nr*ic (column-major)
    k = np.empty((3, Ncyc, Nr, Nt), dtype=T)
    if thetaRot == 0 and phiRot == 0:
        # (-s*c) in the element type, then promoted to Float64 by the Float64 kr
        a1 = (-st * cp).astype(np.float64)
        a2 = (st * sp).astype(np.float64)
        a3 = ct.astype(np.float64)
        k[0] = (a1[:, None, :] * (kr[None, :, None] + delay[0])).astype(T)
        k[1] = (a2[:, None, :] * (kr[None, :, None] + delay[1])).astype(T)
        k[2] = (a3[:, None, :] * (kr[None, :, None] + delay[2])).astype(T)
    else:
        str_, ctr = np.sin(thetaRot), np.cos(thetaRot)
        spr, cpr = np.sin(phiRot), np.cos(phiRot)
        st64, ct64, sp64, cp64 = (a.astype(np.float64) for a in (st, ct, sp, cp))
        a1 = -(cpr * cp64 * ctr * st64 - spr * sp64 * st64 + cpr * ct64 * str_)
        a2 = (cpr * sp64 * st64 + spr * (cp64 * ctr * st64 + ct64 * str_))
        a3 = (ctr * ct64 - str_ * cp64 * st64)
        k[0] = (a1[:, None, :] * (kr[None, :, None] + delay[0])).astype(T)
        k[1] = (a2[:, None, :] * (kr[None, :, None] + delay[1])).astype(T)
        k[2] = (a3[:, None, :] * (kr[None, :, None] + delay[2])).astype(T)
    k = np.clip(k, -0.5, 0.5)
    return k.reshape(3, Nr * Ncyc, Nt)


def traj_2d_radial_goldenratio(Nr, Ncyc, Nt, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0), N=1):
    """``src/Trajectories.jl:81-93``: 2D golden-angle radial, phi starting at 0.

    phi[i] = i * angle_GR with angle_GR = Float32(pi/(tau+N-1)); the product is
    formed exactly and rounded once to float32 (Julia range arithmetic).
    """
    tau = (np.sqrt(5.0) + 1) / 2
    angle = np.float32(np.pi / (tau + N - 1))
    phi = (np.arange(Ncyc * Nt, dtype=np.float64) * np.float64(angle)).astype(np.float32)
    phi = phi.reshape(Ncyc, Nt)          # == reshape(phi, Nt, Ncyc)' in Julia
    theta = np.full_like(phi, np.float32(np.pi / 2))
    k = traj_kooshball(Nr, theta, phi, thetaRot, phiRot, delay)
    return np.ascontiguousarray(k[:2])


def traj_kooshball_goldenratio(Nr, Ncyc, Nt, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0)):
    """``src/Trajectories.jl:51-60``: 3D golden-means koosh ball (float64 angles)."""
    gm1, gm2 = calculate_golden_means()
    i = np.arange(Ncyc * Nt, dtype=np.float64)
    theta = np.arccos(np.mod(i * gm1, 1.0)).reshape(Ncyc, Nt)
    phi = (i * 2 * np.pi * gm2).reshape(Ncyc, Nt)
    return traj_kooshball(Nr, theta, phi, thetaRot, phiRot, delay)


def traj_cartesian(Nx, Ny, Nz, Nt, T=np.int64):
    """``src/Trajectories.jl:15-33``."""
    if np.issubdtype(np.dtype(T), np.integer):
        kx, ky, kz = (np.arange(1, n + 1) for n in (Nx, Ny, Nz))
    else:
        kx, ky, kz = (np.arange(-n / 2, n / 2) / n for n in (Nx, Ny, Nz))
    gx, gy, gz = np.meshgrid(kx, ky, kz, indexing="ij")
    ki = np.stack([gx.reshape(-1, order="F"), gy.reshape(-1, order="F"), gz.reshape(-1, order="F")])
    return np.repeat(ki[:, :, None], Nt, axis=2).astype(T)
