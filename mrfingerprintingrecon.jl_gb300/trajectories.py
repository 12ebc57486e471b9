"""Trajectory generators of the reference (``src/Trajectories.jl``), host side.

They produce inputs only (float32 / integer numpy arrays in the reference's
index order ``k[d, sample, frame]``); every transform runs on the device.
Float32 sines and cosines are evaluated in float64 and rounded once, as
Julia does for ``sin(::Float32)``.
"""
import numpy as np


def calculate_golden_means():
    """``src/Trajectories.jl:168-174``: (gm1, gm2) = (1/l^2, 1/l) for the real root of l^3 = l^2 + 1."""
    roots = np.roots([1.0, -1.0, 0.0, -1.0])
    lam = float(np.real(roots[np.argmin(np.abs(np.imag(roots)))]))
    return 1.0 / lam ** 2, 1.0 / lam


def _trig32(f, a):
    return f(a.astype(np.float64)).astype(np.float32)


def traj_kooshball(Nr, theta, phi, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0)):
    """``src/Trajectories.jl:108-154``; ``theta`` and ``phi`` are (Ncyc, Nt)."""
    theta, phi = np.asarray(theta), np.asarray(phi)
    if theta.dtype != phi.dtype:
        raise AssertionError("Mismatch between input types of `theta` and `phi`")
    T = theta.dtype
    Ncyc, Nt = theta.shape
    kr = (np.arange(Nr, dtype=np.float64) - (Nr - 1) / 2) / Nr
    if T == np.float32:
        st, ct, sp, cp = (_trig32(f, a) for f, a in ((np.sin, theta), (np.cos, theta), (np.sin, phi), (np.cos, phi)))
    else:
        st, ct, sp, cp = np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi)
    if thetaRot == 0 and phiRot == 0:
        a = [(-st * cp).astype(np.float64), (st * sp).astype(np.float64), ct.astype(np.float64)]
    else:
        s_t, c_t, s_p, c_p = np.sin(thetaRot), np.cos(thetaRot), np.sin(phiRot), np.cos(phiRot)
        st, ct, sp, cp = (v.astype(np.float64) for v in (st, ct, sp, cp))
        a = [-(c_p * cp * c_t * st - s_p * sp * st + c_p * ct * s_t),
             c_p * sp * st + s_p * (cp * c_t * st + ct * s_t),
             c_t * ct - s_t * cp * st]
    k = np.empty((3, Ncyc, Nr, Nt), dtype=T)
    for i in range(3):
        k[i] = (a[i][:, None, :] * (kr[None, :, None] + delay[i])).astype(T)
    return np.clip(k, -0.5, 0.5).reshape(3, Nr * Ncyc, Nt)


def traj_2d_radial_goldenratio(Nr, Ncyc, Nt, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0), N=1):
    """``src/Trajectories.jl:81-93``: golden-angle 2D radial (float32), first angle 0."""
    tau = (np.sqrt(5.0) + 1) / 2
    angle = np.float32(np.pi / (tau + N - 1))
    phi = (np.arange(Ncyc * Nt, dtype=np.float64) * np.float64(angle)).astype(np.float32).reshape(Ncyc, Nt)
    theta = np.full_like(phi, np.float32(np.pi / 2))
    return np.ascontiguousarray(traj_kooshball(Nr, theta, phi, thetaRot, phiRot, delay)[:2])


def traj_kooshball_goldenratio(Nr, Ncyc, Nt, thetaRot=0.0, phiRot=0.0, delay=(0, 0, 0)):
    """``src/Trajectories.jl:51-60``: 3D golden-means koosh ball (float64, like the reference)."""
    gm1, gm2 = calculate_golden_means()
    i = np.arange(Ncyc * Nt, dtype=np.float64)
    theta = np.arccos(np.mod(i * gm1, 1.0)).reshape(Ncyc, Nt)
    phi = (i * 2 * np.pi * gm2).reshape(Ncyc, Nt)
    return traj_kooshball(Nr, theta, phi, thetaRot, phiRot, delay)


def traj_cartesian(Nx, Ny, Nz, Nt, T=np.int64):
    """``src/Trajectories.jl:15-33``: integer grid (1..N) or float (-1/2 .. 1/2)."""
    integer = np.issubdtype(np.dtype(T), np.integer)
    axes = [np.arange(1, n + 1) if integer else np.arange(-n / 2, n / 2) / n for n in (Nx, Ny, Nz)]
    g = np.meshgrid(*axes, indexing="ij")
    ki = np.stack([v.reshape(-1, order="F") for v in g])
    return np.repeat(ki[:, :, None], Nt, axis=2).astype(T)
