"""Seeded synthetic MR-fingerprinting inputs shaped like the benchmark workloads.

* dictionary: 1000 inversion-recovery decays (1 - 2 e^{-t/T1}) e^{-t/T2} at
  t = TR (1..Nt), TR = 5 ms, T1 ~ logU[100, 3000] ms, T2 ~ logU[10, 300] ms;
* basis U: the top-K left singular vectors of the dictionary (real, (Nt, K));
* phantom: seeded random ellipses (ellipsoids in 3D), each with one
  dictionary atom and a proton density, projected onto U (coefficients
  x_k = sum_t U[t,k] x_t);
* coil maps: Gaussian magnitude centred on a ring around the object with a
  linear phase per coil, normalised to unit root-sum-of-squares per voxel
  (the pattern of test/grog_recon.jl:27-41);
* data: forward model (device type-2 NUFFT) plus complex Gaussian noise with
  sigma = 1% of the RMS signal.
The reference tests build their inputs the same way from Random.seed!(42)
(ImagePhantoms' Shepp-Logan phantom is replaced by the random ellipses).
"""
import numpy as np


def dictionary(Nt, natoms=1000, TR=5.0, seed=42):
    rng = np.random.default_rng(seed)
    T1 = np.exp(rng.uniform(np.log(100.0), np.log(3000.0), natoms))
    T2 = np.exp(rng.uniform(np.log(10.0), np.log(300.0), natoms))
    t = TR * np.arange(1, Nt + 1)
    D = (1 - 2 * np.exp(-t[:, None] / T1[None, :])) * np.exp(-t[:, None] / T2[None, :])
    return D  # (Nt, natoms) float64


def basis(D, K):
    u, s, vh = np.linalg.svd(D, full_matrices=False)
    return np.ascontiguousarray(u[:, :K].astype(np.float32))


def phantom(img_shape, D, U, n_ellipses=8, seed=42):
    """Coefficient images (img..., K) complex64 of a piecewise-constant phantom."""
    rng = np.random.default_rng(seed + 1)
    d = len(img_shape)
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in img_shape], indexing="ij")
    xt_coef = np.zeros(tuple(img_shape) + (U.shape[1],), dtype=np.complex128)
    coeff_atoms = U.astype(np.float64).T @ D  # (K, natoms)
    for e in range(n_ellipses):
        c = rng.uniform(-0.5, 0.5, d)
        ax = rng.uniform(0.1, 0.45, d)
        m = np.ones(img_shape, dtype=bool)
        r2 = sum(((g - ci) / ai) ** 2 for g, ci, ai in zip(grids, c, ax))
        m &= r2 <= 1.0
        atom = rng.integers(D.shape[1])
        pd = rng.uniform(0.3, 1.0)
        xt_coef[m] += pd * coeff_atoms[:, atom]
    phase = np.exp(1j * np.pi * 0.25 * grids[0])
    return (xt_coef * phase[..., None]).astype(np.complex64)


def coil_maps(img_shape, ncoils, seed=42):
    """(img..., ncoils) complex64 with unit root-sum-of-squares."""
    rng = np.random.default_rng(seed + 2)
    d = len(img_shape)
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in img_shape], indexing="ij")
    maps = np.empty(tuple(img_shape) + (ncoils,), dtype=np.complex128)
    for c in range(ncoils):
        ang = 2 * np.pi * c / ncoils
        if d == 2:
            centre = np.array([np.cos(ang), np.sin(ang)]) * 1.2
        else:
            z = -0.8 + 1.6 * (c + 0.5) / ncoils
            centre = np.array([np.cos(ang), np.sin(ang), z]) * 1.1
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, centre))
        mag = np.exp(-r2 / (2 * 0.9 ** 2))
        slope = rng.uniform(-1.0, 1.0, d)
        ph = np.exp(1j * np.pi * sum(s * g for s, g in zip(slope, grids)))
        maps[..., c] = mag * ph
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=-1, keepdims=True))
    return maps.astype(np.complex64)


def add_noise(data, level=0.01, seed=42):
    """data + complex Gaussian noise with sigma = level * RMS(data) (numpy or torch)."""
    import torch
    rng = np.random.default_rng(seed + 3)
    if isinstance(data, torch.Tensor):
        rms = float(torch.sqrt(torch.mean(torch.abs(data) ** 2)))
        g = torch.Generator(device=data.device).manual_seed(seed + 3)
        n = torch.randn(data.shape, dtype=torch.complex64, device=data.device, generator=g)
        return data + (level * rms) * n.to(data.dtype)
    rms = np.sqrt(np.mean(np.abs(data) ** 2))
    n = (rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape)) / np.sqrt(2)
    return (data + level * rms * n).astype(data.dtype)
