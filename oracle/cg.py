"""Conjugate gradients as IterativeSolvers.jl 0.9 ``cg`` runs it (float64).

Restated from that package's published algorithm (it is a dependency of the
reference, ``Project.toml:7,17``, not part of its tree): x0 = 0, r = b,
u = 0, prev = 1; each iteration u = r + (|r|^2/prev^2) u, c = A u,
alpha = |r|^2 / <u, c>, x += alpha u, r -= alpha c.  Iteration stops after
``maxiter`` steps or once |r| <= max(reltol |b|, abstol); the package default
reltol is sqrt(eps(real(eltype(b)))) = sqrt(eps(Float32)) for ComplexF32 data.
Call sites: ``test/reconstruct_radial.jl:83`` (``cg(A, vec(b), maxiter=20)``),
``src/CoilMaps.jl:136`` (``cg!`` with ``reltol=0``).
"""
import numpy as np

DEFAULT_RELTOL_F32 = float(np.sqrt(np.finfo(np.float32).eps))


def cg(apply, b, maxiter, reltol=DEFAULT_RELTOL_F32, abstol=0.0, x0=None):
    b = np.asarray(b, dtype=np.complex128).ravel(order="F")
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128).ravel(order="F")
    r = b.copy() if x0 is None else b - apply(x)
    u = np.zeros_like(b)
    residual = np.linalg.norm(r)
    tol = max(reltol * residual, abstol)
    prev = 1.0
    it = 0
    history = [residual]
    while it < maxiter and not residual <= tol:
        beta = residual ** 2 / prev ** 2
        u = r + beta * u
        c = apply(u)
        alpha = residual ** 2 / np.vdot(u, c)
        x = x + alpha * u
        r = r - alpha * c
        prev = residual
        residual = np.linalg.norm(r)
        history.append(residual)
        it += 1
    return x, it, history
