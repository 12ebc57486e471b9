"""Stacked right-hand sides: ``A.stack(n)`` and ``cg_stacked``.

``reconstruct_coilwise`` (src/CoilMaps.jl:118-162) solves one system per coil on a
single rank-1 operator.  The stacked operator applies that operator to n images in one
set of launches; ``cg_stacked`` keeps one CG iteration per image.  Checks:
* every plane of a stacked apply equals the rank-1 operator's apply of that plane
  (1e-6: the same line transforms, only tiled differently), for NFFT operators with
  real and complex kernels, with coil maps, on four-step and generic grid lengths,
  2D and 3D, and for the FFT operator;
* ``cg_stacked`` equals n separate ``cg`` calls, with fixed iterations and with the
  tolerance test (the same iteration count per plane);
* the arguments the stacked path refuses.
"""
import numpy as np
import pytest
import torch

from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


def _rank1(mr, img, cplx, Nc, seed=0):
    rng = np.random.default_rng(seed)
    G = tuple(2 * n for n in img)
    cells = np.flatnonzero(rng.random(int(np.prod(G))) < 0.7) + 1
    lam = rand_c(rng, (1, cells.size)) if cplx else (rng.random((1, cells.size)) + 0.5).astype(np.float32)
    cml = [rand_c(rng, img) for _ in range(Nc)] if Nc else None
    return mr.NFFTNormalOp(img, lam, cells, cmaps=cml), rng


def _planes_match(mr, A, n, rng, tol=1e-6):
    S = A.stack(n)
    X = mr.to_jl(rand_c(rng, A.shape_img + (n,)), torch.complex64)
    Y = mr.to_host(S @ X)
    for i in range(n):
        yi = mr.to_host(A @ X[..., i])[..., 0]
        assert rel_l2(Y[..., i], yi) < tol, i
    S.close()


@pytest.mark.parametrize("img,cplx,Nc,n", [
    ((32, 32), False, 0, 32),     # the coil-wise calibration shape: 64-point lines, 32 coils
    ((32, 32), True, 2, 7),
    ((30, 20), True, 0, 5),       # 60 x 40 grid: generic kernels
    ((64, 48), False, 3, 16),
    ((16, 16, 8), True, 0, 6),    # 3D
])
def test_stacked_apply_equals_each_plane(mr, cuda, img, cplx, Nc, n):
    A, rng = _rank1(mr, img, cplx, Nc)
    _planes_match(mr, A, n, rng)


def test_stacked_fft_operator(mr, cuda):
    rng = np.random.default_rng(3)
    N, Nt = 24, 6
    M = (rng.random((N, N, Nt)) < 0.4).astype(np.float32)
    U = rng.standard_normal((Nt, 1)).astype(np.float32)
    A = mr.FFTNormalOp(M, U)
    _planes_match(mr, A, 9, rng)


@pytest.mark.parametrize("tol", [0.0, None])
def test_cg_stacked_equals_separate_cg(mr, cuda, tol):
    A, rng = _rank1(mr, (32, 32), False, 0, seed=5)
    n = 12
    S = A.stack(n)
    B = mr.to_jl(rand_c(rng, (32, 32, n)), torch.complex64)
    kw = dict(maxiter=15) if tol == 0.0 else dict(maxiter=200)
    reltol = 0.0 if tol == 0.0 else mr.solvers.DEFAULT_RELTOL
    r = mr.cg_stacked(S, B, reltol=reltol, log=True, **kw)
    X = mr.to_host(r.x)
    for i in range(n):
        ri = mr.cg(A, B[..., i], reltol=reltol, log=True, **kw)
        assert r.iters[i] == ri.iters, i
        assert abs(r.resnorm[i] - ri.resnorm) <= 1e-5 * max(ri.resnorm, 1e-30), i
        assert rel_l2(X[..., i], mr.to_host(ri.x)[..., 0]) < 1e-5, i
    if tol is None:
        assert max(r.iters) < 200  # the tolerance test ended every plane


def test_stack_refusals(mr, cuda):
    A, rng = _rank1(mr, (16, 16), True, 0)
    with pytest.raises(ValueError):
        A.stack(0)
    S = A.stack(3)
    with pytest.raises(NotImplementedError):
        S.Λ  # the kernel lives in the source operator
    with pytest.raises(NotImplementedError):
        S.stack(2)  # stacking needs a rank-1 source
    cells = np.arange(1, 200)
    A2 = mr.NFFTNormalOp((16, 16), rand_c(rng, (3, cells.size)), cells)  # K = 2
    with pytest.raises(NotImplementedError):
        A2.stack(2)
    A16 = mr.NFFTNormalOp((32, 32), rand_c(rng, (1, cells.size)), cells, precision="fp16")
    with pytest.raises(NotImplementedError):
        A16.stack(2)
    with pytest.raises(ValueError):
        mr.cg_stacked(A, mr.to_jl(rand_c(rng, (16, 16, 1)), torch.complex64))  # not a stacked operator
