"""mul! on host arrays (``mrsr_normalop_apply_host``): x is copied to the device, and the
inverse row pass stores y straight into page-locked host memory (one coil group) or y returns
by a copy.  The kernels are the device apply's, so the host apply must equal it bit for bit
on either path."""
import numpy as np
import pytest
import torch

from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _rand_c(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _op(mr, seed, img, K, Nc, precision="fp32"):
    rng = np.random.default_rng(seed)
    ng = int(np.prod([2 * n for n in img]))
    cells = np.flatnonzero(rng.random(ng) < 0.8) + 1
    lam = rng.standard_normal((K * (K + 1) // 2, cells.size)).astype(np.float32)
    cm = _rand_c(rng, img + (Nc,))
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=[cm[..., c] for c in range(Nc)], precision=precision)
    return A, rng


def _host(a):
    """column-major data of a (img..., K) array in a page-locked flat tensor"""
    t = torch.empty(a.size, dtype=torch.complex64, pin_memory=True)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))))
    return t


@pytest.mark.parametrize("img,K,Nc,precision,pinned", [
    ((256, 256), 5, 20, "fp32", True),     # y stored into host memory by the three-step row pass
    ((128, 96), 3, 6, "fp32", True),       # the same at 256-point rows
    ((32, 8, 8), 2, 3, "fp32", True),      # 3D, 64-point rows (two-step row pass)
    ((64, 256), 4, 4, "fp16-tc", True),    # tensor-core inverse row pass
    ((64, 64), 3, 2, "fp16", True),        # fp16-storage operator
    ((128, 64), 2, 3, "fp32", False),      # pageable y: copied back after the apply
    ((256, 256), 3, 40, "fp32", True),     # two coil groups: y accumulated on the device, copied back
])
def test_host_apply_equals_device_apply(mr, cuda, img, K, Nc, precision, pinned):
    A, rng = _op(mr, 11, img, K, Nc, precision)
    x = _rand_c(rng, img + (K,))
    xd = mr.to_jl(x, torch.complex64)
    yd = mr.jl_empty(xd.shape, torch.complex64)
    A.mul(yd, xd)
    xh = _host(x)
    yh = torch.full((x.size,), float("nan"), dtype=torch.complex64)
    if pinned:
        yh = yh.pin_memory()
    for _ in range(2):  # twice: the second call reuses the operator's device copy of x
        A.mul_host(yh, xh)
        torch.cuda.synchronize()
        ref = yd.permute(*reversed(range(yd.dim()))).reshape(-1).cpu()
        assert torch.equal(yh, ref)


def test_host_apply_alpha_beta(mr, cuda):
    img, K, Nc = (256, 128), 4, 5
    A, rng = _op(mr, 12, img, K, Nc)
    x = _rand_c(rng, img + (K,))
    y0 = _rand_c(rng, img + (K,))
    alpha, beta = 0.75 - 0.5j, -1.25 + 0.25j
    xd = mr.to_jl(x, torch.complex64)
    yd = mr.to_jl(y0, torch.complex64)
    A.mul(yd, xd, alpha, beta)
    yh = _host(y0)
    A.mul_host(yh, _host(x), alpha, beta)
    torch.cuda.synchronize()
    ref = yd.permute(*reversed(range(yd.dim()))).reshape(-1).cpu()
    assert rel_l2(yh.numpy(), ref.numpy()) < 1e-6


def test_host_apply_rejects_bad_arguments(mr, cuda):
    A, rng = _op(mr, 13, (16, 16), 2, 1)
    n = A.shape[0]
    good = torch.zeros(n, dtype=torch.complex64)
    with pytest.raises(ValueError):
        A.mul_host(good, torch.zeros(n, dtype=torch.complex64, device="cuda"))
    with pytest.raises(ValueError):
        A.mul_host(good, torch.zeros(n + 1, dtype=torch.complex64))
    with pytest.raises(ValueError):
        A.mul_host(good, good)
    with pytest.raises(ValueError):  # row-major (C-order) multi-dimensional data
        A.mul_host(good, torch.zeros((16, 16, 2), dtype=torch.complex64))
    # the C entry point itself: host pointers off their 8-byte ComplexF32 alignment
    lib = mr._lib.load()
    buf = torch.zeros(2 * n + 2, dtype=torch.float32).pin_memory()
    status = lib.mrsr_normalop_apply_host(A.handle, buf.data_ptr() + 4, good.data_ptr(), 1.0, 0.0, 0.0, 0.0,
                                          torch.cuda.current_stream().cuda_stream)
    assert status == mr._lib.MRSR_ERR_ARG
