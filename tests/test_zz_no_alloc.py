"""mrsr_cg_noalloc: the CG solve for callers that cannot let the library allocate.

Such callers (a Julia session whose CUDA.jl pool owns the device memory, a
serving loop that must not allocate after start-up) use this entry point; it
keeps its work vectors in a static device array of the library instead of
cudaMalloc'd buffers.  Its results must equal those of mrsr_cg, the regular
entry point, call after call: the shared array keeps the previous call's
contents, so a second solve in a row checks that nothing stale leaks in.
The property it exists for is checked too: across a warm call, the device's
default memory pool (where every other library buffer comes from, through
cudaMallocAsync) neither grows nor hands out a single byte.
Everything goes through the C ABI with ctypes.
"""
import ctypes as C
import gc

import numpy as np
import pytest
import torch

from oracle import normalop as onormal
from oracle import trajectories as otraj
from tests.helpers import rand_c, rel_l2

pytestmark = pytest.mark.gpu


# CUmemPool_attribute values (CUDA driver API)
_RESERVED_MEM_CURRENT, _USED_MEM_CURRENT, _USED_MEM_HIGH = 5, 7, 8


def _default_pool():
    drv = C.CDLL("libcuda.so.1")
    dev = C.c_int(0)
    assert drv.cuDeviceGet(C.byref(dev), 0) == 0
    pool = C.c_void_p()
    assert drv.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    return drv, pool


def _pool_attr(drv, pool, attr):
    v = C.c_uint64(0)
    assert drv.cuMemPoolGetAttribute(pool, attr, C.byref(v)) == 0
    return v.value


def _reset_pool_high_water(drv, pool):
    """Restart the pool's used-bytes high-water mark from its current use (a statistic of this process)."""
    zero = C.c_uint64(0)
    assert drv.cuMemPoolSetAttribute(pool, _USED_MEM_HIGH, C.byref(zero)) == 0


def _solve(lib, entry, A, b, maxiter, reltol):
    x = torch.zeros_like(b)
    it = C.c_int(0)
    rn = C.c_double(0.0)
    st = torch.cuda.current_stream().cuda_stream
    status = getattr(lib, entry)(A.handle, b.data_ptr(), x.data_ptr(), maxiter, reltol, 0.0, C.byref(it),
                                 C.byref(rn), st)
    return status, x, it.value, rn.value


def test_cg_noalloc_matches_cg_on_consecutive_calls(mr, cuda):
    lib = mr.library()
    rng = np.random.default_rng(11)
    N, K, Nc, Nt = 32, 4, 3, 10
    trj = otraj.traj_2d_radial_goldenratio(2 * N, 3, Nt)
    U = np.linalg.svd(rand_c(rng, (Nt, K)), full_matrices=False)[0].astype(np.complex64)
    cm = rand_c(rng, (N, N, Nc))
    Lam, km = onormal.calculate_kernel_noncartesian((2 * N, 2 * N), trj, U)
    A = mr.NFFTNormalOp((N, N), onormal.pack_lambda(Lam).astype(np.complex64), km,
                        cmaps=[cm[..., c] for c in range(Nc)])
    for call, (maxiter, reltol) in enumerate(((15, 0.0), (40, 1e-3))):
        b = torch.from_numpy(rand_c(rng, (N * N * K,))).cuda()
        s_ref, x_ref, it_ref, rn_ref = _solve(lib, "mrsr_cg", A, b, maxiter, reltol)
        s_new, x_new, it_new, rn_new = _solve(lib, "mrsr_cg_noalloc", A, b, maxiter, reltol)
        torch.cuda.synchronize()
        assert s_ref == 0 and s_new == 0, lib.mrsr_last_error()
        assert it_new == it_ref
        assert rel_l2(x_new.cpu().numpy(), x_ref.cpu().numpy()) < 1e-6, f"call {call}"
        assert abs(rn_new - rn_ref) <= 1e-6 * max(rn_ref, 1e-30)
    # a warm call allocates nothing: the pool's reserved and used bytes stay put, and its
    # high-water mark (which would catch a buffer allocated and freed inside the call) does
    # not rise.  Python's collector is held off so that no earlier test's buffers are freed
    # in between.
    b = torch.from_numpy(rand_c(rng, (N * N * K,))).cuda()
    x = torch.zeros_like(b)
    it = C.c_int(0)
    rn = C.c_double(0.0)
    st = torch.cuda.current_stream().cuda_stream
    drv, pool = _default_pool()
    gc.collect()
    gc.disable()
    try:
        torch.cuda.synchronize()  # every stream, the library's own included: pending frees have landed
        _reset_pool_high_water(drv, pool)
        before = (_pool_attr(drv, pool, _RESERVED_MEM_CURRENT), _pool_attr(drv, pool, _USED_MEM_CURRENT))
        status = lib.mrsr_cg_noalloc(A.handle, b.data_ptr(), x.data_ptr(), 20, 1e-4, 0.0, C.byref(it), C.byref(rn),
                                     st)
        torch.cuda.synchronize()
        after = (_pool_attr(drv, pool, _RESERVED_MEM_CURRENT), _pool_attr(drv, pool, _USED_MEM_CURRENT))
        high = _pool_attr(drv, pool, _USED_MEM_HIGH)
    finally:
        gc.enable()
    assert status == 0, lib.mrsr_last_error()
    assert after == before, f"pool (reserved, used) bytes {before} -> {after}"
    assert high <= before[1], f"pool use peaked at {high} bytes inside the call (from {before[1]})"
