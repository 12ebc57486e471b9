"""Reporting of a device wait that gave up inside an apply.

The apply kernels that wait on mbarriers (the TMA / tensor-core passes) bound
every wait: one that runs out writes the operator's device error word and
returns instead of trapping.  Applies are asynchronous, so the word is read
where the library synchronises (the end of a CG solve, a batch result) and by
``NormalOperator.check``.  These tests set the word through the library's test
hook on the host; no kernel is made to time out.
"""
import numpy as np
import pytest
import torch

from tests.helpers import rand_c

pytestmark = pytest.mark.gpu


def _op(mr, seed=0, img=(32, 32), K=3, Nc=2):
    rng = np.random.default_rng(seed)
    G = tuple(2 * n for n in img)
    cells = np.flatnonzero(rng.random(int(np.prod(G))) < 0.7) + 1
    lam = rand_c(rng, (K * (K + 1) // 2, cells.size))
    cml = [rand_c(rng, img) for _ in range(Nc)]
    A = mr.NFFTNormalOp(img, lam, cells, cmaps=cml)
    b = mr.to_jl(rand_c(rng, img + (K,)), torch.complex64)
    return A, b, cml


def _set(mr, A, code):
    mr._lib.check(mr.library().mrsr_test_set_device_error(A.handle, int(code), None))


def test_check_passes_after_clean_applies(mr, cuda):
    A, b, _ = _op(mr)
    for _ in range(3):
        A @ b
    A.check()


def test_check_reports_and_clears(mr, cuda):
    A, b, _ = _op(mr)
    _set(mr, A, 1)
    with pytest.raises(mr._lib.MrsrError, match="bounded device wait"):
        A.check()
    A.check()  # cleared by the report


def test_cg_reports_the_word_and_recovers(mr, cuda):
    A, b, _ = _op(mr, seed=1)
    _set(mr, A, 1)
    with pytest.raises(mr._lib.MrsrError, match="bounded device wait"):
        mr.cg(A, b, maxiter=3, reltol=0.0)
    x = mr.cg(A, b, maxiter=3, reltol=0.0)  # the next solve runs clean
    assert np.isfinite(mr.to_host(x)).all()


def test_word_is_per_operator(mr, cuda):
    """Operators made with share() use the same kernel but their own error word."""
    A, b, cml = _op(mr, seed=2)
    B = A.share(cmaps=cml)
    _set(mr, B, 1)
    A.check()
    mr.cg(A, b, maxiter=2, reltol=0.0)
    with pytest.raises(mr._lib.MrsrError):
        B.check()


def test_batch_result_reports_the_word(mr, cuda):
    A, b, cml = _op(mr, seed=3)
    B = A.share(cmaps=cml)
    bs = [b, b.clone()]
    xs = [mr.jl_empty(b.shape, torch.complex64) for _ in bs]
    batch = mr.CgBatch([A, B], bs, xs, 3)
    batch.launch()
    torch.cuda.synchronize()
    batch.result(0)
    batch.result(1)
    _set(mr, B, 1)
    with pytest.raises(mr._lib.MrsrError, match="bounded device wait"):
        batch.result(1)
    batch.result(1)
