"""tacogb_spmv_noalloc: SpMV for callers that cannot allocate GPU memory during the call
(code under another framework's memory pool or allocator hooks, latency-critical paths where
cudaMalloc/cudaFree may synchronise the device, fixed memory budgets).  Its temporary memory is
a static device array, so its results must match the oracle and the regular entry point's on
consecutive calls that reuse that array, and problems beyond the array's size must be refused
cleanly.

This file sorts last so that a run stopping at its first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from taco_gb300 import _native as N  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = {torch.float64: 1e-12, torch.float32: 1e-6}


def _spmv_both(A, x):
    """(regular entry point, no-alloc entry point) results for the same inputs."""
    L = tg.lib()
    c = A.as_csr()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    y_ref = torch.empty(A.rows, dtype=x.dtype, device="cuda")
    y_na = torch.full((A.rows,), float("nan"), dtype=x.dtype, device="cuda")
    tg.check(L.tacogb_spmv(ctypes.byref(c), x.data_ptr(), y_ref.data_ptr(), -1, sp), "tacogb_spmv")
    tg.check(L.tacogb_spmv_noalloc(ctypes.byref(c), x.data_ptr(), y_na.data_ptr(), sp),
             "tacogb_spmv_noalloc")
    torch.cuda.synchronize()
    return y_ref.double().cpu().numpy(), y_na.double().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_matches_regular_on_consecutive_calls(dtype):
    # two different matrices and vectors back to back: the second call reuses the static
    # scratch that the first one filled
    cases = [W.spmv_powerlaw(rows=300000), W.spec(50000, kind=W.UNIFORM, len_lo=0, len_hi=40,
                                                  seed=99)]
    for k, s in enumerate(cases):
        pos, crd, vals = W.generate(s)
        A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=dtype)
        x = torch.from_numpy(W.dense(70 + k, s.cols)).to("cuda", dtype)
        y_ref, y_na = _spmv_both(A, x)
        assert not np.isnan(y_na).any()
        assert normwise(y_na, y_ref) <= TOL[dtype]
        assert normwise(y_na, O.spmv(pos, crd, vals, W.dense(70 + k, s.cols))) <= TOL[dtype]


def test_noalloc_full_size_powerlaw():
    s = W.spmv_powerlaw()
    pos, crd, vals = W.generate(s)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols)
    x = torch.from_numpy(W.dense(72, s.cols)).cuda()
    ref = O.spmv(pos, crd, vals, W.dense(72, s.cols))
    for _ in range(2):
        y_ref, y_na = _spmv_both(A, x)
        assert normwise(y_na, y_ref) <= TOL[torch.float64]
        assert normwise(y_na, ref) <= TOL[torch.float64]


@pytest.mark.parametrize("scale", [1e15, 1e-15])
def test_noalloc_values_outside_double_float_range(scale):
    # values and x entries beyond the double-float split's range (|v| >= 2^40 or < 2^-40) make
    # their merge tiles redo the tile with native FP64; the result must still match the oracle
    s = W.spec(60000, kind=W.UNIFORM, len_lo=1, len_hi=50, seed=123)
    pos, crd, vals = W.generate(s)
    vals = vals.copy()
    vals[5000:5100] *= scale
    x = W.dense(74, s.cols)
    x[17] *= scale
    ref = O.spmv(pos, crd, vals, x)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols)
    xd = torch.from_numpy(x).cuda()
    for _ in range(2):
        y_ref, y_na = _spmv_both(A, xd)
        assert normwise(y_na, ref) <= TOL[torch.float64]
        assert normwise(y_na, y_ref) <= TOL[torch.float64]


def test_noalloc_rejects_problems_beyond_static_scratch():
    c = N.Csr()
    c.rows, c.cols, c.nnz, c.vtype = 400_000_000, 400_000_000, 2_000_000_000, tg.TACOGB_F64
    rc = tg.lib().tacogb_spmv_noalloc(ctypes.byref(c), None, None, None)
    assert rc == 1  # TACOGB_ERR_ARG, before touching any pointer or the device
    assert b"static scratch" in tg.lib().tacogb_last_error()
