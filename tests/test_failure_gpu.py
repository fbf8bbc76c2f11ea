"""Failure detection on the GPU without a GPU fault.

* Bounded waits.  Every TMA-staged kernel waits for its copies with a bounded wait that, when it
  gives up, sets the timeout bit of the per-device status word, waits once more (bounded) for
  its copies and returns; the taco-ABI entry points turn the bit into TACOGB_ERR_TIMEOUT.  The
  wait probe (libtacogb_probe) makes such a wait run out: its mbarrier expects 16 bytes more than
  its one copy brings, a count that nothing completes.  No trap, assert, bad address or endless
  loop is involved, and the context stays usable, which the tests check by computing after it.
* Index validation on device-resident operands.  Corrupt levels in device memory are rejected
  by the check kernel before any kernel gathers through them.  Every corruption here keeps
  pos[rows] equal to the length of crd, so the check kernel's reads stay in bounds.  Host
  operands are checked on their staged copies without a wait: a failing level is rewritten
  into a harmless one before the product, and the verdict is read at the end.
"""
import ctypes
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import _native as N  # noqa: E402
from taco_gb300 import taco as T  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402
from tests.test_validate_cpu import KINDS, MESSAGES, _corrupt, _csr  # noqa: E402

pytestmark = pytest.mark.gpu
ERR_ARG, ERR_TIMEOUT = 1, 4


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _status():
    s = ctypes.c_int32(0)
    assert tg.lib().tacogb_device_status(ctypes.byref(s)) == 0
    return s.value


def _small_spmv_abi():
    pos, crd, vals, cols = _csr()
    x = W.dense(5, cols)
    y = np.zeros(len(pos) - 1)
    tensors = (T.dense(y, [len(y)]), T.csr(pos, crd, vals, [len(y), cols]), T.dense(x, [cols]))
    return tensors, y, O.spmv(pos, crd, vals, x)


def test_bounded_wait_completes_when_the_copy_arrives():
    src = torch.arange(1024, dtype=torch.int32, device="cuda")
    out = torch.full((1028,), -1, dtype=torch.int32, device="cuda")
    assert _status() == 0
    tg.check(N.probe().tacogb_probe_wait_timeout(src.data_ptr(), out.data_ptr(), 0, _stream()),
             "wait probe")
    torch.cuda.synchronize()
    assert torch.equal(out[:1024], src) and out[1024].item() == 1
    assert _status() == 0


def test_bounded_wait_gives_up_and_reports_timeout():
    src = torch.arange(1024, dtype=torch.int32, device="cuda") * 3
    out = torch.full((1028,), -1, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    tg.check(N.probe().tacogb_probe_wait_timeout(src.data_ptr(), out.data_ptr(), 16, _stream()),
             "wait probe")
    torch.cuda.synchronize()
    waited = time.perf_counter() - t0
    assert out[1024].item() == 0, "the wait should have given up"
    # the copy itself landed before the CTA exited (the second, bounded wait drained it)
    assert torch.equal(out[:1024], src)
    assert waited < 5.0
    assert _status() == 1  # TACOGB_DEV_TIMEOUT; reading clears it
    assert _status() == 0


def test_timeout_reaches_the_taco_abi_and_the_context_stays_usable():
    src = torch.zeros(1024, dtype=torch.int32, device="cuda")
    out = torch.zeros(1028, dtype=torch.int32, device="cuda")
    tg.check(N.probe().tacogb_probe_wait_timeout(src.data_ptr(), out.data_ptr(), 64, _stream()),
             "wait probe")
    torch.cuda.synchronize()
    (Yt, At, Xt), y, ref = _small_spmv_abi()
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == ERR_TIMEOUT
    assert b"timed out" in tg.lib().tacogb_last_error()
    # the word was consumed: the next call succeeds and computes the right answer
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == 0
    assert normwise(y, ref) <= 1e-12


def _device_csr_tensor(pos, crd, vals, cols):
    d = [torch.from_numpy(a).cuda() for a in (pos, crd, vals)]
    return T.csr(d[0], d[1], d[2], [len(pos) - 1, cols]), d


@pytest.mark.parametrize("kind", KINDS)
def test_device_operands_are_validated(kind):
    pos, crd, vals, cols = _csr()
    p, c = _corrupt(kind, pos, crd)
    assert p[-1] == len(c)
    At, keep = _device_csr_tensor(p, c, vals, cols)
    xd = torch.ones(cols, dtype=torch.float64, device="cuda")
    yd = torch.zeros(len(pos) - 1, dtype=torch.float64, device="cuda")
    Xt, Yt = T.dense(xd, [cols]), T.dense(yd, [len(pos) - 1])
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == ERR_ARG
    err = tg.lib().tacogb_last_error()
    assert b"spmv operand A" in err and MESSAGES[kind] in err, err
    # the device-layer check on the same arrays
    c_ = N.Csr()
    c_.rows, c_.cols, c_.nnz, c_.vtype = len(pos) - 1, cols, len(c), tg.TACOGB_F64
    c_.pos, c_.crd, c_.vals = keep[0].data_ptr(), keep[1].data_ptr(), keep[2].data_ptr()
    assert tg.lib().tacogb_csr_validate(ctypes.byref(c_), _stream()) == ERR_ARG


@pytest.mark.parametrize("op", ["spmv", "spmm"])
@pytest.mark.parametrize("kind", KINDS)
def test_host_operands_are_validated(op, kind):
    """Host operands are staged, checked on the device without a wait (a failing level is made
    harmless before the product) and the verdict read at the end: TACOGB_ERR_ARG with the
    fault, and the next call with valid operands computes the oracle's result."""
    pos, crd, vals, cols = _csr()
    p, c = _corrupt(kind, pos, crd)
    rows = len(pos) - 1
    if op == "spmv":
        x = W.dense(5, cols)
        y = np.full(rows, np.nan)
        args = lambda P, C: (T.dense(y, [rows]), T.csr(P, C, vals, [rows, cols]),  # noqa: E731
                             T.dense(x, [cols]))
        fn, ref, out = tg.lib().tacogb_spmv_compute, O.spmv(pos, crd, vals, x), y
    else:
        N = 8
        B = np.ascontiguousarray(W.dense(6, cols * N).reshape(cols, N))
        Cm = np.full((rows, N), np.nan)
        args = lambda P, C: (T.dense(Cm, [rows, N]), T.csr(P, C, vals, [rows, cols]),  # noqa: E731
                             T.dense(B, [cols, N]))
        fn, ref, out = tg.lib().tacogb_spmm_compute, O.spmm(pos, crd, vals, B), Cm
    Rt, At, Xt = args(p, c)
    assert fn(Rt.ptr, At.ptr, Xt.ptr) == ERR_ARG
    err = tg.lib().tacogb_last_error()
    assert (b"%s operand A" % op.encode()) in err and MESSAGES[kind] in err, err
    Rt, At, Xt = args(pos, crd)
    assert fn(Rt.ptr, At.ptr, Xt.ptr) == 0, tg.lib().tacogb_last_error()
    assert normwise(out, ref) <= 1e-12


def test_valid_device_operands_pass_and_compute():
    s = W.spmv_powerlaw()
    pos, crd, vals = W.generate(s)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols)
    c = A.as_csr()
    assert tg.lib().tacogb_csr_validate(ctypes.byref(c), _stream()) == 0
    x = W.dense(8, s.cols)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(s.rows, dtype=torch.float64, device="cuda")
    At = T.csr(A.pos, A.crd, A.vals, [s.rows, s.cols])
    assert tg.lib().tacogb_spmv_compute(T.dense(yd, [s.rows]).ptr, At.ptr,
                                        T.dense(xd, [s.cols]).ptr) == 0
    assert normwise(yd.cpu().numpy(), O.spmv(pos, crd, vals, x)) <= 1e-12


@pytest.mark.parametrize("which", ["A", "B"])
def test_spgemm_rejects_a_corrupt_operand(which):
    pos, crd, vals, _ = _csr(rows=300, cols=300)
    p, c = _corrupt("crd_unsorted", pos, crd)
    good, bad = T.csr(pos, crd, vals, [300, 300]), T.csr(p, c, vals, [300, 300])
    A, B = (bad, good) if which == "A" else (good, bad)
    Ct = T.csr_result([300, 300])
    assert tg.lib().tacogb_spgemm_assemble(Ct.ptr, A.ptr, B.ptr) == ERR_ARG
    assert ("spgemm operand %s" % which).encode() in tg.lib().tacogb_last_error()
    # a valid call right after
    Ct2 = T.csr_result([300, 300])
    assert tg.lib().tacogb_spgemm_evaluate(Ct2.ptr, good.ptr, good.ptr) == 0
