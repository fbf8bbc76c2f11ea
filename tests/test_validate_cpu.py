"""Index validation at the taco-ABI boundary, on the CPU (no GPU is touched).

taco's pack makes pos/crd valid by construction (src/tensor.cpp:295-463) and its generated
kernels trust them; libtacogb's taco-ABI entry points check every compressed level they receive
before any kernel gathers through it.  Host-resident levels are checked by host threads, so
these tests hand corrupt taco_tensor_t's with numpy arrays to the entry points and expect
TACOGB_ERR_ARG with a message naming the fault, whether or not a GPU is present.
"""
import numpy as np
import pytest

import taco_gb300 as tg
from taco_gb300 import taco as T
from taco_gb300 import workloads as W

ERR_ARG = 1


def _csr(rows=200, cols=300, seed=3):
    s = W.spec(rows, cols=cols, kind=W.UNIFORM, len_lo=0, len_hi=12, seed=seed)
    return W.generate(s) + (cols,)


def _corrupt(kind, pos, crd):
    pos, crd = pos.copy(), crd.copy()
    rows = len(pos) - 1
    long_row = int(np.argmax(np.diff(pos)))
    a, b = pos[long_row], pos[long_row + 1]
    if kind == "pos0":
        pos[0] = 1
    elif kind == "pos_order":
        pos[rows // 2] = pos[rows // 2 + 1] + 1
    elif kind == "crd_high":
        crd[a + 1] = 10 ** 6
    elif kind == "crd_negative":
        crd[b - 1] = -1
    elif kind == "crd_unsorted":
        crd[a], crd[a + 1] = crd[a + 1], crd[a]
    elif kind == "crd_duplicate":
        crd[a + 1] = crd[a]
    return pos, crd


KINDS = ["pos0", "pos_order", "crd_high", "crd_negative", "crd_unsorted", "crd_duplicate"]
MESSAGES = {"pos0": b"pos[0]", "pos_order": b"pos decreases", "crd_high": b"out of range",
            "crd_negative": b"out of range", "crd_unsorted": b"not strictly increasing",
            "crd_duplicate": b"not strictly increasing"}


def _host_check(pos, crd, cols):
    return tg.lib().tacogb_validate_level_host(len(pos) - 1, cols, pos.ctypes.data,
                                               crd.ctypes.data, int(pos[-1]))


def test_valid_levels_pass():
    pos, crd, _, cols = _csr()
    assert _host_check(pos, crd, cols) == 0
    empty = np.zeros(6, np.int32)
    assert _host_check(empty, np.zeros(0, np.int32), 5) == 0


@pytest.mark.parametrize("kind", KINDS)
def test_host_validator_finds_each_fault(kind):
    pos, crd, _, cols = _csr()
    p, c = _corrupt(kind, pos, crd)
    assert _host_check(p, c, cols) == ERR_ARG
    assert MESSAGES[kind] in tg.lib().tacogb_last_error()


def test_pos_end_mismatch():
    pos, crd, _, cols = _csr()
    rc = tg.lib().tacogb_validate_level_host(len(pos) - 1, cols, pos.ctypes.data, crd.ctypes.data,
                                             int(pos[-1]) + 1)
    assert rc == ERR_ARG and b"pos leaves" in tg.lib().tacogb_last_error()


@pytest.mark.parametrize("kind", ["crd_high", "crd_unsorted", "pos_order"])
def test_host_validator_threads_find_a_deep_fault(kind):
    """A level large enough for the multi-threaded check, with the fault in its last rows."""
    s = W.spmv_powerlaw(rows=400000)
    pos, crd, _ = W.generate(s)
    assert _host_check(pos, crd, s.cols) == 0
    p, c = pos.copy(), crd.copy()
    i = len(p) - 50
    while p[i + 1] - p[i] < 2:
        i -= 1
    if kind == "crd_high":
        c[p[i]] = s.cols
    elif kind == "crd_unsorted":
        c[p[i]], c[p[i] + 1] = c[p[i] + 1], c[p[i]]
    else:
        p[i] = p[i + 1] + 1
    assert _host_check(p, c, s.cols) == ERR_ARG
    msg = tg.lib().tacogb_last_error().decode()
    where = int(msg.rsplit(" ", 1)[1])
    assert where == {"pos_order": i, "crd_high": p[i], "crd_unsorted": p[i] + 1}[kind]


@pytest.mark.parametrize("kind", KINDS)
def test_spmv_abi_rejects_corrupt_operand(kind):
    pos, crd, vals, cols = _csr()
    p, c = _corrupt(kind, pos, crd)
    At = T.csr(p, c, vals, [len(pos) - 1, cols])
    Xt = T.dense(np.ones(cols), [cols])
    Yt = T.dense(np.zeros(len(pos) - 1), [len(pos) - 1])
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == ERR_ARG
    err = tg.lib().tacogb_last_error()
    assert b"spmv operand A" in err and MESSAGES[kind] in err


@pytest.mark.parametrize("kind", ["crd_high", "crd_unsorted"])
def test_spmm_abi_rejects_corrupt_operand(kind):
    pos, crd, vals, cols = _csr()
    p, c = _corrupt(kind, pos, crd)
    rows, N = len(pos) - 1, 8
    At = T.csr(p, c, vals, [rows, cols])
    Bt = T.dense(np.ones((cols, N)), [cols, N])
    Ct = T.dense(np.zeros((rows, N)), [rows, N])
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == ERR_ARG
    assert b"spmm operand A" in tg.lib().tacogb_last_error()


def test_spgemm_abi_rejects_corrupt_operand():
    pos, crd, vals, _ = _csr(rows=300, cols=300)
    p, c = _corrupt("crd_high", pos, crd)
    bad, good = T.csr(p, c, vals, [300, 300]), T.csr(pos, crd, vals, [300, 300])
    Ct = T.csr_result([300, 300])
    assert tg.lib().tacogb_spgemm_assemble(Ct.ptr, bad.ptr, good.ptr) == ERR_ARG
    assert b"spgemm operand A" in tg.lib().tacogb_last_error()


def test_sddmm_abi_rejects_corrupt_pattern():
    pos, crd, vals, cols = _csr()
    p, c = _corrupt("crd_negative", pos, crd)
    rows, J = len(pos) - 1, 4
    Bt = T.csr(p, c, vals, [rows, cols])
    Ct, Dt = T.dense(np.ones((rows, J)), [rows, J]), T.dense(np.ones((J, cols)), [J, cols])
    At = T.dense(np.zeros((rows, cols)), [rows, cols])
    assert tg.lib().tacogb_sddmm_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) == ERR_ARG
    assert b"sddmm operand B" in tg.lib().tacogb_last_error()


def test_validation_can_be_turned_off():
    pos, crd, vals, cols = _csr()
    p, c = _corrupt("crd_high", pos, crd)
    At = T.csr(p, c, vals, [len(pos) - 1, cols])
    Xt = T.dense(np.ones(cols), [cols])
    Yt = T.dense(np.zeros(len(pos) - 1), [len(pos) - 1])
    L = tg.lib()
    assert L.tacogb_set_validation(0) == 1
    try:
        if not _gpu():
            # no check: the call goes on to the GPU, which this machine lacks
            assert L.tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) != ERR_ARG
    finally:
        assert L.tacogb_set_validation(1) == 0


def _gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False
