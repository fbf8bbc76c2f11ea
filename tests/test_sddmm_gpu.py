"""SDDMM, A(i,k) = B(i,k) * C(i,j) * D(j,k), on the GPU (tacogb_sddmm, tacogb_sddmm_dense and the
taco ABI) against fixtures made by taco's own generated code and against the oracle's
restatement of it.  Bars: bit-exact on taco's integer-valued test inputs (every partial sum is
an integer below 2^24, exact in FP64 and in the double-float pairs); FP64 within 1e-12 normwise
relative error of the oracle otherwise; FP32 within 1e-5."""
import ctypes
import os

import numpy as np
import pytest
import torch

import taco_gb300 as tg
from oracle import oracle as O
from taco_gb300 import taco as T
from taco_gb300 import workloads as W
from tests.helpers import normwise

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
F64_TOL = 1e-12
F32_TOL = 1e-5
VARIANTS = [0, 1, 2, 3]  # warp_native, warp_dfs, tma_native, tma_dfs


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def gpu_sddmm(pos, crd, vals, C, D, variant=-1, dense=False, dtype=torch.float64):
    cols = D.shape[1]
    B = tg.CsrMatrix(dev(pos, torch.int32), dev(crd, torch.int32), dev(vals, dtype), cols)
    out = tg.sddmm(B, dev(C, dtype), dev(D, dtype), dense=dense, variant=variant)
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


def fixture(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "C" in g:
        C, D = g["C"], g["D"]
    else:
        I, K = g["A"].shape
        C = W.dense(17, I * 96).reshape(I, 96)
        D = W.dense(18, 96 * K).reshape(96, K)
    return g["pos"], g["crd"], g["vals"], C, D, g["A"]


def rows_of(pos):
    return np.repeat(np.arange(len(pos) - 1), np.diff(pos))


def test_variant_names():
    assert tg.sddmm_variants() == ["warp_native", "warp_dfs", "tma_native", "tma_dfs"]


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", ["sddmm_taco_gpu", "sddmm_taco_cpu"])
def test_taco_fixtures_exact(case, variant):
    pos, crd, vals, C, D, A = fixture(case)
    assert np.array_equal(gpu_sddmm(pos, crd, vals, C, D, variant, dense=True), A)
    got = gpu_sddmm(pos, crd, vals, C, D, variant)
    assert np.array_equal(got, A[rows_of(pos), crd])


@pytest.mark.parametrize("variant", VARIANTS)
def test_powerlaw_fixture(variant):
    pos, crd, vals, C, D, A = fixture("sddmm_powerlaw_j96")
    assert normwise(gpu_sddmm(pos, crd, vals, C, D, variant, dense=True), A) <= F64_TOL
    assert normwise(gpu_sddmm(pos, crd, vals, C, D, variant), A[rows_of(pos), crd]) <= F64_TOL


def random_case(rows, cols, J, seed, mean=12.0, kind=W.POWERLAW):
    s = W.spec(rows, cols=cols, kind=kind, mean=mean, len_max=min(cols, 4096), seed=seed)
    pos, crd, vals = W.generate(s)
    C = W.dense(seed + 1, rows * J).reshape(rows, J)
    D = W.dense(seed + 2, J * cols).reshape(J, cols)
    return pos, crd, vals, C, D


# every per-lane slice and chunk shape (J <= 32, <= 64, <= 128, <= 256, <= 512) and the
# slab loop past 512, with J off the slice boundaries
@pytest.mark.parametrize("J", [1, 7, 32, 33, 64, 100, 128, 129, 256, 300, 512, 513, 1100])
@pytest.mark.parametrize("variant", VARIANTS)
def test_widths_against_oracle(J, variant):
    pos, crd, vals, C, D = random_case(700, 900, J, 1000 + J)
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    assert normwise(gpu_sddmm(pos, crd, vals, C, D, variant), ref) <= F64_TOL


@pytest.mark.parametrize("J", [16, 128, 200])
@pytest.mark.parametrize("variant", [0, 2])
def test_fp32(J, variant):
    pos, crd, vals, C, D = random_case(600, 800, J, 2000 + J)
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    got = gpu_sddmm(pos, crd, np.float32(vals), np.float32(C), np.float32(D), variant,
                    dtype=torch.float32)
    assert normwise(got, ref) <= F32_TOL


@pytest.mark.parametrize("variant", VARIANTS)
def test_ragged_rows(variant):
    """Empty rows (long runs of them, more than 32 in a batch), a single dense row, rows of
    length 1, and an nnz that is not a multiple of 32 or 256."""
    rng = np.random.default_rng(31)
    rows, cols, J = 5000, 700, 64
    lens = np.zeros(rows, np.int64)
    lens[rng.choice(rows, 150, replace=False)] = 1
    lens[2345] = cols
    lens[rows - 1] = 5
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens if l > 0])
    crd = crd.astype(np.int32)
    vals = rng.uniform(-1, 1, len(crd))
    C, D = rng.uniform(-1, 1, (rows, J)), rng.uniform(-1, 1, (J, cols))
    assert len(crd) % 32 != 0
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    assert normwise(gpu_sddmm(pos, crd, vals, C, D, variant), ref) <= F64_TOL
    A = gpu_sddmm(pos, crd, vals, C, D, variant, dense=True)
    assert normwise(A, O.sddmm(pos, crd, vals, C, D)) <= F64_TOL


def test_empty_shapes():
    pos = np.zeros(5, np.int32)
    none = np.zeros(0, np.int32)
    C, D = np.ones((4, 8)), np.ones((8, 6))
    assert gpu_sddmm(pos, none, np.zeros(0), C, D).shape == (0,)
    assert not gpu_sddmm(pos, none, np.zeros(0), C, D, dense=True).any()
    # J = 0: every value is an empty sum
    pos, crd, vals, _, _ = random_case(50, 60, 1, 77)
    out = gpu_sddmm(pos, crd, vals, np.zeros((50, 0)), np.zeros((0, 60)))
    assert out.shape == (len(crd),) and not out.any()


def test_double_float_range_fallback():
    """Values outside the double-float pairs' range in D (a flag from the transpose) or in a row
    of C (a ballot when the row is loaded) send those groups to native FP64: the result keeps
    FP64 accuracy."""
    pos, crd, vals, C, D = random_case(800, 600, 128, 4242)
    D = D.copy()
    D[5, 17] = 3e45
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    for v in (1, 3):
        assert normwise(gpu_sddmm(pos, crd, vals, C, D, v), ref) <= F64_TOL
    pos, crd, vals, C, D = random_case(800, 600, 128, 4343)
    C = C.copy()
    C[3, :] *= 1e-45
    C[400, 7] = 1e50
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    r = rows_of(pos)
    for v in (1, 3):
        got = gpu_sddmm(pos, crd, vals, C, D, v)
        for row in (3, 400):  # rows far from the rest in magnitude: compare them on their own
            m = r == row
            if m.any():
                assert normwise(got[m], ref[m]) <= F64_TOL
        assert normwise(got[(r != 3) & (r != 400)], ref[(r != 3) & (r != 400)]) <= F64_TOL
    # the next call, with all values in range, runs in double-float again
    pos, crd, vals, C, D = random_case(300, 300, 128, 4444)
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    for v in (1, 3):
        assert normwise(gpu_sddmm(pos, crd, vals, C, D, v), ref) <= F64_TOL


def test_full_size_sampled_nonzeros():
    """The 1,048,576-row power-law matrix with J = 128 (the bench workload): 20,000 nonzeros
    drawn at random against numpy dot products in FP64."""
    s = W.sddmm_powerlaw()
    pos, crd, vals = W.generate(s)
    J = W.SDDMM_J
    C = W.dense(61, s.rows * J).reshape(s.rows, J)
    D = W.dense(62, J * s.cols).reshape(J, s.cols)
    for variant in VARIANTS:
        got = gpu_sddmm(pos, crd, vals, C, D, variant)
        rng = np.random.default_rng(5)
        pick = rng.choice(len(crd), 20000, replace=False)
        r = np.searchsorted(pos, pick, side="right") - 1
        ref = vals[pick] * np.einsum("nj,jn->n", C[r], D[:, crd[pick]])
        assert normwise(got[pick], ref) <= F64_TOL


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("result", ["dense", "csr"])
def test_taco_abi(where, result):
    """tacogb_sddmm_evaluate on taco_tensor_t operands: dense I x K result (taco's test form)
    or a CSR result with B's pattern; operands in host or device memory."""
    pos, crd, vals, C, D, A = fixture("sddmm_taco_gpu")
    I, K = A.shape
    J = C.shape[1]
    keep = []

    def arr(a, dt=None):
        a = np.ascontiguousarray(a if dt is None else a.astype(dt))
        if where == "host":
            keep.append(a)
            return a
        t = torch.from_numpy(a).cuda()
        keep.append(t)
        return t

    Bt = T.csr(arr(pos, np.int32), arr(crd, np.int32), arr(vals), [I, K])
    Ct, Dt = T.dense(arr(C), [I, J]), T.dense(arr(D), [J, K])
    At = T.dense_result([I, K]) if result == "dense" else T.csr_result([I, K])
    L = tg.lib()
    assert L.tacogb_sddmm_evaluate(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) == 0, L.tacogb_last_error()
    torch.cuda.synchronize()
    P = ctypes.POINTER
    if result == "dense":
        got = np.ctypeslib.as_array(ctypes.cast(At.vals_ptr, P(ctypes.c_double)), (I * K,))
        assert np.array_equal(got.reshape(I, K), A)
    else:
        nnz = len(crd)
        gp = np.ctypeslib.as_array(ctypes.cast(At.index(1, 0), P(ctypes.c_int32)), (I + 1,))
        gc = np.ctypeslib.as_array(ctypes.cast(At.index(1, 1), P(ctypes.c_int32)), (nnz,))
        gv = np.ctypeslib.as_array(ctypes.cast(At.vals_ptr, P(ctypes.c_double)), (nnz,))
        assert np.array_equal(gp, pos) and np.array_equal(gc, crd)
        assert np.array_equal(gv, A[rows_of(pos), crd])


def test_rejects_mismatched_shapes():
    pos, crd, vals, C, D, A = fixture("sddmm_taco_gpu")
    I, K = A.shape
    Bt = T.csr(pos.astype(np.int32), crd.astype(np.int32), vals, [I, K])
    Ct = T.dense(np.ascontiguousarray(C[:, :100]), [I, 100])  # J differs from D's rows
    Dt = T.dense(np.ascontiguousarray(D), [D.shape[0], K])
    At = T.dense_result([I, K])
    assert tg.lib().tacogb_sddmm_evaluate(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) != 0


def test_dropin_module_shim_compute():
    """taco's sddmmGPU inputs through libtacogb_sddmm.so's _shim_compute (taco's packed-argument
    entry: result, then B, C, D), into a dense result holding stale values."""
    pos, crd, vals, C, D, A = fixture("sddmm_taco_gpu")
    I, K = A.shape
    J = C.shape[1]
    L = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib", "libtacogb_sddmm.so"))
    out = np.full((I, K), 7.0)
    At = T.dense(out, [I, K])
    Bt = T.csr(pos.astype(np.int32), crd.astype(np.int32), vals, [I, K])
    Ct, Dt = T.dense(np.ascontiguousarray(C), [I, J]), T.dense(np.ascontiguousarray(D), [J, K])
    args = (ctypes.c_void_p * 4)(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr)
    L._shim_compute.argtypes = [ctypes.c_void_p]
    assert L._shim_compute(args) == 0
    assert np.array_equal(out, A)


# ---- the pipelined ABI: host operands of 2^23 nonzeros or more, values at B's nonzeros ----

def _pipelined_case(J, seed, rows=300000):
    """The SDDMM power-law law (mean 32 per row) at 300,000 rows: 9.6e6 nonzeros."""
    s = W.spmm_powerlaw(rows=rows)
    pos, crd, vals = W.generate(s)
    assert len(crd) >= 1 << 23
    C = W.dense(seed, s.rows * J).reshape(s.rows, J)
    D = W.dense(seed + 1, J * s.cols).reshape(J, s.cols)
    return pos, crd, vals, C, D, s.cols


def _abi_sampled(pos, crd, vals, C, D, K, dtype=np.float64, pinned=False):
    """tacogb_sddmm_compute on host arrays (pageable numpy, or pinned torch) into a CSR result
    with B's pattern."""
    I, J = C.shape
    host = (lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()) if pinned else (
        lambda a: np.ascontiguousarray(a))
    p, c = host(pos), host(crd)
    v, Cc, Dd = host(vals.astype(dtype)), host(C.astype(dtype)), host(D.astype(dtype))
    out = host(np.full(len(crd), np.nan, dtype))
    Bt, At = T.csr(p, c, v, [I, K]), T.csr(p, c, out, [I, K])
    Ct, Dt = T.dense(Cc, [I, J]), T.dense(Dd, [J, K])
    rc = tg.lib().tacogb_sddmm_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr)
    return rc, (out.numpy() if pinned else out)


@pytest.mark.parametrize("J,pinned", [(32, False), (128, False), (128, True)])
def test_abi_pipelined_host_operands(J, pinned):
    """D copied and transposed first, then B's rows with their rows of C chunk by chunk: the
    oracle's values, on two calls in a row (pageable operands go through the copier thread)."""
    pos, crd, vals, C, D, K = _pipelined_case(J, 71)
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    for _ in range(2):
        rc, got = _abi_sampled(pos, crd, vals, C, D, K, pinned=pinned)
        assert rc == 0, tg.lib().tacogb_last_error()
        assert normwise(got, ref) <= F64_TOL


def test_abi_pipelined_fp32():
    pos, crd, vals, C, D, K = _pipelined_case(64, 73)
    r32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    ref = O.sddmm_sampled(pos, crd, r32(vals), r32(C), r32(D))
    rc, got = _abi_sampled(pos, crd, vals, C, D, K, np.float32)
    assert rc == 0, tg.lib().tacogb_last_error()
    assert normwise(got.astype(np.float64), ref) <= F32_TOL


def test_abi_pipelined_double_float_range():
    """A D value outside the double-float pairs' range, seen by the one transpose of D, sends
    every chunk's groups to native FP64."""
    pos, crd, vals, C, D, K = _pipelined_case(32, 75)
    D = D.copy()
    D[3, 1000] = 3e45
    ref = O.sddmm_sampled(pos, crd, vals, C, D)
    rc, got = _abi_sampled(pos, crd, vals, C, D, K)
    assert rc == 0, tg.lib().tacogb_last_error()
    m = crd == 1000  # the nonzeros that meet the large value, compared on their own
    assert m.any() and normwise(got[m], ref[m]) <= F64_TOL
    assert normwise(got[~m], ref[~m]) <= F64_TOL


def test_abi_pipelined_rejects_a_corrupt_late_chunk():
    pos, crd, vals, C, D, K = _pipelined_case(32, 77)
    bad = crd.copy()
    bad[len(bad) - 1000] = K + 5  # in the last chunk
    rc, _ = _abi_sampled(pos, bad, vals, C, D, K)
    assert rc == 1
    assert b"out of range at position %d" % (len(bad) - 1000) in tg.lib().tacogb_last_error()
    rc, got = _abi_sampled(pos, crd, vals, C, D, K)  # usable right after
    assert rc == 0 and normwise(got, O.sddmm_sampled(pos, crd, vals, C, D)) <= F64_TOL
