"""SpMV parity on the GPU: every kernel variant against the oracle (taco's loop restated in C)
and against golden fixtures produced by taco's generated code.

Bars: FP64 values within 1e-12 normwise relative error (summation order only); the FP32
compensated path within 1e-6 of the FP64 oracle on the FP64 inputs, and within 1e-7 of the FP64
oracle evaluated on the FP32-rounded inputs (what compensation buys over plain FP32 sums).
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from taco_gb300 import taco as T  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests.helpers import normwise  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
F64_TOL = 1e-12
F32_TOL = 1e-6
F32_COMP_TOL = 1e-7


def variants():
    return list(range(tg.lib().tacogb_spmv_variant_count()))


def by_prefix(prefix):
    L = tg.lib()
    return [v for v in variants() if L.tacogb_spmv_variant_name(v).decode().startswith(prefix)]


def run_dev(pos, crd, vals, x, variant, dtype=torch.float64):
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, len(x), dtype=dtype)
    xd = torch.from_numpy(x).to("cuda", dtype)
    y = tg.spmv(A, xd, variant=variant)
    torch.cuda.synchronize()
    return y.double().cpu().numpy()


@pytest.mark.parametrize("case", ["spmv_taco_rand", "spmv_uniform", "spmv_powerlaw",
                                  "spmv_empty_rows"])
@pytest.mark.parametrize("variant", variants())
def test_golden_f64(case, variant):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    y = run_dev(g["pos"], g["crd"], g["vals"], g["x"], variant)
    assert normwise(y, g["y"]) <= F64_TOL


@pytest.mark.parametrize("case", ["spmv_uniform", "spmv_powerlaw", "spmv_empty_rows"])
@pytest.mark.parametrize("variant", variants())
def test_golden_f32_compensated(case, variant):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    y = run_dev(g["pos"], g["crd"], g["vals"], g["x"], variant, torch.float32)
    assert normwise(y, g["y"]) <= F32_TOL
    v32 = g["vals"].astype(np.float32).astype(np.float64)
    x32 = g["x"].astype(np.float32).astype(np.float64)
    assert normwise(y, O.spmv(g["pos"], g["crd"], v32, x32)) <= F32_COMP_TOL


def _edge_matrices():
    rng = np.random.default_rng(3)
    out = {}
    out["empty_matrix"] = (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), 5)
    out["no_nonzeros"] = (np.zeros(1001, np.int32), np.zeros(0, np.int32), np.zeros(0), 17)
    out["one_row"] = (np.array([0, 3], np.int32), np.array([0, 4, 9], np.int32),
                      np.array([1.0, -2.0, 0.5]), 10)
    # one row spanning many merge tiles, surrounded by short rows
    cols = 50000
    lens = np.ones(4000, np.int32)
    lens[1999] = cols
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.arange(cols) if l == cols else rng.choice(cols, 1) for l in lens])
    out["long_row"] = (pos, crd.astype(np.int32), rng.uniform(-1, 1, len(crd)), cols)
    # every row length 1
    n = 70001
    out["unit_rows"] = (np.arange(n + 1, dtype=np.int32), rng.integers(0, n, n).astype(np.int32),
                        rng.uniform(-1, 1, n), n)
    # two very long rows back to back, then empties
    lens = np.zeros(300, np.int32)
    lens[0], lens[1] = 30000, 29999
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.arange(30000), np.arange(29999)]).astype(np.int32)
    out["two_long_rows"] = (pos, crd, rng.uniform(-1, 1, len(crd)), 30000)
    return out


EDGE = _edge_matrices()


@pytest.mark.parametrize("name", sorted(EDGE))
@pytest.mark.parametrize("variant", variants())
def test_edge_cases(name, variant):
    pos, crd, vals, cols = EDGE[name]
    x = W.dense(21, cols)
    y_ref = O.spmv(pos, crd, vals, x)
    y = run_dev(pos, crd, vals, x, variant)
    assert y.shape == y_ref.shape
    assert normwise(y, y_ref) <= F64_TOL
    y32 = run_dev(pos, crd, vals, x, variant, torch.float32)
    assert normwise(y32, y_ref) <= F32_TOL


@pytest.mark.parametrize("variant", variants())
def test_powerlaw_medium(variant):
    s = W.spmv_powerlaw(rows=200000)
    pos, crd, vals = W.generate(s)
    x = W.dense(22, s.cols)
    assert normwise(run_dev(pos, crd, vals, x, variant), O.spmv(pos, crd, vals, x)) <= F64_TOL


@pytest.fixture(scope="module")
def full_powerlaw():
    s = W.spmv_powerlaw()
    pos, crd, vals = W.generate(s)
    x = W.dense(23, s.cols)
    return pos, crd, vals, x


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_full_size_powerlaw(full_powerlaw, dtype):
    """4,194,304^2 power-law (~1.0e8 nnz): the merge path against the oracle at full size,
    deterministic across runs, and linear in x."""
    pos, crd, vals, x = full_powerlaw
    y_ref = O.spmv(pos, crd, vals, x)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, len(x), dtype=dtype)
    xd = torch.from_numpy(x).to("cuda", dtype)
    y1 = tg.spmv(A, xd)  # the default variant
    y2 = tg.spmv(A, xd)
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    tol = F64_TOL if dtype == torch.float64 else F32_TOL
    assert normwise(y1.double().cpu().numpy(), y_ref) <= tol
    z = torch.from_numpy(W.dense(24, len(x))).to("cuda", dtype)
    lhs = tg.spmv(A, 2 * xd - z)
    rhs = 2 * y1 - tg.spmv(A, z)
    assert normwise(lhs.double().cpu().numpy(), rhs.double().cpu().numpy()) <= 10 * tol


@pytest.mark.parametrize("name", ["wtile_dfs_ipt7", "wtile_dfs_ipt9", "wmerge_dfs_ipt7"])
def test_full_size_powerlaw_double_float(full_powerlaw, name):
    """Double-float variants (FP64 values on the FP32 pipe) at full size."""
    pos, crd, vals, x = full_powerlaw
    y_ref = O.spmv(pos, crd, vals, x)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, len(x))
    xd = torch.from_numpy(x).cuda()
    y = tg.spmv(A, xd, variant=tg.spmv_variants().index(name)).cpu().numpy()
    err = normwise(y, y_ref)
    assert err <= F64_TOL
    assert err <= 1e-13  # 46-bit significands: far inside the bar


def test_full_size_powerlaw_default_is_native(full_powerlaw):
    """The default FP64 variant accumulates with DFMA: error at the level of taco's own."""
    pos, crd, vals, x = full_powerlaw
    y_ref = O.spmv(pos, crd, vals, x)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, len(x))
    y = tg.spmv(A, torch.from_numpy(x).cuda()).cpu().numpy()
    assert normwise(y, y_ref) <= 1e-14


def test_full_size_banded():
    s = W.spmv_banded()
    pos, crd, vals = W.generate(s)
    x = W.dense(25, s.cols)
    y_ref = O.spmv(pos, crd, vals, x)
    names = tg.spmv_variants()
    for nm in ("wmerge_ipt11", "wtile_native_ipt7", "wtile_dfs_ipt9", "wpipe_s_dfs_ipt9"):
        assert normwise(run_dev(pos, crd, vals, x, names.index(nm)), y_ref) <= F64_TOL
    assert normwise(run_dev(pos, crd, vals, x, -1), y_ref) <= F64_TOL


@pytest.mark.parametrize("scale", [2.0 ** 60, 2.0 ** -60, 1e300])
def test_double_float_falls_back_outside_range(scale):
    """Tiles holding values outside [2^-40, 2^40) are recomputed with native DFMA."""
    s = W.spmv_powerlaw(rows=60000)
    pos, crd, vals = W.generate(s)
    vals = vals.copy()
    vals[len(vals) // 3: len(vals) // 3 + 5000] *= scale
    x = W.dense(26, s.cols)
    x[:100] *= 1e-20  # some x out of range too
    y_ref = O.spmv(pos, crd, vals, x)
    for variant in (2, 3, 10, 11, 13, 15, 16) + tuple(by_prefix("wmerge_dfs")):
        assert normwise(run_dev(pos, crd, vals, x, variant), y_ref) <= F64_TOL


# ------------------------------------------------------------------ taco ABI ---------------

D33A = (np.array([0, 1, 1, 3], np.int32), np.array([1, 0, 2], np.int32), np.array([2.0, 3.0, 4.0]))
D3B = np.array([2.0, 0.0, 3.0])


def _abi(fn_name, y, A, x, lib=None):
    L = lib or tg.lib()
    return getattr(L, fn_name)(y.ptr, A.ptr, x.ptr)


def test_abi_kat_host_memory():
    """expr_storage spmv KAT through tacogb_spmv_evaluate with malloc'd (host) operands."""
    A = T.csr(*D33A, [3, 3])
    X = T.dense(D3B, [3])
    Y = T.dense_result([3])
    assert _abi("tacogb_spmv_evaluate", Y, A, X) == 0
    y = np.ctypeslib.as_array(ctypes.cast(Y.vals_ptr, ctypes.POINTER(ctypes.c_double)), (3,))
    assert list(y) == [0.0, 0.0, 18.0]


def test_abi_host_and_device_memory():
    g = np.load(os.path.join(GOLDEN, "spmv_powerlaw.npz"))
    rows, cols = len(g["pos"]) - 1, len(g["x"])
    # host arrays: staged inside compute
    y = np.zeros(rows)
    Y, A, X = T.dense(y, [rows]), T.csr(g["pos"], g["crd"], g["vals"], [rows, cols]), T.dense(g["x"], [cols])
    assert _abi("tacogb_spmv_compute", Y, A, X) == 0
    assert normwise(y, g["y"]) <= F64_TOL
    # device arrays: used in place
    dev = {k: torch.from_numpy(g[k]).cuda() for k in ("pos", "crd", "vals", "x")}
    yd = torch.zeros(rows, dtype=torch.float64, device="cuda")
    Yd, Ad, Xd = (T.dense(yd, [rows]), T.csr(dev["pos"], dev["crd"], dev["vals"], [rows, cols]),
                  T.dense(dev["x"], [cols]))
    assert _abi("tacogb_spmv_compute", Yd, Ad, Xd) == 0
    assert normwise(yd.cpu().numpy(), g["y"]) <= F64_TOL


def test_dropin_module_symbols():
    """libtacogb_spmv.so exports taco's unprefixed names; compute through _shim_compute."""
    L = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib", "libtacogb_spmv.so"))
    A = T.csr(*D33A, [3, 3])
    X = T.dense(D3B, [3])
    y = np.zeros(3)
    Y = T.dense(y, [3])
    args = (ctypes.c_void_p * 3)(Y.ptr, A.ptr, X.ptr)
    L._shim_compute.argtypes = [ctypes.c_void_p]
    assert L._shim_compute(args) == 0
    assert list(y) == [0.0, 0.0, 18.0]


def test_abi_csc_operand_and_mismatch():
    """d33a's CSR arrays read as CSC ({Dense,Sparse} ordered {1,0}) are d33a transposed:
    entries (1,0)=2, (0,2)=3, (2,2)=4, so A x with x = d3b = (2,0,3) is (9, 4, 12)."""
    pos, crd, vals = D33A
    A = T.TacoTensor([3, 3], [T.MODE_DENSE, T.MODE_SPARSE], vals=vals,
                     index_arrays={1: (pos, crd)}, mode_ordering=[1, 0])
    y = np.zeros(3)
    Y, X = T.dense(y, [3]), T.dense(D3B, [3])
    assert _abi("tacogb_spmv_compute", Y, A, X) == 0, tg.lib().tacogb_last_error()
    assert list(y) == [9, 4, 12]
    Y4, A3 = T.dense(np.zeros(4), [4]), T.csr(*D33A, [3, 3])
    rc = _abi("tacogb_spmv_compute", Y4, A3, X)
    assert rc != 0 and b"rows" in tg.lib().tacogb_last_error()


@pytest.mark.parametrize("which", ["powerlaw", "banded", "small_rows", "small_bench",
                                   "small_long_row"])
def test_auto_variant_choice(which):
    """TACOGB_VARIANT_AUTO picks the local-column tiles for banded columns and the
    scattered-column tiles otherwise; below 2^21 nonzeros, the one-launch vector kernel when no
    row holds more than 32 nonzeros.  It caches the choice per matrix and computes exactly what
    the chosen variant computes."""
    s = {"powerlaw": lambda: W.spmv_powerlaw(rows=300000),
         "banded": lambda: W.spmv_banded(rows=300000),
         "small_rows": lambda: W.spec(5000, kind=W.UNIFORM, len_lo=0, len_hi=3, seed=5),
         "small_bench": W.spmv_small,
         "small_long_row": lambda: W.spec(20000, kind=W.POWERLAW, mean=8.0, len_max=2000,
                                          seed=6)}[which]()
    pos, crd, vals = W.generate(s)
    if which == "small_long_row":
        assert np.diff(pos).max() > 32
    x = W.dense(24, s.cols)
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols)
    c = A.as_csr()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    v = tg.lib().tacogb_spmv_auto_variant(ctypes.byref(c), sp)
    assert v == tg.lib().tacogb_spmv_auto_variant(ctypes.byref(c), sp)  # cached
    name = tg.spmv_variants()[v]
    expect = {"banded": "wtile_d_native_ipt9_b10", "small_rows": "vector_g4",
              "small_bench": "vector_g4"}.get(which, "wtile_d_native_ipt11")
    assert name == expect
    xd = torch.from_numpy(x).cuda()
    y_auto = tg.spmv(A, xd).cpu().numpy()
    y_v = tg.spmv(A, xd, variant=v).cpu().numpy()
    assert np.array_equal(y_auto, y_v)
    assert normwise(y_auto, O.spmv(pos, crd, vals, x)) <= F64_TOL


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_abi_pipelined_host_operands(dtype):
    """Host operands of 2^23 nonzeros or more go through the pipelined path (chunked copies,
    checks, products and returns overlapped): the oracle's result, on two calls in a row."""
    s = W.spmv_powerlaw(rows=600000)
    pos, crd, vals = W.generate(s)
    assert len(crd) >= 1 << 23
    x = W.dense(25, s.cols)
    ref = O.spmv(pos, crd, vals, x)
    v = vals.astype(dtype)
    xx = x.astype(dtype)
    for _ in range(2):
        y = np.full(s.rows, np.nan, dtype=dtype)
        At, Xt, Yt = T.csr(pos, crd, v, [s.rows, s.cols]), T.dense(xx, [s.cols]), T.dense(y, [s.rows])
        assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == 0, tg.lib().tacogb_last_error()
        assert normwise(y, ref) <= (F64_TOL if dtype == np.float64 else F32_TOL)


def _off_line(a, pinned, shift=16):
    """A host copy of a whose first element sits `shift` bytes past a 128-byte boundary, in
    pinned (torch) or pageable (numpy) memory: large host -> device copies from such addresses
    go as a short head and a 128-byte-aligned body."""
    pad = 256 // a.itemsize
    if pinned:
        buf = torch.empty(a.size + pad, dtype=torch.from_numpy(a[:0]).dtype).pin_memory()
        base = buf.data_ptr()
    else:
        buf = np.empty(a.size + pad, a.dtype)
        base = buf.ctypes.data
    off = ((shift - base) % 128) // a.itemsize
    view = buf[off:off + a.size]
    if pinned:
        view.copy_(torch.from_numpy(a))
        assert view.data_ptr() % 128 == shift
    else:
        view[:] = a
        assert view.ctypes.data % 128 == shift
    return view


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("rows", [100000, 600000])  # staged whole / pipelined (2^23 + nonzeros)
def test_abi_host_operands_off_line_boundaries(pinned, rows):
    s = W.spmv_powerlaw(rows=rows)
    pos, crd, vals = W.generate(s)
    assert (len(crd) >= 1 << 23) == (rows == 600000) and vals.nbytes >= 4 << 20
    x = W.dense(26, s.cols)
    hp, hc, hv, hx = (_off_line(a, pinned) for a in (pos, crd, vals, x))
    y = np.full(s.rows, np.nan)
    At, Xt, Yt = T.csr(hp, hc, hv, [s.rows, s.cols]), T.dense(hx, [s.cols]), T.dense(y, [s.rows])
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == 0, tg.lib().tacogb_last_error()
    assert normwise(y, O.spmv(pos, crd, vals, x)) <= F64_TOL


def _skewed_pipeline_matrix():
    """2^23 + nonzeros of which one row holds about 60 %, between long runs of empty rows: the
    pipeline's chunk boundaries fall on row starts, so several chunks are empty and the big row
    is one chunk of its own."""
    rng = np.random.default_rng(11)
    rows, cols = 200000, 8000000
    lens = np.zeros(rows, np.int64)
    live = rng.choice(rows, 20000, replace=False)
    lens[live] = rng.integers(1, 350, len(live))
    lens[123457] = 5100000
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.empty(int(pos[-1]), np.int32)
    for r in np.flatnonzero(lens):
        crd[pos[r]:pos[r + 1]] = np.sort(rng.choice(cols, int(lens[r]), replace=False))
    vals = rng.uniform(-1, 1, len(crd))
    return pos, crd, vals, cols


def test_abi_pipelined_skewed_rows():
    pos, crd, vals, cols = _skewed_pipeline_matrix()
    assert len(crd) >= 1 << 23
    rows = len(pos) - 1
    x = W.dense(27, cols)
    y = np.full(rows, np.nan)
    At, Xt, Yt = T.csr(pos, crd, vals, [rows, cols]), T.dense(x, [cols]), T.dense(y, [rows])
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == 0, tg.lib().tacogb_last_error()
    assert normwise(y, O.spmv(pos, crd, vals, x)) <= F64_TOL


def test_abi_pipelined_rejects_a_corrupt_late_chunk():
    s = W.spmv_powerlaw(rows=600000)
    pos, crd, vals = W.generate(s)
    crd = crd.copy()
    crd[len(crd) - 1000] = s.cols + 5  # in the last chunk
    x = W.dense(26, s.cols)
    y = np.zeros(s.rows)
    At, Xt, Yt = T.csr(pos, crd, vals, [s.rows, s.cols]), T.dense(x, [s.cols]), T.dense(y, [s.rows])
    assert tg.lib().tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr) == 1
    # the chunk was checked on the device; the position is the one in the whole operand
    assert b"out of range at position %d" % (len(crd) - 1000) in tg.lib().tacogb_last_error()
    # the library is usable right after
    y2 = np.zeros(s.rows)
    At2, Yt2 = T.csr(pos, W.generate(s)[1], vals, [s.rows, s.cols]), T.dense(y2, [s.rows])
    assert tg.lib().tacogb_spmv_compute(Yt2.ptr, At2.ptr, Xt.ptr) == 0
    assert normwise(y2, O.spmv(pos, W.generate(s)[1], vals, x)) <= F64_TOL
