"""SpMM parity on the GPU against taco's generated code (golden fixtures) and the oracle.

Bars: FP64 (native DFMA and double-float) within 1e-12 normwise relative error of the FP64
oracle; FP32 within 1e-5 of the FP64 oracle and compensated FP32 within 1e-6 (input rounding
dominates); BF16 B with FP32 accumulation within 1e-2 (B rounded to 8 significant bits).
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
TOL = {"f64": 1e-12, "f32": 1e-5, "f32c": 1e-6, "bf16": 1e-2}


def variants():
    return list(range(tg.lib().tacogb_spmm_variant_count()))


def run(pos, crd, vals, B, variant, kind="f64"):
    if kind == "f64":
        A = tg.CsrMatrix.from_numpy(pos, crd, vals, B.shape[0])
        Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    else:
        A = tg.CsrMatrix.from_numpy(pos, crd, vals, B.shape[0], dtype=torch.float32)
        bt = torch.bfloat16 if kind == "bf16" else torch.float32
        Bd = torch.from_numpy(np.ascontiguousarray(B)).to("cuda", bt)
    C = tg.spmm(A, Bd, variant=variant)
    torch.cuda.synchronize()
    return C.double().cpu().numpy()


@pytest.mark.parametrize("case", ["spmm_taco_rand", "spmm_powerlaw_n64"])
@pytest.mark.parametrize("variant", variants())
def test_golden_f64(case, variant):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    C = run(g["pos"], g["crd"], g["vals"], g["B"], variant)
    assert normwise(C, g["C"]) <= F64_TOL


@pytest.mark.parametrize("kind", ["f32", "bf16"])
@pytest.mark.parametrize("variant", variants())
def test_golden_reduced(kind, variant):
    g = np.load(os.path.join(GOLDEN, "spmm_powerlaw_n64.npz"))
    C = run(g["pos"], g["crd"], g["vals"], g["B"], variant, kind)
    df = tg.spmm_variants()[variant].endswith("_df")
    tol = TOL["f32c"] if (kind == "f32" and df) else TOL[kind]
    assert normwise(C, g["C"]) <= tol


def _mat(name):
    rng = np.random.default_rng(7)
    if name == "long_rows":
        cols = 3000
        lens = rng.integers(0, 4, 2000).astype(np.int32)
        lens[[5, 900, 1999]] = [cols, 1500, cols]
    elif name == "empty_rows":
        cols = 500
        lens = np.zeros(4000, np.int32)
        lens[rng.choice(4000, 300, replace=False)] = rng.integers(1, 40, 300)
    else:  # "uniform"
        cols = 2000
        lens = rng.integers(1, 60, 3000).astype(np.int32)
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens]).astype(np.int32)
    return pos, crd, rng.uniform(-1, 1, len(crd)), cols


@pytest.mark.parametrize("name", ["long_rows", "empty_rows", "uniform"])
@pytest.mark.parametrize("N", [1, 3, 32, 64, 96, 256])
@pytest.mark.parametrize("variant", variants())
def test_shapes_f64(name, N, variant):
    pos, crd, vals, cols = _mat(name)
    B = W.dense(31 + N, cols * N).reshape(cols, N)
    C = run(pos, crd, vals, B, variant)
    assert normwise(C, O.spmm(pos, crd, vals, B)) <= F64_TOL


@pytest.mark.parametrize("N", [32, 64, 256])
@pytest.mark.parametrize("kind", ["f32", "bf16"])
def test_shapes_reduced(N, kind):
    pos, crd, vals, cols = _mat("long_rows")
    B = W.dense(41 + N, cols * N).reshape(cols, N)
    ref = O.spmm(pos, crd, vals, B)
    for variant in variants():
        C = run(pos, crd, vals, B, variant, kind)
        df = tg.spmm_variants()[variant].endswith("_df")
        tol = TOL["f32c"] if (kind == "f32" and df) else TOL[kind]
        assert normwise(C, ref) <= tol, (variant, normwise(C, ref))


@pytest.mark.parametrize("scale", [2.0 ** 50, 1e-30])
def test_double_float_fallback(scale):
    pos, crd, vals, cols = _mat("uniform")
    vals = vals.copy()
    vals[1000:1200] *= scale
    B = W.dense(51, cols * 64).reshape(cols, 64)
    B[7, :] *= 1e20
    ref = O.spmm(pos, crd, vals, B)
    names = tg.spmm_variants()
    for v in [i for i, nm in enumerate(names) if nm.endswith(("_df", "_dfs"))]:
        assert normwise(run(pos, crd, vals, B, v), ref) <= F64_TOL, names[v]


def test_double_float_fallback_b_only():
    """An out-of-range entry of B alone sends every tile of the pre-split product to DFMA."""
    pos, crd, vals, cols = _mat("uniform")
    B = W.dense(53, cols * 64).reshape(cols, 64)
    B[11, 5] = 1e-300
    ref = O.spmm(pos, crd, vals, B)
    names = tg.spmm_variants()
    for v in [i for i, nm in enumerate(names) if nm.endswith("_dfs")]:
        assert normwise(run(pos, crd, vals, B, v), ref) <= F64_TOL, names[v]
        # the flag is cleared: an in-range B right after is computed in double-float again
        B2 = W.dense(54, cols * 64).reshape(cols, 64)
        assert normwise(run(pos, crd, vals, B2, v), O.spmm(pos, crd, vals, B2)) <= F64_TOL


def test_medium_powerlaw_n256():
    s = W.spmm_powerlaw(rows=30000)
    pos, crd, vals = W.generate(s)
    B = W.dense(52, s.cols * 256).reshape(s.cols, 256)
    ref = O.spmm(pos, crd, vals, B)
    for variant in variants():
        assert normwise(run(pos, crd, vals, B, variant), ref) <= F64_TOL


def test_abi_matmul_kat():
    """matrix_mul KAT (test/tests-expr_storage.cpp:996-1035) through tacogb_spmm_evaluate and
    the drop-in module's _shim_compute."""
    pos, crd, vals = (np.array([0, 1, 1, 3], np.int32), np.array([1, 0, 2], np.int32),
                      np.array([2.0, 3.0, 4.0]))
    B = np.array([[10, 20, 0], [0, 0, 0], [0, 30, 0]], dtype=np.float64)
    At, Bt, Ct = T.csr(pos, crd, vals, [3, 3]), T.dense(B, [3, 3]), T.dense_result([3, 3])
    assert tg.lib().tacogb_spmm_evaluate(Ct.ptr, At.ptr, Bt.ptr) == 0
    C = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, ctypes.POINTER(ctypes.c_double)), (9,))
    assert list(C) == [0, 0, 0, 0, 0, 0, 30, 180, 0]
    L = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib", "libtacogb_spmm.so"))
    C2 = np.full((3, 3), 7.0)
    Ct2 = T.dense(C2, [3, 3])
    args = (ctypes.c_void_p * 3)(Ct2.ptr, At.ptr, Bt.ptr)
    L._shim_compute.argtypes = [ctypes.c_void_p]
    assert L._shim_compute(args) == 0
    assert list(C2.ravel()) == [0, 0, 0, 0, 0, 0, 30, 180, 0]


def test_abi_host_and_device_f64():
    g = np.load(os.path.join(GOLDEN, "spmm_powerlaw_n64.npz"))
    rows, cols, N = len(g["pos"]) - 1, g["B"].shape[0], g["B"].shape[1]
    C = np.zeros((rows, N))
    Ct, At, Bt = (T.dense(C, [rows, N]), T.csr(g["pos"], g["crd"], g["vals"], [rows, cols]),
                  T.dense(np.ascontiguousarray(g["B"]), [cols, N]))
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 0
    assert normwise(C, g["C"]) <= F64_TOL
    dev = {k: torch.from_numpy(np.ascontiguousarray(g[k])).cuda() for k in ("pos", "crd", "vals", "B")}
    Cd = torch.zeros(rows, N, dtype=torch.float64, device="cuda")
    Ctd, Atd, Btd = (T.dense(Cd, [rows, N]), T.csr(dev["pos"], dev["crd"], dev["vals"], [rows, cols]),
                     T.dense(dev["B"], [cols, N]))
    assert tg.lib().tacogb_spmm_compute(Ctd.ptr, Atd.ptr, Btd.ptr) == 0
    assert normwise(Cd.cpu().numpy(), g["C"]) <= F64_TOL


def test_abi_rejects_mismatch():
    pos, crd, vals = (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([1.0]))
    At = T.csr(pos, crd, vals, [1, 2])
    Bt = T.dense(np.zeros((3, 4)), [3, 4])
    Ct = T.dense(np.zeros((1, 4)), [1, 4])
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 1
    assert b"B has 3 rows" in tg.lib().tacogb_last_error()


_PIPE = {}


def _pipe_matrix():
    if not _PIPE:
        s = W.spmm_powerlaw(rows=300000)
        _PIPE["m"] = (s,) + tuple(W.generate(s))
    return _PIPE["m"]


def _pipe_call(pos, crd, vals, B, s, dtype):
    N = B.shape[1]
    C = np.full((s.rows, N), np.nan, dtype=dtype)
    Bt_ = np.ascontiguousarray(B.astype(dtype))
    Ct, At, Bt = (T.dense(C, [s.rows, N]), T.csr(pos, crd, vals.astype(dtype), [s.rows, s.cols]),
                  T.dense(Bt_, [s.cols, N]))
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 0, tg.lib().tacogb_last_error()
    assert not np.isnan(C).any()
    return C


@pytest.mark.parametrize("dtype,N", [(np.float64, 16), (np.float32, 16), (np.float64, 64),
                                     (np.float64, 7)])
def test_abi_pipelined_host_operands(dtype, N):
    """Host operands of 2^23 nonzeros or more go through the pipelined path (B first, then A's
    chunks copied, checked and multiplied as each lands, C returned chunk by chunk).  FP64 with
    even N multiplies every chunk over one split of B (N=64: the two-wide tile), odd N the
    tile that splits on the fly."""
    from tests.helpers import sub_rows
    s, pos, crd, vals = _pipe_matrix()
    assert len(crd) >= 1 << 23
    B = W.dense(61, s.cols * N).reshape(s.cols, N)
    idx = np.unique(np.concatenate([np.argsort(np.diff(pos))[-32:],
                                    np.random.default_rng(2).choice(s.rows, 3000, False)]))
    ref = O.spmm(*sub_rows(pos, crd, vals, idx), B)
    for _ in range(2):
        C = _pipe_call(pos, crd, vals, B, s, dtype)
        assert normwise(C[idx], ref) <= (F64_TOL if dtype == np.float64 else TOL["f32"])


def test_abi_pipelined_b_outside_double_float_range():
    """An entry of B outside the double-float range sends every chunk's tiles to native FP64
    over B; the next call, with B in range, is split and multiplied in double-float again."""
    from tests.helpers import sub_rows
    s, pos, crd, vals = _pipe_matrix()
    N = 16
    idx = np.random.default_rng(4).choice(s.rows, 3000, False)
    B = W.dense(63, s.cols * N).reshape(s.cols, N)
    B[s.cols // 2, 3] = 1e-300
    B[17, :] *= 1e30
    C = _pipe_call(pos, crd, vals, B, s, np.float64)
    assert normwise(C[idx], O.spmm(*sub_rows(pos, crd, vals, idx), B)) <= F64_TOL
    B2 = W.dense(64, s.cols * N).reshape(s.cols, N)
    C2 = _pipe_call(pos, crd, vals, B2, s, np.float64)
    assert normwise(C2[idx], O.spmm(*sub_rows(pos, crd, vals, idx), B2)) <= F64_TOL


def test_abi_pipelined_skewed_rows():
    """One row with about 60 % of the nonzeros and long runs of empty rows through the pipelined
    SpMM (empty chunks, one chunk for the big row)."""
    from tests.test_spmv_gpu import _skewed_pipeline_matrix
    pos, crd, vals, cols = _skewed_pipeline_matrix()
    rows, N = len(pos) - 1, 8
    B = np.ascontiguousarray(W.dense(65, cols * N).reshape(cols, N))
    C = np.full((rows, N), np.nan)
    Ct, At, Bt = T.dense(C, [rows, N]), T.csr(pos, crd, vals, [rows, cols]), T.dense(B, [cols, N])
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 0, tg.lib().tacogb_last_error()
    assert normwise(C, O.spmm(pos, crd, vals, B)) <= F64_TOL


@pytest.mark.parametrize("kind", ["crd_high", "pos_order"])
def test_abi_pipelined_rejects_a_corrupt_chunk(kind):
    """A corrupt chunk of the pipelined path: TACOGB_ERR_ARG naming the segment or position in
    the whole operand, and the next call with valid operands computes the oracle's result."""
    s = W.spmm_powerlaw(rows=300000)
    pos, crd, vals = W.generate(s)
    N = 8
    B = np.ascontiguousarray(W.dense(62, s.cols * N).reshape(s.cols, N))
    bad_pos, bad_crd = pos.copy(), crd.copy()
    if kind == "crd_high":
        where = len(crd) - 1000  # in the last chunk
        bad_crd[where] = s.cols + 3
        expect = b"out of range at position %d" % where
    else:
        # a middle row of a middle chunk whose segment and the next are non-empty
        i = int(np.searchsorted(pos, len(crd) // 2)) + 7
        while not (pos[i - 1] < pos[i] < pos[i + 1]):
            i += 1
        bad_pos[i] = pos[i + 1] + 1
        expect = b"pos decreases at segment %d" % i
    C = np.zeros((s.rows, N))
    Ct, At, Bt = T.dense(C, [s.rows, N]), T.csr(bad_pos, bad_crd, vals, [s.rows, s.cols]), T.dense(B, [s.cols, N])
    assert tg.lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 1
    assert expect in tg.lib().tacogb_last_error(), tg.lib().tacogb_last_error()
    C2 = np.full((s.rows, N), np.nan)
    Ct2, At2 = T.dense(C2, [s.rows, N]), T.csr(pos, crd, vals, [s.rows, s.cols])
    assert tg.lib().tacogb_spmm_compute(Ct2.ptr, At2.ptr, Bt.ptr) == 0, tg.lib().tacogb_last_error()
    idx = np.random.default_rng(3).choice(s.rows, 2000, False)
    from tests.helpers import sub_rows
    assert normwise(C2[idx], O.spmm(*sub_rows(pos, crd, vals, idx), B)) <= F64_TOL
