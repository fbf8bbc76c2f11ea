"""TTV, TTM and MTTKRP over {Sparse,Sparse,Sparse} / {Dense,Sparse,Sparse} tensors on the GPU
(tacogb_ttv/_dense, tacogb_ttm/_dense, tacogb_mttkrp and the taco ABI) against fixtures made by
taco's own generated code from taco's test inputs (bit-exact: integer values, every partial sum
exact) and against the oracle's restatement of taco's loops (FP64 within 1e-12 normwise
relative error; FP32 within 1e-5)."""
import ctypes
import os

import numpy as np
import pytest
import torch

import taco_gb300 as tg
from oracle import oracle as O
from taco_gb300 import taco as T
from taco_gb300 import workloads as W
from tests.helpers import normwise, taco_csf3_tensor

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
F64_TOL = 1e-12
F32_TOL = 1e-5


def fixture(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    B = (tuple(int(d) for d in g["dims"]), g["crd0"], g["pos1"], g["crd1"], g["pos2"], g["crd2"],
         g["vals"])
    return g, B


def dev_tensor(B, dtype=torch.float64, dense0=False):
    return tg.CsfTensor.from_numpy(*B, dtype=dtype, dense0=dense0)


def cu(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def fiber_coords(B):
    """(i, j) of every fiber."""
    dims, crd0, pos1, crd1 = B[:4]
    return np.repeat(crd0, np.diff(pos1)), crd1


@pytest.mark.parametrize("case", ["ttv_taco_gpu", "ttv_taco_cpu"])
def test_ttv_fixtures(case):
    g, B = fixture(case)
    Bd = dev_tensor(B)
    A = tg.ttv(Bd, cu(g["c"]), dense=True).cpu().numpy()
    assert np.array_equal(A, g["A"])
    fi, fj = fiber_coords(B)
    assert np.array_equal(tg.ttv(Bd, cu(g["c"])).cpu().numpy(), g["A"][fi, fj])


@pytest.mark.parametrize("case", ["ttm_taco_gpu", "ttm_taco_cpu"])
def test_ttm_fixtures(case):
    g, B = fixture(case)
    Bd = dev_tensor(B)
    A = tg.ttm(Bd, cu(g["C"]), dense=True).cpu().numpy()
    assert np.array_equal(A, g["A"])
    fi, fj = fiber_coords(B)
    assert np.array_equal(tg.ttm(Bd, cu(g["C"])).cpu().numpy(), g["A"][fi, fj])


@pytest.mark.parametrize("case", ["mttkrp_taco_gpu", "mttkrp_taco_cpu"])
def test_mttkrp_fixtures(case):
    g, B = fixture(case)
    A = tg.mttkrp(dev_tensor(B), cu(g["C"]), cu(g["D"])).cpu().numpy()
    assert np.array_equal(A, g["A"])


def test_mttkrp_dense_first_level():
    """taco's mttkrpCPU stores B as {Dense,Sparse,Sparse}: the same values through a dense
    level 0 (crd0 absent, one level-1 segment per i, empty ones included)."""
    g, B = fixture("mttkrp_taco_cpu")
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    full = np.zeros(dims[0] + 1, np.int64)
    full[crd0 + 1] = np.diff(pos1)
    pos1d = np.cumsum(full).astype(np.int32)
    Bd = dev_tensor((dims, np.arange(dims[0], dtype=np.int32), pos1d, crd1, pos2, crd2, vals),
                    dense0=True)
    assert np.array_equal(tg.mttkrp(Bd, cu(g["C"]), cu(g["D"])).cpu().numpy(), g["A"])


def small(dims=(300, 200, 400), fib=20.0, leaf=8.0, seed=5):
    return W.tensor3_powerlaw(dims=dims, fib_mean=fib, leaf_mean=leaf, seed=seed)


def spmv_variant_names():
    return tg.spmv_variants()


@pytest.mark.parametrize("seed", [1, 2])
def test_ttv_random(seed):
    """The library's SpMV choice and every SpMV variant on the fiber matrix."""
    B = small(seed=seed)
    c = W.dense(seed + 10, B[0][2])
    ref = O.ttv(B, c)
    Bd = dev_tensor(B)
    fi, fj = fiber_coords(B)
    for v in [-1] + list(range(len(spmv_variant_names()))):
        assert normwise(tg.ttv(Bd, cu(c), dense=True, variant=v).cpu().numpy(), ref) <= F64_TOL, v
        assert normwise(tg.ttv(Bd, cu(c), variant=v).cpu().numpy(), ref[fi, fj]) <= F64_TOL, v


@pytest.mark.parametrize("L", [1, 7, 32, 64, 100, 128])
def test_ttm_random(L):
    B = small(dims=(120, 90, 300), seed=20 + L)
    C = W.dense(L, B[0][2] * L).reshape(B[0][2], L)
    ref = O.ttm(B, C)
    Bd = dev_tensor(B)
    assert normwise(tg.ttm(Bd, cu(C), dense=True).cpu().numpy(), ref) <= F64_TOL
    fi, fj = fiber_coords(B)
    assert normwise(tg.ttm(Bd, cu(C)).cpu().numpy(), ref[fi, fj]) <= F64_TOL


# -1: the library's choice (fiber SpMM and combine); -2: the fused FP64 kernel; a named SpMM
# variant: the fiber SpMM with that variant, then the combine
MTTKRP_PATHS = [-1, -2, "merge_w512_native"]


def path_variant(p):
    return p if isinstance(p, int) else tg.spmm_variants().index(p)


@pytest.mark.parametrize("path", MTTKRP_PATHS)
@pytest.mark.parametrize("J", [1, 7, 16, 32, 33, 64, 100])
def test_mttkrp_random(J, path):
    B = small(seed=40 + J)
    dims = B[0]
    C = W.dense(J + 1, dims[1] * J).reshape(dims[1], J)
    D = W.dense(J + 2, dims[2] * J).reshape(dims[2], J)
    got = tg.mttkrp(dev_tensor(B), cu(C), cu(D), variant=path_variant(path)).cpu().numpy()
    assert normwise(got, O.mttkrp(B, C, D)) <= F64_TOL


@pytest.mark.parametrize("path", MTTKRP_PATHS)
@pytest.mark.parametrize("case", ["mttkrp_taco_gpu", "mttkrp_taco_cpu"])
def test_mttkrp_fixtures_every_path(case, path):
    g, B = fixture(case)
    A = tg.mttkrp(dev_tensor(B), cu(g["C"]), cu(g["D"]), variant=path_variant(path)).cpu().numpy()
    assert np.array_equal(A, g["A"])


def test_mttkrp_fused_range_fallback():
    """B values or D entries outside the double-float range: those batches run natively."""
    B = small(seed=123)
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    vals = vals.copy()
    vals[::97] *= 1e45
    B2 = (dims, crd0, pos1, crd1, pos2, crd2, vals)
    C = W.dense(5, dims[1] * 32).reshape(dims[1], 32)
    D = W.dense(6, dims[2] * 32).reshape(dims[2], 32)
    D2 = D.copy()
    D2[3, 4] = 1e-50
    for v in (-1, -2):
        got = tg.mttkrp(dev_tensor(B2), cu(C), cu(D), variant=v).cpu().numpy()
        assert normwise(got, O.mttkrp(B2, C, D)) <= F64_TOL
        got = tg.mttkrp(dev_tensor(B), cu(C), cu(D2), variant=v).cpu().numpy()
        assert normwise(got, O.mttkrp(B, C, D2)) <= F64_TOL


def test_sparse_first_level_with_missing_i():
    """Level 0 holding only some i: rows of A for absent i stay zero."""
    B = small(seed=77)
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    keep = np.arange(0, dims[0], 3)  # every third i
    f_lo, f_hi = pos1[keep], pos1[keep + 1]
    fib = np.concatenate([np.arange(a, b) for a, b in zip(f_lo, f_hi)])
    npos1 = np.concatenate([[0], np.cumsum(f_hi - f_lo)]).astype(np.int32)
    leaf = np.concatenate([np.arange(pos2[f], pos2[f + 1]) for f in fib])
    npos2 = np.concatenate([[0], np.cumsum(pos2[fib + 1] - pos2[fib])]).astype(np.int32)
    Bs = (dims, keep.astype(np.int32), npos1, crd1[fib], npos2, crd2[leaf], vals[leaf])
    C = W.dense(3, dims[1] * 16).reshape(dims[1], 16)
    D = W.dense(4, dims[2] * 16).reshape(dims[2], 16)
    got = tg.mttkrp(dev_tensor(Bs), cu(C), cu(D)).cpu().numpy()
    ref = O.mttkrp(Bs, C, D)
    assert normwise(got, ref) <= F64_TOL and not got[1::3].any()
    c = W.dense(5, dims[2])
    assert normwise(tg.ttv(dev_tensor(Bs), cu(c), dense=True).cpu().numpy(), O.ttv(Bs, c)) <= F64_TOL


def test_fp32():
    B = small(seed=91)
    dims = B[0]
    C = W.dense(6, dims[1] * 32).reshape(dims[1], 32)
    D = W.dense(7, dims[2] * 32).reshape(dims[2], 32)
    Bf = dev_tensor(B, dtype=torch.float32)
    got = tg.mttkrp(Bf, cu(C, torch.float32), cu(D, torch.float32)).double().cpu().numpy()
    assert normwise(got, O.mttkrp(B, C, D)) <= F32_TOL
    c = W.dense(8, dims[2])
    got = tg.ttv(Bf, cu(c, torch.float32), dense=True).double().cpu().numpy()
    assert normwise(got, O.ttv(B, c)) <= F32_TOL


def test_empty_tensor():
    e = np.zeros(0, np.int32)
    B = ((5, 6, 7), e, np.zeros(1, np.int32), e, np.zeros(1, np.int32), e, np.zeros(0))
    Bd = dev_tensor(B)
    assert not tg.mttkrp(Bd, cu(np.ones((6, 4))), cu(np.ones((7, 4)))).cpu().numpy().any()
    assert not tg.ttv(Bd, cu(np.ones(7)), dense=True).cpu().numpy().any()
    assert tg.ttm(Bd, cu(np.ones((7, 3)))).shape == (0, 3)


def test_full_size_mttkrp_rows():
    """The bench tensor (nell-2's shape, 7.7e7 nonzeros), J = 32: 200 rows of A against the
    oracle on the same rows (a sub-tensor of those i)."""
    B = W.tensor3_powerlaw()
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    J = W.MTTKRP_J
    C = W.dense(71, dims[1] * J).reshape(dims[1], J)
    D = W.dense(72, dims[2] * J).reshape(dims[2], J)
    got = tg.mttkrp(dev_tensor(B), cu(C), cu(D)).cpu().numpy()
    rows = np.random.default_rng(3).choice(dims[0], 200, replace=False)
    rows.sort()
    fib = np.concatenate([np.arange(pos1[i], pos1[i + 1]) for i in rows])
    leaf = np.concatenate([np.arange(pos2[f], pos2[f + 1]) for f in fib])
    npos1 = np.concatenate([[0], np.cumsum(pos1[rows + 1] - pos1[rows])]).astype(np.int32)
    npos2 = np.concatenate([[0], np.cumsum(pos2[fib + 1] - pos2[fib])]).astype(np.int32)
    Bs = (dims, rows.astype(np.int32), npos1, crd1[fib], npos2, crd2[leaf], vals[leaf])
    assert normwise(got[rows], O.mttkrp(Bs, C, D)[rows]) <= F64_TOL


@pytest.mark.parametrize("where", ["host", "device"])
def test_taco_abi(where):
    """tacogb_{ttv,ttm,mttkrp}_evaluate on taco_tensor_t operands, host or device arrays, and
    the drop-in modules' _shim_compute."""
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a)
        if where == "host":
            keep.append(a)
            return a
        t = torch.from_numpy(a).cuda()
        keep.append(t)
        return t

    L = tg.lib()
    P = ctypes.POINTER(ctypes.c_double)
    for pattern, case, ops in (("ttv", "ttv_taco_gpu", ["c"]), ("ttm", "ttm_taco_gpu", ["C"]),
                               ("mttkrp", "mttkrp_taco_gpu", ["C", "D"])):
        g, B = fixture(case)
        dims, crd0, pos1, crd1, pos2, crd2, vals = B
        Bt = taco_csf3_tensor((dims, arr(crd0), arr(pos1), arr(crd1), arr(pos2), arr(crd2),
                               arr(vals)))
        Ot = [T.dense(arr(g[o]), list(g[o].shape)) for o in ops]
        At = T.dense_result(list(g["A"].shape))
        fn = getattr(L, "tacogb_%s_evaluate" % pattern)
        assert fn(At.ptr, Bt.ptr, *[o.ptr for o in Ot]) == 0, L.tacogb_last_error()
        torch.cuda.synchronize()
        got = np.ctypeslib.as_array(ctypes.cast(At.vals_ptr, P), (g["A"].size,))
        assert np.array_equal(got.reshape(g["A"].shape), g["A"]), pattern
        # the drop-in module, into a result holding stale values
        M = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib",
                                     "libtacogb_%s.so" % pattern))
        out = np.full(g["A"].shape, 5.0)
        Ah = T.dense(out, list(out.shape))
        args = (ctypes.c_void_p * (2 + len(ops)))(Ah.ptr, Bt.ptr, *[o.ptr for o in Ot])
        M._shim_compute.argtypes = [ctypes.c_void_p]
        assert M._shim_compute(args) == 0
        assert np.array_equal(out, g["A"]), pattern


def test_rejects_bad_shapes():
    g, B = fixture("mttkrp_taco_gpu")
    Bt = taco_csf3_tensor(B)
    C = np.ascontiguousarray(g["C"][:, :16])  # J differs from D's
    Ct, Dt = T.dense(C, list(C.shape)), T.dense(g["D"], list(g["D"].shape))
    At = T.dense_result([g["A"].shape[0], 32])
    assert tg.lib().tacogb_mttkrp_evaluate(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) != 0


# ---- the pipelined ABI: host operands whose fiber level holds 2^23 nonzeros or more ----

def _pipelined_tensor():
    """The bench tensor's law on smaller modes: 3,000 x 2,000 x 30,000, about 9.6e6 nonzeros."""
    B = W.tensor3_powerlaw(dims=(3000, 2000, 30000), fib_mean=100.0, leaf_mean=32.0)
    assert len(B[5]) >= 1 << 23
    return B


def _abi_mttkrp(B, C, D, dtype=np.float64, dense0=False):
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    J = C.shape[1]
    Bt = taco_csf3_tensor((dims, crd0, pos1, crd1, pos2, crd2, vals.astype(dtype)), dense0=dense0)
    Cc, Dd = np.ascontiguousarray(C.astype(dtype)), np.ascontiguousarray(D.astype(dtype))
    Ct, Dt = T.dense(Cc, [dims[1], J]), T.dense(Dd, [dims[2], J])
    A = np.full((dims[0], J), np.nan, dtype)
    At = T.dense(A, [dims[0], J])
    return tg.lib().tacogb_mttkrp_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr), A


@pytest.mark.parametrize("J,dense0", [(16, False), (32, False), (32, True)])
def test_abi_pipelined_mttkrp(J, dense0):
    """The fiber level copied and multiplied by D chunk by chunk into fiber rows on the device,
    then the upper levels, C and the combine: the oracle's A, on two calls in a row."""
    B = _pipelined_tensor()
    dims = B[0]
    C = W.dense(81, dims[1] * J).reshape(dims[1], J)
    D = W.dense(82, dims[2] * J).reshape(dims[2], J)
    ref = O.mttkrp(B, C, D)
    for _ in range(2):
        rc, A = _abi_mttkrp(B, C, D, dense0=dense0)
        assert rc == 0, tg.lib().tacogb_last_error()
        assert normwise(A, ref) <= F64_TOL


def test_abi_pipelined_mttkrp_fp32():
    B = _pipelined_tensor()
    dims, J = B[0], 16
    r32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    C = W.dense(83, dims[1] * J).reshape(dims[1], J)
    D = W.dense(84, dims[2] * J).reshape(dims[2], J)
    ref = O.mttkrp(B[:6] + (r32(B[6]),), r32(C), r32(D))
    rc, A = _abi_mttkrp(B, C, D, np.float32)
    assert rc == 0, tg.lib().tacogb_last_error()
    assert normwise(A.astype(np.float64), ref) <= F32_TOL


def test_abi_pipelined_mttkrp_rejects_a_corrupt_fiber_chunk():
    B = list(_pipelined_tensor())
    dims = B[0]
    crd2 = B[5].copy()
    crd2[len(crd2) - 700] = dims[2] + 9  # in the last chunk of the fiber level
    B[5] = crd2
    J = 16
    C = W.dense(85, dims[1] * J).reshape(dims[1], J)
    D = W.dense(86, dims[2] * J).reshape(dims[2], J)
    rc, _ = _abi_mttkrp(tuple(B), C, D)
    assert rc == 1
    err = tg.lib().tacogb_last_error()
    assert b"level 2" in err and b"out of range at position %d" % (len(crd2) - 700) in err
