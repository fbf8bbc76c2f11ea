"""Operand formats on the SpMV / SpMM path on the GPU: A DCSR ({Sparse,Sparse}) or CSC
({Dense,Sparse} ordered {1,0}), x {Sparse}, y {Sparse} (with DCSR A), through the taco ABI and the
device layer, against taco's spmv KATs (test/tests-expr_storage.cpp:873-937), fixtures made by
taco's generated code for those formats (spmv, spmmDCSRGPU inputs) and the oracle.  Indices
bit-exact; values bit-exact on integer inputs, within 1e-12 normwise otherwise."""
import ctypes
import os

import numpy as np
import pytest
import torch

import taco_gb300 as tg
from oracle import oracle as O
from taco_gb300 import _native as N
from taco_gb300 import taco as T
from taco_gb300 import workloads as W
from tests.helpers import (normwise, taco_csc_tensor, taco_dcsr_tensor, taco_sparse_vector,
                           taco_sparse_vector_result, to_csc, to_dcsr)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12
PD = ctypes.POINTER(ctypes.c_double)
PI = ctypes.POINTER(ctypes.c_int32)

# taco's d33a (test/test_tensors.cpp:205-211) and d3b (:89-94)
KP, KC, KV = np.array([0, 1, 1, 3], np.int32), np.array([1, 0, 2], np.int32), np.array([2., 3., 4.])
XI, XV = np.array([0, 2], np.int32), np.array([2., 3.])


def lib():
    return tg.lib()


def spmv_abi(At, Xt, rows, sparse_y=False):
    if sparse_y:
        Yt = taco_sparse_vector_result(rows)
    else:
        Yt = T.dense_result([rows])
    assert lib().tacogb_spmv_evaluate(Yt.ptr, At.ptr, Xt.ptr) == 0, lib().tacogb_last_error()
    torch.cuda.synchronize()
    if not sparse_y:
        return np.ctypeslib.as_array(ctypes.cast(Yt.vals_ptr, PD), (rows,)).copy()
    n = np.ctypeslib.as_array(ctypes.cast(Yt.index(0, 0), PI), (2,))[1]
    crd = np.ctypeslib.as_array(ctypes.cast(Yt.index(0, 1), PI), (n,)).copy()
    return crd, np.ctypeslib.as_array(ctypes.cast(Yt.vals_ptr, PD), (n,)).copy()


def test_kat_csr_times_sparse_vector():
    """d33a{Dense,Sparse} * d3b{Sparse} = {0,0,18}."""
    At = T.csr(KP, KC, KV, [3, 3])
    assert list(spmv_abi(At, taco_sparse_vector(XI, XV, 3), 3)) == [0, 0, 18]


def test_kat_dcsr_sparse_result():
    """d33a{Sparse,Sparse} * d3b{Sparse} = a{Sparse}: coordinates {0,2}, values {0,18}."""
    crd0, pos1 = to_dcsr(KP, KC)
    At = taco_dcsr_tensor(crd0, pos1, KC, KV, [3, 3])
    crd, vals = spmv_abi(At, taco_sparse_vector(XI, XV, 3), 3, sparse_y=True)
    assert list(crd) == [0, 2] and list(vals) == [0, 18]


def test_kat_csc_and_dcsr_dense():
    x = np.array([2., 0., 3.])
    colpos, rowidx, cv = to_csc(KP, KC, KV, 3)
    assert list(spmv_abi(taco_csc_tensor(colpos, rowidx, cv, [3, 3]), T.dense(x, [3]), 3)) == [0, 0, 18]
    crd0, pos1 = to_dcsr(KP, KC)
    assert list(spmv_abi(taco_dcsr_tensor(crd0, pos1, KC, KV, [3, 3]), T.dense(x, [3]), 3)) == [0, 0, 18]


def test_taco_generated_fixture():
    g = np.load(os.path.join(GOLDEN, "spmv_formats_taco.npz"))
    pos, crd, vals, x = g["pos"], g["crd"], g["vals"], g["x"]
    rows, cols = len(pos) - 1, len(x)
    crd0, pos1 = to_dcsr(pos, crd)
    y = spmv_abi(taco_dcsr_tensor(crd0, pos1, crd, vals, [rows, cols]), T.dense(x, [cols]), rows)
    assert normwise(y, g["y_dcsr"]) <= TOL
    colpos, rowidx, cv = to_csc(pos, crd, vals, cols)
    y = spmv_abi(taco_csc_tensor(colpos, rowidx, cv, [rows, cols]), T.dense(x, [cols]), rows)
    assert normwise(y, g["y_csc"]) <= TOL
    xi = g["xi"]
    yc, yv = spmv_abi(taco_dcsr_tensor(crd0, pos1, crd, vals, [rows, cols]),
                      taco_sparse_vector(xi, np.ascontiguousarray(x[xi]), cols), rows, sparse_y=True)
    assert np.array_equal(yc, g["ys_crd"]) and normwise(yv, g["ys_vals"]) <= TOL


@pytest.mark.parametrize("where", ["host", "device"])
def test_spmm_dcsr_fixture(where):
    """taco's spmmDCSRGPU inputs (integer values): bit-exact, taco ABI and device layer."""
    g = np.load(os.path.join(GOLDEN, "spmm_dcsr_taco_gpu.npz"))
    pos, crd, vals, B = g["pos"], g["crd"], g["vals"], g["B"]
    rows, (cols, N_) = len(pos) - 1, B.shape
    crd0, pos1 = to_dcsr(pos, crd)
    arrs = [crd0, pos1, crd, vals, np.ascontiguousarray(B)]
    if where == "device":
        arrs = [torch.from_numpy(a).cuda() for a in arrs]
    At = taco_dcsr_tensor(arrs[0], arrs[1], arrs[2], arrs[3], [rows, cols])
    Bt = T.dense(arrs[4], [cols, N_])
    C = np.full((rows, N_), 9.0)
    Ct = T.dense(C, [rows, N_])
    assert lib().tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr) == 0, lib().tacogb_last_error()
    assert np.array_equal(C, g["C"])
    d = N.Dcsr()
    dv = [torch.from_numpy(a).cuda() for a in (crd0, pos1, crd, vals)]
    d.rows, d.cols, d.n0, d.nnz = rows, cols, len(crd0), len(crd)
    d.crd0, d.pos, d.crd, d.vals = [t.data_ptr() for t in dv]
    d.vtype = 0
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    Cd = torch.empty(rows, N_, dtype=torch.float64, device="cuda")
    assert lib().tacogb_spmm_dcsr(ctypes.byref(d), N_, Bd.data_ptr(), Cd.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(Cd.cpu().numpy(), g["C"])


def sparse_rows_matrix(rows, cols, seed, frac=0.2, dtype=np.float64):
    """A matrix whose rows are mostly empty (frac of them stored), some long."""
    rng = np.random.default_rng(seed)
    lens = np.minimum(np.where(rng.random(rows) < frac, rng.integers(1, 60, rows), 0), cols)
    lens[rng.integers(0, rows)] = min(cols, 3000)
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens if l]).astype(np.int32)
    return pos, crd, rng.uniform(-1, 1, len(crd)).astype(dtype)


def dcsr_device(pos, crd, vals, cols, vtype=0):
    crd0, pos1 = to_dcsr(pos, crd)
    keep = [torch.from_numpy(a).cuda() for a in (crd0, pos1, crd, vals)]
    d = N.Dcsr()
    d.rows, d.cols, d.n0, d.nnz = len(pos) - 1, cols, len(crd0), len(crd)
    d.crd0, d.pos, d.crd, d.vals = [t.data_ptr() for t in keep]
    d.vtype = vtype
    return d, keep, crd0


@pytest.mark.parametrize("rows,cols", [(20000, 5000), (3000, 70000), (1, 10)])
def test_dcsr_device_layer(rows, cols):
    pos, crd, vals = sparse_rows_matrix(rows, cols, rows + cols)
    x = W.dense(7, cols)
    ref = O.spmv(pos, crd, vals, x)
    d, keep, crd0 = dcsr_device(pos, crd, vals, cols)
    xd = torch.from_numpy(x).cuda()
    y = torch.empty(rows, dtype=torch.float64, device="cuda")
    assert lib().tacogb_spmv_dcsr(ctypes.byref(d), xd.data_ptr(), y.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    assert normwise(y.cpu().numpy(), ref) <= TOL
    ys = torch.empty(len(crd0), dtype=torch.float64, device="cuda")
    assert lib().tacogb_spmv_dcsr(ctypes.byref(d), xd.data_ptr(), ys.data_ptr(), 0, None) == 0
    torch.cuda.synchronize()
    assert normwise(ys.cpu().numpy(), ref[crd0]) <= TOL


def test_dcsr_fp32():
    pos, crd, vals = sparse_rows_matrix(8000, 4000, 3, dtype=np.float32)
    x = W.dense(8, 4000)
    ref = O.spmv(pos, crd, vals.astype(np.float64), x)
    d, keep, _ = dcsr_device(pos, crd, vals, 4000, vtype=1)
    xd = torch.from_numpy(x).float().cuda()
    y = torch.empty(8000, dtype=torch.float32, device="cuda")
    assert lib().tacogb_spmv_dcsr(ctypes.byref(d), xd.data_ptr(), y.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    assert normwise(y.double().cpu().numpy(), ref) <= 1e-5


@pytest.mark.parametrize("rows,cols", [(5000, 7000), (70000, 300), (300, 1)])
def test_csc(rows, cols):
    """CSC SpMV and the GPU transpose (bit-exact against numpy), empty columns included."""
    pos, crd, vals = sparse_rows_matrix(rows, cols, 11 * rows + cols, frac=0.5)
    colpos, rowidx, cv = to_csc(pos, crd, vals, cols)
    dev = [torch.from_numpy(a).cuda() for a in (colpos, rowidx, cv)]
    p = torch.empty(rows + 1, dtype=torch.int32, device="cuda")
    c = torch.empty(len(crd), dtype=torch.int32, device="cuda")
    v = torch.empty(len(crd), dtype=torch.float64, device="cuda")
    assert lib().tacogb_csc_to_csr(rows, cols, len(crd), dev[0].data_ptr(), dev[1].data_ptr(),
                                   dev[2].data_ptr(), 0, p.data_ptr(), c.data_ptr(), v.data_ptr(),
                                   None) == 0
    assert np.array_equal(p.cpu().numpy(), pos) and np.array_equal(c.cpu().numpy(), crd)
    assert np.array_equal(v.cpu().numpy(), vals)
    a = N.Csr()
    a.rows, a.cols, a.nnz = rows, cols, len(crd)
    a.pos, a.crd, a.vals, a.vtype = dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), 0
    x = W.dense(9, cols)
    y = torch.empty(rows, dtype=torch.float64, device="cuda")
    assert lib().tacogb_spmv_csc(ctypes.byref(a), torch.from_numpy(x).cuda().data_ptr(),
                                 y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert normwise(y.cpu().numpy(), O.spmv(pos, crd, vals, x)) <= TOL


def test_csc_rejects_repeats():
    colpos = torch.tensor([0, 2], dtype=torch.int32, device="cuda")
    rowidx = torch.tensor([1, 1], dtype=torch.int32, device="cuda")
    vals = torch.ones(2, dtype=torch.float64, device="cuda")
    p = torch.empty(3, dtype=torch.int32, device="cuda")
    c = torch.empty(2, dtype=torch.int32, device="cuda")
    v = torch.empty(2, dtype=torch.float64, device="cuda")
    assert lib().tacogb_csc_to_csr(2, 1, 2, colpos.data_ptr(), rowidx.data_ptr(), vals.data_ptr(),
                                   0, p.data_ptr(), c.data_ptr(), v.data_ptr(), None) != 0


def test_sparse_x_random():
    s = W.spmv_powerlaw(rows=50000)
    pos, crd, vals = W.generate(s)
    rng = np.random.default_rng(4)
    xi = np.sort(rng.choice(s.cols, s.cols // 10, replace=False)).astype(np.int32)
    xv = rng.uniform(-1, 1, len(xi))
    xd = np.zeros(s.cols)
    xd[xi] = xv
    y = spmv_abi(T.csr(pos, crd, vals, [s.rows, s.cols]), taco_sparse_vector(xi, xv, s.cols), s.rows)
    assert normwise(y, O.spmv(pos, crd, vals, xd)) <= TOL


def _spgemm_operand(fmt, pos, crd, vals, dims):
    if fmt == "csr":
        return T.csr(pos, crd, vals, dims)
    if fmt == "dcsr":
        crd0, pos1 = to_dcsr(pos, crd)
        return taco_dcsr_tensor(crd0, pos1, crd, vals, dims)
    colpos, rowidx, cv = to_csc(pos, crd, vals, dims[1])
    if fmt == "csc":
        return taco_csc_tensor(colpos, rowidx, cv, dims)
    c0, p1 = to_dcsr(colpos, rowidx)  # DCSC: the stored columns and their ranges
    p0 = np.array([0, len(c0)], np.int32)
    t = T.TacoTensor(list(dims), [T.MODE_SPARSE, T.MODE_SPARSE], vals=cv,
                     index_arrays={0: (p0, c0), 1: (p1, rowidx)}, mode_ordering=[1, 0])
    t._keep.append(p0)
    return t


def _spgemm_abi(At, Bt, rows, cols):
    Ct = T.csr_result([rows, cols])
    assert lib().tacogb_spgemm_evaluate(Ct.ptr, At.ptr, Bt.ptr) == 0, lib().tacogb_last_error()
    torch.cuda.synchronize()
    pos = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 0), PI), (rows + 1,)).copy()
    crd = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 1), PI), (int(pos[-1]),)).copy()
    val = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, PD), (int(pos[-1]),)).copy()
    return pos, crd, val


@pytest.mark.parametrize("afmt,bfmt", [("csr", "csr"), ("dcsr", "csr"), ("dcsr", "dcsr"),
                                       ("csr", "csc"), ("dcsr", "dcsc")])
def test_spgemm_formats_taco_inputs(afmt, bfmt):
    """taco's spgemm format combinations (test/tests-scheduling-eval.cpp:655-662) on its spgemm
    inputs: the CSR result bit-exact against the fixture taco's generated code made."""
    g = np.load(os.path.join(GOLDEN, "spgemm_taco_rand.npz"))
    n = int(g["K"][0])
    At = _spgemm_operand(afmt, g["Apos"], g["Acrd"], g["Avals"], [len(g["Apos"]) - 1, n])
    Bt = _spgemm_operand(bfmt, g["Bpos"], g["Bcrd"], g["Bvals"], [n, n])
    pos, crd, val = _spgemm_abi(At, Bt, len(g["Apos"]) - 1, n)
    assert np.array_equal(pos, g["Cpos"]) and np.array_equal(crd, g["Ccrd"])
    assert np.array_equal(val, g["Cvals"])


@pytest.mark.parametrize("afmt,bfmt", [("dcsr", "dcsc"), ("csr", "csc")])
def test_spgemm_formats_empty_rows_and_columns(afmt, bfmt):
    pa, ca, va = sparse_rows_matrix(3000, 2000, 5, frac=0.3)
    pb, cb, vb = sparse_rows_matrix(2000, 2500, 6, frac=0.3)
    ref = O.spgemm(pa, ca, va, pb, cb, vb, 2500)
    pos, crd, val = _spgemm_abi(_spgemm_operand(afmt, pa, ca, va, [3000, 2000]),
                                _spgemm_operand(bfmt, pb, cb, vb, [2000, 2500]), 3000, 2500)
    assert np.array_equal(pos, ref[0]) and np.array_equal(crd, ref[1])
    assert np.array_equal(val, ref[2])
