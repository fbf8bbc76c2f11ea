"""COO -> CSR pack on the GPU (tacogb_pack_csr, tacogb_pack_taco) against the oracle's
restatement of taco's pack (sort, sum duplicates), taco's own duplicates test
(test/tests-tensor.cpp:68-79) and a fixture packed by taco itself (tests/golden/pack_taco_cli).
Indices bit-exact; values bit-exact too, since duplicates are summed in input order on both
sides (the fixture's integer values make taco's unstable order irrelevant)."""
import ctypes
import os

import numpy as np
import pytest
import torch

import taco_gb300 as tg
from oracle import oracle as O
from taco_gb300 import taco as T
from taco_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gpu_pack(rows, cols, ri, ci, v, dtype=torch.float64):
    d = lambda a, t: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", t)  # noqa: E731
    A = tg.pack_csr(rows, cols, d(ri, torch.int32), d(ci, torch.int32), d(v, dtype))
    return A.pos.cpu().numpy(), A.crd.cpu().numpy(), A.vals.double().cpu().numpy()


def assert_same(got, ref):
    assert np.array_equal(got[0], ref[0])
    assert np.array_equal(got[1], ref[1])
    assert np.array_equal(got[2], ref[2])


def test_taco_duplicates_kat():
    """taco's test tensor/duplicates: (1,2) inserted twice sums to 43."""
    pos, crd, v = gpu_pack(5, 5, [1, 2, 1], [2, 2, 2], [42.0, 10.0, 1.0])
    assert list(pos) == [0, 0, 1, 2, 2, 2]
    assert list(crd) == [2, 2]
    assert list(v) == [43.0, 10.0]


def test_taco_cli_fixture():
    g = np.load(os.path.join(GOLDEN, "pack_taco_cli.npz"))
    got = gpu_pack(int(g["rows"]), int(g["cols"]), g["ri"], g["ci"], g["v"])
    assert_same(got, (g["pos"], g["crd"], g["vals"]))


@pytest.mark.parametrize("rows,cols,n,pool", [(1, 1, 10, 1), (1, 5000, 20000, 0), (5000, 1, 20000, 0),
                                              (3000, 2000, 100000, 0), (300, 300, 50000, 2000),
                                              (70000, 90000, 1, 0), (65537, 65539, 400000, 0)])
def test_random_against_oracle(rows, cols, n, pool):
    """Random coordinates (pool > 0: drawn from `pool` distinct ones, so most repeat), random
    FP64 values: bit-exact against the oracle, which also sums duplicates in input order."""
    rng = np.random.default_rng(rows * 7 + cols + n)
    if pool:
        pr, pc = rng.integers(0, rows, pool), rng.integers(0, cols, pool)
        k = rng.integers(0, pool, n)
        ri, ci = pr[k], pc[k]
    else:
        ri, ci = rng.integers(0, rows, n), rng.integers(0, cols, n)
    v = rng.uniform(-1, 1, n)
    assert_same(gpu_pack(rows, cols, ri, ci, v), O.pack_csr(rows, cols, ri, ci, v))


def test_empty_and_fp32():
    pos, crd, v = gpu_pack(7, 3, np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0))
    assert list(pos) == [0] * 8 and len(crd) == 0
    rng = np.random.default_rng(5)
    ri, ci = rng.integers(0, 900, 30000), rng.integers(0, 700, 30000)
    v = rng.integers(-100, 100, 30000).astype(np.float64)  # exact in FP32 and in any order
    got = gpu_pack(900, 700, ri, ci, v, torch.float32)
    assert_same(got, O.pack_csr(900, 700, ri, ci, v))


@pytest.mark.parametrize("bad", [(-1, 0), (0, -1), (4, 0), (0, 6)])
def test_rejects_out_of_range(bad):
    ri = np.array([0, 1, bad[0]], np.int32)
    ci = np.array([0, 2, bad[1]], np.int32)
    with pytest.raises(tg.TacoGBError):
        gpu_pack(4, 6, ri, ci, np.ones(3))


def test_full_size_round_trip():
    """The 4,194,304-row power-law matrix's coordinates, shuffled, pack back to the matrix."""
    s = W.spmv_powerlaw()
    pos, crd, vals = W.generate(s)
    rows = np.repeat(np.arange(s.rows, dtype=np.int32), np.diff(pos))
    perm = torch.randperm(len(crd), generator=torch.Generator().manual_seed(3)).numpy()
    got = gpu_pack(s.rows, s.cols, rows[perm], crd[perm], vals[perm])
    assert_same(got, (pos, crd, vals))


def _records(ri, ci, v, fp32=False):
    dt = np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f4" if fp32 else "<f8")])
    rec = np.empty(len(ri), dtype=dt)
    rec["r"], rec["c"], rec["v"] = ri, ci, v
    return rec


@pytest.mark.parametrize("where", ["host", "device"])
def test_taco_buffer_entry(where):
    """tacogb_pack_taco on taco's coordinate-buffer layout fills a CSR taco_tensor_t."""
    rng = np.random.default_rng(9)
    rows, cols, n = 400, 300, 20000
    ri, ci = rng.integers(0, rows, n), rng.integers(0, cols, n)
    v = rng.uniform(-1, 1, n)
    rec = _records(ri, ci, v)
    buf = torch.from_numpy(rec.view(np.uint8).copy())
    if where == "device":
        buf = buf.cuda()
    Tt = T.csr_result([rows, cols])
    assert tg.lib().tacogb_pack_taco(Tt.ptr, buf.data_ptr(), n) == 0, tg.lib().tacogb_last_error()
    ref = O.pack_csr(rows, cols, ri, ci, v)
    nnz = len(ref[1])
    P = ctypes.POINTER
    if where == "device":  # managed results: readable from the host after the call
        torch.cuda.synchronize()
    pos = np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 0), P(ctypes.c_int32)), (rows + 1,))
    crd = np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 1), P(ctypes.c_int32)), (nnz,))
    val = np.ctypeslib.as_array(ctypes.cast(Tt.vals_ptr, P(ctypes.c_double)), (nnz,))
    assert_same((pos.copy(), crd.copy(), val.copy()), ref)


def test_taco_buffer_entry_large_host():
    """tacogb_pack_taco on a host buffer of the 1,048,576-row power-law matrix's coordinates,
    shuffled: the results (0.29 GB) come back into malloc'd memory by chunked copies whose pages
    host threads map first, and pack back to the matrix."""
    s = W.spmv_powerlaw(rows=1 << 20)
    pos, crd, vals = W.generate(s)
    assert len(crd) * 12 >= 64 << 20
    rows = np.repeat(np.arange(s.rows, dtype=np.int32), np.diff(pos))
    perm = np.random.default_rng(4).permutation(len(crd))
    rec = _records(rows[perm], crd[perm], vals[perm])
    Tt = T.csr_result([s.rows, s.cols])
    assert tg.lib().tacogb_pack_taco(Tt.ptr, rec.ctypes.data, len(crd)) == 0, \
        tg.lib().tacogb_last_error()
    P = ctypes.POINTER
    got = (np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 0), P(ctypes.c_int32)), (s.rows + 1,)),
           np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 1), P(ctypes.c_int32)), (len(crd),)),
           np.ctypeslib.as_array(ctypes.cast(Tt.vals_ptr, P(ctypes.c_double)), (len(crd),)))
    assert_same(got, (pos, crd, vals))


def test_taco_buffer_entry_large_host_duplicates():
    """Large host results are allocated for every record before the count of distinct ones is
    known: with many duplicates the arrays are longer than nnz, and pos, crd and values still
    equal the oracle's (duplicates summed in input order)."""
    rng = np.random.default_rng(9)
    rows, cols, n = 200000, 300000, 6000000
    pool = 2000000
    pr, pc = rng.integers(0, rows, pool), rng.integers(0, cols, pool)
    k = rng.integers(0, pool, n)
    ri, ci, v = pr[k].astype(np.int32), pc[k].astype(np.int32), rng.uniform(-1, 1, n)
    assert n * 12 >= 64 << 20
    ref = O.pack_csr(rows, cols, ri, ci, v)
    nnz = len(ref[1])
    assert nnz < n
    rec = _records(ri, ci, v)
    Tt = T.csr_result([rows, cols])
    assert tg.lib().tacogb_pack_taco(Tt.ptr, rec.ctypes.data, n) == 0, tg.lib().tacogb_last_error()
    P = ctypes.POINTER
    got = (np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 0), P(ctypes.c_int32)), (rows + 1,)),
           np.ctypeslib.as_array(ctypes.cast(Tt.index(1, 1), P(ctypes.c_int32)), (nnz,)),
           np.ctypeslib.as_array(ctypes.cast(Tt.vals_ptr, P(ctypes.c_double)), (nnz,)))
    assert_same(got, ref)


@pytest.mark.parametrize("name", ["read_general.mtx", "read_symmetric.mtx", "read_array.mtx",
                                  "read_plain.tns", "read_rua32.rb"])
def test_read_csr_matches_taco(name):
    """File -> host parse -> GPU pack equals what taco's reader and pack make of the file."""
    A = tg.read_csr(os.path.join(GOLDEN, name))
    g = np.load(os.path.join(GOLDEN, name.replace(".", "_") + ".npz"))
    pos = A.pos.cpu().numpy()
    nr = len(g["pos"]) - 1
    assert np.array_equal(pos[:nr + 1], g["pos"]) and (pos[nr:] == pos[nr]).all()
    assert np.array_equal(A.crd.cpu().numpy(), g["crd"])
    assert np.array_equal(A.vals.cpu().numpy(), g["vals"])
