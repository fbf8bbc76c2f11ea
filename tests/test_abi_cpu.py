"""The C-ABI libraries load without a GPU and export every symbol their headers declare; the
generators are deterministic and produce valid CSR."""
import ctypes
import os
import re

import numpy as np
import pytest

import taco_gb300 as tg
from taco_gb300 import _native as N
from taco_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    """Function names declared in include/<header> (C declarations ending in ');')."""
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_libtacogb_exports_header():
    names = declared("taco_gb300.h")
    assert "tacogb_spmv" in names and "_shim_tacogb_spmv_compute" in names
    L = ctypes.CDLL(os.path.join(N.LIBDIR, "libtacogb.so"))
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(N.SIGNATURES), "bindings miss %s" % (set(names) - set(N.SIGNATURES))


def test_probe_library_exports_header():
    names = declared("taco_gb300_probe.h")
    assert names == ["tacogb_probe_gather", "tacogb_probe_wait_timeout"]
    assert set(names) == set(N.PROBE_SIGNATURES)
    product = ctypes.CDLL(os.path.join(N.LIBDIR, "libtacogb.so"))
    for n in names:
        assert hasattr(N.probe(), n) and not hasattr(product, n)


def test_libtacogb_gen_exports_header():
    names = declared("taco_gb300_gen.h")
    L = ctypes.CDLL(os.path.join(N.LIBDIR, "libtacogb_gen.so"))
    assert all(hasattr(L, n) for n in names)


@pytest.mark.parametrize("pattern", ["spmv", "spmm", "spgemm", "sddmm", "ttv", "ttm", "mttkrp"])
def test_dropin_modules_export_taco_names(pattern):
    L = ctypes.CDLL(os.path.join(N.LIBDIR, "libtacogb_%s.so" % pattern))
    for n in ("assemble", "compute", "evaluate", "_shim_assemble", "_shim_compute",
              "_shim_evaluate"):
        assert hasattr(L, n)


def test_oracle_generator_build_is_identical():
    """The oracle's own build of the generators (used by the benchmark's taco arm, which maps
    no product library) gives the same matrices bit for bit."""
    from oracle import oracle as O
    O.build()
    specs = [W.spmv_powerlaw(rows=40000), W.spmv_banded(rows=30000), W.spmv_small(),
             W.batch_spec(5), W.spgemm_poisson(64)]
    ours = [W.generate(s) for s in specs] + [W.dense(23, 1000)]
    try:
        N.set_generator_library(O.generator_library())
        theirs = [W.generate(s) for s in specs] + [W.dense(23, 1000)]
        assert N.gen()._name == O.generator_library()
    finally:
        N.set_generator_library(None)
    for a, b in zip(ours, theirs):
        for x, y in zip(a if isinstance(a, tuple) else (a,), b if isinstance(b, tuple) else (b,)):
            assert np.array_equal(x, y)


def test_version_and_error_without_gpu():
    assert tg.lib().tacogb_version().startswith(b"taco_gb300")
    assert tg.lib().tacogb_spmv_variant_count() >= 2


def test_generator_deterministic_and_valid():
    s = W.spmv_powerlaw(rows=50000)
    p1, c1, v1 = W.generate(s)
    p2, c2, v2 = W.generate(s)
    assert np.array_equal(p1, p2) and np.array_equal(c1, c2) and np.array_equal(v1, v2)
    assert p1[0] == 0 and np.all(np.diff(p1) >= 1)
    for i in range(0, 50000, 997):
        row = c1[p1[i]:p1[i + 1]]
        assert np.all(np.diff(row) > 0) and row.min() >= 0 and row.max() < s.cols
    assert np.all(np.abs(v1) < 1.0)


def test_generator_fingerprint():
    """Bytes of a small power-law matrix are fixed: the golden fixtures and the benchmark
    depend on the generator staying bit-identical across machines."""
    s = W.spec(777, kind=W.POWERLAW, mean=24.0, len_max=777, seed=12345)
    pos, crd, vals = W.generate(s)
    h = (int(pos.astype(np.int64).sum()), int((crd.astype(np.int64) * np.arange(len(crd))).sum() % 1000003),
         float(np.round(vals.sum(), 9)))
    expect_path = os.path.join(ROOT, "tests", "golden", "gen_fingerprint.txt")
    got = "%d %d %.9f" % h
    assert open(expect_path).read().strip() == got


def test_powerlaw_calibration():
    for mean, kmax in ((24.0, 20000), (32.0, 10000)):
        c = W.powerlaw_scale(mean, kmax)
        assert 3.0 < c < 7.0
    s = W.spmv_powerlaw(rows=400000)
    pos, _, _ = W.generate(s, values=False)
    assert abs(pos[-1] / 400000 - 24.0) < 1.0


def test_banded_and_poisson_structure():
    pos, crd, _ = W.generate(W.spmv_banded(rows=1000))
    for i in (0, 10, 500, 999):
        row = crd[pos[i]:pos[i + 1]]
        assert len(row) == min(32, min(1000, i + 32) - max(0, i - 32))
        assert row.min() >= i - 32 and row.max() < i + 32
    pos, crd, vals = W.generate(W.spgemm_poisson(grid=512))
    assert pos[-1] == 1308672
    assert set(np.unique(vals)) == {-1.0, 4.0}


def test_batch_plan_rejects_bad_arguments_without_gpu():
    """tacogb_batch_create validates the whole batch on the host before touching the GPU."""
    L = tg.lib()
    assert [L.tacogb_batch_variant_name(i) for i in range(L.tacogb_batch_variant_count())] == \
        [b"merge_ipt7", b"merge_ipt3", b"vector_g2", b"vector_g4", b"vector_g8", b"vector_g16"]
    h = ctypes.c_void_p()
    assert L.tacogb_batch_create(0, None, None, None, 0, None, ctypes.byref(h)) == 1
    assert b"empty" in L.tacogb_last_error() and not h.value
    mats = (N.Csr * 2)()
    for m, vt in enumerate((tg.TACOGB_F64, tg.TACOGB_F32)):
        mats[m].rows, mats[m].cols, mats[m].nnz, mats[m].vtype = 4, 4, 0, vt
        mats[m].pos = 16  # never dereferenced on the host
    ptrs = (ctypes.c_void_p * 2)(16, 16)
    assert L.tacogb_batch_create(2, mats, ptrs, ptrs, 0, None, ctypes.byref(h)) == 1
    assert b"value type" in L.tacogb_last_error()
    mats[1].vtype = tg.TACOGB_F64
    bad = (ctypes.c_int32 * 2)(0, 9)
    assert L.tacogb_batch_create(2, mats, ptrs, ptrs, 0, bad, ctypes.byref(h)) == 1
    assert b"variant 9" in L.tacogb_last_error()
    assert L.tacogb_batch_create(2, mats, ptrs, ptrs, 3, None, ctypes.byref(h)) == 1
    mats[0].rows = -1
    assert L.tacogb_batch_create(2, mats, ptrs, ptrs, 0, None, ctypes.byref(h)) == 1
    assert b"bad size" in L.tacogb_last_error()
    assert L.tacogb_batch_run(None, None) == 1


def test_csf_level0_count_checked_without_gpu():
    """An order-3 operand whose level-0 pos claims more coordinates than B's first mode holds is
    rejected on the host before pos1 is read at that count (no GPU needed)."""
    from taco_gb300 import taco as T
    e = np.zeros(0, np.int32)
    Bt = T.csf3((5, 6, 7), np.arange(5, dtype=np.int32), np.zeros(6, np.int32), e,
                np.zeros(1, np.int32), e, np.zeros(0))
    bad_pos0 = np.array([0, 9], np.int32)  # n0 = 9 > 5
    Bt.mode_arrays[0][0] = bad_pos0.ctypes.data
    C, D = np.ones((6, 4)), np.ones((7, 4))
    A = np.zeros((5, 4))
    At, Ct, Dt = T.dense(A, [5, 4]), T.dense(C, [6, 4]), T.dense(D, [7, 4])
    L = tg.lib()
    assert L.tacogb_mttkrp_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) == 1
    assert b"level-0 pos" in L.tacogb_last_error()


def test_csf_fiber_count_checked_without_gpu():
    """A level-1 pos whose end claims more fibers than n0 x dims[1] is rejected on the host
    before pos2 is read at that count."""
    from taco_gb300 import taco as T
    e = np.zeros(0, np.int32)
    pos1 = np.array([0, 0, 0, 0, 0, 1000], np.int32)  # 5 rows of level 0, 1000 > 5 x 6 fibers
    Bt = T.csf3((5, 6, 7), np.arange(5, dtype=np.int32), pos1, e, np.zeros(1, np.int32), e,
                np.zeros(0))
    A, C, D = np.zeros((5, 4)), np.ones((6, 4)), np.ones((7, 4))
    At, Ct, Dt = T.dense(A, [5, 4]), T.dense(C, [6, 4]), T.dense(D, [7, 4])
    L = tg.lib()
    assert L.tacogb_mttkrp_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) == 1
    assert b"level-1 pos" in L.tacogb_last_error()

