"""The oracle is pinned before it is trusted: against taco's own known-answer tests, against
taco's generated code run here on the same inputs, and against the committed golden fixtures
(made by tests/golden/make_golden.py from taco's generated code)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from taco_gb300 import workloads as W
from tests import helpers as H
from tests.helpers import normwise, ref_spmv, taco_rand_csr

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _csr_from_dense(D):
    pos, crd, vals = [0], [], []
    for row in D:
        nz = np.nonzero(row)[0]
        crd += list(nz)
        vals += list(row[nz])
        pos.append(len(crd))
    return np.array(pos, np.int32), np.array(crd, np.int32), np.array(vals, np.float64)


# d33a, d3b, d33b of test/test_tensors.cpp:89-94, 205-227
D33A = np.array([[0, 2, 0], [0, 0, 0], [3, 0, 4]], dtype=np.float64)
D33B = np.array([[10, 20, 0], [0, 0, 0], [0, 30, 0]], dtype=np.float64)
D3B = np.array([2, 0, 3], dtype=np.float64)


def test_spmv_kat():
    """expr_storage spmv: d33a(i,k) * d3b(k) = {0,0,18} (test/tests-expr_storage.cpp:873-937)."""
    pos, crd, vals = _csr_from_dense(D33A)
    assert list(O.spmv(pos, crd, vals, D3B)) == [0, 0, 18]


def test_matmul_kat():
    """matrix_mul: d33a * d33b = {0,0,0, 0,0,0, 30,180,0} (test/tests-expr_storage.cpp:996-1035),
    as SpMM (dense B) and as SpGEMM (CSR B)."""
    pos, crd, vals = _csr_from_dense(D33A)
    C = O.spmm(pos, crd, vals, D33B)
    assert list(C.ravel()) == [0, 0, 0, 0, 0, 0, 30, 180, 0]
    bp, bc, bv = _csr_from_dense(D33B)
    Cp, Cc, Cv = O.spgemm(pos, crd, vals, bp, bc, bv, 3)
    # row 0 meets only the empty row 1 of B; row 2 = 3*B(0,:) + 4*B(2,:) -> cols {0,1}
    assert list(Cp) == [0, 0, 0, 2] and list(Cc) == [0, 1] and list(Cv) == [30, 180]


@pytest.mark.skipif(not O.ref_available("spmv"), reason="taco generated code not built here")
@pytest.mark.parametrize("sparsity", [0.01, 0.1, 0.3])
def test_spmv_oracle_vs_taco_generated(sparsity):
    (pos, crd, vals, _), _ = taco_rand_csr(1021 // 10, 1039 // 10, sparsity)
    x = W.dense(5, 1039 // 10)
    y_ref = ref_spmv(pos, crd, vals, x, threads=1)
    y = O.spmv(pos, crd, vals, x)
    # same left-to-right loop; -ffast-math may reassociate taco's reduction
    assert normwise(y, y_ref) <= 1e-15


@pytest.mark.skipif(not O.ref_available("spmv"), reason="taco generated code not built here")
def test_spmv_oracle_vs_taco_generated_powerlaw():
    s = W.spmv_powerlaw(rows=20000)
    pos, crd, vals = W.generate(s)
    x = W.dense(7, s.cols)
    assert normwise(O.spmv(pos, crd, vals, x), ref_spmv(pos, crd, vals, x, threads=4)) <= 1e-14


def _golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail("missing golden fixture %s" % name)
    return np.load(path)


@pytest.mark.parametrize("case", ["spmv_taco_rand", "spmv_uniform", "spmv_powerlaw", "spmv_empty_rows"])
def test_oracle_matches_golden_spmv(case):
    g = _golden(case + ".npz")
    y = O.spmv(g["pos"], g["crd"], g["vals"], g["x"])
    assert normwise(y, g["y"]) <= 1e-14


def test_pack_kat():
    """taco's test tensor/duplicates (test/tests-tensor.cpp:68-79): duplicates sum."""
    pos, crd, v = O.pack_csr(5, 5, [1, 2, 1], [2, 2, 2], [42.0, 10.0, 1.0])
    assert list(pos) == [0, 0, 1, 2, 2, 2] and list(crd) == [2, 2] and list(v) == [43.0, 10.0]


def test_pack_oracle_matches_taco():
    """The pack restatement against a fixture taco itself packed (tests/golden/make_golden.py
    runs the taco CLI on a .tns file with duplicates, a cancelling pair and empty rows)."""
    g = np.load(os.path.join(GOLDEN, "pack_taco_cli.npz"))
    pos, crd, v = O.pack_csr(int(g["rows"]), int(g["cols"]), g["ri"], g["ci"], g["v"])
    assert np.array_equal(pos, g["pos"]) and np.array_equal(crd, g["crd"])
    assert np.array_equal(v, g["vals"])
    assert (g["vals"] == 0.0).any()  # the cancelling pair stays an explicit zero, as in taco


def test_pack_oracle_rejects_out_of_range():
    with pytest.raises(ValueError):
        O.pack_csr(3, 3, [0, 3], [0, 0], [1.0, 2.0])


@pytest.mark.parametrize("case", ["sddmm_taco_gpu", "sddmm_taco_cpu", "sddmm_powerlaw_j96"])
def test_oracle_matches_golden_sddmm(case):
    """The SDDMM restatement against taco's own generated code (dense result): bit-exact on
    taco's integer-valued test inputs, and on real values too (same loop order)."""
    g = _golden(case + ".npz")
    if "C" in g:
        C, D = g["C"], g["D"]
    else:  # the power-law case regenerates its dense operands
        I, K = g["A"].shape
        C = W.dense(17, I * 96).reshape(I, 96)
        D = W.dense(18, 96 * K).reshape(96, K)
    A = O.sddmm(g["pos"], g["crd"], g["vals"], C, D)
    assert np.array_equal(A, g["A"])
    rows = np.repeat(np.arange(len(g["pos"]) - 1), np.diff(g["pos"]))
    assert np.array_equal(O.sddmm_sampled(g["pos"], g["crd"], g["vals"], C, D), A[rows, g["crd"]])


def test_sddmm_inputs_follow_taco_draws():
    """taco_sddmm_inputs reproduces the fixture's inputs from taco's srand seed and draw order."""
    from tests.helpers import taco_sddmm_inputs
    g = _golden("sddmm_taco_gpu.npz")
    (pos, crd, vals), C, D = taco_sddmm_inputs(1021 // 10, 128, 1039 // 10, 0.3, 535366)
    for a, b in ((pos, "pos"), (crd, "crd"), (vals, "vals"), (C, "C"), (D, "D")):
        assert np.array_equal(a, g[b])


def _csf3_fixture(name):
    g = _golden(name + ".npz")
    B = (tuple(int(d) for d in g["dims"]), g["crd0"], g["pos1"], g["crd1"], g["pos2"], g["crd2"],
         g["vals"])
    return g, B


@pytest.mark.parametrize("case", ["ttv_taco_gpu", "ttv_taco_cpu", "ttm_taco_gpu", "ttm_taco_cpu",
                                  "mttkrp_taco_gpu", "mttkrp_taco_cpu"])
def test_oracle_matches_golden_tensor3(case):
    """The order-3 restatements against taco's own generated code on taco's test inputs."""
    g, B = _csf3_fixture(case)
    if case.startswith("ttv"):
        A = O.ttv(B, g["c"])
    elif case.startswith("ttm"):
        A = O.ttm(B, g["C"])
    else:
        A = O.mttkrp(B, g["C"], g["D"])
    assert np.array_equal(A, g["A"])


def test_tensor3_inputs_follow_taco_draws():
    from tests.helpers import csf3, taco_tensor3_inputs
    g, B = _csf3_fixture("mttkrp_taco_gpu")
    co, v, (C, D) = taco_tensor3_inputs((25, 25, 30), 0.1, 5464164, [(25, 32), (30, 32)])
    for a, b in zip(csf3((25, 25, 30), co, v)[1:], B[1:]):
        assert np.array_equal(a, b)
    assert np.array_equal(C, g["C"]) and np.array_equal(D, g["D"])


def test_format_fixtures_match_oracle():
    """taco's generated code for DCSR / CSC / sparse-vector SpMV and DCSR SpMM sums in the same
    order as the CSR restatement: the fixtures equal the oracle's results."""
    g = _golden("spmv_formats_taco.npz")
    pos, crd, vals, x = g["pos"], g["crd"], g["vals"], g["x"]
    y = O.spmv(pos, crd, vals, x)
    assert normwise(g["y_dcsr"], y) <= 1e-15 and normwise(g["y_csc"], y) <= 1e-15
    xs = np.zeros_like(x)
    xs[g["xi"]] = x[g["xi"]]
    ys = O.spmv(pos, crd, vals, xs)
    assert np.array_equal(g["ys_crd"], np.flatnonzero(np.diff(pos) > 0))
    assert normwise(g["ys_vals"], ys[g["ys_crd"]]) <= 1e-15
    g = _golden("spmm_dcsr_taco_gpu.npz")
    assert np.array_equal(O.spmm(g["pos"], g["crd"], g["vals"], g["B"]), g["C"])


@pytest.mark.skipif(not O.ref_available("spmv_dcsr_sv"), reason="taco generated code not built here")
def test_taco_generated_sparse_result_kat():
    """taco's own code for a{Sparse} = B{Sparse,Sparse} * c{Sparse} reproduces the KAT
    (test/tests-expr_storage.cpp:922-934): coordinates {0,2}, values {0,18}."""
    from tests.helpers import ref_spmv_formats
    kp, kc, kv = np.array([0, 1, 1, 3], np.int32), np.array([1, 0, 2], np.int32), np.array([2., 3., 4.])
    crd, vals = ref_spmv_formats("dcsr_sv", kp, kc, kv, 3, None,
                                 (np.array([0, 2], np.int32), np.array([2., 3.])))
    assert list(crd) == [0, 2] and list(vals) == [0, 18]


@pytest.mark.skipif(not O.ref_available("spgemm_sched"), reason="taco generated code not built here")
@pytest.mark.parametrize("case", ["spgemm_taco_rand", "spgemm_random_512", "spgemm_poisson_32"])
def test_scheduled_spgemm_matches_serial(case):
    """taco's parallel two-pass SpGEMM (scheduleSpGEMMCPU, test/tests-scheduling-eval.cpp:68-94,
    emitted by taco's CLI with the same scheduling directives) against the golden fixtures made
    by taco's serial default code, on 4 threads: pos, crd and values bit for bit."""
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    K = int(g["K"][0])
    A = (g["Apos"], g["Acrd"], g["Avals"], len(g["Bpos"]) - 1)
    B = (g["Bpos"], g["Bcrd"], g["Bvals"], K)
    cp, cc, cv = H.ref_spgemm(A, B, threads=4, pattern="spgemm_sched")
    assert np.array_equal(cp, g["Cpos"]) and np.array_equal(cc, g["Ccrd"])
    assert np.array_equal(cv, g["Cvals"])
