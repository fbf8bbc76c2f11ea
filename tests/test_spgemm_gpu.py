"""Two-phase SpGEMM parity on the GPU.

Bars: C's pos and crd bit-exact against taco's generated code (golden fixtures) and the oracle;
values bit-exact too, because the GPU sums each column's products in taco's A-row order with
separately rounded multiplies and adds (the golden values were produced by taco's generated C
compiled without FMA contraction).  The normwise 1e-12 bar is asserted as well.
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


def _csr(pos, crd, vals, cols, dtype=torch.float64):
    return tg.CsrMatrix.from_numpy(pos, crd, vals, cols, dtype=dtype)


def gpu_spgemm(A, B, dtype=torch.float64):
    """(pos, crd, vals) of A*B through tacogb_spgemm_symbolic/fill/numeric, after checking that
    the one-pass form (tacogb_spgemm_onepass/_finish) gives the same arrays bit for bit."""
    phases = gpu_spgemm_phases(A, B, dtype)
    one = gpu_spgemm_onepass(A, B, dtype)
    for x, y in zip(phases, one):
        assert np.array_equal(x, y)
    return phases


def gpu_spgemm_onepass(A, B, dtype=torch.float64):
    (ap, ac, av, acols), (bp, bc, bv, bcols) = A, B
    Ad, Bd = _csr(ap, ac, av, acols, dtype), _csr(bp, bc, bv, bcols, dtype)
    a, b = Ad.as_csr(), Bd.as_csr()
    L = tg.lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Cpos = torch.full((len(ap),), -1, dtype=torch.int32, device="cuda")
    nnz = ctypes.c_int64(0)
    tg.check(L.tacogb_spgemm_onepass(ctypes.byref(a), ctypes.byref(b), Cpos.data_ptr(),
                                     ctypes.byref(nnz), sp), "onepass")
    Ccrd = torch.full((max(nnz.value, 1),), -1, dtype=torch.int32, device="cuda")
    Cvals = torch.full((max(nnz.value, 1),), float("nan"), dtype=dtype, device="cuda")
    tg.check(L.tacogb_spgemm_onepass_finish(Cpos.data_ptr(), Ccrd.data_ptr(), Cvals.data_ptr(),
                                            sp), "onepass_finish")
    torch.cuda.synchronize()
    n = nnz.value
    return (Cpos.cpu().numpy(), Ccrd[:n].cpu().numpy(), Cvals[:n].double().cpu().numpy())


def gpu_spgemm_phases(A, B, dtype=torch.float64):
    """(pos, crd, vals) of A*B through tacogb_spgemm_symbolic/fill/numeric."""
    (ap, ac, av, acols), (bp, bc, bv, bcols) = A, B
    Ad, Bd = _csr(ap, ac, av, acols, dtype), _csr(bp, bc, bv, bcols, dtype)
    a, b = Ad.as_csr(), Bd.as_csr()
    L = tg.lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Cpos = torch.empty(len(ap), dtype=torch.int32, device="cuda")
    nnz = ctypes.c_int64(0)
    tg.check(L.tacogb_spgemm_symbolic(ctypes.byref(a), ctypes.byref(b), Cpos.data_ptr(),
                                      ctypes.byref(nnz), sp), "symbolic")
    Ccrd = torch.empty(max(nnz.value, 1), dtype=torch.int32, device="cuda")
    Cvals = torch.empty(max(nnz.value, 1), dtype=dtype, device="cuda")
    tg.check(L.tacogb_spgemm_fill(ctypes.byref(a), ctypes.byref(b), Cpos.data_ptr(),
                                  Ccrd.data_ptr(), sp), "fill")
    tg.check(L.tacogb_spgemm_numeric(ctypes.byref(a), ctypes.byref(b), Cpos.data_ptr(),
                                     Ccrd.data_ptr(), Cvals.data_ptr(), sp), "numeric")
    torch.cuda.synchronize()
    n = nnz.value
    return (Cpos.cpu().numpy(), Ccrd[:n].cpu().numpy(), Cvals[:n].double().cpu().numpy())


@pytest.mark.parametrize("case", ["spgemm_taco_rand", "spgemm_random_512", "spgemm_poisson_32"])
def test_golden(case):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    K = int(g["K"][0])
    A = (g["Apos"], g["Acrd"], g["Avals"], len(g["Bpos"]) - 1)
    B = (g["Bpos"], g["Bcrd"], g["Bvals"], K)
    cp, cc, cv = gpu_spgemm(A, B)
    assert np.array_equal(cp, g["Cpos"])
    assert np.array_equal(cc, g["Ccrd"])
    assert normwise(cv, g["Cvals"]) <= 1e-12
    assert np.array_equal(cv, g["Cvals"])


def _bins_matrix():
    """Rows whose product counts fall in every bin: 0, <=32, <=256, <=4096, >4096."""
    rng = np.random.default_rng(11)
    n, K = 3000, 20000
    # B: mostly short rows, a few long ones
    blens = rng.integers(0, 6, n)
    blens[:10] = 2500
    bpos = np.concatenate([[0], np.cumsum(blens)]).astype(np.int32)
    bcrd = np.concatenate([np.sort(rng.choice(K, l, replace=False)) for l in blens]).astype(np.int32)
    bvals = rng.uniform(-1, 1, len(bcrd))
    alens = rng.integers(0, 12, n)
    alens[100:110] = 0
    arows = []
    for i, l in enumerate(alens):
        if i in (7, 8):          # > 4096 products: several long B rows
            arows.append(np.array([0, 1, 2, 3, 50, 60], dtype=np.int64))
        elif i in (20, 21, 22):  # 2500 < P <= 4096
            arows.append(np.array([4, 70, 80], dtype=np.int64))
        else:
            arows.append(np.sort(rng.choice(np.arange(10, n), l, replace=False)))
    apos = np.concatenate([[0], np.cumsum([len(r) for r in arows])]).astype(np.int32)
    acrd = np.concatenate(arows).astype(np.int32)
    avals = rng.uniform(-1, 1, len(acrd))
    return (apos, acrd, avals, n), (bpos, bcrd, bvals, K)


def test_all_bins_against_oracle():
    A, B = _bins_matrix()
    ref = O.spgemm(A[0], A[1], A[2], B[0], B[1], B[2], B[3])
    cp, cc, cv = gpu_spgemm(A, B)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    assert np.array_equal(cv, ref[2])


def test_all_bins_float32():
    A, B = _bins_matrix()
    ref = O.spgemm(A[0], A[1], A[2], B[0], B[1], B[2], B[3])
    cp, cc, cv = gpu_spgemm(A, B, torch.float32)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    assert normwise(cv, ref[2]) <= 1e-6


def _sort_path_matrix():
    """Rows whose product counts sit on and around every sort-path boundary of bins 1 and 2
    (32/33 products: bin 1 to bin 2; 64/65: two to four keys per lane in registers; 128/129:
    registers to the warp's shared-memory slice; 256/257: bin 2 to bin 3), plus random counts
    in between.  B's rows draw their columns from [0, 150), so most output columns collect
    several products and the runs that are summed cross the lanes' register boundaries."""
    rng = np.random.default_rng(29)
    K, copies = 150, 5
    blens = np.repeat(np.arange(1, 65), copies)  # B row copies*(L-1)+c has L entries
    bpos = np.concatenate([[0], np.cumsum(blens)]).astype(np.int32)
    bcrd = np.concatenate([np.sort(rng.choice(K, l, replace=False)) for l in blens]).astype(np.int32)
    bvals = rng.uniform(-1, 1, len(bcrd))
    targets = [32, 33, 63, 64, 65, 96, 100, 127, 128, 129, 200, 255, 256, 257, 300]
    targets = targets * 3 + list(rng.integers(1, 320, 200))
    arows = []
    for P in targets:
        rows, left = [], int(P)
        cs = list(rng.permutation(copies))
        while left > 64:
            rows.append(copies * 63 + cs.pop())
            left -= 64
        rows.append(copies * (left - 1) + int(rng.integers(copies)))
        arows.append(np.unique(np.array(rows, dtype=np.int64)))
    apos = np.concatenate([[0], np.cumsum([len(r) for r in arows])]).astype(np.int32)
    acrd = np.concatenate(arows).astype(np.int32)
    avals = rng.uniform(-1, 1, len(acrd))
    return (apos, acrd, avals, len(blens)), (bpos, bcrd, bvals, K)


def _long_a_rows_matrix():
    """Rows of A with 33 to 100 entries whose B rows are mostly empty, so that the product
    counts (1 to 128) fall in bins 1 and 2 while the expansion takes A's entries in several
    chunks of 32 lanes; B rows of 0, 1 and 3 entries over 40 columns."""
    rng = np.random.default_rng(31)
    nb, K = 400, 40
    blens = rng.choice([0, 0, 0, 1, 3], nb)
    bpos = np.concatenate([[0], np.cumsum(blens)]).astype(np.int32)
    bcrd = np.concatenate([np.sort(rng.choice(K, l, replace=False)) for l in blens]).astype(np.int32)
    bvals = rng.uniform(-1, 1, len(bcrd))
    arows = [np.sort(rng.choice(nb, int(rng.integers(33, 101)), replace=False)) for _ in range(300)]
    apos = np.concatenate([[0], np.cumsum([len(r) for r in arows])]).astype(np.int32)
    acrd = np.concatenate(arows).astype(np.int32)
    avals = rng.uniform(-1, 1, len(acrd))
    return (apos, acrd, avals, nb), (bpos, bcrd, bvals, K)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_long_a_rows_few_products(dtype):
    A, B = _long_a_rows_matrix()
    prods = [int(np.sum(np.diff(B[0])[A[1][A[0][i]:A[0][i + 1]]])) for i in range(len(A[0]) - 1)]
    assert max(prods) <= 128 and min(np.diff(A[0])) > 32
    ref = O.spgemm(A[0], A[1], A[2], B[0], B[1], B[2], B[3])
    cp, cc, cv = gpu_spgemm(A, B, dtype)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    if dtype == torch.float64:
        assert np.array_equal(cv, ref[2])
    else:
        assert normwise(cv, ref[2]) <= 1e-6


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_wide_column_keys(dtype):
    """B with 2^24 + 7 columns: bins 1 and 2 sort (column, sequence) keys of 64 bits instead
    of the narrow 32-bit keys; columns on both sides of 2^24 and repeated across B's rows."""
    rng = np.random.default_rng(37)
    K, nb = (1 << 24) + 7, 200
    colset = np.concatenate([np.arange(K - 40, K), np.arange((1 << 24) - 40, 1 << 24),
                             rng.choice(1 << 24, 40, replace=False)])
    colset = np.unique(colset)
    blens = rng.integers(0, 9, nb)
    bpos = np.concatenate([[0], np.cumsum(blens)]).astype(np.int32)
    bcrd = np.concatenate([np.sort(rng.choice(colset, l, replace=False)) for l in blens]).astype(np.int32)
    bvals = rng.uniform(-1, 1, len(bcrd))
    arows = [np.sort(rng.choice(nb, int(rng.integers(1, 25)), replace=False)) for _ in range(400)]
    apos = np.concatenate([[0], np.cumsum([len(r) for r in arows])]).astype(np.int32)
    acrd = np.concatenate(arows).astype(np.int32)
    avals = rng.uniform(-1, 1, len(acrd))
    A, B = (apos, acrd, avals, nb), (bpos, bcrd, bvals, K)
    prods = [int(np.sum(blens[acrd[apos[i]:apos[i + 1]]])) for i in range(len(apos) - 1)]
    assert min(prods) <= 32 < max(prods) <= 128 and bcrd.max() >= 1 << 24
    ref = O.spgemm(A[0], A[1], A[2], B[0], B[1], B[2], B[3])
    cp, cc, cv = gpu_spgemm(A, B, dtype)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    if dtype == torch.float64:
        assert np.array_equal(cv, ref[2])
    else:
        assert normwise(cv, ref[2]) <= 1e-6


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sort_path_boundaries(dtype):
    A, B = _sort_path_matrix()
    prods = [int(np.sum(np.diff(B[0])[A[1][A[0][i]:A[0][i + 1]]])) for i in range(len(A[0]) - 1)]
    assert {32, 33, 64, 65, 128, 129, 256, 257} <= set(prods)
    ref = O.spgemm(A[0], A[1], A[2], B[0], B[1], B[2], B[3])
    cp, cc, cv = gpu_spgemm(A, B, dtype)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    if dtype == torch.float64:
        assert np.array_equal(cv, ref[2])
    else:
        assert normwise(cv, ref[2]) <= 1e-6


@pytest.mark.parametrize("which", ["random", "poisson"])
def test_full_size(which):
    """262,144^2 with 8 uniform nonzeros per row, and the 512x512 Poisson stencil squared."""
    s = W.spgemm_random() if which == "random" else W.spgemm_poisson()
    p, c, v = W.generate(s)
    A = (p, c, v, s.cols)
    ref = O.spgemm(p, c, v, p, c, v, s.cols)
    cp, cc, cv = gpu_spgemm(A, A)
    assert np.array_equal(cp, ref[0]) and np.array_equal(cc, ref[1])
    assert np.array_equal(cv, ref[2])
    if which == "poisson":
        assert cp[-1] == 3397636


@pytest.mark.parametrize("where", ["host", "device"])
def test_abi_evaluate_full_size(where):
    """tacogb_spgemm_evaluate on the random 262,144^2 matrix: 0.2 GB of results, returned into
    malloc'd memory by chunked copies whose pages host threads map first (host operands), or
    written into managed memory populated on the GPU first (device operands); bit-exact."""
    s = W.spgemm_random()
    p, c, v = W.generate(s)
    ref = O.spgemm(p, c, v, p, c, v, s.cols)
    nnz = int(ref[0][-1])
    assert nnz * 12 >= 64 << 20
    arrs = (p, c, v) if where == "host" else tuple(torch.from_numpy(a).cuda() for a in (p, c, v))
    At = T.csr(*arrs, [s.rows, s.cols])
    for _ in range(2):
        Ct = T.csr_result([s.rows, s.cols])
        assert tg.lib().tacogb_spgemm_evaluate(Ct.ptr, At.ptr, At.ptr) == 0, \
            tg.lib().tacogb_last_error()
        if where == "device":
            torch.cuda.synchronize()
        P = ctypes.POINTER
        pos = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 0), P(ctypes.c_int32)), (s.rows + 1,))
        crd = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 1), P(ctypes.c_int32)), (nnz,))
        vals = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, P(ctypes.c_double)), (nnz,))
        assert np.array_equal(pos, ref[0]) and np.array_equal(crd, ref[1])
        assert np.array_equal(vals, ref[2])


def test_empty_and_degenerate():
    A = (np.zeros(5, np.int32), np.zeros(0, np.int32), np.zeros(0), 7)
    B = (np.zeros(8, np.int32), np.zeros(0, np.int32), np.zeros(0), 3)
    cp, cc, cv = gpu_spgemm(A, B)
    assert list(cp) == [0] * 5 and len(cc) == 0


def test_abi_assemble_compute_host_and_device():
    g = np.load(os.path.join(GOLDEN, "spgemm_poisson_32.npz"))
    n = len(g["Apos"]) - 1
    for where in ("host", "device"):
        arrs = {k: g[k] for k in ("Apos", "Acrd", "Avals")}
        if where == "device":
            arrs = {k: torch.from_numpy(v).cuda() for k, v in arrs.items()}
        At = T.csr(arrs["Apos"], arrs["Acrd"], arrs["Avals"], [n, n])
        Ct = T.csr_result([n, n])
        assert tg.lib().tacogb_spgemm_assemble(Ct.ptr, At.ptr, At.ptr) == 0
        assert tg.lib().tacogb_spgemm_compute(Ct.ptr, At.ptr, At.ptr) == 0
        if where == "device":
            torch.cuda.synchronize()  # managed results are host-readable after a sync
        nnz = int(g["Cpos"][-1])
        pos = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 0), ctypes.POINTER(ctypes.c_int32)), (n + 1,))
        crd = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 1), ctypes.POINTER(ctypes.c_int32)), (nnz,))
        vals = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, ctypes.POINTER(ctypes.c_double)), (nnz,))
        assert np.array_equal(pos, g["Cpos"]) and np.array_equal(crd, g["Ccrd"])
        assert np.array_equal(vals, g["Cvals"])


def test_abi_matmul_kat_through_dropin_module():
    """d33a * d33b (test/tests-expr_storage.cpp:996-1035) in CSR through libtacogb_spgemm.so's
    _shim_evaluate: structural entries of row 2 are {0: 30, 1: 180}."""
    L = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib", "libtacogb_spgemm.so"))
    L._shim_evaluate.argtypes = [ctypes.c_void_p]
    At = T.csr(np.array([0, 1, 1, 3], np.int32), np.array([1, 0, 2], np.int32),
               np.array([2.0, 3.0, 4.0]), [3, 3])
    Bt = T.csr(np.array([0, 2, 2, 3], np.int32), np.array([0, 1, 1], np.int32),
               np.array([10.0, 20.0, 30.0]), [3, 3])
    Ct = T.csr_result([3, 3])
    args = (ctypes.c_void_p * 3)(Ct.ptr, At.ptr, Bt.ptr)
    assert L._shim_evaluate(args) == 0
    pos = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 0), ctypes.POINTER(ctypes.c_int32)), (4,))
    crd = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 1), ctypes.POINTER(ctypes.c_int32)), (2,))
    vals = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, ctypes.POINTER(ctypes.c_double)), (2,))
    assert list(pos) == [0, 0, 0, 2] and list(crd) == [0, 1] and list(vals) == [30.0, 180.0]


def test_abi_rejects_shape_mismatch():
    At = T.csr(np.array([0, 1], np.int32), np.array([0], np.int32), np.array([1.0]), [1, 4])
    Bt = T.csr(np.array([0, 0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0), [2, 2])
    Ct = T.csr_result([1, 2])
    assert tg.lib().tacogb_spgemm_assemble(Ct.ptr, At.ptr, Bt.ptr) == 1
    assert b"columns" in tg.lib().tacogb_last_error()
