"""ORACLE — test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline
leg).  The taco_gb300 product never imports this module.

Two CPU checkers, both over plain numpy arrays:
  * liboracle.so       — the C restatement in oracle/taco_oracle.c (always built);
  * libtacoref_*.so    — taco's own generated C (oracle/_ref/gen/*.c, emitted by taco's CLI
                         through oracle/Makefile.ref), compiled with taco's JIT flags; present
                         wherever oracle/_ref/gen travelled.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
GEN_DIR = os.path.join(REF_DIR, "gen")
P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stdout))


def build(reference_root=None):
    """Compiles the C restatement; compiles taco's generated C when it is available, first
    regenerating it from taco's source tree when one is named (reference_root, else the
    TACO_REFERENCE environment variable) and exists."""
    reference_root = reference_root or os.environ.get("TACO_REFERENCE") or ""
    src = os.path.join(HERE, "taco_oracle.c")
    out = os.path.join(HERE, "liboracle.so")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", out])
    root = os.path.dirname(HERE)
    # the workload generators (taco_gb300/csrc/gen.c) built again on the oracle side, for
    # processes that time taco's code and must not map the product's libraries
    gsrc = os.path.join(root, "taco_gb300", "csrc", "gen.c")
    gout = generator_library()
    if not os.path.exists(gout) or os.path.getmtime(gout) < os.path.getmtime(gsrc):
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-I" + os.path.join(root, "include"), gsrc, "-o", gout, "-lm"])
    if reference_root and os.path.isdir(os.path.join(reference_root, "src")):
        _run(["make", "-s", "-f", "oracle/Makefile.ref", "-j8", "REF=" + reference_root], cwd=root)
    elif os.path.isdir(GEN_DIR):
        _run(["make", "-s", "-f", "oracle/Makefile.ref", "lib", "REF=/nonexistent"], cwd=root)


def generator_library():
    """Path of the oracle-side build of the workload generators."""
    return os.path.join(HERE, "liboracle_gen.so")


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_spmv_f64.argtypes = [I32, P, P, P, P, P]
        L.oracle_spmm_f64.argtypes = [I32, I32, P, P, P, P, P]
        L.oracle_spgemm_assemble.restype = I64
        L.oracle_spgemm_assemble.argtypes = [I32, I32, P, P, P, P, P, ctypes.POINTER(P)]
        L.oracle_spgemm_compute.argtypes = [I32, I32, P, P, P, P, P, P, P, P, P]
        L.oracle_free.argtypes = [P]
        L.oracle_sddmm_f64.argtypes = [I32, I32, I32, P, P, P, P, P, P]
        L.oracle_sddmm_sampled_f64.argtypes = [I32, I32, I32, P, P, P, P, P, P]
        L.oracle_ttv_f64.argtypes = [I32, I32, I32] + [P] * 8
        L.oracle_ttm_f64.argtypes = [I32, I32, I32, I32] + [P] * 8
        L.oracle_mttkrp_f64.argtypes = [I32, I32, I32] + [P] * 9
        L.oracle_ttm_fibers_f64.argtypes = [I32, I32] + [P] * 5
        L.oracle_pack_csr.restype = I64
        L.oracle_pack_csr.argtypes = [I32, I32, I64, P, P, P, P, P, P]
        L.oracle_num_threads.restype = I32
        L.oracle_set_num_threads.argtypes = [I32]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


def spmv(pos, crd, vals, x):
    y = np.empty(len(pos) - 1, dtype=np.float64)
    lib().oracle_spmv_f64(len(pos) - 1, _p(pos), _p(crd), _p(vals), _p(x), _p(y))
    return y


def spmm(pos, crd, vals, B):
    rows, N = len(pos) - 1, B.shape[1]
    C = np.empty((rows, N), dtype=np.float64)
    lib().oracle_spmm_f64(rows, N, _p(pos), _p(crd), _p(vals), _p(np.ascontiguousarray(B)), _p(C))
    return C


def spgemm(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, K):
    """(Cpos, Ccrd, Cvals) of A*B with taco's structure: every structural product kept,
    columns sorted per row."""
    rows = len(Apos) - 1
    Cpos = np.empty(rows + 1, dtype=np.int32)
    crd_ptr = P()
    nnz = lib().oracle_spgemm_assemble(rows, K, _p(Apos), _p(Acrd), _p(Bpos), _p(Bcrd), _p(Cpos),
                                       ctypes.byref(crd_ptr))
    if nnz < 0:
        raise OverflowError("nnz(C) exceeds int32")
    Ccrd = np.ctypeslib.as_array(ctypes.cast(crd_ptr, ctypes.POINTER(ctypes.c_int32)),
                                 shape=(max(nnz, 1),))[:nnz].copy()
    lib().oracle_free(crd_ptr)
    Cvals = np.empty(nnz, dtype=np.float64)
    if vals_given := (Avals is not None and Bvals is not None):
        lib().oracle_spgemm_compute(rows, K, _p(Apos), _p(Acrd), _p(Avals), _p(Bpos), _p(Bcrd),
                                    _p(Bvals), _p(Cpos), _p(Ccrd), _p(Cvals))
    return Cpos, Ccrd, (Cvals if vals_given else None)


def pack_csr(rows, cols, ri, ci, v):
    """(pos, crd, vals) of the COO coordinates (ri, ci) with values v packed into CSR the way
    taco's pack does: sorted, duplicates summed (in input order)."""
    ri = np.ascontiguousarray(ri, dtype=np.int32)
    ci = np.ascontiguousarray(ci, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.float64)
    n = len(ri)
    pos = np.empty(rows + 1, dtype=np.int32)
    crd = np.empty(max(n, 1), dtype=np.int32)
    out = np.empty(max(n, 1), dtype=np.float64)
    m = lib().oracle_pack_csr(rows, cols, n, _p(ri), _p(ci), _p(v), _p(pos), _p(crd), _p(out))
    if m < 0:
        raise ValueError("coordinate outside the matrix")
    return pos, crd[:m].copy(), out[:m].copy()


def sddmm(pos, crd, vals, C, D):
    """Dense I x K result of A(i,k) = B(i,k) * C(i,j) * D(j,k), B = (pos, crd, vals)."""
    pos, crd, vals = (np.ascontiguousarray(pos, np.int32), np.ascontiguousarray(crd, np.int32),
                      np.ascontiguousarray(vals, np.float64))
    C, D = np.ascontiguousarray(C, np.float64), np.ascontiguousarray(D, np.float64)
    I, J, K = C.shape[0], C.shape[1], D.shape[1]
    A = np.empty((I, K))
    lib().oracle_sddmm_f64(I, K, J, _p(pos), _p(crd), _p(vals), _p(C), _p(D), _p(A))
    return A


def sddmm_sampled(pos, crd, vals, C, D):
    """The same sums kept at B's nonzeros (one value per nonzero)."""
    pos, crd, vals = (np.ascontiguousarray(pos, np.int32), np.ascontiguousarray(crd, np.int32),
                      np.ascontiguousarray(vals, np.float64))
    C, D = np.ascontiguousarray(C, np.float64), np.ascontiguousarray(D, np.float64)
    I, J, K = C.shape[0], C.shape[1], D.shape[1]
    out = np.empty(len(crd))
    lib().oracle_sddmm_sampled_f64(I, K, J, _p(pos), _p(crd), _p(vals), _p(C), _p(D), _p(out))
    return out


def _csf(B):
    """(dims, crd0, pos1, crd1, pos2, crd2, vals) as contiguous arrays."""
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    ints = [np.ascontiguousarray(a, np.int32) for a in (crd0, pos1, crd1, pos2, crd2)]
    return [int(d) for d in dims], ints, np.ascontiguousarray(vals, np.float64)


def ttv(B, c):
    """Dense I x J result of A(i,j) = B(i,j,k) * c(k); B = (dims, crd0, pos1, crd1, pos2,
    crd2, vals), a {Sparse,Sparse,Sparse} tensor."""
    dims, (crd0, pos1, crd1, pos2, crd2), vals = _csf(B)
    c = np.ascontiguousarray(c, np.float64)
    A = np.empty((dims[0], dims[1]))
    lib().oracle_ttv_f64(dims[0], dims[1], len(crd0), _p(crd0), _p(pos1), _p(crd1), _p(pos2),
                         _p(crd2), _p(vals), _p(c), _p(A))
    return A


def ttm(B, C):
    """Dense I x J x L result of A(i,j,l) = B(i,j,k) * C(k,l)."""
    dims, (crd0, pos1, crd1, pos2, crd2), vals = _csf(B)
    C = np.ascontiguousarray(C, np.float64)
    L = C.shape[1]
    A = np.empty((dims[0], dims[1], L))
    lib().oracle_ttm_f64(dims[0], dims[1], L, len(crd0), _p(crd0), _p(pos1), _p(crd1), _p(pos2),
                         _p(crd2), _p(vals), _p(C), _p(A))
    return A


def mttkrp(B, C, D):
    """Dense I x J result of A(i,j) = B(i,k,l) * C(k,j) * D(l,j)."""
    dims, (crd0, pos1, crd1, pos2, crd2), vals = _csf(B)
    C, D = np.ascontiguousarray(C, np.float64), np.ascontiguousarray(D, np.float64)
    J = C.shape[1]
    A = np.empty((dims[0], J))
    lib().oracle_mttkrp_f64(dims[0], J, len(crd0), _p(crd0), _p(pos1), _p(crd1), _p(pos2),
                            _p(crd2), _p(vals), _p(C), _p(D), _p(A))
    return A


def set_threads(n):
    lib().oracle_set_num_threads(n)


def threads():
    return lib().oracle_num_threads()


# ------------------------------------------------------------ taco's generated code --------

def ref_available(pattern):
    return os.path.exists(os.path.join(REF_DIR, "libtacoref_%s.so" % pattern))


_ref = {}


def ref_lib(pattern):
    """taco's generated C for pattern (spmv, spmm, spgemm, sddmm, ttv, ttm, mttkrp) as compiled by Makefile.ref; exports
    taco's own assemble/compute/evaluate(taco_tensor_t*...)."""
    if pattern not in _ref:
        path = os.path.join(REF_DIR, "libtacoref_%s.so" % pattern)
        L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        nargs = 4 if pattern in ("sddmm", "mttkrp") else 3
        fns = ("assemble", "compute", "evaluate")
        for fn in fns:
            getattr(L, fn).argtypes = [P] * nargs
            getattr(L, fn).restype = ctypes.c_int
        _ref[pattern] = L
    return _ref[pattern]


def ref_set_threads(n):
    """OpenMP thread count and static schedule for taco's generated code, as
    Module::callFuncPackedRaw sets them (src/codegen/module.cpp:190-215)."""
    import ctypes.util
    for name in ("libgomp.so.1", ctypes.util.find_library("gomp")):
        if not name:
            continue
        try:
            g = ctypes.CDLL(name)
            g.omp_set_num_threads(int(n))
            g.omp_set_schedule(1, 0)  # omp_sched_static, default chunk
            return
        except OSError:
            continue
