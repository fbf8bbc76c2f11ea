"""taco_gb300 — taco's sparse hot path (CSR SpMV, SpMM, two-phase SpGEMM) as hand-written
sm_103a CUDA behind taco's kernel ABI.

Python here is plumbing for tests and benchmarks: the product is libtacogb.so
(include/taco_gb300.h) and the per-pattern drop-in modules.  Device memory comes from torch.
"""
import ctypes

from . import _native
from ._native import (TACOGB_F64, TACOGB_F32, TACOGB_BF16, VARIANT_AUTO, TacoGBError, check,
                      lib)

__all__ = ["CsrMatrix", "spmv", "spmv_variants", "spmm", "spmm_variants", "spgemm", "pack_csr",
           "sddmm", "sddmm_variants", "CsfTensor", "ttv", "ttm", "mttkrp",
           "read_coo", "read_csr", "read_csc",
           "SpmvBatch",
           "SpmmBatch",
           "batch_variants", "lib", "check", "TacoGBError",
           "TACOGB_F64", "TACOGB_F32", "TACOGB_BF16", "VARIANT_AUTO"]


def _stream_ptr(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


_VTYPE = {8: TACOGB_F64, 4: TACOGB_F32}


class CsrMatrix:
    """A CSR matrix resident on the GPU (torch int32 pos/crd, float64 or float32 vals)."""

    def __init__(self, pos, crd, vals, cols):
        import torch
        assert pos.dtype == torch.int32 and crd.dtype == torch.int32
        assert pos.is_cuda and crd.is_cuda and vals.is_cuda
        self.pos, self.crd, self.vals = pos, crd, vals
        self.rows = pos.numel() - 1
        self.cols = cols
        self.nnz = crd.numel()
        self.vtype = _VTYPE[vals.element_size()]

    @classmethod
    def from_numpy(cls, pos, crd, vals, cols, device="cuda", dtype=None):
        import torch
        v = torch.from_numpy(vals)
        if dtype is not None:
            v = v.to(dtype)
        return cls(torch.from_numpy(pos).to(device), torch.from_numpy(crd).to(device),
                   v.to(device), cols)

    def as_csr(self):
        c = _native.Csr()
        c.rows, c.cols, c.nnz = self.rows, self.cols, self.nnz
        c.pos, c.crd, c.vals = self.pos.data_ptr(), self.crd.data_ptr(), self.vals.data_ptr()
        c.vtype = self.vtype
        return c


class CsfTensor:
    """An order-3 tensor in taco's {Sparse,Sparse,Sparse} storage on the GPU ({Dense,Sparse,Sparse}
    when crd0 is None): int32 torch tensors crd0 (level-0 i), pos1/crd1 (one (i,j) fiber per
    level-1 entry), pos2/crd2 and float64 or float32 vals."""

    def __init__(self, dims, crd0, pos1, crd1, pos2, crd2, vals):
        self.dims = tuple(int(d) for d in dims)
        self.crd0, self.pos1, self.crd1 = crd0, pos1, crd1
        self.pos2, self.crd2, self.vals = pos2, crd2, vals
        self.n0 = self.dims[0] if crd0 is None else crd0.numel()
        self.nfib = crd1.numel()
        self.nnz = crd2.numel()
        self.vtype = _VTYPE[vals.element_size()]

    @classmethod
    def from_numpy(cls, dims, crd0, pos1, crd1, pos2, crd2, vals, device="cuda", dtype=None,
                   dense0=False):
        import torch
        t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
        v = torch.from_numpy(vals)
        if dtype is not None:
            v = v.to(dtype)
        return cls(dims, None if dense0 else t(crd0), t(pos1), t(crd1), t(pos2), t(crd2),
                   v.to(device))

    def as_csf3(self):
        c = _native.Csf3()
        for m in range(3):
            c.dims[m] = self.dims[m]
        c.n0, c.nfib, c.nnz = self.n0, self.nfib, self.nnz
        c.crd0 = None if self.crd0 is None else self.crd0.data_ptr()
        c.pos1, c.crd1 = self.pos1.data_ptr(), self.crd1.data_ptr()
        c.pos2, c.crd2, c.vals = self.pos2.data_ptr(), self.crd2.data_ptr(), self.vals.data_ptr()
        c.vtype = self.vtype
        return c


def ttv(B, c, dense=False, variant=VARIANT_AUTO, stream=None):
    """A(i,j) = B(i,j,k) * c(k): one value per (i,j) fiber of B (tacogb_ttv) or, with dense=True,
    taco's dense dims[0] x dims[1] result (tacogb_ttv_dense)."""
    import torch
    b = B.as_csf3()
    shape = (B.dims[0], B.dims[1]) if dense else (B.nfib,)
    out = torch.empty(shape, dtype=B.vals.dtype, device=B.vals.device)
    fn = lib().tacogb_ttv_dense if dense else lib().tacogb_ttv
    check(fn(ctypes.byref(b), c.data_ptr(), out.data_ptr(), variant, _stream_ptr(stream)),
          "tacogb_ttv")
    return out


def ttm(B, C, dense=False, variant=VARIANT_AUTO, stream=None):
    """A(i,j,l) = B(i,j,k) * C(k,l): one row of L values per (i,j) fiber (tacogb_ttm) or taco's
    dense dims[0] x dims[1] x L result (tacogb_ttm_dense)."""
    import torch
    L = C.shape[1]
    b = B.as_csf3()
    shape = (B.dims[0], B.dims[1], L) if dense else (B.nfib, L)
    out = torch.empty(shape, dtype=B.vals.dtype, device=B.vals.device)
    fn = lib().tacogb_ttm_dense if dense else lib().tacogb_ttm
    check(fn(ctypes.byref(b), L, C.data_ptr(), out.data_ptr(), variant, _stream_ptr(stream)),
          "tacogb_ttm")
    return out


def mttkrp(B, C, D, variant=VARIANT_AUTO, stream=None):
    """A(i,j) = B(i,k,l) * C(k,j) * D(l,j): dense dims[0] x J result (tacogb_mttkrp)."""
    import torch
    J = C.shape[1]
    b = B.as_csf3()
    out = torch.empty(B.dims[0], J, dtype=B.vals.dtype, device=B.vals.device)
    check(lib().tacogb_mttkrp(ctypes.byref(b), J, C.data_ptr(), D.data_ptr(), out.data_ptr(),
                              variant, _stream_ptr(stream)), "tacogb_mttkrp")
    return out


def spmv(A, x, y=None, variant=VARIANT_AUTO, stream=None):
    """y = A x on the GPU through tacogb_spmv (FP64, or FP32 with compensated accumulation)."""
    import torch
    if y is None:
        y = torch.empty(A.rows, dtype=x.dtype, device=x.device)
    c = A.as_csr()
    check(lib().tacogb_spmv(ctypes.byref(c), x.data_ptr(), y.data_ptr(), variant,
                            _stream_ptr(stream)), "tacogb_spmv")
    return y


_BTYPE = {8: TACOGB_F64, 4: TACOGB_F32, 2: TACOGB_BF16}


def spmm(A, B, C=None, variant=VARIANT_AUTO, stream=None):
    """C = A B on the GPU through tacogb_spmm.  B is a (A.cols x N) row-major torch tensor of
    float64 (A FP64), float32 or bfloat16 (A FP32); C is float64 or float32 accordingly."""
    import torch
    N = B.shape[1]
    if C is None:
        C = torch.empty(A.rows, N, dtype=torch.float64 if A.vtype == TACOGB_F64 else torch.float32,
                        device=B.device)
    c = A.as_csr()
    check(lib().tacogb_spmm(ctypes.byref(c), N, B.data_ptr(), _BTYPE[B.element_size()],
                            C.data_ptr(), variant, _stream_ptr(stream)), "tacogb_spmm")
    return C


def sddmm(B, C, D, out=None, dense=False, variant=VARIANT_AUTO, stream=None):
    """A(i,k) = B(i,k) * C(i,j) * D(j,k) on the GPU: B a CsrMatrix, C (B.rows x J) and D
    (J x B.cols) row-major torch tensors of B's value type.  Returns the values at B's nonzeros
    (tacogb_sddmm) or, with dense=True, taco's dense B.rows x B.cols result, zero outside B's
    pattern (tacogb_sddmm_dense)."""
    import torch
    J = C.shape[1]
    b = B.as_csr()
    if dense:
        if out is None:
            out = torch.empty(B.rows, B.cols, dtype=B.vals.dtype, device=C.device)
        check(lib().tacogb_sddmm_dense(ctypes.byref(b), J, C.data_ptr(), D.data_ptr(),
                                       out.data_ptr(), B.cols, variant, _stream_ptr(stream)),
              "tacogb_sddmm_dense")
        return out
    if out is None:
        out = torch.empty(B.nnz, dtype=B.vals.dtype, device=C.device)
    check(lib().tacogb_sddmm(ctypes.byref(b), J, C.data_ptr(), D.data_ptr(), out.data_ptr(),
                             variant, _stream_ptr(stream)), "tacogb_sddmm")
    return out


def sddmm_variants():
    L = lib()
    return [L.tacogb_sddmm_variant_name(i).decode() for i in range(L.tacogb_sddmm_variant_count())]


def spgemm(A, B, stream=None):
    """C = A B for CSR A and B on the GPU (two phases, as taco's assemble then compute):
    tacogb_spgemm_symbolic writes C's pos and returns nnz(C) (synchronising), tacogb_spgemm_fill
    writes the sorted columns, tacogb_spgemm_numeric the values.  Returns a CsrMatrix."""
    import torch
    a, b = A.as_csr(), B.as_csr()
    L, sp = lib(), _stream_ptr(stream)
    pos = torch.empty(A.rows + 1, dtype=torch.int32, device=A.pos.device)
    nnz = ctypes.c_int64(0)
    check(L.tacogb_spgemm_symbolic(ctypes.byref(a), ctypes.byref(b), pos.data_ptr(),
                                   ctypes.byref(nnz), sp), "tacogb_spgemm_symbolic")
    crd = torch.empty(nnz.value, dtype=torch.int32, device=A.pos.device)
    vals = torch.empty(nnz.value, dtype=A.vals.dtype, device=A.pos.device)
    check(L.tacogb_spgemm_fill(ctypes.byref(a), ctypes.byref(b), pos.data_ptr(), crd.data_ptr(),
                               sp), "tacogb_spgemm_fill")
    check(L.tacogb_spgemm_numeric(ctypes.byref(a), ctypes.byref(b), pos.data_ptr(),
                                  crd.data_ptr(), vals.data_ptr(), sp), "tacogb_spgemm_numeric")
    return CsrMatrix(pos, crd, vals, B.cols)


def pack_csr(rows, cols, coord_rows, coord_cols, vals, stream=None):
    """COO -> CSR on the GPU through tacogb_pack_csr: int32 coordinate tensors and float64 or
    float32 values on the GPU, any order, duplicates summed.  Returns a CsrMatrix."""
    import torch
    n = coord_rows.numel()
    dev = coord_rows.device
    pos = torch.empty(rows + 1, dtype=torch.int32, device=dev)
    crd = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    out = torch.empty(max(n, 1), dtype=vals.dtype, device=dev)
    nnz = ctypes.c_int64(0)
    check(lib().tacogb_pack_csr(rows, cols, n, coord_rows.data_ptr(), coord_cols.data_ptr(),
                                vals.data_ptr(), _VTYPE[vals.element_size()], pos.data_ptr(),
                                crd.data_ptr(), out.data_ptr(), ctypes.byref(nnz),
                                _stream_ptr(stream)), "tacogb_pack_csr")
    k = nnz.value
    return CsrMatrix(pos, crd[:k].clone(), out[:k].clone(), cols)


def read_coo(path):
    """(rows, cols, coord_rows, coord_cols, vals) numpy arrays of a .mtx or .tns file, as taco's
    readers insert them (tacogb_read_coo)."""
    import numpy as np
    L = lib()
    rows, cols, n = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
    pr, pc, pv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    check(L.tacogb_read_coo(str(path).encode(), ctypes.byref(rows), ctypes.byref(cols),
                            ctypes.byref(n), ctypes.byref(pr), ctypes.byref(pc), ctypes.byref(pv)),
          "tacogb_read_coo")
    k = n.value
    try:
        as_np = lambda p, ct: np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ct)),  # noqa
                                                     (max(k, 1),))[:k].copy()
        out = (rows.value, cols.value, as_np(pr, ctypes.c_int32), as_np(pc, ctypes.c_int32),
               as_np(pv, ctypes.c_double))
    finally:
        for p in (pr, pc, pv):
            L.tacogb_free_host(p)
    return out


def read_csc(path):
    """(rows, cols, colptr, rowidx, vals) numpy arrays of a Rutherford-Boeing (.rb, RUA) file, as
    taco's readRB loads it into CSC (tacogb_read_rb)."""
    import numpy as np
    L = lib()
    rows, cols, n = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
    pp, pr, pv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    check(L.tacogb_read_rb(str(path).encode(), ctypes.byref(rows), ctypes.byref(cols),
                           ctypes.byref(n), ctypes.byref(pp), ctypes.byref(pr), ctypes.byref(pv)),
          "tacogb_read_rb")
    k = n.value
    try:
        as_np = lambda p, ct, m: np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ct)),  # noqa
                                                        (max(m, 1),))[:m].copy()
        out = (rows.value, cols.value, as_np(pp, ctypes.c_int32, cols.value + 1),
               as_np(pr, ctypes.c_int32, k), as_np(pv, ctypes.c_double, k))
    finally:
        for p in (pp, pr, pv):
            L.tacogb_free_host(p)
    return out


def read_csr(path, device="cuda"):
    """A .mtx, .tns or .rb file as a CsrMatrix on the GPU: parsed on the host (all threads for
    .mtx/.tns), then packed (tacogb_pack_csr, duplicates summed in file order) or, for a
    Rutherford-Boeing file's CSC, transposed (tacogb_csc_to_csr) on the GPU."""
    import torch
    t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
    if str(path).lower().endswith(".rb"):
        rows, cols, colptr, rowidx, v = read_csc(path)
        nnz = len(rowidx)
        pos = torch.empty(rows + 1, dtype=torch.int32, device=device)
        crd = torch.empty(nnz, dtype=torch.int32, device=device)
        vals = torch.empty(nnz, dtype=torch.float64, device=device)
        cp, ri, vv = t(colptr), t(rowidx), t(v)
        check(lib().tacogb_csc_to_csr(rows, cols, nnz, cp.data_ptr(), ri.data_ptr(), vv.data_ptr(),
                                      TACOGB_F64, pos.data_ptr(), crd.data_ptr(), vals.data_ptr(),
                                      None), "tacogb_csc_to_csr")
        return CsrMatrix(pos, crd, vals, cols)
    rows, cols, ri, ci, v = read_coo(path)
    return pack_csr(rows, cols, t(ri), t(ci), t(v))


def spmm_variants():
    L = lib()
    return [L.tacogb_spmm_variant_name(i).decode() for i in range(L.tacogb_spmm_variant_count())]


def spmv_variants():
    L = lib()
    return [L.tacogb_spmv_variant_name(i).decode() for i in range(L.tacogb_spmv_variant_count())]


class _BatchPlan:
    _h = None

    def run(self, stream=None):
        check(lib().tacogb_batch_run(self._h, _stream_ptr(stream)), "tacogb_batch_run")

    def matrix_cycles(self, stream=None):
        """Per-matrix SM cycles of the last run (the autotuner's cost measure)."""
        import numpy as np
        out = np.empty(self.count, dtype=np.int64)
        check(lib().tacogb_batch_matrix_cycles(self._h, out.ctypes.data, _stream_ptr(stream)),
              "tacogb_batch_matrix_cycles")
        return out

    def close(self):
        if self._h:
            lib().tacogb_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SpmvBatch(_BatchPlan):
    """A plan for y_m = A_m x_m over many CsrMatrix objects, run as one CUDA-graph launch
    (tacogb_batch_create / tacogb_batch_run).  variants[m] names how matrix m is cut into work
    units (an index into batch_variants()); precision 1 selects native FP64 accumulation."""

    def __init__(self, mats, xs, ys, precision=0, variants=None):
        n = self.count = len(mats)
        if not (n == len(xs) == len(ys)):
            raise ValueError("mats, xs and ys differ in length")
        self._keep = (list(mats), list(xs), list(ys))
        csr = (_native.Csr * n)(*[A.as_csr() for A in mats])
        xp = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
        yp = (ctypes.c_void_p * n)(*[y.data_ptr() for y in ys])
        var = None if variants is None else (ctypes.c_int32 * n)(*[int(v) for v in variants])
        self._h = ctypes.c_void_p()
        check(lib().tacogb_batch_create(n, csr, xp, yp, precision, var, ctypes.byref(self._h)),
              "tacogb_batch_create")


class SpmmBatch(_BatchPlan):
    """A plan for C_m = A_m B_m over many CsrMatrix objects with dense row-major B_m (cols x N)
    and C_m (rows x N), N shared, run as one CUDA-graph launch (tacogb_batch_spmm_create)."""

    def __init__(self, mats, Bs, Cs, precision=0):
        n = self.count = len(mats)
        if not (n == len(Bs) == len(Cs)):
            raise ValueError("mats, Bs and Cs differ in length")
        N = int(Bs[0].shape[1])
        self._keep = (list(mats), list(Bs), list(Cs))
        csr = (_native.Csr * n)(*[A.as_csr() for A in mats])
        bp = (ctypes.c_void_p * n)(*[b.data_ptr() for b in Bs])
        cp = (ctypes.c_void_p * n)(*[c.data_ptr() for c in Cs])
        self._h = ctypes.c_void_p()
        check(lib().tacogb_batch_spmm_create(n, csr, N, bp, _BTYPE[Bs[0].element_size()], cp,
                                             precision, ctypes.byref(self._h)),
              "tacogb_batch_spmm_create")


def batch_variants():
    L = lib()
    return [L.tacogb_batch_variant_name(i).decode() for i in range(L.tacogb_batch_variant_count())]
