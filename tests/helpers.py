"""Shared test helpers: taco's own randomized test inputs, error norms, and the taco-generated
reference kernels driven through taco_tensor_t."""
import ctypes
import ctypes.util

import numpy as np

from oracle import oracle as O
from taco_gb300 import taco as T

_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.rand.restype = ctypes.c_int
RAND_MAX = 2147483647  # glibc


def taco_rand_csr(rows, cols, sparsity, seed=75883, dense_b_cols=None, b_sparse=False):
    """The inputs of taco's randomized scheduling tests (test/tests-scheduling-eval.cpp:549-662,
    843-889): srand(seed); A(i,j) inserted when rand_float < SPARSITY with value
    (double)(int)(rand_float*3/SPARSITY); then B filled by the same draw, densely or sparsely.
    rand_float is (float)rand()/(float)RAND_MAX, evaluated in single precision."""
    _libc.srand(seed)
    sp = np.float32(sparsity)

    def draw():
        return np.float32(_libc.rand()) / np.float32(RAND_MAX)

    def fill(nr, nc, sparse):
        pos = [0]
        crd, vals = [], []
        dense = np.zeros((nr, nc))
        for i in range(nr):
            for j in range(nc):
                r = draw()
                if (not sparse) or r < sp:
                    v = float(int(np.float32(np.float32(r * np.float32(3)) / sp)))
                    crd.append(j)
                    vals.append(v)
                    dense[i, j] = v
            pos.append(len(crd))
        return (np.array(pos, np.int32), np.array(crd, np.int32), np.array(vals, np.float64),
                dense)

    A = fill(rows, cols, True)
    B = None
    if dense_b_cols is not None:
        B = fill(cols, dense_b_cols, b_sparse)
    return A, B


def taco_sddmm_inputs(I, J, K, sparsity, seed):
    """The inputs of taco's sddmm tests (test/tests-scheduling-eval.cpp:783-840 and
    1360-1417): srand(seed); C (I x J) dense, then B (I x K) with an entry where
    rand_float < SPARSITY, then D (J x K) dense, every value (double)(int)(rand_float*3/SPARSITY).
    Returns (pos, crd, vals), C, D."""
    _libc.srand(seed)
    sp = np.float32(sparsity)

    def draw():
        r = np.float32(_libc.rand()) / np.float32(RAND_MAX)
        return r, float(int(np.float32(np.float32(r * np.float32(3)) / sp)))

    C = np.array([[draw()[1] for _ in range(J)] for _ in range(I)])
    pos, crd, vals = [0], [], []
    for i in range(I):
        for k in range(K):
            r, v = draw()
            if r < sp:
                crd.append(k)
                vals.append(v)
        pos.append(len(crd))
    D = np.array([[draw()[1] for _ in range(K)] for _ in range(J)])
    return (np.array(pos, np.int32), np.array(crd, np.int32), np.array(vals)), C, D


def taco_tensor3_inputs(dims, sparsity, seed, dense_shapes):
    """The inputs of taco's order-3 tests (test/tests-scheduling-eval.cpp:993-1206, 1420-1580):
    srand(seed); B's coordinates in lexicographic order with an entry where
    rand_float < SPARSITY, value (double)(int)(rand_float*3/SPARSITY); then each dense operand
    in row-major order, value (double)(int)(rand_float*3).  Returns (coords n x 3, vals,
    [dense arrays])."""
    _libc.srand(seed)
    sp = np.float32(sparsity)

    def draw():
        return np.float32(_libc.rand()) / np.float32(RAND_MAX)

    coords, vals = [], []
    I, J, K = dims
    for i in range(I):
        for j in range(J):
            for k in range(K):
                r = draw()
                if r < sp:
                    coords.append((i, j, k))
                    vals.append(float(int(np.float32(np.float32(r * np.float32(3)) / sp))))
    mats = []
    for shape in dense_shapes:
        n = int(np.prod(shape))
        mats.append(np.array([float(int(np.float32(draw() * np.float32(3)))) for _ in range(n)])
                    .reshape(shape))
    return np.array(coords, np.int32).reshape(-1, 3), np.array(vals), mats


def csf3(dims, coords, vals, dense0=False):
    """taco's {Sparse,Sparse,Sparse} (or {Dense,Sparse,Sparse}) storage of lexicographically
    sorted, distinct coordinates: (dims, crd0, pos1, crd1, pos2, crd2, vals); with dense0 the
    first level lists every i (crd0 = 0..I-1)."""
    coords = np.asarray(coords, np.int64).reshape(-1, 3)
    n = len(coords)
    new_f = np.ones(n, bool)
    new_f[1:] = np.any(coords[1:, :2] != coords[:-1, :2], axis=1)
    fib = np.flatnonzero(new_f)
    pos2 = np.append(fib, n).astype(np.int32)
    crd2 = coords[:, 2].astype(np.int32)
    fi, fj = coords[fib, 0], coords[fib, 1]
    if dense0:
        crd0 = np.arange(dims[0], dtype=np.int32)
    else:
        crd0 = np.unique(fi).astype(np.int32)
    pos1 = np.searchsorted(fi, crd0, side="left").astype(np.int32)
    pos1 = np.append(pos1, len(fib)).astype(np.int32)
    return (tuple(int(d) for d in dims), crd0, pos1, fj.astype(np.int32), pos2, crd2,
            np.asarray(vals, np.float64))


def taco_csf3_tensor(B, dense0=False):
    """A taco_tensor_t over a csf3 tuple (taco_gb300.taco.csf3)."""
    return T.csf3(*B, dense0=dense0)


def ref_tensor3(pattern, B, *dense):
    """taco's generated compute for ttv / ttm / mttkrp ({Sparse,Sparse,Sparse} B, dense
    operands and result) on host arrays."""
    L = O.ref_lib(pattern)
    O.ref_set_threads(1)
    dims = B[0]
    Bt = taco_csf3_tensor(B)
    ops = [np.ascontiguousarray(d, np.float64) for d in dense]
    if pattern == "ttv":
        A = np.empty((dims[0], dims[1]))
    elif pattern == "ttm":
        A = np.empty((dims[0], dims[1], ops[0].shape[1]))
    else:
        A = np.empty((dims[0], ops[0].shape[1]))
    At = T.dense(A, list(A.shape))
    ts = [T.dense(o, list(o.shape)) for o in ops]
    assert L.compute(At.ptr, Bt.ptr, *[t.ptr for t in ts]) == 0
    return A


def to_dcsr(pos, crd):
    """(crd0, pos1) of the {Sparse,Sparse} form of a CSR matrix: its nonempty rows."""
    lens = np.diff(pos)
    crd0 = np.flatnonzero(lens > 0).astype(np.int32)
    pos1 = np.concatenate([[0], np.cumsum(lens[crd0])]).astype(np.int32)
    return crd0, pos1


def to_csc(pos, crd, vals, cols):
    """(colpos, rowidx, vals) of a CSR matrix's CSC form, rows ascending in each column."""
    rows = np.repeat(np.arange(len(pos) - 1, dtype=np.int32), np.diff(pos))
    o = np.lexsort((rows, crd))
    colpos = np.searchsorted(crd[o], np.arange(cols + 1), side="left").astype(np.int32)
    return colpos, rows[o].astype(np.int32), np.asarray(vals)[o]


def taco_dcsr_tensor(crd0, pos1, crd, vals, dims):
    pos0 = np.array([0, len(crd0)], np.int32)
    t = T.TacoTensor(list(dims), [T.MODE_SPARSE, T.MODE_SPARSE], vals=vals,
                     index_arrays={0: (pos0, crd0), 1: (pos1, crd)})
    t._keep.append(pos0)
    return t


def taco_csc_tensor(colpos, rowidx, vals, dims):
    return T.TacoTensor(list(dims), [T.MODE_DENSE, T.MODE_SPARSE], vals=vals,
                        index_arrays={1: (colpos, rowidx)}, mode_ordering=[1, 0])


def taco_sparse_vector(idx, vals, n):
    pos = np.array([0, len(idx)], np.int32)
    t = T.TacoTensor([n], [T.MODE_SPARSE], vals=vals, index_arrays={0: (pos, idx)})
    t._keep.append(pos)
    return t


def taco_sparse_vector_result(n, csize=64):
    return T.TacoTensor([n], [T.MODE_SPARSE], vals=None, csize=csize,
                        index_arrays={0: (None, None)})


def ref_spmv_formats(kind, pos, crd, vals, cols, x, x_sparse=None):
    """taco's generated SpMV for A DCSR ("dcsr"), CSC ("csc") or DCSR with {Sparse} x and y
    ("dcsr_sv": x_sparse = (idx, vals); returns (crd, vals) of y)."""
    import ctypes
    rows = len(pos) - 1
    L = O.ref_lib("spmv_" + kind)
    O.ref_set_threads(1)
    if kind == "csc":
        At = taco_csc_tensor(*to_csc(pos, crd, vals, cols), [rows, cols])
    else:
        crd0, pos1 = to_dcsr(pos, crd)
        At = taco_dcsr_tensor(crd0, pos1, crd, vals, [rows, cols])
    if kind != "dcsr_sv":
        y = np.empty(rows)
        Yt, Xt = T.dense(y, [rows]), T.dense(x, [cols])
        assert L.compute(Yt.ptr, At.ptr, Xt.ptr) == 0
        return y
    Xt = taco_sparse_vector(x_sparse[0], x_sparse[1], cols)
    Yt = taco_sparse_vector_result(rows)
    assert L.assemble(Yt.ptr, At.ptr, Xt.ptr) == 0
    assert L.compute(Yt.ptr, At.ptr, Xt.ptr) == 0
    n = np.ctypeslib.as_array(ctypes.cast(Yt.index(0, 0), ctypes.POINTER(ctypes.c_int32)), (2,))[1]
    yc = np.ctypeslib.as_array(ctypes.cast(Yt.index(0, 1), ctypes.POINTER(ctypes.c_int32)), (n,))
    yv = np.ctypeslib.as_array(ctypes.cast(Yt.vals_ptr, ctypes.POINTER(ctypes.c_double)), (n,))
    return yc.copy(), yv.copy()


def ref_spmm_dcsr(pos, crd, vals, B):
    L = O.ref_lib("spmm_dcsr")
    O.ref_set_threads(1)
    rows, cols, N = len(pos) - 1, B.shape[0], B.shape[1]
    crd0, pos1 = to_dcsr(pos, crd)
    At = taco_dcsr_tensor(crd0, pos1, crd, vals, [rows, cols])
    C = np.empty((rows, N))
    Ct, Bt = T.dense(C, [rows, N]), T.dense(np.ascontiguousarray(B), [cols, N])
    assert L.compute(Ct.ptr, At.ptr, Bt.ptr) == 0
    return C


def normwise(approx, exact):
    """||approx - exact||_2 / ||exact||_2 (0 when both are zero)."""
    a = np.asarray(approx, dtype=np.float64).ravel()
    e = np.asarray(exact, dtype=np.float64).ravel()
    scale = max(np.max(np.abs(e)) if e.size else 0.0, 1e-300)
    a, e = a / scale, e / scale  # no overflow in the squares
    den = np.linalg.norm(e)
    num = np.linalg.norm(a - e)
    return num / den if den > 0 else num


def ref_spmv(pos, crd, vals, x, threads=1):
    """taco's generated SpMV (assemble + compute) on host arrays."""
    L = O.ref_lib("spmv")
    O.ref_set_threads(threads)
    rows, cols = len(pos) - 1, len(x)
    A = T.csr(pos, crd, vals, [rows, cols])
    X = T.dense(x, [cols])
    y = np.empty(rows, dtype=np.float64)
    Y = T.dense(y, [rows])
    assert L.compute(Y.ptr, A.ptr, X.ptr) == 0
    return y


def ref_spmm(pos, crd, vals, B, threads=1):
    """taco's generated SpMM compute (C(i,k) = A(i,j) * B(j,k), dense row-major B, C)."""
    L = O.ref_lib("spmm")
    O.ref_set_threads(threads)
    rows, cols, N = len(pos) - 1, B.shape[0], B.shape[1]
    B = np.ascontiguousarray(B)
    C = np.empty((rows, N), dtype=np.float64)
    At, Bt, Ct = T.csr(pos, crd, vals, [rows, cols]), T.dense(B, [cols, N]), T.dense(C, [rows, N])
    assert L.compute(Ct.ptr, At.ptr, Bt.ptr) == 0
    return C


def ref_sddmm(pos, crd, vals, C, D, threads=1):
    """taco's generated SDDMM compute (dense I x K result) on host arrays."""
    L = O.ref_lib("sddmm")
    O.ref_set_threads(threads)
    C, D = np.ascontiguousarray(C, np.float64), np.ascontiguousarray(D, np.float64)
    I, J, K = C.shape[0], C.shape[1], D.shape[1]
    A = np.empty((I, K))
    At, Bt = T.dense(A, [I, K]), T.csr(pos, crd, vals, [I, K])
    Ct, Dt = T.dense(C, [I, J]), T.dense(D, [J, K])
    assert L.compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr) == 0
    return A


def ref_spgemm(A, B, threads=1, pattern="spgemm"):
    """taco's generated SpGEMM (assemble then compute) on host CSR arrays; A, B = (pos, crd,
    vals, cols).  Returns (pos, crd, vals) of C copied out of the arrays taco allocated.
    pattern "spgemm_sched" runs taco's parallel two-pass schedule (scheduleSpGEMMCPU)."""
    import ctypes
    L = O.ref_lib(pattern)
    O.ref_set_threads(threads)
    (ap, ac, av, acols), (bp, bc, bv, bcols) = A, B
    rows = len(ap) - 1
    At, Bt = T.csr(ap, ac, av, [rows, acols]), T.csr(bp, bc, bv, [acols, bcols])
    Ct = T.csr_result([rows, bcols])
    assert L.assemble(Ct.ptr, At.ptr, Bt.ptr) == 0
    assert L.compute(Ct.ptr, At.ptr, Bt.ptr) == 0
    pos = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 0), ctypes.POINTER(ctypes.c_int32)),
                                (rows + 1,)).copy()
    nnz = int(pos[-1])
    crd = np.ctypeslib.as_array(ctypes.cast(Ct.index(1, 1), ctypes.POINTER(ctypes.c_int32)),
                                (max(nnz, 1),))[:nnz].copy()
    vals = np.ctypeslib.as_array(ctypes.cast(Ct.vals_ptr, ctypes.POINTER(ctypes.c_double)),
                                 (max(nnz, 1),))[:nnz].copy()
    return pos, crd, vals


def sample_rows(pos, count, seed=0, longest=64):
    """Sorted distinct row indices for a sampled check of a large result: the `longest` longest
    rows (they span many merge tiles, so their carries cross tile and CTA boundaries), the first
    and last rows, and random rows up to `count`."""
    rows = len(pos) - 1
    lens = np.diff(pos)
    rng = np.random.default_rng(seed)
    pick = [np.argsort(lens, kind="stable")[-longest:], [0, rows - 1],
            rng.choice(rows, min(count, rows), replace=False)]
    return np.unique(np.concatenate(pick).astype(np.int64))


def sub_rows(pos, crd, vals, idx):
    """(pos, crd, vals) of the CSR matrix made of rows idx of (pos, crd, vals), in that order."""
    lens = (pos[idx + 1] - pos[idx]).astype(np.int64)
    spos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    take = np.concatenate([np.arange(pos[i], pos[i + 1], dtype=np.int64) for i in idx]) \
        if len(idx) else np.zeros(0, np.int64)
    return spos, crd[take], vals[take]


def read_abi_record(path):
    """The calls recorded by tests/cpp/tacogb_recorder.c: a list of calls, each a list of
    tensors {order, csize, dims, ordering, types, levels, vals}; levels[m] is None for a dense
    mode or an unassembled level, else (pos, crd); vals is None when absent."""
    raw = open(path, "rb").read()
    off = 0

    def i64():
        nonlocal off
        v = int(np.frombuffer(raw, np.int64, 1, off)[0])
        off += 8
        return v

    def arr(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype, count, off).copy()
        off += a.nbytes
        return a

    calls = []
    while off < len(raw):
        tensors = []
        for _ in range(i64()):
            order, csize = i64(), i64()
            dims = [i64() for _ in range(order)]
            ordering = [i64() for _ in range(order)]
            types = [i64() for _ in range(order)]
            levels = []
            for m in range(order):
                if types[m] == 0:
                    levels.append(None)
                    continue
                np_ = i64()
                if np_ < 0:
                    levels.append(None)
                    continue
                pos = arr(np.int32, np_)
                crd = arr(np.int32, i64())
                levels.append((pos, crd))
            nv = i64()
            vals = arr(np.float64 if csize == 64 else np.float32, nv) if nv >= 0 else None
            tensors.append({"order": order, "csize": csize, "dims": dims, "ordering": ordering,
                            "types": types, "levels": levels, "vals": vals})
        calls.append(tensors)
    return calls


def read_result_dump(path):
    """(levels, vals) of a result written by taco_dropin's dump_result: levels[m] None for a
    dense mode, else (pos, crd)."""
    raw = open(path, "rb").read()
    off = 0
    order = int(np.frombuffer(raw, np.int32, 1, off)[0])
    off += 4
    levels = []
    for _ in range(order):
        kind = int(np.frombuffer(raw, np.int32, 1, off)[0])
        off += 4
        if not kind:
            levels.append(None)
            continue
        n = int(np.frombuffer(raw, np.int64, 1, off)[0])
        off += 8
        pos = np.frombuffer(raw, np.int32, n, off).copy()
        off += 4 * n
        n = int(np.frombuffer(raw, np.int64, 1, off)[0])
        off += 8
        crd = np.frombuffer(raw, np.int32, n, off).copy()
        off += 4 * n
        levels.append((pos, crd))
    n = int(np.frombuffer(raw, np.int64, 1, off)[0])
    off += 8
    vals = np.frombuffer(raw, np.float64, n, off).copy()
    return levels, vals


def record_to_arrays(prefix, tensor):
    """Flattens one recorded tensor into npz-ready arrays under `prefix`."""
    out = {prefix + "_hdr": np.array([tensor["order"], tensor["csize"]] + tensor["dims"]
                                     + tensor["ordering"] + tensor["types"], np.int64)}
    for m, lv in enumerate(tensor["levels"]):
        if lv is not None:
            out["%s_pos%d" % (prefix, m)], out["%s_crd%d" % (prefix, m)] = lv
    if tensor["vals"] is not None:
        out[prefix + "_vals"] = tensor["vals"]
    return out


def arrays_to_taco(g, prefix, with_arrays=True):
    """A taco_tensor_t (taco_gb300.taco.TacoTensor) rebuilt from record_to_arrays's arrays: the
    same order, csize, dimensions, mode ordering, mode types, index arrays and values."""
    h = [int(v) for v in g[prefix + "_hdr"]]
    order, csize = h[0], h[1]
    dims, ordering, types = h[2:2 + order], h[2 + order:2 + 2 * order], h[2 + 2 * order:]
    idx = {}
    for m in range(order):
        if types[m] == 1:
            key = "%s_pos%d" % (prefix, m)
            if with_arrays and key in g:
                idx[m] = (np.ascontiguousarray(g[key]), np.ascontiguousarray(g["%s_crd%d" % (prefix, m)]))
            else:
                idx[m] = (None, None)
    vals = None
    if with_arrays and prefix + "_vals" in g:
        vals = np.ascontiguousarray(g[prefix + "_vals"])
    return T.TacoTensor(dims, types, vals=vals, index_arrays=idx, csize=csize,
                        mode_ordering=ordering)
