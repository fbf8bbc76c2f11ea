"""Generates the golden fixtures in tests/golden/ by running taco's own generated C code.

The generated code comes from taco's CLI built from the reference sources by
oracle/Makefile.ref (taco "y(i) = A(i,j) * x(j)" -f=A:ds -write-source=..., etc.) and is
compiled with taco's JIT flags.  Run from the repository root, naming taco's source tree:

    TACO_REFERENCE=<taco source tree> python tests/golden/make_golden.py

Each fixture stores its inputs and taco's outputs, so the tests that read it need neither the
reference nor the generator.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from taco_gb300 import build as B  # noqa: E402
from taco_gb300 import workloads as W  # noqa: E402
from tests import helpers as H  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, **arrays):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)
    print("wrote", name, {k: v.shape for k, v in arrays.items()})


def spmv_cases():
    (pos, crd, vals, _), _ = H.taco_rand_csr(1021 // 10, 1039 // 10, 0.3)
    x = W.dense(11, 1039 // 10)
    save("spmv_taco_rand", pos=pos, crd=crd, vals=vals, x=x, y=H.ref_spmv(pos, crd, vals, x))

    s = W.spec(1024, kind=W.UNIFORM, len_lo=4, len_hi=28, seed=W.SEED_BASE + 101)
    pos, crd, vals = W.generate(s)
    x = W.dense(12, s.cols)
    save("spmv_uniform", pos=pos, crd=crd, vals=vals, x=x, y=H.ref_spmv(pos, crd, vals, x))

    s = W.spec(1024, kind=W.POWERLAW, mean=24.0, len_max=1024, seed=W.SEED_BASE + 102)
    pos, crd, vals = W.generate(s)
    x = W.dense(13, s.cols)
    save("spmv_powerlaw", pos=pos, crd=crd, vals=vals, x=x, y=H.ref_spmv(pos, crd, vals, x))

    # mostly empty rows, one dense row, rows of length 1
    rng = np.random.default_rng(14)
    rows, cols = 3000, 700
    lens = np.zeros(rows, np.int32)
    lens[rng.choice(rows, 200, replace=False)] = 1
    lens[1234] = cols
    lens[rows - 1] = 3
    pos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    crd = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens if l > 0]).astype(np.int32)
    vals = rng.uniform(-1, 1, len(crd))
    x = W.dense(15, cols)
    save("spmv_empty_rows", pos=pos, crd=crd, vals=vals, x=x, y=H.ref_spmv(pos, crd, vals, x))


def spmm_cases():
    # taco's spmmCPU inputs (test/tests-scheduling-eval.cpp:549-598): 102x103 CSR at 0.3,
    # dense 103x128 B, both from srand(75883)
    (pos, crd, vals, _), (_, _, _, Bd) = H.taco_rand_csr(1021 // 10, 1039 // 10, 0.3,
                                                          dense_b_cols=128)
    save("spmm_taco_rand", pos=pos, crd=crd, vals=vals, B=Bd, C=H.ref_spmm(pos, crd, vals, Bd))

    s = W.spec(512, kind=W.POWERLAW, mean=32.0, len_max=512, seed=W.SEED_BASE + 103)
    pos, crd, vals = W.generate(s)
    B = W.dense(16, s.cols * 64).reshape(s.cols, 64)
    save("spmm_powerlaw_n64", pos=pos, crd=crd, vals=vals, B=B, C=H.ref_spmm(pos, crd, vals, B))


def spgemm_cases():
    # taco's spgemm test inputs (test/tests-scheduling-eval.cpp:602-662): 100x100 A and B at
    # sparsity 0.03 from srand(75883), CSR x CSR
    (ap, ac, av, _), (bp, bc, bv, _) = H.taco_rand_csr(100, 100, 0.03, dense_b_cols=100,
                                                         b_sparse=True)
    cp, cc, cv = H.ref_spgemm((ap, ac, av, 100), (bp, bc, bv, 100))
    save("spgemm_taco_rand", Apos=ap, Acrd=ac, Avals=av, Bpos=bp, Bcrd=bc, Bvals=bv,
         Cpos=cp, Ccrd=cc, Cvals=cv, K=np.array([100]))

    s = W.spgemm_random(rows=512)
    ap, ac, av = W.generate(s)
    cp, cc, cv = H.ref_spgemm((ap, ac, av, s.cols), (ap, ac, av, s.cols))
    save("spgemm_random_512", Apos=ap, Acrd=ac, Avals=av, Bpos=ap, Bcrd=ac, Bvals=av,
         Cpos=cp, Ccrd=cc, Cvals=cv, K=np.array([s.cols]))

    s = W.spgemm_poisson(grid=32)
    ap, ac, av = W.generate(s)
    cp, cc, cv = H.ref_spgemm((ap, ac, av, s.cols), (ap, ac, av, s.cols))
    save("spgemm_poisson_32", Apos=ap, Acrd=ac, Avals=av, Bpos=ap, Bcrd=ac, Bvals=av,
         Cpos=cp, Ccrd=cc, Cvals=cv, K=np.array([s.cols]))


def sddmm_cases():
    # taco's sddmmGPU inputs (test/tests-scheduling-eval.cpp:1360-1417): I 102, K 103, J 128
    (pos, crd, vals), C, D = H.taco_sddmm_inputs(1021 // 10, 128, 1039 // 10, 0.3, 535366)
    save("sddmm_taco_gpu", pos=pos, crd=crd, vals=vals, C=C, D=D,
         A=H.ref_sddmm(pos, crd, vals, C, D))
    # taco's sddmmCPU inputs (:783-840): I 102, J 103, K 105
    (pos, crd, vals), C, D = H.taco_sddmm_inputs(1021 // 10, 1039 // 10, 1057 // 10, 0.3, 268238)
    save("sddmm_taco_cpu", pos=pos, crd=crd, vals=vals, C=C, D=D,
         A=H.ref_sddmm(pos, crd, vals, C, D))
    # power-law rows, real values, J 96 (three quarters of a 128-wide slab); C and D are
    # W.dense(17, 512 * 96) and W.dense(18, 96 * 512), regenerated by the tests
    s = W.spec(512, kind=W.POWERLAW, mean=32.0, len_max=512, seed=W.SEED_BASE + 104)
    pos, crd, vals = W.generate(s)
    C = W.dense(17, s.rows * 96).reshape(s.rows, 96)
    D = W.dense(18, 96 * s.cols).reshape(96, s.cols)
    save("sddmm_powerlaw_j96", pos=pos, crd=crd, vals=vals, A=H.ref_sddmm(pos, crd, vals, C, D))


def _save_csf3(name, B, A, **dense):
    dims, crd0, pos1, crd1, pos2, crd2, vals = B
    save(name, dims=np.array(dims), crd0=crd0, pos1=pos1, crd1=crd1, pos2=pos2, crd2=crd2,
         vals=vals, A=A, **dense)


def tensor3_cases():
    """taco's order-3 test inputs (test/tests-scheduling-eval.cpp), B {Sparse,Sparse,Sparse}
    (taco's mttkrpCPU has a dense first level; its values are the same)."""
    for name, dims, sp, seed in (("ttv_taco_gpu", (102, 103, 105), 0.3, 35325),
                                 ("ttv_taco_cpu", (102, 103, 105), 0.3, 9536)):
        co, v, (c,) = H.taco_tensor3_inputs(dims, sp, seed, [(dims[2],)])
        B = H.csf3(dims, co, v)
        _save_csf3(name, B, H.ref_tensor3("ttv", B, c), c=c)
    for name, dims, L, seed in (("ttm_taco_gpu", (25, 25, 30), 128, 34644),
                                ("ttm_taco_cpu", (25, 25, 26), 30, 935)):
        co, v, (C,) = H.taco_tensor3_inputs(dims, 0.1, seed, [(dims[2], L)])
        B = H.csf3(dims, co, v)
        _save_csf3(name, B, H.ref_tensor3("ttm", B, C), C=C)
    for name, dims, J, seed in (("mttkrp_taco_gpu", (25, 25, 30), 32, 5464164),
                                ("mttkrp_taco_cpu", (51, 52, 61), 51, 549694)):
        co, v, (C, D) = H.taco_tensor3_inputs(dims, 0.1, seed, [(dims[1], J), (dims[2], J)])
        B = H.csf3(dims, co, v)
        _save_csf3(name, B, H.ref_tensor3("mttkrp", B, C, D), C=C, D=D)


def format_cases():
    """SpMV with A DCSR or CSC, with A DCSR and {Sparse} x and y, and taco's spmmDCSRGPU
    (test/tests-scheduling-eval.cpp:1309-1358, srand 25643), through taco's generated code."""
    (pos, crd, vals, _), _ = H.taco_rand_csr(1021 // 10, 1039 // 10, 0.3)
    cols = 1039 // 10
    x = W.dense(21, cols)
    xi = np.arange(0, cols, 3, dtype=np.int32)
    ys_crd, ys_vals = H.ref_spmv_formats("dcsr_sv", pos, crd, vals, cols, None, (xi, x[xi]))
    save("spmv_formats_taco", pos=pos, crd=crd, vals=vals, x=x, xi=xi,
         y_dcsr=H.ref_spmv_formats("dcsr", pos, crd, vals, cols, x),
         y_csc=H.ref_spmv_formats("csc", pos, crd, vals, cols, x), ys_crd=ys_crd, ys_vals=ys_vals)
    (pos, crd, vals, _), (_, _, _, Bd) = H.taco_rand_csr(1021 // 10, 1039 // 10, 0.3, seed=25643,
                                                          dense_b_cols=128)
    save("spmm_dcsr_taco_gpu", pos=pos, crd=crd, vals=vals, B=Bd,
         C=H.ref_spmm_dcsr(pos, crd, vals, Bd))


def taco_pack_cli(rows, cols, ri, ci, v, workdir):
    """CSR (pos, crd, vals) that taco itself makes of the coordinates: the taco CLI reads them
    from a .tns file (Tensor::insert for every line, then TensorBase::pack: sort, sum
    duplicates), evaluates B(i,j) = A(i,j) with A and B in CSR, and writes B.  .tns coordinates
    are 1-based and the CLI infers each dimension from the largest coordinate, so the caller
    puts an entry at (rows-1, cols-1)."""
    import subprocess
    src = os.path.join(workdir, "pack_in.tns")
    dst = os.path.join(workdir, "pack_out.tns")
    with open(src, "w") as f:
        for a, b, x in zip(ri, ci, v):
            f.write("%d %d %r\n" % (a + 1, b + 1, float(x)))
    cli = os.path.join(ROOT, "oracle", "_ref", "bin", "taco")
    subprocess.run([cli, "B(i,j) = A(i,j)", "-f=A:ds", "-f=B:ds", "-i=A:" + src, "-o=B:" + dst,
                    "-time=1"], check=True, cwd=workdir, stdout=subprocess.DEVNULL)
    entries = [line.split() for line in open(dst) if line.strip()]
    r = np.array([int(e[0]) - 1 for e in entries], np.int64)
    c = np.array([int(e[1]) - 1 for e in entries], np.int32)
    x = np.array([float(e[2]) for e in entries])
    order = np.lexsort((c, r))
    r, c, x = r[order], c[order], x[order]
    pos = np.searchsorted(r, np.arange(rows + 1), side="left").astype(np.int32)
    return pos, c, x


def pack_cases():
    """COO with duplicates (integer values, so every summation order gives the same sums and
    the CLI's printed values are exact), a pair that cancels to an explicit zero, empty rows,
    and the last row/column present."""
    import tempfile
    rng = np.random.default_rng(21)
    rows, cols, n = 700, 500, 30000
    ri = rng.integers(0, rows, n)
    ci = rng.integers(0, cols, n)
    ri[ri % 7 == 3] = 0                     # rows 3, 10, ... stay empty
    dup = rng.choice(n, 4000, replace=False)  # repeat some coordinates
    ri = np.concatenate([ri, ri[dup], [5, 5, rows - 1]])
    ci = np.concatenate([ci, ci[dup], [7, 7, cols - 1]])
    v = np.concatenate([rng.integers(-50, 51, n + len(dup)), [13, -13, 2]]).astype(np.float64)
    perm = rng.permutation(len(ri))
    ri, ci, v = ri[perm].astype(np.int32), ci[perm].astype(np.int32), v[perm]
    with tempfile.TemporaryDirectory() as d:
        pos, crd, vals = taco_pack_cli(rows, cols, ri, ci, v, d)
    save("pack_taco_cli", rows=np.int32(rows), cols=np.int32(cols), ri=ri, ci=ci, v=v, pos=pos,
         crd=crd, vals=vals)


def reader_cases():
    """Small .mtx / .tns files (general with comments and duplicates, symmetric, array, tns)
    and, for each, the CSR that taco makes of it: the CLI reads the file with its own reader
    (readMTX / readTNS, then pack) and writes B(i,j) = A(i,j).  Values are multiples of 1/4 so
    that the CLI's printed output is exact."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(31)
    q = lambda k: rng.integers(-400, 401, k) / 4.0  # noqa: E731
    files = {}
    # general coordinate, comments, duplicates, corner entries present
    rows, cols, k = 60, 45, 700
    r, c = rng.integers(1, rows + 1, k), rng.integers(1, cols + 1, k)
    r[:2], c[:2] = [rows, 1], [cols, 1]
    r[2:12], c[2:12] = r[12:22], c[12:22]  # repeats
    lines = ["%%MatrixMarket matrix coordinate real general", "% a comment", "%another",
             "%d %d %d" % (rows, cols, k)]
    lines += ["%d %d %r" % (a, b, float(v)) for a, b, v in zip(r, c, q(k))]
    files["read_general.mtx"] = "\n".join(lines) + "\n"
    # symmetric coordinate (lower triangle with diagonal)
    n, k = 50, 300
    a, b = rng.integers(1, n + 1, k), rng.integers(1, n + 1, k)
    lo, hi = np.maximum(a, b), np.minimum(a, b)
    lo[0], hi[0] = n, n
    lines = ["%%MatrixMarket matrix coordinate real symmetric", "%d %d %d" % (n, n, k)]
    lines += ["%d %d %r" % (x, y, float(v)) for x, y, v in zip(lo, hi, q(k))]
    files["read_symmetric.mtx"] = "\n".join(lines) + "\n"
    # array (column-major, every entry, zeros included)
    rows, cols = 9, 7
    vals = q(rows * cols)
    vals[rng.choice(rows * cols, 20, replace=False)] = 0.0
    lines = ["%%MatrixMarket matrix array real general", "%d %d" % (rows, cols)]
    lines += ["%r" % float(v) for v in vals]
    files["read_array.mtx"] = "\n".join(lines) + "\n"
    # tns
    rows, cols, k = 80, 33, 500
    r, c = rng.integers(1, rows + 1, k), rng.integers(1, cols + 1, k)
    r[0], c[0] = rows, cols
    files["read_plain.tns"] = "".join("%d %d %r\n" % (a, b, float(v))
                                      for a, b, v in zip(r, c, q(k)))
    cli = os.path.join(ROOT, "oracle", "_ref", "bin", "taco")
    for name, text in files.items():
        path = os.path.join(OUT, name)
        with open(path, "w") as f:
            f.write(text)
        with tempfile.TemporaryDirectory() as d:
            dst = os.path.join(d, "out.tns")
            subprocess.run([cli, "B(i,j) = A(i,j)", "-f=A:ds", "-f=B:ds", "-i=A:" + path,
                            "-o=B:" + dst, "-time=1"], check=True, cwd=d, stdout=subprocess.DEVNULL)
            ent = [line.split() for line in open(dst) if line.strip()]
        rr = np.array([int(e[0]) - 1 for e in ent], np.int64)
        cc = np.array([int(e[1]) - 1 for e in ent], np.int32)
        vv = np.array([float(e[2]) for e in ent])
        o = np.lexsort((cc, rr))
        rr, cc, vv = rr[o], cc[o], vv[o]
        nrows = int(rr.max()) + 1
        pos = np.searchsorted(rr, np.arange(nrows + 1), side="left").astype(np.int32)
        save(name.replace(".", "_"), pos=pos, crd=cc, vals=vv)


def _write_rb(path, rows, cols, colptr, rowidx, vals, rhs_line=None):
    """A Rutherford-Boeing file (RUA) in this script's own layout: 10 integers or 4 values per
    line; with rhs_line, right-hand sides are announced (a fifth header line, no data)."""
    chunk = lambda xs, k: [xs[i:i + k] for i in range(0, len(xs), k)]  # noqa: E731
    pl = [" ".join("%d" % (x + 1) for x in c) for c in chunk(list(colptr), 10)]
    il = [" ".join("%d" % (x + 1) for x in c) for c in chunk(list(rowidx), 10)]
    vl = [" ".join("%r" % float(x) for x in c) for c in chunk(list(vals), 4)]
    hdr = ["%-72s%-8s" % ("a test matrix written by make_golden", "GOLDEN"),
           "%14d%14d%14d%14d%14d" % (len(pl) + len(il) + len(vl), len(pl), len(il), len(vl),
                                     1 if rhs_line else 0),
           "RUA%11s%14d%14d%14d%14d" % ("", rows, cols, len(rowidx), 0),
           "%-16s%-16s%-20s%-20s" % ("(10I8)", "(10I8)", "(4E24.16)", "(4E24.16)" if rhs_line else "")]
    if rhs_line:
        hdr.append(rhs_line)
    with open(path, "w") as f:
        f.write("\n".join(hdr + pl + il + vl) + "\n")


def rb_cases(reference_root):
    """Rutherford-Boeing: taco's own test matrix rua_32 (test/data/rua_32.rb and its .mtx twin).
    taco's CLI crashes on .rb input and output here, so the CSR expected of the .rb file is the
    one taco's CLI makes of rua_32.mtx; this script writes the matrix again in its own RB layout
    (read_rua32.rb) and checks that libtacogb's reader gives the same CSC for taco's file and for
    this one.  read_rhs.rb (a random matrix, right-hand sides announced) checks the fifth header
    line."""
    import subprocess
    import tempfile
    import taco_gb300 as tg
    cli = os.path.join(ROOT, "oracle", "_ref", "bin", "taco")
    src_mtx = os.path.join(reference_root, "test", "data", "rua_32.mtx")
    src_rb = os.path.join(reference_root, "test", "data", "rua_32.rb")
    with tempfile.TemporaryDirectory() as d:
        dst = os.path.join(d, "out.tns")
        subprocess.run([cli, "B(i,j) = A(i,j)", "-f=A:ds", "-f=B:ds", "-i=A:" + src_mtx,
                        "-o=B:" + dst, "-time=1"], check=True, cwd=d, stdout=subprocess.DEVNULL)
        ent = [line.split() for line in open(dst) if line.strip()]
    rr = np.array([int(e[0]) - 1 for e in ent], np.int64)
    cc = np.array([int(e[1]) - 1 for e in ent], np.int32)
    vv = np.array([float(e[2]) for e in ent])
    o = np.lexsort((cc, rr))
    rr, cc, vv = rr[o], cc[o], vv[o]
    rows, cols, colptr, rowidx, cvals = tg.read_csc(src_rb)
    pos = np.searchsorted(rr, np.arange(rows + 1), side="left").astype(np.int32)
    save("read_rua32_rb", pos=pos, crd=cc, vals=vv, colptr=colptr, rowidx=rowidx, cvals=cvals,
         dims=np.array([rows, cols]))
    out = os.path.join(OUT, "read_rua32.rb")
    _write_rb(out, rows, cols, colptr, rowidx, cvals)
    again = tg.read_csc(out)
    assert again[:2] == (rows, cols)
    for a, b in zip(again[2:], (colptr, rowidx, cvals)):
        assert np.array_equal(a, b)
    # CSR of the CSC read equals taco's CSR of the .mtx twin
    cr = np.repeat(np.arange(cols, dtype=np.int32), np.diff(colptr))
    o = np.lexsort((cr, rowidx))
    assert np.array_equal(rowidx[o], rr) and np.array_equal(cr[o], cc) and np.array_equal(cvals[o], vv)
    rng = np.random.default_rng(41)
    r, c = 23, 17
    dense = np.where(rng.random((r, c)) < 0.3, rng.integers(-40, 41, (r, c)) / 4.0, 0.0)
    cp = np.concatenate([[0], np.cumsum((dense != 0).sum(axis=0))]).astype(np.int32)
    ri = np.concatenate([np.flatnonzero(dense[:, j]) for j in range(c)]).astype(np.int32)
    cv = np.concatenate([dense[np.flatnonzero(dense[:, j]), j] for j in range(c)])
    _write_rb(os.path.join(OUT, "read_rhs.rb"), r, c, cp, ri, cv,
              rhs_line="F%13s%14d%14d" % ("", 1, 0))
    save("read_rhs_rb", colptr=cp, rowidx=ri, cvals=cv, dims=np.array([r, c]))


def dropin_cases(reference_root):
    """taco's own API into the library: tests/cpp/taco_dropin.cpp builds taco::Tensor<double>
    statements for SpMV, SpMM and SpGEMM with taco's library (compiled from the taco sources by
    oracle/Makefile.ref), gives each the forwarding source of INTEGRATION.md through
    TensorBase::compileSource, and runs assemble() and compute().  Without a GPU here the
    forwarding source is linked against the recorder (tests/cpp/tacogb_recorder.c), which keeps
    every argument pack taco passes and completes the call with taco's generated code; the
    driver checks the result equals taco's own.  The fixtures hold the packs of the assemble
    and compute calls and taco's result; tests/test_taco_dropin_gpu.py replays them into the
    drop-in modules on a GPU."""
    import subprocess
    import tempfile
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", "-j8", "REF=" + reference_root,
                    "dropin"], cwd=ROOT, check=True)
    with tempfile.TemporaryDirectory() as d:
        env = dict(os.environ, TACOGB_RECORD_DIR=d, TACOGB_REF_DIR=ref_dir,
                   TACO_CFLAGS="-O3 -std=c99 -I%s -Wl,--no-as-needed -L%s -ltacogb_recorder "
                               "-Wl,-rpath,%s" % (os.path.join(ROOT, "include"), ref_dir, ref_dir))
        subprocess.run([os.path.join(ref_dir, "bin", "taco_dropin"), d], env=env, check=True)
        for p in ("spmv", "spmm", "spgemm"):
            arrays = {}
            (a_call,) = H.read_abi_record(os.path.join(d, p + "_assemble.bin"))
            (c_call,) = H.read_abi_record(os.path.join(d, p + "_compute.bin"))
            for k, t in enumerate(a_call):
                arrays.update(H.record_to_arrays("a%d" % k, t))
            for k, t in enumerate(c_call):
                arrays.update(H.record_to_arrays("c%d" % k, t))
            levels, vals = H.read_result_dump(os.path.join(d, p + "_expected.bin"))
            for m, lv in enumerate(levels):
                if lv is not None:
                    arrays["e_pos%d" % m], arrays["e_crd%d" % m] = lv
            arrays["e_vals"] = vals
            save("taco_dropin_" + p, **arrays)


if __name__ == "__main__":
    ref_root = os.environ.get("TACO_REFERENCE")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src")):
        sys.exit("set TACO_REFERENCE to taco's source tree")
    B.build()
    O.build(ref_root)
    assert O.ref_available("spmv"), "taco's generated code is not built (oracle/Makefile.ref)"
    spmv_cases()
    assert O.ref_available("spmm")
    spmm_cases()
    assert O.ref_available("spgemm")
    spgemm_cases()
    assert O.ref_available("sddmm")
    sddmm_cases()
    assert O.ref_available("ttv") and O.ref_available("ttm") and O.ref_available("mttkrp")
    tensor3_cases()
    assert O.ref_available("spmv_dcsr") and O.ref_available("spmm_dcsr")
    format_cases()
    pack_cases()
    reader_cases()
    rb_cases(ref_root)
    dropin_cases(ref_root)
