"""Benchmark of taco_gb300's sparse hot path on one GB300 (or N replicas under torchrun).

Default workload (the headline): FP64 CSR SpMV y(i) = A(i,j) * x(j) on the 4,194,304 x
4,194,304 power-law matrix (Zipf(2) row lengths scaled to mean 24, clipped to [1, 20000];
~1.0e8 nnz; columns uniform, sorted; values U(-1,1)).  One step = one SpMV over the matrix.
`--workload spmm_powerlaw --n 64|256 --dtype f64|f32|bf16` measures SpMM C = A B on the
1,048,576^2 power-law matrix (mean 32, max 10,000) with a dense row-major B.

  value  algorithmic GB/s of the device path (inputs resident in HBM):
           SpMV  B = nnz*(4+s_v) + 4*(rows+1) + s_x*cols (x once) + s_y*rows (y)
           SpMM  B = nnz*(4+s_a) + 4*(rows+1) + s_b*cols*N (B once) + s_c*rows*N (C)
         (SpMM also reports the gather model, B read once per nonzero, and GFLOP/s)
  e2e    the same metric through taco's kernel ABI (tacogb_<op>_compute on taco_tensor_t with
         pinned host arrays): every step copies the operands to the GPU and the result back
  roofline  the dominant kernel's algorithmic bytes / its mean event-timed duration, against
         the measured HBM copy bandwidth
  cpu_baseline  taco's own generated C for the statement (oracle/_ref, compiled with taco's JIT
         flags, OpenMP over all host cores), or the C restatement when that is absent

`--impl reference` times taco's generated CPU code alone (rank 0) and prints its line.
Every working set but the 65,536-row SpMV's (labelled L2-resident) is larger than L2 (129 MB):
no flush between steps.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

# OpenMP placement for the reference arm, a process that runs taco's generated CPU code alone
# (OpenMP over all host cores): set before anything loads the OpenMP runtime, which reads it
# once; the schedule is set to static per call, as taco's module does.  A value already in the
# environment wins.  The GPU arm's process stays unbound: binding pins its main thread to one
# core, and every thread it starts afterwards (the CUDA driver's, the library's page mapping)
# inherits that core.
if "--impl=reference" in sys.argv or any(
        a == "--impl" and b == "reference" for a, b in zip(sys.argv, sys.argv[1:])):
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
PROFILE_EVERY = 8  # timed steps per step whose kernels are bracketed by CUDA events
L2_BYTES = 129e6  # GB300's L2
ESZ = {"f64": 8, "f32": 4, "bf16": 2}


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="spmv_powerlaw",
                   choices=["spmv_powerlaw", "spmv_banded", "spmv_small", "spmm_powerlaw",
                            "spgemm_random", "spgemm_poisson", "batched_spmv", "batched_spmm",
                            "gather_probe", "pack_powerlaw", "sddmm_powerlaw", "mttkrp_nell2", "ttv_nell2",
                            "ttm_nell2"])
    p.add_argument("--batch-count", type=int, default=4096, help="matrices of batched_spmv")
    p.add_argument("--select", default="default", choices=["default", "exhaustive", "learned"],
                   help="how batched_spmv picks each matrix's work-unit kind")
    p.add_argument("--dtype", default="f64", choices=["f64", "f32", "bf16"])
    p.add_argument("--n", type=int, default=None,
                   help="dense columns of B for SpMM (default 64; 32 for batched_spmm)")
    p.add_argument("--variant", type=int, default=-1)
    p.add_argument("--e2e-steps", type=int, default=30)
    p.add_argument("--pack-n", type=int, default=0,
                   help="pack_powerlaw: pack only the first N shuffled records (0 = all)")
    p.add_argument("--rows", type=int, default=0,
                   help="sddmm_powerlaw: rows (and columns) of B (0 = 1,048,576); mttkrp_nell2: "
                        "B's first dimension (0 = 12,092)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-secondary", action="store_true",
                   help="skip the secondary workloads the default run reports beside the headline")
    p.add_argument("--graph", action="store_true",
                   help="capture the K timed steps in one CUDA graph and time its replay (for "
                        "launch-bound workloads; per-kernel times come from an untimed pass)")
    a = p.parse_args(argv)
    if a.n is None:
        a.n = 32 if a.workload == "batched_spmm" else 64
    if a.workload.startswith("spmv") and a.dtype == "bf16":
        p.error("bf16 applies to SpMM's dense operand only")
    return a


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def max_over_ranks(torch, value, world):
    """The largest of every rank's value (a job's time is its slowest replica's); the value
    itself on one rank.  Works on the job's process group, NCCL on GPUs or gloo on CPUs."""
    if world <= 1:
        return value
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, steps, world, seconds):
    """Whole-job throughput of `world` replicas that each process units_per_step per step."""
    return units_per_step * steps * world / seconds


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` on `workload` from the committed ncu summaries."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.split()
        if len(f) >= 3 and not line.startswith("#") and f[0] == kernel and f[1] == workload:
            return float(f[2])
    return None


# ----------------------------------------------------------------------------- workloads

class SpmvOp:
    pattern = "spmv"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        self.spec = {"spmv_powerlaw": W.spmv_powerlaw, "spmv_banded": W.spmv_banded,
                     "spmv_small": W.spmv_small}[args.workload]()
        s = self.spec
        self.pos, self.crd, self.vals = W.generate(s)
        self.x = W.dense(23, s.cols)
        self.rows, self.cols, self.nnz = s.rows, s.cols, len(self.crd)
        e = ESZ[args.dtype]
        self.bytes = self.nnz * (4 + e) + 4 * (self.rows + 1) + e * self.cols + e * self.rows
        self.flops = 2 * self.nnz
        self.metric = "spmv_%s_hbm_gbs" % args.dtype
        self.workload = "%s_%d" % (args.workload, self.rows)

    def device(self, torch, tg):
        dt = torch.float64 if self.args.dtype == "f64" else torch.float32
        A = tg.CsrMatrix.from_numpy(self.pos, self.crd, self.vals, self.cols, dtype=dt)
        xd = torch.from_numpy(self.x).to("cuda", dt)
        yd = torch.empty(self.rows, dtype=dt, device="cuda")
        csr = A.as_csr()
        L, v = tg.lib(), self.args.variant
        keep = (A, xd, yd, csr)

        def step(sp):
            rc = L.tacogb_spmv(ctypes.byref(csr), xd.data_ptr(), yd.data_ptr(), v, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
        return step, keep

    def abi(self, torch, tg, T):
        dt = torch.float64 if self.args.dtype == "f64" else torch.float32
        e = ESZ[self.args.dtype]
        hp, hc = torch.from_numpy(self.pos).pin_memory(), torch.from_numpy(self.crd).pin_memory()
        hv = torch.from_numpy(self.vals).to(dt).pin_memory()
        hx = torch.from_numpy(self.x).to(dt).pin_memory()
        hy = torch.empty(self.rows, dtype=dt).pin_memory()
        At = T.csr(hp, hc, hv, [self.rows, self.cols])
        Xt, Yt = T.dense(hx, [self.cols]), T.dense(hy, [self.rows])
        L = tg.lib()
        keep = (hp, hc, hv, hx, hy, At, Xt, Yt)

        def step():
            tg.check(L.tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr), "tacogb_spmv_compute")
        h2d = (self.rows + 1) * 4 + self.nnz * (4 + e) + self.cols * e
        return step, keep, h2d, self.rows * e, "tacogb_spmv_compute(taco_tensor_t*) on pinned host arrays"

    def cpu(self):
        """(kind, one-step callable, keep-alive) for taco's generated code or the port."""
        from oracle import oracle as O
        from taco_gb300 import taco as T
        y = np.empty(self.rows)
        if O.ref_available("spmv"):
            L = O.ref_lib("spmv")
            At = T.csr(self.pos, self.crd, self.vals, [self.rows, self.cols])
            Xt, Yt = T.dense(self.x, [self.cols]), T.dense(y, [self.rows])
            return "reference", lambda: L.compute(Yt.ptr, At.ptr, Xt.ptr), (At, Xt, Yt, y)
        lib = O.lib()
        p, c, v, x = self.pos, self.crd, self.vals, self.x
        return "port", lambda: lib.oracle_spmv_f64(self.rows, p.ctypes.data, c.ctypes.data,
                                                   v.ctypes.data, x.ctypes.data, y.ctypes.data), y


class SpmmOp:
    pattern = "spmm"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        s = self.spec = W.spmm_powerlaw()
        self.pos, self.crd, self.vals = W.generate(s)
        self.N = args.n
        self.B = W.dense(29, s.cols * self.N).reshape(s.cols, self.N)
        self.rows, self.cols, self.nnz = s.rows, s.cols, len(self.crd)
        sa = 8 if args.dtype == "f64" else 4
        sb = ESZ[args.dtype]
        sc = 8 if args.dtype == "f64" else 4
        self.bytes = (self.nnz * (4 + sa) + 4 * (self.rows + 1) + sb * self.cols * self.N
                      + sc * self.rows * self.N)
        self.gather_bytes = (self.nnz * (4 + sa) + 4 * (self.rows + 1) + sb * self.nnz * self.N
                             + sc * self.rows * self.N)
        self.flops = 2 * self.nnz * self.N
        self.metric = "spmm_%s_n%d_hbm_gbs" % (args.dtype, self.N)
        self.workload = "%s_%d_n%d" % (args.workload, self.rows, self.N)

    def _types(self, torch):
        a = torch.float64 if self.args.dtype == "f64" else torch.float32
        b = {"f64": torch.float64, "f32": torch.float32, "bf16": torch.bfloat16}[self.args.dtype]
        return a, b

    def device(self, torch, tg):
        at, bt = self._types(torch)
        A = tg.CsrMatrix.from_numpy(self.pos, self.crd, self.vals, self.cols, dtype=at)
        Bd = torch.from_numpy(self.B).to("cuda", bt)
        Cd = torch.empty(self.rows, self.N, dtype=at, device="cuda")
        csr = A.as_csr()
        L, v = tg.lib(), self.args.variant
        btype = {"f64": 0, "f32": 1, "bf16": 2}[self.args.dtype]
        keep = (A, Bd, Cd, csr)

        def step(sp):
            rc = L.tacogb_spmm(ctypes.byref(csr), self.N, Bd.data_ptr(), btype, Cd.data_ptr(), v, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
        return step, keep

    def abi(self, torch, tg, T):
        at, bt = self._types(torch)
        hp, hc = torch.from_numpy(self.pos).pin_memory(), torch.from_numpy(self.crd).pin_memory()
        hv = torch.from_numpy(self.vals).to(at).pin_memory()
        hb = torch.from_numpy(self.B).to(bt).pin_memory()
        hcm = torch.empty(self.rows, self.N, dtype=at).pin_memory()
        At = T.csr(hp, hc, hv, [self.rows, self.cols])
        Bt, Ct = T.dense(hb, [self.cols, self.N]), T.dense(hcm, [self.rows, self.N])
        L = tg.lib()
        keep = (hp, hc, hv, hb, hcm, At, Bt, Ct)

        def step():
            tg.check(L.tacogb_spmm_compute(Ct.ptr, At.ptr, Bt.ptr), "tacogb_spmm_compute")
        sa, sb = (8 if self.args.dtype == "f64" else 4), ESZ[self.args.dtype]
        h2d = (self.rows + 1) * 4 + self.nnz * (4 + sa) + self.cols * self.N * sb
        return step, keep, h2d, self.rows * self.N * sa, "tacogb_spmm_compute(taco_tensor_t*) on pinned host arrays"

    def cpu(self):
        from oracle import oracle as O
        from taco_gb300 import taco as T
        C = np.empty((self.rows, self.N))
        if O.ref_available("spmm"):
            L = O.ref_lib("spmm")
            At = T.csr(self.pos, self.crd, self.vals, [self.rows, self.cols])
            Bt, Ct = T.dense(self.B, [self.cols, self.N]), T.dense(C, [self.rows, self.N])
            return "reference", lambda: L.compute(Ct.ptr, At.ptr, Bt.ptr), (At, Bt, Ct, C)
        lib = O.lib()
        p, c, v, B = self.pos, self.crd, self.vals, self.B
        return "port", lambda: lib.oracle_spmm_f64(self.rows, self.N, p.ctypes.data, c.ctypes.data,
                                                   v.ctypes.data, B.ctypes.data, C.ctypes.data), C


class BatchOp:
    """4,096 CSR matrices from the batch generator (rows log-uniform in [256, 262,144], square,
    mean nnz/row in {2,...,64}, uniform / power-law / banded by index mod 3), y_m = A_m x_m for
    all m per step.  Metric: GFLOP/s = sum_m 2*nnz_m per step."""
    pattern = "batch"
    unit = "GFLOP/s"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        self.count = args.batch_count
        self.specs = [W.batch_spec(m) for m in range(self.count)]
        self.rows = sum(s.rows for s in self.specs)
        self.cols = self.rows
        self.nnz = 0
        self.metric = "batched_spmv_%s_gflops" % ("f32c" if args.dtype == "f32" else "f64")
        self.workload = "batched_spmv_%d" % self.count

    def upload(self, torch):
        """Generates every matrix on the host and keeps it on the GPU: int32 pos/crd, FP64 and
        FP32 values; x and y of all matrices are views into four flat buffers."""
        from taco_gb300 import workloads as W
        dev = {"pos": [], "crd": [], "v64": [], "v32": []}
        nnz = []
        for s in self.specs:
            pos, crd, vals = W.generate(s)
            dev["pos"].append(torch.from_numpy(pos).cuda())
            dev["crd"].append(torch.from_numpy(crd).cuda())
            v = torch.from_numpy(vals).cuda()
            dev["v64"].append(v)
            dev["v32"].append(v.float())
            nnz.append(len(crd))
        self.nnz = int(sum(nnz))
        self.nnz_m = nnz
        off = np.concatenate([[0], np.cumsum([s.rows for s in self.specs])])
        self.off = off
        x64 = torch.from_numpy(W.dense(41, int(off[-1]))).cuda()
        dev["x64"], dev["x32"] = x64, x64.float()
        dev["y64"] = torch.empty_like(x64)
        dev["y32"] = torch.empty_like(dev["x32"])
        e = ESZ["f32" if self.args.dtype == "f32" else "f64"]
        self.bytes = self.nnz * (4 + e) + sum(4 * (s.rows + 1) + 2 * e * s.rows
                                              for s in self.specs)
        self.flops = 2 * self.nnz
        return dev

    def matrices(self, tg, dev, vals_key):
        mats, xs, ys = [], [], []
        xk, yk = ("x32", "y32") if vals_key == "v32" else ("x64", "y64")
        for m, s in enumerate(self.specs):
            mats.append(tg.CsrMatrix(dev["pos"][m], dev["crd"][m], dev[vals_key][m], s.cols))
            a, b = int(self.off[m]), int(self.off[m + 1])
            xs.append(dev[xk][a:b])
            ys.append(dev[yk][a:b])
        return mats, xs, ys

    def cpu(self):
        """taco's generated SpMV called once per matrix (each call OpenMP-parallel over rows) on
        the first matrices of the batch up to about 4e8 nonzeros."""
        from oracle import oracle as O
        from taco_gb300 import taco as T
        from taco_gb300 import workloads as W
        keep, calls, nnz, rows = [], [], 0, 0
        ref = O.ref_available("spmv")
        L = O.ref_lib("spmv") if ref else O.lib()
        for m, s in enumerate(self.specs):
            if nnz > 4e8:
                break
            pos, crd, vals = W.generate(s)
            x, y = W.dense(41 + m, s.cols), np.empty(s.rows)
            if ref:
                At = T.csr(pos, crd, vals, [s.rows, s.cols])
                Xt, Yt = T.dense(x, [s.cols]), T.dense(y, [s.rows])
                keep.append((At, Xt, Yt, pos, crd, vals, x, y))
                calls.append(lambda At=At, Xt=Xt, Yt=Yt: L.compute(Yt.ptr, At.ptr, Xt.ptr))
            else:
                keep.append((pos, crd, vals, x, y))
                calls.append(lambda s=s, pos=pos, crd=crd, vals=vals, x=x, y=y: L.oracle_spmv_f64(
                    s.rows, pos.ctypes.data, crd.ctypes.data, vals.ctypes.data, x.ctypes.data,
                    y.ctypes.data))
            nnz += len(crd)
            rows += s.rows
        self.cpu_units = 2 * nnz
        self.cpu_sample = "first %d of %d matrices (%d rows, %d nnz), FP64" % (
            len(calls), self.count, rows, nnz)

        def once():
            for c in calls:
                c()
        return ("reference" if ref else "port"), once, keep


class BatchSpmmOp(BatchOp):
    """The batched_spmv matrices with a dense B_m (cols x N, row-major, U(-1,1)) per matrix:
    C_m = A_m B_m for all m per step.  Metric: GFLOP/s = sum_m 2*N*nnz_m per step."""

    def __init__(self, args):
        super().__init__(args)
        self.N = args.n
        self.metric = "batched_spmm_n%d_%s_gflops" % (self.N, args.dtype if args.dtype != "f32"
                                                          else "f32c")
        self.workload = "batched_spmm_%d_n%d" % (self.count, self.N)

    def upload(self, torch):
        dev = super().upload(torch)
        N, total = self.N, int(self.off[-1])
        g = torch.Generator(device="cuda")
        g.manual_seed(43)
        dev["B64"] = torch.rand(total, N, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        dev["Bl"] = dev["B64"].to(torch.bfloat16 if self.args.dtype == "bf16" else torch.float32)
        dev["C64"] = torch.empty(total, N, dtype=torch.float64, device="cuda")
        dev["Cl"] = torch.empty(total, N, dtype=torch.float32, device="cuda")
        sa = 8 if self.args.dtype == "f64" else 4
        sb = ESZ[self.args.dtype]
        self.bytes = self.nnz * (4 + sa) + sum(4 * (s.rows + 1) + (sb + sa) * N * s.rows
                                               for s in self.specs)
        self.flops = 2 * N * self.nnz
        return dev

    def operands(self, tg, dev, low):
        vk, bk, ck = ("v32", "Bl", "Cl") if low else ("v64", "B64", "C64")
        mats, Bs, Cs = [], [], []
        for m, s in enumerate(self.specs):
            mats.append(tg.CsrMatrix(dev["pos"][m], dev["crd"][m], dev[vk][m], s.cols))
            a, b = int(self.off[m]), int(self.off[m + 1])
            Bs.append(dev[bk][a:b])
            Cs.append(dev[ck][a:b])
        return mats, Bs, Cs

    def cpu(self):
        """taco's generated SpMM called once per matrix on the first matrices of the batch up to
        about 5e7 nonzeros (N = 32 dense columns)."""
        from oracle import oracle as O
        from taco_gb300 import taco as T
        from taco_gb300 import workloads as W
        keep, calls, nnz, rows, N = [], [], 0, 0, self.N
        ref = O.ref_available("spmm")
        L = O.ref_lib("spmm") if ref else O.lib()
        for m, s in enumerate(self.specs):
            if nnz > 5e7:
                break
            pos, crd, vals = W.generate(s)
            B = W.dense(41 + m, s.cols * N).reshape(s.cols, N)
            C = np.empty((s.rows, N))
            if ref:
                At = T.csr(pos, crd, vals, [s.rows, s.cols])
                Bt, Ct = T.dense(B, [s.cols, N]), T.dense(C, [s.rows, N])
                keep.append((At, Bt, Ct, pos, crd, vals, B, C))
                calls.append(lambda At=At, Bt=Bt, Ct=Ct: L.compute(Ct.ptr, At.ptr, Bt.ptr))
            else:
                keep.append((pos, crd, vals, B, C))
                calls.append(lambda s=s, pos=pos, crd=crd, vals=vals, B=B, C=C: L.oracle_spmm_f64(
                    s.rows, N, pos.ctypes.data, crd.ctypes.data, vals.ctypes.data, B.ctypes.data,
                    C.ctypes.data))
            nnz += len(crd)
            rows += s.rows
        self.cpu_units = 2 * N * nnz
        self.cpu_sample = "first %d of %d matrices (%d rows, %d nnz, N=%d), FP64" % (
            len(calls), self.count, rows, nnz, N)

        def once():
            for c in calls:
                c()
        return ("reference" if ref else "port"), once, keep


class SpgemmOp:
    """C = A A with every structural product kept, columns sorted per row.  One step = the
    one-pass product (pos and nnz(C) read back, then columns and values moved into C's arrays,
    allocated once for the known nnz(C)); --variant 1 runs the three phases (symbolic, column
    fill, numeric) instead."""
    pattern = "spgemm"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        s = self.spec = W.spgemm_random() if args.workload == "spgemm_random" else W.spgemm_poisson()
        self.pos, self.crd, self.vals = W.generate(s)
        self.phase_s = {}
        self.rows, self.cols, self.nnz = s.rows, s.cols, len(self.crd)
        lens = np.diff(self.pos).astype(np.int64)
        self.products = int(lens[self.crd].sum())  # sum over A's nonzeros of B's row lengths
        self.metric = "spgemm_f64_gbs"
        self.workload = "%s_%d" % (args.workload, self.rows)
        self.nnzC = None

    def set_nnzC(self, nnzC):
        n, a = self.rows, self.nnz
        self.nnzC = nnzC
        self.sym_bytes = 4 * (n + 1) * 2 + 4 * a + 4 * (n + 1) + 4 * a
        self.num_bytes = 4 * (n + 1) * 2 + 12 * a + 4 * (n + 1) + 12 * a + 12 * nnzC
        self.bytes = self.sym_bytes + self.num_bytes
        self.flops = 2 * self.products

    def device(self, torch, tg):
        A = tg.CsrMatrix.from_numpy(self.pos, self.crd, self.vals, self.cols)
        a = A.as_csr()
        L = tg.lib()
        pos = torch.empty(self.rows + 1, dtype=torch.int32, device="cuda")
        nnz = ctypes.c_int64(0)
        sp0 = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        tg.check(L.tacogb_spgemm_symbolic(ctypes.byref(a), ctypes.byref(a), pos.data_ptr(),
                                          ctypes.byref(nnz), sp0), "symbolic")
        self.set_nnzC(nnz.value)
        crd = torch.empty(max(nnz.value, 1), dtype=torch.int32, device="cuda")
        vals = torch.empty(max(nnz.value, 1), dtype=torch.float64, device="cuda")
        keep = (A, a, pos, crd, vals, nnz)

        def phases(sp):
            tg.check(L.tacogb_spgemm_symbolic(ctypes.byref(a), ctypes.byref(a), pos.data_ptr(),
                                              ctypes.byref(nnz), sp), "symbolic")
            tg.check(L.tacogb_spgemm_fill(ctypes.byref(a), ctypes.byref(a), pos.data_ptr(),
                                          crd.data_ptr(), sp), "fill")
            tg.check(L.tacogb_spgemm_numeric(ctypes.byref(a), ctypes.byref(a), pos.data_ptr(),
                                             crd.data_ptr(), vals.data_ptr(), sp), "numeric")

        def onepass(sp):
            tg.check(L.tacogb_spgemm_onepass(ctypes.byref(a), ctypes.byref(a), pos.data_ptr(),
                                             ctypes.byref(nnz), sp), "onepass")
            tg.check(L.tacogb_spgemm_onepass_finish(pos.data_ptr(), crd.data_ptr(),
                                                    vals.data_ptr(), sp), "onepass_finish")
        # --variant 1: the three phases (symbolic, fill, numeric); default: one pass
        return (phases if self.args.variant == 1 else onepass), keep

    def abi(self, torch, tg, T):
        import ctypes.util
        libc = ctypes.CDLL(ctypes.util.find_library("c"))
        libc.free.argtypes = [ctypes.c_void_p]
        hp, hc = torch.from_numpy(self.pos).pin_memory(), torch.from_numpy(self.crd).pin_memory()
        hv = torch.from_numpy(self.vals).pin_memory()
        At = T.csr(hp, hc, hv, [self.rows, self.cols])
        L = tg.lib()
        keep = (hp, hc, hv, At)

        def step():
            Ct = T.csr_result([self.rows, self.cols])
            tg.check(L.tacogb_spgemm_evaluate(Ct.ptr, At.ptr, At.ptr), "tacogb_spgemm_evaluate")
            for q in (Ct.index(1, 0), Ct.index(1, 1), Ct.vals_ptr):
                libc.free(q)
        h2d = 2 * ((self.rows + 1) * 4 + self.nnz * 12)
        d2h = (self.rows + 1) * 4 + self.nnzC * 12
        return step, keep, h2d, d2h, "tacogb_spgemm_evaluate(taco_tensor_t*) on pinned host arrays"

    def _taco_step(self, pattern):
        """One assemble + compute of taco's generated code for `pattern` (a callable that
        returns nnz(C) and frees C's arrays); each call's assemble and compute times are
        appended to self.phase_s[pattern]."""
        import ctypes.util
        from oracle import oracle as O
        from taco_gb300 import taco as T
        libc = ctypes.CDLL(ctypes.util.find_library("c"))
        libc.free.argtypes = [ctypes.c_void_p]
        At = T.csr(self.pos, self.crd, self.vals, [self.rows, self.cols])
        L = O.ref_lib(pattern)
        times = self.phase_s.setdefault(pattern, {"assemble": [], "compute": []})

        def once():
            Ct = T.csr_result([self.rows, self.cols])
            t0 = time.perf_counter()
            L.assemble(Ct.ptr, At.ptr, At.ptr)
            t1 = time.perf_counter()
            L.compute(Ct.ptr, At.ptr, At.ptr)
            t2 = time.perf_counter()
            times["assemble"].append(t1 - t0)
            times["compute"].append(t2 - t1)
            nnzC = ctypes.cast(Ct.index(1, 0), ctypes.POINTER(ctypes.c_int32))[self.rows]
            for q in (Ct.index(1, 0), Ct.index(1, 1), Ct.vals_ptr):
                libc.free(q)
            return nnzC
        return once, At

    def phase_ms(self, pattern):
        """Medians (ms) of taco's assemble and compute over the timed calls of `pattern`."""
        t = self.phase_s.get(pattern)
        if not t or not t["assemble"]:
            return {}
        return {"assemble_ms": float(np.median(t["assemble"])) * 1e3,
                "compute_ms": float(np.median(t["compute"])) * 1e3}

    def cpu_serial(self):
        """taco's default (serial) generated SpGEMM, timed beside the scheduled one."""
        from oracle import oracle as O
        if not O.ref_available("spgemm"):
            return None
        once, At = self._taco_step("spgemm")
        return once, At

    def cpu(self):
        import ctypes.util
        from oracle import oracle as O
        from taco_gb300 import taco as T
        libc = ctypes.CDLL(ctypes.util.find_library("c"))
        libc.free.argtypes = [ctypes.c_void_p]
        At = T.csr(self.pos, self.crd, self.vals, [self.rows, self.cols])
        if O.ref_available("spgemm_sched"):
            # taco's parallel two-pass schedule (scheduleSpGEMMCPU) on all host cores
            once, At = self._taco_step("spgemm_sched")
            self.set_nnzC(int(once()))
            self.cpu_sample_desc = ("whole workload, taco's scheduleSpGEMMCPU (parallel two-pass "
                                    "assembly, dense workspace) on all threads")
            self.cpu_phases = "spgemm_sched"
            return "reference", once, (At,)
        if O.ref_available("spgemm"):
            L = O.ref_lib("spgemm")

            def once():
                Ct = T.csr_result([self.rows, self.cols])
                L.assemble(Ct.ptr, At.ptr, At.ptr)
                L.compute(Ct.ptr, At.ptr, At.ptr)
                nnzC = ctypes.cast(Ct.index(1, 0), ctypes.POINTER(ctypes.c_int32))[self.rows]
                for q in (Ct.index(1, 0), Ct.index(1, 1), Ct.vals_ptr):
                    libc.free(q)
                return nnzC
            self.set_nnzC(int(once()))
            return "reference", once, (At,)
        p, c, v = self.pos, self.crd, self.vals
        self.set_nnzC(int(O.spgemm(p, c, None, p, c, None, self.cols)[0][-1]))
        return "port", lambda: O.spgemm(p, c, v, p, c, v, self.cols), (At,)


class PackOp:
    """COO -> CSR pack (taco's TensorBase::pack): the coordinates of the 4,194,304-row power-law
    matrix (1.0e8 entries) in a fixed random order, with their FP64 values, packed into CSR.
    value = algorithmic GB/s: 16 bytes read per coordinate record + 12 written per CSR entry +
    4 per pos entry.  The CPU baseline is the oracle's restatement of taco's pack (one qsort of
    the records, then the merge), single-threaded like taco's, on a 1/16 sample."""
    pattern = "pack"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        s = self.spec = W.spmv_powerlaw()
        pos, crd, vals = W.generate(s)
        self.rows, self.cols, self.nnz = s.rows, s.cols, len(crd)
        rng = np.random.default_rng(77)
        perm = rng.permutation(self.nnz)
        if args.pack_n > 0:  # a smaller case of the same records (profiling captures)
            perm = perm[:args.pack_n]
        self.ri = np.repeat(np.arange(s.rows, dtype=np.int32), np.diff(pos))[perm]
        self.ci = crd[perm]
        self.v = vals[perm]
        self.nnz = len(perm)
        self.bytes = 16 * self.nnz + 12 * self.nnz + 4 * (self.rows + 1)
        self.flops = 0
        self.metric = "pack_f64_gbs"
        self.workload = "pack_powerlaw_%d" % self.rows + (
            "_n%d" % self.nnz if args.pack_n > 0 else "")
        k = self.nnz // 16
        self.cpu_sample = (self.ri[:k], self.ci[:k], self.v[:k])
        self.cpu_bytes = 28 * k + 4 * (self.rows + 1)
        self.cpu_sample_desc = "first 1/16 of the records (%d), packed by the oracle's qsort" % k

    def device(self, torch, tg):
        L = tg.lib()
        ri = torch.from_numpy(self.ri).cuda()
        ci = torch.from_numpy(self.ci).cuda()
        v = torch.from_numpy(self.v).cuda()
        pos = torch.empty(self.rows + 1, dtype=torch.int32, device="cuda")
        crd = torch.empty(self.nnz, dtype=torch.int32, device="cuda")
        out = torch.empty(self.nnz, dtype=torch.float64, device="cuda")
        nnz = ctypes.c_int64(0)
        keep = (ri, ci, v, pos, crd, out, nnz)

        def step(sp):
            tg.check(L.tacogb_pack_csr(self.rows, self.cols, self.nnz, ri.data_ptr(), ci.data_ptr(),
                                       v.data_ptr(), 0, pos.data_ptr(), crd.data_ptr(),
                                       out.data_ptr(), ctypes.byref(nnz), sp), "tacogb_pack_csr")
        return step, keep

    def abi(self, torch, tg, T):
        import ctypes.util
        libc = ctypes.CDLL(ctypes.util.find_library("c"))
        libc.free.argtypes = [ctypes.c_void_p]
        dt = np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")])
        rec = np.empty(self.nnz, dtype=dt)
        rec["r"], rec["c"], rec["v"] = self.ri, self.ci, self.v
        buf = torch.from_numpy(rec.view(np.uint8)).pin_memory()
        L = tg.lib()
        keep = (buf,)

        def step():
            Tt = T.csr_result([self.rows, self.cols])
            tg.check(L.tacogb_pack_taco(Tt.ptr, buf.data_ptr(), self.nnz), "tacogb_pack_taco")
            for q in (Tt.index(1, 0), Tt.index(1, 1), Tt.vals_ptr):
                libc.free(q)
        return (step, keep, 16 * self.nnz, 12 * self.nnz + 4 * (self.rows + 1),
                "tacogb_pack_taco(taco_tensor_t*) on taco's coordinate-buffer layout, pinned host")

    def cpu(self):
        from oracle import oracle as O
        ri, ci, v = self.cpu_sample
        return "port", lambda: O.pack_csr(self.rows, self.cols, ri, ci, v), None


class SddmmOp:
    """SDDMM A(i,k) = B(i,k) * C(i,j) * D(j,k) kept at B's nonzeros: B the 1,048,576-row
    power-law matrix (3.4e7 nonzeros), J = 128 (taco's sddmmGPU width), C and D U(-1,1).
    value = GFLOP/s on 2 J flops per nonzero; the roofline is on the compulsory bytes (B's crd
    and values, pos, C and D once, the result once).  The CPU baseline is the oracle's
    restatement of taco's loop in its sampled form (taco's generated dense-result code would
    need an I x K result of 8.8 TB here) on the first 1/16 of the rows, all host cores."""
    pattern = "sddmm"
    unit = "GFLOP/s"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        s = self.spec = W.sddmm_powerlaw(args.rows) if args.rows > 0 else W.sddmm_powerlaw()
        self.pos, self.crd, self.vals = W.generate(s)
        self.rows, self.cols, self.nnz = s.rows, s.cols, len(self.crd)
        J = self.J = W.SDDMM_J
        self.C = W.dense(61, s.rows * J).reshape(s.rows, J)
        self.D = W.dense(62, J * s.cols).reshape(J, s.cols)
        e = self.esz = 8 if args.dtype == "f64" else 4
        self.bytes = (self.nnz * (4 + 2 * e) + 4 * (self.rows + 1) + e * self.rows * J
                      + e * J * self.cols)
        self.gather_bytes = (self.nnz * (4 + 2 * e) + 4 * (self.rows + 1) + e * self.rows * J
                             + e * self.nnz * J)
        # the columns of B are uniform over 1,048,576, so no order of the nonzeros reuses Dt rows
        # beyond what L2 holds: every nonzero's J-vector of D is algorithmic traffic
        self.roofline_bytes = self.gather_bytes
        self.flops = self.work = 2 * J * self.nnz
        self.metric = "sddmm_%s_j%d_gflops" % (args.dtype, J)
        self.workload = "%s_%d_j%d" % (args.workload, self.rows, J)
        R = self.cpu_rows = self.rows // 16
        self.cpu_work = 2 * J * int(self.pos[R])
        self.cpu_sample_desc = ("first %d rows (%d nonzeros), oracle's sampled restatement of "
                                "taco's loop" % (R, int(self.pos[R])))

    def _dtype(self, torch):
        return torch.float64 if self.args.dtype == "f64" else torch.float32

    def device(self, torch, tg):
        dt = self._dtype(torch)
        B = tg.CsrMatrix.from_numpy(self.pos, self.crd, self.vals, self.cols, dtype=dt)
        Cd = torch.from_numpy(self.C).to("cuda", dt)
        Dd = torch.from_numpy(self.D).to("cuda", dt)
        out = torch.empty(self.nnz, dtype=dt, device="cuda")
        b = B.as_csr()
        L, v = tg.lib(), self.args.variant
        keep = (B, Cd, Dd, out, b)

        def step(sp):
            rc = L.tacogb_sddmm(ctypes.byref(b), self.J, Cd.data_ptr(), Dd.data_ptr(),
                                out.data_ptr(), v, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
        return step, keep

    def abi(self, torch, tg, T):
        dt = self._dtype(torch)
        hp, hc = torch.from_numpy(self.pos).pin_memory(), torch.from_numpy(self.crd).pin_memory()
        hv = torch.from_numpy(self.vals).to(dt).pin_memory()
        hC = torch.from_numpy(self.C).to(dt).pin_memory()
        hD = torch.from_numpy(self.D).to(dt).pin_memory()
        ho = torch.empty(self.nnz, dtype=dt).pin_memory()
        Bt = T.csr(hp, hc, hv, [self.rows, self.cols])
        At = T.csr(hp, hc, ho, [self.rows, self.cols])  # result with B's pattern
        Ct, Dt = T.dense(hC, [self.rows, self.J]), T.dense(hD, [self.J, self.cols])
        L = tg.lib()
        keep = (hp, hc, hv, hC, hD, ho, Bt, At, Ct, Dt)

        def step():
            tg.check(L.tacogb_sddmm_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr),
                     "tacogb_sddmm_compute")
        e = self.esz
        h2d = ((self.rows + 1) * 4 + self.nnz * (4 + e) + e * self.rows * self.J
               + e * self.J * self.cols)
        return (step, keep, h2d, self.nnz * e,
                "tacogb_sddmm_compute(taco_tensor_t*) on pinned host arrays, CSR result")

    def cpu(self):
        from oracle import oracle as O
        lib = O.lib()
        R = self.cpu_rows
        out = np.empty(int(self.pos[R]))
        p, c, v, C, D = self.pos, self.crd, self.vals, self.C, self.D
        return "port", lambda: lib.oracle_sddmm_sampled_f64(
            R, self.cols, self.J, p.ctypes.data, c.ctypes.data, v.ctypes.data, C.ctypes.data,
            D.ctypes.data, out.ctypes.data), out


class MttkrpOp:
    """MTTKRP A(i,j) = B(i,k,l) * C(k,j) * D(l,j), B {Sparse,Sparse,Sparse} with nell-2's shape
    (12,092 x 9,184 x 28,818) and 7.7e7 synthetic nonzeros (power-law fibers), rank J = 32,
    FP64.  value = GFLOP/s on taco's 3 J flops per nonzero.  The roofline is on the fiber
    SpMM's compulsory bytes (B's level-2 arrays, D once, T written), its dominant kernel.  The
    CPU baseline is taco's own generated code for the statement on all host cores (the whole
    tensor; A is only 12,092 x 32)."""
    pattern = "mttkrp"
    unit = "GFLOP/s"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        dims = W.TENSOR3_DIMS if args.rows <= 0 else (args.rows,) + W.TENSOR3_DIMS[1:]
        self.B = W.tensor3_powerlaw(dims=dims)
        dims, crd0, pos1, crd1, pos2, crd2, vals = self.B
        J = self.J = W.MTTKRP_J
        self.C = W.dense(71, dims[1] * J).reshape(dims[1], J)
        self.D = W.dense(72, dims[2] * J).reshape(dims[2], J)
        self.rows, self.cols, self.nnz = dims[0], dims[2], len(crd2)
        self.nfib = len(crd1)
        e = 8 if args.dtype == "f64" else 4
        self.roofline_bytes = (self.nnz * (4 + e) + 4 * (self.nfib + 1) + e * dims[2] * J
                               + e * self.nfib * J)
        self.bytes = (self.roofline_bytes + 4 * (dims[0] + 1) + 4 * self.nfib
                      + e * self.nfib * J + e * dims[1] * J + e * dims[0] * J)
        self.flops = self.work = self.cpu_work = 3 * J * self.nnz
        self.metric = "mttkrp_%s_r%d_gflops" % (args.dtype, J)
        self.workload = "mttkrp_nell2_%d_%d_%d_r%d" % (dims[0], dims[1], dims[2], J)

    def _dtype(self, torch):
        return torch.float64 if self.args.dtype == "f64" else torch.float32

    def device(self, torch, tg):
        dt = self._dtype(torch)
        Bd = tg.CsfTensor.from_numpy(*self.B, dtype=dt)
        Cd = torch.from_numpy(self.C).to("cuda", dt)
        Dd = torch.from_numpy(self.D).to("cuda", dt)
        A = torch.empty(self.rows, self.J, dtype=dt, device="cuda")
        b = Bd.as_csf3()
        L = tg.lib()
        keep = (Bd, Cd, Dd, A, b)

        v = self.args.variant

        def step(sp):
            rc = L.tacogb_mttkrp(ctypes.byref(b), self.J, Cd.data_ptr(), Dd.data_ptr(),
                                 A.data_ptr(), v, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
        return step, keep

    def abi(self, torch, tg, T):
        dt = self._dtype(torch)
        dims, crd0, pos1, crd1, pos2, crd2, vals = self.B
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()  # noqa: E731
        hb = [pin(a) for a in (crd0, pos1, crd1, pos2, crd2)]
        hv = torch.from_numpy(vals).to(dt).pin_memory()
        hC, hD = torch.from_numpy(self.C).to(dt).pin_memory(), torch.from_numpy(self.D).to(dt).pin_memory()
        hA = torch.empty(self.rows, self.J, dtype=dt).pin_memory()
        Bt = T.csf3(dims, *hb, hv)
        Ct, Dt = T.dense(hC, list(self.C.shape)), T.dense(hD, list(self.D.shape))
        At = T.dense(hA, [self.rows, self.J])
        L = tg.lib()
        keep = (hb, hv, hC, hD, hA, Bt, Ct, Dt, At)

        def step():
            tg.check(L.tacogb_mttkrp_compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr),
                     "tacogb_mttkrp_compute")
        e = 8 if self.args.dtype == "f64" else 4
        h2d = (4 * (len(crd0) + len(pos1) + len(crd1) + len(pos2) + len(crd2)) + e * self.nnz
               + e * (self.C.size + self.D.size))
        return (step, keep, h2d, e * self.rows * self.J,
                "tacogb_mttkrp_compute(taco_tensor_t*) on pinned host arrays")

    def cpu(self):
        from oracle import oracle as O
        from taco_gb300 import taco as T
        A = np.empty((self.rows, self.J))
        if O.ref_available("mttkrp"):
            L = O.ref_lib("mttkrp")
            Bt = T.csf3(*self.B)
            Ct, Dt = T.dense(self.C, list(self.C.shape)), T.dense(self.D, list(self.D.shape))
            At = T.dense(A, [self.rows, self.J])
            return ("reference", lambda: L.compute(At.ptr, Bt.ptr, Ct.ptr, Dt.ptr),
                    (Bt, Ct, Dt, At, A))
        return "port", lambda: O.mttkrp(self.B, self.C, self.D), A


class Tensor3Op:
    """TTV (A(i,j) = B(i,j,k) c(k)) or TTM (A(i,j,l) = B(i,j,k) C(k,l), L = 128 as in taco's
    ttmGPU) over the MTTKRP tensor (nell-2's shape, 7.7e7 synthetic nonzeros), FP64, results per
    (i,j) fiber.  value = GFLOP/s on 2 flops per nonzero (TTV) or 2 L (TTM); the roofline is on
    the compulsory bytes (B's level-2 arrays, c or C once, the fiber results written).  CPU
    baseline: TTV by taco's generated code (dense 12,092 x 9,184 result), TTM by the oracle's
    loop with per-fiber results (the dense result would be 113 GB)."""
    unit = "GFLOP/s"

    def __init__(self, args):
        from taco_gb300 import workloads as W
        self.args = args
        self.pattern = args.workload.split("_")[0]
        self.B = W.tensor3_powerlaw()
        dims, crd0, pos1, crd1, pos2, crd2, vals = self.B
        self.rows, self.cols, self.nnz, self.nfib = dims[0], dims[2], len(crd2), len(crd1)
        self.L = 128 if self.pattern == "ttm" else 1
        self.C = W.dense(81, dims[2] * self.L).reshape(dims[2], self.L)
        self.bytes = self.roofline_bytes = (12 * self.nnz + 4 * (self.nfib + 1) + 8 * dims[2] * self.L
                                            + 8 * self.nfib * self.L)
        self.flops = self.work = self.cpu_work = 2 * self.L * self.nnz
        self.metric = "%s_f64_gflops" % self.pattern + ("_l%d" % self.L if self.L > 1 else "")
        self.workload = "%s_nell2_%d_%d_%d" % (self.pattern, *dims)

    def device(self, torch, tg):
        Bd = tg.CsfTensor.from_numpy(*self.B)
        b = Bd.as_csf3()
        Cd = torch.from_numpy(np.ascontiguousarray(self.C if self.L > 1 else self.C[:, 0])).cuda()
        out = torch.empty(self.nfib * self.L, dtype=torch.float64, device="cuda")
        L = tg.lib()
        keep = (Bd, b, Cd, out)
        if self.pattern == "ttv":
            def step(sp):
                tg.check(L.tacogb_ttv(ctypes.byref(b), Cd.data_ptr(), out.data_ptr(),
                                      self.args.variant, sp), "ttv")
        else:
            def step(sp):
                tg.check(L.tacogb_ttm(ctypes.byref(b), self.L, Cd.data_ptr(), out.data_ptr(),
                                      self.args.variant, sp), "ttm")
        return step, keep

    def abi(self, torch, tg, T):
        return None

    def cpu(self):
        from oracle import oracle as O
        from taco_gb300 import taco as T
        dims, crd0, pos1, crd1, pos2, crd2, vals = self.B
        if self.pattern == "ttv" and O.ref_available("ttv"):
            L = O.ref_lib("ttv")
            A = np.empty((dims[0], dims[1]))
            c = np.ascontiguousarray(self.C[:, 0])
            Bt, Ct, At = T.csf3(*self.B), T.dense(c, [dims[2]]), T.dense(A, [dims[0], dims[1]])
            return "reference", lambda: L.compute(At.ptr, Bt.ptr, Ct.ptr), (Bt, Ct, At, A, c)
        out = np.empty(self.nfib * self.L)
        lib = O.lib()
        C = np.ascontiguousarray(self.C)
        return "port", lambda: lib.oracle_ttm_fibers_f64(
            self.L, self.nfib, pos2.ctypes.data, crd2.ctypes.data, vals.ctypes.data,
            C.ctypes.data, out.ctypes.data), (out, C)


def make_op(args):
    if args.workload in ("ttv_nell2", "ttm_nell2"):
        return Tensor3Op(args)
    if args.workload == "mttkrp_nell2":
        return MttkrpOp(args)
    if args.workload == "sddmm_powerlaw":
        return SddmmOp(args)
    if args.workload.startswith("spgemm"):
        return SpgemmOp(args)
    if args.workload == "pack_powerlaw":
        return PackOp(args)
    if args.workload == "batched_spmv":
        return BatchOp(args)
    if args.workload == "batched_spmm":
        return BatchSpmmOp(args)
    return SpmmOp(args) if args.workload.startswith("spmm") else SpmvOp(args)


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.out = index, None, None

    def start(self):
        try:
            self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.flush()
        self.out.seek(0)
        rows = [l.strip().split(", ") for l in self.out.read().splitlines() if l.strip()]
        os.unlink(self.out.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for n, v in zip(names, r[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU legs

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or None."""
    try:
        r = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                           text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def omp_setup():
    return "OMP_PROC_BIND=%s OMP_PLACES=%s, static schedule" % (
        os.environ.get("OMP_PROC_BIND", "unset"), os.environ.get("OMP_PLACES", "unset"))


def time_cpu(op, budget_s=8.0, reps=None):
    """Median seconds of one step of taco's generated code (or the port) on all host cores."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    O.ref_set_threads(ncores)
    O.set_threads(ncores)
    kind, once, keep = op.cpu()
    for _ in range(3):
        once()
    times = []
    t_end = time.perf_counter() + budget_s
    while (reps is None and time.perf_counter() < t_end and len(times) < 200) or \
            (reps is not None and len(times) < reps):
        t0 = time.perf_counter()
        once()
        times.append(time.perf_counter() - t0)
    del keep
    return kind, ncores, float(np.median(times)), len(times)


def workload_config(op, world):
    """The workload as both arms print it: the same dict from the same op, so that a line of
    this implementation and a line of taco's generated code name one configuration.  Results
    and implementation choices (variant, threads, derived rates) go outside it."""
    if op.pattern == "batch":
        c = {"workload": op.workload, "matrices": op.count, "rows": op.rows}
        if getattr(op, "N", None):
            c["n"] = op.N
    else:
        c = {"workload": op.workload, "rows": op.rows, "cols": op.cols, "nnz": op.nnz,
             "bytes_per_step": op.bytes,
             "l2": ("inputs larger than L2 (%.2f GB per step), no flush" % (op.bytes / 1e9)
                    if op.bytes > L2_BYTES else
                    "L2-resident (%.1f MB per step fits the 129 MB L2), no flush"
                    % (op.bytes / 1e6))}
        if op.pattern == "spgemm":
            c.update({"nnz_c": op.nnzC, "products": op.products})
        for key, attr in (("n", "N"), ("j", "J")):
            if getattr(op, attr, None) is not None and op.pattern in ("spmm", "sddmm", "mttkrp",
                                                                       "ttm"):
                c[key] = getattr(op, attr)
    c["parallelism"] = "replicas" if world > 1 else "single"
    return c


def mapped_libraries():
    """Shared objects of this repository mapped into the process (from /proc/self/maps)."""
    out = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1] if len(line.split()) >= 6 else ""
            if path.startswith(ROOT) and ".so" in path:
                out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from taco_gb300 import _native as N
    O.build()
    # the inputs come from the oracle's own build of the generators: this arm maps no library
    # of taco_gb300
    N.set_generator_library(O.generator_library())
    op = make_op(args)
    ncores = os.cpu_count() or 1
    O.ref_set_threads(ncores)
    O.set_threads(ncores)
    kind, once, keep = op.cpu()
    for _ in range(max(3, args.warmup)):
        once()
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        once()
        if time.perf_counter() - t0 > 120.0:  # keep the reference arm within a few minutes
            steps = _ + 1
            break
    dt = time.perf_counter() - t0
    unit = getattr(op, "unit", "GB/s")
    work = (op.cpu_units if op.pattern == "batch"
            else getattr(op, "cpu_work", getattr(op, "cpu_bytes", op.bytes)))
    sample = (op.cpu_sample if op.pattern == "batch"
              else getattr(op, "cpu_sample_desc", "whole workload")) + \
        " per step, %d steps" % steps
    v = work * steps / dt / 1e9
    code = ("taco generated C, -O3 -ffast-math -std=c99 -fopenmp" if kind == "reference"
            else "C restatement of taco's pack: qsort + merge, one thread" if op.pattern == "pack"
            else "C restatement of taco's loop, -O2 -fopenmp")
    out = {"metric": op.metric, "value": v, "unit": unit, "impl": "reference",
           "n_gpus": world, "steps": steps, "warmup": args.warmup,
           "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(op, world),
           "cpu_baseline": {"value": v, "unit": unit, "cores": ncores, "kind": kind,
                            "sample": sample, "code": code, "work_per_step": work,
                            "cpu_model": cpu_model(), "omp": omp_setup()},
           "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if getattr(op, "cpu_phases", None):
        out["cpu_baseline"].update(op.phase_ms(op.cpu_phases))  # assemble, compute separately
    if op.pattern != "batch":
        out["gflops"] = getattr(op, "cpu_work" if op.pattern == "sddmm" else "flops",
                                op.flops) * steps / dt / 1e9
    libs = mapped_libraries()
    product = [l for l in libs if l.startswith("taco_gb300")]
    if product:
        raise RuntimeError("the reference arm mapped this repository's product libraries: %s"
                           % product)
    out["native_libs"] = libs
    print(json.dumps(out), flush=True)
    del keep


# ----------------------------------------------------------------------------- batched

def batch_variants_for(args, op, tg, dev):
    """Per-matrix work-unit kinds: None (merge_ipt7 everywhere) or the autotuner's choice."""
    if args.select == "default":
        return None, "merge_ipt7 for every matrix"
    from taco_gb300 import autotune as AT
    mats, xs, ys = op.matrices(tg, dev, "v32")
    if args.select == "exhaustive":
        kinds, _ = AT.exhaustive_select(mats, xs, ys, precision=0)
        return kinds, "exhaustive autotuner (per-matrix argmin of measured unit cycles)"
    model = AT.load_model(os.path.join(ROOT, "taco_gb300", "data", "batch_mlp.npz"))
    kinds = AT.learned_select(model, mats)
    return kinds, "MLP cost model (argmin of predicted cycles over sparsity features)"


def main_batch(args, torch, tg, T, L, rank, world):
    """Batched SpMV: one graph launch per step over all matrices, against the same matrices
    computed with one plain FP64 tacogb_spmv call per matrix."""
    op = make_op(args)
    dev = op.upload(torch)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    vkey = "v32" if args.dtype == "f32" else "v64"
    kinds, how = batch_variants_for(args, op, tg, dev)
    mats, xs, ys = op.matrices(tg, dev, vkey)
    plan = tg.SpmvBatch(mats, xs, ys, precision=0, variants=kinds)
    for _ in range(max(3, args.warmup)):
        plan.run(stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(0) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.tacogb_launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        plan.run(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = L.tacogb_launch_count() - launches0
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1) / args.steps
    status = ctypes.c_int32(0)
    L.tacogb_device_status(ctypes.byref(status))
    if status.value:
        raise RuntimeError("device status %d after the timed region" % status.value)
    value = op.flops / (ms / 1e3) / 1e9

    # plain FP64: one tacogb_spmv (the library's default FP64 path, DFMA accumulation) per
    # matrix, issued from a host loop
    m64, x64, y64 = op.matrices(tg, dev, "v64")
    csrs = [A.as_csr() for A in m64]
    native = -1

    def per_matrix():
        for c, x, y in zip(csrs, x64, y64):
            rc = L.tacogb_spmv(ctypes.byref(c), x.data_ptr(), y.data_ptr(), native, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
    for _ in range(3):
        per_matrix()
    torch.cuda.synchronize()
    k64 = max(2, min(args.steps, 10))
    e0.record(stream)
    for _ in range(k64):
        per_matrix()
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / k64

    # error of every matrix's result against the FP64 result
    plan.run(stream)
    torch.cuda.synchronize()
    yb = dev["y32" if vkey == "v32" else "y64"].double()
    errs = []
    for m in range(op.count):
        a, b = int(op.off[m]), int(op.off[m + 1])
        ref = dev["y64"][a:b]
        den = float(ref.abs().max()) or 1.0
        d = (yb[a:b] - ref) / den
        nr = float(torch.linalg.vector_norm(ref / den))
        errs.append(float(torch.linalg.vector_norm(d)) / nr if nr > 0 else 0.0)
    max_err = max(errs)
    del yb

    # end to end: all x from pinned host memory, the graph, all y back to pinned host memory
    xk = "x32" if vkey == "v32" else "x64"
    yk = "y32" if vkey == "v32" else "y64"
    hx = dev[xk].cpu().pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    for _ in range(2):
        dev[xk].copy_(hx, non_blocking=True)
        plan.run(stream)
        hy.copy_(dev[yk], non_blocking=True)
    torch.cuda.synchronize()
    ne = max(3, min(args.e2e_steps, 20))
    t0 = time.perf_counter()
    for _ in range(ne):
        dev[xk].copy_(hx, non_blocking=True)
        plan.run(stream)
        hy.copy_(dev[yk], non_blocking=True)
        stream.synchronize()
    e2e_s = (time.perf_counter() - t0) / ne
    nbytes = hx.numel() * hx.element_size()
    e2e = {"value": op.flops / e2e_s / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_s * 1e3, "steps": ne,
           "api": "SpmvBatch.run (tacogb_batch_run) with x/y copied from/to pinned host memory; "
                  "matrices resident"}

    cpu = None
    if not args.no_cpu:
        kind, cores, t, reps = time_cpu(op, budget_s=10.0)
        cpu = {"value": op.cpu_units / t / 1e9, "unit": "GFLOP/s", "cores": cores, "kind": kind,
               "sample": op.cpu_sample + ", median of %d reps" % reps, "ms_per_step": t * 1e3}

    peak, peak_kind = measured_peak()
    achieved = op.bytes / (ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic("batch_spmv_kernel", op.workload),
                "kernel": "batch_spmv_kernel (graph: partition + persistent queue + fix-up)",
                "kernel_ms": ms, "peak_source": peak_kind}
    kinds_used = {}
    for k in (kinds if kinds is not None else [0] * op.count):
        nm = tg.batch_variants()[k]
        kinds_used[nm] = kinds_used.get(nm, 0) + 1
    out = {"metric": op.metric, "value": value, "unit": "GFLOP/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32c" if vkey == "v32" else "f64", "data": "synthetic",
           "config": workload_config(op, world),
           "detail": {"nnz": op.nnz, "bytes_per_step": op.bytes, "selection": how,
                      "kinds": kinds_used,
                      "l2": "inputs larger than L2 (%.1f GB per step), no flush" % (op.bytes / 1e9)},
           "fp64_per_matrix": {"gflops": op.flops / (ms64 / 1e3) / 1e9, "ms_per_step": ms64,
                               "launch": "tacogb_spmv with TACOGB_VARIANT_AUTO (the library's own "
                                         "choice per matrix, DFMA accumulation), one call per "
                                         "matrix from a host loop, after 3 untimed passes",
                               "steps": k64},
           "speedup_vs_fp64_per_matrix": ms64 / ms,
           "max_normwise_err_vs_fp64": max_err,
           "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
           "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(out), flush=True)
    plan.close()


def main_batch_spmm(args, torch, tg, L, rank):
    """Batched SpMM: one graph launch per step over all matrices, against one plain FP64
    tacogb_spmm call per matrix on the same matrices."""
    op = make_op(args)
    dev = op.upload(torch)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    low = args.dtype != "f64"
    mats, Bs, Cs = op.operands(tg, dev, low)
    plan = tg.SpmmBatch(mats, Bs, Cs, precision=0)
    for _ in range(max(3, args.warmup)):
        plan.run(stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(0) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.tacogb_launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        plan.run(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = L.tacogb_launch_count() - launches0
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1) / args.steps
    status = ctypes.c_int32(0)
    L.tacogb_device_status(ctypes.byref(status))
    if status.value:
        raise RuntimeError("device status %d after the timed region" % status.value)

    m64, B64, C64 = op.operands(tg, dev, False)
    csrs = [A.as_csr() for A in m64]
    native = tg.spmm_variants().index("merge_w512_native")

    def per_matrix():
        for c, B, C in zip(csrs, B64, C64):
            rc = L.tacogb_spmm(ctypes.byref(c), op.N, B.data_ptr(), tg.TACOGB_F64, C.data_ptr(),
                               native, sp)
            if rc:
                raise RuntimeError(L.tacogb_last_error().decode())
    for _ in range(2):
        per_matrix()
    torch.cuda.synchronize()
    k64 = max(2, min(args.steps, 5))
    e0.record(stream)
    for _ in range(k64):
        per_matrix()
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / k64

    plan.run(stream)
    torch.cuda.synchronize()
    errs = []
    key = "Cl" if low else "C64"
    for m in range(op.count):
        a, b = int(op.off[m]), int(op.off[m + 1])
        ref = dev["C64"][a:b]
        den = float(ref.abs().max()) if b > a else 0.0
        if den == 0.0:
            continue
        d = (dev[key][a:b].double() - ref) / den
        errs.append(float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref / den)))
    max_err = max(errs) if errs else 0.0

    cpu = None
    if not args.no_cpu:
        kind, cores, t, reps = time_cpu(op, budget_s=10.0)
        cpu = {"value": op.cpu_units / t / 1e9, "unit": "GFLOP/s", "cores": cores, "kind": kind,
               "sample": op.cpu_sample + ", median of %d reps" % reps, "ms_per_step": t * 1e3}
    peak, peak_kind = measured_peak()
    achieved = op.bytes / (ms / 1e3) / 1e9
    out = {"metric": op.metric, "value": op.flops / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": {"f64": "f64", "f32": "f32c", "bf16": "bf16b_f32"}[args.dtype],
           "data": "synthetic",
           "config": workload_config(op, 1),
           "detail": {"nnz": op.nnz, "bytes_per_step": op.bytes,
                      "l2": "inputs larger than L2 (%.1f GB per step), no flush" % (op.bytes / 1e9)},
           "fp64_per_matrix": {"gflops": op.flops / (ms64 / 1e3) / 1e9, "ms_per_step": ms64,
                               "launch": "tacogb_spmm merge_w512_native FP64, one call per "
                                         "matrix from a host loop", "steps": k64},
           "speedup_vs_fp64_per_matrix": ms64 / ms,
           "max_normwise_err_vs_fp64": max_err,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak,
                        "traffic": ncu_traffic("batch_spmm_kernel", op.workload),
                        "kernel": "batch_spmm_kernel (graph: partition + queue + fix-up)",
                        "kernel_ms": ms, "peak_source": peak_kind},
           "cpu_baseline": cpu, "e2e": None, "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(out), flush=True)
    plan.close()


# ----------------------------------------------------------------------------- main

# The workloads the default run measures beside the headline, each in its own process (the
# same bench.py, so the same code paths and timing rules), summarised into the headline line.
SECONDARY = [
    ("spmv_small_f64 (L2-resident: 13.9 MB fits the 129 MB L2; steps replayed as a CUDA graph)",
     ["--workload", "spmv_small", "--steps", "500", "--warmup", "20", "--e2e-steps", "10",
      "--graph"]),
    ("spmv_banded_f64", ["--workload", "spmv_banded", "--steps", "50", "--warmup", "5",
                         "--e2e-steps", "20"]),
    ("spmv_powerlaw_f32c", ["--workload", "spmv_powerlaw", "--dtype", "f32", "--steps", "50",
                            "--warmup", "5", "--e2e-steps", "20"]),
    ("spmm_powerlaw_n64_f64", ["--workload", "spmm_powerlaw", "--n", "64", "--steps", "20",
                               "--warmup", "3", "--e2e-steps", "10"]),
    ("spgemm_random_f64", ["--workload", "spgemm_random", "--steps", "20", "--warmup", "3",
                           "--e2e-steps", "10"]),
    ("batched_spmv_4096_f32c_learned", ["--workload", "batched_spmv", "--dtype", "f32",
                                        "--select", "learned", "--steps", "5", "--warmup", "3"]),
    ("sddmm_powerlaw_j128_f64", ["--workload", "sddmm_powerlaw", "--steps", "10", "--warmup", "3",
                                 "--e2e-steps", "10"]),
    ("mttkrp_nell2_r32_f64", ["--workload", "mttkrp_nell2", "--steps", "20", "--warmup", "3",
                              "--e2e-steps", "10"]),
]


def run_secondary():
    keys = ("metric", "value", "unit", "ms_per_step", "dtype", "gpu_launches", "clocks",
            "speedup_vs_fp64_per_matrix", "max_normwise_err_vs_fp64", "derived", "variant",
            "timing")
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT")}
    out = []
    for name, argv in SECONDARY:
        t0 = time.perf_counter()
        try:
            r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--no-secondary"]
                               + argv, cwd=ROOT, env=env, stdout=subprocess.PIPE,
                               stderr=subprocess.PIPE, text=True, timeout=400)
            line = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not line:
                out.append({"workload": name, "error": (r.stderr or r.stdout)[-300:]})
                continue
            d = json.loads(line[-1])
        except subprocess.TimeoutExpired:
            out.append({"workload": name, "error": "timed out"})
            continue
        e = {"workload": name, "config": d.get("config")}
        e.update({k: d[k] for k in keys if k in d})
        rf = d.get("roofline") or {}
        e["roofline"] = {k: rf.get(k) for k in ("bound", "achieved", "peak", "unit", "frac",
                                                 "traffic", "kernel", "kernel_ms")}
        e["cpu_baseline"] = d.get("cpu_baseline")
        e["e2e"] = d.get("e2e")
        e["wall_s"] = time.perf_counter() - t0
        out.append(e)
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    from taco_gb300 import build as Bd
    Bd.build()
    import taco_gb300 as tg
    from taco_gb300 import taco as T
    L = tg.lib()

    if args.workload == "gather_probe":
        if rank == 0:
            main_gather_probe(args, torch, tg, L)
        return
    if args.workload == "batched_spmv":
        main_batch(args, torch, tg, T, L, rank, world)
        return
    if args.workload == "batched_spmm":
        main_batch_spmm(args, torch, tg, L, rank)
        return
    op = make_op(args)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    step, keep = op.device(torch, tg)
    for _ in range(max(3, args.warmup)):
        step(sp)
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    names = ctypes.create_string_buffer(64 * 16)
    tot, cnt = (ctypes.c_double * 16)(), (ctypes.c_int32 * 16)()
    if args.graph:
        # the per-kernel pass, untimed: every PROFILE_EVERY-th step bracketed by events
        L.tacogb_profile_begin()
        for i in range(args.steps):
            L.tacogb_profile_enable(1 if i % PROFILE_EVERY == 0 else 0)
            step(sp)
        torch.cuda.synchronize()
        nk = L.tacogb_profile_end(16, names, tot, cnt)
        # the K steps captured once (the library's launches are counted at capture) and replayed
        cs = torch.cuda.Stream()
        csp = ctypes.c_void_p(cs.cuda_stream)
        cs.wait_stream(stream)
        with torch.cuda.stream(cs):
            step(csp)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        launches0 = L.tacogb_launch_count()
        with torch.cuda.graph(graph, stream=cs):
            for _ in range(args.steps):
                step(csp)
        launches = L.tacogb_launch_count() - launches0
        graph.replay()
        torch.cuda.synchronize()
        e0.record(stream)
        graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
    else:
        launches0 = L.tacogb_launch_count()
        # per-kernel device times: CUDA events bracket the launches of every PROFILE_EVERY-th
        # step of the timed region only, so that event records stay out of the headline time
        L.tacogb_profile_begin()
        e0.record(stream)
        for i in range(args.steps):
            L.tacogb_profile_enable(1 if i % PROFILE_EVERY == 0 else 0)
            step(sp)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = L.tacogb_launch_count() - launches0
        nk = L.tacogb_profile_end(16, names, tot, cnt)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    status = ctypes.c_int32(0)
    L.tacogb_device_status(ctypes.byref(status))
    if status.value:
        raise RuntimeError("device status %d after the timed region" % status.value)
    ms = max_over_ranks(torch, e0.elapsed_time(e1), world)
    unit = getattr(op, "unit", "GB/s")
    work = getattr(op, "work", op.bytes)  # units of the metric per step (bytes or flops)
    value = whole_job_rate(work, args.steps, world, ms / 1e3) / 1e9

    kernels = {}
    for k in range(nk):
        nm = names.raw[64 * k:64 * (k + 1)].split(b"\0")[0].decode()
        kernels[nm] = (tot[k], cnt[k])
    dom = max(kernels, key=lambda k: kernels[k][0])
    dom_ms = kernels[dom][0] / kernels[dom][1]
    dom_share = kernels[dom][0] / sum(v[0] for v in kernels.values())
    if args.graph:
        # events around single launches overstate microsecond kernels; the replayed step bounds
        # the kernel from above (exact when the step is that one launch)
        dom_ms = min(dom_ms, ms / args.steps)
    if op.pattern == "spgemm":  # the bytes model covers all three phases of a step
        what = ("symbolic + fill + numeric" if args.variant == 1 else
                "one pass: binning, sort into product slots, scans, compaction")
        dom, dom_ms = "spgemm %s (%s largest)" % (what, dom), ms / args.steps
    peak, peak_kind = measured_peak()
    achieved = getattr(op, "roofline_bytes", op.bytes) / (dom_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": ncu_traffic(dom, "%s_%s" % (op.workload, args.dtype)),
                "kernel": dom, "kernel_ms": dom_ms, "peak_source": peak_kind,
                "kernel_share": dom_share}
    if op.pattern == "spmv" and rank == 0:
        # everything but x goes through L2 as streamed sectors; x is gathered, one per nonzero
        roofline["gather"] = gather_roofline(torch, L, op.nnz, dom_ms,
                                             op.bytes - op.cols * ESZ[args.dtype])
    del keep

    e2e = None
    abi = op.abi(torch, tg, T) if args.e2e_steps > 0 else None
    if abi is not None:
        astep, akeep, h2d, d2h, api = abi
        for _ in range(3):  # untimed, like the device steps' warm-up (first calls allocate)
            astep()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        calls = []  # each call's own time: the host link is shared, so a few calls can stall
        for _ in range(args.e2e_steps):
            tc = time.perf_counter()
            astep()
            calls.append(time.perf_counter() - tc)
        e2e_s = max_over_ranks(torch, time.perf_counter() - t0, world)
        e2e = {"value": whole_job_rate(work, args.e2e_steps, world, e2e_s) / 1e9,
               "unit": unit,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": args.e2e_steps, "ms_per_step": e2e_s / args.e2e_steps * 1e3, "api": api,
               "call_ms_median": float(np.median(calls)) * 1e3,
               "call_ms_min": float(min(calls)) * 1e3}
        del akeep
        e2e["link"] = host_link(torch, h2d, d2h)

    cpu = None
    if rank == 0 and not args.no_cpu:
        kind, cores, t, reps = time_cpu(op)
        cpu_work = getattr(op, "cpu_work", getattr(op, "cpu_bytes", work))
        cpu = {"value": cpu_work / t / 1e9, "unit": unit,
               "cores": 1 if op.pattern == "pack" else cores, "kind": kind,
               "sample": "%s, median of %d reps" % (getattr(op, "cpu_sample_desc",
                                                            "whole workload"), reps),
               "ms_per_step": t * 1e3, "cpu_model": cpu_model(), "omp": omp_setup()}
        if getattr(op, "cpu_phases", None):
            cpu.update(op.phase_ms(op.cpu_phases))  # taco's assemble and compute, separately
        serial = op.cpu_serial() if hasattr(op, "cpu_serial") else None
        if serial is not None:
            once, keep_s = serial
            once()
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                once()
                ts.append(time.perf_counter() - t0)
            cpu["serial"] = {"value": cpu_work / float(np.median(ts)) / 1e9, "unit": unit,
                             "cores": 1, "ms_per_step": float(np.median(ts)) * 1e3,
                             "code": "taco's default generated SpGEMM (serial)"}
            cpu["serial"].update(op.phase_ms("spgemm"))
            del keep_s

    if rank == 0:
        names_v = {"spmv": tg.spmv_variants, "spmm": tg.spmm_variants,
                   "sddmm": tg.sddmm_variants, "spgemm": lambda: ["one pass", "phases"],
                   "mttkrp": tg.spmm_variants, "ttm": tg.spmm_variants,
                   "ttv": tg.spmv_variants,
                   "pack": lambda: ["default"]}[op.pattern]()
        config = workload_config(op, world)
        variant = ("auto" if args.variant == -1 else "fused" if args.variant == -2
                   else names_v[args.variant])
        derived = {}
        if op.pattern == "spgemm":
            derived.update({"products_per_s": op.products * args.steps * world / (ms / 1e3),
                            "symbolic_bytes": op.sym_bytes, "numeric_bytes": op.num_bytes})
        if op.pattern == "spmm":
            derived["gather_model_gbs"] = op.gather_bytes * args.steps * world / (ms / 1e3) / 1e9
        if op.pattern == "sddmm":
            derived["compulsory_gbs"] = op.bytes * args.steps * world / (ms / 1e3) / 1e9
            derived["gather_model_gbs"] = op.gather_bytes * args.steps * world / (ms / 1e3) / 1e9
        out = {"metric": op.metric, "value": value, "unit": unit,
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": args.dtype, "data": "synthetic", "config": config,
               "variant": variant, "derived": derived,
               "pct_of_peak": value / peak if unit == "GB/s" else None, "gflops": op.flops * args.steps * world / (ms / 1e3) / 1e9,
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": clocks,
               "timing": ("one CUDA-graph replay of the %d steps (captured after warm-up)"
                          % args.steps if args.graph else "the %d steps launched from the host"
                          % args.steps),
               "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kernels.items()}}
        if args.workload == "spmv_powerlaw" and args.dtype == "f64" and world == 1 and \
                not args.no_secondary:
            torch.cuda.empty_cache()
            out["secondary"] = run_secondary()
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def host_link(torch, h2d, d2h, reps=5):
    """What the host link alone allows for a step's copies: one pinned host -> device copy of
    h2d bytes and one device -> host copy of d2h bytes, timed back to back (the bound of the
    e2e number, which moves the same bytes)."""
    if h2d <= 0:
        return None
    hb = torch.empty(h2d, dtype=torch.uint8).pin_memory()
    db = torch.empty(h2d, dtype=torch.uint8, device="cuda")
    hy = torch.empty(max(d2h, 1), dtype=torch.uint8).pin_memory()
    dy = torch.empty(max(d2h, 1), dtype=torch.uint8, device="cuda")
    db.copy_(hb, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        db.copy_(hb, non_blocking=True)
        if d2h > 0:
            hy.copy_(dy, non_blocking=True)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    return {"ms_per_step": ms, "h2d_gbs": h2d / (ms / 1e3) / 1e9,
            "how": "pinned copies of the step's bytes alone (cudaMemcpyAsync via torch)"}


def gather_ceiling(torch, L, reps=5):
    """Random 8-byte gathers per second of tacogb_probe_gather (ld.global.cg, 32 warps per SM,
    shared memory as the SpMV kernels hold it): the ceiling of an x-gathering SpMV."""
    from taco_gb300 import _native as N
    PR = N.probe()
    rows, n = 1 << 21, 1 << 25
    table = torch.zeros(rows * 2, dtype=torch.float64, device="cuda")
    idx = torch.randint(0, rows, (n,), dtype=torch.int32, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(7))
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    out = torch.empty(sms * 1024, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    def run():
        rc = PR.tacogb_probe_gather(table.data_ptr(), rows, idx.data_ptr(), n, out.data_ptr(),
                                   out.numel(), 1, 160, 70, sp)
        if rc:
            raise RuntimeError(L.tacogb_last_error().decode())
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    return n * reps / (e0.elapsed_time(e1) / 1e3), sms


def gather_roofline(torch, L, nnz, kernel_ms, streamed_bytes):
    """The SpMV kernel's x gathers (one per nonzero) per second against the gather ceiling
    measured now on this GPU (run after the timed region).  `l2_sectors` counts every 32-byte
    L2 sector both move: the kernel's gathers plus the operands it streams (crd, values, pos,
    y), against the probe's gathers plus its index reads (one sector per eight gathers)."""
    ceiling, sms = gather_ceiling(torch, L)
    achieved = nnz / (kernel_ms / 1e3)
    return {"achieved": achieved, "peak": ceiling, "unit": "gathers/s", "frac": achieved / ceiling,
            "floor_ms": nnz / ceiling * 1e3,
            "probe": "tacogb_probe_gather: random 8-byte ld.global.cg from a 32 MiB L2-resident "
                     "table, 160 KB shared memory held per SM (carveout 70 %), as the kernel",
            "l2_sectors": l2_sector_roofline(nnz, streamed_bytes, kernel_ms, ceiling)}


def l2_sector_roofline(nnz, streamed_bytes, kernel_ms, probe_gathers_per_s):
    """32-byte L2 sectors per second: the SpMV's one per x gather plus its streamed bytes, against
    the gather probe's one per gather plus its index reads (eight 4-byte indices per sector)."""
    sectors = nnz + streamed_bytes / 32
    achieved = sectors / (kernel_ms / 1e3)
    peak = probe_gathers_per_s * (1 + 1 / 8)
    return {"achieved": achieved, "peak": peak, "unit": "sectors/s", "frac": achieved / peak,
            "floor_ms": sectors / peak * 1e3}


def main_gather_probe(args, torch, tg, L):
    """The random-gather ceiling behind the SpMV roofline: random 8-byte loads from a 32 MiB
    L2-resident table of 16-byte rows (one L2 sector each, like the x gathers of a random-column
    SpMV), eight in flight per thread, 32 warps per SM, by load form and by the shared memory
    held per SM (which sets the L1 left).  One JSON line per configuration."""
    from taco_gb300 import _native as N
    PR = N.probe()
    rows, n = 1 << 21, 1 << 26
    table = torch.zeros(rows * 2, dtype=torch.float64, device="cuda")  # zero: see probe.cu
    idx = torch.randint(0, rows, (n,), dtype=torch.int32, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(7))
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    out = torch.empty(sms * 1024, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    clock_ghz = 2.07
    forms = {0: "ld.global.nc", 1: "ld.global.cg", 2: "ld.global.nc.L1::no_allocate"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for smem_kb, carve in ((0, -1), (192, -1), (64, 100)):
        for mode in (0, 1, 2):
            def run():
                tg.check(PR.tacogb_probe_gather(table.data_ptr(), rows, idx.data_ptr(), n,
                                               out.data_ptr(), out.numel(), mode, smem_kb, carve,
                                               sp), "tacogb_probe_gather")
            for _ in range(max(3, args.warmup)):
                run()
            reps = max(3, min(args.steps, 20))
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                run()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            rate = n / (ms / 1e3)
            print(json.dumps({
                "metric": "random_gather_rate", "value": rate / (sms * clock_ghz * 1e9),
                "unit": "gathers/clk/SM at %.2f GHz" % clock_ghz, "gathers_per_s": rate,
                "ms_per_launch": ms, "load": forms[mode], "smem_kb_per_sm": smem_kb,
                "carveout": carve, "config": {"workload": "gather_probe", "table_rows": rows,
                                              "gathers": n, "sms": sms}}), flush=True)
    # host -> device link: the bound of the end-to-end (taco ABI, host operands) numbers
    del table, idx
    hbuf = torch.empty(1 << 30, dtype=torch.uint8).pin_memory()
    dbuf = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")
    for _ in range(2):
        dbuf.copy_(hbuf, non_blocking=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(5):
        dbuf.copy_(hbuf, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 5
    print(json.dumps({"metric": "h2d_copy_gbs", "value": (1 << 30) / (ms / 1e3) / 1e9,
                      "unit": "GB/s", "ms_per_copy": ms,
                      "config": {"workload": "gather_probe", "bytes": 1 << 30,
                                 "how": "pinned host -> device copy (cudaMemcpyAsync), 1 GiB"}}),
          flush=True)


if __name__ == "__main__":
    main()
