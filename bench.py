"""Benchmark of taco_gb300's sparse hot path on one GB300 (or N replicas under torchrun).

Default workload: FP64 CSR SpMV y(i) = A(i,j) * x(j) on the 4,194,304 x 4,194,304 power-law
matrix (Zipf(2) row lengths scaled to mean 24, clipped to [1, 20000]; ~1.0e8 nnz; columns
uniform, sorted; values U(-1,1)).  One step = one SpMV over the whole matrix.

  value  algorithmic GB/s of the device path (inputs resident in HBM), bytes model
         B = nnz*(4+8) + 4*(rows+1) + 8*cols (x once) + 8*rows (y)
  e2e    the same metric through taco's kernel ABI (tacogb_spmv_compute on taco_tensor_t with
         pinned host arrays): every step copies pos/crd/vals/x to the GPU and y back
  roofline  the dominant kernel's algorithmic bytes / its mean event-timed duration, against
         the measured HBM copy bandwidth
  cpu_baseline  taco's own generated C for the statement (oracle/_ref, compiled with taco's JIT
         flags, OpenMP over all host cores), or the C restatement when that is absent

`--impl reference` times taco's generated CPU code alone (rank 0) and prints its line.
Working set (1.29 GB) is larger than L2 (129 MB): no flush between steps.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="spmv_powerlaw",
                   choices=["spmv_powerlaw", "spmv_banded", "spmv_small"])
    p.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    p.add_argument("--variant", type=int, default=-1)
    p.add_argument("--e2e-steps", type=int, default=30)
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def workload_spec(name):
    from taco_gb300 import workloads as W
    return {"spmv_powerlaw": W.spmv_powerlaw, "spmv_banded": W.spmv_banded,
            "spmv_small": W.spmv_small}[name]()


def bytes_model(rows, cols, nnz, sv=8, sx=8, sy=8):
    return nnz * (4 + sv) + 4 * (rows + 1) + sx * cols + sy * rows


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
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


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = None

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


def cpu_baseline(pos, crd, vals, x, reps=None, budget_s=8.0):
    """taco's generated SpMV (or the C restatement) on all host cores."""
    from oracle import oracle as O
    from taco_gb300 import taco as T
    rows, cols = len(pos) - 1, len(x)
    ncores = os.cpu_count() or 1
    y = np.empty(rows)
    if O.ref_available("spmv"):
        kind = "reference"
        L = O.ref_lib("spmv")
        O.ref_set_threads(ncores)
        At, Xt, Yt = T.csr(pos, crd, vals, [rows, cols]), T.dense(x, [cols]), T.dense(y, [rows])

        def once():
            L.compute(Yt.ptr, At.ptr, Xt.ptr)
    else:
        kind = "port"
        O.set_threads(ncores)

        def once():
            O.lib().oracle_spmv_f64(rows, pos.ctypes.data, crd.ctypes.data, vals.ctypes.data,
                                    x.ctypes.data, y.ctypes.data)
    for _ in range(3):
        once()
    times = []
    t_end = time.perf_counter() + budget_s
    while (reps is None and time.perf_counter() < t_end and len(times) < 200) or \
            (reps is not None and len(times) < reps):
        t0 = time.perf_counter()
        once()
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    return kind, ncores, t, len(times)


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    s = workload_spec(args.workload)
    from taco_gb300 import workloads as W
    from oracle import oracle as O
    O.build()
    pos, crd, vals = W.generate(s)
    x = W.dense(23, s.cols)
    nnz = len(crd)
    B = bytes_model(s.rows, s.cols, nnz)
    kind, cores, _, _ = cpu_baseline(pos, crd, vals, x, reps=args.warmup)
    # timed: exactly K steps
    from taco_gb300 import taco as T
    y = np.empty(s.rows)
    if kind == "reference":
        L = O.ref_lib("spmv")
        At, Xt, Yt = T.csr(pos, crd, vals, [s.rows, s.cols]), T.dense(x, [s.cols]), T.dense(y, [s.rows])
        step = lambda: L.compute(Yt.ptr, At.ptr, Xt.ptr)  # noqa: E731
    else:
        step = lambda: O.lib().oracle_spmv_f64(s.rows, pos.ctypes.data, crd.ctypes.data,  # noqa: E731
                                               vals.ctypes.data, x.ctypes.data, y.ctypes.data)
    steps = max(1, min(args.steps, 200))
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    v = B * steps / dt / 1e9
    out = {"metric": "spmv_fp64_hbm_gbs", "value": v, "unit": "GB/s", "impl": "reference",
           "n_gpus": world, "steps": steps, "warmup": args.warmup,
           "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "%s_%d" % (args.workload, s.rows), "rows": s.rows,
                      "nnz": nnz, "bytes_per_step": B,
                      "code": "taco generated C, -O3 -ffast-math -fopenmp" if kind == "reference"
                      else "C restatement of taco's loop, -O2 -fopenmp"},
           "cpu_baseline": {"value": v, "unit": "GB/s", "cores": cores, "kind": kind,
                            "sample": "whole matrix per step, %d steps" % steps},
           "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


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
    from taco_gb300 import workloads as W
    L = tg.lib()

    s = workload_spec(args.workload)
    pos, crd, vals = W.generate(s)
    x = W.dense(23, s.cols)
    nnz = len(crd)
    dt = torch.float64 if args.dtype == "f64" else torch.float32
    esz = 8 if args.dtype == "f64" else 4
    A = tg.CsrMatrix.from_numpy(pos, crd, vals, s.cols, dtype=dt)
    xd = torch.from_numpy(x).to("cuda", dt)
    yd = torch.empty(s.rows, dtype=dt, device="cuda")
    B = bytes_model(s.rows, s.cols, nnz, esz, esz, esz)
    stream = torch.cuda.current_stream()
    csr = A.as_csr()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        rc = L.tacogb_spmv(ctypes.byref(csr), xd.data_ptr(), yd.data_ptr(), args.variant, sp)
        if rc:
            raise RuntimeError(L.tacogb_last_error().decode())

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.tacogb_launch_count()
    L.tacogb_profile_begin()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = L.tacogb_launch_count() - launches0
    names = ctypes.create_string_buffer(64 * 16)
    tot = (ctypes.c_double * 16)()
    cnt = (ctypes.c_int32 * 16)()
    nk = L.tacogb_profile_end(16, names, tot, cnt)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = B * args.steps * world / (ms / 1e3) / 1e9

    kernels = {}
    for k in range(nk):
        nm = names.raw[64 * k:64 * (k + 1)].split(b"\0")[0].decode()
        kernels[nm] = (tot[k], cnt[k])
    dom = max(kernels, key=lambda k: kernels[k][0])
    dom_ms = kernels[dom][0] / kernels[dom][1]
    peak, peak_kind = measured_peak()
    achieved = B / (dom_ms / 1e3) / 1e9
    traffic = ncu_traffic(dom, "%s_%s" % (args.workload, args.dtype))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": dom, "kernel_ms": dom_ms, "peak_source": peak_kind,
                "kernel_share": kernels[dom][0] / sum(v[0] for v in kernels.values())}

    # e2e through the taco kernel ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        hp = torch.from_numpy(pos).pin_memory()
        hc = torch.from_numpy(crd).pin_memory()
        hv = torch.from_numpy(vals).to(dt).pin_memory()
        hx = torch.from_numpy(x).to(dt).pin_memory()
        hy = torch.empty(s.rows, dtype=dt).pin_memory()
        At = T.csr(hp, hc, hv, [s.rows, s.cols])
        Xt, Yt = T.dense(hx, [s.cols]), T.dense(hy, [s.rows])
        for _ in range(2):
            tg.check(L.tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr), "spmv_compute")
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            tg.check(L.tacogb_spmv_compute(Yt.ptr, At.ptr, Xt.ptr), "spmv_compute")
        e2e_s = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([e2e_s], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = (s.rows + 1) * 4 + nnz * (4 + esz) + s.cols * esz
        e2e = {"value": B * args.e2e_steps * world / e2e_s / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": s.rows * esz,
               "steps": args.e2e_steps, "ms_per_step": e2e_s / args.e2e_steps * 1e3,
               "api": "tacogb_spmv_compute(taco_tensor_t*) on pinned host arrays"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        kind, cores, t, reps = cpu_baseline(pos, crd, vals, x)
        cpu = {"value": B / t / 1e9, "unit": "GB/s", "cores": cores, "kind": kind,
               "sample": "whole matrix, median of %d reps" % reps, "ms_per_step": t * 1e3}

    if rank == 0:
        variant = args.variant if args.variant >= 0 else -1
        out = {"metric": "spmv_%s_hbm_gbs" % args.dtype, "value": value, "unit": "GB/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
               "config": {"workload": "%s_%d" % (args.workload, s.rows), "rows": s.rows,
                          "cols": s.cols, "nnz": nnz, "bytes_per_step": B,
                          "variant": "auto" if variant < 0 else tg.spmv_variants()[variant],
                          "l2": "inputs larger than L2 (%.2f GB per step), no flush" % (B / 1e9),
                          "parallelism": "replicas" if world > 1 else "single"},
               "pct_of_peak": value / peak,
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": clocks,
               "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kernels.items()}}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
