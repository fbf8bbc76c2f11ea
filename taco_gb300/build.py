"""Builds the native parts of taco_gb300 in-tree.

  libtacogb.so          CUDA kernels (sm_103a) + the C ABI (include/taco_gb300.h)
  libtacogb_<p>.so      per-pattern modules exporting taco's unprefixed kernel names
                        (assemble / compute / evaluate / _shim_*) for p in spmv, spmm, spgemm
  libtacogb_gen.so      deterministic synthetic-matrix generators (include/taco_gb300_gen.h)
  libtacogb_probe.so    the random-gather probe bench.py measures the SpMV ceiling with
                        (include/taco_gb300_probe.h); not part of libtacogb

Every .cu file compiles in parallel with one -gencode (compute_103a / sm_103a); objects are
reused when their source and the shared headers are older than the object.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")

CU_SOURCES = ["abi.cu", "spmv.cu", "spmm.cu", "spgemm.cu", "batched.cu", "batched_spmm.cu",
              "tuner.cu", "pack.cu", "sddmm.cu", "tensor3.cu", "formats.cu", "validate.cu",
              "fileio.cpp"]
PATTERNS = ["spmv", "spmm", "spgemm", "sddmm", "ttv", "ttm", "mttkrp"]
NARGS = {"sddmm": 4, "mttkrp": 4}  # tensors per call (result and operands); 3 otherwise
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    "--expt-relaxed-constexpr", "--extended-lambda", "-I" + INC, "-I" + CSRC,
]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _compile_cu(src, extra):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + _headers()
    if _stale(obj, deps):
        _run([NVCC] + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj])
    return obj


def build(verbose=False, extra_flags=()):
    os.makedirs(OBJDIR, exist_ok=True)
    extra = list(extra_flags)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile_cu(s, extra), CU_SOURCES + ["probe.cu"]))
        probe_obj = objs.pop()
        gen_src = os.path.join(CSRC, "gen.c")
        gen_lib = os.path.join(LIBDIR, "libtacogb_gen.so")
        fut_gen = None
        if _stale(gen_lib, [gen_src, os.path.join(INC, "taco_gb300_gen.h")]):
            fut_gen = ex.submit(_run, ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC",
                                       "-shared", "-I" + INC, gen_src, "-o", gen_lib, "-lm"])
        lib = os.path.join(LIBDIR, "libtacogb.so")
        if _stale(lib, objs):
            _run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a"] + objs
                 + ["-o", lib])
        probe_lib = os.path.join(LIBDIR, "libtacogb_probe.so")
        if _stale(probe_lib, [probe_obj, lib]):
            _run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", probe_obj,
                  "-o", probe_lib, "-L" + LIBDIR, "-ltacogb", "-Xlinker", "-rpath,$ORIGIN"])
        mods = []
        mod_src = os.path.join(CSRC, "module.c")
        for p in PATTERNS:
            out = os.path.join(LIBDIR, "libtacogb_%s.so" % p)
            if _stale(out, [mod_src, lib, os.path.join(INC, "taco_gb300.h")]):
                mods.append(ex.submit(_run, ["gcc", "-O2", "-fPIC", "-shared", "-I" + INC,
                                             "-DTACOGB_PATTERN=%s" % p,
                                             "-DTACOGB_NARGS=%d" % NARGS.get(p, 3), mod_src, "-o", out,
                                             "-L" + LIBDIR, "-ltacogb", "-Wl,-rpath,$ORIGIN"]))
        for f in mods:
            f.result()
        if fut_gen:
            fut_gen.result()
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True, extra_flags=sys.argv[1:])
