"""bench.py's own line on the GPU: the contract's keys, and the CUDA-graph timing of a
launch-bound workload (the K steps captured once and replayed; launches counted at capture)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "roofline",
        "e2e", "gpu_launches", "clocks", "timing")


def _bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--no-secondary",
                        "--no-cpu", *args], cwd=ROOT, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


@pytest.mark.parametrize("graph", [False, True])
def test_small_spmv_line(graph):
    steps = 50
    d = _bench("--workload", "spmv_small", "--steps", str(steps), "--warmup", "3",
               "--e2e-steps", "2", *(["--graph"] if graph else []))
    for k in KEYS:
        assert k in d, k
    assert d["steps"] == steps and d["value"] > 0 and d["ms_per_step"] > 0
    assert "L2-resident" in d["config"]["l2"]
    # the small matrix of short rows runs the one-launch vector kernel, one launch per step
    assert d["roofline"]["kernel"] == "spmv_vector_kernel"
    assert d["gpu_launches"] == steps
    assert ("CUDA-graph" in d["timing"]) == graph
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert 0 < d["e2e"]["call_ms_min"] <= d["e2e"]["call_ms_median"]
    # the gather roofline counts gathers alone and every L2 sector moved; the second is larger
    g = d["roofline"]["gather"]
    assert g["unit"] == "gathers/s" and g["l2_sectors"]["unit"] == "sectors/s"
    assert g["l2_sectors"]["achieved"] > g["achieved"] > 0
