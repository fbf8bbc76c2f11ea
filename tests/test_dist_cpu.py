"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).  bench.py runs one
independent replica per GPU (the SpMV/SpMM/SpGEMM path needs no exchange between GPUs), joins
them with barriers, takes the slowest rank's time, and reports the whole job's throughput;
the reference arm runs on rank 0 only.  No GPU is used."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, lr, w = bench.dist_env()
        ms = bench.max_over_ranks(torch, 10.0 + 5.0 * rank, w)   # rank 1 is the slow one
        dist.barrier()
        value = bench.whole_job_rate(1000, 4, w, ms / 1e3)
        # the reference arm is rank 0's alone: other ranks return before doing any work
        ref = bench.run_reference(bench.parse(["--impl", "reference"])) if rank != 0 else None
        out.put((rank, r, lr, w, ms, value, ref))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, lr, w, ms, value, ref in res:
        assert (r, lr, w) == (rank, rank, 2)
        assert ms == 15.0                       # every rank sees the slowest rank's time
        assert value == pytest.approx(1000 * 4 * 2 / 0.015)  # both replicas' work
        assert ref is None


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(torch, 3.5, 1) == 3.5
    assert bench.whole_job_rate(10, 2, 1, 0.5) == 40.0

