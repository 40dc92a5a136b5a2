"""The multi-GPU path of bench.py is replicas only: each rank runs the whole
gate layer on its own GPU, and the only cross-rank step is the maximum of
the ranks' times (plus a barrier).  Covered here with world size 2 on the
gloo backend (CPU): the aggregation, the job throughput, and the reference
arm printing on rank 0 only."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    try:
        os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                           "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
        sys.path.insert(0, ROOT)
        import torch.distributed as dist
        import bench
        dist.init_process_group("gloo", rank=rank, world_size=world)
        w, r, loc = bench.dist_env()
        per_rank_ms = [120.0, 95.5][rank]
        dist.barrier()
        mx = bench.max_over_ranks(per_rank_ms, w, "cpu")
        value = bench.job_throughput(4096 * 10, w, mx)
        dist.destroy_process_group()
        q.put((rank, w, r, loc, mx, value))
    except Exception as e:  # reported to the parent
        q.put((rank, "error", repr(e)))


def test_replicas_aggregate_with_gloo():
    pytest.importorskip("torch")
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, *rest in res:
        assert rest[0] != "error", rest
        w, r, loc, mx, value = rest
        assert (w, r, loc) == (world, rank, rank)
        assert mx == 120.0  # the slowest rank's time
        assert abs(value - 2 * 4096 * 10 / 0.120) < 1e-6


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.job_throughput(100, 1, 1000.0) == 100.0


def test_reference_arm_runs_on_rank0_only(capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    args = argparse.Namespace(steps=1, warmup=0, gpus=2)
    assert bench.run_reference(args, 2, 1) is None
    assert capsys.readouterr().out == ""
