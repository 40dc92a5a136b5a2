"""The multi-GPU path of bench.py: the layer's gate list is split into
contiguous shards, one per rank, each rank bootstraps its shard on its own
GPU, and the output ciphertexts are gathered to rank 0 on the host (the
between-layer exchange); the job's time is the slowest rank's.  (--replicas:
the whole layer on every rank.)  Covered here with world size 2 on the gloo
backend (CPU): the partition, the gather's order, the aggregation, the job
throughput, and the reference arm printing on rank 0 only."""
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


def _gather_main(rank, world, port, count, q):
    try:
        os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                           "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
        sys.path.insert(0, ROOT)
        import numpy as np
        import torch.distributed as dist
        import bench
        dist.init_process_group("gloo", rank=rank, world_size=world)
        lo, hi = bench.layer_shards(count, world)[rank]
        # this rank's "outputs": row g holds (g, rank, g * 7) -- the gate
        # index it computed, the rank that computed it, a payload
        rows = np.array([[g, rank, g * 7] for g in range(lo, hi)], np.int32).reshape(-1, 3)
        full = bench.gather_layer(rows, count, world, rank)
        dist.destroy_process_group()
        q.put((rank, None if full is None else full.tolist()))
    except Exception as e:  # reported to the parent
        q.put((rank, "error", repr(e)))


@pytest.mark.parametrize("count", [4096, 37, 1])
def test_layer_split_and_gather_with_gloo(count):
    """Each rank bootstraps a contiguous shard of the layer; rank 0 receives
    every gate's output exactly once, in layer order (shards of unequal size
    included; a 1-gate layer leaves rank 1 an empty shard)."""
    pytest.importorskip("torch")
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gather_main, args=(r, world, port, count, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict((r[0], r[1:]) for r in (q.get(timeout=120) for _ in range(world)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] != "error" and res[1][0] != "error", res
    assert res[1][0] is None
    full = res[0][0]
    assert [row[0] for row in full] == list(range(count))
    assert [row[2] for row in full] == [7 * g for g in range(count)]
    sys.path.insert(0, ROOT)
    import bench
    shards = bench.layer_shards(count, world)
    assert [row[1] for row in full] == [r for r, (lo, hi) in enumerate(shards) for _ in range(lo, hi)]


def test_layer_shards_cover_the_layer():
    sys.path.insert(0, ROOT)
    import bench
    for count in (1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            sh = bench.layer_shards(count, world)
            assert sh[0][0] == 0 and sh[-1][1] == count
            assert all(sh[i][1] == sh[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in sh]
            assert max(sizes) - min(sizes) <= 1


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
