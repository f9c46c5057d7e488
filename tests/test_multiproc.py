"""The benchmark's N > 1 host logic on CPU: two gloo ranks on 127.0.0.1.

Each rank steps its own shard of independent scenes (weak scaling, no
data-path collective); the job's time is the slowest rank's; the whole-job
throughput counts every rank's particles; the reference arm runs on rank 0
only. No GPU is involved."""
import os
import socket
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        import bench
        _, scenes = bench.workload("sand_column", rank)
        pos = np.asarray(scenes[0]["positions"], np.float64)
        sigs = [None] * world
        dist.all_gather_object(sigs, float(pos.sum()))
        slowest = bench.max_over_ranks(10.0 * (rank + 1), dist, device="cpu")
        q.put((rank, sigs, slowest, len(pos)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_scenes_and_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        results = sorted(q.get(timeout=300) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    (r0, sigs0, t0, n0), (r1, sigs1, t1, n1) = results
    assert (r0, r1) == (0, 1)
    assert sigs0 == sigs1 and sigs0[0] != sigs0[1]  # each rank has its own seeded scene
    assert t0 == t1 == 20.0                           # the slowest rank's time
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(n0, 2, 10, t0) == pytest.approx(n0 * 2 * 10 / 20.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    args = types.SimpleNamespace(cpu_scale=0.01, warmup=0, steps=0, gpus=2, workload="dam_mix4")
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
