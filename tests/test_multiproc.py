"""The benchmark's N > 1 host logic on CPU: two gloo ranks on 127.0.0.1.

Each rank steps its own shard of independent scenes (no data-path
collective): a caller's batch is split by the particle-count bin-pack of
shard.py, which every rank computes alike; the job's time is the slowest
rank's; the whole-job throughput counts every rank's particles; the
reference arm runs on rank 0 only. No GPU is involved."""
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
        import importlib

        import bench
        S = importlib.import_module("xpbi-webgpu_gb300.scenes")
        shard = importlib.import_module("xpbi-webgpu_gb300.shard")
        # the 256-scene mixed batch: particle counts only (the bin-pack reads nothing else)
        counts = [len(s["positions"]) for s in S.config_batch(seed=0)]
        mine = shard.partition(counts, world)[rank]
        parts = [None] * world
        dist.all_gather_object(parts, mine)
        # a per-rank workload through the benchmark's own split
        _, scenes, scaling = bench.workload("sand_column", rank, world)
        pos = np.asarray(scenes[0]["positions"], np.float64)
        sigs = [None] * world
        dist.all_gather_object(sigs, float(pos.sum()))
        slowest = bench.max_over_ranks(10.0 * (rank + 1), dist, device="cpu")
        job = bench.job_particles(len(pos) * (rank + 1), dist, device="cpu")
        q.put((rank, sigs, slowest, len(pos), parts, counts, job))
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
        results = sorted((q.get(timeout=300) for _ in range(2)), key=lambda r: r[0])
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    (r0, sigs0, t0, n0, parts0, counts, job0), (r1, sigs1, t1, n1, parts1, _, job1) = results
    assert (r0, r1) == (0, 1)
    assert sigs0 == sigs1 and sigs0[0] != sigs0[1]  # each rank has its own seeded scene
    assert t0 == t1 == 20.0                           # the slowest rank's time
    assert job0 == job1 == n0 + 2 * n1                 # every rank's particles
    # the batch split: both ranks computed the same partition, the shards are
    # disjoint, together they are the batch, and the loads differ by at most
    # the largest scene
    assert parts0 == parts1
    a, b = set(parts0[0]), set(parts0[1])
    assert not (a & b) and (a | b) == set(range(len(counts))) and len(counts) == 256
    sys.path.insert(0, ROOT)
    import importlib
    shard = importlib.import_module("xpbi-webgpu_gb300.shard")
    la, lb = shard.loads(counts, parts0)
    assert abs(la - lb) <= max(counts)
    assert abs(la - lb) <= 0.01 * (la + lb)           # in practice within 1% for this batch
    import bench
    assert bench.job_throughput(job0, 10, t0) == pytest.approx(job0 * 10 / 20.0)


def test_partition_is_deterministic_and_balanced():
    sys.path.insert(0, ROOT)
    import importlib
    shard = importlib.import_module("xpbi-webgpu_gb300.shard")
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 4, 8):
        counts = [int(x) for x in np.exp(rng.uniform(np.log(2000), np.log(60000), 97))]
        parts = shard.partition(counts, world)
        assert parts == shard.partition(list(counts), world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(counts)))
        ld = shard.loads(counts, parts)
        assert max(ld) - sum(ld) / world <= max(counts)
    assert shard.partition([], 3) == [[], [], []]
    assert shard.partition([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]  # ties: list order, lowest rank
    with pytest.raises(ValueError):
        shard.partition([1], 0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    args = types.SimpleNamespace(cpu_scale=0.01, warmup=0, steps=0, gpus=2, workload="dam_mix4")
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
