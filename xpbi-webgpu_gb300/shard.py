"""Scene batches across GPUs: one process per GPU, no data-path collective.

Scenes of a batch are independent (the reference steps one scene per
Simulation, web/js/sim.js:9-30), so a job over several GPUs gives each rank
a disjoint subset of the caller's scenes and each rank steps its subset in
one batched handle. The only work that scales with a scene is its particle
count (every stage is one launch over all particles of a handle), so the
subsets are balanced on particle counts by a greedy bin-pack: scenes in
decreasing particle count (ties by position in the list) each go to the
rank with the least particles so far (ties to the lowest rank). The result
depends only on the list and the rank count, so every rank computes the
same partition without exchanging anything. The largest rank load exceeds
the mean by at most the largest scene.
"""
from __future__ import annotations

from typing import Sequence


def partition(counts: Sequence[int], world: int) -> list[list[int]]:
    """Indices of the scenes each of `world` ranks steps (each list in
    ascending order), by greedy bin-pack on the particle counts."""
    if world < 1:
        raise ValueError("world must be >= 1")
    counts = [int(c) for c in counts]
    if any(c < 0 for c in counts):
        raise ValueError("particle counts must be >= 0")
    order = sorted(range(len(counts)), key=lambda i: (-counts[i], i))
    load = [0] * world
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += counts[i]
    return [sorted(s) for s in shards]


def shard(scenes: Sequence[dict], rank: int, world: int) -> list[dict]:
    """This rank's scenes of a batch (see partition)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    parts = partition([len(s["positions"]) for s in scenes], world)
    return [scenes[i] for i in parts[rank]]


def loads(counts: Sequence[int], parts: list[list[int]]) -> list[int]:
    """Particles per rank of a partition."""
    return [sum(int(counts[i]) for i in p) for p in parts]
