"""Cost-balanced split of a batch of independent instances across ranks.

Instances never exchange data, so N GPUs run N independent shares with no
collective on the data path; only the counts and the step time are reduced.
"""
from __future__ import annotations


def instance_cost(d) -> float:
    """Work of one propagator pass: nodes x contour steps."""
    return float(d["n_nodes"]) * float(d["nsteps"])


def partition(costs, world: int):
    """Longest-first greedy assignment; returns one sorted index list per rank."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += costs[i]
        parts[r].append(i)
    return [sorted(p) for p in parts]


def shard(instances, rank: int, world: int):
    """Indices of the instances rank `rank` of `world` solves."""
    if world == 1:
        return list(range(len(instances)))
    return partition([instance_cost(d) for d in instances], world)[rank]
