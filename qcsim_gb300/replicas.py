"""Host logic for running the engine on several GPUs of one node, one process per GPU.

The statevector path does not shard: a 30-33-qubit register fits one GB300, so the layered-circuit
benchmark runs N independent replicas and only the timing is reduced (max over ranks).  The batched
QAOA workload is a set of independent instances: they are dealt to ranks by cost, each rank runs
its share in one launch, and the energies are gathered once at the end (no collective on the data
path).  The collectives here work on any torch.distributed group (NCCL on GPUs, gloo on CPUs).
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_by_cost(costs, world: int) -> list[list[int]]:
    """deal items to `world` ranks, largest cost first, each to the currently lightest rank (LPT);
    returns the item indices of every rank in ascending order"""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shards]


def qaoa_costs(instances) -> list[float]:
    """work of one QAOA instance: its amplitude count"""
    return [float(1 << inst["n"]) for inst in instances]


def max_over_ranks(dist, value: float, device: str = "cpu") -> float:
    """the largest `value` over the ranks of the default group (the job's time is its slowest rank's)"""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_values(dist, indices, values, total: int, device: str = "cpu") -> np.ndarray:
    """every rank's (index, value) pairs into one array of length `total` on every rank"""
    import torch
    local = np.full(total, np.nan)
    local[np.asarray(indices, dtype=np.int64)] = np.asarray(values, dtype=np.float64)
    if dist is None:
        return local
    t = torch.tensor(local, dtype=torch.float64, device=device)
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    out = np.full(total, np.nan)
    for p in parts:
        v = p.cpu().numpy()
        ok = ~np.isnan(v)
        out[ok] = v[ok]
    return out
