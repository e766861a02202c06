"""Replica parallelism over independent variational points.

The solve path does not shard: one GPU holds the largest sector it needs, and
each variational point is an independent vca_solve.  N GPUs therefore run N
replicas, each over its own slice of the points.  No collective runs on the
data path.  The only collectives are host-side: a barrier around the timed
region, a max over the ranks' timings, and an optional gather of the Omega
values (torch.distributed, gloo).
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple


def dist_env() -> Tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def partition(n_points: int, rank: int, world: int) -> List[int]:
    """Point indices of one rank: the round-robin slice rank, rank+world, ...
    Every point belongs to exactly one rank."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return list(range(rank, n_points, world))


class Group:
    """Host-side helpers over an initialised gloo process group (or none)."""

    def __init__(self, dist=None):
        self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def gather_values(self, idx: Sequence[int], vals: Sequence[float], n_points: int) -> List[float]:
        """All ranks' (index, value) pairs assembled into one list of n_points."""
        out = [float("nan")] * n_points
        if self.dist is None:
            for i, v in zip(idx, vals):
                out[i] = float(v)
            return out
        import torch
        t = torch.full((n_points,), float("nan"), dtype=torch.float64)
        for i, v in zip(idx, vals):
            t[i] = float(v)
        # each point is set on exactly one rank: a MAX over ranks with NaN
        # elsewhere would drop it, so sum with zeros instead
        z = torch.nan_to_num(t, nan=0.0)
        m = (~torch.isnan(t)).to(torch.float64)
        self.dist.all_reduce(z)
        self.dist.all_reduce(m)
        return [float(z[i]) if m[i] > 0 else float("nan") for i in range(n_points)]
