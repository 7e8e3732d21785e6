"""Garment shards across ranks (one process per GPU).

Garments are independent, so a batch splits into contiguous shards, one per rank,
and the step exchanges nothing between ranks.  The reference's Simulator
(src/simulation.cu) steps one garment on one device; its batched form shards by
garment only.  Collectives appear only around the steps:

* a barrier and a max over ranks, to time a run by its slowest rank;
* an optional gather of every shard's positions to one rank, for output.

The step itself never waits on another rank.  `RankGroup` wraps torch.distributed
(NCCL between GPUs, gloo on the host) or nothing when there is one rank.
"""
from __future__ import annotations

import os
from typing import Sequence

import numpy as np


def shard_bounds(weights: Sequence[int], world: int) -> list[int]:
    """Contiguous partition of items with the given weights (e.g. vertex counts) into
    `world` shards: the cut between shards r - 1 and r is the item boundary whose
    running total is nearest to r / world of the whole.  The cuts never decrease
    and each shard's weight is within one item of total / world.  Returns world + 1
    bounds; shard r holds items [bounds[r], bounds[r + 1])."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(weights, dtype=np.int64)
    if (w < 0).any():
        raise ValueError("weights must be non-negative")
    cum = np.concatenate([[0], np.cumsum(w)])
    total = int(cum[-1])
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        k = int(np.searchsorted(cum, target))  # first boundary with running total >= target
        if k > 0 and abs(cum[k - 1] - target) <= abs(cum[min(k, len(w))] - target):
            k -= 1
        bounds.append(min(max(k, bounds[-1]), len(w)))
    bounds.append(len(w))
    return bounds


def my_shard(weights: Sequence[int], rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of the items rank `rank` owns."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    b = shard_bounds(weights, world)
    return b[rank], b[rank + 1]


class RankGroup:
    """The ranks of one job: rank / world from the launcher's environment (RANK,
    WORLD_SIZE, MASTER_ADDR / MASTER_PORT), torch.distributed when world > 1."""

    def __init__(self, backend: str = "nccl", device=None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.backend = backend
        self.dist = None
        self.device = device if device is not None else "cpu"
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                if backend == "nccl":
                    dist.init_process_group("nccl", device_id=device)
                else:
                    dist.init_process_group(backend)
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """The largest x over the ranks (every rank gets it)."""
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        """The sum of x over the ranks (every rank gets it)."""
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def gather_rows(self, local: np.ndarray, dst: int = 0) -> np.ndarray | None:
        """Concatenate every rank's rows (e.g. its shard's positions, n_r x 3) in rank
        order on rank `dst`; None on the other ranks.  Shards may differ in length."""
        if self.dist is None:
            return np.array(local, copy=True)
        import torch
        local = np.ascontiguousarray(local)
        n = torch.tensor([local.shape[0]], dtype=torch.int64, device=self.device)
        counts = [torch.zeros_like(n) for _ in range(self.world)]
        self.dist.all_gather(counts, n)
        counts = [int(c.item()) for c in counts]
        width = int(np.prod(local.shape[1:])) if local.ndim > 1 else 1
        m = max(counts)
        buf = torch.zeros((m, width), dtype=torch.from_numpy(local[:0]).dtype, device=self.device)
        buf[: local.shape[0]] = torch.from_numpy(local.reshape(local.shape[0], width)).to(self.device)
        parts = [torch.zeros_like(buf) for _ in range(self.world)] if self.rank == dst else None
        self.dist.gather(buf, parts, dst=dst)
        if self.rank != dst:
            return None
        rows = np.concatenate([p[:c].cpu().numpy() for p, c in zip(parts, counts)])
        return rows.reshape((rows.shape[0],) + local.shape[1:])

    def close(self) -> None:
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()
