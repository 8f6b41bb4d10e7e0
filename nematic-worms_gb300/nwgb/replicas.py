"""Replicas across ranks: the only multi-GPU form of the workloads.

A single worm system does not shard without halo exchange and ghosted
filament segments, so several GPUs run independent replicas.  Batched
replicas of uneven size (the 256-replica sweep) are spread over the ranks by
bead count; the differentiable rollout (64 replicas of one configuration)
splits its replicas into equal contiguous blocks, and its loss and the four
parameter gradients are means over all replicas, reduced once per
optimisation step with one all-reduce of six numbers.

Host logic only (lists and torch.distributed calls); each rank's compute is
the batched engine or the rollout on its own GPU.
"""
from __future__ import annotations

from typing import Sequence

import torch


def partition(bead_counts: Sequence[int], world: int) -> list[list[int]]:
    """Greedy longest-first bin packing of replicas onto `world` ranks by bead
    count: replicas in decreasing bead count (ties by index), each to the rank
    with the fewest beads so far (ties to the lowest rank).  The largest rank
    load exceeds the smallest by at most one replica's beads.  Returns, per
    rank, its replica indices in increasing order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(bead_counts)), key=lambda r: (-int(bead_counts[r]), r))
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for r in order:
        k = min(range(world), key=lambda q: (load[q], q))
        out[k].append(r)
        load[k] += int(bead_counts[r])
    return [sorted(x) for x in out]


def contiguous_block(n_replicas: int, world: int, rank: int) -> range:
    """Replicas [lo, hi) of `rank` when all replicas have the same size: equal
    contiguous blocks (sizes differ by at most one), so that replica r keeps
    its global index, seed and initial state on whichever rank runs it."""
    base, extra = divmod(n_replicas, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def replica_mean(local_sum: torch.Tensor, local_count: int, dist=None) -> torch.Tensor:
    """Mean over the replicas of all ranks of per-replica values whose sum over
    this rank's replicas is `local_sum` (1-D): one SUM all-reduce of
    [local_sum, local_count] in float64.  Without a process group (one rank)
    it is local_sum / local_count."""
    v = torch.cat([local_sum.detach().to(torch.float64).reshape(-1),
                   torch.tensor([float(local_count)], dtype=torch.float64, device=local_sum.device)])
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(v, op=dist.ReduceOp.SUM)
    if v[-1] <= 0:
        raise ValueError("no replicas on any rank")
    return v[:-1] / v[-1]


def loss_and_gradient_mean(local_loss_mean: torch.Tensor, local_grad_mean: torch.Tensor, local_count: int,
                           dist=None):
    """Global (loss, gradient) of a loss that is a mean over replicas, from each
    rank's mean over its own replicas (what nwgb.observables.loss_s_cv and the
    rollout's backward give): the rank's means are weighted by its replica
    count.  Returns (loss, grad) float64 tensors on every rank."""
    dev = local_loss_mean.device  # the loss's device (CUDA under NCCL, the CPU under gloo)
    s = torch.cat([local_grad_mean.detach().to(device=dev, dtype=torch.float64).reshape(-1),
                   local_loss_mean.detach().to(torch.float64).reshape(1)]) * float(local_count)
    m = replica_mean(s, local_count, dist)
    return m[-1], m[:-1]
