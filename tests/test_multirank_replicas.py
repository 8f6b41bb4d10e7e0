"""Replicas across ranks without a GPU: the bin packing of uneven replicas by
bead count, and the distributed loss and gradient of the differentiable
rollout on two gloo ranks, each computing its own replicas with the FP64
torch restatement of the rollout (the oracle), against one process computing
all of them."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import REPO
from nwgb.replicas import contiguous_block, loss_and_gradient_mean, partition


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_every_replica_and_balances_beads(world):
    rng = np.random.default_rng(world)
    # the 256-replica sweep's sizes: 50-2000 worms of 5-30 beads
    beads = [int(rng.integers(50, 2001) * rng.integers(5, 31)) for _ in range(256)]
    parts = partition(beads, world)
    assert len(parts) == world
    flat = sorted(r for p in parts for r in p)
    assert flat == list(range(256))
    loads = [sum(beads[r] for r in p) for p in parts]
    assert max(loads) - min(loads) <= max(beads)
    assert parts == partition(beads, world)  # deterministic


def test_contiguous_blocks_tile_the_replicas():
    for n, w in ((64, 1), (64, 2), (64, 3), (5, 8), (0, 2)):
        blocks = [contiguous_block(n, w, k) for k in range(w)]
        assert [r for b in blocks for r in b] == list(range(n))
        sizes = [len(b) for b in blocks]
        assert max(sizes) - min(sizes) <= 1


R_ALL, H, SEG = 3, 6, 3


def _case(lib):
    from nwgb.init import initial_state, wca_config

    cfg = wca_config(24, 8, (18.0, 18.0), seed=5, lib=lib)
    states = [initial_state(cfg, seed=40 + r, layout="rows") for r in range(R_ALL)]
    return cfg, states


def _loss_grad(cfg, states, reps):
    """Mean loss over `reps` (global replica indices) and its gradient, from
    the FP64 torch rollout with each replica's own noise and pair sample."""
    import torch

    import torch_rollout
    from nwgb.observables import PairSample, loss_s_cv

    nb = cfg.n_beads
    pos = np.concatenate([states[r][0] for r in reps])
    vel = np.concatenate([states[r][1] for r in reps])
    xi_all = torch_rollout.noise_table(cfg, R_ALL, H)
    xi = np.concatenate([xi_all[:, r * nb:(r + 1) * nb] for r in reps], axis=1)
    every = PairSample(R_ALL, nb, 2000, seed=3)
    pairs = PairSample(1, nb, 1, seed=0)
    pairs.i, pairs.j = every.i[list(reps)], every.j[list(reps)]
    th = torch.tensor([1.0, 10.0, 57.0, 0.5], dtype=torch.float64, requires_grad=True)
    r, v = torch_rollout.rollout(cfg, th, pos, vel, len(reps), H, SEG, xi)
    box = [cfg.box[0], cfg.box[1], cfg.box[2]]
    target = torch.zeros((len(reps), 32), dtype=torch.float64)
    L = loss_s_cv(r.reshape(len(reps), -1, 3), v.reshape(len(reps), -1, 3), cfg.filament_size, box, pairs, target)
    L.backward()
    return L.detach(), th.grad.detach()


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO / "nematic-worms_gb300"))
    sys.path.insert(0, str(REPO / "oracle"))
    import torch.distributed as dist

    import nwgb

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    cfg, states = _case(nwgb.load_library())
    mine = list(contiguous_block(R_ALL, world, rank))
    L, g = _loss_grad(cfg, states, mine)
    loss, grad = loss_and_gradient_mean(L, g, len(mine), dist)
    dist.destroy_process_group()
    np.save(Path(out_dir, f"r{rank}.npy"), np.concatenate([[loss.item()], grad.numpy(), [len(mine)]]))


@pytest.mark.timeout(600)
def test_two_ranks_reduce_the_rollout_gradient_like_one_process(lib, tmp_path):
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    got = [np.load(Path(tmp_path, f"r{k}.npy")) for k in range(2)]
    assert got[0][-1] + got[1][-1] == R_ALL and got[0][-1] == 2  # replicas 0, 1 | 2
    assert np.array_equal(got[0][:-1], got[1][:-1])  # every rank holds the same result
    sys.path.insert(0, str(REPO / "oracle"))
    cfg, states = _case(lib)
    L, g = _loss_grad(cfg, states, list(range(R_ALL)))
    want = np.concatenate([[L.item()], g.numpy()])
    assert np.allclose(got[0][:-1], want, rtol=1e-12, atol=0.0), (got[0][:-1], want)
