"""The multi-rank layout of bench.py --gpus N, on CPU with the gloo backend.

Each rank owns the paths [r n, (r+1) n) (path_offset = r n) and the normals are
addressed by global path index, so the ranks' EE sums add up to the EE of one
run over all N n paths.  Here each rank values its shard with the oracle on
the counter-addressed host normals and the sums are all-reduced over gloo
(world size 2, 127.0.0.1); the result must equal the oracle's single run.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle_lib as O
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

N_PER_RANK, N_STEPS = 24, 300


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard_ee_sum(rank: int, mk: Market, sw: Swap, cfg: RunConfig) -> np.ndarray:
    normals = O.host_normals(cfg.seed, rank * N_PER_RANK, N_PER_RANK, N_STEPS)
    x = O.exposure_paths(mk, sw, N_STEPS, cfg.dt, normals)
    return x.sum(axis=0)


def _worker(rank: int, world: int, port: int, out) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mk, sw = Market(), Swap(n_periods=5)
        cfg = RunConfig(n_paths=N_PER_RANK, n_steps=N_STEPS, seed=1234, path_offset=rank * N_PER_RANK)
        s = torch.from_numpy(_shard_ee_sum(rank, mk, sw, cfg))
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        t = torch.tensor([float(rank + 1)])
        dist.all_reduce(t, op=dist.ReduceOp.MAX)  # bench.py's max-over-ranks timing
        if rank == 0:
            out.put((s.numpy() / (world * N_PER_RANK), float(t.item())))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_reproduce_one_run():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), q), nprocs=world, join=True, start_method="spawn")
    ee_ranks, tmax = q.get()
    assert tmax == 2.0
    mk, sw = Market(), Swap(n_periods=5)
    normals = O.host_normals(1234, 0, world * N_PER_RANK, N_STEPS)
    ee_one = O.expected_exposure(O.exposure_paths(mk, sw, N_STEPS, 0.01, normals))
    np.testing.assert_allclose(ee_ranks, ee_one, rtol=1e-13, atol=1e-13 * np.max(np.abs(ee_one)))
