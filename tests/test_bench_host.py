"""Host logic of bench.py's multi-rank path, on CPU with gloo (world size 2).

Ranks run independent slices of the IV sweep (no data-path collective); the only collectives
are a barrier and a max over the ranks' elapsed times.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bias = bench.bias_slice(rank, world, W=8)
    el = torch.tensor([0.5 + rank])              # stand-in elapsed times
    dist.barrier()
    dist.all_reduce(el, op=dist.ReduceOp.MAX)
    out[rank] = (bias.tolist(), float(el.item()))
    dist.destroy_process_group()


def test_bias_slices_tile_the_sweep():
    world, W = 4, 512
    parts = [bench.bias_slice(r, world, W) for r in range(world)]
    full = np.concatenate(parts)
    assert np.array_equal(full, np.linspace(0.0, 2.0, W * world))
    assert all(len(p) == W for p in parts)


def test_two_ranks_gloo():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    b0, e0 = res[0]
    b1, e1 = res[1]
    assert e0 == e1 == pytest.approx(1.5)        # max over ranks
    assert b0[-1] < b1[0]                        # disjoint, ordered slices
    assert np.allclose(np.concatenate([b0, b1]), np.linspace(0.0, 2.0, 16))
