"""The multi-rank host logic of bench.py on CPU: world_size 2 over gloo (no GPU).  Each
rank runs its own fields (weak scaling, replicas only); the step time is the max over
ranks and the value counts every rank's bytes."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    times = [3.25, 7.5]
    out[rank] = (bench.max_over_ranks(times[rank], dist), bench.rank_seed0(rank, 8))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_disjoint_fields_gloo():
    world = 2
    with mp.get_context("spawn").Manager() as m:  # no fork of this (threaded) process
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        got = dict(out)
    assert got[0][0] == got[1][0] == 7.5          # the slowest rank's time, on every rank
    assert got[0][1] == 1 and got[1][1] == 9       # seeds 1..8 and 9..16: no field twice


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(4.0, None) == 4.0


def test_weak_scaling_value_formula():
    """value = fields x 2 x 4n x steps x world / time: whole-job bytes over the max time."""
    fields, n, steps, world, ms = 8, 15209600, 10, 2, 4.0
    bytes_step = fields * 2 * 4 * n
    value = bytes_step * steps * world / (ms / 1e3) / 1e9
    assert value == pytest.approx(2 * bytes_step * steps / 4e-3 / 1e9)
