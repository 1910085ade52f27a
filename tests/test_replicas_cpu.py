"""Multi-GPU replicas: the host logic of bench.py --gpus N (one process per
GPU, independent integrations, no collective on the data path) as two gloo
ranks on the CPU: the reduction of the per-rank times and evaluation counts
(slowest rank's time, all ranks' evaluations) and distinct seeds per rank."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench

        t_local = 1.0 + rank  # rank 1 is the slowest
        got = bench.reduce_over_ranks(t_local, 0.5 * (1 + rank), 1000 * (rank + 1), 10 * (rank + 1), ws,
                                      torch.device("cpu"))
        seeds = [bench.rank_seed(rank, k) for k in range(5)]
        out[rank] = (got, seeds)
    finally:
        dist.destroy_process_group()


def test_replica_reduction_and_seeds():
    ws = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(ws, _free_port(), out), nprocs=ws, join=True)
        res = dict(out)
    for rank in range(ws):
        (t_max, e2e_t, evals, e2e_evals), _ = res[rank]
        assert (t_max, e2e_t, evals, e2e_evals) == (2.0, 1.0, 3000, 30)  # same on every rank
    s0, s1 = set(res[0][1]), set(res[1][1])
    assert not (s0 & s1)


def test_single_process_reduction_is_identity():
    import bench

    assert bench.reduce_over_ranks(1.5, 0.5, 7, 3, 1, torch.device("cpu")) == (1.5, 0.5, 7, 3)
