"""The multi-process path of bench.py (replicas, one process per GPU) on CPU:
two gloo ranks rendezvous on 127.0.0.1, pass the barrier and agree on the
maximum of their per-rank times, as the bench does before rank 0 prints."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, w, local, pg = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(pg)
    m = bench.allmax(pg, 10.0 + rank)
    out[rank] = m
    pg.destroy_process_group()


def test_two_gloo_ranks_agree_on_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: 11.0, 1: 11.0}
