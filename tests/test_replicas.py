"""bench.py's replica path on CPU: two gloo ranks (127.0.0.1) run the same
set-up, barrier and max-over-ranks timing that N-GPU runs use (one
independent replica per GPU, no data exchange on the product path)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    t = bench.max_over_ranks(pg, 1.0 + rank)  # each replica's own time; the slowest counts
    out[rank] = t
    pg.destroy_process_group()


def test_two_gloo_replicas_take_the_max():
    world, port = 2, _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}
