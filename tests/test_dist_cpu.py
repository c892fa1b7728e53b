"""Multi-process (gloo, world size 2) check of the replica timing path of bench.py:
a barrier and the max-over-ranks reduction the JSON line reports."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, lr, pg = bench._dist()
    bench._barrier(pg)
    v = bench._max_over_ranks(pg, 10.0 + r)
    out[r] = (r, w, v)
    pg.destroy_process_group()


def test_gloo_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == (0, 2, 11.0) and out[1] == (1, 2, 11.0)
