"""The multi-rank host path of bench.py (one replica per rank under torchrun):
rendezvous, barrier and the max over ranks, as world_size-2 gloo processes on
the CPU (127.0.0.1)."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    r, w = bench.dist_init(world)
    bench.barrier(w)
    out[rank] = (r, w, dist.get_backend(), bench.max_over_ranks(1.5 + rank, w))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_ranks_take_the_max_over_ranks():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (r, w, backend, mx) in res.items():
        assert (r, w, backend) == (rank, world, "gloo")
        assert mx == 2.5
