"""bench.py's multi-process helpers on CPU: two gloo ranks (replicas only).

`bench.py --gpus N` runs N independent replicas under torchrun; the only
collectives are the barrier around the timed region and the max over ranks
of the elapsed time.  Both run here with world_size 2 on the gloo backend.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench
    w, r = bench.dist_setup()
    assert (w, r) == (ws, rank)
    bench.barrier(w)
    t = bench.reduce_max(1.5 + rank, w)  # rank 1 is the slower one
    out.put((rank, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_and_barrier():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]
