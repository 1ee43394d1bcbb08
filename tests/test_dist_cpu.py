"""bench.py's multi-rank path on CPU: two gloo ranks rendezvous on 127.0.0.1,
pass the barrier and agree on the max-over-ranks time (the bench's timed
value under torchrun). Replicas only: no data-path collective exists."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, root, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, root)
    import bench
    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    m = bench.dist_max(10.0 * (rank + 1), w)
    out[rank] = m
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_barrier_and_max_over_ranks():
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    import torch.multiprocessing as mp
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, root, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        assert dict(out) == {0: 20.0, 1: 20.0}
