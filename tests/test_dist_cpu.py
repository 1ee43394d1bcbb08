"""bench.py's multi-rank path on CPU (gloo, 127.0.0.1).

Two ranks rendezvous, pass the barrier and agree on the max-over-ranks time
and the job-wide cell count (the bench's timed value under torchrun). Then
the partition of an ensemble's members: rank r takes members r, r + N, ...
of the job's member list (workloads.shard), advances them (here with the
oracle, the CPU restatement of the reference, standing in for the GPU), and
the gathered results show every member advanced exactly once and equal, bit
for bit, to one rank advancing all of them. No data-path collective exists:
the members are independent.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

EDGES = [10, 12, 14, 11, 13, 9, 12]
STEPS = 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _specs(wl):
    specs = wl.config4_specs(len(EDGES))
    for s, e in zip(specs, EDGES):  # small grids: the oracle finishes in milliseconds
        s["edge"] = e
    return specs


def _advance(ge, specs):
    """{member index: (P, S)} after STEPS oracle steps of each spec."""
    pkg = ge.load_package()
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    O = ge.load_oracle_module()
    lib = O.inputs_library(pkg.abi)
    orc = O.Oracle(pkg.abi)
    out = {}
    for s in specs:
        mem = wl.build_member(lib, s)
        st = O.State(mem.model, mem.media, mem.K, mem.phi)
        P, S = mem.initial_state()
        st["P1"][...] = P
        st["S2"][...] = S
        orc.step(st, STEPS)
        out[s["index"]] = (st["P1"].copy(), st["S2"].copy())
    return out


def _worker(rank, world, port, root, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), OMP_NUM_THREADS="1")
    sys.path.insert(0, root)
    import bench
    import __graft_entry__ as ge
    import torch.distributed as dist
    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    pkg = ge.load_package()
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    mine = wl.shard(_specs(wl), r, w)
    res = _advance(ge, mine)
    cells = sum(wl.spec_cells(s) for s in mine)
    gathered = [None] * w
    dist.all_gather_object(gathered, {k: (P.tobytes(), S.tobytes()) for k, (P, S) in res.items()})
    out[rank] = {"max": bench.dist_max(10.0 * (rank + 1), w), "cells": bench.dist_sum(float(cells), w),
                 "gathered": gathered if rank == 0 else None, "mine": sorted(res)}
    dist.destroy_process_group()


def test_two_ranks_partition_members_and_agree_with_one_rank():
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    import torch.multiprocessing as mp
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as ge
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, root, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=300)
            assert p.exitcode == 0
        out = dict(out)
    assert out[0]["max"] == out[1]["max"] == 20.0
    total = float(sum(e ** 3 for e in EDGES))
    assert out[0]["cells"] == out[1]["cells"] == total
    assert out[0]["mine"] == [0, 2, 4, 6] and out[1]["mine"] == [1, 3, 5]
    # every member exactly once across the ranks
    seen = [k for part in out[0]["gathered"] for k in part]
    assert sorted(seen) == list(range(len(EDGES)))
    # and the same bits as one rank advancing all members
    pkg = ge.load_package()
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    one = _advance(ge, wl.shard(_specs(wl), 0, 1))
    for part in out[0]["gathered"]:
        for k, (Pb, Sb) in part.items():
            P1, S1 = one[k]
            assert Pb == P1.tobytes() and Sb == S1.tobytes(), k


def test_shard_rejects_bad_ranks():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    items = list(range(10))
    assert sorted(wl.shard(items, 0, 3) + wl.shard(items, 1, 3) + wl.shard(items, 2, 3)) == items
    for rank, world in ((3, 3), (-1, 2), (0, 0)):
        with pytest.raises(ValueError):
            wl.shard(items, rank, world)
