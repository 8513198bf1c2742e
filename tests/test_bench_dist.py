"""bench.py's multi-rank logic on CPU (world size 2, gloo, 127.0.0.1): ranks rendezvous,
the timing is the maximum over ranks, and the reference arm runs on rank 0 only (the other
ranks return without work).  With one GPU per rank the GPU arm runs independent replicas of
the path with no collective on the data path; only the barrier and this maximum use the
process group."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist

    ws, r, local = bench.dist_setup(types.SimpleNamespace(impl="reference"))
    assert (ws, r, local) == (2, rank, rank)
    bench.barrier(ws)
    m = bench.max_over_ranks(1.5 + rank, ws)
    if rank == 1:
        # the reference arm: every rank but 0 leaves without work or output
        assert bench.run_reference(types.SimpleNamespace(), ws, rank) is None
    bench.barrier(ws)
    dist.destroy_process_group()
    out.put((rank, m))


def test_two_ranks_gloo():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 2.5, 1: 2.5}
