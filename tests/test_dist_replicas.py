"""The N > 1 path of bench.py on CPU: the solver does not shard (exact
Gauss-Seidel is one global order), so N ranks run N replicas.  What needs
checking is the host logic around them -- rendezvous on 127.0.0.1, the
barrier, and the max over ranks that the timed value takes -- with two
gloo ranks and no GPU.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local = bench.dist_setup()
    bench.dist_barrier(w)
    # each replica reports its own step time; the job's time is the slowest
    t = bench.dist_max(1.5 + r, w)
    bench.dist_barrier(w)
    q.put((r, w, local, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_over_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert [o[2] for o in out] == [0, 1]
    assert all(o[3] == 2.5 for o in out)


def test_single_process_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    ws, rank, local = bench.dist_setup()
    assert (ws, rank, local) == (1, 0, 0)
    assert bench.dist_max(3.25, ws) == 3.25
    bench.dist_barrier(ws)
