"""The multi-rank path of bench.py on CPU (gloo, world size 2).

The hot path shards as replicas only: each rank runs the whole workload on its
own GPU with no data-path collective.  What crosses ranks is the timing: a
barrier on both sides of the timed region and the maximum of the per-rank
times, from which rank 0 reports the whole-job rate (units x ranks / max time).
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(ws),
                       "RANK": str(rank), "LOCAL_RANK": str(rank), "CFDWM_GLOO": "1"})
    import bench
    w, r, local = bench.dist_init()
    bench.barrier(w)
    t = bench.allmax(w, 10.0 + 5.0 * r)      # rank 1 is the slower replica
    bench.barrier(w)
    q.put((r, w, local, t))
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 for x in res)
    # both ranks see the slower rank's time: the whole-job rate uses it
    assert all(abs(x[3] - 15.0) < 1e-12 for x in res)
