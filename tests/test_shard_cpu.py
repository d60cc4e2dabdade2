"""The column shard of the s-grid ring across ranks, on CPU (gloo).

The reference's MPI build gives each rank a contiguous block of the grid's
rows of columns (lsgrid_spline.cpp:652-664 with mpi_utils.h:46-64), fills
the block of the new slot, all-gathers the slot (lsgrid_spline.cpp:907-910,
mpi_utils.h:69-79) and recomputes the gradients on every rank.  Checked here:

* the library's partition (cfdwm_partition_columns, host code) against the
  reference's own partition_weighted, compiled from its header by
  ``make -C oracle ref`` (oracle/ref_partition.cpp), and against hand-worked
  cases of its rule;
* two gloo ranks that each fill their block with the FP64 oracle and
  exchange it with cfdwavemaker_gb300.shard.allgather_rows: every ring array
  on both ranks is byte-identical to the single-process update, on a grid
  with an ignored subdomain (uneven row weights) and one with more ranks'
  worth of rows.
"""
import ctypes as C
import os
import socket

import numpy as np
import pytest

from conftest import REPO, golden_cfg, load_golden

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402

REF_PART = os.path.join(REPO, "oracle", "_ref", "libref_partition.so")


@pytest.fixture(scope="module")
def lib():
    from cfdwavemaker_gb300 import build
    import cfdwavemaker_gb300 as cw
    build.build()
    return cw.load()


def _ref_partition(w, s):
    L = C.CDLL(REF_PART)
    L.refp_partition.restype = C.c_int
    L.refp_partition.argtypes = [C.POINTER(C.c_long), C.c_int, C.c_int, C.POINTER(C.c_int)]
    w = np.ascontiguousarray(w, dtype=np.int64)
    b = np.zeros(s + 1, dtype=np.int32)
    n = L.refp_partition(w.ctypes.data_as(C.POINTER(C.c_long)), int(w.size), int(s),
                         b.ctypes.data_as(C.POINTER(C.c_int)))
    return [int(v) for v in b[:n]]


def test_partition_known_answers(lib):
    from cfdwavemaker_gb300.shard import partition
    # even weights: boundary r after the first row with acc * s >= r * total
    assert partition([1] * 10, 3, lib) == [0, 4, 7, 10]
    # all rows ignored: the even split, larger blocks first
    assert partition([0] * 10, 3, lib) == [0, 4, 7, 10]
    assert partition([0] * 10, 4, lib) == [0, 3, 6, 8, 10]
    # one rank, and more ranks than rows
    assert partition([5, 1, 2], 1, lib) == [0, 3]
    assert partition([1, 1], 4, lib) == [0, 1, 2, 2, 2]
    # a heavy row takes one boundary only; the next ones follow it
    assert partition([1, 100, 1, 1], 3, lib) == [0, 2, 3, 4]
    with pytest.raises(ValueError):
        partition([1, -1], 2, lib)


@pytest.mark.skipif(not os.path.exists(REF_PART), reason="reference partition not built (make -C oracle ref)")
def test_partition_matches_reference(lib):
    from cfdwavemaker_gb300.shard import partition
    rng = np.random.default_rng(8)
    cases = [(np.full(256, 256), s) for s in (1, 2, 3, 4, 7, 8)]
    for _ in range(300):
        n = int(rng.integers(0, 40))
        kind = rng.integers(4)
        if kind == 0:
            w = rng.integers(0, 10, n)
        elif kind == 1:
            w = np.where(rng.random(n) < 0.5, 0, rng.integers(1, 1000, n))
        elif kind == 2:
            w = np.zeros(n, dtype=np.int64)
        else:
            w = rng.integers(0, 3, n) * (10 ** rng.integers(0, 6, n))
        cases.append((w, int(rng.integers(1, 12))))
    for w, s in cases:
        assert partition(w, s, lib) == _ref_partition(w, s), (list(w), s)


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _grid(case):
    import oracle
    g = load_golden(case)
    cfg = golden_cfg(g)
    sea = oracle.Sea(cfg)
    return cfg, oracle.Sgrid(cfg, sea, nthreads=1)


def _worker(rank, ws, port, case, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import cfdwavemaker_gb300 as cw
        from cfdwavemaker_gb300.shard import allgather_rows, partition
        cfg, sg = _grid(case)
        lg = cfg["lsgrid"]
        nx, ny, nl = lg["nx"], lg["ny"], lg["nl"]
        ign = sg.array(19).reshape(nx, ny)
        bounds = partition((ign == 0).sum(axis=1), ws, cw.load())
        i0, i1 = bounds[rank], bounds[rank + 1]
        for _ in range(2):
            sg.advance()
            t0, ts = sg.state()
            sg.update_columns(t0 + 2 * lg["dt"], i0 * ny, i1 * ny, nthreads=1)
            slot = (ts + 3) % 4
            for which in range(4):
                a = sg.array(which).reshape((4, nx, ny) + ((nl,) if which else ()))[slot]
                whole = allgather_rows(torch.from_numpy(np.ascontiguousarray(a[i0:i1])), bounds)
                sg.set_slot(which, whole.numpy())
            sg.gradients()
        q.put((rank, bounds, [sg.array(k) for k in range(19)]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case,ws", [("sgrid_ignore", 2), ("sgrid_small", 3)])
def test_sharded_ring_matches_single_grid(lib, case, ws):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, case, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, sg = _grid(case)
    for _ in range(2):
        sg.update(nthreads=1)
    want = [sg.array(k) for k in range(19)]
    bounds = res[0][1]
    assert bounds[0] == 0 and bounds[-1] > 0 and all(b - a > 0 for a, b in zip(bounds, bounds[1:]))
    for rank, b, arrs in res:
        assert b == bounds
        for k in range(19):
            assert np.array_equal(arrs[k], want[k]), (rank, k)
