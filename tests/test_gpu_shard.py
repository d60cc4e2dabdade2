"""The rank side of the column shard of the s-grid ring, on one GPU.

Several GPUs are not available to these tests, so the ranks are emulated one
after another in this process, each on a freshly loaded copy of the same
model: rank r runs cfdwm_sgrid_step_block over its rows (the partition of
cfdwm_sgrid_partition) and exports them; then rank 0's model imports every
other rank's rows (what the all-gather delivers) and finishes the step.  Two
ring updates later every array of the ring (the 19 of the reference's
lsGridSpline) must equal the single-grid update (wave_force_update) within a
few FP32 roundings (the column kernels of a block launch may sum a column's
pair tiles in another order than the whole-grid launch, and the tensor-core
form adds its tiles with atomics in no fixed order): 1e-6 normwise.  The
gather itself is tested across processes on CPU (tests/test_shard_cpu.py).
"""
import os

import numpy as np
import pytest

from conftest import load_golden, norm_rel_err

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("shard"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


def _load(wm, txt, method):
    assert wm.initialize_text(txt) == 0, cw.last_error()
    wm.sgrid_method(method)


def _rows(wm, f, a, b):
    n = wm.lib.cfdwm_sgrid_block_count(f, a, b)
    assert n >= 0
    out = np.zeros(n, dtype=np.float32)
    if n:
        assert wm.lib.cfdwm_sgrid_block_export(f, a, b, cw._ptr(out)) == 0, cw.last_error()
    return out


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("case,nranks", [("sgrid_small", 2), ("sgrid_small", 3), ("sgrid_ignore", 2)])
def test_block_steps_reassemble_the_ring(wm, case, nranks, method):
    txt = str(load_golden(case)["waveinput"])
    _load(wm, txt, method)
    t0, _ = wm.sgrid_state()
    import ctypes as C
    dt = 0.5 if case == "sgrid_small" else 0.4
    times = [t0 + 1.01 * dt, t0 + 2.01 * dt]
    for t in times:
        wm.lib.wave_force_update(t)
    want = [wm.sgrid_array(k) for k in range(19)]
    b = (C.c_int * (nranks + 1))()
    assert wm.lib.cfdwm_sgrid_partition(nranks, b) == 0
    bounds = list(b)
    assert bounds[0] == 0 and all(y > x for x, y in zip(bounds, bounds[1:]))
    nf = 4
    # every rank's rows of both updates
    blocks = {}
    for r in range(nranks):
        _load(wm, txt, method)
        for k, t in enumerate(times):
            assert wm.lib.cfdwm_sgrid_due(t) == 1
            assert wm.lib.cfdwm_sgrid_step_block(bounds[r], bounds[r + 1]) == 0, cw.last_error()
            for f in range(nf):
                blocks[r, k, f] = _rows(wm, f, bounds[r], bounds[r + 1])
    # rank 0's model with the other ranks' rows imported
    _load(wm, txt, method)
    for k, t in enumerate(times):
        assert wm.lib.cfdwm_sgrid_step_block(bounds[0], bounds[1]) == 0, cw.last_error()
        for r in range(1, nranks):
            for f in range(nf):
                a = blocks[r, k, f]
                assert wm.lib.cfdwm_sgrid_block_import(f, bounds[r], bounds[r + 1], cw._ptr(a)) == 0
        assert wm.lib.cfdwm_sgrid_step_finish() == 0, cw.last_error()
        assert wm.lib.cfdwm_sgrid_due(t) == 0
    got = [wm.sgrid_array(k) for k in range(19)]
    for k in range(19):
        assert norm_rel_err(got[k], want[k]) <= 1e-6, (k, norm_rel_err(got[k], want[k]))
    # the block calls check their arguments
    assert wm.lib.cfdwm_sgrid_block_count(0, 2, 1) == -3
    assert wm.lib.cfdwm_sgrid_step_block(-1, 2) == -3
