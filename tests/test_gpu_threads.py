"""Concurrent callers: the reference's host codes call the point functions
from OpenMP threads (wave_VeloX & co. are read-only and reentrant there).
Here several host threads call the scalar and batched entry points at once
(ctypes releases the GIL during the calls, so the calls overlap); every
thread must get the reference's values."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import load_golden, norm_rel_err

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("thr"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


@pytest.mark.parametrize("case", ["config1_point", "smit_spread", "fenton24"])
def test_concurrent_scalar_and_batched_calls(wm, case):
    g = load_golden(case)
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    lib = wm.lib
    x, y, z, t = (np.ascontiguousarray(g["pt_" + k]) for k in "xyzt")
    n = x.size
    ref_u, ref_p = g["api_VeloX"], g["api_DynPres"]

    def work(k):
        idx = np.arange(k, n, 8)
        u = np.array([lib.wave_VeloX(float(x[i]), float(y[i]), float(z[i]), float(t[i])) for i in idx])
        p = wm.dynamic_pressure_batch(x[idx], y[idx], z[idx], t[idx])
        return idx, u, p

    with ThreadPoolExecutor(8) as ex:
        res = list(ex.map(work, range(8)))
    u = np.zeros(n)
    p = np.zeros(n)
    for idx, ui, pi in res:
        u[idx] = ui
        p[idx] = pi
    assert norm_rel_err(u, ref_u) <= TOL
    assert norm_rel_err(p, ref_p) <= TOL


def test_concurrent_sgrid_queries(wm):
    g = load_golden("sgrid_small")
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    qx, qy, qz = g["query_x"], g["query_y"], g["query_z"]
    qt = np.full_like(qx, float(np.ravel(g["s0_query_t"])[0]))
    ref = g["s0_kin"]

    def work(k):
        return wm.kinematics_batch(qx, qy, qz, qt)

    with ThreadPoolExecutor(6) as ex:
        outs = list(ex.map(work, range(12)))
    for o in outs:
        for c in range(4):
            assert norm_rel_err(o[:, c], ref[:, c]) <= TOL
