"""GPU parity of the dynamic pressure on the s-grid ring (cfdwm_sgrid_pressure)
with the FP64 oracle, through the C ABI.

The field is dp1(z0) + rho uvw2.p(z0) + dp1_dz max(0, z - swl) at every node
(the reference computes uvw2.p in its grid update, lsgrid_spline.cpp:892,
and drops it); wave_DynPres / wave_nhPres of wave type 5 then return
ramp * p and ramp * (p - rho g eta) from the spline query.  Bars as the other
s-grid parity tests: normwise relative error TOL = 1e-5 for node values and
queries, TOL_GRAD = 1e-4 for the finite-difference arrays.
"""
import os

import numpy as np
import pytest

from conftest import golden_cfg, load_golden, norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_GRAD = 1e-4
# product array numbers of the pressure (dt, dx, dy, ds, field) -> the oracle's
P_ARRAYS = {19: 21, 20: 22, 21: 23, 22: 24, 23: 20}


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("run")
    cwd = os.getcwd()
    os.chdir(d)
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


def _valid_dt_slots(ts):
    return {1, 2} if ts == 0 else {1, 2} | {(s + 2) % 4 for s in range(1, ts + 1)}


def _compare_pressure(wm, og, ts, label):
    for which, ow in P_ARRAYS.items():
        got, ref = wm.sgrid_array(which), og.array(ow)
        assert got.size == ref.size, (label, which)
        tol = TOL if which == 23 else TOL_GRAD
        if which == 19:
            n = got.size // 4
            for s in _valid_dt_slots(ts):
                err = norm_rel_err(got[s * n:(s + 1) * n], ref[s * n:(s + 1) * n])
                assert err <= tol, (label, which, s, err)
        else:
            err = norm_rel_err(got, ref)
            assert err <= tol, (label, which, err)


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("case", ["sgrid_small", "sgrid_ignore"])
def test_sgrid_pressure_vs_oracle(wm, case, method):
    g = load_golden(case)
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    wm.sgrid_method(method)
    wm.sgrid_pressure(True)
    cfg = golden_cfg(g)
    sea = oracle.Sea(cfg)
    og = oracle.Sgrid(cfg, sea, pressure=True)
    updates = {"sgrid_small": [0.7, 1.6], "sgrid_ignore": [1.5]}[case]
    qx, qy, qz = g["query_x"], g["query_y"], g["query_z"]
    for k in range(len(updates) + 1):
        if k > 0:
            wm.force_update(updates[k - 1])
            og.force_update(updates[k - 1])
        t0, ts = wm.sgrid_state()
        assert (t0, ts) == og.state()
        _compare_pressure(wm, og, ts, (case, method, k))
        # the velocities are the golden ones with the pressure field beside them
        for which in range(4):
            assert norm_rel_err(wm.sgrid_array(which), g["s%d_arr%d" % (k, which)]) <= TOL, (k, which)
        qt = np.full_like(qx, float(np.ravel(g["s%d_query_t" % k])[0]))
        ref = og.query(qx, qy, np.maximum(qz, -cfg["depth"]), qt)
        rr = oracle.ramp(cfg, qx, qy, qt)
        p = wm.dynamic_pressure_batch(qx, qy, qz, qt)
        nh = wm.nonhydrostatic_pressure_batch(qx, qy, qz, qt)
        assert norm_rel_err(p, rr * ref[:, 4]) <= TOL, (case, method, k)
        nh_ref = rr * (ref[:, 4] - cfg["rho"] * cfg["gravity"] * ref[:, 0])
        assert norm_rel_err(nh, nh_ref) <= TOL, (case, method, k)
        # the scalar entry point serves the same value
        i = int(np.argmax(np.abs(p)))
        v = wm.lib.wave_DynPres(float(qx[i]), float(qy[i]), float(qz[i]), float(qt[i]))
        assert abs(v - p[i]) <= 1e-12 * max(1.0, abs(p[i]))


def test_sgrid_pressure_tensor_core_vs_plain(wm):
    """The pressure blocks of the depth-separable tensor-core form against the
    plain column sums on the 1024-component short-crested sea (64 x 16),
    40 x 36 x 16 patch, after the initial fill and two updates."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea()
    grid = {"bounds": (100.0, 100.0 + 39 * 3.92, 200.0, 200.0 + 35 * 3.92), "nx": 40, "ny": 36, "nl": 16,
            "t0": 5.0, "dt": 0.5, "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)
    arrs = {}
    for method in (0, 1):
        assert wm.initialize_text(txt) == 0, cw.last_error()
        wm.sgrid_method(method)
        wm.sgrid_pressure(True)
        t0, _ = wm.sgrid_state()
        wm.force_update(t0 + 2 * 0.5 + 0.25)
        arrs[method] = {w: wm.sgrid_array(w) for w in P_ARRAYS}
    for w in P_ARRAYS:
        err = norm_rel_err(arrs[1][w], arrs[0][w])
        assert err <= (TOL if w == 23 else TOL_GRAD), (w, err)


def test_sgrid_pressure_oracle_on_the_1024_sea_sample(wm):
    """Plain and tensor-core node pressure of the 1024-component sea against
    the FP64 oracle on a small 6 x 5 x 16 patch (the oracle's cost grows with
    the pairs, 521k here)."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea()
    grid = {"bounds": (300.0, 300.0 + 5 * 3.92, 40.0, 40.0 + 4 * 3.92), "nx": 6, "ny": 5, "nl": 16,
            "t0": 5.0, "dt": 0.5, "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)
    cfg = oracle.waveinput.read_text(txt)
    og = oracle.Sgrid(cfg, oracle.Sea(cfg), pressure=True)
    ref = og.array(20)
    for method in (0, 1):
        assert wm.initialize_text(txt) == 0, cw.last_error()
        wm.sgrid_method(method)
        wm.sgrid_pressure(True)
        err = norm_rel_err(wm.sgrid_array(23), ref)
        assert err <= TOL, (method, err)


def test_sgrid_pressure_off_and_exclusions(wm):
    g = load_golden("sgrid_small")
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    qx, qy, qz = g["query_x"], g["query_y"], g["query_z"]
    qt = np.full_like(qx, float(np.ravel(g["s0_query_t"])[0]))
    # the reference's wave type 5 returns 0.0 for both pressures
    assert np.all(wm.dynamic_pressure_batch(qx, qy, qz, qt) == 0.0)
    assert np.all(wm.nonhydrostatic_pressure_batch(qx, qy, qz, qt) == 0.0)
    with pytest.raises(RuntimeError):
        wm.sgrid_array(23)
    wm.sgrid_pressure(True)
    assert np.max(np.abs(wm.dynamic_pressure_batch(qx, qy, qz, qt))) > 0.0
    # the learned update predicts no pressure: it is refused while the field is on
    if wm.lib.cfdwm_surrogate_nparams() <= 0:
        assert wm.lib.cfdwm_surrogate_create(int(golden_cfg(g)["lsgrid"]["nl"]), 1) == 0
    assert wm.lib.cfdwm_surrogate_enable(1, 4, 0.05, 8) == -2
    assert wm.lib.cfdwm_surrogate_step(1, 0.05, 8, None, None) == -2
    wm.sgrid_pressure(False)
    assert np.all(wm.dynamic_pressure_batch(qx, qy, qz, qt) == 0.0)
    # and the velocities after switching back are the golden ones again
    for which in range(4):
        assert norm_rel_err(wm.sgrid_array(which), g["s0_arr%d" % which]) <= TOL


def test_sgrid_pressure_with_component_ramps(wm):
    """Individual (per-component) ramps still rising during the ring steps:
    the ramps enter the pressure's phase-free height table per time step."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(3.0, 8.0, 2.0, 10, 0.45, 1.6, 30.0, 77, ndir=3, spreading_s=5.0)
    n = comps["omega"].size
    rng = np.random.default_rng(12)
    rcols = [rng.uniform(1.0, 3.0, n), rng.uniform(-0.5, 0.5, n), rng.uniform(30.0, 60.0, n)]
    grid = {"bounds": (0.0, 60.0, -20.0, 20.0), "nx": 9, "ny": 7, "nl": 6, "t0": 0.2, "dt": 0.4,
            "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 30.0, extrap=2, lsgrid=grid, ramp_columns=rcols)
    cfg = oracle.waveinput.read_text(txt)
    og = oracle.Sgrid(cfg, oracle.Sea(cfg), pressure=True)
    for method in (0, 1):
        assert wm.initialize_text(txt) == 0, cw.last_error()
        wm.sgrid_method(method)
        wm.sgrid_pressure(True)
        if method == 1:
            og = oracle.Sgrid(cfg, oracle.Sea(cfg), pressure=True)
        for k, tt in enumerate([None, 1.3, 2.2]):
            if tt is not None:
                wm.force_update(tt)
                og.force_update(tt)
            _, ts = wm.sgrid_state()
            _compare_pressure(wm, og, ts, ("ramps", method, k))
            for which in range(4):      # elevation and velocities of the ring too
                err = norm_rel_err(wm.sgrid_array(which), og.array(which))
                assert err <= TOL, ("ramps", method, k, which, err)
