"""GPU parity of vertical_theory smit (Smit et al. 2017 s-coordinate second
order, Irregular.cpp:1622-2027; experimental upstream) through the C ABI.

The reference's own outputs at the golden points are checked in
test_gpu_parity.py (cases smit_spread, smit_ramps).  Here, against the FP64
oracle (pinned exactly to those golden values): random points below, at and
above the surface on both golden seas; a 120-component short-crested sea;
the scalar entry points; and the s-grid, which the theory leaves unchanged
(its update calls u1 and uvw2 directly, lsgrid_spline.cpp:880-903).
Bar: normwise relative error 1e-5 per field (FP32 pair sums, FP64 phases).
"""
import os

import numpy as np
import pytest

from conftest import golden_cfg, load_golden, norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-5
API = ["SurfElev", "VeloX", "VeloY", "VeloZ", "DynPres", "nhPres"]


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("smit"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


def _api(wm, x, y, z, t):
    eta = wm.surface_elevation_batch(x, y, t)
    u, v, w = wm.velocity_batch(x, y, z, t)
    return [eta, u, v, w, wm.dynamic_pressure_batch(x, y, z, t), wm.nonhydrostatic_pressure_batch(x, y, z, t)]


def _check(wm, txt, x, y, z, t, label):
    assert wm.initialize_text(txt) == 0, cw.last_error()
    cfg = oracle.waveinput.read_text(txt)
    assert cfg["vertical_theory"] == 1
    got = _api(wm, x, y, z, t)
    ref = oracle.Model(cfg).api(x, y, z, t)
    for q, name in enumerate(API):
        err = norm_rel_err(got[q], ref[:, q])
        assert err <= TOL, (label, name, err)
    return got, ref


@pytest.mark.parametrize("case", ["smit_spread", "smit_ramps"])
def test_smit_random_points_vs_oracle(wm, case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    rng = np.random.default_rng(8)
    n = 600
    x = rng.uniform(-150, 300, n)
    y = rng.uniform(-80, 80, n)
    z = rng.uniform(-cfg["depth"] - 2.0, 4.0, n)     # below the seabed, through the surface, above
    t = rng.uniform(0.0, 30.0, n)
    got, ref = _check(wm, str(g["waveinput"]), x, y, z, t, case)
    # points above the surface are 0.0 for u, v, w, dp (Irregular.cpp:1628)
    above = ref[:, 1] == 0.0
    assert np.any(above) and np.all(got[1][above] == 0.0) and np.all(got[4][above] == 0.0)


def test_smit_few_point_kernel_matches_batch_kernel(wm):
    """600 points in one batch (per-thread kernel) and in batches of 1, 9
    and 100 (few-point kernel, a block per point): within 1e-6 normwise of
    each other, and the batched ones within TOL of the FP64 oracle."""
    g = load_golden("smit_spread")
    cfg = golden_cfg(g)
    rng = np.random.default_rng(10)
    n = 600
    x = rng.uniform(-150, 300, n)
    y = rng.uniform(-80, 80, n)
    z = rng.uniform(-cfg["depth"], 2.0, n)
    t = rng.uniform(0.0, 30.0, n)
    whole, ref = _check(wm, str(g["waveinput"]), x, y, z, t, "smit_spread whole")
    for size, count in ((1, 30), (9, 600), (100, 600)):
        parts = [_api(wm, x[b:b + size], y[b:b + size], z[b:b + size], t[b:b + size])
                 for b in range(0, count, size)]
        for q, name in enumerate(API):
            got = np.concatenate([pt[q] for pt in parts])
            m = got.size
            assert norm_rel_err(got, whole[q][:m]) <= 1e-6, (size, name, norm_rel_err(got, whole[q][:m]))
            assert norm_rel_err(got, ref[:m, q]) <= TOL, (size, name)


def test_smit_short_crested_120(wm):
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(4.0, 10.0, 2.5, 24, 0.35, 1.7, 60.0, 123, ndir=5, spreading_s=5.0)
    txt = ss.write_irregular(None, comps, 60.0, extrap=2, swl=0.3, mtheta=-35.0, rho=1025.0,
                             vertical_theory="smit")
    rng = np.random.default_rng(9)
    n = 400
    x = rng.uniform(-300, 300, n)
    y = rng.uniform(-300, 300, n)
    z = rng.uniform(-60.0, 3.0, n)
    t = rng.uniform(0.0, 60.0, n)
    _check(wm, txt, x, y, z, t, "smit_120")


def test_smit_scalar_entry_points(wm):
    g = load_golden("smit_spread")
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    lib = wm.lib
    for i in range(0, g["pt_x"].size, 5):
        x, y, z, t = (float(g["pt_" + k][i]) for k in "xyzt")
        vals = [lib.wave_VeloX(x, y, z, t), lib.wave_VeloY(x, y, z, t), lib.wave_VeloZ(x, y, z, t),
                lib.wave_DynPres(x, y, z, t)]
        for v, name in zip(vals, ["VeloX", "VeloY", "VeloZ", "DynPres"]):
            ref = g["api_" + name]
            assert abs(v - ref[i]) <= TOL * max(np.max(np.abs(ref)), 1e-30), (name, i)


def test_sgrid_unchanged_by_smit(wm):
    g = load_golden("sgrid_small")
    txt = str(g["waveinput"])
    smit = txt.replace("kinematics_surf_extrap 2", "kinematics_surf_extrap 2\nvertical_theory smit")
    assert smit != txt
    arrs = []
    for text in (txt, smit):
        assert wm.initialize_text(text) == 0, cw.last_error()
        wm.force_update(0.7)
        arrs.append([wm.sgrid_array(w) for w in range(4)])
    for a, b in zip(*arrs):
        np.testing.assert_array_equal(a, b)
