"""Pin the CPU oracle against the reference.

The fixtures in tests/golden/ were recorded from the unmodified reference
(oystelan/CFDwavemaker v3.1.0, compiled from its own sources) by
tests/golden/make_golden.py; two of them also carry the reference's own
golden vectors (t005 targetwave.dat, t002 exact_solution.mat).  The oracle is
an FP64 restatement, so it must reproduce them to ~1e-10 or better.
"""
import numpy as np
import pytest

from conftest import golden_cfg, load_golden, norm_rel_err

import oracle

IRREGULAR = ["t005_focused", "t002_exact", "config1_point", "short_spread", "ramps_swl", "linear",
             "smit_spread", "smit_ramps"]
REGULAR = ["stokes5", "fenton24", "stokes5_len", "fenton_len"]
API = ["SurfElev", "VeloX", "VeloY", "VeloZ", "DynPres", "nhPres"]


@pytest.mark.parametrize("case", IRREGULAR + REGULAR)
def test_parser_matches_reference(case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    if "components" in g:
        comp = g["components"]
        for row, key in enumerate(("omega", "A", "k", "phase", "theta", "ramptime", "starttime",
                                   "duration")):
            np.testing.assert_array_equal(np.asarray(cfg[key]), comp[row], err_msg=key)
        # the reference builds its pair cache only for second order
        # (CFDwavemaker.cpp:1365-1369)
        if cfg["order"] == 2:
            assert oracle.Sea(cfg).npairs == int(g["npairs"])


@pytest.mark.parametrize("case", IRREGULAR)
def test_irregular_api(case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    m = oracle.Model(cfg)
    out = m.api(g["pt_x"], g["pt_y"], g["pt_z"], g["pt_t"])
    for q, name in enumerate(API):
        ref = g["api_" + name]
        assert norm_rel_err(out[:, q], ref) < 1e-11, (case, name, norm_rel_err(out[:, q], ref))


@pytest.mark.parametrize("case", IRREGULAR)
def test_irregular_internals(case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    sea = oracle.Sea(cfg)
    x, y, z, t = g["pt_x"], g["pt_y"], g["pt_z"], g["pt_t"]
    assert norm_rel_err(sea.eta2(x, y, t), g["irr_eta2"]) < 1e-11
    u = sea.uvw2(x, y, g["irr_uvw2_z"], t)
    for q in range(4):
        assert norm_rel_err(u[:, q], g["irr_uvw2"][:, q]) < 1e-11, q


def test_t005_target_wave():
    """The reference's own golden elevation series (tests/t005_focused_wave/targetwave.dat)."""
    g = load_golden("t005_focused")
    cfg = golden_cfg(g)
    m = oracle.Model(cfg)
    t = g["extra_targetwave_t"]
    eta = m.api(np.full_like(t, 10.0), np.zeros_like(t), np.zeros_like(t), t)[:, 0]
    ref = g["extra_targetwave_eta"]
    # targetwave.dat was written with 19 significant digits by np.savetxt
    assert norm_rel_err(eta, ref) < 1e-13


def test_t002_exact_solution():
    """The reference's own golden momentum integrals
    (tests/t002_spline_momentum_conservation/exact_solution.mat, generated by
    momentum_conservation.py:123-171): eta and the integrals of u|u|, v|v|,
    w|w| over z in [-20, 12) with the volume-fraction weight."""
    g = load_golden("t002_exact")
    cfg = golden_cfg(g)
    m = oracle.Model(cfg)
    time = g["extra_time"]
    sel = np.arange(0, time.size, 67)
    dz = 0.1
    z = np.arange(-20.0, 12, dz)
    T, Z = np.meshgrid(time[sel], z, indexing="ij")
    out = m.api(np.zeros(T.size), np.zeros(T.size), Z.ravel(), T.ravel()).reshape(sel.size, z.size, 6)
    eta = m.api(np.zeros(sel.size), np.zeros(sel.size), np.zeros(sel.size), time[sel])[:, 0]
    ratio = np.clip((eta[:, None] - (z[None, :] - dz / 2.0)) / ((z + dz / 2.0) - (z - dz / 2.0))[None, :], 0.0, 1.0)
    for q, key in ((1, "umom1"), (2, "vmom1"), (3, "wmom1")):
        mom = np.sum(out[:, :, q] * np.abs(out[:, :, q]) * dz * ratio, axis=1)
        ref = g["extra_" + key][sel]
        assert norm_rel_err(mom, ref) < 1e-10, (key, norm_rel_err(mom, ref))
    assert norm_rel_err(eta, g["extra_wave_elev1"][sel]) < 1e-12


@pytest.mark.parametrize("case", REGULAR)
def test_regular_api(case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    m = oracle.Model(cfg)
    out = m.api(g["pt_x"], g["pt_y"], g["pt_z"], g["pt_t"])
    for q, name in enumerate(API):
        ref = g["api_" + name]
        assert norm_rel_err(out[:, q], ref) < 1e-11, (case, name, norm_rel_err(out[:, q], ref))
    if "fenton_solution" in g:
        sol = m.reg.solution()
        ref = g["fenton_solution"]
        np.testing.assert_allclose(sol[: ref.size], ref, rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("case", ["sgrid_small", "sgrid_ignore"])
def test_sgrid(case):
    g = load_golden(case)
    cfg = golden_cfg(g)
    sea = oracle.Sea(cfg)
    grid = oracle.Sgrid(cfg, sea)
    updates = {"sgrid_small": [0.7, 1.6], "sgrid_ignore": [1.5]}[case]
    r = oracle.ramp(cfg, g["query_x"], g["query_y"], np.zeros_like(g["query_x"]))
    for k in range(int(g["nsnap"])):
        if k > 0:
            grid.force_update(updates[k - 1])
        t0, ts = grid.state()
        assert ts == g["s%d_dims" % k][3]
        assert abs(t0 - g["s%d_vals" % k][0]) < 1e-12
        for which in range(19):
            ref = g["s%d_arr%d" % (k, which)]
            got = grid.array(which)
            if which in (7, 11, 15, 6):
                # time-derivative slots the reference never writes hold
                # uninitialised memory; compare the written slots only.
                nslot = got.size // 4
                ts_ = g["s%d_dims" % k][3]
                slots = [1, 2] if ts_ == 0 else [1, 2] + [(s + 2) % 4 for s in range(1, ts_ + 1)]
                for s in set(slots):
                    a, b = got[s * nslot:(s + 1) * nslot], ref[s * nslot:(s + 1) * nslot]
                    assert norm_rel_err(a, b) < 1e-11, (k, which, s)
            else:
                assert norm_rel_err(got, ref) < 1e-11, (k, which)
        qt = float(np.ravel(g["s%d_query_t" % k])[0])
        qx, qy, qz = g["query_x"], g["query_y"], g["query_z"]
        q = grid.query(qx, qy, np.maximum(-cfg["depth"], qz), np.full_like(qx, qt))
        kin = grid.query(qx, qy, qz, np.full_like(qx, qt))
        assert norm_rel_err(kin, g["s%d_kin" % k]) < 1e-11
        for c, name in ((1, "VeloX"), (2, "VeloY"), (3, "VeloZ")):
            assert norm_rel_err(q[:, c], g["s%d_api_%s" % (k, name)]) < 1e-11
        e = grid.query(qx, qy, np.zeros_like(qx), np.full_like(qx, qt))[:, 0]
        assert norm_rel_err(e * r, g["s%d_api_SurfElev" % k]) < 1e-11


def test_unit_known_answers():
    """unittests/irregular_tests.cpp:46-76: a 3-component first-order sea with
    zero phases sums to eta(0,0,0) = 6; normalize gives 1, then amplify 3 gives 3."""
    import math
    PI = 3.1415926535897
    base = {"omega": [2 * PI / 10., 2 * PI / 5., 2 * PI / 4.], "A": [3.0, 2.0, 1.0],
            "phase": [0.0, 0.0, 0.0], "theta": [PI / 8., 0.0, 0.0]}
    base["k"] = [w * w / 9.81 for w in base["omega"]]
    cfg = oracle.waveinput.default_config()
    cfg.update(base)
    cfg.update({"depth": 300.0, "mtheta": 10.0, "order": 1, "wavetype": 1,
                "ramptime": [0.0] * 3, "starttime": [-1e-12] * 3, "duration": [1e12] * 3})
    assert oracle.Sea(cfg).fields(0.0, 0.0, 0.0, 0.0)[0, 0] == 6.0
    cfg["normalize"] = True
    cfg["ampl"] = 1.0
    oracle.waveinput.normalize_data(cfg)
    assert math.isclose(oracle.Sea(cfg).fields(0.0, 0.0, 0.0, 0.0)[0, 0], 1.0, rel_tol=1e-15)
    cfg["ampl"] = 3.0
    oracle.waveinput.normalize_data(cfg)
    assert math.isclose(oracle.Sea(cfg).fields(0.0, 0.0, 0.0, 0.0)[0, 0], 3.0, rel_tol=1e-15)
