"""CPU checks of the oracle's dynamic-pressure field on the s-grid ring.

The reference's grid keeps no pressure (lsgrid_spline.cpp:892-897 computes
uvw2's pressure and drops it); the field both the oracle and the CUDA path
hold is, at every node, dp1(z0) + rho uvw2.p(z0) + dp1_dz max(0, z - swl)
with z0 = min(0, z), the convention of the velocities beside it.

* One component: uvw2 has no pairs and keeps every diagonal term, so the
  node pressure equals the irregular sea's point pressure Irregular::dp
  (Irregular.cpp:142-148) at the node -- a check of the field against the
  pinned point API.
* The pressure field leaves the elevation, the velocities and their
  gradients unchanged, and the query's first four outputs too.
"""
import math

import numpy as np

import oracle
from oracle import surrogate_ref as sr
from cfdwavemaker_gb300 import seastate as ss


def _text(comps, depth, nx=10, ny=8, nl=6, t0=3.0, dt=0.8):
    grid = {"bounds": (10.0, 10.0 + (nx - 1) * 7.0, -5.0, -5.0 + (ny - 1) * 6.0), "nx": nx, "ny": ny, "nl": nl,
            "t0": t0, "dt": dt, "stretch": (0.7, 1.5)}
    return ss.write_irregular(None, comps, depth, extrap=2, lsgrid=grid, rho=1025.0)


def test_single_component_node_pressure_is_point_dp():
    depth = 40.0
    om = np.array([0.62])
    comps = {"omega": om, "A": np.array([1.3]), "k": ss.dispersion_k(om, depth), "phase": np.array([0.7]),
             "theta": np.array([0.4])}
    cfg = oracle.waveinput.read_text(_text(comps, depth))
    sea = oracle.Sea(cfg)
    og = oracle.Sgrid(cfg, sea, pressure=True)
    g = cfg["lsgrid"]
    nx, ny, nl = g["nx"], g["ny"], g["nl"]
    dx = (g["domain"][1] - g["domain"][0]) / (nx - 1)
    dy = (g["domain"][3] - g["domain"][2]) / (ny - 1)
    ETA = og.array(0).reshape(4, nx, ny)
    P = og.array(20).reshape(4, nx, ny, nl)
    for slot in range(4):
        t = g["t0"] + (slot - 1) * g["dt"]
        I, J, M = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nl), indexing="ij")
        x = g["domain"][0] + dx * I
        y = g["domain"][2] + dy * J
        z = np.array([sr.sigma_s2cart(g, depth, cfg["swl"], m, e)
                      for m, e in zip(M.ravel(), ETA[slot][I, J].ravel())])
        dp = sea.fields(x.ravel(), y.ravel(), z, np.full(z.size, t), fields=16)[:, 4]
        got = P[slot].ravel()
        assert np.max(np.abs(got - dp)) <= 1e-10 * np.max(np.abs(dp)), slot


def test_pressure_field_leaves_velocities_unchanged():
    comps = ss.irregular_components(3.0, 9.0, 2.0, 6, 0.4, 1.3, 60.0, 11, ndir=3, spreading_s=4.0)
    cfg = oracle.waveinput.read_text(_text(comps, 60.0, nx=7, ny=6, nl=5))
    sea = oracle.Sea(cfg)
    a = oracle.Sgrid(cfg, sea)
    b = oracle.Sgrid(cfg, sea, pressure=True)
    a.update()
    b.update()
    for which in range(19):
        np.testing.assert_array_equal(a.array(which), b.array(which))
    rng = np.random.default_rng(4)
    t0, _ = a.state()
    x = rng.uniform(10.0, 52.0, 50)
    y = rng.uniform(-5.0, 25.0, 50)
    z = rng.uniform(-60.0, 1.0, 50)
    t = rng.uniform(t0, t0 + cfg["lsgrid"]["dt"], 50)
    qa, qb = a.query(x, y, z, t), b.query(x, y, z, t)
    assert qa.shape == (50, 4) and qb.shape == (50, 5)
    np.testing.assert_array_equal(qa, qb[:, :4])
    assert np.all(np.isfinite(qb[:, 4])) and np.max(np.abs(qb[:, 4])) > 0.0
    # gradients exist for the pressure: dt (4 slots), dx, dy, ds (2 slots)
    v = 7 * 6 * 5
    assert [b.array(w).size for w in range(20, 25)] == [4 * v, 4 * v, 2 * v, 2 * v, 2 * v]
    assert math.isfinite(float(np.sum(b.array(21))))
