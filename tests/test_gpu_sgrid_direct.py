"""The s-grid spline against the direct point evaluation of the same sea: the
reference's own grid-versus-direct unit test (unittests/lsgrid_tests.cpp:
61-123), re-targeted from its legacy lsGrid class to the s-grid ring it
became (lsGridSpline), on the sea of that test.

The sea: three long-crested components of periods 10, 5 and 4 s, deep-water
wavenumbers w^2 / g, amplitudes 3.1, 2.1 and 1.1 m, zero phases, directions
pi/8, 0, 0 with mtheta 10 degrees, depth 300 m, second order
(lsgrid_tests.cpp:13-48), plus one component of zero amplitude that lifts the
pair cache's sum-frequency filter (see _comps): the legacy grid of that test
called the point API itself, the s-grid ring sums the pair cache.  At a grid column and at a ring slot's time the
spline passes through the nodes, so there the grid must give what the point
API gives (wave type 1, the same waveinput.dat without the [lsgrid]
section):

* the surface elevation: the reference test asks EXPECT_DOUBLE_EQ; the ring
  stores FP32, so here 1e-6 normwise;
* u, v, w at the surface and at the seabed: 1e-5 absolute (the test's bar);
* u, v, w at z = -10 m, between levels: 1e-1 absolute (the test's bar).

Both column forms of the ring are checked, at several columns and at the two
slot times a query reads after initialisation.
"""
import math
import os

import numpy as np
import pytest

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu


def _comps():
    # the test's three components, and a fourth of zero amplitude at 2.5 times
    # the largest wavenumber: the pair cache that the grid update uses drops
    # sum-frequency pairs with k_i + k_m above the largest wavenumber of the
    # sea (Irregular.cpp:833-835, 903), the point API's u2/v2/w2 do not
    # (Irregular.cpp:642), so the extra component lifts that filter and both
    # paths sum the same terms; with zero amplitude it adds nothing itself
    om = np.array([2 * math.pi / 10, 2 * math.pi / 5, 2 * math.pi / 4])
    k = om ** 2 / 9.81
    k4 = 2.5 * k[-1]
    om4 = math.sqrt(9.81 * k4)
    return {"omega": np.append(om, om4), "A": np.array([3.1, 2.1, 1.1, 0.0]), "k": np.append(k, k4),
            "phase": np.zeros(4), "theta": np.array([math.pi / 8, 0.0, 0.0, 0.0])}


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("direct"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


@pytest.mark.parametrize("method", [0, 1])
def test_spline_matches_direct_at_nodes(wm, method):
    from cfdwavemaker_gb300 import seastate as ss
    comps = _comps()
    t0, dt = 4.0, 0.5
    grid = {"bounds": (-30.0, 30.0, -20.0, 20.0), "nx": 7, "ny": 5, "nl": 20, "t0": t0, "dt": dt,
            "stretch": (0.7, 1.5)}
    direct_txt = ss.write_irregular(None, comps, 300.0, extrap=2, mtheta=10.0)
    grid_txt = ss.write_irregular(None, comps, 300.0, extrap=2, mtheta=10.0, lsgrid=grid)
    # columns of the grid (nodes at x = -30 + 10 i, y = -20 + 10 j) and the
    # times of the two slots a query reads after initialisation, t0 and t0 + dt
    xs = np.array([0.0, -30.0, 10.0, 30.0, 20.0])
    ys = np.array([0.0, -20.0, 10.0, 0.0, 20.0])
    ts = np.array([t0, t0 + dt])
    X, T = np.meshgrid(xs, ts, indexing="ij")
    Y, _ = np.meshgrid(ys, ts, indexing="ij")
    x, y, t = X.ravel(), Y.ravel(), T.ravel()
    assert wm.initialize_text(direct_txt) == 0, cw.last_error()
    eta_d = wm.surface_elevation_batch(x, y, t)
    zs = {"surface": eta_d, "seabed": np.full(x.size, -300.0), "mid": np.full(x.size, -10.0)}
    vel_d = {k: np.stack(wm.velocity_batch(x, y, z, t)) for k, z in zs.items()}
    assert wm.initialize_text(grid_txt) == 0, cw.last_error()
    wm.sgrid_method(method)
    eta_g = wm.surface_elevation_batch(x, y, t)
    err = np.max(np.abs(eta_g - eta_d)) / np.max(np.abs(eta_d))
    print("method %d eta normwise %.3e" % (method, err))
    assert err <= 1e-6, err
    for key, bar in (("surface", 1e-5), ("seabed", 1e-5), ("mid", 1e-1)):
        z = eta_g if key == "surface" else zs[key]
        vel_g = np.stack(wm.velocity_batch(x, y, z, t))
        dev = np.max(np.abs(vel_g - vel_d[key]))
        print("method %d %s max |u_grid - u_direct| %.3e" % (method, key, dev))
        assert dev <= bar, (key, dev)
