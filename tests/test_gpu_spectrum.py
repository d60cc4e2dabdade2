"""GPU sea-state generator (cfdwm_spectrum_components) against its host
restatement (seastate.irregular_components with the library's SplitMix64
phases): omega, A, k and theta to 1e-12 relative, the phases bit for bit, and
a generated sea initialises the library."""
import math
import os

import numpy as np
import pytest

import cfdwavemaker_gb300 as cw
from cfdwavemaker_gb300 import seastate as ss

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from cfdwavemaker_gb300 import build
    build.build()
    return cw.load()


@pytest.mark.parametrize("args", [
    (6.0, 12.0, 2.0, 64, 0.25, 1.6, 100.0, 2024, 16, 10.0),
    (2.0, 7.0, 3.3, 128, 0.3, 2.0, 50.0, 12345, 1, 10.0),
    (4.0, 9.0, 1.0, 1, 0.6, 0.6, 30.0, 7, 3, 4.0),
])
def test_spectrum_matches_host(lib, args):
    hs, tp, gam, nf, w0, w1, h, seed, nd, s = args
    got = cw.spectrum_components(hs, tp, gam, nf, w0, w1, h, seed, ndir=nd, spreading_s=s)
    ref = ss.irregular_components(hs, tp, gam, nf, w0, w1, h, seed, ndir=nd, spreading_s=s, phase_rng="splitmix")
    for key in ("omega", "A", "k", "theta"):
        a, b = got[key], np.asarray(ref[key], dtype=np.float64)
        assert a.shape == b.shape, key
        den = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) <= 1e-12 * den, (key, np.max(np.abs(a - b)) / den)
    np.testing.assert_array_equal(got["phase"], ref["phase"])
    if nf > 1:
        assert abs(4.0 * math.sqrt(0.5 * np.sum(got["A"] ** 2)) - hs) < 1e-9


def test_generated_sea_initialises(lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    comps = cw.spectrum_components(3.0, 9.0, 2.5, 24, 0.4, 1.5, 40.0, 5, ndir=3, spreading_s=6.0)
    wm = cw.CFDwavemaker()
    assert wm.initialize_text(ss.write_irregular(None, comps, 40.0, extrap=2)) == 0, cw.last_error()
    eta = wm.surface_elevation_batch(np.array([0.0, 10.0]), np.array([0.0, 5.0]), np.array([1.0, 2.0]))
    assert np.all(np.isfinite(eta)) and np.max(np.abs(eta)) > 0
    wm.cleanup()


def test_spectrum_bad_parameters(lib):
    p = np.array([3.0, -1.0, 2.0, 0.4, 1.5, 40.0, 6.0, 1.5, 9.81])
    out = np.zeros(5 * 10)
    assert lib.cfdwm_spectrum_components(p.ctypes.data_as(cw._dp), 10, 1, 1, out.ctypes.data) == -3
