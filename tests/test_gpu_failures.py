"""Failure statuses and host-side helpers of a loaded model, against what the
reference itself did on the same inputs (fixtures recorded from it by
tests/golden/make_golden.py).

* Fenton set-ups the Newton iteration does not solve (FentonStream.cpp:141-239):
  - a wave near the highest one: the reference warns that the iteration did
    not fully converge (:208-209) and serves the iterate; here
    wave_Initialize returns 0, cfdwm_regular_status() is 3 and the iterate
    matches the reference's;
  - a wave beyond the highest one: the reference warns and serves NaN
    coefficients; here the solve's status word is 4 and wave_Initialize
    returns -7 (the model is not loaded);
  - a steep deep-water wave whose Jacobian turns singular: the reference
    throws (:200-201) and the process ends; here the status word is 2 and
    wave_Initialize returns -7.
  Every loop of the device solve is capped, so none of these can hang.
* wave_mean_period, wave_phase_speed, wave_mean_length (opt 1 and 2) and
  wave_water_depth of two irregular seas (Irregular.cpp:1336-1437).
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("fail"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


def test_fenton_not_converged_is_served_with_the_warning(wm, capfd):
    g = load_golden("fenton_failures")
    assert bool(g["nonconv_exit_ok"]) and bool(g["nonconv_warned"])
    assert wm.initialize_text(str(g["nonconv_waveinput"])) == 0, cw.last_error()
    assert wm.lib.cfdwm_regular_status() == 3
    assert "did not fully converge" in capfd.readouterr().err
    ref = g["nonconv_solution"]
    got = np.zeros(ref.size)
    assert wm.lib.cfdwm_regular_solution(cw._ptr(got), ref.size) == ref.size
    assert np.all(np.isfinite(got))
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("tag,status", [("nan", 4), ("singular", 2)])
def test_fenton_failure_returns_minus_seven(wm, tag, status):
    g = load_golden("fenton_failures")
    if tag == "nan":
        assert bool(g["nan_exit_ok"]) and not np.any(np.isfinite(g["nan_solution"]))
    else:
        assert not bool(g["singular_exit_ok"]) and bool(g["singular_singular"])
    assert wm.initialize_text(str(g[tag + "_waveinput"])) == -7
    assert wm.lib.cfdwm_regular_status() == status
    msg = cw.last_error()
    assert ("singular" in msg) if status == 2 else ("finite" in msg), msg
    assert wm.lib.CFDwavemaker_is_initialized() == 0
    assert wm.lib.wave_VeloX(0.0, 0.0, -1.0, 0.0) == 0.0
    # the library stays usable: a good wave loads afterwards
    from cfdwavemaker_gb300 import seastate as ss
    assert wm.initialize_text(ss.write_regular(None, "stream", 8.0, 20.0, period=12.0, order=24)) == 0
    assert wm.lib.cfdwm_regular_status() == 0


@pytest.mark.parametrize("case", ["helpers_config1", "helpers_t005"])
def test_spectral_helpers_match_reference(wm, case):
    g = load_golden(case)
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    lib = wm.lib
    for name in ("wave_mean_period", "wave_phase_speed", "wave_mean_length"):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_int]
    lib.wave_water_depth.restype = C.c_double
    got = [lib.wave_mean_period(1), lib.wave_mean_period(2), lib.wave_phase_speed(1), lib.wave_phase_speed(2),
           lib.wave_mean_length(1), lib.wave_mean_length(2), lib.wave_water_depth()]
    np.testing.assert_allclose(got, g["helpers"], rtol=1e-13, atol=0)
    assert lib.wave_mean_period(3) == 0.0
