"""GPU checks of the .vtu export of the s-grid ring ([lsgrid2vtk],
lsgrid_spline.cpp:1200-1403) against the files the unmodified reference wrote
(tests/golden/sgrid_vtu*.npz): the file the library writes itself after the
initial fill and after a ring update, the export of the slot after the base
slot (cfdwm_sgrid_write_vtu and wave_Cleanup), for both column forms.  Markup
and cells must be identical, velocities within normwise 1e-5 per component,
node coordinates within 2e-4 (printed with 4 decimals)."""
import pytest

from conftest import load_golden
from vtu_text import compare_vtu

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wm():
    from cfdwavemaker_gb300 import build
    build.build()
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()


@pytest.mark.parametrize("method", [1, 0])
@pytest.mark.parametrize("case", ["sgrid_vtu", "sgrid_vtu_flat"])
def test_vtu_files_match_reference(wm, case, method, tmp_path, monkeypatch):
    g = load_golden(case)
    monkeypatch.chdir(tmp_path)
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    auto0 = tmp_path / "vtk" / "kin00000.vtu"
    assert auto0.exists()
    if method == 1:
        compare_vtu(auto0.read_text(), str(g["s0_vtu"]))
    else:
        wm.sgrid_method(0)        # refills the ring with the plain form; no file of its own
        p = tmp_path / "m0.vtu"
        assert wm.lib.cfdwm_sgrid_write_vtu(str(p).encode(), 0) == 0
        compare_vtu(p.read_text(), str(g["s0_vtu"]))
    p = tmp_path / "last0.vtu"
    assert wm.lib.cfdwm_sgrid_write_vtu(str(p).encode(), 1) == 0
    compare_vtu(p.read_text(), str(g["s0_vtu_last"]))
    wm.force_update(1.2)
    auto1 = tmp_path / "vtk" / "kin00001.vtu"
    compare_vtu(auto1.read_text(), str(g["s1_vtu"]))
    # at cleanup the slot after the base slot, as the reference's destructor
    wm.cleanup()
    compare_vtu(auto1.read_text(), str(g["s1_vtu_last"]))


def test_vtu_write_errors(wm, tmp_path, monkeypatch):
    g = load_golden("sgrid_vtu")
    monkeypatch.chdir(tmp_path)
    assert wm.initialize_text(str(g["waveinput"])) == 0, cw.last_error()
    assert wm.lib.cfdwm_sgrid_write_vtu(str(tmp_path / "no" / "such" / "dir.vtu").encode(), 0) == -5
    assert wm.lib.cfdwm_sgrid_write_vtu(None, 0) == -3
