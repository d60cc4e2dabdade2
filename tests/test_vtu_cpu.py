"""CPU checks of the .vtu export of the s-grid ring ([lsgrid2vtk],
lsgrid_spline.cpp:1200-1403):

* the oracle's restatement of export_vtu writes the reference's own files
  byte for byte (the files the unmodified reference wrote at init and after an
  update, and its export of the slot after the base slot);
* the comparison helper the GPU tests use accepts them and rejects a change;
* the product's parser accepts the section for an s-grid and refuses it
  otherwise, as the reference does (CFDwavemaker.cpp:1205-1213).
"""
import os

import pytest

from conftest import golden_cfg, load_golden
from vtu_text import compare_vtu

import cfdwavemaker_gb300 as cw
import oracle


@pytest.mark.parametrize("case", ["sgrid_vtu", "sgrid_vtu_flat"])
def test_oracle_export_is_the_reference_file(case, tmp_path):
    g = load_golden(case)
    cfg = golden_cfg(g)
    og = oracle.Sgrid(cfg, oracle.Sea(cfg))
    for k, upd in enumerate([None, 1.2]):
        if upd is not None:
            og.force_update(upd)
        for key, last in (("vtu", False), ("vtu_last", True)):
            p = tmp_path / ("%d_%s.vtu" % (k, key))
            og.export_vtu(p, last)
            assert p.read_text() == str(g["s%d_%s" % (k, key)]), (k, key)


def test_compare_helper_detects_changes():
    g = load_golden("sgrid_vtu")
    ref = str(g["s0_vtu"])
    compare_vtu(ref, ref)
    lines = ref.split("\n")
    i = next(q for q, ln in enumerate(lines) if ln.count(" ") == 2 and ln[:1] in "-0123456789")
    bad = list(lines)
    bad[i] = " ".join("%g" % (float(v) * 1.01 + 0.01) for v in bad[i].split())
    with pytest.raises(AssertionError):
        compare_vtu("\n".join(bad), ref)


def test_parser_lsgrid2vtk_section():
    g = load_golden("sgrid_vtu")
    text = str(g["waveinput"])
    assert "[lsgrid2vtk]" in text
    scal, _ = cw.parse_text(text)
    assert int(scal[0]) == 5
    # without the grid the reference stops with an input error
    bad = text.replace("[lsgrid]", "[not lsgrid]")
    with pytest.raises(RuntimeError):
        cw.parse_text(bad)
