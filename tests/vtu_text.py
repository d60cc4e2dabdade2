"""Comparison of .vtu texts (lsGridSpline::export_vtu layout) for the tests:
the markup lines must be identical and the numeric lines agree within a
tolerance (the GPU ring is FP32, the reference's FP64)."""
import numpy as np


def split_vtu(text):
    """(markup lines, velocity [n,3], points [n,3], cell lines) of a .vtu text."""
    markup, vel, pts, cells = [], [], [], []
    sect = None
    for ln in text.split("\n"):
        s = ln.strip()
        if s.startswith("<"):
            markup.append(ln)
            if s.startswith("</DataArray"):
                sect = None
            elif 'Name="Velocity"' in s:
                sect = "vel"
            elif s.startswith('<DataArray type="Float64" NumberOfComponents="3"'):
                sect = "pts"
            elif s.startswith('<DataArray type="Int64"') or s.startswith('<DataArray type="UInt8"'):
                sect = "cells"
            continue
        if sect == "vel":
            vel.append([float(v) for v in s.split()])
        elif sect == "pts":
            pts.append([float(v) for v in s.split()])
        elif sect == "cells":
            cells.append(s)
        else:
            markup.append(ln)          # the time value of FieldData, the final newline
    return markup, np.array(vel), np.array(pts), cells


def compare_vtu(got, ref, vel_tol=1e-5, pts_atol=2e-4):
    """Markup and cells identical, velocities normwise within vel_tol per
    component, point coordinates within pts_atol (they are printed with 4
    decimals)."""
    mg, vg, pg, cg = split_vtu(got)
    mr, vr, pr, cr = split_vtu(ref)
    assert mg == mr
    assert cg == cr
    assert vg.shape == vr.shape and pg.shape == pr.shape
    for c in range(3):
        den = max(np.max(np.abs(vr[:, c])), 1e-30)
        assert np.max(np.abs(vg[:, c] - vr[:, c])) / den <= vel_tol, c
    assert np.max(np.abs(pg - pr)) <= pts_atol
