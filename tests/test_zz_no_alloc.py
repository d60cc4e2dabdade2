"""The allocation-free entry point, cfdwm_irregular_fields_noalloc.

It serves host codes that cannot let the library allocate device memory
while they run (solvers that reserve all device memory for their own pool,
or run under a fixed device-memory budget).  Its workspace is one fixed
device array shared by all calls, so the tests check two calls in a row on
different points against the allocating entry point, cfdwm_irregular_fields,
and against the FP64 oracle, within the parity tolerance of the other GPU
tests; the same for the Smit s-coordinate theory; that a call near the
workspace limit leaves the device's free memory unchanged; and that
oversize batches, host arrays and arrays of another device are refused.  The
file name sorts last so that a run that stops at the first failure has
already run every other test; each test sets up its own model, so they also
pass alone in a fresh process.
"""
import os

import numpy as np
import pytest

from conftest import norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the parity tolerance of tests/test_gpu_parity.py


@pytest.fixture
def model(tmp_path):
    torch = pytest.importorskip("torch")
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path)
    wm = cw.CFDwavemaker()
    try:
        yield wm, torch
    finally:
        wm.cleanup()
        os.chdir(cwd)


def _sea_text(smit=False):
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(4.0, 10.0, 3.3, 96, 0.3, 2.0, 50.0, 41, ndir=2, spreading_s=8.0)
    return ss.write_irregular(None, comps, 50.0, extrap=2, vertical_theory="smit" if smit else None)


def _noalloc(wm, torch, pts, mask=31):
    n = pts[0].size
    dev = [torch.tensor(a, device="cuda:0", dtype=torch.float64) for a in pts]
    out = torch.full((5, n), np.nan, device="cuda:0", dtype=torch.float64)
    torch.cuda.synchronize()
    rc = wm.lib.cfdwm_irregular_fields_noalloc(*[cw._ptr(a) for a in dev], n, mask, cw._ptr(out))
    assert rc == 0, cw.last_error()
    return out.cpu().numpy()


def _oracle(txt, pts, smit):
    cfg = oracle.waveinput.read_text(txt)
    sea = oracle.Sea(cfg)
    ref = sea.fields(*pts).T.copy()            # eta, u, v, w, dp (no ramp, no clamp)
    if smit:
        ref[1:] = sea.smit(*pts).T
    return ref


@pytest.mark.parametrize("smit", [False, True], ids=["sharma_dean", "smit"])
def test_noalloc_matches_allocating_entry_point_and_oracle(model, smit):
    wm, torch = model
    txt = _sea_text(smit)
    assert wm.initialize_text(txt) == 0, cw.last_error()
    rng = np.random.default_rng(11)
    for call in range(2):
        n = 3000 + 517 * call
        pts = [rng.uniform(-100, 500, n), rng.uniform(-80, 80, n), rng.uniform(-50, 4, n), rng.uniform(0, 60, n)]
        ref = wm.irregular_fields(*pts)                      # allocating entry point
        got = _noalloc(wm, torch, pts)
        o64 = _oracle(txt, [a[:400] for a in pts], smit)     # FP64 oracle on the first 400 points
        for q in range(5):
            assert norm_rel_err(got[q], ref[q]) <= TOL, (call, q, norm_rel_err(got[q], ref[q]))
            assert norm_rel_err(got[q, :400], o64[q]) <= TOL, (call, q, norm_rel_err(got[q, :400], o64[q]))


def test_noalloc_allocates_nothing_and_refuses_what_it_cannot_serve(model):
    wm, torch = model
    assert wm.initialize_text(_sea_text()) == 0, cw.last_error()
    lib = wm.lib
    big = 1 << 22
    dbig = torch.zeros(big, device="cuda:0", dtype=torch.float64)
    obig = torch.zeros((5, big), device="cuda:0", dtype=torch.float64)
    p = cw._ptr(dbig)
    # a batch beyond the fixed workspace is refused with a clear message
    assert lib.cfdwm_irregular_fields_noalloc(p, p, p, p, big, 31, cw._ptr(obig)) == -8
    assert "workspace" in cw.last_error()
    # the largest accepted batch (the size check comes before any GPU work)
    lo, hi = 1, big
    while hi - lo > 1:
        mid = (lo + hi) // 2
        rc = lib.cfdwm_irregular_fields_noalloc(p, p, p, p, mid, 1, cw._ptr(obig))
        assert rc in (0, -8), cw.last_error()
        lo, hi = (mid, hi) if rc == 0 else (lo, mid)
    assert lo > 5000, lo
    rng = np.random.default_rng(3)
    pts = [torch.tensor(rng.uniform(*r, lo), device="cuda:0", dtype=torch.float64)
           for r in ((-100, 500), (-80, 80), (-50, 4), (0, 60))]
    out = torch.zeros((5, lo), device="cuda:0", dtype=torch.float64)
    args = [cw._ptr(a) for a in pts] + [lo, 31, cw._ptr(out)]
    assert lib.cfdwm_irregular_fields_noalloc(*args) == 0, cw.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert lib.cfdwm_irregular_fields_noalloc(*args) == 0, cw.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    ref = wm.irregular_fields(*[a.cpu().numpy() for a in pts])
    got = out.cpu().numpy()
    for q in range(5):
        assert norm_rel_err(got[q], ref[q]) <= TOL, (q, norm_rel_err(got[q], ref[q]))
    # host arrays are refused (the call cannot stage them without allocating)
    h = np.zeros(4)
    assert lib.cfdwm_irregular_fields_noalloc(cw._ptr(h), cw._ptr(h), cw._ptr(h), cw._ptr(h), 4, 31,
                                              cw._ptr(np.zeros(20))) == -3
    # pinned host memory is not device memory either
    hp = torch.zeros(8, dtype=torch.float64).pin_memory()
    assert lib.cfdwm_irregular_fields_noalloc(*([cw._ptr(hp)] * 4), 1, 31, cw._ptr(out)) == -3
