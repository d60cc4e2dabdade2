"""The allocation-free entry point, cfdwm_irregular_fields_noalloc.

It serves host codes that cannot let the library allocate device memory
while they run (solvers that reserve all device memory for their own pool,
or run under a fixed device-memory budget).  Its workspace is one fixed
device array shared by all calls, so the test checks two calls in a row on
different points against the allocating entry point, cfdwm_irregular_fields,
within the parity tolerance of the other GPU tests, and that an oversize
batch is refused.  The file name sorts last so that a run that stops at the
first failure has already run every other test; the test sets up its own
model, so it also passes alone in a fresh process.
"""
import os

import numpy as np
import pytest

from conftest import norm_rel_err

import cfdwavemaker_gb300 as cw

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the parity tolerance of tests/test_gpu_parity.py


def test_noalloc_matches_allocating_entry_point(tmp_path):
    torch = pytest.importorskip("torch")
    from cfdwavemaker_gb300 import build, seastate as ss
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        wm = cw.CFDwavemaker()
        comps = ss.irregular_components(4.0, 10.0, 3.3, 96, 0.3, 2.0, 50.0, 41, ndir=2, spreading_s=8.0)
        assert wm.initialize_text(ss.write_irregular(None, comps, 50.0, extrap=2)) == 0, cw.last_error()
        lib = wm.lib
        rng = np.random.default_rng(11)
        for call in range(2):
            n = 3000 + 517 * call
            pts = [rng.uniform(-100, 500, n), rng.uniform(-80, 80, n), rng.uniform(-50, 4, n),
                   rng.uniform(0, 60, n)]
            ref = wm.irregular_fields(*pts)                      # allocating entry point
            dev = [torch.tensor(a, device="cuda:0", dtype=torch.float64) for a in pts]
            out = torch.full((5, n), np.nan, device="cuda:0", dtype=torch.float64)
            torch.cuda.synchronize()
            rc = lib.cfdwm_irregular_fields_noalloc(*[cw._ptr(a) for a in dev], n, 31, cw._ptr(out))
            assert rc == 0, cw.last_error()
            got = out.cpu().numpy()
            for q in range(5):
                assert norm_rel_err(got[q], ref[q]) <= TOL, (call, q, norm_rel_err(got[q], ref[q]))
        # a batch beyond the fixed workspace is refused with a clear message
        big = 1 << 22
        dbig = torch.zeros(big, device="cuda:0", dtype=torch.float64)
        obig = torch.zeros((5, big), device="cuda:0", dtype=torch.float64)
        p = cw._ptr(dbig)
        assert lib.cfdwm_irregular_fields_noalloc(p, p, p, p, big, 31, cw._ptr(obig)) == -8
        assert "workspace" in cw.last_error()
        # host arrays are refused (the call cannot stage them without allocating)
        h = np.zeros(4)
        assert lib.cfdwm_irregular_fields_noalloc(cw._ptr(h), cw._ptr(h), cw._ptr(h), cw._ptr(h), 4, 31,
                                                  cw._ptr(np.zeros(20))) == -3
        wm.cleanup()
    finally:
        os.chdir(cwd)
