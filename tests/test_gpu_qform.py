"""Parity of the precision form (second-order sums at z0 = 0 as quadratic
forms) with the FP64 oracle: eta2 from the pair cache (Irregular.cpp:223-293)
and the uvw2 velocities at z = 0 (Irregular.cpp:975-1102).

Tolerance: normwise relative error max|gpu - ref| / max|ref| per field,
TOL = 1e-5 for the plain FP32 form and the fp16-split tensor-core form.

The bf16-split form keeps 8 + 8 = 16 significant bits per operand: each
operand's split leaves a relative error up to 2^-17 and the dropped lo x lo
product is up to 2^-16 of the product, so every one of the 2N-term dot
products carries an error of about 2^-16 of its terms' scale.  Over random
phases the outputs and these errors are both sums of many independent terms of
the same coefficients, so the normwise error settles near 2^-16 = 1.5e-5 at
any N: above the 1e-5 bar.  Its bar is therefore TOL_BF16 = 2^-15 = 3.05e-5
(two units of the split's rounding), and the fp16 split is the form that meets
1e-5.
"""
import os

import numpy as np
import pytest

from conftest import norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_BF16 = 2.0 ** -15


def _sea(ncomp_freq, ndir, seed):
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(6.0, 12.0, 2.0, ncomp_freq, 0.25, 1.6, 100.0, seed, ndir=ndir,
                                    spreading_s=10.0)
    return ss.write_irregular(None, comps, 100.0, extrap=2)


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _run(wm, torch, txt, n, method, fp16, seed=5):
    assert wm.initialize_text(txt) == 0, cw.last_error()
    assert wm.lib.cfdwm_qform_build(int(fp16)) == 0, cw.last_error()
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1000, n)
    y = rng.uniform(0, 1000, n)
    t = rng.uniform(0, 100, n)
    d = [torch.tensor(a, device="cuda:0", dtype=torch.float64) for a in (x, y, t)]
    out = torch.zeros((n, 4), device="cuda:0", dtype=torch.float32)
    torch.cuda.synchronize()
    rc = wm.lib.cfdwm_qform_eval(*[cw._ptr(a) for a in d], n, method, cw._ptr(out))
    assert rc == 0, cw.last_error()
    return x, y, t, out.cpu().numpy().astype(np.float64)


def _reference(txt, x, y, t):
    cfg = oracle.waveinput.read_text(txt)
    sea = oracle.Sea(cfg)
    eta2 = sea.eta2(x, y, t)
    uvw = sea.uvw2(x, y, np.zeros_like(x), t)
    return np.stack([eta2, uvw[:, 0], uvw[:, 1], uvw[:, 2]], axis=1)


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("qf"))
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


@pytest.mark.parametrize("nf,nd", [(12, 4), (40, 8)])
def test_plain_form(wm, torch, nf, nd):
    txt = _sea(nf, nd, 17)
    x, y, t, got = _run(wm, torch, txt, 333, 0, False)
    ref = _reference(txt, x, y, t)
    for f in range(4):
        assert norm_rel_err(got[:, f], ref[:, f]) <= TOL, (f, norm_rel_err(got[:, f], ref[:, f]))


@pytest.mark.parametrize("nf,nd", [(12, 4), (40, 8)])
def test_tensor_core_fp16_split(wm, torch, nf, nd):
    txt = _sea(nf, nd, 17)
    x, y, t, got = _run(wm, torch, txt, 333, 1, True)
    ref = _reference(txt, x, y, t)
    for f in range(4):
        err = norm_rel_err(got[:, f], ref[:, f])
        print("fp16x3 field", f, "err", err)
        assert err <= TOL, (f, err)


@pytest.mark.parametrize("nf,nd", [(12, 4), (40, 8)])
def test_tensor_core_bf16_split(wm, torch, nf, nd):
    txt = _sea(nf, nd, 17)
    x, y, t, got = _run(wm, torch, txt, 333, 1, False)
    ref = _reference(txt, x, y, t)
    for f in range(4):
        err = norm_rel_err(got[:, f], ref[:, f])
        print("bf16x3 field", f, "err", err)
        assert err <= TOL_BF16, (f, err)


def test_tensor_core_fp16_split_wide(wm, torch):
    """2048 components: long K-loops with both accumulator buffers in turn."""
    txt = _sea(128, 16, 23)
    x, y, t, got = _run(wm, torch, txt, 64, 1, True)
    ref = _reference(txt, x, y, t)
    for f in range(4):
        err = norm_rel_err(got[:, f], ref[:, f])
        print("fp16x3 N=2048 field", f, "err", err)
        assert err <= TOL, (f, err)


@pytest.mark.parametrize("env", [{"CFDWM_QFORM_KSEG": "1"}, {"CFDWM_QFORM_KSEG": "3"},
                                 {"CFDWM_QFORM_TWO_ACC": "1"}])
def test_tensor_core_fp16_accumulation_arrangements(wm, torch, env, monkeypatch):
    """The fp16 split's other accumulation arrangements on 2048 components
    (column tiles of 4 to 32 K blocks of 64): one accumulator over K segments
    of 1 block and of at most 3 blocks (segments of 2 and 3 blocks in one
    tile where its count does not divide by 3), and the second
    accumulator for the cross products over the whole K range; each against
    the plain FP32 form of the same sea and points (which is within a few 1e-7
    of FP64)."""
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    txt = _sea(128, 16, 23)
    _, _, _, got = _run(wm, torch, txt, 256, 1, True)
    _, _, _, plain = _run(wm, torch, txt, 256, 0, True)
    for f in range(4):
        err = norm_rel_err(got[:, f], plain[:, f])
        print(env, "field", f, "err", err)
        assert err <= TOL, (f, err)


@pytest.mark.parametrize("method", [0, 1])
def test_host_arrays(wm, torch, method):
    """Host arrays (pageable NumPy and pinned, and a mix with device arrays)
    give the device-array results: staged through the library's device
    buffers, 70,001 points (more than one 65,536-row chunk)."""
    txt = _sea(12, 4, 31)
    n = 70001
    x, y, t, want = _run(wm, torch, txt, n, method, True, seed=12)
    out = np.zeros((n, 4), dtype=np.float32)
    rc = wm.lib.cfdwm_qform_eval(cw._ptr(x), cw._ptr(y), cw._ptr(t), n, method, cw._ptr(out))
    assert rc == 0, cw.last_error()
    scale = np.max(np.abs(want), axis=0)
    assert np.all(np.max(np.abs(out - want), axis=0) <= 1e-6 * scale)
    dx = torch.tensor(x, device="cuda:0", dtype=torch.float64)
    py = torch.from_numpy(y).pin_memory()
    pout = torch.zeros((n, 4), dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    rc = wm.lib.cfdwm_qform_eval(cw._ptr(dx), cw._ptr(py), cw._ptr(t), n, method, cw._ptr(pout))
    assert rc == 0, cw.last_error()
    assert np.all(np.max(np.abs(pout.numpy() - want), axis=0) <= 1e-6 * scale)
    assert wm.lib.cfdwm_qform_eval(None, cw._ptr(y), cw._ptr(t), n, method, cw._ptr(out)) != 0


def test_tensor_core_several_chunks(wm, torch):
    """More than one 65,536-row chunk: the operands of the next chunk are
    prepared on a second stream while the GEMM of the previous one runs."""
    txt = _sea(12, 4, 29)
    n = 140000
    x, y, t, got = _run(wm, torch, txt, n, 1, True, seed=8)
    rng = np.random.default_rng(2)
    rows = np.concatenate([rng.choice(65536, 60, replace=False), 65536 + rng.choice(65536, 60, replace=False),
                           131072 + rng.choice(n - 131072, 60, replace=False)])
    ref = _reference(txt, x[rows], y[rows], t[rows])
    for f in range(4):
        err = norm_rel_err(got[rows, f], ref[:, f])
        assert err <= TOL, (f, err)


def _rms(a, b):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return float(np.sqrt(np.mean(d * d)) / np.max(np.abs(b)))


@pytest.mark.parametrize("fp16", [True, False])
def test_full_size_sea(wm, torch, fp16):
    """The benchmark's sea at full size: 256 frequencies x 16 directions = 4096
    components (8.4e6 pair-cache pairs), 131,072 rows in two chunks.

    Two references: the GPU plain FP32 form on every row (it is itself pinned
    to the oracle below), and the FP64 oracle on 256 rows spread evenly over
    both chunks.  Per field the normwise max and RMS errors are printed; the
    max is held to TOL (fp16 split) or TOL_BF16 (bf16 split)."""
    txt = _sea(256, 16, 2024)
    n = 131072
    x, y, t, plain = _run(wm, torch, txt, n, 0, fp16, seed=13)
    _, _, _, got = _run(wm, torch, txt, n, 1, fp16, seed=13)
    rows = np.unique(np.linspace(0, n - 1, 256).round().astype(np.int64))
    assert (rows < 65536).sum() >= 100 and (rows >= 65536).sum() >= 100
    ref = _reference(txt, x[rows], y[rows], t[rows])
    bar = TOL if fp16 else TOL_BF16
    for f in range(4):
        e_plain = norm_rel_err(plain[rows, f], ref[:, f])
        e_fp64 = norm_rel_err(got[rows, f], ref[:, f])
        e_all = norm_rel_err(got[:, f], plain[:, f])
        print("%s N=4096 field %d: vs FP64 (256 rows) max %.3e rms %.3e; vs plain (all %d rows) max %.3e "
              "rms %.3e; plain vs FP64 %.3e" % ("fp16x3" if fp16 else "bf16x3", f, e_fp64,
                                                _rms(got[rows, f], ref[:, f]), n, e_all,
                                                _rms(got[:, f], plain[:, f]), e_plain))
        assert e_plain <= 1e-6, (f, e_plain)
        assert e_fp64 <= bar, (f, e_fp64)
        assert e_all <= bar, (f, e_all)


def test_tensor_core_fp16_split_component_ramps(wm, torch):
    """Individual component ramps still rising at the evaluation times: the
    ramp enters the operands per (row, component)."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(6.0, 12.0, 2.0, 24, 0.25, 1.6, 100.0, 31, ndir=4, spreading_s=10.0)
    n = comps["omega"].size
    rng = np.random.default_rng(6)
    rcols = [rng.uniform(20.0, 120.0, n), rng.uniform(-5.0, 10.0, n), rng.uniform(300.0, 600.0, n)]
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, ramp_columns=rcols)
    x, y, t, got = _run(wm, torch, txt, 3000, 1, True, seed=9)
    ref = _reference(txt, x, y, t)
    for f in range(4):
        err = norm_rel_err(got[:, f], ref[:, f])
        assert err <= TOL, (f, err)


@pytest.mark.parametrize("fp16", [True, False])
@pytest.mark.parametrize("n", [1, 333, 1000, 70001])
def test_tensor_core_pair_and_single_forms_agree(wm, torch, fp16, n):
    """The GEMM on CTA pairs (cta_group::2, M = 256) and on single CTAs
    (M = 128) gives the same sums: every 128-row block runs the same K
    sequence, and only the order of the per-tile atomic adds into each output
    (not fixed even between two runs) differs, so the bar is a few FP32
    roundings, 1e-6 normwise.  Row counts of 1, 3, 8 and 547 row blocks (two
    chunks) leave a row block past the last row in the last pair."""
    txt = _sea(40, 8, 37)
    outs = {}
    old = os.environ.get("CFDWM_TC_PAIR")
    try:
        for pr in ("0", "1"):
            os.environ["CFDWM_TC_PAIR"] = pr
            outs[pr] = _run(wm, torch, txt, n, 1, fp16, seed=41)
    finally:
        if old is None:
            os.environ.pop("CFDWM_TC_PAIR", None)
        else:
            os.environ["CFDWM_TC_PAIR"] = old
    single, pair = outs["0"][3], outs["1"][3]
    assert np.all(np.isfinite(pair))
    for f in range(4):
        err = norm_rel_err(pair[:, f], single[:, f])
        assert err <= 1e-6, (f, err)
    if n == 1000:
        x, y, t, _ = outs["1"]
        ref = _reference(txt, x, y, t)
        for f in range(4):
            assert norm_rel_err(pair[:, f], ref[:, f]) <= (TOL if fp16 else TOL_BF16)
