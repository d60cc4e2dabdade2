"""GPU checks of the learned s-grid update (cfdwm_surrogate_*), through the
C ABI, against the FP64 oracle (oracle/surrogate_ref.py):

* first-order channels and the U1 / eta1 base: normwise error <= TOL_FEAT;
* network forward: normwise <= TOL_NET; loss and parameter gradient of the
  CUDA backward against the oracle's: loss <= TOL_NET, gradient normwise per
  layer <= TOL_GRAD (FP32 accumulation over up to 32k pixels);
* training on plain-method slots lowers the loss;
* the sampled check falls back to the plain method (the slot then equals a
  full plain fill) and wave_force_update routes through the learned update;
* the committed trained network beats the method without it (first order
  only, i.e. a zero network) on a sea it was not trained on.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle
from oracle import surrogate_ref as sr

pytestmark = pytest.mark.gpu

TOL_FEAT = 1e-5
TOL_NET = 1e-5
TOL_GRAD = 1e-4
NL = 16


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def env(tmp_path_factory, torch):
    from cfdwavemaker_gb300 import build
    build.build()
    cwd = os.getcwd()
    os.chdir(tmp_path_factory.mktemp("surr"))
    wm = cw.CFDwavemaker()
    lib = cw.load()
    yield wm, lib
    wm.cleanup()
    os.chdir(cwd)


def _text(nx, ny, nfreq=24, ndir=6, seed=5, hs=5.0, tp=10.0, dt=1.0, mtheta=20.0, x0=120.0, y0=260.0):
    from cfdwavemaker_gb300 import surrogate as S
    p = {"hs": hs, "tp": tp, "gamma": 2.5, "s": 8.0, "mtheta": mtheta, "seed": seed, "nfreq": nfreq,
         "ndir": ndir}
    return S.sea_text(p, nx, ny, NL, x0, y0, dt, t0=5.0)


def _ok(rc):
    assert rc == 0, (rc, cw.last_error())


@pytest.mark.parametrize("x0,y0", [(120.0, 260.0), (431.0, 77.0)])
def test_features_match_oracle(env, torch, x0, y0):
    # the second case re-initialises a grid of the same shape at another place
    wm, lib = env
    nx, ny = 20, 17
    txt = _text(nx, ny, x0=x0, y0=y0)
    _ok(wm.initialize_text(txt))
    if lib.cfdwm_surrogate_nparams() != sr.layout(NL)[3]:    # none, or one for other levels
        _ok(lib.cfdwm_surrogate_create(NL, 1))
    nxh, nyh = nx + 8, ny + 8
    feat = torch.zeros((8 * NL, nxh * nyh), device="cuda")
    base = torch.zeros((3, nx * ny, NL), device="cuda")
    eta1 = torch.zeros(nx * ny, device="cuda")
    t = 7.3
    _ok(lib.cfdwm_surrogate_features(t, cw._ptr(feat), cw._ptr(base), cw._ptr(eta1)))
    cfg = oracle.waveinput.read_text(txt)
    g = cfg["lsgrid"]
    dx = (g["domain"][1] - g["domain"][0]) / (nx - 1)
    dy = (g["domain"][3] - g["domain"][2]) / (ny - 1)
    rng = np.random.default_rng(3)
    ph = rng.choice(nxh * nyh, 40, replace=False)
    ih, jh = ph // nyh, ph % nyh
    x = g["domain"][0] + dx * (ih - 4)
    y = g["domain"][2] + dy * (jh - 4)
    f_ref, _, _ = sr.features_columns(cfg, x, y, t)
    f_gpu = feat.cpu().numpy()[:, ph].T
    for q in range(8):
        err = norm_rel_err(f_gpu[:, q::8].ravel(), f_ref[:, q::8].ravel())
        assert err <= TOL_FEAT, (q, err)
    pc = rng.choice(nx * ny, 30, replace=False)
    i, j = pc // ny, pc % ny
    _, b_ref, e_ref = sr.features_columns(cfg, g["domain"][0] + dx * i, g["domain"][2] + dy * j, t)
    b_gpu = base.cpu().numpy()[:, pc, :].transpose(1, 0, 2)
    for f in range(3):
        assert norm_rel_err(b_gpu[:, f].ravel(), b_ref[:, f].ravel()) <= TOL_FEAT, f
    assert norm_rel_err(eta1.cpu().numpy()[pc], e_ref) <= TOL_FEAT


def _rand_params(lib, seed):
    n = lib.cfdwm_surrogate_nparams()
    rng = np.random.default_rng(seed)
    ch, off_w, off_b, nn = sr.layout(NL)
    assert n == nn
    p = np.zeros(n, np.float32)
    for l in range(4):
        m = ch[l + 1] * ch[l] * 9
        p[off_w[l]:off_w[l] + m] = rng.normal(0, np.sqrt(2.0 / (9 * ch[l])), m)
        p[off_b[l]:off_b[l] + ch[l + 1]] = rng.normal(0, 0.1, ch[l + 1])
    _ok(lib.cfdwm_surrogate_set_params(p.ctypes.data, n))
    return p


def test_forward_matches_oracle(env, torch):
    wm, lib = env
    _ok(lib.cfdwm_surrogate_create(NL, 2))
    p = _rand_params(lib, 4)
    rng = np.random.default_rng(5)
    x = rng.normal(size=(2, 8 * NL, 15, 41)).astype(np.float32)
    dx = torch.tensor(x, device="cuda")
    dy = torch.zeros((2, 1 + 3 * NL, 7, 33), device="cuda")
    _ok(lib.cfdwm_surrogate_forward(cw._ptr(dx), 2, 15, 41, cw._ptr(dy)))
    ref, _ = sr.forward(p, NL, x.astype(np.float64))
    assert norm_rel_err(dy.cpu().numpy().ravel(), ref.ravel()) <= TOL_NET


def test_backward_matches_oracle(env, torch):
    wm, lib = env
    _ok(lib.cfdwm_surrogate_create(NL, 3))
    p = _rand_params(lib, 6)
    rng = np.random.default_rng(7)
    B, H, W = 2, 18, 44
    x = rng.normal(size=(B, 8 * NL, H, W)).astype(np.float32)
    t = rng.normal(size=(B, 1 + 3 * NL, H - 8, W - 8)).astype(np.float32)
    dx, dt = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    n = lib.cfdwm_surrogate_nparams()
    g = torch.zeros(n, device="cuda")
    loss = C.c_double(0.0)
    _ok(lib.cfdwm_surrogate_loss_grad(cw._ptr(dx), cw._ptr(dt), B, H, W, C.byref(loss), cw._ptr(g)))
    l_ref, g_ref = sr.loss_grad(p, NL, x.astype(np.float64), t.astype(np.float64))
    assert abs(loss.value - l_ref) <= TOL_NET * abs(l_ref)
    ch, off_w, off_b, _ = sr.layout(NL)
    gg = g.cpu().numpy().astype(np.float64)
    for l in range(4):
        sw = slice(off_w[l], off_w[l] + ch[l + 1] * ch[l] * 9)
        sb = slice(off_b[l], off_b[l] + ch[l + 1])
        assert norm_rel_err(gg[sw], g_ref[sw]) <= TOL_GRAD, ("w", l, norm_rel_err(gg[sw], g_ref[sw]))
        assert norm_rel_err(gg[sb], g_ref[sb]) <= TOL_GRAD, ("b", l, norm_rel_err(gg[sb], g_ref[sb]))


def test_training_lowers_loss(env, torch):
    from cfdwavemaker_gb300 import surrogate as S
    tr = S.Trainer(nl=NL, seed=9)
    X, T = tr.generate(3, 21, nx=24, ny=24, per_sea=5, dt=1.5)
    assert torch.isfinite(X).all() and torch.isfinite(T).all()
    l0 = tr.eval_loss(X, T)
    tr.train(X, T, 300, batch=4, lr=2e-3)
    l1 = tr.eval_loss(X, T)
    print("training loss %.4g -> %.4g" % (l0, l1))
    assert l1 < 0.5 * l0


def test_fallback_restores_plain(env, torch):
    wm, lib = env
    _ok(wm.initialize_text(_text(20, 18)))
    _ok(lib.cfdwm_surrogate_create(NL, 11))       # untrained: the check must fail
    fb = C.c_int(0)
    err = (C.c_double * 4)()
    _ok(lib.cfdwm_surrogate_step(1, 1e-9, 16, C.byref(fb), err))
    assert fb.value == 1
    assert max(err) > 1e-9
    e2 = (C.c_double * 4)()
    _ok(lib.cfdwm_surrogate_compare(e2))
    # the slot is the plain method's own (summation order of the tensor-core
    # form's atomics aside)
    assert max(e2) <= 1e-6, list(e2)
    # routed through wave_force_update: every update falls back at this tolerance
    _ok(lib.cfdwm_surrogate_enable(1, 3, 1e-9, 8))
    t0 = C.c_double(0.0)
    _ok(lib.cfdwm_sgrid_state(C.byref(t0), None))
    wm.force_update(t0.value + 6.5)
    st = [C.c_long(0) for _ in range(3)]
    _ok(lib.cfdwm_surrogate_stats(*[C.byref(v) for v in st]))
    steps, fbs, plain = [v.value for v in st]
    assert plain >= 1 and steps >= 1 and fbs == steps, (steps, fbs, plain)
    _ok(lib.cfdwm_surrogate_enable(0, 1, 0.0, 0))


def test_trained_network_gain(env, torch):
    from cfdwavemaker_gb300 import surrogate as S
    wm, lib = env
    if not os.path.exists(S.WEIGHTS):
        pytest.skip("no trained weights committed")
    # a sea outside the training set: the 1024-component short-crested sea of the
    # s-grid workload (Hs 6 m, Tp 12 s), on a 48 x 48 patch
    txt = _text(48, 48, nfreq=64, ndir=16, seed=777, hs=6.0, tp=12.0, dt=0.5, mtheta=0.0)
    errs = {}
    for name in ("net", "zero"):
        _ok(wm.initialize_text(txt))
        _ok(lib.cfdwm_surrogate_load(S.WEIGHTS.encode()))
        if name == "zero":
            n = lib.cfdwm_surrogate_nparams()
            z = np.zeros(n, np.float32)
            _ok(lib.cfdwm_surrogate_set_params(z.ctypes.data, n))
        e = []
        for _ in range(3):
            _ok(lib.cfdwm_surrogate_step(2, 0.0, 0, None, None))
            err = (C.c_double * 4)()
            _ok(lib.cfdwm_surrogate_compare(err))
            e.append(list(err))
        errs[name] = np.max(np.array(e), axis=0)
    print("max errors eta,u,v,w  trained:", errs["net"], " first order only:", errs["zero"])
    assert errs["net"][0] < 0.5 * errs["zero"][0]
    assert errs["net"][1] < 0.5 * errs["zero"][1]
