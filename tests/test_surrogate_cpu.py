"""CPU checks of the learned s-grid update's host side: the FP64 oracle's
network gradient against finite differences, its BF16 rounding, and the
committed weight file's header."""
import os

import numpy as np
import pytest

from oracle import surrogate_ref as sr


def _params(nl, seed):
    ch, off_w, off_b, n = sr.layout(nl)
    rng = np.random.default_rng(seed)
    p = np.zeros(n)
    for l in range(4):
        m = ch[l + 1] * ch[l] * 9
        p[off_w[l]:off_w[l] + m] = rng.normal(0, np.sqrt(2.0 / (9 * ch[l])), m)
        p[off_b[l]:off_b[l] + ch[l + 1]] = rng.normal(0, 0.1, ch[l + 1])
    return p


def test_layout_sizes():
    ch, off_w, off_b, n = sr.layout(16)
    assert ch == [128, 32, 32, 32, 49]
    assert n == 128 * 32 * 9 + 2 * 32 * 32 * 9 + 32 * 49 * 9 + 32 * 3 + 49


def test_oracle_gradient_matches_finite_differences():
    nl = 1
    p = _params(nl, 1)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 8 * nl, 11, 12))
    t = rng.normal(size=(2, 1 + 3 * nl, 3, 4))
    loss, g = sr.loss_grad(p, nl, x, t, rounded=False)
    idx = rng.choice(p.size, 40, replace=False)
    h = 1e-6
    for e in idx:
        pp, pm = p.copy(), p.copy()
        pp[e] += h
        pm[e] -= h
        fd = (sr.loss_grad(pp, nl, x, t, rounded=False)[0] - sr.loss_grad(pm, nl, x, t, rounded=False)[0]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-6 * max(1.0, abs(fd)), (e, fd, g[e])


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.140625, 1e-3], np.float32)
    r = sr.bf16_round(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even
    assert r[2] == 1.0 + 2 ** -7            # above the tie rounds up
    assert r[3] == -3.140625
    assert abs(r[4] - 1e-3) <= 2 ** -9 * 1e-3


def test_committed_weights_header():
    from cfdwavemaker_gb300 import surrogate as S
    if not os.path.exists(S.WEIGHTS):
        pytest.skip("no trained weights committed")
    raw = open(S.WEIGHTS, "rb").read()
    assert raw[:8] == b"CFDWMSR1"
    nl, _ = np.frombuffer(raw[8:16], np.int32)
    n = int(np.frombuffer(raw[16:24], np.int64)[0])
    assert nl == 16 and n == sr.layout(16)[3]
    w = np.frombuffer(raw[24:], np.float32)
    assert w.size == n and np.all(np.isfinite(w))


def test_oracle_features_per_column():
    # each column's channels depend on that column alone
    from cfdwavemaker_gb300 import surrogate as S
    import oracle
    p = {"hs": 4.0, "tp": 9.0, "gamma": 2.0, "s": 6.0, "mtheta": 30.0, "seed": 3, "nfreq": 8, "ndir": 3}
    cfg = oracle.waveinput.read_text(S.sea_text(p, 6, 5, 3, 50.0, 20.0, 1.0, t0=2.0))
    x = np.array([50.0, 61.5, 70.25])
    y = np.array([20.0, 33.0, 24.5])
    f_all, b_all, e_all = sr.features_columns(cfg, x, y, 4.2)
    assert f_all.shape == (3, 8 * cfg["lsgrid"]["nl"])
    for j in range(3):
        f1, b1, e1 = sr.features_columns(cfg, x[j:j + 1], y[j:j + 1], 4.2)
        np.testing.assert_array_equal(f1[0], f_all[j])
        np.testing.assert_array_equal(b1[0], b_all[j])
        assert e1[0] == e_all[j]
