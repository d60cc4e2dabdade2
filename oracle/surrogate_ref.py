"""FP64 NumPy restatement of the learned s-grid update's arithmetic.

TEST INFRASTRUCTURE ONLY: the tests use it to check the CUDA kernels of
cfdwavemaker_gb300/csrc/surrogate.cu (first-order channels, network forward,
loss and backward).  The product never imports it.

The first-order sums follow the reference's Irregular.cpp:178-198 (eta1),
:394-447 (u1, v1, w1, dp1 profiles) and :1107-1192 (phi1_dxdz/dydz, the
Taylor gradients); the level heights follow lsgrid_spline.cpp:117-122
(sigmaS2cart).  The quadrature channels (phase - pi/2) and the network are
this build's own.
"""
from __future__ import annotations

import math

import numpy as np

SH = 4          # halo columns per side
NQ = 8          # channels per level: u, u~, v, v~, w, w~, p, p~
HID = 32
PI_IRR = 3.1415926535897      # Irregular.h:14 (truncated, as the reference)
SMALL = 1.0e-12


def sea_scales(cfg):
    A = np.asarray(cfg["A"], float)
    a2 = A * A
    s2 = a2.sum()
    sigma = math.sqrt(0.5 * s2) if s2 > 0 else 1.0
    om = float((a2 * np.asarray(cfg["omega"], float)).sum() / s2) if s2 > 0 else 1.0
    km = float((a2 * np.asarray(cfg["k"], float)).sum() / s2) if s2 > 0 else 1.0
    return sigma, om, km


def _freq_ramp(t, rt, ts, du):
    """Irregular::freq_ramp, Irregular.cpp:200-204."""
    down = np.clip(1.0 - ((t - ts - du + rt) / (rt + SMALL)), 0.0, 1.0)
    up = np.clip((t - ts) / (rt + SMALL), 0.0, 1.0)
    return up * down


def sigma_s2cart(grid, depth, swl, m, e):
    """sigmaS2cart (lsgrid_spline.cpp:117-122) at level m, s = m ds."""
    nl = grid["nl"]
    ds = 1.0 / max(1.0, nl - 1.0)
    s = ds * m
    base = max(math.tan(-(s - 1.0) * grid["tan_a"]), 0.0)
    sig = -base ** grid["tan_b"] / math.tan(grid["tan_a"]) ** grid["tan_b"]
    return (e - swl) + sig * (depth + (e - swl))


def features_columns(cfg, x, y, t):
    """First-order channels at the columns (x[j], y[j]) at time t.

    Returns feat [n][NQ nl] (scaled), base [n][3][nl] (u1, v1, w1 with the
    Taylor term above swl, unscaled) and eta1 [n]."""
    g = cfg["lsgrid"]
    nl = g["nl"]
    depth, swl, grav = cfg["depth"], cfg["swl"], cfg["gravity"]
    om = np.asarray(cfg["omega"], float)
    A = np.asarray(cfg["A"], float)
    k = np.asarray(cfg["k"], float)
    th = np.asarray(cfg["theta"], float) + cfg["mtheta"] * PI_IRR / 180.0
    ph0 = om * cfg["tofmax"] + np.asarray(cfg["phase"], float)
    r = _freq_ramp(t, np.asarray(cfg["ramptime"], float), np.asarray(cfg["starttime"], float),
                   np.asarray(cfg["duration"], float))
    sigma, om_m, _ = sea_scales(cfg)
    ct, st = np.cos(th), np.sin(th)
    x = np.atleast_1d(np.asarray(x, float))
    y = np.atleast_1d(np.asarray(y, float))
    n = x.size
    feat = np.zeros((n, NQ * nl))
    base = np.zeros((n, 3, nl))
    eta1 = np.zeros(n)
    au = A * grav * k / om
    for j in range(n):
        arg = k * (ct * (x[j] - cfg["x_pos"]) + st * (y[j] - cfg["y_pos"])) - om * t + ph0
        c, s = np.cos(arg) * r, np.sin(arg) * r
        e1 = float((A * c).sum())
        eta1[j] = e1
        gx = float((ct * A * om * k * c).sum())
        gy = float((st * A * om * k * c).sum())
        for m in range(nl):
            z = sigma_s2cart(g, depth, swl, m, e1 + swl)
            z0, za = min(0.0, z), max(0.0, z - swl)
            px = np.cosh(k * (z0 + depth)) / np.cosh(k * depth)
            pz = np.sinh(k * (z0 + depth)) / np.cosh(k * depth)
            u, uq = (au * ct * px * c).sum(), (au * ct * px * s).sum()
            v, vq = (au * st * px * c).sum(), (au * st * px * s).sum()
            w, wq = (au * pz * s).sum(), -(au * pz * c).sum()
            p, pq = (A * px * c).sum(), (A * px * s).sum()
            su, sp = 1.0 / (sigma * om_m), 1.0 / sigma
            feat[j, NQ * m:NQ * (m + 1)] = [u * su, uq * su, v * su, vq * su, w * su, wq * su, p * sp, pq * sp]
            gz = float((A * om * k / np.tanh(k * depth) * s).sum())
            base[j, :, m] = [u + gx * za, v + gy * za, w + gz * za]
    return feat, base, eta1


# ---------------------------------------------------------------------------
# network
# ---------------------------------------------------------------------------
def layout(nl):
    """Channel counts and offsets of the flat parameter vector: all weight
    blocks [O][C][3][3] first, then the biases."""
    ch = [NQ * nl, HID, HID, HID, 1 + 3 * nl]
    off_w, off_b, o = [], [], 0
    for l in range(4):
        off_w.append(o)
        o += ch[l + 1] * ch[l] * 9
    for l in range(4):
        off_b.append(o)
        o += ch[l + 1]
    return ch, off_w, off_b, o


def bf16_round(w):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP64."""
    f = np.asarray(w, np.float32).copy()
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, nl, rounded=True):
    """Weights ([O][C][3][3], BF16-rounded as the kernels use them unless
    rounded is False) and biases (FP32 values) of the flat vector."""
    ch, off_w, off_b, n = layout(nl)
    p = np.asarray(params, np.float32 if rounded else np.float64)
    assert p.size == n
    W, b = [], []
    for l in range(4):
        w = p[off_w[l]:off_w[l] + ch[l + 1] * ch[l] * 9]
        w = bf16_round(w) if rounded else w.astype(np.float64)
        W.append(w.reshape(ch[l + 1], ch[l], 3, 3))
        b.append(p[off_b[l]:off_b[l] + ch[l + 1]].astype(np.float64))
    return W, b


def _conv(x, W, b):
    B, C, H, Wd = x.shape
    Ho, Wo = H - 2, Wd - 2
    y = np.zeros((B, W.shape[0], Ho, Wo)) + b[None, :, None, None]
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("oc,bchw->bohw", W[:, :, ky, kx], x[:, :, ky:ky + Ho, kx:kx + Wo], optimize=True)
    return y


def _sig(a):
    return 1.0 / (1.0 + np.exp(-a))


def forward(params, nl, x, rounded=True):
    W, b = unpack(params, nl, rounded)
    h = np.asarray(x, np.float64)
    cache = []
    for l in range(4):
        a = _conv(h, W[l], b[l])
        cache.append((h, a))
        h = a * _sig(a) if l < 3 else a
    return h, cache


def loss_grad(params, nl, x, tgt, rounded=True):
    """Weighted mean-square loss (w_0 = nl, other channels 1) and its gradient
    with respect to the flat parameter vector (the BF16-rounded weights are
    the ones used, the gradient is with respect to them)."""
    ch, off_w, off_b, n = layout(nl)
    W, b = unpack(params, nl, rounded)
    y, cache = forward(params, nl, x, rounded)
    tgt = np.asarray(tgt, np.float64)
    B, O, Ho, Wo = y.shape
    wch = np.ones(O)
    wch[0] = nl
    norm = B * Ho * Wo * wch.sum()
    d = y - tgt
    loss = float((wch[None, :, None, None] * d * d).sum() / norm)
    dy = 2.0 * wch[None, :, None, None] * d / norm
    grad = np.zeros(n)
    for l in range(3, -1, -1):
        h, a = cache[l]
        Hh, Wh = h.shape[2], h.shape[3]
        Hy, Wy = Hh - 2, Wh - 2
        gW = np.zeros_like(W[l])
        dh = np.zeros_like(h)
        for ky in range(3):
            for kx in range(3):
                xs = h[:, :, ky:ky + Hy, kx:kx + Wy]
                gW[:, :, ky, kx] = np.einsum("bohw,bchw->oc", dy, xs, optimize=True)
                dh[:, :, ky:ky + Hy, kx:kx + Wy] += np.einsum("oc,bohw->bchw", W[l][:, :, ky, kx], dy, optimize=True)
        grad[off_w[l]:off_w[l] + gW.size] = gW.ravel()
        grad[off_b[l]:off_b[l] + W[l].shape[0]] = dy.sum(axis=(0, 2, 3))
        if l > 0:
            ap = cache[l - 1][1]
            s = _sig(ap)
            dy = dh * s * (1.0 + ap * (1.0 - s))
    return loss, grad
