"""Learned s-grid update: training data, training and evaluation.

Everything that computes runs in the library's CUDA kernels through its C ABI
(``cfdwm_surrogate_*``, include/cfdwavemaker_gb300.h part 5); PyTorch only
provides device memory.  Training data are ring slots filled by the plain
second-order method for randomly drawn JONSWAP seas:

    Hs 2-10 m (capped at Lp / 14), Tp 6-16 s, gamma 1-5, cos-2s spreading
    s 2-20, mean direction uniform, 64 frequencies x 16 directions = 1024
    components in 0.25-1.6 rad/s, depth 100 m, seeded phases;

each sea gives several slots of a 64 x 64 x 16 grid patch with the spacing of
the 256 x 256 / 1 km grid (the network is convolutional, so patches train the
operator that then runs on the full grid).

    python -m cfdwavemaker_gb300.surrogate train --seas 400 --steps 6000 --out W.bin
    python -m cfdwavemaker_gb300.surrogate analyse     (how local the predicted part is)
    python -m cfdwavemaker_gb300.surrogate time        (device time of the network)
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
import os
import tempfile
import time

import numpy as np

from . import seastate as ss

SH = 4
DEPTH = 100.0
BAND = (0.25, 1.6)
SPACING = 1000.0 / 255.0
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_nl16.bin")


def random_sea(rng, nfreq=64, ndir=16):
    """One random sea state of the training distribution (dict of parameters)."""
    tp = rng.uniform(6.0, 16.0)
    lp = 9.81 * tp * tp / (2.0 * math.pi)
    hs = rng.uniform(2.0, min(10.0, lp / 14.0))
    return {"hs": hs, "tp": tp, "gamma": rng.uniform(1.0, 5.0), "s": rng.uniform(2.0, 20.0),
            "mtheta": rng.uniform(0.0, 360.0), "seed": int(rng.integers(1 << 31)),
            "nfreq": nfreq, "ndir": ndir}


def sea_text(p, nx, ny, nl, x0, y0, dt, t0=0.0):
    comps = ss.irregular_components(p["hs"], p["tp"], p["gamma"], p["nfreq"], BAND[0], BAND[1], DEPTH,
                                    p["seed"], ndir=p["ndir"], spreading_s=p["s"])
    grid = {"bounds": (x0, x0 + SPACING * (nx - 1), y0, y0 + SPACING * (ny - 1)), "nx": nx, "ny": ny,
            "nl": nl, "t0": t0, "dt": dt, "stretch": (0.7, 1.5)}
    return ss.write_irregular(None, comps, DEPTH, extrap=2, lsgrid=grid, mtheta=p["mtheta"])


class Trainer:
    """Owns the library handle and the device datasets."""

    def __init__(self, nl=16, seed=1, device="cuda"):
        import torch
        import cfdwavemaker_gb300 as cw
        self.torch = torch
        self.cw = cw
        self.lib = cw.load()
        self.nl = nl
        self.dev = device
        self.wm = cw.CFDwavemaker()
        self._ok(self.lib.cfdwm_surrogate_create(nl, seed))

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError("cfdwavemaker_gb300: %d %s" % (rc, self.cw.last_error()))

    def slot_time(self, k):
        t0 = C.c_double(0.0)
        ts = C.c_int(0)
        self._ok(self.lib.cfdwm_sgrid_state(C.byref(t0), C.byref(ts)))
        # ring slot (tstep + q) % 4 holds t0 + (q - 1) dt
        q = (k - ts.value) % 4
        return t0.value + (q - 1) * self.dt

    def snapshot(self, slot, feat, tgt):
        """Features of the loaded grid at the slot's time and the normalised
        targets of that (plain-filled) slot, into the given device tensors."""
        torch = self.torch
        nx, ny, nl = self.nx, self.ny, self.nl
        base = torch.empty(3 * nx * ny * nl, device=self.dev, dtype=torch.float32)
        eta1 = torch.empty(nx * ny, device=self.dev, dtype=torch.float32)
        p = self.cw._ptr
        self._ok(self.lib.cfdwm_surrogate_features(self.slot_time(slot), p(feat), p(base), p(eta1)))
        self._ok(self.lib.cfdwm_surrogate_targets(slot, p(base), p(eta1), p(tgt)))

    def generate(self, nsea, seed, nx=64, ny=64, per_sea=8, dt=1.7):
        """Datasets X [S][8 nl][nx+8][ny+8] and T [S][1+3 nl][nx][ny] on the device."""
        torch = self.torch
        self.nx, self.ny, self.dt = nx, ny, dt
        rng = np.random.default_rng(seed)
        S = nsea * per_sea
        X = torch.empty((S, 8 * self.nl, nx + 2 * SH, ny + 2 * SH), device=self.dev, dtype=torch.float32)
        T = torch.empty((S, 1 + 3 * self.nl, nx, ny), device=self.dev, dtype=torch.float32)
        cwd = os.getcwd()
        os.chdir(tempfile.mkdtemp())
        try:
            s = 0
            self.skipped = 0
            while s < S:
                p = random_sea(rng)
                x0, y0 = rng.uniform(0.0, 750.0, 2)
                txt = sea_text(p, nx, ny, self.nl, x0, y0, dt, t0=rng.uniform(0.0, 200.0))
                self._ok(self.wm.initialize_text(txt))
                s1 = s
                for k in range(min(4, per_sea)):
                    self.snapshot(k, X[s1], T[s1])
                    s1 += 1
                for _ in range(per_sea - 4):
                    self._ok(self.lib.cfdwm_surrogate_step(0, 0.0, 0, None, None))
                    ts = C.c_int(0)
                    self._ok(self.lib.cfdwm_sgrid_state(None, C.byref(ts)))
                    self.snapshot((ts.value + 3) % 4, X[s1], T[s1])
                    s1 += 1
                # a sea whose slots are not finite is not kept
                if bool(torch.isfinite(X[s:s1]).all()) and bool(torch.isfinite(T[s:s1]).all()):
                    s = s1
                else:
                    self.skipped += 1
        finally:
            os.chdir(cwd)
        return X, T

    def train(self, X, T, steps, batch=8, lr=2e-3, lr_min=2e-5, seed=3, log_every=200, log=None):
        """Adam with a cosine learning-rate schedule over random batches."""
        rng = np.random.default_rng(seed)
        S, _, H, W = X.shape
        p = self.cw._ptr
        hist = []
        loss = C.c_double(0.0)
        for it in range(steps):
            lr_t = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * it / max(1, steps)))
            idx = (C.c_int * batch)(*rng.integers(0, S, batch).tolist())
            self._ok(self.lib.cfdwm_surrogate_train_step(p(X), p(T), S, idx, batch, H, W, lr_t, C.byref(loss)))
            if it % log_every == 0 or it == steps - 1:
                hist.append((it, loss.value))
                if log:
                    log("step %d loss %.5g lr %.3g" % (it, loss.value, lr_t))
        return hist

    def eval_loss(self, X, T, batch=8):
        S, _, H, W = X.shape
        p = self.cw._ptr
        tot, n = 0.0, 0
        loss = C.c_double(0.0)
        for b0 in range(0, S, batch):
            b = min(batch, S - b0)
            self._ok(self.lib.cfdwm_surrogate_loss_grad(p(X[b0:b0 + b]), p(T[b0:b0 + b]), b, H, W, C.byref(loss),
                                                        None))
            tot += loss.value * b
            n += b
        return tot / max(1, n)

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        self._ok(self.lib.cfdwm_surrogate_save(path.encode()))


def _cubic_mid(a, axis):
    """Values half-way between the samples of a along an axis: the 4-point
    cubic (-1, 9, 9, -1) / 16, edge samples repeated."""
    n = a.shape[axis]
    idx = np.arange(n)
    t = lambda d: np.take(a, np.clip(idx + d, 0, n - 1), axis=axis)
    return (-t(-1) + 9 * t(0) + 9 * t(1) - t(2)) / 16.0


def analyse(nx=256, ny=256, nl=16, dt=0.1, steps=20, margin=6):
    """How local the second-order part of a ring slot is, on the 1024-component
    sea of the s-grid workload (plain-method slots, the network's normalised
    targets).  Returns, per field group (eta; u, v, w over the levels):

    * share: max of the second-order part / max of the whole field (the
      learned update's error bar is relative to the whole field);
    * spectrum: fraction of the part's energy at wavelengths under 10, 8 and
      6 columns;
    * interp: max error, relative to the part's max, of recovering the
      columns between exact samples: every other column in both directions
      (a quarter exact), every other row (half), a checkerboard (half);
    * time: the same for the slot half-way through a window of `steps`
      ring steps from the two ends (linear in time).
    """
    import torch
    import cfdwavemaker_gb300 as cw
    from . import seastate as ss
    lib = cw.load()
    wm = cw.CFDwavemaker()
    comps = ss.config3_sea()
    grid = {"bounds": (0.0, 1000.0, 0.0, 1000.0), "nx": nx, "ny": ny, "nl": nl, "t0": 0.0, "dt": dt,
            "stretch": (0.7, 1.5)}
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp())
    try:
        if wm.initialize_text(ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)) != 0:
            raise RuntimeError(cw.last_error())
        if lib.cfdwm_surrogate_create(nl, 1) != 0:
            raise RuntimeError(cw.last_error())
        feat = torch.empty((8 * nl, nx + 2 * SH, ny + 2 * SH), device="cuda")
        base = torch.empty(3 * nx * ny * nl, device="cuda")
        eta1 = torch.empty(nx * ny, device="cuda")
        tgt = torch.empty((1 + 3 * nl, nx, ny), device="cuda")
        p = cw._ptr

        def newest():
            t0 = C.c_double(0.0)
            ts = C.c_int(0)
            lib.cfdwm_sgrid_state(C.byref(t0), C.byref(ts))
            slot = (ts.value + 3) % 4
            if lib.cfdwm_surrogate_features(t0.value + 2 * dt, p(feat), p(base), p(eta1)) != 0 or \
                    lib.cfdwm_surrogate_targets(slot, p(base), p(eta1), p(tgt)) != 0:
                raise RuntimeError(cw.last_error())
            torch.cuda.synchronize()
            return tgt.cpu().numpy().astype(np.float64), slot

        snaps = []
        for k in range(steps + 1):
            if k:
                if lib.cfdwm_surrogate_step(0, 0.0, 0, None, None) != 0:
                    raise RuntimeError(cw.last_error())
            if k in (0, steps // 2, steps):
                snaps.append(newest())
        X, slot = snaps[-1]
        eta = wm.sgrid_array(0).reshape(4, nx, ny)[slot]
        U = [wm.sgrid_array(f).reshape(4, nx, ny, nl)[slot] for f in (1, 2, 3)]
        umax = max(np.abs(u).max() for u in U)
    finally:
        os.chdir(cwd)
    A2 = comps["A"] ** 2
    sig2, km, om = A2.sum() / 2, (A2 * comps["k"]).sum() / A2.sum(), (A2 * comps["omega"]).sum() / A2.sum()
    groups = {"eta": [0], "u": list(range(1, 1 + nl)), "v": list(range(1 + nl, 1 + 2 * nl)),
              "w": list(range(1 + 2 * nl, 1 + 3 * nl))}
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.fftfreq(ny)[None, :]
    kk = np.sqrt(kx ** 2 + ky ** 2)
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    inner = (slice(margin, nx - margin), slice(margin, ny - margin))
    out = {}
    for g, chans in groups.items():
        scale = km * sig2 if g == "eta" else km * sig2 * om
        full = np.abs(eta).max() if g == "eta" else umax
        r = {"share": float(max(np.abs(X[c]).max() for c in chans) * scale / full)}
        P = sum(np.abs(np.fft.fft2(X[c] - X[c].mean())) ** 2 for c in chans)
        r["spectrum"] = {"under_%d_columns" % L: float(P[kk > 1.0 / L].sum() / P.sum()) for L in (10, 8, 6)}
        e = {"quarter": 0.0, "rows": 0.0, "checkerboard": 0.0}
        for c in chans:
            Z = X[c]
            m = np.abs(Z).max()
            # every other column both ways: the odd rows/columns from the even ones
            Ze = Z[::2, ::2]
            Zx = _cubic_mid(Ze, 0)                       # between even rows
            G = np.zeros_like(Z)
            G[::2, ::2] = Ze
            G[1::2, ::2] = Zx[: G[1::2, ::2].shape[0]]
            G[:, 1::2] = _cubic_mid(G[:, ::2], 1)[:, : G[:, 1::2].shape[1]]
            e["quarter"] = max(e["quarter"], float(np.abs(G - Z)[inner].max() / m))
            R = Z.copy()
            R[1::2, :] = _cubic_mid(Z[::2, :], 0)[: R[1::2, :].shape[0]]
            e["rows"] = max(e["rows"], float(np.abs(R - Z)[inner].max() / m))
            odd = (I + J) % 2 == 1
            Q = Z.copy()
            ax = (-np.roll(Z, 3, 0) + 9 * np.roll(Z, 1, 0) + 9 * np.roll(Z, -1, 0) - np.roll(Z, -3, 0)) / 16
            ay = (-np.roll(Z, 3, 1) + 9 * np.roll(Z, 1, 1) + 9 * np.roll(Z, -1, 1) - np.roll(Z, -3, 1)) / 16
            Q[odd] = (0.5 * (ax + ay))[odd]
            e["checkerboard"] = max(e["checkerboard"], float(np.abs(Q - Z)[inner].max() / m))
        r["interp"] = e
        X0, Xm, X1 = snaps[0][0], snaps[1][0], snaps[2][0]
        r["time"] = float(max(np.abs(0.5 * (X0[c] + X1[c]) - Xm[c]).max() for c in chans) /
                          max(np.abs(Xm[c]).max() for c in chans))
        out[g] = r
    return out


def time_network(nl=16, nx=256, ny=256, batch=8, patch=64, reps=20):
    """Device time of the network (the committed weights): one forward over an
    nx x ny grid with its halo, and one training step (forward, loss,
    backward, Adam) on `batch` patches of patch x patch outputs.  Inputs are
    random; times in ms (CUDA events / host clock after a synchronise)."""
    import torch
    import cfdwavemaker_gb300 as cw
    lib = cw.load()
    if lib.cfdwm_surrogate_create(nl, 1) != 0 or lib.cfdwm_surrogate_load(WEIGHTS.encode()) != 0:
        raise RuntimeError(cw.last_error())
    H, W = nx + 2 * SH, ny + 2 * SH
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn((1, 8 * nl, H, W), device="cuda", generator=g)
    y = torch.empty((1, 1 + 3 * nl, nx, ny), device="cuda")

    def fwd():
        if lib.cfdwm_surrogate_forward(cw._ptr(x), 1, H, W, cw._ptr(y)) != 0:
            raise RuntimeError(cw.last_error())
    for _ in range(3):
        fwd()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fwd()
    e1.record()
    torch.cuda.synchronize()
    out = {"forward_ms": e0.elapsed_time(e1) / reps, "grid": [nx, ny]}
    P = patch + 2 * SH
    X = torch.randn((4 * batch, 8 * nl, P, P), device="cuda", generator=g)
    T = torch.randn((4 * batch, 1 + 3 * nl, patch, patch), device="cuda", generator=g)
    loss = C.c_double(0.0)
    idx = (C.c_int * batch)(*range(batch))

    def step():
        if lib.cfdwm_surrogate_train_step(cw._ptr(X), cw._ptr(T), 4 * batch, idx, batch, P, P, C.c_float(1e-5),
                                          C.byref(loss)) != 0:
            raise RuntimeError(cw.last_error())
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        step()
    torch.cuda.synchronize()
    out["train_step_ms"] = (time.perf_counter() - t0) * 1e3 / reps
    out["train_batch"] = [batch, patch, patch]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "analyse", "time"])
    ap.add_argument("--seas", type=int, default=250)
    ap.add_argument("--per-sea", type=int, default=8)
    ap.add_argument("--val-seas", type=int, default=16)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
    if args.cmd in ("analyse", "time"):
        import json
        print(json.dumps(analyse() if args.cmd == "analyse" else time_network(), indent=1))
        return
    tr = Trainer(seed=args.seed)
    t0 = time.time()
    X, T = tr.generate(args.seas, args.seed, per_sea=args.per_sea)
    Xv, Tv = tr.generate(args.val_seas, args.seed + 1000, per_sea=args.per_sea)
    t1 = time.time()
    print("data: %d train / %d validation snapshots in %.1f s" % (X.shape[0], Xv.shape[0], t1 - t0), flush=True)
    print("validation loss before: %.5g" % tr.eval_loss(Xv, Tv), flush=True)
    tr.train(X, T, args.steps, batch=args.batch, lr=args.lr, log=lambda s: print(s, flush=True))
    t2 = time.time()
    print("trained %d steps in %.1f s; validation loss %.5g" % (args.steps, t2 - t1, tr.eval_loss(Xv, Tv)),
          flush=True)
    tr.save(args.out)
    print("saved", args.out)


if __name__ == "__main__":
    main()
