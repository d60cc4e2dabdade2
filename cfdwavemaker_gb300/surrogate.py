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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--seas", type=int, default=250)
    ap.add_argument("--per-sea", type=int, default=8)
    ap.add_argument("--val-seas", type=int, default=16)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
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
