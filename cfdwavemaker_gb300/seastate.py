"""Synthetic sea states and ``waveinput.dat`` writers.

The reference library reads its spectral components from ``waveinput.dat``
(CFDwavemaker.cpp:677-800); it does not generate spectra.  These helpers
produce seeded JONSWAP seas (optionally with cos-2s spreading) in the
``ndir 0`` five-column format, which gives every component its own phase
(the ``ndir > 0`` format shares one phase per frequency,
CFDwavemaker.cpp:772-780), and Stokes5 / Fenton regular-wave inputs.
Wavenumbers come from the FP64 Newton solve of w^2 = g k tanh(k h).
"""
from __future__ import annotations

import math
import os

import numpy as np


def dispersion_k(omega, depth, g=9.81, iters=60):
    """Wavenumber from w^2 = g k tanh(k h) by Newton iteration in FP64."""
    w = np.asarray(omega, dtype=np.float64)
    k = np.maximum(w * w / g, w / np.sqrt(g * depth))
    for _ in range(iters):
        th = np.tanh(k * depth)
        f = g * k * th - w * w
        df = g * (th + k * depth * (1.0 - th * th))
        k = k - f / df
    return k


def jonswap(omega, hs, tp, gamma, g=9.81):
    """JONSWAP spectral density S(w), scaled so that 4 sqrt(m0) = hs over the given band."""
    w = np.asarray(omega, dtype=np.float64)
    wp = 2.0 * math.pi / tp
    sig = np.where(w <= wp, 0.07, 0.09)
    r = np.exp(-((w - wp) ** 2) / (2.0 * sig * sig * wp * wp))
    s = g * g * w ** -5.0 * np.exp(-1.25 * (wp / w) ** 4) * gamma ** r
    dw = np.gradient(w) if w.size > 1 else np.ones_like(w)
    m0 = np.sum(s * dw)
    return s * (hs * hs / 16.0) / m0


def cos2s_weights(theta, s, theta0=0.0):
    """cos-2s spreading weights D(theta_j) dtheta_j, summing to 1."""
    th = np.asarray(theta, dtype=np.float64)
    d = np.cos(0.5 * (th - theta0)) ** (2.0 * s)
    return d / np.sum(d)


def splitmix64(seed, n):
    """The first n outputs of SplitMix64 (Steele, Lea & Flood 2014) from state
    ``seed``: the mix of seed + c 0x9E3779B97F4A7C15, c = 1..n (uint64)."""
    with np.errstate(over="ignore"):
        c = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed % (1 << 64)) + c * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def splitmix_phases(seed, n):
    """Phases 2 pi u_c, u_c = the top 53 bits of the c-th SplitMix64 output / 2^53:
    the phases the library's device generator gives (cfdwm_spectrum_components)."""
    z = splitmix64(seed, n)
    return 2.0 * math.pi * ((z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0))


def irregular_components(hs, tp, gamma, nfreq, wmin, wmax, depth, seed, ndir=1,
                         spreading_s=None, theta_span=math.pi / 2, g=9.81, phase_rng="numpy"):
    """Component arrays (omega, A, k, phase, theta) for a seeded sea state.

    Frequencies are equally spaced in [wmin, wmax]; amplitudes are
    sqrt(2 S(w) dw D(theta) dtheta); phases are uniform in [0, 2 pi) from
    ``seed`` (numpy's generator, or with phase_rng="splitmix" the library's
    own, see splitmix_phases).  With ndir > 1 the directions are equally
    spaced over +-theta_span around 0 and weighted with cos-2s spreading.
    """
    rng = np.random.default_rng(seed)
    om = np.linspace(wmin, wmax, nfreq)
    dw = (wmax - wmin) / (nfreq - 1) if nfreq > 1 else 1.0
    S = jonswap(om, hs, tp, gamma, g)
    if ndir > 1:
        th = np.linspace(-theta_span, theta_span, ndir)
        D = cos2s_weights(th, spreading_s if spreading_s is not None else 10.0)
    else:
        th = np.zeros(1)
        D = np.ones(1)
    omega = np.repeat(om, th.size)
    theta = np.tile(th, om.size)
    A = np.sqrt(2.0 * np.repeat(S, th.size) * dw * np.tile(D, om.size))
    k = dispersion_k(omega, depth, g)
    if phase_rng == "splitmix":
        phase = splitmix_phases(seed, omega.size)
    else:
        phase = rng.uniform(0.0, 2.0 * math.pi, omega.size)
    return {"omega": omega, "A": A, "k": k, "phase": phase, "theta": theta}


def write_irregular(path, comps, depth, *, extrap=2, bandwidth=None, cutoff=None,
                    gravity=None, rho=None, swl=None, mtheta=None, ref_point=None,
                    ramps=None, lsgrid=None, normalize=None, amplify=None, ramp_columns=None,
                    vertical_theory=None):
    """Write an irregular-sea ``waveinput.dat`` (ndir 0 format).  vertical_theory:
    None (the default Sharma-Dean theory) or "smit"."""
    L = ["@v310", "[wave type]", "irregular", "", "[general input data]", "depth %.17g" % depth]
    if mtheta is not None:
        L.append("mtheta %.17g" % mtheta)
    if normalize is not None:
        L.append("normalize %d" % int(normalize))
    if amplify is not None:
        L.append("amplify %.17g" % amplify)
    if swl is not None:
        L.append("swl %.17g" % swl)
    if gravity is not None:
        L.append("gravity %.17g" % gravity)
    if rho is not None:
        L.append("rho %.17g" % rho)
    L.append("")
    if ref_point is not None:
        L += ["[wave reference point]", "time %.17g" % ref_point[0], "x %.17g" % ref_point[1],
              "y %.17g" % ref_point[2], ""]
    if ramps:
        L.append("[ramps]")
        for name, (a, b) in ramps.items():
            L.append("%s %.17g %.17g" % (name, a, b))
        L.append("")
    L.append("[wave input irregular]")
    L.append("kinematics_surf_extrap %d" % extrap)
    if bandwidth is not None:
        L.append("bandwidth %s" % bandwidth)
    if cutoff is not None:
        L.append("cutoff %.17g" % cutoff)
    if ramp_columns is not None:
        L.append("individual_ramp true")
    if vertical_theory is not None:
        L.append("vertical_theory %s" % vertical_theory)
    n = len(comps["omega"])
    L.append("nfreq %d" % n)
    L.append("ndir 0")
    for i in range(n):
        row = "%.17g %.17g %.17g %.17g %.17g" % (comps["omega"][i], comps["A"][i], comps["k"][i],
                                                   comps["phase"][i], comps["theta"][i])
        if ramp_columns is not None:
            row += " %.17g %.17g %.17g" % tuple(ramp_columns[j][i] for j in range(3))
        L.append(row)
    L.append("")
    if lsgrid is not None:
        L.append("[lsgrid]")
        L.append("bounds %.17g %.17g %.17g %.17g" % tuple(lsgrid["bounds"]))
        L.append("nx %d" % lsgrid["nx"])
        L.append("ny %d" % lsgrid["ny"])
        L.append("nl %d" % lsgrid["nl"])
        L.append("t0 %.17g" % lsgrid.get("t0", 0.0))
        L.append("dt %.17g" % lsgrid["dt"])
        L.append("stretch_params %.17g %.17g" % tuple(lsgrid.get("stretch", (0.7, 1.5))))
        if "ignore" in lsgrid:
            L.append("ignore_subdomain %.17g %.17g %.17g %.17g" % tuple(lsgrid["ignore"]))
        if lsgrid.get("ignore_at_init"):
            L.append("ignore_at_init 1")
        L.append("")
        if lsgrid.get("vtk"):
            # .vtu output of the grid: {"path": dir (with trailing /), "prefix": ..., "label": ...}
            v = lsgrid["vtk"]
            L.append("[lsgrid2vtk]")
            if "path" in v:
                L.append("storage_path %s" % v["path"])
            if "prefix" in v:
                L.append("filename %s" % v["prefix"])
            if "label" in v:
                L.append("vtk_timelabel %s" % v["label"])
            L.append("")
    text = "\n".join(L) + "\n"
    if path is not None:
        d = os.path.dirname(os.path.abspath(path))
        os.makedirs(d, exist_ok=True)
        with open(path, "w") as fh:
            fh.write(text)
    return text


def write_regular(path, theory, height, depth, *, period=None, length=None, order=None,
                  current=None, gravity=None, rho=None, mtheta=None, swl=None, ref_point=None):
    """Write a regular-wave ``waveinput.dat`` (Stokes5 or Fenton stream function)."""
    L = ["@v310", "[wave type]", "regular", "", "[general input data]", "depth %.17g" % depth]
    if mtheta is not None:
        L.append("mtheta %.17g" % mtheta)
    if swl is not None:
        L.append("swl %.17g" % swl)
    if gravity is not None:
        L.append("gravity %.17g" % gravity)
    if rho is not None:
        L.append("rho %.17g" % rho)
    L.append("")
    if ref_point is not None:
        L += ["[wave reference point]", "time %.17g" % ref_point[0], "x %.17g" % ref_point[1],
              "y %.17g" % ref_point[2], ""]
    L.append("[wave input regular]")
    L.append("theory_type %s" % theory)
    if order is not None:
        L.append("wave_order %d" % order)
    if period is not None:
        L.append("wave_period %.17g" % period)
    if length is not None:
        L.append("wave_length %.17g" % length)
    L.append("wave_height %.17g" % height)
    if current is not None:
        L.append("current_speed %.17g" % current)
    L.append("")
    text = "\n".join(L) + "\n"
    if path is not None:
        with open(path, "w") as fh:
            fh.write(text)
    return text


# The named workloads of the benchmark and parity suite.
def config1_sea(seed=12345):
    """Long-crested JONSWAP Hs=4 m Tp=10 s gamma=3.3, 128 components in 0.3-2.0 rad/s, depth 50 m."""
    return irregular_components(4.0, 10.0, 3.3, 128, 0.3, 2.0, 50.0, seed)


def config3_sea(seed=2024, nfreq=64, ndir=16):
    """Short-crested JONSWAP Hs=6 m Tp=12 s gamma=2 with cos-2s (s=10), depth 100 m.

    The band 0.25-1.6 rad/s is an assumption of this build (the workload names
    only the frequency and direction counts)."""
    return irregular_components(6.0, 12.0, 2.0, nfreq, 0.25, 1.6, 100.0, seed, ndir=ndir,
                                spreading_s=10.0)
