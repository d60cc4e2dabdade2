"""Python restatement of the reference's ``waveinput.dat`` reader (oracle side).

TEST INFRASTRUCTURE ONLY: used by the tests and the CPU-baseline leg of
``bench.py`` to build the oracle's inputs from the same file the product
library reads.  It restates ``wave_Initialize`` (comment stripping and the
``@v`` version check, CFDwavemaker.cpp:2065-2149) and ``process_inputdata``
(CFDwavemaker.cpp:232-1530) for the hot-path wave types: irregular (1),
irregular + s-grid (5) and regular Stokes5/Fenton (21).  Piston, SWD, VTK and
slope inputs are recognised but carry no kinematics on this path.
"""
from __future__ import annotations

import math

SMALL = 1.0e-12
HUGE = 1.0e12
LARGEVAL = 1.0e12


class _Lines:
    """std::istringstream + std::getline semantics (CFDwavemaker.cpp:239-256)."""

    def __init__(self, text: str):
        self.lines = text.split("\n")
        if self.lines and self.lines[-1] == "":
            self.lines.pop()
        self.pos = 0
        self.eof = False

    def getline(self) -> str:
        if self.pos >= len(self.lines):
            self.eof = True
            return ""
        s = self.lines[self.pos]
        self.pos += 1
        return s


def _tokens(line: str):
    return line.split()


def _num(tok, default=0.0):
    """``operator>>`` into a double; a failed extraction leaves 0."""
    try:
        return float(tok)
    except (TypeError, ValueError):
        return default


def _int(tok, default=0):
    try:
        return int(float(tok)) if tok is not None and "." in tok else int(tok)
    except (TypeError, ValueError):
        return default


class ParseError(RuntimeError):
    pass


def read_text(text: str) -> dict:
    """Strip comments and check the version line (CFDwavemaker.cpp:2113-2138)."""
    kept = []
    for raw in text.split("\n"):
        line = raw.split("#", 1)[0]
        if len(line) > 0:
            kept.append(line)
    res = "".join(l + "\n" for l in kept)
    first = res.split("\n", 1)[0].strip()
    if first[:2] != "@v":
        raise ParseError("input file version line (@vNNN) missing")
    if int(first[2:5]) < 300:
        raise ParseError("input file version older than 300")
    return process(res)


def default_config() -> dict:
    return {
        "wavetype": 0,
        "depth": 0.0, "mtheta": 0.0, "normalize": False, "ampl": 1.0, "swl": 0.0,
        "gravity": 9.81, "rho": 1.0, "nhpres_include_kinetic": False,
        "tofmax": 0.0, "x_pos": 0.0, "y_pos": 0.0,
        "ramp_init": False, "ramp_flags": 0, "ramp_lim": [0.0] * 12,
        "extrapolation_met": 0, "order": 2, "dw_cutoff": 100000.0, "dw_bandwidth": 100.0,
        "bw_auto": False, "individual_ramp": False, "vertical_theory": 0,
        "nfreq": 0, "ndir": 1, "property_read": False,
        "omega": [], "A": [], "k": [], "phase": [], "theta": [],
        "ramptime": [], "starttime": [], "duration": [],
        "regular_theory": 0, "wave_order": 16, "regular_specify_length": True,
        "wave_length": 0.0, "wave_period": 0.0, "wave_height": 0.0, "current": 0.0,
        "lsgrid": None,
    }


def _sorted_push(cfg, cols):
    """Stable sort by omega (CFDwavemaker.cpp:160-175, 714, 785)."""
    order = sorted(range(len(cols["omega"])), key=lambda i: cols["omega"][i])
    for key in ("omega", "A", "k", "phase", "theta", "ramptime", "starttime", "duration"):
        cfg[key] = [cols[key][i] for i in order]


def process(res: str) -> dict:
    cfg = default_config()
    f = _Lines(res)
    skip = False
    line = ""
    while not f.eof:
        if skip:
            skip = False
        else:
            line = f.getline().strip()

        if line == "[wave type]":
            line = f.getline().strip()
            wt = {"irregular": 1, "1": 1, "piston": 11, "regular": 21, "swd": 31,
                  "vtk": 41, "slope": 51}
            if line not in wt:
                raise ParseError("unknown wave type: %r" % line)
            cfg["wavetype"] = wt[line]

        if line == "[general input data]":
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line)
                if line.startswith("depth"):
                    cfg["depth"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("mtheta"):
                    cfg["mtheta"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("normalize"):
                    cfg["normalize"] = bool(_int(t[1] if len(t) > 1 else None))
                if line.startswith("amplify"):
                    cfg["ampl"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("swl"):
                    cfg["swl"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("gravity"):
                    cfg["gravity"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("rho"):
                    cfg["rho"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("nhpres_include_kinetic"):
                    cfg["nhpres_include_kinetic"] = len(t) > 1 and t[1].startswith("true")
                if line.startswith("["):
                    skip = True
                    break

        if line == "[wave reference point]":
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line)
                if line.startswith("time"):
                    cfg["tofmax"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("x"):
                    cfg["x_pos"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("y"):
                    cfg["y_pos"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("["):
                    skip = True
                    break

        if line == "[ramps]":
            cfg["ramp_init"] = True
            names = ["time_rampup", "time_rampdown", "x_rampup", "x_rampdown",
                     "y_rampup", "y_rampdown"]
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line)
                for q, nm in enumerate(names):
                    if line.startswith(nm):
                        cfg["ramp_flags"] |= 1 << q
                        cfg["ramp_lim"][2 * q] = _num(t[1] if len(t) > 1 else None)
                        cfg["ramp_lim"][2 * q + 1] = _num(t[2] if len(t) > 2 else None)
                if line.startswith("["):
                    skip = True
                    break

        if line == "[wave input irregular]":
            if cfg["wavetype"] != 1:
                raise ParseError("irregular components do not match the wave type")
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line)
                if line.startswith("kinematics_surf_extrap"):
                    em = _int(t[1] if len(t) > 1 else None)
                    cfg["extrapolation_met"] = em
                    if em == 2:
                        cfg["order"] = 2
                    elif em in (0, 1):
                        cfg["order"] = 0
                    else:
                        raise ParseError("unknown extrapolation method")
                if line.startswith("cutoff"):
                    cfg["dw_cutoff"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("bandwidth"):
                    v = t[1] if len(t) > 1 else ""
                    if v.startswith("off"):
                        pass
                    elif v.startswith("auto"):
                        cfg["bw_auto"] = True
                    else:
                        cfg["dw_bandwidth"] = _num(v)
                if line.startswith("individual_ramp"):
                    if len(t) > 1 and t[1].startswith("true"):
                        cfg["individual_ramp"] = True
                if line.startswith("vertical_theory"):
                    cfg["vertical_theory"] = 1 if (len(t) > 1 and t[1].startswith("smit")) else 0
                if line.startswith("nfreq"):
                    break
            if not line.startswith("nfreq"):
                raise ParseError("nfreq missing")
            cfg["nfreq"] = _int(_tokens(line)[1])
            line = f.getline().strip()
            if not line.startswith("ndir"):
                raise ParseError("ndir missing")
            cfg["ndir"] = _int(_tokens(line)[1])
            nf = cfg["nfreq"]
            cols = {k: [] for k in ("omega", "A", "k", "phase", "theta", "ramptime",
                                    "starttime", "duration")}
            if cfg["ndir"] == 0:
                cfg["ndir"] = 1
                for _ in range(nf):
                    raw = f.getline()
                    if raw.startswith("["):
                        raise ParseError("not enough frequency components")
                    t = _tokens(raw) + [None] * 8
                    cols["omega"].append(_num(t[0])); cols["A"].append(_num(t[1]))
                    cols["k"].append(_num(t[2])); cols["phase"].append(_num(t[3]))
                    cols["theta"].append(_num(t[4]))
                    if cfg["individual_ramp"]:
                        cols["ramptime"].append(_num(t[5])); cols["starttime"].append(_num(t[6]))
                        cols["duration"].append(_num(t[7]))
                    else:
                        cols["ramptime"].append(0.0); cols["starttime"].append(-SMALL)
                        cols["duration"].append(HUGE)
            else:
                fr = []
                for _ in range(nf):
                    t = _tokens(f.getline()) + [None] * 4
                    fr.append((_num(t[0]), _num(t[1]), _num(t[2]), _num(t[3])))
                dr = []
                for _ in range(cfg["ndir"]):
                    raw = f.getline()
                    if raw.startswith("["):
                        raise ParseError("too few directional components")
                    t = _tokens(raw) + [None] * 2
                    dr.append((_num(t[0]), _num(t[1])))
                for (om, a, kk, ph) in fr:
                    for (th, dd) in dr:
                        cols["omega"].append(om); cols["k"].append(kk)
                        cols["A"].append(a * dd); cols["phase"].append(ph)
                        cols["theta"].append(th); cols["ramptime"].append(0.0)
                        cols["starttime"].append(-SMALL); cols["duration"].append(HUGE)
            _sorted_push(cfg, cols)
            cfg["property_read"] = True

        if line == "[wave input regular]":
            if cfg["wavetype"] != 21:
                raise ParseError("regular wave properties do not match the wave type")
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line)
                if line.startswith("theory_type"):
                    tt = t[1] if len(t) > 1 else ""
                    cfg["regular_theory"] = 1 if tt in ("stream", "fenton") else 0
                if line.startswith("wave_order"):
                    cfg["wave_order"] = _int(t[1] if len(t) > 1 else None)
                if line.startswith("wave_length"):
                    cfg["wave_length"] = _num(t[1] if len(t) > 1 else None)
                    cfg["regular_specify_length"] = True
                    cfg["wave_period"] = period_from_length(cfg["wave_length"], cfg["depth"], cfg["gravity"])
                if line.startswith("wave_period"):
                    cfg["wave_period"] = _num(t[1] if len(t) > 1 else None)
                    cfg["regular_specify_length"] = False
                    cfg["wave_length"] = wavelength_from_period(cfg["wave_period"], cfg["depth"], cfg["gravity"])
                if line.startswith("wave_height"):
                    cfg["wave_height"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("current_speed"):
                    cfg["current"] = _num(t[1] if len(t) > 1 else None)
                if line.startswith("["):
                    skip = True
                    break
            cfg["property_read"] = True

        if line == "[lsgrid]":
            g = {"domain": [0.0] * 4, "nx": 5, "ny": 0, "nl": 4, "t0": 0.0, "dt": 0.1,
                 "tan_a": 0.0, "tan_b": 0.0,
                 "domain_ignore": [LARGEVAL, -LARGEVAL, LARGEVAL, -LARGEVAL],
                 "ignore_domain": False, "ignore_at_init": False, "init_only": False}
            while not f.eof:
                line = f.getline().strip()
                t = _tokens(line) + [None] * 5
                if line.startswith("bounds"):
                    g["domain"] = [_num(t[1]), _num(t[2]), _num(t[3]), _num(t[4])]
                if line.startswith("nx"):
                    g["nx"] = _int(t[1])
                if line.startswith("ny"):
                    g["ny"] = _int(t[1])
                if line.startswith("nl"):
                    g["nl"] = _int(t[1])
                if line.startswith("t0"):
                    g["t0"] = _num(t[1])
                if line.startswith("dt"):
                    g["dt"] = _num(t[1])
                if line.startswith("stretch_params"):
                    g["tan_a"] = _num(t[1]); g["tan_b"] = _num(t[2])
                if line.startswith("ignore_subdomain"):
                    g["domain_ignore"] = [_num(t[1]), _num(t[2]), _num(t[3]), _num(t[4])]
                    g["ignore_domain"] = True
                if line.startswith("ignore_at_init"):
                    g["ignore_at_init"] = bool(_int(t[1]))
                if line.startswith("init_only"):
                    g["init_only"] = bool(_int(t[1]))
                if line.startswith("["):
                    skip = True
                    break
            if cfg["wavetype"] == 1:
                cfg["wavetype"] = 5
            else:
                raise ParseError("s-grid only with irregular second order theory")
            cfg["lsgrid"] = g

    if cfg["wavetype"] == 5 and cfg["order"] != 2:
        raise ParseError("s-grid requires second order theory")
    if cfg["wavetype"] in (1, 5):
        if not cfg["property_read"]:
            raise ParseError("irregular wave selected but no components found")
        if cfg["bw_auto"]:
            cfg["dw_bandwidth"] = bandwidth_estimator(cfg)
        normalize_data(cfg)
    return cfg


def normalize_data(cfg):
    """Irregular::normalize_data, Irregular.cpp:1282-1297."""
    sumA = 0.0
    for a in cfg["A"]:
        sumA += a
    if cfg["normalize"]:
        cfg["A"] = [cfg["ampl"] * a / sumA for a in cfg["A"]]
        cfg["phase"] = [0.0 for _ in cfg["phase"]]
    else:
        cfg["A"] = [cfg["ampl"] * a for a in cfg["A"]]


def spectral_moments(cfg):
    """Irregular::spectral_moments, Irregular.cpp:1336-1369 (nfreq-1 terms)."""
    m0 = m1 = m2 = 0.0
    om, A = cfg["omega"], cfg["A"]
    for i in range(cfg["nfreq"] - 1):
        m0 += A[i] * A[i] / 2.0
        m1 += om[i] * A[i] * A[i] / 2.0
        m2 += om[i] * om[i] * A[i] * A[i] / 2.0
    return m0, m1, m2


PI_TRUNC = 3.1415926535897      # the truncated PI of Irregular.h:14


def _interpolate_extrap(xd, yd, x):
    """Irregular::interpolate with extrapolation, Irregular.cpp:1311-1334."""
    n = len(xd)
    i = 0
    if x >= xd[n - 2]:
        i = n - 2
    else:
        while x > xd[i + 1]:
            i += 1
    xL, yL, xR, yR = xd[i], yd[i], xd[i + 1], yd[i + 1]
    return yL + (yR - yL) / (xR - xL) * (x - xL)


def _mean_periods(cfg):
    m0, m1, m2 = spectral_moments(cfg)
    return 2.0 * PI_TRUNC * (m0 / m1), 2.0 * PI_TRUNC * math.sqrt(m0 / m2)


def mean_wave_period(cfg, opt):
    """Irregular::mean_wave_period, Irregular.cpp:1420-1436 (T1 for opt 1, T2 for opt 2)."""
    t1, t2 = _mean_periods(cfg)
    return {1: t1, 2: t2}.get(opt, 0.0)


def phase_speed(cfg, opt):
    """Irregular::phase_speed, Irregular.cpp:1372-1393."""
    if opt not in (1, 2):
        return 0.0
    w = 2 * PI_TRUNC / _mean_periods(cfg)[opt - 1]
    return w / _interpolate_extrap(cfg["omega"], cfg["k"], w)


def mean_wave_length(cfg, opt):
    """Irregular::mean_wave_length, Irregular.cpp:1399-1417."""
    if opt not in (1, 2):
        return 0.0
    w = 2 * PI_TRUNC / _mean_periods(cfg)[opt - 1]
    return (2.0 * PI_TRUNC) / _interpolate_extrap(cfg["omega"], cfg["k"], w)


def bandwidth_estimator(cfg):
    """Irregular::bandwidth_estimator, Irregular.cpp:1439-1452."""
    if cfg["ndir"] > 1:
        raise ParseError("automatic bandwidth only for one direction")
    m0, m1, _ = spectral_moments(cfg)
    return 0.7 * (m1 / m0)


PI_FULL = 3.14159265358979323846


def wavenumber_from_period(T, depth, g):
    """Stokes5::wavenumberFromPeriod, Stokes5.cpp:187-212."""
    omega = 2.0 * PI_FULL / T
    kd, ks = omega * omega / g, omega / math.sqrt(g * depth)
    kk = 0.5 * (kd + ks)
    for _ in range(40):
        th = math.tanh(kk * depth)
        fv = g * kk * th - omega * omega
        if abs(fv) < 1e-14:
            break
        df = g * (th + kk * depth * (1.0 - th * th))
        if abs(df) < 1e-14:
            break
        dk = -fv / df
        kk += dk
        if kk < 1e-12:
            kk = 1e-12
        if abs(dk) < 1e-12 * kk:
            break
    return kk


def wavelength_from_period(T, depth, g):
    kk = wavenumber_from_period(T, depth, g)
    return 2.0 * PI_FULL / kk if kk > 0.0 else 0.0


def period_from_length(L, depth, g):
    kk = 2.0 * PI_FULL / L
    return 2.0 * PI_FULL / math.sqrt(g * kk * math.tanh(kk * depth))


def read_file(path: str) -> dict:
    with open(path, "r") as fh:
        return read_text(fh.read())
