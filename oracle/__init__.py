"""CPU oracle for the CFDwavemaker point-kinematics hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package; the product
(``cfdwavemaker_gb300``) never does.  It wraps ``oracle/liboracle.so``, a
plain-C FP64 restatement of the reference (oystelan/CFDwavemaker v3.1.0,
src/Irregular.cpp, src/lsgrid_spline.cpp, src/Stokes5.cpp,
src/FentonStream.cpp, src/Utils.cpp), and mirrors the reference's public
``wave_*`` semantics (CFDwavemaker.cpp:1543-2009) on top of it.

Parity of the restatement is pinned by tests/test_oracle_golden.py against
fixtures recorded from the unmodified reference (tests/golden/) and against
the reference's own golden vectors.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import waveinput  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = C.POINTER(C.c_double)


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with the committed Makefile; returns its path."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        src = [os.path.join(HERE, f) for f in ("oracle_irregular.c", "oracle_sgrid.c",
                                               "oracle_regular.c", "oracle.h")]
        if (not os.path.exists(path)) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in src):
            build()
        L = C.CDLL(path)
        L.orc_sea_create.restype = C.c_void_p
        L.orc_sea_create.argtypes = [C.c_int] + [_dp] * 8 + [C.c_double] * 10 + [C.c_int]
        L.orc_sea_free.argtypes = [C.c_void_p]
        L.orc_sea_npairs.restype = C.c_long
        L.orc_sea_npairs.argtypes = [C.c_void_p]
        L.orc_irregular_batch.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, C.c_int, _dp, C.c_int]
        L.orc_uvw2_batch.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_eta2.restype = C.c_double
        L.orc_eta2.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.orc_eta1.restype = C.c_double
        L.orc_eta1.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.orc_ramp.restype = C.c_double
        L.orc_ramp.argtypes = [C.c_int, C.c_int, _dp, C.c_double, C.c_double, C.c_double]
        L.orc_sgrid_create.restype = C.c_void_p
        L.orc_sgrid_create.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp] + [C.c_double] * 6
        L.orc_sgrid_free.argtypes = [C.c_void_p]
        L.orc_sgrid_init.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_sgrid_update.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.orc_sgrid_update_columns.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_long, C.c_long, C.c_int]
        L.orc_sgrid_check_time.restype = C.c_int
        L.orc_sgrid_check_time.argtypes = [C.c_void_p, C.c_double]
        L.orc_sgrid_query.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_smit_batch.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_sgrid_query5.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_sgrid_set_pressure.argtypes = [C.c_void_p, C.c_int]
        L.orc_sgrid_export_vtu.restype = C.c_int
        L.orc_sgrid_export_vtu.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_char_p]
        L.orc_sgrid_array.restype = C.c_long
        L.orc_sgrid_array.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_sgrid_state.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_int)]
        L.orc_sgrid_advance.argtypes = [C.c_void_p]
        L.orc_sgrid_gradients.argtypes = [C.c_void_p]
        L.orc_sgrid_set_slot.restype = C.c_int
        L.orc_sgrid_set_slot.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_stokes5_create.restype = C.c_void_p
        L.orc_stokes5_create.argtypes = [C.c_double] * 11
        L.orc_stokes5_free.argtypes = [C.c_void_p]
        L.orc_stokes5_batch.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_stokes5_coeffs.argtypes = [C.c_void_p, _dp]
        L.orc_fenton_create.restype = C.c_void_p
        L.orc_fenton_create.argtypes = [C.c_double] * 3 + [C.c_int] * 4 + [C.c_double] * 9 + [C.POINTER(C.c_int)]
        L.orc_fenton_free.argtypes = [C.c_void_p]
        L.orc_fenton_batch.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_fenton_solution.restype = C.c_int
        L.orc_fenton_solution.argtypes = [C.c_void_p, _dp]
        _LIB = L
    return _LIB


def _arr(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _pts(*cols):
    n = None
    out = []
    keep = []
    for c in cols:
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(c, dtype=np.float64), np.shape(cols[0])).ravel())
        keep.append(a)
        out.append(a.ctypes.data_as(_dp))
        n = a.size
    return n, out, keep


class Sea:
    """An irregular sea (orc_sea) built from a parsed config dict."""

    def __init__(self, cfg: dict):
        self.cfg = cfg
        L = lib()
        arrs = [_arr(cfg[k]) for k in ("omega", "A", "k", "phase", "theta", "ramptime",
                                       "starttime", "duration")]
        self._keep = arrs
        self.h = L.orc_sea_create(len(cfg["omega"]), *[p for _, p in arrs], cfg["depth"],
                                  cfg["mtheta"], cfg["tofmax"], cfg["x_pos"], cfg["y_pos"],
                                  cfg["swl"], cfg["gravity"], cfg["rho"], cfg["dw_bandwidth"],
                                  cfg["dw_cutoff"], cfg["order"])

    def __del__(self):
        try:
            lib().orc_sea_free(self.h)
        except Exception:
            pass

    @property
    def npairs(self):
        return lib().orc_sea_npairs(self.h)

    def fields(self, x, y, z, t, fields=31, nthreads=0):
        """eta, u, v, w, dp of Irregular::eta/u/v/w/dp (no ramp, no clamp): [n,5]."""
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 5))
        lib().orc_irregular_batch(self.h, n, p[0], p[1], p[2], p[3], fields,
                                  out.ctypes.data_as(_dp), nthreads)
        return out

    def uvw2(self, x, y, z, t, nthreads=0):
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 4))
        lib().orc_uvw2_batch(self.h, n, p[0], p[1], p[2], p[3], out.ctypes.data_as(_dp), nthreads)
        return out

    def smit(self, x, y, z, t, nthreads=0):
        """u_smit, v_smit, w_smit, dp_smit (no ramp): [n, 4]."""
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 4))
        lib().orc_smit_batch(self.h, n, p[0], p[1], p[2], p[3], out.ctypes.data_as(_dp), nthreads)
        return out

    def eta2(self, x, y, t):
        return np.array([lib().orc_eta2(self.h, float(tt), float(xx), float(yy))
                         for xx, yy, tt in zip(np.ravel(x), np.ravel(y), np.ravel(t))])


def ramp(cfg, x, y, t):
    lim, lp = _arr(cfg["ramp_lim"])
    L = lib()
    return np.array([L.orc_ramp(int(cfg["ramp_init"]), int(cfg["ramp_flags"]), lp, float(tt),
                                float(xx), float(yy))
                     for xx, yy, tt in zip(np.ravel(x), np.ravel(y), np.ravel(t))])


class Sgrid:
    """lsGridSpline restatement (orc_sgrid) driven by a Sea."""

    def __init__(self, cfg: dict, sea: Sea, nthreads=0, init=True, pressure=False):
        g = cfg["lsgrid"]
        self.cfg, self.sea = cfg, sea
        d, dp = _arr(g["domain"])
        di, dip = _arr(g["domain_ignore"])
        self.h = lib().orc_sgrid_create(g["nx"], g["ny"], g["nl"], dp, dip, g["t0"], g["dt"],
                                        g["tan_a"], g["tan_b"], cfg["depth"], cfg["swl"])
        self.pressure = bool(pressure)
        if pressure:
            lib().orc_sgrid_set_pressure(self.h, 1)
        if init:
            lib().orc_sgrid_init(self.h, sea.h, int(g["ignore_at_init"]), nthreads)

    def __del__(self):
        try:
            lib().orc_sgrid_free(self.h)
        except Exception:
            pass

    def update(self, nthreads=0):
        lib().orc_sgrid_update(self.h, self.sea.h, nthreads)

    def force_update(self, t, nthreads=0):
        """wave_force_update (CFDwavemaker.cpp:2253-2262)."""
        while lib().orc_sgrid_check_time(self.h, float(t)):
            self.update(nthreads)

    def update_columns(self, t, c0, c1, nthreads=0):
        lib().orc_sgrid_update_columns(self.h, self.sea.h, float(t), int(c0), int(c1), nthreads)

    def advance(self):
        lib().orc_sgrid_advance(self.h)

    def gradients(self):
        lib().orc_sgrid_gradients(self.h)

    def set_slot(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if lib().orc_sgrid_set_slot(self.h, int(which), a.ctypes.data_as(_dp)) != 0:
            raise ValueError(which)

    def query(self, x, y, z, t, nthreads=0):
        """[n][4] eta, u, v, w; with the pressure field [n][5] (and p)."""
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 5 if self.pressure else 4))
        fn = lib().orc_sgrid_query5 if self.pressure else lib().orc_sgrid_query
        fn(self.h, n, p[0], p[1], p[2], p[3], out.ctypes.data_as(_dp), nthreads)
        return out

    def export_vtu(self, path, last=False, label="TimeValue"):
        """lsGridSpline::export_vtu into the file `path`."""
        if lib().orc_sgrid_export_vtu(self.h, str(path).encode(), int(bool(last)), label.encode()) != 0:
            raise OSError("cannot write " + str(path))

    def array(self, which):
        n = lib().orc_sgrid_array(self.h, which, None)
        out = np.zeros(n)
        lib().orc_sgrid_array(self.h, which, out.ctypes.data_as(_dp))
        return out

    def state(self):
        t0 = C.c_double()
        ts = C.c_int()
        lib().orc_sgrid_state(self.h, C.byref(t0), C.byref(ts))
        return t0.value, ts.value


class Stokes5:
    def __init__(self, cfg: dict):
        self.cfg = cfg
        self.h = lib().orc_stokes5_create(cfg["wave_length"], cfg["wave_height"], cfg["depth"],
                                          cfg["current"], cfg["gravity"], cfg["rho"],
                                          cfg["x_pos"], cfg["y_pos"], cfg["swl"], cfg["tofmax"],
                                          cfg["mtheta"])

    def __del__(self):
        try:
            lib().orc_stokes5_free(self.h)
        except Exception:
            pass

    def fields(self, x, y, z, t, nthreads=0):
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 5))
        lib().orc_stokes5_batch(self.h, n, p[0], p[1], p[2], p[3], out.ctypes.data_as(_dp), nthreads)
        return out

    def coeffs(self):
        out = np.zeros(32)
        lib().orc_stokes5_coeffs(self.h, out.ctypes.data_as(_dp))
        return out


class Fenton:
    def __init__(self, cfg: dict):
        st = C.c_int(0)
        self.cfg = cfg
        self.h = lib().orc_fenton_create(cfg["wave_height"], cfg["wave_length"], cfg["wave_period"],
                                         int(cfg["regular_specify_length"]), 0, cfg["wave_order"], 5,
                                         cfg["depth"], cfg["current"], cfg["gravity"], cfg["rho"],
                                         cfg["x_pos"], cfg["y_pos"], cfg["swl"], cfg["tofmax"],
                                         cfg["mtheta"], C.byref(st))
        self.status = st.value
        if not self.h:
            raise RuntimeError("Fenton solve failed, status %d" % self.status)

    def __del__(self):
        try:
            lib().orc_fenton_free(self.h)
        except Exception:
            pass

    def fields(self, x, y, z, t, nthreads=0):
        n, p, keep = _pts(x, y, z, t)
        out = np.zeros((n, 5))
        lib().orc_fenton_batch(self.h, n, p[0], p[1], p[2], p[3], out.ctypes.data_as(_dp), nthreads)
        return out

    def solution(self):
        out = np.zeros(6 + 2 * self.cfg["wave_order"])
        n = lib().orc_fenton_solution(self.h, out.ctypes.data_as(_dp))
        return out[:n]


class Model:
    """The reference's public point API semantics on the oracle
    (wave_SurfElev / wave_VeloX/Y/Z / wave_DynPres / wave_nhPres,
    CFDwavemaker.cpp:1543-1988): ramp x kinematics, z clamped to the seabed."""

    def __init__(self, cfg: dict, nthreads=0):
        self.cfg = cfg
        wt = cfg["wavetype"]
        self.sea = self.grid = self.reg = None
        if wt in (1, 5):
            self.sea = Sea(cfg)
        if wt == 5:
            self.grid = Sgrid(cfg, self.sea, nthreads)
        if wt == 21:
            self.reg = Fenton(cfg) if cfg["regular_theory"] == 1 else Stokes5(cfg)

    def api(self, x, y, z, t, nthreads=0):
        """[n,6]: SurfElev, VeloX, VeloY, VeloZ, DynPres, nhPres."""
        x, y, z, t = [np.ascontiguousarray(np.ravel(a), dtype=np.float64) for a in np.broadcast_arrays(x, y, z, t)]
        cfg = self.cfg
        zc = np.maximum(-cfg["depth"], z)
        r = ramp(cfg, x, y, t)
        out = np.zeros((x.size, 6))
        wt = cfg["wavetype"]
        if wt == 1:
            f = self.sea.fields(x, y, zc, t, 31, nthreads)
            if cfg.get("vertical_theory") == 1:
                # u, v, w, dp of the Smit s-coordinate theory (Irregular.cpp:25, 53, 77, 143)
                f[:, 1:5] = self.sea.smit(x, y, zc, t, nthreads)
            out[:, 0:5] = r[:, None] * f
            out[:, 5] = r * (f[:, 4] - cfg["rho"] * cfg["gravity"] * f[:, 0])
        elif wt == 5:
            q0 = self.grid.query(x, y, np.zeros_like(x), t, nthreads)
            q = self.grid.query(x, y, zc, t, nthreads)
            out[:, 0] = q0[:, 0] * r
            out[:, 1:4] = q[:, 1:4] * r[:, None]
        elif wt == 21:
            f = self.reg.fields(x, y, zc, t, nthreads)
            fe = self.reg.fields(x, y, z, t, nthreads)
            out[:, 0] = r * fe[:, 0]
            out[:, 1:4] = r[:, None] * f[:, 1:4]
            out[:, 5] = r * f[:, 4]
        return out
