"""Record golden vectors from the unmodified reference (oystelan/CFDwavemaker v3.1.0).

Run here, where the reference tree exists:

    make -C oracle ref          # compiles the reference sources into oracle/_ref/
    python tests/golden/make_golden.py

Each case writes a ``waveinput.dat`` into a scratch directory and runs the
reference in a fresh subprocess (its state lives in global singletons,
CFDwavemaker.cpp:129-163): ``wave_Initialize`` through the reference's own C
API, then the public ``wave_*`` queries and a few internal arrays
(oracle/ref_probe.cpp).  The outputs, the inputs and the ``waveinput.dat``
text are stored as ``tests/golden/<case>.npz``.  Two cases also keep a
subsample of the reference's own golden vectors
(tests/t005_focused_wave/targetwave.dat,
tests/t002_spline_momentum_conservation/exact_solution.mat).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_TREE = "/root/reference"
REF_LIB = os.path.join(REPO, "oracle", "_ref", "libcfdwm_ref.so")
sys.path.insert(0, REPO)

_dp = C.POINTER(C.c_double)


def _p(a):
    return a.ctypes.data_as(_dp)


# ----------------------------------------------------------------------------
# child side: one case per process
# ----------------------------------------------------------------------------
def child(case_dir, spec_json, out_path):
    spec = json.loads(spec_json)
    L = C.CDLL(REF_LIB)
    L.refp_init.restype = C.c_int
    L.refp_init.argtypes = [C.c_char_p]
    L.refp_api.argtypes = [C.c_int, C.c_long, _dp, _dp, _dp, _dp, _dp]
    L.refp_irr.argtypes = [C.c_int, C.c_long, _dp, _dp, _dp, _dp, _dp]
    L.refp_components.restype = C.c_int
    L.refp_components.argtypes = [_dp]
    L.refp_npairs.restype = C.c_long
    L.refp_force_update.argtypes = [C.c_double]
    L.refp_sgrid_dims.argtypes = [C.POINTER(C.c_int), _dp]
    L.refp_sgrid_array.restype = C.c_long
    L.refp_sgrid_array.argtypes = [C.c_int, _dp]
    L.refp_fenton.restype = C.c_int
    L.refp_fenton.argtypes = [_dp]
    L.refp_sgrid_export_vtu.restype = C.c_int
    L.refp_sgrid_export_vtu.argtypes = [C.c_char_p, C.c_int]
    rc = L.refp_init(case_dir.encode())
    res = {"rc": np.array(rc)}
    with open(os.path.join(case_dir, "waveinput.dat")) as fh:
        res["waveinput"] = np.array(fh.read())
    pts = {k: np.ascontiguousarray(spec["points"][k], dtype=np.float64) for k in "xyzt"}
    n = pts["x"].size
    for k in "xyzt":
        res["pt_" + k] = pts[k]
    kind = spec["kind"]
    if kind in ("irregular", "regular"):
        for name, which in (("SurfElev", 0), ("VeloX", 1), ("VeloY", 2), ("VeloZ", 3),
                            ("DynPres", 4), ("nhPres", 5), ("VFrac", 6)):
            o = np.zeros(n)
            L.refp_api(which, n, _p(pts["x"]), _p(pts["y"]), _p(pts["z"]), _p(pts["t"]), _p(o))
            res["api_" + name] = o
    if kind == "irregular":
        nc = L.refp_components(None)
        comp = np.zeros(8 * nc)
        L.refp_components(_p(comp))
        res["components"] = comp.reshape(8, nc)
        res["npairs"] = np.array(L.refp_npairs())
        for name, which in (("eta1", 0), ("eta2", 1), ("u2", 2), ("v2", 3), ("w2", 4), ("dp2", 5)):
            o = np.zeros(n)
            L.refp_irr(which, n, _p(pts["x"]), _p(pts["y"]), _p(pts["z"]), _p(pts["t"]), _p(o))
            res["irr_" + name] = o
        o = np.zeros(4 * n)
        zz = np.minimum(0.0, pts["z"])
        L.refp_irr(6, n, _p(pts["x"]), _p(pts["y"]), _p(zz), _p(pts["t"]), _p(o))
        res["irr_uvw2"] = o.reshape(n, 4)
        res["irr_uvw2_z"] = zz
    if kind == "helpers":
        # the irregular sea's spectral helpers (Irregular.cpp:1372-1437 through
        # CFDwavemaker.cpp's wave_* exports) and the water depth
        for name in ("wave_mean_period", "wave_phase_speed", "wave_mean_length"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_int]
        L.wave_water_depth.restype = C.c_double
        res["helpers"] = np.array([L.wave_mean_period(1), L.wave_mean_period(2), L.wave_phase_speed(1),
                                   L.wave_phase_speed(2), L.wave_mean_length(1), L.wave_mean_length(2),
                                   L.wave_water_depth()])
    if kind == "regular" and spec.get("fenton"):
        o = np.zeros(6 + 2 * 64)
        q = L.refp_fenton(_p(o))
        res["fenton_solution"] = o[:q]
    if kind == "sgrid":
        dims = (C.c_int * 4)()
        vals = np.zeros(5)
        steps = spec.get("updates", [])
        snaps = []
        for k in range(len(steps) + 1):
            if k > 0:
                L.refp_force_update(steps[k - 1])
            L.refp_sgrid_dims(dims, _p(vals))
            snap = {"dims": np.array(list(dims)), "vals": vals.copy()}
            for which in range(19):
                m = L.refp_sgrid_array(which, None)
                a = np.zeros(m)
                L.refp_sgrid_array(which, _p(a))
                snap["arr%d" % which] = a
            qt = np.ascontiguousarray(spec["query_t"][k], dtype=np.float64)
            qx = np.ascontiguousarray(spec["query_x"], dtype=np.float64)
            qy = np.ascontiguousarray(spec["query_y"], dtype=np.float64)
            qz = np.ascontiguousarray(spec["query_z"], dtype=np.float64)
            qtt = np.full(qx.size, qt)
            o = np.zeros(4 * qx.size)
            L.refp_api(7, qx.size, _p(qx), _p(qy), _p(qz), _p(qtt), _p(o))
            snap["kin"] = o.reshape(-1, 4)
            for name, which in (("SurfElev", 0), ("VeloX", 1), ("VeloY", 2), ("VeloZ", 3)):
                o = np.zeros(qx.size)
                L.refp_api(which, qx.size, _p(qx), _p(qy), _p(qz), _p(qtt), _p(o))
                snap["api_" + name] = o
            snap["query_t"] = qt
            if spec.get("vtu"):
                # the file the reference wrote itself for this ring ([lsgrid2vtk])
                # and the export of the slot after the base slot
                v = spec["vtu"]
                auto = os.path.join(case_dir, v["path"], "%s%05d.vtu" % (v["prefix"], int(dims[3])))
                with open(auto) as fh:
                    snap["vtu"] = np.array(fh.read())
                last = os.path.join(case_dir, "last.vtu")
                assert L.refp_sgrid_export_vtu(last.encode(), 1) == 0
                with open(last) as fh:
                    snap["vtu_last"] = np.array(fh.read())
            snaps.append(snap)
        res["nsnap"] = np.array(len(snaps))
        for k, snap in enumerate(snaps):
            for key, v in snap.items():
                res["s%d_%s" % (k, key)] = v
        res["query_x"] = np.asarray(spec["query_x"])
        res["query_y"] = np.asarray(spec["query_y"])
        res["query_z"] = np.asarray(spec["query_z"])
    for key, v in spec.get("extra", {}).items():
        res["extra_" + key] = np.asarray(v)
    np.savez_compressed(out_path, **res)


# ----------------------------------------------------------------------------
# parent side: the cases
# ----------------------------------------------------------------------------
def _grid_points(xs, ys, zs, ts):
    X, Y, Z, T = np.meshgrid(xs, ys, zs, ts, indexing="ij")
    return {"x": X.ravel().tolist(), "y": Y.ravel().tolist(), "z": Z.ravel().tolist(),
            "t": T.ravel().tolist()}


ONLY = set()     # case names given on the command line (none: every case)


def _run_case(name, text, spec):
    if ONLY and name not in ONLY:
        return
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "waveinput.dat"), "w") as fh:
            fh.write(text)
        out = os.path.join(HERE, name + ".npz")
        r = subprocess.run([sys.executable, __file__, "--child", d, json.dumps(spec), out],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("case %s failed:\n%s\n%s" % (name, r.stdout[-2000:], r.stderr[-2000:]))
        print("wrote", out, os.path.getsize(out), "bytes")


def main():
    from cfdwavemaker_gb300 import seastate as ss
    if not os.path.exists(REF_LIB):
        raise SystemExit("build the reference first: make -C oracle ref")
    rng = np.random.default_rng(7)

    # (1) t005 focused wave: the reference's own golden elevation series.
    with open(os.path.join(REF_TREE, "tests/t005_focused_wave/waveinput.dat")) as fh:
        t005 = fh.read()
    tgt = np.loadtxt(os.path.join(REF_TREE, "tests/t005_focused_wave/targetwave.dat"))
    sel = np.arange(0, tgt.shape[0], 8)
    ts = tgt[sel, 0]
    spec = {"kind": "irregular",
            "points": {"x": [10.0] * ts.size, "y": [0.0] * ts.size, "z": [-0.1] * ts.size,
                       "t": ts.tolist()},
            "extra": {"targetwave_t": ts.tolist(), "targetwave_eta": tgt[sel, 1].tolist()}}
    _run_case("t005_focused", t005, spec)

    # (2) t002 exact solution: elevation and momentum integrals at (0,0).
    from scipy.io import loadmat
    mat = loadmat(os.path.join(REF_TREE, "tests/t002_spline_momentum_conservation/exact_solution.mat"))
    with open(os.path.join(REF_TREE, "tests/t002_spline_momentum_conservation/waveinput_exact.dat")) as fh:
        t002 = fh.read()
    tt = np.arange(0, 20, 0.05)
    pts = _grid_points([0.0], [0.0], [-20.0, -5.0, 0.0, 2.0], tt[::40])
    spec = {"kind": "irregular", "points": pts,
            "extra": {"time": tt.tolist(), "wave_elev1": np.squeeze(mat["wave_elev1"]).tolist(),
                      "umom1": np.squeeze(mat["umom1"]).tolist(),
                      "vmom1": np.squeeze(mat["vmom1"]).tolist(),
                      "wmom1": np.squeeze(mat["wmom1"]).tolist()}}
    _run_case("t002_exact", t002, spec)

    # (3) the 128-component long-crested JONSWAP sea (depth 50 m), point API.
    comps = ss.config1_sea()
    txt = ss.write_irregular(None, comps, 50.0, extrap=2)
    pts = _grid_points([0.0, 137.5, 321.0, 500.0], [0.0], [-50.0, -31.0, -12.5, -3.0, 0.0, 1.5, 3.5],
                       [0.0, 3.0, 7.0])
    _run_case("config1_point", txt, {"kind": "irregular", "points": pts})

    # (4) short-crested, ndir>0 spreading format, bandwidth + cutoff filters.
    om = np.linspace(0.4, 1.6, 24)
    kk = ss.dispersion_k(om, 30.0)
    A = 0.2 * np.sqrt(ss.jonswap(om, 3.0, 9.0, 3.3) * (om[1] - om[0]) * 2)
    ph = rng.uniform(0, 2 * math.pi, om.size)
    th = np.linspace(-0.6, 0.6, 5)
    D = ss.cos2s_weights(th, 6.0)
    L = ["@v310", "[wave type]", "irregular", "[general input data]", "depth 30", "mtheta 12.5",
         "rho 1025", "[wave reference point]", "time 4.0", "x 3.0", "y -2.0",
         "[wave input irregular]", "kinematics_surf_extrap 2", "bandwidth 0.3", "cutoff 1.45",
         "nfreq %d" % om.size, "ndir %d" % th.size]
    for i in range(om.size):
        L.append("%.17g %.17g %.17g %.17g" % (om[i], A[i], kk[i], ph[i]))
    for j in range(th.size):
        L.append("%.17g %.17g" % (th[j], math.sqrt(D[j])))
    txt = "\n".join(L) + "\n"
    pts = _grid_points([-20.0, 15.0], [-7.0, 11.0], [-30.0, -9.0, -0.5, 0.8], [0.0, 5.5])
    _run_case("short_spread", txt, {"kind": "irregular", "points": pts})

    # (5) ramps, individual ramps, swl, mtheta, normalize + amplify.
    comps = ss.irregular_components(2.0, 7.0, 3.3, 20, 0.5, 1.8, 25.0, 11, ndir=3, spreading_s=4.0)
    n = comps["omega"].size
    rcols = [rng.uniform(0.5, 3.0, n), rng.uniform(-1.0, 2.0, n), rng.uniform(20.0, 60.0, n)]
    txt = ss.write_irregular(None, comps, 25.0, extrap=2, swl=0.7, mtheta=20.0, gravity=9.80665,
                             rho=1000.0, ref_point=(2.0, 1.0, -1.0), normalize=1, amplify=1.5,
                             ramps={"time_rampup": (0.0, 4.0), "x_rampdown": (40.0, 90.0),
                                    "y_rampup": (-30.0, -10.0)},
                             ramp_columns=rcols)
    pts = _grid_points([0.0, 60.0], [-20.0, 5.0], [-25.0, -6.0, 0.7, 1.9], [-0.5, 1.0, 3.3, 9.0])
    _run_case("ramps_swl", txt, {"kind": "irregular", "points": pts})

    # (5b) vertical_theory smit (Smit et al. 2017 s-coordinate second order,
    #      Irregular.cpp:1622-2027): a short-crested sea with pair filters and
    #      swl, and one with individual ramps; points below, at and above the
    #      surface.
    comps = ss.irregular_components(2.5, 8.0, 2.5, 10, 0.45, 1.6, 30.0, 17, ndir=3, spreading_s=6.0)
    txt = ss.write_irregular(None, comps, 30.0, extrap=2, swl=0.4, mtheta=25.0, rho=1025.0, bandwidth=0.6,
                             cutoff=1.5, vertical_theory="smit")
    pts = _grid_points([-12.0, 7.5, 31.0], [3.0, -9.0], [-30.0, -17.0, -4.0, -0.6, 0.2, 1.1, 3.5], [0.0, 4.2])
    _run_case("smit_spread", txt, {"kind": "irregular", "points": pts})
    comps = ss.irregular_components(3.0, 9.0, 2.0, 14, 0.4, 1.5, 50.0, 29, ndir=3, spreading_s=4.0)
    n = comps["omega"].size
    r5 = np.random.default_rng(505)    # own stream: the cases after this one keep theirs
    rcols = [r5.uniform(1.0, 4.0, n), r5.uniform(-1.0, 1.0, n), r5.uniform(30.0, 80.0, n)]
    txt = ss.write_irregular(None, comps, 50.0, extrap=2, ramp_columns=rcols, vertical_theory="smit")
    pts = _grid_points([0.0, 22.0], [0.0, 5.0], [-50.0, -20.0, -5.0, -1.0, 0.0, 0.9], [0.5, 2.5, 6.0])
    _run_case("smit_ramps", txt, {"kind": "irregular", "points": pts})

    # (6) linear theory (kinematics_surf_extrap 0, unclipped above swl).
    comps = ss.irregular_components(3.0, 8.0, 2.0, 30, 0.4, 1.9, 40.0, 5)
    txt = ss.write_irregular(None, comps, 40.0, extrap=0, swl=0.3)
    pts = _grid_points([0.0, 30.0], [0.0], [-40.0, -10.0, 0.0, 1.0, 2.5], [0.0, 2.0])
    _run_case("linear", txt, {"kind": "irregular", "points": pts})

    # (7) s-grid: init, two ring updates, queries.
    comps = ss.irregular_components(3.0, 9.0, 2.0, 12, 0.45, 1.5, 40.0, 21, ndir=4, spreading_s=8.0)
    grid = {"bounds": (-60.0, 60.0, -40.0, 40.0), "nx": 9, "ny": 7, "nl": 6, "t0": 0.0,
            "dt": 0.5, "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 40.0, extrap=2, lsgrid=grid)
    qx = rng.uniform(-70, 70, 60)
    qy = rng.uniform(-45, 45, 60)
    qz = rng.uniform(-42, 3.0, 60)
    spec = {"kind": "sgrid", "points": {"x": [0.0], "y": [0.0], "z": [0.0], "t": [0.0]},
            "updates": [0.7, 1.6], "query_t": [0.2, 0.8, 1.3],
            "query_x": qx.tolist(), "query_y": qy.tolist(), "query_z": qz.tolist()}
    _run_case("sgrid_small", txt, spec)

    # (8) s-grid with an ignore subdomain (frozen after init).  swl stays 0: with
    #     swl != 0 the reference's cart2sigmaS takes pow() of a negative number
    #     for eta - swl < z <= eta (lsgrid_spline.cpp:109-113) and then indexes
    #     its arrays with the NaN, which crashes wave_SurfElev (it queries z=0).
    #     ignore_at_init 1 is not recorded: the reference then leaves the ignored
    #     columns of its new[]-allocated arrays uninitialised
    #     (lsgrid_spline.cpp:756-790), so its queries there read garbage.
    grid = {"bounds": (0.0, 80.0, -30.0, 30.0), "nx": 8, "ny": 6, "nl": 5, "t0": 1.0,
            "dt": 0.4, "stretch": (0.6, 1.2), "ignore": (20.0, 60.0, -10.0, 10.0)}
    comps = ss.irregular_components(2.5, 8.0, 2.5, 10, 0.5, 1.6, 30.0, 33, ndir=3, spreading_s=6.0)
    txt = ss.write_irregular(None, comps, 30.0, extrap=2, lsgrid=grid)
    qx = rng.uniform(-5, 85, 40)
    qy = rng.uniform(-33, 33, 40)
    qz = rng.uniform(-31, 3.0, 40)
    spec = {"kind": "sgrid", "points": {"x": [0.0], "y": [0.0], "z": [0.0], "t": [0.0]},
            "updates": [1.5], "query_t": [1.1, 1.7],
            "query_x": qx.tolist(), "query_y": qy.tolist(), "query_z": qz.tolist()}
    _run_case("sgrid_ignore", txt, spec)

    # (8b) .vtu output of the s-grid ([lsgrid2vtk], lsgrid_spline.cpp:1200-1403):
    #      the files the reference writes at init and after an update, and the
    #      export of the slot after the base slot; a 3-D grid and one that is
    #      flat in y (quad cells).
    for name, nx, ny, nl, bounds in (("sgrid_vtu", 6, 5, 4, (-30.0, 30.0, -20.0, 20.0)),
                                     ("sgrid_vtu_flat", 7, 1, 5, (-30.0, 30.0, 0.0, 0.0))):
        vtk = {"path": "vtk/", "prefix": "kin", "label": "TimeValue"}
        grid = {"bounds": bounds, "nx": nx, "ny": ny, "nl": nl, "t0": 0.5, "dt": 0.5, "stretch": (0.7, 1.5),
                "vtk": vtk}
        comps = ss.irregular_components(3.0, 9.0, 2.0, 8, 0.45, 1.5, 40.0, 41, ndir=3, spreading_s=8.0)
        txt = ss.write_irregular(None, comps, 40.0, extrap=2, lsgrid=grid)
        spec = {"kind": "sgrid", "points": {"x": [0.0], "y": [0.0], "z": [0.0], "t": [0.0]},
                "updates": [1.2], "query_t": [0.6, 1.1], "query_x": [0.0], "query_y": [0.0], "query_z": [-1.0],
                "vtu": vtk}
        _run_case(name, txt, spec)

    # (9) Stokes 5th (H=6 T=10 d=30) and Fenton (N=24 H=8 T=12 d=20), plus
    #     length-specified variants with direction, current and reference point.
    def reg_points(L_, d, H):
        xs = np.linspace(0, 2 * L_, 5)
        zs = np.linspace(-d, 0.6 * H, 5)
        return _grid_points(xs.tolist(), [0.0, 7.0], zs.tolist(), [0.0, 2.5, 7.1])
    for name, txt, L_, d, H in (
            ("stokes5", ss.write_regular(None, "stokes", 6.0, 30.0, period=10.0), 130.0, 30.0, 6.0),
            ("fenton24", ss.write_regular(None, "stream", 8.0, 20.0, period=12.0, order=24), 160.0, 20.0, 8.0),
            ("stokes5_len", ss.write_regular(None, "stokes", 3.0, 15.0, length=60.0, mtheta=30.0,
                                             swl=0.4, rho=1025.0, ref_point=(1.0, 2.0, 3.0)), 60.0, 15.0, 3.0),
            ("fenton_len", ss.write_regular(None, "stream", 2.0, 10.0, length=40.0, order=16,
                                            current=0.3, mtheta=-15.0, rho=1000.0,
                                            ref_point=(0.5, 1.0, -2.0)), 40.0, 10.0, 2.0)):
        _run_case(name, txt, {"kind": "regular", "points": reg_points(L_, d, H),
                              "fenton": name.startswith("fenton")})

    # (10) spectral helpers of the irregular sea (wave_mean_period,
    #      wave_phase_speed, wave_mean_length for opt 1 and 2, wave_water_depth)
    one = {"x": [0.0], "y": [0.0], "z": [0.0], "t": [0.0]}
    _run_case("helpers_config1", ss.write_irregular(None, ss.config1_sea(), 50.0, extrap=2),
              {"kind": "helpers", "points": one})
    _run_case("helpers_t005", t005, {"kind": "helpers", "points": one})

    # (11) Fenton set-ups that the Newton iteration does not solve, with the
    #      reference's own outcome: a wave near the highest one (warning, the
    #      unconverged iterate is served), one beyond it (warning, NaN
    #      coefficients served) and a steep deep-water wave whose Jacobian
    #      turns singular (FentonStream.cpp:200-201 throws; the process ends).
    if not ONLY or "fenton_fail" in ONLY:
        res = {}
        for tag, (H, d, T) in (("nonconv", (19.0, 20.0, 12.0)), ("nan", (30.0, 20.0, 12.0)),
                               ("singular", (15.0, 20.0, 3.0))):
            txt = ss.write_regular(None, "stream", H, d, period=T, order=24)
            with tempfile.TemporaryDirectory() as dd:
                with open(os.path.join(dd, "waveinput.dat"), "w") as fh:
                    fh.write(txt)
                out = os.path.join(dd, "o.npz")
                spec = {"kind": "regular", "points": one, "fenton": True}
                r = subprocess.run([sys.executable, __file__, "--child", dd, json.dumps(spec), out],
                                   capture_output=True, text=True)
                msg = r.stdout + r.stderr
                res[tag + "_waveinput"] = np.array(txt)
                res[tag + "_exit_ok"] = np.array(r.returncode == 0)
                res[tag + "_warned"] = np.array("did not fully converge" in msg)
                res[tag + "_singular"] = np.array("singular Jacobian" in msg)
                if r.returncode == 0:
                    res[tag + "_solution"] = np.load(out)["fenton_solution"]
        out = os.path.join(HERE, "fenton_failures.npz")
        np.savez_compressed(out, **res)
        print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--child":
        child(sys.argv[2], sys.argv[3], sys.argv[4])
    else:
        ONLY.update(sys.argv[1:])
        main()
