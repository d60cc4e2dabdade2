"""Benchmark of the second-order point-kinematics path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload qform|sgrid|point]

Workloads (synthetic seeded sea states of the named shapes; no dataset):
  qform  (default) precision form: short-crested JONSWAP Hs=6 m Tp=12 s
         gamma=2, cos-2s s=10, 256 frequencies x 16 directions = 4096
         components, depth 100 m; second-order eta and z=0 / Taylor-layer
         u, v, w at 4e6 random (x, y, t) points as split 16-bit tcgen05 GEMMs
         (fp16x3 and bf16x3), beside the plain FP32 CUDA-core form; errors of
         every field against the FP64 oracle on a row sample.
  sgrid  the same sea at 64 x 16 = 1024 components; an s-grid of 256 x 256
         columns x 16 sigma levels over 1 km x 1 km at dt = 0.5 s.  One step
         = one ring update (second-order kinematics at all 1,048,576 grid
         nodes: eta2 + uvw2 pair sums over 521k pairs) plus the 4-D spline
         query of 1e6 uniformly random (x, y, z, t) points.
  point  long-crested JONSWAP Hs=4 m Tp=10 s gamma=3.3, 128 components,
         depth 50 m; eta, u, w, dp on 256 x-points x 32 z-points x 8 times.
Metric: second-order points per second (grid nodes updated per second for
sgrid).  The reference arm times the FP64 CPU restatement (oracle/) on a
bounded sample of the same workload with all host threads.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import ctypes as C

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "2nd-order pts/s at <=1e-5 rel err vs FP64: split-BF16 TC & surrogate vs plain"


def sgrid_config(nx=256, ny=256, nl=16, dt=0.5):
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea()
    grid = {"bounds": (0.0, 1000.0, 0.0, 1000.0), "nx": nx, "ny": ny, "nl": nl, "t0": 0.0,
            "dt": dt, "stretch": (0.7, 1.5)}
    return ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)


SURR_WORKLOAD = ("learned s-grid update: the 1024-component short-crested JONSWAP sea (Hs 6 m, Tp 12 s, gamma 2, "
                 "cos-2s s=10, depth 100 m) on the 256x256x16 s-grid over 1 km^2, %d ring steps at dt 0.1 s, "
                 "a full plain update every %d steps, the others predicted by the conv operator (4 layers, 32 "
                 "channels, 3x3, BF16 weights) and checked on %d sampled columns against the plain method "
                 "(fallback above tol %g); + 1e5 random spline queries per step")


def run_surrogate(args):
    """Learned s-grid update against the plain update on the same grid.

    value: grid nodes updated per second over the surrogate-assisted loop
    (plain every --plain-every steps, the others predicted and checked,
    routed through wave_force_update with cfdwm_surrogate_enable); the plain
    rate is the same loop with every update plain (timed on fewer steps,
    its cost per step is constant).  Accuracy: max errors of eta and U
    against a full plain fill at 4 points of a 20-step window (unchecked
    prediction).  The target tolerance 1e-3 is run too, on a short loop, and
    its fallback fraction reported."""
    import torch
    import cfdwavemaker_gb300 as cw
    from cfdwavemaker_gb300 import surrogate as S
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = cw.load()
    os.chdir(tempfile.mkdtemp())
    wm = cw.CFDwavemaker()
    txt = sgrid_config(256, 256, 16, dt=0.1)
    nodes = 256 * 256 * 16
    stream = torch.cuda.current_stream()
    lib.cfdwm_set_stream(C.c_void_p(stream.cuda_stream))
    nq = 100_000
    rng = np.random.default_rng(4321 + rank)
    qx, qy, qz = rng.uniform(0, 1000, nq), rng.uniform(0, 1000, nq), rng.uniform(-100, 6.0, nq)
    dq = [torch.tensor(a, device="cuda", dtype=torch.float64) for a in (qx, qy, qz)]
    dtq = torch.empty(nq, device="cuda", dtype=torch.float64)
    dout = torch.empty((nq, 4), device="cuda", dtype=torch.float64)
    hq = [np.ascontiguousarray(a) for a in (qx, qy, qz)]
    htq = np.empty(nq)
    hout = np.empty((nq, 4))

    def ok(rc):
        assert rc == 0, (rc, cw.last_error())

    def fresh(weights=True, method=0):
        # the plain steps of this workload are the plain FP32 form (method 0)
        # unless the tensor-core s-grid form is asked for
        ok(wm.initialize_text(txt))
        ok(lib.cfdwm_sgrid_method(method, None))
        if weights:
            ok(lib.cfdwm_surrogate_load(S.WEIGHTS.encode()))

    def loop(nsteps, host=False):
        t0, _ = wm.sgrid_state()
        t = t0
        for _ in range(nsteps):
            t += 0.1
            lib.wave_force_update(t + 1e-9)
            ts, _ = wm.sgrid_state()
            if host:
                htq.fill(ts + 0.05)
                ok(lib.wave_Kinematics_batch(*[cw._ptr(a) for a in hq], cw._ptr(htq), nq, cw._ptr(hout)))
            else:
                dtq.fill_(ts + 0.05)
                ok(lib.wave_Kinematics_batch(*[cw._ptr(a) for a in dq], cw._ptr(dtq), nq, cw._ptr(dout)))

    def timed(nsteps, host=False):
        torch.cuda.synchronize()
        l0 = lib.cfdwm_kernel_launches()
        if host:
            c0 = time.perf_counter()
            loop(nsteps, host=True)
            torch.cuda.synchronize()
            return (time.perf_counter() - c0) * 1e3 / nsteps, lib.cfdwm_kernel_launches() - l0
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        loop(nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps, lib.cfdwm_kernel_launches() - l0

    res = {"ws": ws, "rank": rank}
    # plain every step
    fresh(weights=False)
    ok(lib.cfdwm_surrogate_enable(0, 1, 0.0, 0))
    loop(max(1, args.warmup))
    lib.cfdwm_profile_enable(1)
    lib.cfdwm_profile_read(0, None)
    ms_plain, _ = timed(args.plain_steps)
    tot = C.c_double(0.0)
    nk = lib.cfdwm_profile_read(0, C.byref(tot))
    lib.cfdwm_profile_enable(0)
    res["plain"] = {"ms_per_step": ms_plain, "steps": args.plain_steps, "nodes_per_s": nodes / (ms_plain / 1e3),
                    "column_pairs": {"launches": int(nk), "avg_ms": tot.value / max(1, nk)}}
    res["npairs"] = int(lib.cfdwm_npairs())
    res["ncomp"] = int(lib.cfdwm_components(None))
    # the tensor-core s-grid form every step, and the learned update with its
    # plain steps on that form (context for the comparison above)
    fresh(weights=False, method=1)
    loop(max(1, args.warmup))
    ms_tc, _ = timed(args.plain_steps)
    res["tc_every_step"] = {"ms_per_step": ms_tc, "nodes_per_s": nodes / (ms_tc / 1e3)}
    fresh(method=1)
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, args.surr_tol, args.nsample))
    loop(max(1, args.warmup))
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, args.surr_tol, args.nsample))
    ms_stc, _ = timed(args.surr_steps)
    res["surrogate_tc_plain"] = {"ms_per_step": ms_stc, "nodes_per_s": nodes / (ms_stc / 1e3),
                                 "speedup_vs_tc_every_step": ms_tc / ms_stc}
    ok(lib.cfdwm_surrogate_enable(0, 1, 0.0, 0))
    # surrogate-assisted loop at the working tolerance
    fresh()
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, args.surr_tol, args.nsample))
    loop(max(1, args.warmup))
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, args.surr_tol, args.nsample))
    lib.cfdwm_profile_enable(1)
    for k in range(9):
        lib.cfdwm_profile_read(k, None)
    sampler = ClockSampler(local)
    sampler.start()
    barrier(ws)
    ms, launches = timed(args.surr_steps)
    clocks = sampler.stop()
    prof = {}
    for k, name in enumerate(["column_pairs", "eta_pairs", "point_pairs", "phasors", "query", "gradients",
                              "qform", "surr_features", "surr_net"]):
        tot = C.c_double(0.0)
        nk = lib.cfdwm_profile_read(k, C.byref(tot))
        if nk > 0:
            prof[name] = {"launches": int(nk), "avg_ms": tot.value / nk, "total_ms": tot.value}
    lib.cfdwm_profile_enable(0)
    st = [C.c_long(0) for _ in range(3)]
    ok(lib.cfdwm_surrogate_stats(*[C.byref(v) for v in st]))
    res.update(ms=ms, launches=launches, clocks=clocks, prof=prof,
               stats={"predicted": st[0].value, "fell_back": st[1].value, "plain": st[2].value})
    # end to end (host query arrays), same loop
    fresh()
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, args.surr_tol, args.nsample))
    res["e2e_ms"], _ = timed(args.surr_steps, host=True)
    # the target tolerance, short loop
    fresh()
    ok(lib.cfdwm_surrogate_enable(1, args.plain_every, 1e-3, args.nsample))
    ms3, _ = timed(args.plain_every * 2)
    ok(lib.cfdwm_surrogate_stats(*[C.byref(v) for v in st]))
    res["tol_1e-3"] = {"ms_per_step": ms3, "steps": args.plain_every * 2, "predicted": st[0].value,
                       "fell_back": st[1].value, "nodes_per_s": nodes / (ms3 / 1e3)}
    ok(lib.cfdwm_surrogate_enable(0, 1, 0.0, 0))
    # accuracy over one window: unchecked predictions against full plain fills
    acc = {}
    for name, zero in (("network", False), ("first_order_only", True)):
        fresh()
        if zero:
            n = lib.cfdwm_surrogate_nparams()
            z = np.zeros(n, np.float32)
            ok(lib.cfdwm_surrogate_set_params(z.ctypes.data, n))
        rows = []
        for i in range(args.plain_every):
            ok(lib.cfdwm_surrogate_step(0 if i == 0 else 2, 0.0, 0, None, None))
            if i in (1, args.plain_every // 4, args.plain_every // 2, args.plain_every - 1):
                err = (C.c_double * 4)()
                ok(lib.cfdwm_surrogate_compare(err))
                rows.append([i] + [float(v) for v in err])
        acc[name] = {"rows_step_eta_u_v_w": rows,
                     "max_eta": max(r[1] for r in rows), "max_u": max(r[2] for r in rows),
                     "max_uvw": max(max(r[2:]) for r in rows)}
    res["accuracy"] = acc
    res["nodes"] = nodes
    res["h2d"] = 3 * 8 * nq + 8 * nq
    res["d2h"] = 4 * 8 * nq
    return res


REG_WORKLOAD = ("regular waves: Stokes 5th H=6 m T=10 s depth 30 m and Fenton stream function order 24 H=8 m "
                "T=12 s depth 20 m (FP64 Newton solve on the device), each evaluated (eta, u, v, w) at 1e7 points "
                "of a uniform x-z-t grid (500 x in [0, 2L], 100 z from the seabed to the crest, 200 t in [0, T))")


def regular_cases():
    from cfdwavemaker_gb300 import seastate as ss
    return [("stokes5", ss.write_regular(None, "stokes", 6.0, 30.0, period=10.0), 30.0, 6.0),
            ("fenton24", ss.write_regular(None, "stream", 8.0, 20.0, period=12.0, order=24), 20.0, 8.0)]


def run_regular(args):
    """The regular-wave workload: Stokes 5th and Fenton stream function at 1e7
    points each per step, through wave_Kinematics_batch (device arrays for
    value; host arrays for e2e)."""
    import torch
    import cfdwavemaker_gb300 as cw
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = cw.load()
    os.chdir(tempfile.mkdtemp())
    wm = cw.CFDwavemaker()
    stream = torch.cuda.current_stream()
    lib.cfdwm_set_stream(C.c_void_p(stream.cuda_stream))
    nx, nz, nt = 500, 100, 200
    cases = []
    for name, txt, depth, H in regular_cases():
        assert wm.initialize_text(txt) == 0, cw.last_error()
        L, T = wm.mean_length(1), wm.mean_period(1)
        xs = np.linspace(0.0, 2.0 * L, nx)
        zs = np.linspace(-depth, 0.75 * H, nz)
        ts = np.linspace(0.0, T, nt, endpoint=False)
        X, Z, TT = np.meshgrid(xs, zs, ts, indexing="ij")
        host = [np.ascontiguousarray(a.ravel()) for a in (X, np.zeros_like(X), Z, TT)]
        dev = [torch.tensor(a, device="cuda", dtype=torch.float64) for a in host]
        cases.append({"name": name, "txt": txt, "host": host, "dev": dev, "L": L, "T": T})
    n = nx * nz * nt
    dout = torch.empty((n, 4), device="cuda", dtype=torch.float64)
    hout = np.empty((n, 4))

    res = {"ws": ws, "rank": rank, "cases": {}}
    tot_ms, tot_e2e = 0.0, 0.0
    launches = 0
    clocks = None
    for c in cases:
        assert wm.initialize_text(c["txt"]) == 0, cw.last_error()
        p = [cw._ptr(a) for a in c["dev"]]
        for _ in range(args.warmup):
            assert lib.wave_Kinematics_batch(*p, n, cw._ptr(dout)) == 0
        torch.cuda.synchronize()
        lib.cfdwm_profile_enable(1)
        lib.cfdwm_profile_read(9, None)
        sampler = ClockSampler(local)
        sampler.start()
        l0 = lib.cfdwm_kernel_launches()
        # a step is about 1 ms: the timed region repeats it so that it spans
        # at least a few hundred ms of clock samples
        reps = max(args.steps, 400)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            assert lib.wave_Kinematics_batch(*p, n, cw._ptr(dout)) == 0
        e1.record(stream)
        torch.cuda.synchronize()
        launches += (lib.cfdwm_kernel_launches() - l0) * args.steps // reps
        ms = e0.elapsed_time(e1) / reps
        kt = C.c_double(0.0)
        nk = lib.cfdwm_profile_read(9, C.byref(kt))     # per launch, over the reps
        lib.cfdwm_profile_enable(0)
        ck = sampler.stop()
        clocks = ck if clocks is None else clocks
        hp = [cw._ptr(a) for a in c["host"]]
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            assert lib.wave_Kinematics_batch(*hp, n, cw._ptr(hout)) == 0
        e2e_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps // 2)
        res["cases"][c["name"]] = {"ms_per_eval": ms, "kernel_ms": kt.value / max(1, nk), "e2e_ms": e2e_ms,
                                   "pts_per_s": n / (ms / 1e3), "wave_length": c["L"], "period": c["T"]}
        tot_ms += ms
        tot_e2e += e2e_ms
    res.update(ms=tot_ms, e2e_ms=tot_e2e, n=n, launches=launches, clocks=clocks)
    return res


def regular_line(args, r):
    pk, src = peaks()
    ws = r["ws"]
    units = 2 * r["n"]
    value = units * ws / (r["ms"] / 1e3)
    # algorithmic bytes per point: x, y, z, t in (4 x 8 B) and eta, u, v, w out (4 x 8 B)
    kms = sum(c["kernel_ms"] for c in r["cases"].values())
    bytes_pt = 64.0
    ach = bytes_pt * units / (kms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 phase; FP64 Newton set-up)", "data": "synthetic",
        "config": {"workload": REG_WORKLOAD, "l2": "inputs larger than L2 (640 MB in, 320 MB out per case)"},
        "e2e": {"value": units * ws / (r["e2e_ms"] / 1e3), "unit": "points/s",
                "h2d_bytes_per_step": 2 * 32 * r["n"], "d2h_bytes_per_step": 2 * 32 * r["n"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "cases": r["cases"],
        "roofline": {"kernel": "k_regular_eval", "bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": ach / pk["hbm_gbs"], "traffic": traffic_from_profiles("k_regular_eval"),
                     "algorithmic": "64 B per point (x, y, z, t in; eta, u, v, w out; FP64)",
                     "peak_source": src + " HBM copy, MEASURED_PEAKS.json"},
        "peaks_source": src,
    }
    return line


def regular_cpu_baseline(budget_s=10.0):
    import oracle
    from oracle import waveinput
    nthr = os.cpu_count() or 1
    tot, npts = 0.0, 0
    for name, txt, depth, H in regular_cases():
        cfg = waveinput.read_text(txt)
        m = oracle.Model(cfg)
        rng = np.random.default_rng(3)
        n = 20000
        x = rng.uniform(0, 200, n); z = rng.uniform(-depth, 0, n); t = rng.uniform(0, 10, n)
        t0 = time.perf_counter()
        m.api(x, 0 * x, z, t, nthr)
        tot += time.perf_counter() - t0
        npts += n
    return {"value": npts / tot, "unit": "points/s", "cores": nthr, "kind": "port",
            "sample": "2 x 20000 random points, all API fields (Stokes5, Fenton 24), FP64 oracle"}


def surrogate_line(args, r):
    pk, src = peaks()
    n = r["ws"]
    value = r["nodes"] * n / (r["ms"] / 1e3)
    plain = r["plain"]["nodes_per_s"] * n
    prof = r["prof"]
    line = {
        "metric": METRIC, "value": value, "unit": "grid nodes/s", "n_gpus": n, "steps": args.surr_steps,
        "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 phases); network bf16 weights, f32 accumulate",
        "data": "synthetic",
        "config": {"workload": SURR_WORKLOAD % (args.surr_steps, args.plain_every, args.nsample, args.surr_tol),
                   "l2": "working set > L2 (grid 340 MB, phasor scratch 856 MB)"},
        "e2e": {"value": r["nodes"] * n / (r["e2e_ms"] / 1e3), "unit": "grid nodes/s",
                "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "plain_every_step": {"value": plain, "ms_per_step": r["plain"]["ms_per_step"],
                             "steps": r["plain"]["steps"], "form": "plain FP32 column sums"},
        "tensor_core_every_step": r["tc_every_step"],
        "surrogate_with_tensor_core_plain_steps": r["surrogate_tc_plain"],
        "speedup_vs_plain": value / plain,
        "surrogate_steps": r["stats"],
        "tol_1e-3": r["tol_1e-3"],
        "accuracy": r["accuracy"],
        "kernels": prof,
        "peaks_source": src,
    }
    # the dominant kernel is still the plain column pair sum (every plain-every-th
    # step); its roofline is taken from the plain loop's full-grid launches
    fake = {"prof": {"column_pairs": r["plain"]["column_pairs"]}, "clocks": r["clocks"], "units": r["nodes"],
            "npairs": r["npairs"], "ncomp": r["ncomp"]}
    line["roofline"] = roofline(argparse.Namespace(workload="sgrid", grid=256), fake, pk, src)
    return line


def surrogate_summary(args, r):
    """The learned update's numbers for the default line: rate and speed-up
    over the plain FP32 update at the working tolerance and at 1e-3, the
    fallbacks, and the max errors of unchecked predictions over a window."""
    sl = surrogate_line(args, r)
    t3 = r["tol_1e-3"]
    plain = sl["plain_every_step"]["value"]
    return {
        "workload": sl["config"]["workload"],
        "value": sl["value"], "unit": "grid nodes/s", "ms_per_step": r["ms"],
        "speedup_vs_plain": sl["speedup_vs_plain"], "working_tol": args.surr_tol,
        "steps": sl["surrogate_steps"],
        "plain_every_step": sl["plain_every_step"],
        "tensor_core_every_step": r["tc_every_step"],
        # the learned update with its plain steps on the tensor-core s-grid form
        "tensor_core_plain_steps": r["surrogate_tc_plain"],
        "tol_1e-3": dict(t3, speedup_vs_plain=t3["nodes_per_s"] / plain),
        "max_err_eta": r["accuracy"]["network"]["max_eta"], "max_err_u": r["accuracy"]["network"]["max_u"],
        "max_err_first_order_only": {"eta": r["accuracy"]["first_order_only"]["max_eta"],
                                     "u": r["accuracy"]["first_order_only"]["max_u"]},
        "target": ">= 10x the plain FP32 update at max error <= 1e-3 (eta, u; normwise)",
        "clocks": r["clocks"],
    }


def scalar_calls(ncall=1000, nthreads=8):
    """The reference's own calling pattern: one point per call (wave_VeloX,
    wave_SurfElev) on the 128-component point sea, host wall time per call
    (each call returns its value, so it includes the device round trip), on
    one host thread and on `nthreads` threads calling at once."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    import cfdwavemaker_gb300 as cw
    lib = cw.load()
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp())
    wm = cw.CFDwavemaker()
    assert wm.initialize_text(point_config()) == 0, cw.last_error()
    rng = np.random.default_rng(5)
    xs = rng.uniform(0, 500, ncall); zs = rng.uniform(-40, 0, ncall); ts = rng.uniform(0, 8, ncall)
    res = {}
    for name, call in (("wave_VeloX", lambda i: lib.wave_VeloX(xs[i], 0.0, zs[i], ts[i])),
                       ("wave_SurfElev", lambda i: lib.wave_SurfElev(xs[i], 0.0, ts[i]))):
        for i in range(20):
            call(i)
        t0 = time.perf_counter()
        for i in range(ncall):
            call(i)
        res[name + "_us_per_call"] = (time.perf_counter() - t0) / ncall * 1e6

    def work(k):
        for i in range(k * 250, k * 250 + 250):
            lib.wave_VeloX(xs[i % ncall], 0.0, zs[i % ncall], ts[i % ncall])
    with ThreadPoolExecutor(nthreads) as ex:
        list(ex.map(work, range(nthreads)))
        t0 = time.perf_counter()
        list(ex.map(work, range(2 * nthreads)))
        res["wave_VeloX_calls_per_s_%d_threads" % nthreads] = 2 * nthreads * 250 / (time.perf_counter() - t0)
    wm.cleanup()
    os.chdir(cwd)
    torch.cuda.synchronize()
    return res


def other_workloads(args):
    """Short runs of the other workloads for the default line (single GPU, no
    CPU baselines; each has its own --workload run with the full record): the
    s-grid update + 1e6 queries in both column forms, the point API, and the
    regular waves."""
    out = {}
    for key, wl, method in (("sgrid_tensor_core", "sgrid", 1), ("sgrid_plain", "sgrid", 0), ("point", "point", 1)):
        a = argparse.Namespace(**vars(args))
        a.workload, a.sgrid_method, a.grid, a.shard, a.vertical_theory = wl, method, 256, False, "sharma"
        a.steps, a.warmup = (3, 2) if (wl, method) == ("sgrid", 0) else (5, 3)
        r = run_ours(a)
        unit = "grid nodes/s" if wl == "sgrid" else "points/s"
        out[key] = {"value": r["units"] / (r["ms"] / 1e3), "unit": unit, "ms_per_step": r["ms"],
                    "steps": a.steps, "e2e": r["units"] / r["e2e_s"], "gpu_launches": r["launches"],
                    "clocks": r["clocks"], "kernels": r["prof"]}
        if "pressure_ms" in r:
            out[key]["with_pressure_ms_per_step"] = r["pressure_ms"]
    out["scalar_calls"] = scalar_calls()
    a = argparse.Namespace(**vars(args))
    a.workload, a.steps, a.warmup = "regular", 3, 2
    r = run_regular(a)
    out["regular"] = {"value": 2 * r["n"] / (r["ms"] / 1e3), "unit": "points/s", "ms_per_step": r["ms"],
                      "e2e": 2 * r["n"] / (r["e2e_ms"] / 1e3), "cases": r["cases"], "clocks": r["clocks"]}
    out["workloads"] = {"sgrid": "256x256x16 s-grid of the 1024-component sea, one ring update (dt 0.5 s) + 1e6 "
                                 "random spline queries per step",
                        "point": "eta, u, w, dp of the 128-component long-crested sea at 256 x 32 z x 8 t",
                        "regular": REG_WORKLOAD}
    return out


QFORM_WORKLOAD = ("precision form: second-order eta and z=0/Taylor-layer u, v, w (pair-cache coefficients) of "
                  "a 4096-component short-crested JONSWAP sea (256 freq x 16 dir, Hs 6 m, Tp 12 s, gamma 2, "
                  "cos-2s s=10, depth 100 m) at %d random (x, y, t) points")


def qform_config():
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea(nfreq=256, ndir=16)
    return ss.write_irregular(None, comps, 100.0, extrap=2)


def run_qform(args):
    """Precision form: eta2 and the Taylor-layer u2, v2, w2 at z0 = 0 of the
    4096-component sea (256 frequencies x 16 directions) at 4e6 points, as
    split 16-bit tcgen05 GEMMs; the plain FP32 CUDA-core form is timed on a
    row subset (its time is linear in rows) and the error of both against
    the FP64 oracle is taken on a sample of rows."""
    import torch
    import cfdwavemaker_gb300 as cw
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = cw.load()
    os.chdir(tempfile.mkdtemp())
    wm = cw.CFDwavemaker()
    txt = qform_config()
    t0 = time.time()
    assert wm.initialize_text(txt) == 0, cw.last_error()
    init_s = time.time() - t0
    R = args.rows
    rng = np.random.default_rng(99 + rank)
    x = rng.uniform(0, 1000, R); y = rng.uniform(0, 1000, R); t = rng.uniform(0, 100, R)
    d = [torch.tensor(a, device="cuda", dtype=torch.float64) for a in (x, y, t)]
    out = torch.zeros((R, 4), device="cuda", dtype=torch.float32)
    stream = torch.cuda.current_stream()
    lib.cfdwm_set_stream(C.c_void_p(stream.cuda_stream))
    ptr = [cw._ptr(a) for a in d]
    res = {"init_s": init_s, "forms": {}}
    # Accuracy, outside the timed regions, on two references:
    #  * the FP64 oracle on NS rows spread evenly over every 65,536-row chunk;
    #  * the GPU plain FP32 form (itself within a few 1e-7 of FP64) on every
    #    row of the first chunk, normalised by that chunk's max |plain|.
    import oracle
    cfg = oracle.waveinput.read_text(txt)
    sea = oracle.Sea(cfg)
    ns = min(R, args.oracle_rows)
    orows = np.unique(np.linspace(0, R - 1, ns).round().astype(np.int64))
    refE = oracle_eta2_parallel(sea, x[orows], y[orows], t[orows])
    refU = sea.uvw2(x[orows], y[orows], np.zeros(orows.size), t[orows])
    ref = np.stack([refE, refU[:, 0], refU[:, 1], refU[:, 2]], axis=1)
    names = ("eta", "u", "v", "w")

    def stats(got, want):
        g = got.astype(np.float64)
        d = g - want
        den = np.max(np.abs(want), axis=0)
        return {"max": [float(v) for v in np.max(np.abs(d), axis=0) / den],
                "rms": [float(v) for v in np.sqrt(np.mean(d * d, axis=0)) / den],
                "rms_rel": [float(v) for v in np.sqrt(np.mean(d * d, axis=0) / np.mean(want * want, axis=0))]}

    def timed(method, rows, steps, warm):
        for _ in range(warm):
            assert lib.cfdwm_qform_eval(ptr[0], ptr[1], ptr[2], rows, method, cw._ptr(out)) == 0, cw.last_error()
        torch.cuda.synchronize()
        lib.cfdwm_profile_read(6, None)      # drop the warm-up launches
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        l0 = lib.cfdwm_kernel_launches()
        e0.record(stream)
        for _ in range(steps):
            assert lib.cfdwm_qform_eval(ptr[0], ptr[1], ptr[2], rows, method, cw._ptr(out)) == 0, cw.last_error()
        e1.record(stream)
        torch.cuda.synchronize()
        timed.launches = lib.cfdwm_kernel_launches() - l0
        return e0.elapsed_time(e1) / steps

    plain_chunk = None
    for fp16 in (0, 1):
        name = "tc_fp16x3" if fp16 else "tc_bf16x3"
        tb = time.time()
        assert lib.cfdwm_qform_build(fp16) == 0, cw.last_error()
        build_s = time.time() - tb
        if fp16 == 0:
            # the plain FP32 form on the first chunk, and on the oracle rows
            sub = min(R, args.plain_rows)
            lib.cfdwm_profile_enable(1)
            ms = timed(0, sub, 1, 1)
            kt = C.c_double(0.0)
            nk = lib.cfdwm_profile_read(6, C.byref(kt))
            lib.cfdwm_profile_enable(0)
            # the rows the plain form wrote (the first `sub` rows)
            plain_chunk = out[:sub].cpu().numpy().astype(np.float64)
            orow_t = torch.tensor(orows, device="cuda")
            od = [a[orow_t].contiguous() for a in d]
            oo = torch.zeros((orows.size, 4), device="cuda", dtype=torch.float32)
            assert lib.cfdwm_qform_eval(*[cw._ptr(a) for a in od], orows.size, 0, cw._ptr(oo)) == 0
            res["forms"]["plain_fp32"] = {"ms_rows": ms, "rows": sub, "pts_per_s": sub / (ms / 1e3),
                                          "kernel_ms": kt.value / max(1, nk),
                                          "err_vs_fp64": stats(oo.cpu().numpy(), ref)}
        lib.cfdwm_profile_enable(1)
        lib.cfdwm_profile_read(6, None)
        sampler = ClockSampler(local)
        sampler.start()
        ms = timed(1, R, args.steps, args.warmup)
        clocks = sampler.stop()
        tot = C.c_double(0.0)
        nk = lib.cfdwm_profile_read(6, C.byref(tot))
        lib.cfdwm_profile_enable(0)
        o = out.cpu().numpy()
        ev64 = stats(o[orows], ref)
        evp = stats(o[:plain_chunk.shape[0]], plain_chunk)
        res["forms"][name] = {"ms": ms, "rows": R, "pts_per_s": R / (ms / 1e3),
                              "err_vs_fp64": ev64, "err_vs_plain_chunk": evp,
                              # the bar: the worse of the two references, per field
                              "err": [max(a, b) for a, b in zip(ev64["max"], evp["max"])],
                              "build_s": build_s, "gemm_launches": int(nk), "launches": int(timed.launches),
                              "gemm_ms_per_step": tot.value / max(1, args.steps), "clocks": clocks}
    res["accuracy_rows"] = {"fp64_oracle_rows": int(orows.size), "fields": names,
                            "plain_chunk_rows": int(plain_chunk.shape[0]),
                            "norm": "max and rms of |form - ref| over the rows / max |ref| over the same rows; "
                                    "rms_rel = rms(form - ref) / rms(ref)"}
    # end to end: the C-ABI call on host arrays in pinned memory (the library
    # stages them through its device buffers), copies inside the timed region
    hx = [torch.from_numpy(a).pin_memory() for a in (x, y, t)]
    hout = torch.empty((R, 4), dtype=torch.float32).pin_memory()
    hp = [cw._ptr(a) for a in hx]
    assert lib.cfdwm_qform_eval(hp[0], hp[1], hp[2], R, 1, cw._ptr(hout)) == 0, cw.last_error()
    # the epilogue's atomic adds run in no fixed order: equal to FP32 rounding
    o_dev = out.cpu().numpy()
    assert np.max(np.abs(hout.numpy() - o_dev)) <= 1e-6 * np.max(np.abs(o_dev)), "host-array call differs"
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    for _ in range(args.steps):
        assert lib.cfdwm_qform_eval(hp[0], hp[1], hp[2], R, 1, cw._ptr(hout)) == 0, cw.last_error()
    torch.cuda.synchronize()
    te = (time.perf_counter() - te0) / args.steps
    res["e2e_s"] = te
    res["h2d"] = 3 * 8 * R
    res["d2h"] = 4 * 4 * R
    res["ws"] = ws
    res["rank"] = rank
    res["npad"] = 4096
    return res


def qform_line(args, r):
    """The contract line of the precision-form workload.  value: points/s of
    the tensor-core form that meets the 1e-5 bar (fp16 split; bf16 split if it
    meets it); the plain FP32 form, the other split and their errors are
    reported beside it.  Algorithmic work per point: 2 flop for each of the
    4 N (N + 1) nonzero quadratic-form coefficients (the three split
    products are not counted)."""
    pk, src = peaks()
    forms = r["forms"]
    n = r["ws"]
    N = r["npad"]
    flop_pt = 2.0 * 4 * N * (N + 1)
    ok = [k for k in ("tc_bf16x3", "tc_fp16x3") if k in forms and max(forms[k]["err"]) <= 1e-5]
    head = ok[0] if ok else "tc_fp16x3"
    f = forms[head]
    value = f["pts_per_s"] * n
    gemm_ms = f["gemm_ms_per_step"]
    achieved = flop_pt * f["rows"] / (gemm_ms / 1e3) / 1e12 if gemm_ms > 0 else None
    peak_s = pk.get("bf16_tflops_sustained", pk["bf16_tflops"])
    plain = forms.get("plain_fp32", {})
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": n, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": f["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": head.replace("tc_", "") + " split, FP32 accumulate", "data": "synthetic",
        "config": {"workload": QFORM_WORKLOAD % f["rows"],
                   "l2": "inputs larger than L2 (split operands 4 GB per 65,536-row chunk, W 537 MB)",
                   "form": head},
        "e2e": {"value": f["rows"] * n / r["e2e_s"], "unit": "points/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": f["launches"],
        "clocks": f["clocks"],
        "roofline": {"kernel": "k_qform_tc", "bound": "tensor", "achieved": achieved, "peak": peak_s,
                     "unit": "TFLOP/s", "frac": (achieved / peak_s) if achieved else None,
                     "traffic": traffic_from_profiles("k_qform_tc"),
                     "issued_frac": (3 * achieved / peak_s) if achieved else None,
                     "algorithmic": "2 flop x 4 N (N+1) coefficients per point, N = %d" % N,
                     "peak_source": src + " bf16 sustained (dense; the GEMM runs inside steps of about a "
                                          "second), MEASURED_PEAKS.json"},
        "forms": {k: {kk: vv for kk, vv in v.items() if kk != "clocks"} for k, v in forms.items()},
        "speedup_vs_plain": (f["pts_per_s"] / plain["pts_per_s"]) if plain else None,
        "accuracy": dict(r["accuracy_rows"], head_form=head,
                         err_max=f["err_vs_plain_chunk"]["max"], err_rms=f["err_vs_plain_chunk"]["rms"],
                         err_max_fp64=f["err_vs_fp64"]["max"], err_rms_fp64=f["err_vs_fp64"]["rms"],
                         bar=1e-5),
        "init_s": r["init_s"],
        "peaks_source": src,
    }
    if plain and plain.get("kernel_ms"):
        # the plain form's kernel against the FP32 CUDA-core peak: 8 FMA per
        # (pair, row), pairs counted over the visited tiles (diagonal tiles in
        # full: their lower triangle holds zeros); peak = 152 SMs x 128 lanes
        # x 2 flop x the maximum SM clock (no measured FP32 figure exists)
        nt = N // 32
        pairs = nt * (nt + 1) // 2 * 1024
        ach = 16.0 * pairs * plain["rows"] / (plain["kernel_ms"] / 1e3) / 1e12
        fp32_peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        line["plain_roofline"] = {"kernel": "k_qform_plain", "bound": "fp32 FMA", "achieved": ach,
                                  "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                                  "peak_source": "derived: 152 SMs x 128 FP32 lanes x 2 flop x sm_max_mhz"}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = qform_cpu_baseline()
    return line


def oracle_eta2_parallel(sea, x, y, t):
    """Irregular::eta2 of the FP64 oracle at many points on all host cores
    (one point per call; the ctypes calls release the GIL)."""
    import concurrent.futures as cf
    nthr = os.cpu_count() or 1
    parts = np.array_split(np.arange(len(x)), nthr)
    with cf.ThreadPoolExecutor(nthr) as ex:
        outs = list(ex.map(lambda ix: sea.eta2(x[ix], y[ix], t[ix]), parts))
    return np.concatenate(outs) if outs else np.zeros(0)


def qform_cpu_baseline(budget_s=12.0):
    """FP64 oracle on a few rows: eta2 from the pair cache and uvw2 at z = 0,
    the same four outputs per point as the GPU forms."""
    import oracle
    cfg = oracle.waveinput.read_text(qform_config())
    sea = oracle.Sea(cfg)
    nthr = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    n = nthr
    x = rng.uniform(0, 1000, n); y = rng.uniform(0, 1000, n); t = rng.uniform(0, 100, n)
    t0 = time.perf_counter()
    sea.uvw2(x, y, np.zeros(n), t, nthr)
    oracle_eta2_parallel(sea, x, y, t)
    el = time.perf_counter() - t0
    return {"value": n / el, "unit": "points/s", "cores": nthr, "kind": "port",
            "sample": "%d points, eta2 and uvw2 at z=0 (4096 components, FP64 oracle)" % n}


def point_config(vertical_theory=None):
    from cfdwavemaker_gb300 import seastate as ss
    return ss.write_irregular(None, ss.config1_sea(), 50.0, extrap=2,
                              vertical_theory=None if vertical_theory in (None, "sharma") else vertical_theory)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # return once nvidia-smi is running and has written a sample, so that
        # short timed regions are sampled too
        t0 = time.time()
        while time.time() - t0 < 3.0:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("CFDWM_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, v):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "sm_max_mhz": 2070.0}, "fallback"


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import cfdwavemaker_gb300 as cw
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = cw.load()
    work = tempfile.mkdtemp()
    os.chdir(work)
    wm = cw.CFDwavemaker()
    if args.workload == "sgrid":
        txt = sgrid_config(args.grid, args.grid)
    else:
        txt = point_config(args.vertical_theory)
    t_init = time.time()
    rc = wm.initialize_text(txt)
    if rc != 0:
        raise SystemExit("initialize failed: %d %s" % (rc, cw.last_error()))
    depth_rank = 0
    if args.workload == "sgrid":
        R = C.c_int(0)
        rc = lib.cfdwm_sgrid_method(args.sgrid_method, C.byref(R))
        if rc != 0:
            raise SystemExit("s-grid method %d unavailable: %s" % (args.sgrid_method, cw.last_error()))
        depth_rank = R.value
    init_s = time.time() - t_init
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(1234 + rank)
    res = {}
    if args.workload == "sgrid":
        nq = 1_000_000
        qx = rng.uniform(0, 1000, nq)
        qy = rng.uniform(0, 1000, nq)
        qz = rng.uniform(-100, 6.0, nq)
        dt = 0.5
        state = {"t": 0.0}
        dq = [torch.tensor(a, device="cuda", dtype=torch.float64) for a in (qx, qy, qz)]
        dtq = torch.empty(nq, device="cuda", dtype=torch.float64)
        dout = torch.empty((nq, 4), device="cuda", dtype=torch.float64)
        hq = [torch.from_numpy(a).pin_memory() for a in (qx, qy, qz)]
        htq = torch.empty(nq, dtype=torch.float64).pin_memory()
        hout = np.empty((nq, 4))
        nodes = args.grid * args.grid * 16
        ring = None
        if args.shard:
            # the column shard: each rank fills its rows of every new slot and
            # the slots are all-gathered (NCCL); the whole grid is the job
            from cfdwavemaker_gb300.shard import ShardedRing
            ring = ShardedRing(wm)
            res["shard"] = {"bounds": ring.bounds, "rows": [ring.i0, ring.i1]}

        def update(t):
            if ring is not None:
                ring.force_update(t)
            else:
                lib.wave_force_update(t)

        def step_device():
            # one ring update + 1e6 queries at a time inside the new interval
            state["t"] += dt
            update(state["t"] + 1e-9)
            t0, _ = wm.sgrid_state()
            dtq.fill_(t0 + 0.5 * dt)
            rc = lib.wave_Kinematics_batch(cw._ptr(dq[0]), cw._ptr(dq[1]), cw._ptr(dq[2]), cw._ptr(dtq),
                                           nq, cw._ptr(dout))
            assert rc == 0

        def step_host():
            state["t"] += dt
            update(state["t"] + 1e-9)
            t0, _ = wm.sgrid_state()
            htq.fill_(t0 + 0.5 * dt)
            rc = lib.wave_Kinematics_batch(cw._ptr(hq[0].numpy()), cw._ptr(hq[1].numpy()),
                                           cw._ptr(hq[2].numpy()), cw._ptr(htq.numpy()), nq, cw._ptr(hout))
            assert rc == 0
            return float(hout[0, 1])

        units = nodes
        h2d = 4 * 8 * nq
        d2h = 4 * 8 * nq
    else:
        xs = np.linspace(0.0, 500.0, 256)
        ts = np.arange(8.0)
        X, T = np.meshgrid(xs, ts, indexing="ij")
        eta = wm.surface_elevation_batch(X.ravel(), np.zeros(X.size), T.ravel())
        zz = -50.0 + (eta[:, None] + 50.0) * np.linspace(0.0, 1.0, 32)[None, :]
        XX = np.repeat(X.ravel(), 32)
        TT = np.repeat(T.ravel(), 32)
        ZZ = zz.ravel()
        npt = XX.size
        d = [torch.tensor(a, device="cuda", dtype=torch.float64) for a in (XX, np.zeros(npt), ZZ, TT)]
        do = [torch.empty(npt, device="cuda", dtype=torch.float64) for _ in range(4)]
        hin = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (XX, np.zeros(npt), ZZ, TT)]
        hout = [np.empty(npt) for _ in range(4)]

        def step_device():
            p = [cw._ptr(a) for a in d]
            assert lib.wave_SurfElev_batch(p[0], p[1], p[3], npt, cw._ptr(do[0])) == 0
            assert lib.wave_VeloXYZ_batch(p[0], p[1], p[2], p[3], npt, cw._ptr(do[1]), None, cw._ptr(do[2])) == 0
            assert lib.wave_DynPres_batch(p[0], p[1], p[2], p[3], npt, cw._ptr(do[3])) == 0

        def step_host():
            p = [cw._ptr(a.numpy()) for a in hin]
            assert lib.wave_SurfElev_batch(p[0], p[1], p[3], npt, cw._ptr(hout[0])) == 0
            assert lib.wave_VeloXYZ_batch(p[0], p[1], p[2], p[3], npt, cw._ptr(hout[1]), None, cw._ptr(hout[2])) == 0
            assert lib.wave_DynPres_batch(p[0], p[1], p[2], p[3], npt, cw._ptr(hout[3])) == 0
            return float(hout[1][0])

        units = npt
        h2d = 4 * 8 * npt * 3
        d2h = 8 * npt * 4

    lib.cfdwm_set_stream(C.c_void_p(stream.cuda_stream))
    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    lib.cfdwm_profile_enable(1)
    for k in range(7):
        lib.cfdwm_profile_read(k, None)
    sampler = ClockSampler(local)
    sampler.start()
    barrier(ws)
    torch.cuda.synchronize()
    l0 = lib.cfdwm_kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = lib.cfdwm_kernel_launches() - l0
    prof = {}
    for k, name in enumerate(["column_pairs", "eta_pairs", "point_pairs", "phasors", "query",
                              "gradients", "qform"]):
        tot = C.c_double(0.0)
        nk = lib.cfdwm_profile_read(k, C.byref(tot))
        if nk > 0:
            prof[name] = {"launches": int(nk), "avg_ms": tot.value / nk, "total_ms": tot.value}
    lib.cfdwm_profile_enable(0)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = allmax(ws, ms)
    # end-to-end through the host-buffer API
    for _ in range(1):
        step_host()
    torch.cuda.synchronize()
    barrier(ws)
    te0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    torch.cuda.synchronize()
    te = (time.perf_counter() - te0) / args.steps
    te = allmax(ws, te)
    clocks = sampler.stop()
    if args.workload == "sgrid":
        # the same step with the dynamic pressure on the ring (a fourth field
        # of the update, its gradients and its query)
        assert lib.cfdwm_sgrid_pressure(1) == 0, cw.last_error()
        for _ in range(2):
            step_device()
        torch.cuda.synchronize()
        ep0 = torch.cuda.Event(enable_timing=True)
        ep1 = torch.cuda.Event(enable_timing=True)
        ep0.record(stream)
        for _ in range(args.steps):
            step_device()
        ep1.record(stream)
        torch.cuda.synchronize()
        res["pressure_ms"] = allmax(ws, ep0.elapsed_time(ep1) / args.steps)
        assert lib.cfdwm_sgrid_pressure(0) == 0, cw.last_error()
        # .vtu export of the ring (lsGridSpline::export_vtu layout), host formatting
        vpath = os.path.join(work, "ring.vtu")
        tv = []
        for _ in range(3):
            tw0 = time.perf_counter()
            assert lib.cfdwm_sgrid_write_vtu(vpath.encode(), 0) == 0, cw.last_error()
            tv.append(time.perf_counter() - tw0)
        res["vtu_s"] = float(np.median(tv))
        res["vtu_bytes"] = os.path.getsize(vpath)
        os.remove(vpath)
    res.update(depth_rank=depth_rank)
    res.update(ms=ms, e2e_s=te, units=units, launches=launches, init_s=init_s, h2d=h2d, d2h=d2h,
               clocks=clocks, ws=ws, rank=rank, prof=prof, npairs=int(lib.cfdwm_npairs()),
               ncomp=int(lib.cfdwm_components(None)))
    return res


def roofline(args, r, pk, src):
    """Roofline object of the dominant kernel from the in-library CUDA-event
    timings.  The column pair kernel is bound by the SFU (MUFU ex2) pipe: the
    depth ratios of both interaction wavenumbers need exp(kz) and
    exp(-2k(z+h)), i.e. 4 ex2 per (pair, level); a pair costs 22 FP32 flops
    per level on top (6 FMA for u, v, w and the ratio assembly).  The SFU
    (XU) pipe of a GB300 SM executes 32 lanes of ex2 per clock (ncu:
    the kernel's ex2 rate of 4.46 T/s was 49.4% of the XU peak at 2070 MHz);
    the peak is 152 SMs x 32 lanes x the median SM clock seen during the run
    (MEASURED_PEAKS.json holds no SFU or FP32 figure)."""
    prof = r["prof"]
    f_mhz = r["clocks"].get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    if args.workload == "sgrid" and r.get("depth_rank") and "qform" in prof:
        # depth-separable form: eta2 and 3R quadratic forms per column, each
        # 2 flop per nonzero coefficient of two N x N upper triangles
        kp = prof["qform"]
        N = r["ncomp"]
        nout = 1 + 3 * r["depth_rank"]
        flops = 2.0 * nout * N * (N + 1) * r["units"] / 16    # units = nodes; one row per column
        t = kp["avg_ms"] / 1e3
        ach = flops / t / 1e12
        return {"kernel": "k_qform_tc (depth-separable s-grid form)", "bound": "tensor", "achieved": ach,
                "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": ach / pk["bf16_tflops"],
                "traffic": traffic_from_profiles("k_qform_tc_sgrid"),
                "issued_frac": 3 * ach / pk["bf16_tflops"],
                "algorithmic": "2 flop x (1 + 3R) forms x N (N+1) coefficients per column, N = %d, R = %d, "
                               "%d columns" % (N, r["depth_rank"], r["units"] // 16),
                "avg_launch_ms": kp["avg_ms"],
                "peak_source": "measured bf16 burst (dense), MEASURED_PEAKS.json"}
    if args.workload == "sgrid" and "column_pairs" in prof:
        kp = prof["column_pairs"]
        units = r["units"]                     # grid nodes per launch (all columns, 16 levels)
        terms = units * (r["npairs"] + r["ncomp"])
        t = kp["avg_ms"] / 1e3
        ex2 = 4.0 * terms / t
        peak = 152 * 32 * f_mhz * 1e6
        return {"kernel": "k_pairs_columns", "bound": "sfu", "achieved": ex2 / 1e9, "peak": peak / 1e9,
                "unit": "Gex2/s", "frac": ex2 / peak, "traffic": traffic_from_profiles("k_pairs_columns"),
                "algorithmic": "4 ex2 + 22 FP32 flop per (pair, level); %d pairs + %d diagonal terms x %d nodes "
                               "per launch" % (r["npairs"], r["ncomp"], units),
                "fp32_tflops": 22.0 * terms / t / 1e12,
                "fp32_peak_tflops": 152 * 128 * 2 * f_mhz * 1e6 / 1e12,
                "avg_launch_ms": kp["avg_ms"],
                "peak_source": "derived: 152 SM x 32 XU lanes/clk x median SM clock %.0f MHz" % f_mhz}
    if "point_pairs" in prof:
        kp = prof["point_pairs"]
        n = r["units"]
        smit = getattr(args, "vertical_theory", "sharma") == "smit"
        # Sharma-Dean point sums: every pair of the triangle (no filter);
        # Smit: the pair-cache pairs and every diagonal term
        P = (r["npairs"] + r["ncomp"]) if smit else r["ncomp"] * (r["ncomp"] + 1) / 2
        t = kp["avg_ms"] / 1e3
        ex2 = 4.0 * n * P / t
        peak = 152 * 32 * f_mhz * 1e6
        name = "k_smit_points" if smit else "k_pairs_points"
        return {"kernel": name, "bound": "sfu", "achieved": ex2 / 1e9, "peak": peak / 1e9,
                "unit": "Gex2/s", "frac": ex2 / peak, "traffic": traffic_from_profiles(name),
                "algorithmic": "4 ex2 per (pair, point); %d pairs x %d points per launch" % (P, n),
                "avg_launch_ms": kp["avg_ms"],
                "peak_source": "derived: 152 SM x 32 XU lanes/clk x median SM clock %.0f MHz" % f_mhz}
    return None


def traffic_from_profiles(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            v = json.load(fh).get(kernel)
            return v.get("bytes_per_launch") if isinstance(v, dict) else v
    except (OSError, ValueError):
        return None


def vtu_cpu_baseline(n):
    """The oracle's single-threaded restatement of export_vtu (the reference's
    fprintf loop) on an n x n x 16 grid of the same shape.  Its arrays are not
    filled (zeros print shorter than the ring's values), so the time is a lower
    bound of the reference's."""
    from oracle import waveinput
    import oracle
    cfg = waveinput.read_text(sgrid_config(n, n))
    og = oracle.Sgrid(cfg, oracle.Sea(cfg), init=False)
    path = os.path.join(tempfile.mkdtemp(), "ring.vtu")
    t0 = time.perf_counter()
    og.export_vtu(path)
    dt = time.perf_counter() - t0
    size = os.path.getsize(path)
    os.remove(path)
    return {"s": dt, "MB": size / 1e6, "kind": "port", "cores": 1,
            "sample": "the same grid shape with unfilled (zero) arrays: a lower bound"}


def cpu_baseline(args, budget_s=15.0):
    """FP64 CPU restatement (oracle/) on a bounded sample, all host threads."""
    import oracle
    from oracle import waveinput
    nthr = os.cpu_count() or 1
    if args.workload in ("sgrid", "surrogate"):
        cfg = waveinput.read_text(sgrid_config())
        sea = oracle.Sea(cfg)
        grid = oracle.Sgrid(cfg, sea, init=False)
        # columns of the next ring slot, timed on a growing sample until the budget
        ncols = max(4, nthr)
        t0 = time.perf_counter()
        grid.update_columns(1.0, 0, ncols, nthr)
        el = time.perf_counter() - t0
        if el < budget_s / 4:
            ncols2 = int(ncols * min(64.0, (budget_s / 2) / max(el, 1e-3)))
            t0 = time.perf_counter()
            grid.update_columns(1.0, 0, ncols2, nthr)
            el = time.perf_counter() - t0
            ncols = ncols2
        rate = ncols * 16 / el
        return {"value": rate, "unit": "grid nodes/s", "cores": nthr, "kind": "port",
                "sample": "%d columns x 16 levels of one ring update (1024 components, 521k pairs), "
                          "FP64 oracle restatement of lsGridSpline::update, extrapolates linearly" % ncols}
    smit = getattr(args, "vertical_theory", "sharma") == "smit"
    cfg = waveinput.read_text(point_config(args.vertical_theory if smit else None))
    m = oracle.Model(cfg)
    rng = np.random.default_rng(5)
    n = max(nthr * 8, 64)
    x = rng.uniform(0, 500, n); z = rng.uniform(-50, 0, n); t = rng.uniform(0, 7, n)
    t0 = time.perf_counter()
    if smit:
        m.sea.fields(x, 0 * x, z, t, 1, nthr)
        m.sea.smit(x, 0 * x, z, t, nthr)
    else:
        m.sea.fields(x, 0 * x, z, t, 1 | 2 | 8 | 16, nthr)
    el = time.perf_counter() - t0
    return {"value": n / el, "unit": "points/s", "cores": nthr, "kind": "port",
            "sample": "%d random points of the 256x32x8 set, eta+u+w+dp%s, FP64 oracle"
                      % (n, " (Smit theory: u, v, w, dp)" if smit else "")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="qform", choices=["qform", "sgrid", "point", "surrogate", "regular"])
    ap.add_argument("--surr-steps", type=int, default=600, help="ring steps of the learned-update loop")
    ap.add_argument("--vertical-theory", default="sharma", choices=["sharma", "smit"],
                    help="point workload: the Sharma-Dean theory or the Smit s-coordinate theory")
    ap.add_argument("--plain-every", type=int, default=20)
    ap.add_argument("--plain-steps", type=int, default=20, help="steps on which the plain loop is timed")
    ap.add_argument("--surr-tol", type=float, default=5e-2,
                    help="fallback tolerance of the sampled check in the timed loop")
    ap.add_argument("--nsample", type=int, default=64)
    ap.add_argument("--sgrid-method", type=int, default=1, choices=[0, 1],
                    help="s-grid column sums: 0 plain FP32 CUDA cores, 1 depth-separable tensor-core form")
    ap.add_argument("--rows", type=int, default=4_000_000, help="points of the precision-form workload")
    ap.add_argument("--plain-rows", type=int, default=65536,
                    help="row subset on which the plain FP32 form of the precision workload is timed")
    ap.add_argument("--oracle-rows", type=int, default=256,
                    help="rows of the precision workload checked against the FP64 oracle (spread over every chunk)")
    ap.add_argument("--shard", action="store_true",
                    help="s-grid workload under torchrun: split the ring's rows of columns over the ranks "
                         "(strong scaling, one all-gather per new slot) instead of running replicas")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="precision workload: leave out the learned-update summary")
    ap.add_argument("--no-others", action="store_true",
                    help="precision workload: leave out the short runs of the other workloads")
    ap.add_argument("--grid", type=int, default=256,
                    help="columns per side of the s-grid (256 is the named workload; smaller sizes "
                         "are for profiling captures only)")
    args = ap.parse_args()
    unit = "grid nodes/s" if args.workload in ("sgrid", "surrogate") else "points/s"
    workload = {
        "sgrid": "s-grid second-order update: 1024-component short-crested JONSWAP (64 freq x 16 dir, "
                 "Hs 6 m, Tp 12 s, gamma 2, cos-2s s=10), depth 100 m, 256x256 columns x 16 levels over "
                 "1 km^2, dt 0.5 s, + 1e6 random spline queries per step",
        "point": "point API: 128-component JONSWAP (Hs 4 m, Tp 10 s, gamma 3.3), depth 50 m, eta/u/w/dp at "
                 "256 x 32 z x 8 t points",
        "qform": QFORM_WORKLOAD % args.rows,
        "surrogate": SURR_WORKLOAD % (args.surr_steps, args.plain_every, args.nsample, args.surr_tol),
        "regular": REG_WORKLOAD,
    }[args.workload]
    if args.workload == "point" and args.vertical_theory == "smit":
        workload += "; vertical_theory smit (Smit et al. 2017 s-coordinate second order)"
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        steps = []
        for _ in range(args.steps):
            if args.workload == "qform":
                steps.append(qform_cpu_baseline())
            elif args.workload == "regular":
                steps.append(regular_cpu_baseline())
            else:
                steps.append(cpu_baseline(args, budget_s=8.0))
        v = float(np.median([s["value"] for s in steps]))
        cb = dict(steps[-1])
        cb["value"] = v
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": unit, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": workload}, "cpu_baseline": cb,
                "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    if args.workload == "qform":
        r = run_qform(args)
        if r["rank"] != 0:
            return
        line = qform_line(args, r)
        if r["ws"] == 1 and not args.no_surrogate:
            # the other half of the metric: the learned s-grid update against
            # the plain FP32 update, at the target tolerance 1e-3 (a shorter
            # loop than --workload surrogate; single GPU only)
            sa = argparse.Namespace(**vars(args))
            sa.surr_steps, sa.plain_steps = 200, 10
            line["surrogate"] = surrogate_summary(sa, run_surrogate(sa))
        if r["ws"] == 1 and not args.no_others:
            line["other_workloads"] = other_workloads(args)
        print(json.dumps(line))
        return
    if args.workload == "regular":
        r = run_regular(args)
        if r["rank"] != 0:
            return
        line = regular_line(args, r)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = regular_cpu_baseline()
        print(json.dumps(line))
        return
    if args.workload == "surrogate":
        r = run_surrogate(args)
        if r["rank"] != 0:
            return
        line = surrogate_line(args, r)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(argparse.Namespace(workload="sgrid"))
        print(json.dumps(line))
        return
    r = run_ours(args)
    if r["rank"] != 0:
        return
    n = r["ws"]
    # replicas: every rank updates its own whole grid; shard: the ranks share one
    shared = args.workload == "sgrid" and args.shard
    value = r["units"] * (1 if shared else n) / (r["ms"] / 1e3)
    e2e = r["units"] * (1 if shared else n) / r["e2e_s"]
    pk, src = peaks()
    line = {
        "metric": METRIC, "value": value, "unit": unit, "n_gpus": n, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
        "scaling": "strong" if shared else "weak",
        "vs_baseline": None,
        "dtype": "fp16x3 split tcgen05, FP32 accumulate (FP64 phases)" if r.get("depth_rank") else
                 "f32 (FP64 phases)", "data": "synthetic",
        "config": {"workload": workload, "l2": "working set > L2 (phasor scratch 805 MB, grid 340 MB)",
                   "form": ("depth-separable tensor-core form, R = %d (fp16x3 split GEMM)" % r["depth_rank"])
                   if r.get("depth_rank") else "plain FP32 compensated"},
        "e2e": {"value": e2e, "unit": unit, "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "init_s": r["init_s"],
        "roofline": roofline(args, r, pk, src),
        "kernels": r["prof"],
        "peaks_source": src,
    }
    if "shard" in r:
        line["shard"] = r["shard"]
    if "vtu_s" in r:
        line["vtu_export"] = {"s": r["vtu_s"], "MB": r["vtu_bytes"] / 1e6,
                              "MB_per_s": r["vtu_bytes"] / 1e6 / r["vtu_s"], "threads": os.cpu_count()}
        if not args.no_cpu_baseline:
            line["vtu_export"]["cpu_baseline"] = vtu_cpu_baseline(args.grid)
    if "pressure_ms" in r:
        line["with_pressure"] = {"ms_per_step": r["pressure_ms"],
                                 "nodes_per_s": r["units"] * n / (r["pressure_ms"] / 1e3),
                                 "note": "dynamic pressure on the ring (cfdwm_sgrid_pressure): a fourth field"}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
