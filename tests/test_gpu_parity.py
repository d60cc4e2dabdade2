"""Parity of the CUDA path with the reference.

Every check goes through the C ABI of libcfdwavemaker_gb300.so.  Golden
values are the reference's own FP64 outputs (tests/golden/, recorded by
make_golden.py from the unmodified reference) and, at more points, the FP64
oracle.  The kernels compute in FP32 (phases in FP64), so the bar is the
normwise relative error max|gpu - ref| / max|ref| per output field:

    TOL = 1e-5   for elevation, velocities and pressures
    TOL_GRAD = 1e-4  for the s-grid finite-difference arrays (differences of
                     FP32 node values divided by the spacing)
"""
import os

import numpy as np
import pytest

from conftest import golden_cfg, load_golden, norm_rel_err

import cfdwavemaker_gb300 as cw
import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_GRAD = 1e-4
API = ["SurfElev", "VeloX", "VeloY", "VeloZ", "DynPres", "nhPres"]
IRREGULAR = ["t005_focused", "t002_exact", "config1_point", "short_spread", "ramps_swl", "linear",
             "smit_spread", "smit_ramps"]
REGULAR = ["stokes5", "fenton24", "stokes5_len", "fenton_len"]


@pytest.fixture(scope="module")
def wm(tmp_path_factory):
    from cfdwavemaker_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("run")
    cwd = os.getcwd()
    os.chdir(d)            # wave_Initialize writes spectral_components.dat here
    m = cw.CFDwavemaker()
    yield m
    m.cleanup()
    os.chdir(cwd)


def init(wm, g):
    rc = wm.initialize_text(str(g["waveinput"]))
    assert rc == 0, cw.last_error()


def api_all(wm, x, y, z, t):
    eta = wm.surface_elevation_batch(x, y, t)
    u, v, w = wm.velocity_batch(x, y, z, t)
    p = wm.dynamic_pressure_batch(x, y, z, t)
    nh = wm.nonhydrostatic_pressure_batch(x, y, z, t)
    return [eta, u, v, w, p, nh]


@pytest.mark.parametrize("case", IRREGULAR + REGULAR)
def test_api_vs_reference(wm, case):
    g = load_golden(case)
    init(wm, g)
    out = api_all(wm, g["pt_x"], g["pt_y"], g["pt_z"], g["pt_t"])
    for q, name in enumerate(API):
        ref = g["api_" + name]
        err = norm_rel_err(out[q], ref)
        assert err <= TOL, (case, name, err)
    vf = wm.volume_fraction_batch(g["pt_x"], g["pt_y"], g["pt_z"], g["pt_t"], 0.1)
    assert np.max(np.abs(vf - g["api_VFrac"])) <= 1e-3


@pytest.mark.parametrize("case", ["config1_point", "ramps_swl", "fenton24"])
def test_scalar_entry_points(wm, case):
    """The reference's scalar functions are batches of one point here."""
    g = load_golden(case)
    init(wm, g)
    lib = wm.lib
    idx = np.arange(0, g["pt_x"].size, max(1, g["pt_x"].size // 7))
    for i in idx:
        x, y, z, t = (float(g["pt_" + k][i]) for k in "xyzt")
        vals = [lib.wave_SurfElev(x, y, t), lib.wave_VeloX(x, y, z, t), lib.wave_VeloY(x, y, z, t),
                lib.wave_VeloZ(x, y, z, t), lib.wave_DynPres(x, y, z, t), lib.wave_nhPres(x, y, z, t)]
        for q, name in enumerate(API):
            ref = g["api_" + name]
            scale = max(np.max(np.abs(ref)), 1e-30)
            assert abs(vals[q] - ref[i]) / scale <= TOL, (case, name, i)
        # COMFLOW aliases are the same functions
        assert lib.VelocityX(0, 0, 0, x, y, z, t) == vals[1]
        assert lib.SurfaceElevation(0, 0, x, y, t) == vals[0]


def test_few_point_kernels_large_sea(wm):
    """The few-point kernels on a 1280-component short-crested sea (80 pair
    tiles a side: 3240 tile pairs, so the slices of a few-point launch loop
    over several passes): batches of 1 and 300 points against one batch of
    all 600 (the per-thread kernels), every field within 1e-6 normwise."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(5.0, 11.0, 2.5, 80, 0.3, 1.8, 60.0, 77, ndir=16, spreading_s=8.0)
    txt = ss.write_irregular(None, comps, 60.0, extrap=2)
    assert wm.initialize_text(txt) == 0, cw.last_error()
    rng = np.random.default_rng(5)
    n = 600
    x = rng.uniform(-200, 200, n); y = rng.uniform(-200, 200, n)
    z = rng.uniform(-60.0, 2.0, n); t = rng.uniform(0, 50, n)
    whole = api_all(wm, x, y, z, t)
    for size, count in ((1, 12), (300, 600)):
        parts = [api_all(wm, x[b:b + size], y[b:b + size], z[b:b + size], t[b:b + size])
                 for b in range(0, count, size)]
        for q, name in enumerate(API):
            got = np.concatenate([pt[q] for pt in parts])
            err = norm_rel_err(got, whole[q][:got.size])
            assert err <= 1e-6, (size, name, err)


def test_scalar_calls_after_model_and_workspace_changes(wm):
    """Scalar calls replay a per-thread capture of the one-point pipeline; it
    must follow a re-initialised model and workspaces that a large batch has
    regrown.  The reference's values at the golden points, each time, and for
    irregular waves wave_Kinematics' (eta, u, v, w) record of the point."""
    def check(g, irregular):
        scale = {name: max(np.max(np.abs(g["api_" + name])), 1e-30) for name in API}
        for i in range(0, g["pt_x"].size, max(1, g["pt_x"].size // 6)):
            x, y, z, t = (float(g["pt_" + k][i]) for k in "xyzt")
            got = {"SurfElev": wm.lib.wave_SurfElev(x, y, t), "VeloX": wm.lib.wave_VeloX(x, y, z, t),
                   "VeloZ": wm.lib.wave_VeloZ(x, y, z, t), "DynPres": wm.lib.wave_DynPres(x, y, z, t)}
            for name, v in got.items():
                assert abs(v - g["api_" + name][i]) / scale[name] <= TOL, (name, i)
            if irregular:
                k = wm.kinematics(x, y, z, t)
                for q, name in enumerate(("SurfElev", "VeloX", "VeloY", "VeloZ")):
                    assert abs(k[q] - g["api_" + name][i]) / scale[name] <= TOL, ("Kinematics", name, i)
    for case, irregular in (("config1_point", True), ("ramps_swl", True), ("stokes5", False),
                            ("config1_point", True)):
        g = load_golden(case)
        init(wm, g)
        check(g, irregular)
        n = 300_000
        wm.velocity_batch(np.linspace(0, 300, n), np.zeros(n), np.full(n, -5.0), np.full(n, 1.0))
        check(g, irregular)


def test_t005_target_wave(wm):
    """The reference's own golden elevation series (tests/t005_focused_wave/targetwave.dat)."""
    g = load_golden("t005_focused")
    init(wm, g)
    t = g["extra_targetwave_t"]
    eta = wm.surface_elevation_batch(np.full_like(t, 10.0), np.zeros_like(t), t)
    assert norm_rel_err(eta, g["extra_targetwave_eta"]) <= TOL


def test_t002_exact_solution(wm):
    """The reference's own golden momentum integrals (exact_solution.mat)."""
    g = load_golden("t002_exact")
    init(wm, g)
    time = g["extra_time"]
    dz = 0.1
    z = np.arange(-20.0, 12, dz)
    T, Z = np.meshgrid(time, z, indexing="ij")
    n = T.size
    u, v, w = wm.velocity_batch(np.zeros(n), np.zeros(n), Z.ravel(), T.ravel())
    eta = wm.surface_elevation_batch(np.zeros(time.size), np.zeros(time.size), time)
    ratio = np.clip((eta[:, None] - (z[None, :] - dz / 2.0)) / dz, 0.0, 1.0)
    for arr, key in ((u, "umom1"), (v, "vmom1"), (w, "wmom1")):
        a = arr.reshape(time.size, z.size)
        mom = np.sum(a * np.abs(a) * dz * ratio, axis=1)
        # the momentum integral is quadratic in the velocity
        assert norm_rel_err(mom, g["extra_" + key]) <= 2 * TOL, key
    assert norm_rel_err(eta, g["extra_wave_elev1"]) <= TOL


@pytest.mark.parametrize("case", ["config1_point", "short_spread", "ramps_swl"])
def test_irregular_fields_vs_oracle_random(wm, case):
    """Irregular::eta/u/v/w/dp (no ramp) at random points against the oracle,
    including points above swl (Taylor layer), below, and t < 0."""
    g = load_golden(case)
    init(wm, g)
    cfg = golden_cfg(g)
    rng = np.random.default_rng(3)
    n = 700
    x = rng.uniform(-200, 600, n)
    y = rng.uniform(-100, 100, n)
    z = rng.uniform(-cfg["depth"], 4.0, n)
    t = rng.uniform(-1.0, 40.0, n)
    got = wm.irregular_fields(x, y, z, t)
    ref = oracle.Sea(cfg).fields(x, y, z, t)
    for q, name in enumerate(["eta", "u", "v", "w", "dp"]):
        err = norm_rel_err(got[q], ref[:, q])
        assert err <= TOL, (case, name, err)


def test_config1_workload_vs_oracle(wm):
    """The 128-component long-crested sea on its 256 x 32 x 8 point set
    (a sampled subset against the oracle)."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config1_sea()
    txt = ss.write_irregular(None, comps, 50.0, extrap=2)
    assert wm.initialize_text(txt) == 0
    cfg = oracle.waveinput.read_text(txt)
    xs = np.linspace(0.0, 500.0, 256)
    ts = np.arange(8.0)
    X, T = np.meshgrid(xs, ts, indexing="ij")
    eta = wm.surface_elevation_batch(X.ravel(), np.zeros(X.size), T.ravel())
    # 32 z-points from the seabed to the local crest
    zz = -50.0 + (eta[:, None] + 50.0) * np.linspace(0.0, 1.0, 32)[None, :]
    XX = np.repeat(X.ravel(), 32)
    TT = np.repeat(T.ravel(), 32)
    ZZ = zz.ravel()
    u, v, w = wm.velocity_batch(XX, np.zeros_like(XX), ZZ, TT)
    p = wm.dynamic_pressure_batch(XX, np.zeros_like(XX), ZZ, TT)
    sel = np.random.default_rng(0).choice(XX.size, 600, replace=False)
    ref = oracle.Model(cfg).api(XX[sel], 0.0 * XX[sel], ZZ[sel], TT[sel])
    for arr, q in ((u, 1), (w, 3), (p, 4)):
        assert norm_rel_err(arr[sel], ref[:, q]) <= TOL, q
    refe = oracle.Model(cfg).api(X.ravel(), 0 * X.ravel(), 0 * X.ravel(), T.ravel())[:, 0]
    assert norm_rel_err(eta, refe) <= TOL


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("case", ["sgrid_small", "sgrid_ignore"])
def test_sgrid_vs_reference(wm, case, method):
    """method 0: plain FP32 column sums; 1: the depth-separable tensor-core
    form, switched on after the initial fill (every update after it)."""
    import ctypes as C
    g = load_golden(case)
    init(wm, g)
    R = C.c_int(0)
    assert wm.lib.cfdwm_sgrid_method(method, C.byref(R)) == 0, cw.last_error()
    assert (R.value >= 8) if method else (R.value == 0)
    cfg = golden_cfg(g)
    updates = {"sgrid_small": [0.7, 1.6], "sgrid_ignore": [1.5]}[case]
    for k in range(int(g["nsnap"])):
        if k > 0:
            wm.force_update(updates[k - 1])
        t0, ts = wm.sgrid_state()
        assert ts == g["s%d_dims" % k][3] and abs(t0 - g["s%d_vals" % k][0]) < 1e-12
        for which in range(19):
            ref = g["s%d_arr%d" % (k, which)]
            got = wm.sgrid_array(which)
            tol = TOL if which <= 3 else TOL_GRAD
            if which in (6, 7, 11, 15):
                nslot = got.size // 4
                slots = {1, 2} if ts == 0 else {1, 2} | {(s + 2) % 4 for s in range(1, ts + 1)}
                for s in slots:
                    a, b = got[s * nslot:(s + 1) * nslot], ref[s * nslot:(s + 1) * nslot]
                    assert norm_rel_err(a, b) <= tol, (k, which, s)
            else:
                assert norm_rel_err(got, ref) <= tol, (k, which, norm_rel_err(got, ref))
        qt = float(np.ravel(g["s%d_query_t" % k])[0])
        qx, qy, qz = g["query_x"], g["query_y"], g["query_z"]
        kin = wm.kinematics_batch(qx, qy, qz, np.full_like(qx, qt))
        for c in range(4):
            assert norm_rel_err(kin[:, c], g["s%d_kin" % k][:, c]) <= TOL, (k, c)
        u, v, w = wm.velocity_batch(qx, qy, qz, np.full_like(qx, qt))
        for arr, name in ((u, "VeloX"), (v, "VeloY"), (w, "VeloZ")):
            assert norm_rel_err(arr, g["s%d_api_%s" % (k, name)]) <= TOL, (k, name)
        e = wm.surface_elevation_batch(qx, qy, np.full_like(qx, qt))
        assert norm_rel_err(e, g["s%d_api_SurfElev" % k]) <= TOL
        # scalar calls (captured per ring state: they must follow the updates)
        for i in range(0, qx.size, max(1, qx.size // 5)):
            x, y, z = float(qx[i]), float(qy[i]), float(qz[i])
            for name, val in (("VeloX", wm.lib.wave_VeloX(x, y, z, qt)),
                              ("VeloZ", wm.lib.wave_VeloZ(x, y, z, qt)),
                              ("SurfElev", wm.lib.wave_SurfElev(x, y, qt))):
                ref = g["s%d_api_%s" % (k, name)]
                assert abs(val - ref[i]) <= TOL * np.max(np.abs(ref)), (k, name, i)
            kin = wm.kinematics(x, y, z, qt)
            for c in range(4):
                ref = g["s%d_kin" % k][:, c]
                assert abs(kin[c] - ref[i]) <= TOL * np.max(np.abs(ref)), (k, "Kinematics", c, i)


def test_sgrid_tensor_core_method_vs_plain(wm):
    """The depth-separable tensor-core form against the plain form on the
    1024-component short-crested sea (64 x 16) on a 40 x 36 x 16 patch:
    every slot array of the ring after the initial fill and two updates."""
    import ctypes as C
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea()
    grid = {"bounds": (100.0, 100.0 + 39 * 3.92, 200.0, 200.0 + 35 * 3.92), "nx": 40, "ny": 36, "nl": 16,
            "t0": 5.0, "dt": 0.5, "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)
    arrs = {}
    for method in (0, 1):
        assert wm.initialize_text(txt) == 0, cw.last_error()
        R = C.c_int(0)
        assert wm.lib.cfdwm_sgrid_method(method, C.byref(R)) == 0, cw.last_error()   # refills the ring
        for k in range(2):
            wm.lib.cfdwm_surrogate_step(0, 0.0, 0, None, None)
        arrs[method] = [wm.sgrid_array(w) for w in range(19)]
        if method:
            print("depth basis rank", R.value)
    for w in range(19):
        tol = TOL if w <= 3 else TOL_GRAD
        err = norm_rel_err(arrs[1][w], arrs[0][w])
        print("tensor-core vs plain, array", w, "err", err)
        assert err <= tol, (w, err)


def test_sgrid_full_size_tensor_core_vs_plain(wm):
    """The benchmark's grid at full size: 256 x 256 columns x 16 levels of the
    1024-component sea; the tensor-core form against the plain form (itself
    pinned to the reference) on every node of the ring after the initial fill
    and one update."""
    import ctypes as C
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.config3_sea()
    grid = {"bounds": (0.0, 1000.0, 0.0, 1000.0), "nx": 256, "ny": 256, "nl": 16, "t0": 0.0, "dt": 0.5,
            "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid)
    arrs = {}
    for method in (0, 1):
        assert wm.initialize_text(txt) == 0, cw.last_error()
        R = C.c_int(0)
        assert wm.lib.cfdwm_sgrid_method(method, C.byref(R)) == 0, cw.last_error()
        wm.force_update(0.7)
        arrs[method] = [wm.sgrid_array(w) for w in range(4)]
    for w in range(4):
        err = norm_rel_err(arrs[1][w], arrs[0][w])
        print("full size, tensor-core vs plain, array", w, "err", err)
        assert err <= TOL, (w, err)


def test_sgrid_opposite_directions_vs_oracle(wm):
    """Directions exactly opposite at equal frequency (theta = -90 and +90 deg
    of a spread rotated by mtheta = 228.70473821303267 deg): the radicand of
    |k_i + k_m| is zero up to rounding.  The grid must stay finite and match
    the FP64 oracle (compiled without contraction, as the reference)."""
    from cfdwavemaker_gb300 import seastate as ss
    comps = ss.irregular_components(2.2, 7.2, 1.7, 8, 0.25, 1.6, 100.0, 714772915, ndir=16, spreading_s=6.4)
    grid = {"bounds": (435.0, 470.0, 442.0, 470.0), "nx": 8, "ny": 7, "nl": 6, "t0": 164.4, "dt": 1.7,
            "stretch": (0.7, 1.5)}
    txt = ss.write_irregular(None, comps, 100.0, extrap=2, lsgrid=grid, mtheta=228.70473821303267)
    assert wm.initialize_text(txt) == 0, cw.last_error()
    cfg = oracle.waveinput.read_text(txt)
    sea = oracle.Sea(cfg)
    og = oracle.Sgrid(cfg, sea)
    for which in range(4):
        got, ref = wm.sgrid_array(which), og.array(which)
        assert np.all(np.isfinite(got)), which
        assert np.all(np.isfinite(ref)), which
        assert norm_rel_err(got, ref) <= TOL, (which, norm_rel_err(got, ref))


@pytest.mark.parametrize("case", ["fenton24", "fenton_len"])
def test_fenton_solution_vs_reference(wm, case):
    g = load_golden(case)
    init(wm, g)
    sol = wm.regular_solution()
    ref = g["fenton_solution"]
    np.testing.assert_allclose(sol[:ref.size], ref, rtol=1e-9, atol=1e-12)


def test_device_pointer_batch(wm):
    """Device-resident inputs and outputs (torch tensors on cuda:0)."""
    torch = pytest.importorskip("torch")
    g = load_golden("config1_point")
    init(wm, g)
    x = torch.tensor(g["pt_x"], device="cuda:0", dtype=torch.float64)
    y = torch.tensor(g["pt_y"], device="cuda:0", dtype=torch.float64)
    z = torch.tensor(g["pt_z"], device="cuda:0", dtype=torch.float64)
    t = torch.tensor(g["pt_t"], device="cuda:0", dtype=torch.float64)
    u = torch.empty_like(x)
    n = x.numel()
    torch.cuda.synchronize()
    rc = wm.lib.wave_VeloXYZ_batch(cw._ptr(x), cw._ptr(y), cw._ptr(z), cw._ptr(t), n, cw._ptr(u), None, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert norm_rel_err(u.cpu().numpy(), g["api_VeloX"]) <= TOL


def test_empty_and_ragged_batches(wm):
    """Batches of every size agree with the scalar calls.  Up to 512 points
    the few-point kernels run (a block per point), above it the per-thread
    ones; the two sum in different orders, so they agree to FP32 rounding."""
    g = load_golden("config1_point")
    init(wm, g)
    assert wm.lib.wave_SurfElev_batch(None, None, None, 0, None) == 0
    for n in (1, 2, 127, 129, 512, 513, 1000):
        x = np.linspace(0, 300, n)
        eta = wm.surface_elevation_batch(x, np.zeros(n), np.full(n, 2.0))
        ref = np.array([wm.lib.wave_SurfElev(float(a), 0.0, 2.0) for a in x[:3]])
        np.testing.assert_allclose(eta[:3], ref, rtol=0, atol=1e-6 * np.max(np.abs(eta)))


@pytest.mark.parametrize("case", ["config1_point", "short_spread", "ramps_swl", "linear"])
def test_few_point_kernels_match_batch_kernels(wm, case):
    """The same points through the few-point kernels (batches of 1, 7 and
    512 points) and through the per-thread kernels (one batch of all 600):
    every field within 1e-6 normwise of each other, and both within TOL of
    the reference's golden values where the golden points are used."""
    g = load_golden(case)
    init(wm, g)
    rng = np.random.default_rng(3)
    n0 = g["pt_x"].size
    idx = np.concatenate([np.arange(n0), rng.choice(n0, max(0, 600 - n0), replace=True)])[:600]
    x, y, z, t = (np.ascontiguousarray(g["pt_" + k][idx]) for k in "xyzt")
    whole = api_all(wm, x, y, z, t)
    for size, count in ((1, 40), (7, 140), (512, 600)):
        parts = [api_all(wm, x[b:b + size], y[b:b + size], z[b:b + size], t[b:b + size])
                 for b in range(0, count, size)]
        got = [np.concatenate([pt[q] for pt in parts]) for q in range(len(API))]
        m = got[0].size
        for q, name in enumerate(API):
            err = norm_rel_err(got[q], whole[q][:m])
            assert err <= 1e-6, (case, size, name, err)
    sel = np.arange(min(n0, 600))
    for q, name in enumerate(API):
        assert norm_rel_err(whole[q][sel], g["api_" + name][sel]) <= TOL, (case, name)


def test_batches_across_chunk_boundaries(wm):
    """A host batch of 1,100,000 points crosses the host staging chunk
    (2^20 points) and the device evaluation chunk (2^18 points); points on
    both sides of every boundary against the FP64 oracle."""
    g = load_golden("config1_point")
    init(wm, g)
    cfg = golden_cfg(g)
    n = 1_100_000
    rng = np.random.default_rng(21)
    x = rng.uniform(0, 500, n)
    z = rng.uniform(-50, 0, n)
    t = rng.uniform(0, 7, n)
    y = np.zeros(n)
    u, v, w = wm.velocity_batch(x, y, z, t)
    p = wm.dynamic_pressure_batch(x, y, z, t)
    idx = np.unique(np.concatenate([np.arange(0, 3), np.arange((1 << 18) - 3, (1 << 18) + 3),
                                    np.arange((1 << 19) - 2, (1 << 19) + 2), np.arange((1 << 20) - 3, (1 << 20) + 3),
                                    np.arange(n - 3, n), rng.choice(n, 20, replace=False)]))
    ref = oracle.Model(cfg).api(x[idx], y[idx], z[idx], t[idx])
    for arr, q in ((u, 1), (w, 3), (p, 4)):
        assert norm_rel_err(arr[idx], ref[:, q]) <= TOL, q


def test_host_arrays_direct_and_staged_agree(wm):
    """Host (pageable) arrays reach the kernels either directly -- where the
    device reads pageable memory through the host's page tables -- or staged
    through pinned buffers in 2^20-point chunks (CFDWM_HOST_STAGING=1): the
    same kernels on the same values, so the results are identical.  Velocity,
    pressure and the interleaved Kinematics records of 1,100,000 points."""
    import os
    g = load_golden("config1_point")
    init(wm, g)
    n = 1_100_000
    rng = np.random.default_rng(33)
    x = rng.uniform(0, 500, n)
    z = rng.uniform(-50, 0, n)
    t = rng.uniform(0, 7, n)
    y = np.zeros(n)
    res = {}
    old = os.environ.get("CFDWM_HOST_STAGING")
    try:
        for mode in ("0", "1"):
            os.environ["CFDWM_HOST_STAGING"] = mode
            u, v, w = wm.velocity_batch(x, y, z, t)
            p = wm.dynamic_pressure_batch(x, y, z, t)
            k = wm.kinematics_batch(x, y, z, t)
            res[mode] = (u, v, w, p, k)
    finally:
        if old is None:
            os.environ.pop("CFDWM_HOST_STAGING", None)
        else:
            os.environ["CFDWM_HOST_STAGING"] = old
    for a, b in zip(res["0"], res["1"]):
        assert np.all(np.isfinite(a))
        assert np.array_equal(a, b)
