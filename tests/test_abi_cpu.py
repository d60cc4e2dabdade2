"""CPU checks of the product library: it loads, exports every symbol its
header declares, and its host logic (the waveinput.dat parser, error paths)
behaves like the reference without touching a GPU."""
import os
import re

import numpy as np
import pytest

from conftest import REF_TREE, REPO, golden_cfg, load_golden

import cfdwavemaker_gb300 as cw

HEADER = os.path.join(REPO, "include", "cfdwavemaker_gb300.h")
CASES = ["t005_focused", "t002_exact", "config1_point", "short_spread", "ramps_swl", "linear",
         "sgrid_small", "sgrid_ignore", "stokes5", "fenton24", "stokes5_len", "fenton_len"]


@pytest.fixture(scope="module")
def lib():
    from cfdwavemaker_gb300 import build
    build.build()
    return cw.load()


def declared_symbols():
    text = open(HEADER).read()
    return re.findall(r"CFDWM_EXPORT\s+[\w\s\*]+?\b(\w+)\s*\(", text)


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 40
    for s in syms:
        assert hasattr(lib, s), s


def test_reference_symbols_present(lib):
    # the reference's exported names (CFDwavemaker.h:25-69)
    ref = ["CFDwavemaker_is_initialized", "wave_Initialize", "wave_Cleanup", "wave_VeloX", "wave_VeloY",
           "wave_VeloZ", "wave_DynPres", "wave_nhPres", "wave_SurfElev", "wave_VFrac", "wave_Seabed",
           "wave_Kinematics", "wave_piston_position", "wave_force_update", "wave_set_mpi_comm",
           "update_probes", "wave_phase_speed", "wave_mean_period", "wave_mean_length",
           "wave_water_depth", "VelocityX", "VelocityY", "VelocityZ", "DynamicPressure",
           "SurfaceElevation", "VolumeFraction", "Init", "Prepare", "Cleanup"]
    for s in ref:
        assert hasattr(lib, s), s


@pytest.mark.parametrize("case", CASES)
def test_parser_matches_reference(lib, case):
    g = load_golden(case)
    sc, comps = cw.parse_text(str(g["waveinput"]))
    cfg = golden_cfg(g)
    assert int(sc[0]) == cfg["wavetype"]
    assert sc[2] == cfg["depth"] and sc[5] == cfg["gravity"] and sc[6] == cfg["rho"]
    if "components" in g:
        np.testing.assert_array_equal(comps, g["components"])
    if cfg["wavetype"] == 21:
        assert sc[12] == pytest.approx(cfg["wave_length"], rel=1e-15)
        assert sc[13] == pytest.approx(cfg["wave_period"], rel=1e-15)


def test_parser_errors(lib):
    with pytest.raises(RuntimeError):
        cw.parse_text("[wave type]\nirregular\n")             # no @v line
    with pytest.raises(RuntimeError):
        cw.parse_text("@v200\n[wave type]\nirregular\n")      # too old
    with pytest.raises(RuntimeError):
        cw.parse_text("@v310\n[wave type]\nbreaking\n")       # unknown type
    with pytest.raises(RuntimeError):
        cw.parse_text("@v310\n[wave type]\nirregular\n[general input data]\ndepth 10\n")  # no components
    txt = "@v310\n[wave type]\nirregular\n[wave input irregular]\nnfreq 3\nndir 0\n1 1 1 0 0\n[x]\n"
    with pytest.raises(RuntimeError):
        cw.parse_text(txt)                                     # too few component lines


def test_unserved_wave_types_are_refused_without_gpu(lib):
    piston = "@v310\n[wave type]\npiston\n[general input data]\ndepth 1\n"
    assert lib.cfdwm_initialize_text(piston.encode()) == -2
    slope = "@v310\n[wave type]\nslope\n[general input data]\ndepth 1\n"
    assert lib.cfdwm_initialize_text(slope.encode()) == -2
    assert lib.CFDwavemaker_is_initialized() == 0


def test_uninitialised_queries(lib):
    lib.wave_Cleanup()
    assert lib.wave_VeloX(0.0, 0.0, -1.0, 0.0) == 0.0
    assert lib.wave_SurfElev(0.0, 0.0, 0.0) == 0.0
    x = np.zeros(3)
    out = np.zeros(3)
    assert lib.wave_SurfElev_batch(cw._ptr(x), cw._ptr(x), cw._ptr(x), 3, cw._ptr(out)) == -1


def test_missing_waveinput_returns_minus_one(lib, tmp_path):
    cwd = os.getcwd()
    sub = tmp_path / "a" / "b"
    sub.mkdir(parents=True)
    os.chdir(sub)
    try:
        assert lib.wave_Initialize() == -1
    finally:
        os.chdir(cwd)


@pytest.mark.parametrize("case", ["helpers_config1", "helpers_t005"])
def test_spectral_helper_restatement_matches_reference(case):
    """The oracle's restatement of wave_mean_period, wave_phase_speed and
    wave_mean_length (Irregular.cpp:1336-1437) against the values the
    reference returned for the same seas (tests/golden/helpers_*.npz).  The
    library's own values are checked against the same fixtures on the GPU
    (tests/test_gpu_failures.py), where a sea can be loaded."""
    from oracle import waveinput
    g = load_golden(case)
    cfg = golden_cfg(g)
    got = [waveinput.mean_wave_period(cfg, 1), waveinput.mean_wave_period(cfg, 2), waveinput.phase_speed(cfg, 1),
           waveinput.phase_speed(cfg, 2), waveinput.mean_wave_length(cfg, 1), waveinput.mean_wave_length(cfg, 2),
           cfg["depth"]]
    np.testing.assert_allclose(got, g["helpers"], rtol=1e-14, atol=0)


REF_HEADER = os.path.join(REF_TREE, "src", "CFDwavemaker.h")
REF_EXAMPLE = os.path.join(REF_TREE, "examples", "python", "cfdwavemaker.py")


@pytest.mark.skipif(not os.path.exists(REF_HEADER), reason="reference tree not present")
def test_prototypes_match_reference_header(lib, tmp_path):
    """One C++ translation unit includes the reference's CFDwavemaker.h and
    this library's header: a reference function declared here with another
    return or parameter type is a conflicting declaration of a C function
    (a compile error).  The unit takes the address of every function of the
    reference header and links against the library, so each one resolves."""
    import subprocess
    text = re.sub(r"//[^\n]*|/\*.*?\*/", "", open(REF_HEADER).read(), flags=re.S)
    names = re.findall(r"\b(\w+)\s*\([^;{()]*\)\s*;", text)
    names = sorted(set(n for n in names if n not in ("if", "defined")))
    assert len(names) >= 29, names
    src = tmp_path / "proto.cpp"
    src.write_text('#include "CFDwavemaker.h"\n#include "cfdwavemaker_gb300.h"\n'
                   "extern \"C\" void *const cfdwm_addrs[] = {\n" +
                   "".join("    (void *)&%s,\n" % n for n in names) + "};\nint main() { return 0; }\n")
    libdir = os.path.join(REPO, "cfdwavemaker_gb300")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.dirname(REF_HEADER),
           "-I" + os.path.join(REPO, "include"), str(src), "-L" + libdir, "-lcfdwavemaker_gb300",
           "-Wl,-rpath," + libdir, "-o", str(tmp_path / "proto")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not os.path.exists(REF_EXAMPLE), reason="reference tree not present")
def test_reference_python_binding_loads_unchanged(lib, tmp_path):
    """The reference's own ctypes wrapper (examples/python/cfdwavemaker.py,
    unmodified, imported from the reference tree) binds every function it
    declares against this library, and the calls that need no loaded model
    answer as the reference's do before wave_Initialize."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_cfdwavemaker_example", REF_EXAMPLE)
    mod = importlib.util.module_from_spec(spec)
    cwd = os.getcwd()
    try:
        spec.loader.exec_module(mod)
        wm = mod.CFDwavemaker(os.path.join(REPO, "cfdwavemaker_gb300", "libcfdwavemaker_gb300.so"),
                              workdir=str(tmp_path))
    finally:
        os.chdir(cwd)
    wm.cleanup()
    assert wm.is_initialized() is False
    assert wm.lib.wave_Seabed.restype is not None
    assert wm.lib.wave_VeloX(0.0, 0.0, -1.0, 0.0) == 0.0
    assert wm.lib.wave_SurfElev(0.0, 0.0, 0.0) == 0.0


def test_depth_basis_host(lib):
    """The depth basis of the tensor-core s-grid form is built on the host:
    rank and reconstruction error for a few (K, h)."""
    import ctypes as C
    for K, h, rmax in ((0.52, 100.0, 18), (0.3, 50.0, 16), (1.2, 100.0, 24), (0.05, 30.0, 12)):
        R = C.c_int(0)
        e = C.c_double(1.0)
        assert lib.cfdwm_depth_basis(K, h, C.byref(R), C.byref(e)) == 0
        assert 8 <= R.value <= rmax and e.value <= 8e-6, (K, h, R.value, e.value)
    assert lib.cfdwm_depth_basis(-1.0, 10.0, None, None) != 0
