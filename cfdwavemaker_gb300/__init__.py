"""GB300 build of CFDwavemaker's point-kinematics path.

The product is the shared library ``libcfdwavemaker_gb300.so`` (C ABI in
``include/cfdwavemaker_gb300.h``).  This module loads it with ctypes and
offers the same Python surface as the reference's binding
(examples/python/cfdwavemaker.py: class ``CFDwavemaker`` with
``initialize``, ``velocity``, ``surface_elevation``, ...), plus NumPy batch
helpers over the batched entry points.  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcfdwavemaker_gb300.so")
_LIB = None

_d = C.c_double
_dp = C.POINTER(C.c_double)
_XYZT = [_d, _d, _d, _d]


class LibraryMissing(RuntimeError):
    pass


def load(path: str | None = None):
    """Load (once) and bind the shared library."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise LibraryMissing("libcfdwavemaker_gb300.so not built: run python -m cfdwavemaker_gb300.build")
    L = C.CDLL(p)
    L.wave_Initialize.restype = C.c_int
    L.wave_Initialize.argtypes = []
    L.wave_Cleanup.restype = C.c_int
    L.wave_Cleanup.argtypes = []
    L.CFDwavemaker_is_initialized.restype = C.c_int
    for name in ("wave_VeloX", "wave_VeloY", "wave_VeloZ", "wave_DynPres", "wave_nhPres"):
        fn = getattr(L, name)
        fn.restype = _d
        fn.argtypes = _XYZT
    L.wave_SurfElev.restype = _d
    L.wave_SurfElev.argtypes = [_d, _d, _d]
    L.wave_VFrac.restype = _d
    L.wave_VFrac.argtypes = [_d] * 5
    L.wave_Seabed.restype = _d
    L.wave_Seabed.argtypes = [_d, _d]
    L.wave_Kinematics.restype = _dp
    L.wave_Kinematics.argtypes = _XYZT
    L.wave_piston_position.restype = _d
    L.wave_piston_position.argtypes = [_d]
    L.wave_force_update.restype = None
    L.wave_force_update.argtypes = [_d]
    L.update_probes.restype = None
    L.update_probes.argtypes = [_d]
    for name in ("wave_phase_speed", "wave_mean_period", "wave_mean_length"):
        fn = getattr(L, name)
        fn.restype = _d
        fn.argtypes = [C.c_int]
    L.wave_water_depth.restype = _d
    L.wave_water_depth.argtypes = []
    L.wave_set_mpi_comm.restype = None
    L.wave_set_mpi_comm.argtypes = [C.c_int]
    # COMFLOW aliases (CFDwavemaker.h:61-69)
    for name in ("VelocityX", "VelocityY", "VelocityZ", "DynamicPressure"):
        fn = getattr(L, name)
        fn.restype = _d
        fn.argtypes = [C.c_int, C.c_int, C.c_int] + _XYZT
    L.SurfaceElevation.restype = _d
    L.SurfaceElevation.argtypes = [C.c_int, C.c_int, _d, _d, _d]
    L.VolumeFraction.restype = _d
    L.VolumeFraction.argtypes = [_d] * 5
    L.Init.restype = C.c_int
    L.Init.argtypes = [C.c_void_p]
    L.Prepare.restype = C.c_int
    L.Prepare.argtypes = [_d, C.c_int]
    L.Cleanup.restype = C.c_int
    L.Cleanup.argtypes = []
    L.cfdwm_kernel_launches.restype = C.c_long
    L.cfdwm_kernel_launches.argtypes = []
    # batched entry points (pointers may be host or device memory)
    vp = C.c_void_p
    L.wave_SurfElev_batch.restype = C.c_int
    L.wave_SurfElev_batch.argtypes = [vp, vp, vp, C.c_long, vp]
    L.wave_VeloXYZ_batch.restype = C.c_int
    L.wave_VeloXYZ_batch.argtypes = [vp, vp, vp, vp, C.c_long, vp, vp, vp]
    L.wave_DynPres_batch.restype = C.c_int
    L.wave_DynPres_batch.argtypes = [vp, vp, vp, vp, C.c_long, vp]
    L.wave_nhPres_batch.restype = C.c_int
    L.wave_nhPres_batch.argtypes = [vp, vp, vp, vp, C.c_long, vp]
    L.wave_VFrac_batch.restype = C.c_int
    L.wave_VFrac_batch.argtypes = [vp, vp, vp, vp, _d, C.c_long, vp]
    L.wave_Kinematics_batch.restype = C.c_int
    L.wave_Kinematics_batch.argtypes = [vp, vp, vp, vp, C.c_long, vp]
    L.cfdwm_initialize_text.restype = C.c_int
    L.cfdwm_initialize_text.argtypes = [C.c_char_p]
    L.cfdwm_set_stream.restype = C.c_int
    L.cfdwm_set_stream.argtypes = [vp]
    L.cfdwm_last_error.restype = C.c_int
    L.cfdwm_last_error.argtypes = [C.c_char_p, C.c_int]
    L.cfdwm_wavetype.restype = C.c_int
    L.cfdwm_irregular_fields.restype = C.c_int
    L.cfdwm_irregular_fields.argtypes = [vp, vp, vp, vp, C.c_long, C.c_int, vp]
    L.cfdwm_npairs.restype = C.c_long
    L.cfdwm_components.restype = C.c_int
    L.cfdwm_components.argtypes = [vp]
    L.cfdwm_sgrid_array.restype = C.c_long
    L.cfdwm_sgrid_array.argtypes = [C.c_int, vp, C.c_long]
    L.cfdwm_sgrid_state.restype = C.c_int
    L.cfdwm_sgrid_state.argtypes = [_dp, C.POINTER(C.c_int)]
    L.cfdwm_regular_solution.restype = C.c_int
    L.cfdwm_regular_solution.argtypes = [vp, C.c_int]
    L.cfdwm_regular_status.restype = C.c_int
    L.cfdwm_regular_status.argtypes = []
    # column shard of the s-grid ring (cfdwavemaker_gb300.shard)
    L.cfdwm_partition_columns.restype = C.c_int
    L.cfdwm_partition_columns.argtypes = [C.POINTER(C.c_long), C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.cfdwm_sgrid_partition.restype = C.c_int
    L.cfdwm_sgrid_partition.argtypes = [C.c_int, C.POINTER(C.c_int)]
    L.cfdwm_sgrid_due.restype = C.c_int
    L.cfdwm_sgrid_due.argtypes = [_d]
    L.cfdwm_sgrid_step_block.restype = C.c_int
    L.cfdwm_sgrid_step_block.argtypes = [C.c_int, C.c_int]
    L.cfdwm_sgrid_block_count.restype = C.c_long
    L.cfdwm_sgrid_block_count.argtypes = [C.c_int, C.c_int, C.c_int]
    L.cfdwm_sgrid_block_export.restype = C.c_int
    L.cfdwm_sgrid_block_export.argtypes = [C.c_int, C.c_int, C.c_int, vp]
    L.cfdwm_sgrid_block_import.restype = C.c_int
    L.cfdwm_sgrid_block_import.argtypes = [C.c_int, C.c_int, C.c_int, vp]
    L.cfdwm_sgrid_step_finish.restype = C.c_int
    L.cfdwm_sgrid_step_finish.argtypes = []
    L.cfdwm_parse_text.restype = C.c_int
    L.cfdwm_parse_text.argtypes = [C.c_char_p, vp, vp, C.c_int]
    L.cfdwm_irregular_fields_noalloc.restype = C.c_int
    L.cfdwm_irregular_fields_noalloc.argtypes = [vp, vp, vp, vp, C.c_long, C.c_int, vp]
    L.cfdwm_qform_build.restype = C.c_int
    L.cfdwm_qform_build.argtypes = [C.c_int]
    L.cfdwm_qform_eval.restype = C.c_int
    L.cfdwm_qform_eval.argtypes = [vp, vp, vp, C.c_long, C.c_int, vp]
    L.cfdwm_profile_enable.restype = C.c_int
    L.cfdwm_profile_enable.argtypes = [C.c_int]
    L.cfdwm_profile_read.restype = C.c_long
    L.cfdwm_profile_read.argtypes = [C.c_int, _dp]
    # learned s-grid update
    ip = C.POINTER(C.c_int)
    lp = C.POINTER(C.c_long)
    L.cfdwm_surrogate_create.restype = C.c_int
    L.cfdwm_surrogate_create.argtypes = [C.c_int, C.c_ulonglong]
    L.cfdwm_surrogate_nparams.restype = C.c_long
    L.cfdwm_surrogate_nparams.argtypes = []
    L.cfdwm_surrogate_get_params.restype = C.c_int
    L.cfdwm_surrogate_get_params.argtypes = [vp, C.c_long]
    L.cfdwm_surrogate_set_params.restype = C.c_int
    L.cfdwm_surrogate_set_params.argtypes = [vp, C.c_long]
    L.cfdwm_surrogate_save.restype = C.c_int
    L.cfdwm_surrogate_save.argtypes = [C.c_char_p]
    L.cfdwm_surrogate_load.restype = C.c_int
    L.cfdwm_surrogate_load.argtypes = [C.c_char_p]
    L.cfdwm_surrogate_features.restype = C.c_int
    L.cfdwm_surrogate_features.argtypes = [_d, vp, vp, vp]
    L.cfdwm_surrogate_targets.restype = C.c_int
    L.cfdwm_surrogate_targets.argtypes = [C.c_int, vp, vp, vp]
    L.cfdwm_surrogate_forward.restype = C.c_int
    L.cfdwm_surrogate_forward.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
    L.cfdwm_surrogate_loss_grad.restype = C.c_int
    L.cfdwm_surrogate_loss_grad.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, _dp, vp]
    L.cfdwm_surrogate_train_step.restype = C.c_int
    L.cfdwm_surrogate_train_step.argtypes = [vp, vp, C.c_long, vp, C.c_int, C.c_int, C.c_int, C.c_float, _dp]
    L.cfdwm_surrogate_step.restype = C.c_int
    L.cfdwm_surrogate_step.argtypes = [C.c_int, _d, C.c_int, ip, _dp]
    L.cfdwm_surrogate_compare.restype = C.c_int
    L.cfdwm_surrogate_compare.argtypes = [_dp]
    L.cfdwm_surrogate_enable.restype = C.c_int
    L.cfdwm_surrogate_enable.argtypes = [C.c_int, C.c_int, _d, C.c_int]
    L.cfdwm_sgrid_method.restype = C.c_int
    L.cfdwm_sgrid_method.argtypes = [C.c_int, ip]
    L.cfdwm_depth_basis.restype = C.c_int
    L.cfdwm_depth_basis.argtypes = [_d, _d, ip, _dp]
    L.cfdwm_sgrid_pressure.restype = C.c_int
    L.cfdwm_sgrid_pressure.argtypes = [C.c_int]
    L.cfdwm_sgrid_write_vtu.restype = C.c_int
    L.cfdwm_sgrid_write_vtu.argtypes = [C.c_char_p, C.c_int]
    L.cfdwm_spectrum_components.restype = C.c_int
    L.cfdwm_spectrum_components.argtypes = [_dp, C.c_int, C.c_int, C.c_ulonglong, vp]
    L.cfdwm_surrogate_set_carry.restype = C.c_int
    L.cfdwm_surrogate_set_carry.argtypes = [_d]
    L.cfdwm_surrogate_stats.restype = C.c_int
    L.cfdwm_surrogate_stats.argtypes = [lp, lp, lp]
    if path is None:
        _LIB = L
    return L


def _ptr(a):
    """Address of a NumPy array or of a CUDA tensor (anything with data_ptr())."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def last_error() -> str:
    buf = C.create_string_buffer(512)
    load().cfdwm_last_error(buf, 512)
    return buf.value.decode()


def _check(rc):
    if rc != 0:
        raise RuntimeError("cfdwavemaker_gb300 status %d: %s" % (rc, last_error()))


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size == 1 and n > 1:
        a = np.full(n, float(a.ravel()[0]))
    return a


class CFDwavemaker:
    """Mirror of the reference's Python binding (examples/python/cfdwavemaker.py:39-220).

    ``CFDwavemaker(workdir=...)`` changes into ``workdir`` so that
    ``initialize()`` finds ``waveinput.dat`` there, exactly like the
    reference; ``initialize_text()`` loads a configuration from a string.
    """

    def __init__(self, libpath: str | None = None, workdir: str | None = None):
        if workdir is not None:
            os.chdir(workdir)
        self.lib = load(libpath)

    # lifecycle
    def initialize(self):
        return self.lib.wave_Initialize()

    def initialize_text(self, text: str):
        return self.lib.cfdwm_initialize_text(text.encode())

    def cleanup(self):
        return self.lib.wave_Cleanup()

    def is_initialized(self):
        return bool(self.lib.CFDwavemaker_is_initialized())

    def set_mpi_comm(self, fortran_comm):
        self.lib.wave_set_mpi_comm(int(fortran_comm))

    # point queries
    def velocity_x(self, x, y, z, t):
        return self.lib.wave_VeloX(x, y, z, t)

    def velocity_y(self, x, y, z, t):
        return self.lib.wave_VeloY(x, y, z, t)

    def velocity_z(self, x, y, z, t):
        return self.lib.wave_VeloZ(x, y, z, t)

    def velocity(self, x, y, z, t):
        return (self.lib.wave_VeloX(x, y, z, t), self.lib.wave_VeloY(x, y, z, t),
                self.lib.wave_VeloZ(x, y, z, t))

    def dynamic_pressure(self, x, y, z, t):
        return self.lib.wave_DynPres(x, y, z, t)

    def nonhydrostatic_pressure(self, x, y, z, t):
        return self.lib.wave_nhPres(x, y, z, t)

    def surface_elevation(self, x, y, t):
        return self.lib.wave_SurfElev(x, y, t)

    def volume_fraction(self, x, y, z, t, delta_cellsize):
        return self.lib.wave_VFrac(x, y, z, t, delta_cellsize)

    def seabed(self, x, y):
        return self.lib.wave_Seabed(x, y)

    def piston_position(self, t):
        return self.lib.wave_piston_position(t)

    def kinematics(self, x, y, z, t, n=4):
        ptr = self.lib.wave_Kinematics(x, y, z, t)
        return [ptr[i] for i in range(n)]

    def force_update(self, t):
        self.lib.wave_force_update(t)

    def update_probes(self, t):
        self.lib.update_probes(t)

    def phase_speed(self, opt=1):
        return self.lib.wave_phase_speed(opt)

    def mean_period(self, opt=1):
        return self.lib.wave_mean_period(opt)

    def mean_length(self, opt=1):
        return self.lib.wave_mean_length(opt)

    def water_depth(self):
        return self.lib.wave_water_depth()

    # batched NumPy helpers (host arrays)
    def surface_elevation_batch(self, x, y, t):
        x = _f64(x); n = x.size
        y, t = _f64(y, n), _f64(t, n)
        out = np.empty(n)
        _check(self.lib.wave_SurfElev_batch(_ptr(x), _ptr(y), _ptr(t), n, _ptr(out)))
        return out

    def velocity_batch(self, x, y, z, t):
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        u, v, w = np.empty(n), np.empty(n), np.empty(n)
        _check(self.lib.wave_VeloXYZ_batch(_ptr(x), _ptr(y), _ptr(z), _ptr(t), n, _ptr(u), _ptr(v), _ptr(w)))
        return u, v, w

    def dynamic_pressure_batch(self, x, y, z, t):
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        p = np.empty(n)
        _check(self.lib.wave_DynPres_batch(_ptr(x), _ptr(y), _ptr(z), _ptr(t), n, _ptr(p)))
        return p

    def nonhydrostatic_pressure_batch(self, x, y, z, t):
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        p = np.empty(n)
        _check(self.lib.wave_nhPres_batch(_ptr(x), _ptr(y), _ptr(z), _ptr(t), n, _ptr(p)))
        return p

    def volume_fraction_batch(self, x, y, z, t, dcell):
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        out = np.empty(n)
        _check(self.lib.wave_VFrac_batch(_ptr(x), _ptr(y), _ptr(z), _ptr(t), float(dcell), n, _ptr(out)))
        return out

    def kinematics_batch(self, x, y, z, t):
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        out = np.empty((n, 4))
        _check(self.lib.wave_Kinematics_batch(_ptr(x), _ptr(y), _ptr(z), _ptr(t), n, _ptr(out)))
        return out

    def irregular_fields(self, x, y, z, t, mask=31):
        """Irregular::eta/u/v/w/dp without ramp or seabed clamp: [5, n]."""
        x = _f64(x); n = x.size
        y, z, t = _f64(y, n), _f64(z, n), _f64(t, n)
        out = np.zeros((5, n))
        _check(self.lib.cfdwm_irregular_fields(_ptr(x), _ptr(y), _ptr(z), _ptr(t), n, mask, _ptr(out)))
        return out

    def sgrid_array(self, which):
        n = self.lib.cfdwm_sgrid_array(which, None, 0)
        if n < 0:
            _check(n)
        out = np.empty(n)
        self.lib.cfdwm_sgrid_array(which, _ptr(out), n)
        return out

    def sgrid_state(self):
        t0 = C.c_double()
        ts = C.c_int()
        _check(self.lib.cfdwm_sgrid_state(C.byref(t0), C.byref(ts)))
        return t0.value, ts.value

    def sgrid_method(self, method):
        """Method of the s-grid column sums (0 plain, 1 tensor-core form); refills the ring.
        Returns the rank of the depth basis (0 for the plain form)."""
        r = C.c_int(0)
        _check(self.lib.cfdwm_sgrid_method(int(method), C.byref(r)))
        return r.value

    def sgrid_pressure(self, on=True):
        """Dynamic pressure on the s-grid ring (wave type 5); refills the ring."""
        _check(self.lib.cfdwm_sgrid_pressure(1 if on else 0))

    def components(self):
        n = self.lib.cfdwm_components(None)
        out = np.empty((8, n))
        self.lib.cfdwm_components(_ptr(out))
        return out

    def npairs(self):
        return self.lib.cfdwm_npairs()

    def regular_solution(self):
        out = np.zeros(256)
        n = self.lib.cfdwm_regular_solution(_ptr(out), 256)
        return out[:max(n, 0)]


def spectrum_components(hs, tp, gamma, nfreq, wmin, wmax, depth, seed, ndir=1, spreading_s=10.0,
                        theta_span=math.pi / 2, g=9.81):
    """Seeded JONSWAP / cos-2s components generated on the GPU
    (cfdwm_spectrum_components): dict of omega, A, k, phase, theta."""
    L = load()
    p = np.array([hs, tp, gamma, wmin, wmax, depth, spreading_s, theta_span, g], dtype=np.float64)
    out = np.zeros((5, nfreq * ndir))
    _check(L.cfdwm_spectrum_components(p.ctypes.data_as(_dp), int(nfreq), int(ndir), int(seed), _ptr(out)))
    return dict(zip(("omega", "A", "k", "phase", "theta"), out))


def parse_text(text: str):
    """Run only the C++ waveinput.dat parser (no GPU): (scalars[16], comps[8, n])."""
    L = load()
    sc = np.zeros(16)
    n = L.cfdwm_parse_text(text.encode(), _ptr(sc), None, 0)
    if n < 0:
        raise RuntimeError("parse error %d: %s" % (n, last_error()))
    comps = np.zeros((8, n))
    L.cfdwm_parse_text(text.encode(), _ptr(sc), _ptr(comps), n)
    return sc, comps
