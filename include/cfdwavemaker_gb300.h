/*
 * cfdwavemaker_gb300.h -- C ABI of the GB300 build of CFDwavemaker's
 * point-kinematics path (libcfdwavemaker_gb300.so).
 *
 * Part 1 is a drop-in for the reference's exported functions
 * (oystelan/CFDwavemaker v3.1.0, src/CFDwavemaker.h:25-69, implemented in
 * src/CFDwavemaker.cpp:1533-2292): same names, argument order and meaning,
 * same return conventions.  Part 2 adds array-batched entry points beside
 * them.  Part 3 holds introspection hooks used by the tests.
 *
 * Threading: the point and batched queries may be called concurrently from
 * several host threads (each thread gets its own CUDA stream and workspace);
 * wave_Initialize, wave_Cleanup and wave_force_update must be called from one
 * thread at a time, as in the reference.
 *
 * Memory: every pointer argument of the batched entry points may point to
 * host memory or to device memory of the current CUDA device.  Host arrays
 * are staged through the library's own device buffers and the call returns
 * when the results are in place.  When all arrays of a call are device
 * memory and a stream was set with cfdwm_set_stream(), the call only
 * enqueues work on that stream and returns.
 */
#ifndef CFDWAVEMAKER_GB300_H
#define CFDWAVEMAKER_GB300_H

#if defined(__GNUC__)
#define CFDWM_EXPORT __attribute__((visibility("default")))
#else
#define CFDWM_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* Part 1: the reference's interface (CFDwavemaker.h:25-69)                */
/* ---------------------------------------------------------------------- */

/* CFDwavemaker.h:25, CFDwavemaker.cpp:2164 */
CFDWM_EXPORT int CFDwavemaker_is_initialized(void);
/* CFDwavemaker.h:27, CFDwavemaker.cpp:2065-2149: reads waveinput.dat from
 * ./, ./constant/, ../input_files/ or ../ .  Returns 0 on success, -1 when no
 * file is found.  Instead of the reference's exit() on malformed input it
 * returns -6 (parse error), -2 (a wave type this build does not serve:
 * piston, swd, vtk, slope) or -7 (Fenton solver failure). */
CFDWM_EXPORT int wave_Initialize(void);
/* CFDwavemaker.h:28, CFDwavemaker.cpp:2152 */
CFDWM_EXPORT int wave_Cleanup(void);
/* CFDwavemaker.h:29-33, CFDwavemaker.cpp:1543, 1682, 1744, 1808, 1822:
 * (x, y, z, t); z is clamped to the seabed; 0.0 for unsupported types. */
CFDWM_EXPORT double wave_VeloX(double x, double y, double z, double t);
CFDWM_EXPORT double wave_VeloY(double x, double y, double z, double t);
CFDWM_EXPORT double wave_VeloZ(double x, double y, double z, double t);
CFDWM_EXPORT double wave_DynPres(double x, double y, double z, double t);
CFDWM_EXPORT double wave_nhPres(double x, double y, double z, double t);
/* CFDwavemaker.h:34, CFDwavemaker.cpp:1894: (x, y, t) */
CFDWM_EXPORT double wave_SurfElev(double x, double y, double t);
/* CFDwavemaker.h:35, CFDwavemaker.cpp:1990-2009: (x, y, z, t, cell size) */
CFDWM_EXPORT double wave_VFrac(double x, double y, double z, double t, double dcell);
/* CFDwavemaker.h:36, CFDwavemaker.cpp:1970 */
CFDWM_EXPORT double wave_Seabed(double x, double y);
/* CFDwavemaker.h:37, CFDwavemaker.cpp:1619: returns {eta, u, v, w} (ramped)
 * in a thread-local buffer owned by the library (the reference returns a
 * new[] array that is never freed, and an uninitialised pointer for wave
 * type 1; here wave types 1 and 5 both fill the buffer). */
CFDWM_EXPORT double *wave_Kinematics(double x, double y, double z, double t);
/* CFDwavemaker.h:38, CFDwavemaker.cpp:2286 (piston only: 0 here) */
CFDWM_EXPORT double wave_piston_position(double t);
/* CFDwavemaker.h:41, CFDwavemaker.cpp:2253: advance the s-grid ring until
 * t <= t0 + dt (while CheckTime(t) -> update). */
CFDWM_EXPORT void wave_force_update(double t);
/* CFDwavemaker.h:48, CFDwavemaker.cpp:2241: one device-resident grid, no MPI:
 * a no-op kept for binary compatibility. */
CFDWM_EXPORT void wave_set_mpi_comm(int fortran_comm);
/* CFDwavemaker.h:51, CFDwavemaker.cpp:2012: probes are inert in v3.1.0. */
CFDWM_EXPORT void update_probes(double t);
/* CFDwavemaker.h:54-58, CFDwavemaker.cpp:2200-2237, Irregular.cpp:1372-1437 */
CFDWM_EXPORT double wave_phase_speed(int opt);
CFDWM_EXPORT double wave_mean_period(int opt);
CFDWM_EXPORT double wave_mean_length(int opt);
CFDWM_EXPORT double wave_water_depth(void);
/* COMFLOW aliases, CFDwavemaker.h:61-69, CFDwavemaker.cpp:2168-2198 */
CFDWM_EXPORT double VelocityX(int i, int j, int k, double x, double y, double z, double t);
CFDWM_EXPORT double VelocityY(int i, int j, int k, double x, double y, double z, double t);
CFDWM_EXPORT double VelocityZ(int i, int j, int k, double x, double y, double z, double t);
CFDWM_EXPORT double DynamicPressure(int i, int j, int k, double x, double y, double z, double t);
CFDWM_EXPORT double SurfaceElevation(int i, int j, double x, double y, double t);
CFDWM_EXPORT double VolumeFraction(double x, double y, double z, double t, double dcell);
CFDWM_EXPORT int Init(void *fptr);
CFDWM_EXPORT int Prepare(double t, int mode);
CFDWM_EXPORT int Cleanup(void);

/* ---------------------------------------------------------------------- */
/* Part 2: batched entry points (no counterpart in the reference; each    */
/* returns exactly what n calls of the scalar function named would)       */
/* ---------------------------------------------------------------------- */
/* Status: 0 ok, -1 not initialised, -2 unsupported wave type, -3 bad
 * argument, -4 CUDA error, -8 too large.  n may be 0. */

/* n x wave_SurfElev */
CFDWM_EXPORT int wave_SurfElev_batch(const double *x, const double *y, const double *t, long n,
                                     double *eta);
/* n x (wave_VeloX, wave_VeloY, wave_VeloZ); any of u, v, w may be NULL */
CFDWM_EXPORT int wave_VeloXYZ_batch(const double *x, const double *y, const double *z,
                                    const double *t, long n, double *u, double *v, double *w);
/* n x wave_DynPres */
CFDWM_EXPORT int wave_DynPres_batch(const double *x, const double *y, const double *z,
                                    const double *t, long n, double *p);
/* n x wave_nhPres */
CFDWM_EXPORT int wave_nhPres_batch(const double *x, const double *y, const double *z,
                                   const double *t, long n, double *p);
/* n x wave_VFrac with one cell size */
CFDWM_EXPORT int wave_VFrac_batch(const double *x, const double *y, const double *z,
                                  const double *t, double dcell, long n, double *vf);
/* n x wave_Kinematics: out is [n][4] = eta, u, v, w (ramped) */
CFDWM_EXPORT int wave_Kinematics_batch(const double *x, const double *y, const double *z,
                                       const double *t, long n, double *out);

/* Initialise from the text of a waveinput.dat instead of the file search
 * (same grammar and return codes as wave_Initialize). */
CFDWM_EXPORT int cfdwm_initialize_text(const char *text);
/* Stream for the calling thread's device-pointer calls (NULL: synchronous). */
CFDWM_EXPORT int cfdwm_set_stream(void *cuda_stream);
/* Last error message of the calling thread; returns its length. */
CFDWM_EXPORT int cfdwm_last_error(char *buf, int len);

/* ---------------------------------------------------------------------- */
/* Part 3: introspection hooks for tests and diagnostics                   */
/* ---------------------------------------------------------------------- */
/* Number of CUDA kernels the library has launched so far (process-wide). */
CFDWM_EXPORT long cfdwm_kernel_launches(void);
/* Per-kernel timing with CUDA events on the launching stream: enable, run,
 * then read the summed duration (ms) and the launch count of one kernel:
 * 0 s-grid column pair sums, 1 elevation pair sums, 2 point pair sums,
 * 3 phasors, 4 s-grid query, 5 s-grid gradients, 6 quadratic-form GEMM.
 * Reading clears the record. */
CFDWM_EXPORT int cfdwm_profile_enable(int on);
CFDWM_EXPORT long cfdwm_profile_read(int kernel, double *total_ms);
/* Wave type code of the loaded model (1, 5, 21; 0 when none). */
CFDWM_EXPORT int cfdwm_wavetype(void);
/* Irregular::eta/u/v/w/dp without ramp or seabed clamp (Irregular.cpp:9-157)
 * for wave types 1 and 5; out is [5][n]; mask bits 1 eta 2 u 4 v 8 w 16 dp. */
CFDWM_EXPORT int cfdwm_irregular_fields(const double *x, const double *y, const double *z,
                                        const double *t, long n, int mask, double *out);
/* Number of pairs kept by the pair cache (Irregular.cpp:840-967). */
CFDWM_EXPORT long cfdwm_npairs(void);
/* Parsed component arrays [8][n]: omega, A, k, phase, theta, ramptime,
 * starttime, duration; returns n (dst may be NULL). */
CFDWM_EXPORT int cfdwm_components(double *dst);
/* s-grid arrays (numbering of the reference's lsGridSpline members: 0 ETA,
 * 1-3 UX UY UZ, 4 ETAdx, 5 ETAdy, 6 ETAdt, 7+4f+q with q = dt, dx, dy, ds of
 * field f); returns the element count (dst may be NULL). */
CFDWM_EXPORT long cfdwm_sgrid_array(int which, double *dst, long cap);
CFDWM_EXPORT int cfdwm_sgrid_state(double *t0, int *tstep);
/* Regular-wave solution: k, c, mean velocity, Bernoulli R, L, T, then B_j
 * (Fenton); returns the count written. */
CFDWM_EXPORT int cfdwm_regular_solution(double *dst, int cap);
/* Parse waveinput.dat text without touching the GPU.  scalars[16] receives
 * wavetype, order, depth, mtheta, swl, gravity, rho, tofmax, x0, y0,
 * dw_cutoff, dw_bandwidth, wave_length, wave_period, wave_height, ndir;
 * comps (may be NULL) the [8][n] component arrays as cfdwm_components.
 * Returns n (>= 0) or a negative status. */
CFDWM_EXPORT int cfdwm_parse_text(const char *text, double *scalars, double *comps, int cap);

/* Precision form (no counterpart in the reference): the second-order sums
 * at z0 = 0 -- eta2 and the Taylor-layer u2, v2, w2 of the pair cache
 * (Irregular.cpp:223-293, 975-1102) -- as quadratic forms over the phasor
 * vectors.  build: fp16 != 0 splits operands into fp16 hi/lo parts, else
 * bf16 hi/lo.  eval: device arrays x, y, t (n points), out [n][4] FP32;
 * method 0 plain FP32 CUDA cores, 1 tcgen05 tensor cores. */
CFDWM_EXPORT int cfdwm_qform_build(int fp16);
CFDWM_EXPORT int cfdwm_qform_eval(const double *x, const double *y, const double *t, long n, int method,
                                  float *out);

/* ---------------------------------------------------------------------- */
/* Part 4: allocation-free evaluation                                      */
/* ---------------------------------------------------------------------- */
/* No counterpart in the reference.  Same results as cfdwm_irregular_fields,
 * for host codes that cannot let the library allocate device memory while
 * they run (solvers that reserve all device memory for their own pool at
 * start-up, or run under a fixed device-memory budget): this call performs
 * no cudaMalloc/cudaFree or other allocation.  x, y, z, t and out ([5][n])
 * must be device memory of the current device.  The workspace is one fixed
 * 32 MiB device array per GPU, held from library load until process exit;
 * a batch needs about (12 * Npad + 64) bytes per point, Npad = component
 * count rounded up to a multiple of 32, and larger batches are rejected with
 * -8 (message in cfdwm_last_error).  The first call on a device looks up the
 * array's device address, so make it before any stream capture.  All calls
 * share the array: calls that overlap on the GPU (several host threads or
 * streams at once) race.  The call returns after the results are written.
 * Wave type 5 models need one cfdwm_irregular_fields call first (it builds
 * the point-API pair table); without it the call returns -2. */
CFDWM_EXPORT int cfdwm_irregular_fields_noalloc(const double *x, const double *y, const double *z,
                                                const double *t, long n, int mask, double *out);

#ifdef __cplusplus
}
#endif
#endif
