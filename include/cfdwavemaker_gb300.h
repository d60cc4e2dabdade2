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
 * 3 phasors, 4 s-grid query, 5 s-grid gradients, 6 quadratic-form GEMM,
 * 7 learned-update first-order channels, 8 learned-update network forward,
 * 9 regular-wave (Stokes5 / Fenton) point evaluation.
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
 * field f; with the pressure field (cfdwm_sgrid_pressure): 19-22 its dt, dx,
 * dy, ds and 23 the field); returns the element count (dst may be NULL). */
CFDWM_EXPORT long cfdwm_sgrid_array(int which, double *dst, long cap);
CFDWM_EXPORT int cfdwm_sgrid_state(double *t0, int *tstep);
/* Regular-wave solution: k, c, mean velocity, Bernoulli R, L, T, then B_j
 * (Fenton); returns the count written. */
CFDWM_EXPORT int cfdwm_regular_solution(double *dst, int cap);
/* Status word of the last regular-wave set-up by wave_Initialize (the Fenton
 * Newton solve of FentonStream::set_stream_properties, FentonStream.cpp:141-239):
 *   0  converged (and always for Stokes 5th);
 *   3  not fully converged at the last continuation step: the reference's
 *      warning (FentonStream.cpp:208-209) is printed and the iterate is
 *      served, as the reference serves it;
 *   2  singular Jacobian (the reference throws, FentonStream.cpp:200-201):
 *      wave_Initialize returned -7;
 *   4  the iterate left the finite numbers (a wave beyond the highest one;
 *      the reference warns and serves NaN coefficients): wave_Initialize
 *      returned -7;
 *  -1  no regular-wave set-up has run. */
CFDWM_EXPORT int cfdwm_regular_status(void);
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
 * bf16 hi/lo.  The fp16 split sums its three products in one FP32
 * accumulator over K segments of 8 blocks of 64 components (environment
 * CFDWM_QFORM_KSEG at build: another segment length, 0 for whole column
 * tiles; CFDWM_QFORM_TWO_ACC=1: a second accumulator for the cross products
 * instead).  eval: arrays x, y, t (n points), out [n][4] FP32, in device
 * or host memory (host arrays are staged through a device buffer in chunks of
 * 2^22 points, 40 bytes a point); method 0 plain FP32 CUDA cores, 1 tcgen05 tensor cores. */
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
 * no cudaMalloc/cudaFree or other allocation.  Make the call with the device
 * that wave_Initialize ran on current, with x, y, z, t and out ([5][n]) in
 * that device's memory; anything else is rejected with -3.  The workspace is
 * one fixed 32 MiB device array per GPU, held until process exit.  Under
 * lazy module loading (the CUDA default) it is committed when
 * wave_Initialize loads an irregular sea (wave types 1 and 5), which also
 * looks up its device address, so later calls make no set-up of their own
 * (should that lookup have failed there, the first call retries it: make
 * that call before any stream capture).
 * A batch needs about (12 * Npad + 64) bytes per point, Npad = component
 * count rounded up to a multiple of 32, and larger batches are rejected with
 * -8 (message in cfdwm_last_error).  All calls share the array: calls that
 * overlap on the GPU (several host threads or streams at once) race.  The
 * call returns after the results are written.
 * Wave type 5 models need one cfdwm_irregular_fields call first (it builds
 * the point-API pair table); without it the call returns -2. */
CFDWM_EXPORT int cfdwm_irregular_fields_noalloc(const double *x, const double *y, const double *z,
                                                const double *t, long n, int mask, double *out);

/* ===========================================================================
 * Part 4b -- method of the s-grid column sums (new).
 * 0: the plain form, FP32 CUDA-core pair sums per (pair, level) with
 *    compensated accumulation.
 * 1: (default; environment CFDWM_SGRID_METHOD=0 at wave_Initialize selects
 *    the plain form) the depth-separable tensor-core form: the depth profiles
 *    e^{kz} +- e^{-k(z+2h)} are expanded in R orthonormal functions of z
 *    (R chosen so that the expansion error is <= 4e-6 of max F), each
 *    coefficient sum is a quadratic form over the column's phasors, and all
 *    of them with eta2 run as one split-fp16 tcgen05 GEMM over the columns.
 * rank (may be NULL) receives R.  The ring is refilled at the current t0
 * (tstep restarts at 0) and the updates that follow use the method. */
CFDWM_EXPORT int cfdwm_sgrid_method(int method, int *rank);
/* Host-only check of the depth basis for wavenumbers up to K and depth h:
 * R and the max reconstruction error over a test set of (k, z). */
CFDWM_EXPORT int cfdwm_depth_basis(double K, double h, int *rank, double *err);
/* Dynamic pressure on the s-grid ring (new; the reference's grid stores
 * none: lsgrid_spline.cpp:892-897 computes uvw2's pressure and drops it, and
 * wave_DynPres / wave_nhPres return 0.0 for wave type 5).  on = 1 adds a
 * fourth field to the ring, at every node
 *   dp1(z0) + rho uvw2.p(z0) + dp1_dz max(0, z - swl),  z0 = min(0, z)
 * (Irregular.cpp:1107-1120, 975-1102, 1142-1155; the velocities' own
 * convention, lsgrid_spline.cpp:889-897), with its finite-difference
 * gradients, and wave_DynPres / wave_nhPres (and their batched forms) then
 * return ramp * p and ramp * (p - rho g eta) from the spline query, as for
 * the irregular sea (CFDwavemaker.cpp:1807-1808, 1826-1830).  on = 0 removes
 * it (the default).  The ring is refilled at the current t0 (tstep restarts
 * at 0).  Not combined with the learned update (Part 5): either call
 * refuses while the other is on.  Returns 0, -2 (no s-grid model, a
 * first-order sea, or the learned update on) or another status. */
CFDWM_EXPORT int cfdwm_sgrid_pressure(int on);
/* .vtu file of the s-grid ring as lsGridSpline::export_vtu writes it
 * (lsgrid_spline.cpp:1222-1403): the base slot at t0 (last = 0) or the slot
 * after it at t0 + dt (last = 1), velocities as point data, node positions
 * from that slot's elevation, hexahedral cells; the time label of the
 * [lsgrid2vtk] section.  With a [lsgrid2vtk] section in waveinput.dat the
 * library writes <storage_path><filename><tstep %05d>.vtu itself, as the
 * reference does: after the initial fill, after every ring update and, with
 * last = 1, at wave_Cleanup (the reference at its exit).  Returns 0, -2 (no
 * s-grid model) or -5 (the file cannot be written). */
CFDWM_EXPORT int cfdwm_sgrid_write_vtu(const char *path, int last);
/* Sea-state components generated on the device (new; the reference reads
 * them from waveinput.dat, CFDwavemaker.cpp:677-800, and leaves generating
 * them to external tools).  params[9] = Hs, Tp, gamma, wmin, wmax, depth,
 * spreading s, direction span (rad), gravity.  comps (host or device) receives
 * [5][nfreq ndir] = omega, A, k, phase, theta: the five columns of the
 * "ndir 0" format, component f ndir + d with
 *   omega_f = linspace(wmin, wmax, nfreq), theta_d = linspace(-span, span, ndir)
 *   (theta = 0 when ndir = 1),
 *   A = sqrt(2 S(omega_f) dw D_d), S the JONSWAP density (sigma 0.07 / 0.09)
 *   scaled to 4 sqrt(sum S dw) = Hs, D_d = cos(theta_d / 2)^(2 s) normalised
 *   to sum 1, k from w^2 = g k tanh(k h) (FP64 Newton), phase = 2 pi u with
 *   u the top 53 bits of SplitMix64(seed + (c + 1) 0x9E3779B97F4A7C15) / 2^53.
 * Returns 0, -3 (bad parameters) or -4. */
CFDWM_EXPORT int cfdwm_spectrum_components(const double *params, int nfreq, int ndir, unsigned long long seed,
                                           double *comps);

/* ---------------------------------------------------------------------- */
/* Part 4d: column shard of the s-grid ring over several GPUs (new beside  */
/* the reference's MPI build, which these calls replace)                   */
/* ---------------------------------------------------------------------- */
/* The reference's MPI build splits the grid's rows of columns (index i) over
 * the ranks (lsGridSpline::compute_mpi_partition, lsgrid_spline.cpp:652-664,
 * with cfdwm_mpi::partition_weighted, mpi_utils.h:46-64), lets each rank fill
 * its rows of the new slot and all-gathers the slot's ETA, UX, UY, UZ
 * (lsgrid_spline.cpp:907-910, mpi_utils.h:69-79) before every rank
 * recomputes the gradients.  Here one process per GPU loads the same model;
 * the calls below are the rank's side of one such step, and the all-gather
 * between them is the caller's (cfdwavemaker_gb300.shard does it with
 * torch.distributed: NCCL on GPUs).
 *
 * Work-balanced contiguous partition of n rows with weights w (>= 0) over
 * nranks: bounds[0..nranks], rank r owns rows [bounds[r], bounds[r+1]).  The
 * reference's rule (mpi_utils.h:46-64), host only (no GPU needed). */
CFDWM_EXPORT int cfdwm_partition_columns(const long *weights, int n, int nranks, int *bounds);
/* The same for the loaded grid: weights = live (not ignored) columns per row
 * (lsgrid_spline.cpp:652-664). */
CFDWM_EXPORT int cfdwm_sgrid_partition(int nranks, int *bounds);
/* 1 when wave_force_update(t) would step the ring (lsGridSpline::CheckTime,
 * lsgrid_spline.cpp:610-615), else 0. */
CFDWM_EXPORT int cfdwm_sgrid_due(double t);
/* One ring step of the rank that owns rows [i0, i1): advances the ring
 * (lsgrid_spline.cpp:847-860) and fills only those rows of the new slot (in
 * the s-grid method of the model). */
CFDWM_EXPORT int cfdwm_sgrid_step_block(int i0, int i1);
/* Elements of rows [i0, i1) of one field of a slot: field 0 ETA ((i1-i0) ny),
 * 1..3 UX, UY, UZ and 4 the pressure when the ring holds it
 * ((i1-i0) ny nl). */
CFDWM_EXPORT long cfdwm_sgrid_block_count(int field, int i0, int i1);
/* Copies rows [i0, i1) of a field of the newest slot to dst / from src (host
 * or device memory, [rows][ny] or [rows][ny][nl] as the ring stores them);
 * return when the copy is done. */
CFDWM_EXPORT int cfdwm_sgrid_block_export(int field, int i0, int i1, float *dst);
CFDWM_EXPORT int cfdwm_sgrid_block_import(int field, int i0, int i1, const float *src);
/* After every rank's rows are in the newest slot: the finite-difference
 * gradients and the query image (lsgrid_spline.cpp:912-922), and the .vtu
 * file of a [lsgrid2vtk] section. */
CFDWM_EXPORT int cfdwm_sgrid_step_finish(void);

/* ===========================================================================
 * Part 5 -- learned s-grid update (new; no counterpart in the reference).
 *
 * Between full plain ring updates (lsgrid_spline.cpp:847-931) a small
 * convolutional network predicts the second-order part of the new slot from
 * first-order channels of the columns.  Network: 4 valid 3x3 convolutions,
 * 8 nl -> 32 -> 32 -> 32 -> 1 + 3 nl channels, SiLU between them, BF16
 * weights, FP32 accumulation; nl = sigma levels of the grid (1..32).
 * Tensors are [B][C][H][W] FP32 planes in device memory; the network maps
 * H x W inputs to (H - 8) x (W - 8) outputs.
 *   input channel  8 m + q, level m, q = u, u~, v, v~, w, w~, p, p~ (first
 *                  order at the levels placed under eta1; ~ = the quadrature
 *                  sum, phase - pi/2), over the grid plus a 4-column halo,
 *                  scaled by 1/(sigma omega_m) (u, v, w) and 1/sigma (p);
 *   output channel 0 = (eta - swl - eta1) / (k_m sigma^2),
 *                  1 + f nl + m = (U_f - U1_f) / (k_m sigma^2 omega_m),
 *                  U1 = first order with the Taylor term at the eta1 levels;
 * sigma^2 = sum A^2 / 2; omega_m, k_m = A^2-weighted means.
 * All calls return 0 or a negative status. */
/* Creates the network for nl levels with seeded He-normal weights. */
CFDWM_EXPORT int cfdwm_surrogate_create(int nl, unsigned long long seed);
CFDWM_EXPORT long cfdwm_surrogate_nparams(void);
/* Parameters (FP32 master copy; host or device pointers), n = nparams. */
CFDWM_EXPORT int cfdwm_surrogate_get_params(float *dst, long n);
CFDWM_EXPORT int cfdwm_surrogate_set_params(const float *src, long n);
/* Weight file: "CFDWMSR1", int32 nl, int32 0, int64 n, n float32. */
CFDWM_EXPORT int cfdwm_surrogate_save(const char *path);
CFDWM_EXPORT int cfdwm_surrogate_load(const char *path);
/* Of the loaded wave type 5 model at time t: feat [8 nl][nx+8][ny+8],
 * base [3][nx ny nl] (U1), eta1 [nx ny]; device pointers. */
CFDWM_EXPORT int cfdwm_surrogate_features(double t, float *feat, float *base, float *eta1);
/* Normalised targets of ring slot `slot` (filled by the plain method, with
 * base/eta1 from cfdwm_surrogate_features at that slot's time):
 * tgt [1 + 3 nl][nx][ny]. */
CFDWM_EXPORT int cfdwm_surrogate_targets(int slot, const float *base, const float *eta1, float *tgt);
/* y [B][1 + 3 nl][H-8][W-8] = network(x [B][8 nl][H][W]). */
CFDWM_EXPORT int cfdwm_surrogate_forward(const float *x, int B, int H, int W, float *y);
/* Loss L = sum_c w_c (y - tgt)^2 / (B P sum w), w_0 = nl, w_c = 1 otherwise,
 * P = (H-8)(W-8), and dL/dparams into grad [nparams] (device, may be NULL). */
CFDWM_EXPORT int cfdwm_surrogate_loss_grad(const float *x, const float *tgt, int B, int H, int W, double *loss,
                                           float *grad);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on samples idx[0..B) (host ints,
 * each in [0, S)) of the datasets xs [S][8 nl][H][W] and
 * ts [S][1 + 3 nl][H-8][W-8], S = nsamples. */
CFDWM_EXPORT int cfdwm_surrogate_train_step(const float *xs, const float *ts, long nsamples, const int *idx,
                                            int B, int H, int W, float lr, double *loss);
/* One ring update of the loaded s-grid: mode 0 plain, 1 predicted and
 * checked against the plain method on nsample random live columns (the plain
 * method fills the slot when the error exceeds tol), 2 predicted unchecked.
 * A predicted slot is first order + network output + the low-passed
 * residual (plain - network) of the last plain slot, carried forward (see
 * cfdwm_surrogate_set_carry); adding 4 to the mode leaves the residual out
 * (network alone).  err4 (may be
 * NULL): the check's max errors of eta, u, v, w, each relative to the
 * max |eta - swl| / max |U| of the last plain slot. */
CFDWM_EXPORT int cfdwm_surrogate_step(int mode, double tol, int nsample, int *fell_back, double *err4);
/* Errors of the newest slot against a full plain fill at its time
 * (normalised as in cfdwm_surrogate_step, by the plain slot's own maxima). */
CFDWM_EXPORT int cfdwm_surrogate_compare(double *err4);
/* Route wave_force_update through the learned update: every plain_every-th
 * ring update is plain, the others mode 1 with (tol, nsample). */
CFDWM_EXPORT int cfdwm_surrogate_enable(int on, int plain_every, double tol, int nsample);
CFDWM_EXPORT int cfdwm_surrogate_stats(long *steps, long *fallbacks, long *plain_steps);
/* Low-pass scale of the carried residual, in mean wavelengths 2 pi / k_m
 * (Gaussian standard deviation; default 0: nothing is carried). */
CFDWM_EXPORT int cfdwm_surrogate_set_carry(double wavelengths);

#ifdef __cplusplus
}
#endif
#endif
