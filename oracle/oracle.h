/*
 * CPU oracle for the CFDwavemaker point-kinematics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference algorithms (oystelan/CFDwavemaker v3.1.0).  It is used by the
 * test-suite as the parity checker, by __graft_entry__.smoke() as the
 * checker of one small GPU invocation, and by bench.py's CPU-baseline leg.
 * The product library (cfdwavemaker_gb300) never links, loads or calls it.
 *
 * Parity of this restatement is pinned against the reference itself: the
 * reference sources are compiled by oracle/Makefile into oracle/_ref/ and
 * tests/golden/make_golden.py records their outputs as fixtures; the
 * reference's own golden vectors (tests/t005_focused_wave/targetwave.dat and
 * tests/t002_spline_momentum_conservation/exact_solution.mat) are pinned too.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef CFDWM_ORACLE_H
#define CFDWM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Irregular sea (Irregular.h / Irregular.cpp)                          */
/* ------------------------------------------------------------------ */
typedef struct orc_sea orc_sea;

/* Create a sea from component arrays that are already sorted by omega and
 * already normalised/amplified (Irregular::normalize_data,
 * Irregular.cpp:1282).  ramp arrays may be NULL: the parser's defaults
 * (ramptime 0, start -SMALL, duration HUGE; CFDwavemaker.cpp:719-722) are
 * used then.  order: 0 linear (unclipped), 1 clipped, 2 second order with
 * Taylor expansion (Irregular.cpp:9-157). */
orc_sea *orc_sea_create(int n, const double *omega, const double *A, const double *k,
                        const double *phase, const double *theta,
                        const double *ramptime, const double *starttime, const double *duration,
                        double depth, double mtheta, double tofmax, double fx, double fy,
                        double swl, double g, double rho, double dw_bandwidth, double dw_cutoff,
                        int order);
void orc_sea_free(orc_sea *s);
long orc_sea_npairs(const orc_sea *s);

/* normalize_data (Irregular.cpp:1282-1297): in place on A/phase. */
void orc_normalize(int n, double *A, double *phase, int normalize, double ampl);

/* Scalar reference methods (Irregular.cpp). */
double orc_eta(const orc_sea *s, double t, double x, double y);
double orc_u(const orc_sea *s, double t, double x, double y, double z);
double orc_v(const orc_sea *s, double t, double x, double y, double z);
double orc_w(const orc_sea *s, double t, double x, double y, double z);
double orc_dp(const orc_sea *s, double t, double x, double y, double z);
double orc_eta1(const orc_sea *s, double t, double x, double y);
double orc_eta2(const orc_sea *s, double t, double x, double y);
void orc_uvw2(const orc_sea *s, double t, double x, double y, double z, double out[4]);

/* Batched versions (OpenMP over points; nthreads<=0 uses the default).
 * fields bit mask: 1 eta, 2 u, 4 v, 8 w, 16 dp.  out is [n][5]. */
void orc_irregular_batch(const orc_sea *s, long n, const double *x, const double *y,
                         const double *z, const double *t, int fields, double *out,
                         int nthreads);
/* Smit et al. (2017) s-coordinate kinematics of vertical_theory smit
 * (u_smit, v_smit, w_smit, dp_smit, Irregular.cpp:1622-2027): out [n][4] =
 * u, v, w, dp without ramp; 0 above eta1 + eta2 + swl. */
void orc_smit_batch(const orc_sea *s, long n, const double *x, const double *y, const double *z,
                    const double *t, double *out, int nthreads);
/* uvw2 batched: out [n][4]. */
void orc_uvw2_batch(const orc_sea *s, long n, const double *x, const double *y,
                    const double *z, const double *t, double *out, int nthreads);

/* ------------------------------------------------------------------ */
/* Ramp (Utils.cpp:26-68)                                               */
/* ------------------------------------------------------------------ */
/* flags bit i enables ramp i of (time up, time down, x up, x down, y up,
 * y down); lim[2i], lim[2i+1] are its start/end.  init=0 returns 1. */
double orc_ramp(int init, int flags, const double lim[12], double t, double x, double y);

/* ------------------------------------------------------------------ */
/* Lagrangian stretched grid with spline query (lsgrid_spline.cpp)       */
/* ------------------------------------------------------------------ */
typedef struct orc_sgrid orc_sgrid;
orc_sgrid *orc_sgrid_create(int nx, int ny, int nl, const double domain[4],
                            const double domain_ignore[4], double t0, double dt,
                            double tan_a, double tan_b, double water_depth, double swl);
void orc_sgrid_free(orc_sgrid *g);
/* initialize_kinematics[_with_ignore] (lsgrid_spline.cpp:666-844). */
void orc_sgrid_init(orc_sgrid *g, const orc_sea *s, int with_ignore, int nthreads);
/* update (lsgrid_spline.cpp:847-931): one ring step. */
void orc_sgrid_update(orc_sgrid *g, const orc_sea *s, int nthreads);
/* CheckTime (lsgrid_spline.cpp:610). */
int orc_sgrid_check_time(const orc_sgrid *g, double t);
/* get_kinematics_at_point (lsgrid_spline.cpp:505-605): out [n][4]. */
void orc_sgrid_query(const orc_sgrid *g, long n, const double *x, const double *y,
                     const double *z, const double *t, double *out, int nthreads);
/* Dynamic pressure on the ring (extension of the reference's grid): before
 * orc_sgrid_init, on = 1 adds the field dp1(z0) + rho uvw2.p(z0) +
 * dp1_dz max(0, z - swl) at every node, with its gradients. */
void orc_sgrid_set_pressure(orc_sgrid *g, int on);
/* The query with the pressure: out [n][5] = eta, u, v, w, p. */
void orc_sgrid_query5(const orc_sgrid *g, long n, const double *x, const double *y,
                      const double *z, const double *t, double *out, int nthreads);
/* Column-subset update for the CPU baseline: only columns [c0, c1) of the
 * flattened (i*ny+j) order are computed, into the next ring slot. */
void orc_sgrid_update_columns(orc_sgrid *g, const orc_sea *s, double t, long c0, long c1,
                              int nthreads);
/* Raw access to the grid arrays for tests.  which: 0 ETA, 1 UX, 2 UY, 3 UZ,
 * 4 ETAdx, 5 ETAdy, 6 ETAdt, 7 Udt, 8 Udx, 9 Udy, 10 Uds, 11 Vdt, 12 Vdx,
 * 13 Vdy, 14 Vds, 15 Wdt, 16 Wdx, 17 Wdy, 18 Wds, 19 IGNORE (as double);
 * with the pressure: 20 PP, 21 Pdt, 22 Pdx, 23 Pdy, 24 Pds. */
long orc_sgrid_array(const orc_sgrid *g, int which, double *dst);
/* update() split as a rank of the reference's MPI build runs it: advance the
 * ring, fill columns (orc_sgrid_update_columns at t0 + 2 dt), replace the
 * newest slot of ETA/UX/UY/UZ (which 0..3) by the gathered one, gradients. */
void orc_sgrid_advance(orc_sgrid *g);
void orc_sgrid_gradients(orc_sgrid *g);
int orc_sgrid_set_slot(orc_sgrid *g, int which, const double *src);
/* export_vtu (lsgrid_spline.cpp:1222-1403) of the base slot (last = 0) or the
 * slot after it (last = 1) into the file `path`; 0 or -1. */
int orc_sgrid_export_vtu(const orc_sgrid *g, const char *path, int last, const char *label);
void orc_sgrid_state(const orc_sgrid *g, double *t0, int *tstep);

/* ------------------------------------------------------------------ */
/* Stokes 5th order (Stokes5.cpp)                                       */
/* ------------------------------------------------------------------ */
typedef struct orc_stokes5 orc_stokes5;
orc_stokes5 *orc_stokes5_create(double wave_length, double wave_height, double depth,
                                double current, double gravity, double rho, double x0,
                                double y0, double z0, double t0, double theta);
void orc_stokes5_free(orc_stokes5 *s);
/* out [n][5] = eta, u, v, w, dp (no ramp, no clamp) */
void orc_stokes5_batch(const orc_stokes5 *s, long n, const double *x, const double *y,
                       const double *z, const double *t, double *out, int nthreads);
void orc_stokes5_coeffs(const orc_stokes5 *s, double *dst /* 32 */);
/* Linear dispersion (Stokes5.cpp:187-229). */
double orc_wavenumber_from_period(double T, double depth, double g);
double orc_wavelength_from_period(double T, double depth, double g);
double orc_period_from_length(double L, double depth, double g);

/* ------------------------------------------------------------------ */
/* Fenton stream function (FentonStream.cpp)                           */
/* ------------------------------------------------------------------ */
typedef struct orc_fenton orc_fenton;
/* Returns NULL and sets *status (1 bad input, 2 singular) on failure.
 * *status = 0 converged, 3 not fully converged (reference only warns). */
orc_fenton *orc_fenton_create(double wave_height, double wave_length, double wave_period,
                              int specify_length, int current_type, int n_fourier,
                              int n_steps, double depth, double current, double gravity,
                              double rho, double x0, double y0, double z0, double t0,
                              double theta, int *status);
void orc_fenton_free(orc_fenton *f);
/* out [n][5] = eta, u, v, w, dp */
void orc_fenton_batch(const orc_fenton *f, long n, const double *x, const double *y,
                      const double *z, const double *t, double *out, int nthreads);
/* k, c, ubar, R, L, T, then B[1..N], then Y[1..N]: returns count written. */
int orc_fenton_solution(const orc_fenton *f, double *dst);

#ifdef __cplusplus
}
#endif
#endif
