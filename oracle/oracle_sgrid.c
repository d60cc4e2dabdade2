/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY): FP64 restatement of the reference's
 * Lagrangian stretched grid with cubic-Hermite query,
 * oystelan/CFDwavemaker v3.1.0 src/lsgrid_spline.cpp.
 * The product never links this file; see oracle.h.
 */
#include "oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

double orc__eta1(const orc_sea *s, double t, double x, double y);
double orc__u1(const orc_sea *s, double t, double x, double y, double z);
double orc__v1(const orc_sea *s, double t, double x, double y, double z);
double orc__w1(const orc_sea *s, double t, double x, double y, double z);
double orc__phi1_dxdz(const orc_sea *s, double t, double x, double y);
double orc__phi1_dydz(const orc_sea *s, double t, double x, double y);
double orc__phi1_dzdz(const orc_sea *s, double t, double x, double y);
double orc__dp1(const orc_sea *s, double t, double x, double y, double z);
double orc__dp1_dz(const orc_sea *s, double t, double x, double y);
double orc__rho(const orc_sea *s);

struct orc_sgrid {
    int nx, ny, nl;
    double domain[4], domain_ignore[4];
    double t0, dt, tan_a, tan_b, water_depth, swl, dx, dy, ds;
    int tstep;
    /* lsgrid_spline.cpp:35-61 */
    double *ETA, *UX, *UY, *UZ, *ETAdx, *ETAdy, *ETAdt;
    double *Udt, *Udx, *Udy, *Uds, *Vdt, *Vdx, *Vdy, *Vds, *Wdt, *Wdx, *Wdy, *Wds;
    int *IGNORE;
    /* dynamic pressure on the ring (an extension: the reference's grid keeps
     * no pressure; its update computes uvw2.p, lsgrid_spline.cpp:892, and
     * drops it) */
    int pressure;
    double *PP, *Pdt, *Pdx, *Pdy, *Pds;
};

static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }
static int iclamp(int n, int lo, int hi) { return n < lo ? lo : (n > hi ? hi : n); }
static double dclamp(double n, double lo, double hi) { return dmax(lo, dmin(n, hi)); }

orc_sgrid *orc_sgrid_create(int nx, int ny, int nl, const double domain[4],
                            const double domain_ignore[4], double t0, double dt,
                            double tan_a, double tan_b, double water_depth, double swl) {
    orc_sgrid *g = (orc_sgrid *)calloc(1, sizeof(orc_sgrid));
    g->nx = nx; g->ny = ny; g->nl = nl;
    memcpy(g->domain, domain, sizeof(double) * 4);
    memcpy(g->domain_ignore, domain_ignore, sizeof(double) * 4);
    g->t0 = t0; g->dt = dt; g->tan_a = tan_a; g->tan_b = tan_b;
    g->water_depth = water_depth; g->swl = swl;
    size_t c = (size_t)nx * ny, v = c * nl;
    g->ETA = calloc(4 * c, sizeof(double));
    g->UX = calloc(4 * v, sizeof(double)); g->UY = calloc(4 * v, sizeof(double));
    g->UZ = calloc(4 * v, sizeof(double));
    g->ETAdx = calloc(2 * c, sizeof(double)); g->ETAdy = calloc(2 * c, sizeof(double));
    g->ETAdt = calloc(4 * c, sizeof(double));
    g->Udt = calloc(4 * v, sizeof(double)); g->Udx = calloc(2 * v, sizeof(double));
    g->Udy = calloc(2 * v, sizeof(double)); g->Uds = calloc(2 * v, sizeof(double));
    g->Vdt = calloc(4 * v, sizeof(double)); g->Vdx = calloc(2 * v, sizeof(double));
    g->Vdy = calloc(2 * v, sizeof(double)); g->Vds = calloc(2 * v, sizeof(double));
    g->Wdt = calloc(4 * v, sizeof(double)); g->Wdx = calloc(2 * v, sizeof(double));
    g->Wdy = calloc(2 * v, sizeof(double)); g->Wds = calloc(2 * v, sizeof(double));
    g->IGNORE = calloc(c, sizeof(int));
    /* set_ignore, lsgrid_spline.cpp:1406-1425 */
    g->dx = (domain[1] - domain[0]) / dmax(1., (double)(nx - 1));
    g->dy = (domain[3] - domain[2]) / dmax(1., (double)(ny - 1));
    g->ds = 1. / dmax(1., (double)(nl - 1));
    for (int i = 0; i < nx; i++) {
        double xp = domain[0] + g->dx * i;
        for (int j = 0; j < ny; j++) {
            double yp = domain[2] + g->dy * j;
            g->IGNORE[i * ny + j] = (xp >= domain_ignore[0] && xp <= domain_ignore[1] &&
                                     yp >= domain_ignore[2] && yp <= domain_ignore[3]) ? 1 : 0;
        }
    }
    return g;
}

void orc_sgrid_free(orc_sgrid *g) {
    if (!g) return;
    double *a[] = {g->ETA, g->UX, g->UY, g->UZ, g->ETAdx, g->ETAdy, g->ETAdt, g->Udt, g->Udx,
                   g->Udy, g->Uds, g->Vdt, g->Vdx, g->Vdy, g->Vds, g->Wdt, g->Wdx, g->Wdy, g->Wds,
                   g->PP, g->Pdt, g->Pdx, g->Pdy, g->Pds};
    for (size_t i = 0; i < sizeof(a) / sizeof(a[0]); i++) free(a[i]);
    free(g->IGNORE);
    free(g);
}

void orc_sgrid_set_pressure(orc_sgrid *g, int on) {
    size_t v = (size_t)g->nx * g->ny * g->nl;
    g->pressure = on ? 1 : 0;
    if (on && !g->PP) {
        g->PP = calloc(4 * v, sizeof(double)); g->Pdt = calloc(4 * v, sizeof(double));
        g->Pdx = calloc(2 * v, sizeof(double)); g->Pdy = calloc(2 * v, sizeof(double));
        g->Pds = calloc(2 * v, sizeof(double));
    }
}

/* z2s/s2z/cart2sigmaS/sigmaS2cart, lsgrid_spline.cpp:91-122 */
static double z2s(const orc_sgrid *g, double z, double e, double d) { return (z - (e - g->swl)) / (d + (e - g->swl)); }
static double s2z(const orc_sgrid *g, double s, double e, double d) { return (e - g->swl) + s * (d + (e - g->swl)); }
static double cart2sigmaS(const orc_sgrid *g, double zpt, double e, double d) {
    double z = dmin(zpt, e);
    double sigma = dmax(z2s(g, z, e, d), -1.);
    return 1 - atan(pow(-sigma * pow(tan(g->tan_a), g->tan_b), 1. / g->tan_b)) / g->tan_a;
}
static double sigmaS2cart(const orc_sgrid *g, double s, double e, double d) {
    double sigma = -pow(tan(-(s - 1) * g->tan_a), g->tan_b) / pow(tan(g->tan_a), g->tan_b);
    return s2z(g, sigma, e, d);
}

/* One column at time t into ring slot tt (body of lsgrid_spline.cpp:695-720 / 880-903). */
static void fill_column(orc_sgrid *g, const orc_sea *s, int tt, int i, int j, double t) {
    int nx = g->nx, ny = g->ny, nl = g->nl;
    double xp = g->domain[0] + g->dx * i, yp = g->domain[2] + g->dy * j;
    double e = orc__eta1(s, t, xp, yp) + orc_eta2(s, t, xp, yp) + g->swl;
    g->ETA[(size_t)tt * nx * ny + i * ny + j] = e;
    double gx = orc__phi1_dxdz(s, t, xp, yp), gy = orc__phi1_dydz(s, t, xp, yp),
           gz = orc__phi1_dzdz(s, t, xp, yp);
    for (int m = 0; m < nl; m++) {
        double z0 = sigmaS2cart(g, g->ds * m, e, g->water_depth);
        double zmax = dmax(0., z0 - g->swl), zmin = dmin(0., z0);
        double o[4];
        orc_uvw2(s, t, xp, yp, zmin, o);
        size_t id = (size_t)tt * nx * ny * nl + (size_t)i * ny * nl + (size_t)j * nl + m;
        g->UX[id] = orc__u1(s, t, xp, yp, zmin) + o[0] + gx * zmax;
        g->UY[id] = orc__v1(s, t, xp, yp, zmin) + o[1] + gy * zmax;
        g->UZ[id] = orc__w1(s, t, xp, yp, zmin) + o[2] + gz * zmax;
        /* the pressure with the velocities' convention: dp1 + rho uvw2.p at
         * zmin, the Taylor term dp1_dz above swl (Irregular.cpp:1107-1155) */
        if (g->pressure)
            g->PP[id] = orc__dp1(s, t, xp, yp, zmin) + orc__rho(s) * o[3] + orc__dp1_dz(s, t, xp, yp) * zmax;
    }
}

/* update_gradient_dt / _eta_dt, lsgrid_spline.cpp:124-164 */
static void grad_dt(const orc_sgrid *g, const double *d, double *gd, size_t stride) {
    if (g->tstep > 0) {
        int tid = (g->tstep + 2) % 4, tid1 = (g->tstep + 3) % 4, tid0 = (g->tstep + 1) % 4;
        for (size_t i = 0; i < stride; i++)
            gd[tid * stride + i] = (d[tid1 * stride + i] - d[tid0 * stride + i]) / (2 * g->dt);
    } else {
        for (size_t i = 0; i < stride; i++) {
            gd[1 * stride + i] = (d[2 * stride + i] - d[1 * stride + i]) / g->dt;
            gd[2 * stride + i] = (d[3 * stride + i] - d[1 * stride + i]) / (2 * g->dt);
        }
    }
}

/* update_gradient_eta_dxdy and update_gradient_dxdydz,
 * lsgrid_spline.cpp:166-366; nlv=1 gives the elevation version (no s). */
static void grad_space(const orc_sgrid *g, const double *d, double *gx, double *gy, double *gs, int nlv) {
    int nx = g->nx, ny = g->ny, nl = nlv;
    size_t S = (size_t)nx * ny * nl;
    int tids[2] = {(g->tstep + 1) % 4, (g->tstep + 2) % 4};
    for (int q = 0; q < 2; q++) {
        const double *D = d + tids[q] * S;
        double *GX = gx + q * S, *GY = gy + q * S, *GS = gs ? gs + q * S : NULL;
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < ny; j++)
                for (int m = 0; m < nl; m++) {
                    size_t id = (size_t)i * ny * nl + (size_t)j * nl + m;
                    if (nx == 1) GX[id] = 0.;
                    else if (i == 0) GX[id] = (D[id + (size_t)ny * nl] - D[id]) / g->dx;
                    else if (i == nx - 1) GX[id] = (D[id] - D[id - (size_t)ny * nl]) / g->dx;
                    else GX[id] = (D[id + (size_t)ny * nl] - D[id - (size_t)ny * nl]) / (2 * g->dx);
                    if (ny == 1) GY[id] = 0.;
                    else if (j == 0) GY[id] = (D[id + nl] - D[id]) / g->dy;
                    else if (j == ny - 1) GY[id] = (D[id] - D[id - nl]) / g->dy;
                    else GY[id] = (D[id + nl] - D[id - nl]) / (2 * g->dy);
                    if (GS) {
                        if (nl == 1) GS[id] = 0.;
                        else if (m == 0) GS[id] = (D[id + 1] - D[id]) / g->ds;
                        else if (m == nl - 1) GS[id] = (D[id] - D[id - 1]) / g->ds;
                        else GS[id] = (D[id + 1] - D[id - 1]) / (2 * g->ds);
                    }
                }
    }
}

static void all_gradients(orc_sgrid *g) {
    size_t c = (size_t)g->nx * g->ny, v = c * g->nl;
    grad_space(g, g->ETA, g->ETAdx, g->ETAdy, NULL, 1);
    grad_dt(g, g->ETA, g->ETAdt, c);
    grad_space(g, g->UX, g->Udx, g->Udy, g->Uds, g->nl);
    grad_dt(g, g->UX, g->Udt, v);
    grad_space(g, g->UY, g->Vdx, g->Vdy, g->Vds, g->nl);
    grad_dt(g, g->UY, g->Vdt, v);
    grad_space(g, g->UZ, g->Wdx, g->Wdy, g->Wds, g->nl);
    grad_dt(g, g->UZ, g->Wdt, v);
    if (g->pressure) {
        grad_space(g, g->PP, g->Pdx, g->Pdy, g->Pds, g->nl);
        grad_dt(g, g->PP, g->Pdt, v);
    }
}

void orc_sgrid_init(orc_sgrid *g, const orc_sea *s, int with_ignore, int nthreads) {
    double tt0a[4] = {g->t0 - g->dt, g->t0, g->t0 + g->dt, g->t0 + 2 * g->dt};
    double tt0b[4] = {g->t0, g->t0, g->t0 + g->dt, g->t0 + 2 * g->dt};
    double *tt0 = with_ignore ? tt0b : tt0a;
    long ncol = (long)g->nx * g->ny;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long q = 0; q < 4 * ncol; q++) {
        int tt = (int)(q / ncol);
        long c = q % ncol;
        int i = (int)(c / g->ny), j = (int)(c % g->ny);
        if (with_ignore && g->IGNORE[c]) continue;
        fill_column(g, s, tt, i, j, tt0[tt]);
    }
    all_gradients(g);
    (void)nthreads;
}

void orc_sgrid_update(orc_sgrid *g, const orc_sea *s, int nthreads) {
    g->tstep++;
    g->t0 += g->dt;
    double t2 = g->t0 + 2 * g->dt;
    int tt = (g->tstep + 3) % 4;
    long ncol = (long)g->nx * g->ny;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long c = 0; c < ncol; c++) {
        if (g->IGNORE[c]) continue;
        fill_column(g, s, tt, (int)(c / g->ny), (int)(c % g->ny), t2);
    }
    all_gradients(g);
    (void)nthreads;
}

void orc_sgrid_update_columns(orc_sgrid *g, const orc_sea *s, double t, long c0, long c1,
                              int nthreads) {
    int tt = (g->tstep + 3) % 4;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long c = c0; c < c1; c++) {
        if (g->IGNORE[c]) continue;
        fill_column(g, s, tt, (int)(c / g->ny), (int)(c % g->ny), t);
    }
    (void)nthreads;
}

int orc_sgrid_check_time(const orc_sgrid *g, double t) { return t > g->t0 + g->dt; }

/* The three parts of update() (lsgrid_spline.cpp:847-931) as the MPI build
 * runs them on each rank: advance the ring, fill a column subset
 * (orc_sgrid_update_columns at t0 + 2 dt), set the gathered slot, gradients. */
void orc_sgrid_advance(orc_sgrid *g) {
    g->tstep++;
    g->t0 += g->dt;
}

void orc_sgrid_gradients(orc_sgrid *g) { all_gradients(g); }

/* Replaces the newest slot of array which (0 ETA, 1 UX, 2 UY, 3 UZ) by src. */
int orc_sgrid_set_slot(orc_sgrid *g, int which, const double *src) {
    size_t c = (size_t)g->nx * g->ny, v = c * g->nl;
    int tt = (g->tstep + 3) % 4;
    double *arr[4] = {g->ETA, g->UX, g->UY, g->UZ};
    if (which < 0 || which > 3) return -1;
    size_t n = which == 0 ? c : v;
    memcpy(arr[which] + (size_t)tt * n, src, n * sizeof(double));
    return 0;
}

/* square_vals / cube_vals, lsgrid_spline.cpp:368-384 */
static void square_vals(const orc_sgrid *g, double *C, const double *d, int xp, int yp, int tid) {
    int nx = g->nx, ny = g->ny;
    size_t b = (size_t)tid * nx * ny;
    int x1 = iclamp(xp + 1, 0, nx - 1), y1 = iclamp(yp + 1, 0, ny - 1);
    C[0] = d[b + (size_t)xp * ny + yp];
    C[1] = d[b + (size_t)xp * ny + y1];
    C[2] = d[b + (size_t)x1 * ny + yp];
    C[3] = d[b + (size_t)x1 * ny + y1];
}
static void cube_vals(const orc_sgrid *g, double *C, const double *d, int xp, int yp, int lp, int tid) {
    int nx = g->nx, ny = g->ny, nl = g->nl;
    size_t b = (size_t)tid * nx * ny * nl;
    int x1 = iclamp(xp + 1, 0, nx - 1), y1 = iclamp(yp + 1, 0, ny - 1), l1 = iclamp(lp + 1, 0, nl - 1);
#define ID(a, bb, c) (b + (size_t)(a) * ny * nl + (size_t)(bb) * nl + (c))
    C[0] = d[ID(xp, yp, lp)]; C[1] = d[ID(xp, y1, lp)]; C[2] = d[ID(x1, yp, lp)]; C[3] = d[ID(x1, y1, lp)];
    C[4] = d[ID(xp, yp, l1)]; C[5] = d[ID(xp, y1, l1)]; C[6] = d[ID(x1, yp, l1)]; C[7] = d[ID(x1, y1, l1)];
#undef ID
}

/* Cubic Hermite on [0,1] in the reference's form:
 * f0(1-r) + f1 r + r(1-r)(a(1-r) + b r), a = h f0' - (f1-f0), b = -h f1' + (f1-f0). */
static double herm(double f0, double f1, double d0, double d1, double h, double r) {
    double a = h * d0 - (f1 - f0), b = -h * d1 + (f1 - f0);
    return f0 * (1. - r) + f1 * r + r * (1 - r) * (a * (1 - r) + b * r);
}
static double lin(double f0, double f1, double r) { return f0 * (1. - r) + f1 * r; }

/* spline_interp_velo, lsgrid_spline.cpp:386-502 */
static double spline_velo(const orc_sgrid *g, const double *U, const double *Ut, const double *Ux,
                          const double *Uy, const double *Us, int xp, int yp, int s0, int s1,
                          double xd, double yd, double sd0, double sd1, double td, int t1, int t2) {
    double C[8], D[8], Ct[8], Dt[8], Cx[8], Dx[8], Cy[8], Dy[8], Cs[8], Ds[8];
    cube_vals(g, C, U, xp, yp, s0, t1); cube_vals(g, D, U, xp, yp, s1, t2);
    cube_vals(g, Ct, Ut, xp, yp, s0, t1); cube_vals(g, Dt, Ut, xp, yp, s1, t2);
    cube_vals(g, Cx, Ux, xp, yp, s0, 0); cube_vals(g, Dx, Ux, xp, yp, s1, 1);
    cube_vals(g, Cy, Uy, xp, yp, s0, 0); cube_vals(g, Dy, Uy, xp, yp, s1, 1);
    cube_vals(g, Cs, Us, xp, yp, s0, 0); cube_vals(g, Ds, Us, xp, yp, s1, 1);
    /* x reduction: corner pairs (0,2) (1,3) (4,6) (5,7) */
    static const int lo[4] = {0, 1, 4, 5}, hi[4] = {2, 3, 6, 7};
    double Cv[4], Dv[4], Cyv[4], Dyv[4], Ctv[4], Dtv[4], Csv[4], Dsv[4];
    for (int q = 0; q < 4; q++) {
        Cv[q] = herm(C[lo[q]], C[hi[q]], Cx[lo[q]], Cx[hi[q]], g->dx, xd);
        Dv[q] = herm(D[lo[q]], D[hi[q]], Dx[lo[q]], Dx[hi[q]], g->dx, xd);
        Cyv[q] = lin(Cy[lo[q]], Cy[hi[q]], xd); Dyv[q] = lin(Dy[lo[q]], Dy[hi[q]], xd);
        Ctv[q] = lin(Ct[lo[q]], Ct[hi[q]], xd); Dtv[q] = lin(Dt[lo[q]], Dt[hi[q]], xd);
        Csv[q] = lin(Cs[lo[q]], Cs[hi[q]], xd); Dsv[q] = lin(Ds[lo[q]], Ds[hi[q]], xd);
    }
    /* y reduction: (00,10) -> 0, (01,11) -> 1 */
    double C0 = herm(Cv[0], Cv[1], Cyv[0], Cyv[1], g->dy, yd);
    double C1 = herm(Cv[2], Cv[3], Cyv[2], Cyv[3], g->dy, yd);
    double D0 = herm(Dv[0], Dv[1], Dyv[0], Dyv[1], g->dy, yd);
    double D1 = herm(Dv[2], Dv[3], Dyv[2], Dyv[3], g->dy, yd);
    double C0s = lin(Csv[0], Csv[1], yd), C1s = lin(Csv[2], Csv[3], yd);
    double D0s = lin(Dsv[0], Dsv[1], yd), D1s = lin(Dsv[2], Dsv[3], yd);
    double C0t = lin(Ctv[0], Ctv[1], yd), C1t = lin(Ctv[2], Ctv[3], yd);
    double D0t = lin(Dtv[0], Dtv[1], yd), D1t = lin(Dtv[2], Dtv[3], yd);
    /* s reduction */
    double CC = herm(C0, C1, C0s, C1s, g->ds, sd0);
    double DD = herm(D0, D1, D0s, D1s, g->ds, sd1);
    double CCt = lin(C0t, C1t, sd0), DDt = lin(D0t, D1t, sd1);
    /* t reduction */
    return herm(CC, DD, CCt, DDt, g->dt, td);
}

/* get_kinematics_at_point, lsgrid_spline.cpp:505-605.  The reference calls
 * std::modf with a float* second argument, which selects the float overload:
 * the cell fractions are therefore rounded to float before splitting. */
static void query_one(const orc_sgrid *g, double tpt, double xpt, double ypt, double zpt, double *o) {
    int nx = g->nx, ny = g->ny;
    int tid1 = (g->tstep + 1) % 4, tid2 = (g->tstep + 2) % 4;
    float xi, yi;
    double xd = modff((float)dclamp((xpt - g->domain[0]) / g->dx, 0., nx - 1.), &xi);
    double yd = modff((float)dclamp((ypt - g->domain[2]) / g->dy, 0., ny - 1.), &yi);
    double td = dmin(1., dmax(0., (tpt - g->t0) / g->dt));
    int xp = (int)xi, yp = (int)yi;
    double C[4], D[4], Ct[4], Dt[4], Cx[4], Dx[4], Cy[4], Dy[4];
    square_vals(g, C, g->ETA, xp, yp, tid1); square_vals(g, D, g->ETA, xp, yp, tid2);
    square_vals(g, Ct, g->ETAdt, xp, yp, tid1); square_vals(g, Dt, g->ETAdt, xp, yp, tid2);
    square_vals(g, Cx, g->ETAdx, xp, yp, 0); square_vals(g, Dx, g->ETAdx, xp, yp, 1);
    square_vals(g, Cy, g->ETAdy, xp, yp, 0); square_vals(g, Dy, g->ETAdy, xp, yp, 1);
    double C0 = herm(C[0], C[2], Cx[0], Cx[2], g->dx, xd);
    double C1 = herm(C[1], C[3], Cx[1], Cx[3], g->dx, xd);
    double D0 = herm(D[0], D[2], Dx[0], Dx[2], g->dx, xd);
    double D1 = herm(D[1], D[3], Dx[1], Dx[3], g->dx, xd);
    double C0y = lin(Cy[0], Cy[2], xd), C1y = lin(Cy[1], Cy[3], xd);
    double D0y = lin(Dy[0], Dy[2], xd), D1y = lin(Dy[1], Dy[3], xd);
    double C0t = lin(Ct[0], Ct[2], xd), C1t = lin(Ct[1], Ct[3], xd);
    double D0t = lin(Dt[0], Dt[2], xd), D1t = lin(Dt[1], Dt[3], xd);
    double e0 = herm(C0, C1, C0y, C1y, g->dy, yd);
    double e1 = herm(D0, D1, D0y, D1y, g->dy, yd);
    double CCt = lin(C0t, C1t, yd), DDt = lin(D0t, D1t, yd);
    double eta = herm(e0, e1, CCt, DDt, g->dt, td);
    double spt0 = cart2sigmaS(g, zpt, e0, g->water_depth), n0 = spt0 / g->ds;
    double spt1 = cart2sigmaS(g, zpt, e1, g->water_depth), n1 = spt1 / g->ds;
    float s0i, s1i;
    double sd0 = modff((float)n0, &s0i), sd1 = modff((float)n1, &s1i);
    int s0 = (int)s0i, s1 = (int)s1i;
    o[0] = eta;
    o[1] = spline_velo(g, g->UX, g->Udt, g->Udx, g->Udy, g->Uds, xp, yp, s0, s1, xd, yd, sd0, sd1, td, tid1, tid2);
    o[2] = spline_velo(g, g->UY, g->Vdt, g->Vdx, g->Vdy, g->Vds, xp, yp, s0, s1, xd, yd, sd0, sd1, td, tid1, tid2);
    o[3] = spline_velo(g, g->UZ, g->Wdt, g->Wdx, g->Wdy, g->Wds, xp, yp, s0, s1, xd, yd, sd0, sd1, td, tid1, tid2);
    if (g->pressure)
        o[4] = spline_velo(g, g->PP, g->Pdt, g->Pdx, g->Pdy, g->Pds, xp, yp, s0, s1, xd, yd, sd0, sd1, td, tid1,
                           tid2);
}

void orc_sgrid_query(const orc_sgrid *g, long n, const double *x, const double *y,
                     const double *z, const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) {
        double o[5];
        query_one(g, t[p], x[p], y[p], z[p], o);
        for (int q = 0; q < 4; q++) out[4 * p + q] = o[q];
    }
    (void)nthreads;
}

void orc_sgrid_query5(const orc_sgrid *g, long n, const double *x, const double *y,
                      const double *z, const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) {
        double o[5] = {0, 0, 0, 0, 0};
        query_one(g, t[p], x[p], y[p], z[p], o);
        for (int q = 0; q < 5; q++) out[5 * p + q] = o[q];
    }
    (void)nthreads;
}

long orc_sgrid_array(const orc_sgrid *g, int which, double *dst) {
    size_t c = (size_t)g->nx * g->ny, v = c * g->nl;
    const double *src = NULL;
    size_t n = 0;
    switch (which) {
    case 0: src = g->ETA; n = 4 * c; break;
    case 1: src = g->UX; n = 4 * v; break;
    case 2: src = g->UY; n = 4 * v; break;
    case 3: src = g->UZ; n = 4 * v; break;
    case 4: src = g->ETAdx; n = 2 * c; break;
    case 5: src = g->ETAdy; n = 2 * c; break;
    case 6: src = g->ETAdt; n = 4 * c; break;
    case 7: src = g->Udt; n = 4 * v; break;
    case 8: src = g->Udx; n = 2 * v; break;
    case 9: src = g->Udy; n = 2 * v; break;
    case 10: src = g->Uds; n = 2 * v; break;
    case 11: src = g->Vdt; n = 4 * v; break;
    case 12: src = g->Vdx; n = 2 * v; break;
    case 13: src = g->Vdy; n = 2 * v; break;
    case 14: src = g->Vds; n = 2 * v; break;
    case 15: src = g->Wdt; n = 4 * v; break;
    case 16: src = g->Wdx; n = 2 * v; break;
    case 17: src = g->Wdy; n = 2 * v; break;
    case 18: src = g->Wds; n = 2 * v; break;
    case 19:
        if (dst) for (size_t i = 0; i < c; i++) dst[i] = g->IGNORE[i];
        return (long)c;
    case 20: case 21: case 22: case 23: case 24: {
        if (!g->pressure) return -1;
        const double *pa[5] = {g->PP, g->Pdt, g->Pdx, g->Pdy, g->Pds};
        src = pa[which - 20];
        n = (which <= 21 ? 4 : 2) * v;
        break;
    }
    default: return -1;
    }
    if (dst) memcpy(dst, src, n * sizeof(double));
    return (long)n;
}

/* export_vtu, lsgrid_spline.cpp:1222-1403: ASCII VTK UnstructuredGrid of the
 * base slot (last = 0) or the slot after it (last = 1). */
static void vtu_cells_tail(FILE *fp, long ncell, int per, const char *type) {
    fputs("\t\t\t\t </DataArray>\n", fp);
    fputs("\t\t\t\t <DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n", fp);
    for (long q = 1; q < ncell + 1; q++) fprintf(fp, "%d \n", (int)(q * per));
    fputs("\t\t\t\t </DataArray>\n", fp);
    fputs("\t\t\t\t <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n", fp);
    for (long q = 1; q < ncell + 1; q++) fprintf(fp, "%s \n", type);
}

int orc_sgrid_export_vtu(const orc_sgrid *g, const char *path, int last, const char *label) {
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    int nx = g->nx, ny = g->ny, nl = g->nl;
    double tv = last ? g->t0 + g->dt : g->t0;
    fputs("<?xml version=\"1.0\"?>\n"
          "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n", fp);
    fputs("\t <UnstructuredGrid>\n", fp);
    fprintf(fp, "\t\t <FieldData> \n");
    fprintf(fp, "\t\t\t <DataArray type = \"Float64\" Name = \"%s\" NumberOfTuples = \"1\" format = \"ascii\" "
                "RangeMin = \"%.3f\" RangeMax = \"%.3f\"> \n", label, tv, tv);
    fprintf(fp, "\t\t\t %.3f \n", tv);
    fprintf(fp, "\t\t\t </DataArray > \n");
    fprintf(fp, "\t\t </FieldData> \n");
    fprintf(fp, "\t\t <Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nx * ny * nl,
            (nx > 1 ? nx - 1 : 1) * (ny > 1 ? ny - 1 : 1) * (nl > 1 ? nl - 1 : 1));
    fputs("\t\t\t <PointData Scalars=\"scalars\">\n", fp);
    fprintf(fp, "\t\t\t\t <DataArray type=\"Float64\" NumberOfComponents=\"3\" Name=\"Velocity\" format=\"ascii\">\n");
    int tt = last ? (g->tstep + 2) % 4 : (g->tstep + 1) % 4;
    size_t b = (size_t)tt * nx * ny * nl;
    for (size_t e = 0; e < (size_t)nx * ny * nl; e++)
        fprintf(fp, "%g %g %g\n", g->UX[b + e], g->UY[b + e], g->UZ[b + e]);
    fputs("\t\t\t\t </DataArray>\n", fp);
    fputs("\t\t\t </PointData>\n", fp);
    fputs("\t\t\t <Points>\n", fp);
    fputs("\t\t\t\t <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n", fp);
    for (int i = 0; i < nx; i++) {
        double xpt = g->domain[0] + g->dx * i;
        for (int j = 0; j < ny; j++) {
            double ypt = g->domain[2] + g->dy * j;
            double et = g->ETA[(size_t)tt * nx * ny + (size_t)i * ny + j];
            for (int m = 0; m < nl; m++) {
                double sp = -pow(tan(-(-1. + g->ds * m) * g->tan_a), g->tan_b) / pow(tan(g->tan_a), g->tan_b);
                fprintf(fp, "%12.4f %12.4f %12.4f\n", xpt, ypt, s2z(g, sp, et, g->water_depth));
            }
        }
    }
    fputs("\t\t\t\t </DataArray>\n", fp);
    fputs("\t\t\t </Points>\n", fp);
    fputs("\t\t\t <Cells>\n", fp);
    fputs("\t\t\t\t <DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n", fp);
    if (nx > 1 && ny > 1 && nl > 1) {
        for (int i = 0; i < nx - 1; i++)
            for (int j = 0; j < ny - 1; j++)
                for (int m = 0; m < nl - 1; m++) {
                    unsigned a1 = nl * ny * i + nl * j + m, a2 = nl * ny * (i + 1) + nl * j + m;
                    unsigned a3 = nl * ny * (i + 1) + nl * (j + 1) + m, a4 = nl * ny * i + nl * (j + 1) + m;
                    fprintf(fp, "%u %u %u %u %u %u %u %u\n", a1, a2, a3, a4, a1 + 1, a2 + 1, a3 + 1, a4 + 1);
                }
        vtu_cells_tail(fp, (long)(nx - 1) * (ny - 1) * (nl - 1), 8, "12");
    } else if (nx > 1 && ny == 1 && nl > 1) {
        for (int i = 0; i < nx - 1; i++)
            for (int m = 0; m < nl - 1; m++)
                fprintf(fp, "%u %u %u %u\n", nl * i + m, nl * (i + 1) + m, nl * (i + 1) + m + 1, nl * i + m + 1);
        vtu_cells_tail(fp, (long)(nx - 1) * (nl - 1), 4, "9");
    } else if (nx == 1 && ny > 1 && nl > 1) {
        for (int j = 0; j < ny - 1; j++)
            for (int m = 0; m < nl - 1; m++)
                fprintf(fp, "%u %u %u %u\n", nl * j + m, nl * (j + 1) + m, nl * (j + 1) + m + 1, nl * j + m + 1);
        vtu_cells_tail(fp, (long)(ny - 1) * (nl - 1), 4, "9");
    } else if (nx > 1 && ny > 1 && nl == 1) {
        for (int i = 0; i < nx - 1; i++)
            for (int j = 0; j < ny - 1; j++)
                fprintf(fp, "%u %u %u %u\n", ny * i + j, ny * (i + 1) + j, ny * (i + 1) + j + 1, ny * i + j + 1);
        vtu_cells_tail(fp, (long)(nx - 1) * (ny - 1), 4, "9");
    }
    fputs("\t\t\t\t </DataArray>\n", fp);
    fputs("\t\t\t </Cells>\n", fp);
    fputs("\t\t </Piece>\n", fp);
    fputs("\t </UnstructuredGrid>\n", fp);
    fputs("</VTKFile>\n", fp);
    return fclose(fp) == 0 ? 0 : -1;
}

void orc_sgrid_state(const orc_sgrid *g, double *t0, int *tstep) {
    if (t0) *t0 = g->t0;
    if (tstep) *tstep = g->tstep;
}
