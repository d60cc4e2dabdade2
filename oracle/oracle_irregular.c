/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY): FP64 restatement of the reference's
 * irregular-sea kinematics, oystelan/CFDwavemaker v3.1.0 src/Irregular.cpp.
 * The product never links this file; see oracle.h.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Irregular.h:6-15 (the truncated PI is what Irregular.cpp sees). */
#define ORC_SMALL 1.e-12
#define ORC_HUGE 1.e12
#define ORC_PI_IRR 3.1415926535897

struct orc_sea {
    int n;
    double *omega, *A, *k, *theta, *phase, *ramptime, *starttime, *duration;
    double depth, mtheta, tofmax, fx, fy, swl, g, rho, dw_bandwidth, dw_cutoff;
    int order;
    /* component cache, Irregular.cpp:805-838 */
    double *cth, *sth, *R, *Rs, *agw, *cosh2kd, *phase0;
    double kmax;
    /* pair cache, Irregular.cpp:840-967 */
    long np;
    int *pi, *pm;
    unsigned char *hp, *hm;
    double *kp, *km, *Dp, *Dm, *ap, *am;
};

static double *dup_or_fill(int n, const double *src, double fill) {
    double *d = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) d[i] = src ? src[i] : fill;
    return d;
}

static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }

/* Irregular::freq_ramp, Irregular.cpp:200-204 */
static double freq_ramp(double t, double ramptime, double tstart, double duration) {
    double rampdown = dmax(dmin(1. - ((t - tstart - duration + ramptime) / (ramptime + ORC_SMALL)), 1.), 0.);
    double rampup = dmax(dmin(((t - tstart) / (ramptime + ORC_SMALL)), 1.), 0.);
    return rampup * rampdown;
}

/* rebuild_component_cache, Irregular.cpp:805-838 */
static void build_component_cache(orc_sea *s) {
    int N = s->n;
    double mt = s->mtheta * ORC_PI_IRR / 180.0;
    s->kmax = 0.0;
    for (int i = 0; i < N; ++i) {
        double th = s->theta[i] + mt;
        s->cth[i] = cos(th);
        s->sth[i] = sin(th);
        double R = s->k[i] * tanh(s->k[i] * s->depth);
        s->R[i] = R;
        s->Rs[i] = sqrt(R);
        s->agw[i] = s->A[i] * s->g / s->omega[i];
        s->cosh2kd[i] = cosh(2.0 * s->k[i] * s->depth);
        s->phase0[i] = s->omega[i] * s->tofmax + s->phase[i];
        if (s->k[i] > s->kmax) s->kmax = s->k[i];
    }
}

/* rebuild_pair_cache, Irregular.cpp:840-967 (H coefficients of the Smit
 * theory are not part of this path and are not kept). */
static void build_pair_cache(orc_sea *s) {
    int N = s->n;
    long cap = (long)N * (N - 1) / 2;
    if (cap < 1) cap = 1;
    s->pi = (int *)malloc(sizeof(int) * cap);
    s->pm = (int *)malloc(sizeof(int) * cap);
    s->hp = (unsigned char *)malloc(cap);
    s->hm = (unsigned char *)malloc(cap);
    s->kp = (double *)malloc(sizeof(double) * cap);
    s->km = (double *)malloc(sizeof(double) * cap);
    s->Dp = (double *)malloc(sizeof(double) * cap);
    s->Dm = (double *)malloc(sizeof(double) * cap);
    s->ap = (double *)malloc(sizeof(double) * cap);
    s->am = (double *)malloc(sizeof(double) * cap);
    long np = 0;
    double h = s->depth;
    for (int i = 0; i < N; ++i) {
        if (s->omega[i] > s->dw_cutoff) continue;
        double ki = s->k[i], oi = s->omega[i], Rni = s->R[i], Rsni = s->Rs[i];
        for (int m = i + 1; m < N; ++m) {
            if (s->omega[m] > s->dw_cutoff) continue;
            if (fabs(oi - s->omega[m]) > s->dw_bandwidth) continue;
            double km = s->k[m], Rnm = s->R[m], Rsm = s->Rs[m];
            double gamma = s->cth[i] * s->cth[m] + s->sth[i] * s->sth[m];
            double ki2 = ki * ki, km2 = km * km, kikm = ki * km;
            double kpl = sqrt(ki2 + km2 + 2.0 * kikm * gamma);
            double kmi = sqrt(ki2 + km2 - 2.0 * kikm * gamma);
            double sp = Rsni + Rsm, sm = Rsni - Rsm;
            double R2p = sp * sp, R2m = sm * sm;
            int hasp = 0, hasm = 0;
            double Dp = 0.0, Dm = 0.0, ap = 0.0, am = 0.0;
            if ((ki + km) <= s->kmax) {
                double den = R2p - kpl * tanh(kpl * h);
                Dp = (2.0 * R2p * (kikm * gamma - Rni * Rnm)) / den +
                     (sp * (Rsni * (km2 - Rnm * Rnm) + Rsm * (ki2 - Rni * Rni))) / den;
                ap = (Dp - (kikm * gamma - Rni * Rnm)) / sqrt(Rni * Rnm) + (Rni + Rnm);
                hasp = 1;
            }
            if (ki != km) {
                double den = R2m - kmi * tanh(kmi * h);
                Dm = (2.0 * R2m * (kikm * gamma + Rni * Rnm)) / den +
                     (sm * (-Rsni * (km2 - Rnm * Rnm) + Rsm * (ki2 - Rni * Rni))) / den;
                am = (Dm - (kikm * gamma + Rni * Rnm)) / sqrt(Rni * Rnm) + (Rni + Rnm);
                hasm = 1;
            }
            if (hasp || hasm) {
                s->pi[np] = i; s->pm[np] = m;
                s->hp[np] = (unsigned char)hasp; s->hm[np] = (unsigned char)hasm;
                s->kp[np] = kpl; s->km[np] = kmi;
                s->Dp[np] = Dp; s->Dm[np] = Dm; s->ap[np] = ap; s->am[np] = am;
                np++;
            }
        }
    }
    s->np = np;
}

orc_sea *orc_sea_create(int n, const double *omega, const double *A, const double *k,
                        const double *phase, const double *theta,
                        const double *ramptime, const double *starttime, const double *duration,
                        double depth, double mtheta, double tofmax, double fx, double fy,
                        double swl, double g, double rho, double dw_bandwidth, double dw_cutoff,
                        int order) {
    orc_sea *s = (orc_sea *)calloc(1, sizeof(orc_sea));
    s->n = n;
    s->omega = dup_or_fill(n, omega, 0.0);
    s->A = dup_or_fill(n, A, 0.0);
    s->k = dup_or_fill(n, k, 0.0);
    s->phase = dup_or_fill(n, phase, 0.0);
    s->theta = dup_or_fill(n, theta, 0.0);
    /* parser defaults, CFDwavemaker.cpp:719-722 */
    s->ramptime = dup_or_fill(n, ramptime, 0.0);
    s->starttime = dup_or_fill(n, starttime, -ORC_SMALL);
    s->duration = dup_or_fill(n, duration, ORC_HUGE);
    s->depth = depth; s->mtheta = mtheta; s->tofmax = tofmax; s->fx = fx; s->fy = fy;
    s->swl = swl; s->g = g; s->rho = rho; s->dw_bandwidth = dw_bandwidth;
    s->dw_cutoff = dw_cutoff; s->order = order;
    s->cth = dup_or_fill(n, NULL, 0.0); s->sth = dup_or_fill(n, NULL, 0.0);
    s->R = dup_or_fill(n, NULL, 0.0); s->Rs = dup_or_fill(n, NULL, 0.0);
    s->agw = dup_or_fill(n, NULL, 0.0); s->cosh2kd = dup_or_fill(n, NULL, 0.0);
    s->phase0 = dup_or_fill(n, NULL, 0.0);
    build_component_cache(s);
    build_pair_cache(s);
    return s;
}

void orc_sea_free(orc_sea *s) {
    if (!s) return;
    double *arrs[] = {s->omega, s->A, s->k, s->phase, s->theta, s->ramptime, s->starttime,
                      s->duration, s->cth, s->sth, s->R, s->Rs, s->agw, s->cosh2kd, s->phase0,
                      s->kp, s->km, s->Dp, s->Dm, s->ap, s->am};
    for (size_t i = 0; i < sizeof(arrs) / sizeof(arrs[0]); i++) free(arrs[i]);
    free(s->pi); free(s->pm); free(s->hp); free(s->hm);
    free(s);
}

long orc_sea_npairs(const orc_sea *s) { return s->np; }

/* Irregular::normalize_data, Irregular.cpp:1282-1297 */
void orc_normalize(int n, double *A, double *phase, int normalize, double ampl) {
    double sumA = 0.;
    for (int i = 0; i < n; i++) sumA += A[i];
    for (int i = 0; i < n; i++) {
        if (normalize) { A[i] = ampl * A[i] / sumA; phase[i] = 0.; }
        else A[i] = ampl * A[i];
    }
}

/* --- first order sums (Irregular.cpp:178-198, 394-447, 1107-1192) --- */

static double thmt(const orc_sea *s, int i) { return s->theta[i] + (s->mtheta * ORC_PI_IRR / 180.); }

static double arg1(const orc_sea *s, int i, double t, double xx, double yy) {
    double phi = s->omega[i] * s->tofmax + s->phase[i];
    return s->k[i] * (cos(thmt(s, i)) * (xx - s->fx) + sin(thmt(s, i)) * (yy - s->fy)) -
           s->omega[i] * t + phi;
}
static double framp(const orc_sea *s, int i, double t) {
    return freq_ramp(t, s->ramptime[i], s->starttime[i], s->duration[i]);
}
static double profX(const orc_sea *s, int i, double z) {
    return cosh(s->k[i] * (z + s->depth)) / cosh(s->k[i] * s->depth);
}
static double profZ(const orc_sea *s, int i, double z) {
    return sinh(s->k[i] * (z + s->depth)) / cosh(s->k[i] * s->depth);
}

double orc_eta1(const orc_sea *s, double t, double xx, double yy) {
    double w = 0.0;
    for (int i = 0; i < s->n; i++) w += s->A[i] * cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return w;
}
static double u1(const orc_sea *s, double t, double xx, double yy, double zz) {
    double u = 0.0;
    for (int i = 0; i < s->n; i++)
        u += s->A[i] * s->g * s->k[i] / s->omega[i] * profX(s, i, zz) * cos(thmt(s, i)) *
             cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return u;
}
static double v1(const orc_sea *s, double t, double xx, double yy, double zz) {
    double v = 0.0;
    for (int i = 0; i < s->n; i++)
        v += s->A[i] * s->g * s->k[i] / s->omega[i] * profX(s, i, zz) * sin(thmt(s, i)) *
             cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return v;
}
static double w1(const orc_sea *s, double t, double xx, double yy, double zz) {
    double w = 0.0;
    for (int i = 0; i < s->n; i++)
        w += s->A[i] * s->g * s->k[i] / s->omega[i] * profZ(s, i, zz) *
             sin(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return w;
}
static double dp1(const orc_sea *s, double t, double xx, double yy, double zz) {
    double p = 0.0;
    for (int i = 0; i < s->n; i++)
        p += s->A[i] * s->rho * s->g * (cosh(s->k[i] * (zz + s->depth)) / cosh(s->k[i] * s->depth)) *
             cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return p;
}
static double phi1_dxdz(const orc_sea *s, double t, double xx, double yy) {
    double u = 0.0;
    for (int i = 0; i < s->n; i++)
        u += cos(thmt(s, i)) * s->A[i] * s->omega[i] * s->k[i] * cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return u;
}
static double phi1_dydz(const orc_sea *s, double t, double xx, double yy) {
    double v = 0.0;
    for (int i = 0; i < s->n; i++)
        v += sin(thmt(s, i)) * s->A[i] * s->omega[i] * s->k[i] * cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return v;
}
static double phi1_dzdz(const orc_sea *s, double t, double xx, double yy) {
    double w = 0.0;
    for (int i = 0; i < s->n; i++)
        w += s->A[i] * s->omega[i] * s->k[i] * (cosh(s->k[i] * s->depth) / sinh(s->k[i] * s->depth)) *
             sin(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return w;
}
static double dp1_dz(const orc_sea *s, double t, double xx, double yy) {
    double p = 0.0;
    for (int i = 0; i < s->n; i++)
        p += s->A[i] * s->rho * s->g * s->k[i] * cos(arg1(s, i, t, xx, yy)) * framp(s, i, t);
    return p;
}

/* --- second order elevation from the pair cache (Irregular.cpp:223-293) --- */
double orc_eta2(const orc_sea *s, double t, double xx, double yy) {
    int N = s->n;
    double dxp = xx - s->fx, dyp = yy - s->fy, tot = 0.0;
    double *cphi = (double *)malloc(sizeof(double) * 3 * (size_t)(N > 0 ? N : 1));
    double *sphi = cphi + N, *ramp = sphi + N;
    for (int i = 0; i < N; ++i) {
        double ph = s->k[i] * (s->cth[i] * dxp + s->sth[i] * dyp) - s->omega[i] * t + s->phase0[i];
        cphi[i] = cos(ph); sphi[i] = sin(ph);
        ramp[i] = framp(s, i, t);
    }
    for (int i = 0; i < N; ++i) {
        if (s->omega[i] > s->dw_cutoff) continue;
        double ki = s->k[i], Rni = s->R[i], Rsni = s->Rs[i];
        double Dnn = (6.0 * Rsni * Rsni * (ki * ki - Rni * Rni)) /
                     (2.0 * Rsni * Rsni - ki * tanh(2.0 * ki * s->depth));
        double ann = (Dnn - (ki * ki - Rni * Rni)) / Rni + 2.0 * Rni;
        if (2.0 * ki <= s->kmax) {
            double c2 = cphi[i] * cphi[i] - sphi[i] * sphi[i];
            tot += 0.25 * s->A[i] * s->A[i] * ann * c2 * ramp[i];
        }
    }
    for (long p = 0; p < s->np; p++) {
        int i = s->pi[p], m = s->pm[p];
        double amp = 0.5 * s->A[i] * s->A[m], ri = ramp[i];
        if (s->hp[p]) tot += amp * s->ap[p] * (cphi[i] * cphi[m] - sphi[i] * sphi[m]) * ri;
        if (s->hm[p]) tot += amp * s->am[p] * (cphi[i] * cphi[m] + sphi[i] * sphi[m]) * ri;
    }
    free(cphi);
    return tot;
}

/* --- second order point-API velocity/pressure: u2/v2/w2/dp2
 *     (Irregular.cpp:450-506, 544-601, 638-695, 739-803).  The four
 *     reference functions share one loop body here; each output
 *     accumulates exactly the reference's terms. --- */
static void point_second_order(const orc_sea *s, double t, double xx, double yy, double zz,
                               int want, double out[4]) {
    int N = s->n;
    double g = s->g, h = s->depth;
    double ut = 0, vt = 0, wt = 0, pt = 0;
    for (int i = 0; i < N; i++) {
        double us = 0, vs = 0, ws = 0, ps = 0;
        double thi = thmt(s, i);
        double phi_i = s->k[i] * (cos(thi) * (xx - s->fx) + sin(thi) * (yy - s->fy)) -
                       s->omega[i] * t + s->omega[i] * s->tofmax + s->phase[i];
        double ki = s->k[i], oi = s->omega[i];
        double Rn = ki * tanh(ki * h), Rsn = sqrt(Rn);
        double Dnn = (6. * Rsn * Rsn * (ki * ki - Rn * Rn)) / (2. * Rsn * Rsn - ki * tanh(2 * ki * h));
        double AAd = 0.25 * (s->A[i] * g / oi) * (s->A[i] * g / oi) * (Dnn / (2 * oi));
        double cf = cosh(2 * ki * (zz + h)) / cosh(2 * ki * h);
        if (want & 1) us += AAd * (2 * ki * cos(thi)) * cos(2 * phi_i) * cf;
        if (want & 2) vs += AAd * (2 * ki * sin(thi)) * cos(2 * phi_i) * cf;
        if (want & 4) ws += AAd * 2 * ki * sin(2 * phi_i) * sinh(2 * ki * (zz + h)) / cosh(2 * ki * h);
        if (want & 8) {
            ps += AAd * (2 * oi) * cos(2 * phi_i) * cf;
            ps -= (g * g * (2 * ki * cos(thi) + 2 * ki * sin(thi)) * 2 * profX(s, i, zz)) / (2 * oi);
            ps += (g * g * (2 * ki) * 2 * profZ(s, i, zz)) / (2 * oi);
        }
        for (int m = i + 1; m < N; m++) {
            double thm = thmt(s, m);
            double km = s->k[m], om = s->omega[m];
            double phi_m = km * (cos(thm) * (xx - s->fx) + sin(thm) * (yy - s->fy)) - om * t +
                           om * s->tofmax + s->phase[m];
            double gam = cos(thi - thm);
            double kpl = sqrt(ki * ki + km * km + (2. * ki * km * gam));
            double kmi = sqrt(ki * ki + km * km - (2. * ki * km * gam));
            double Rm = km * tanh(km * h), Rsm = sqrt(Rm);
            double R2p = pow(Rsn + Rsm, 2.), R2m = pow(Rsn - Rsm, 2.);
            double Dp = (2. * R2p * (ki * km * gam - Rn * Rm)) / (R2p - kpl * tanh(kpl * h)) +
                        ((Rsn + Rsm) * (Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) /
                            (R2p - kpl * tanh(kpl * h));
            double Dm = (2. * R2m * (ki * km * gam + Rn * Rm)) / (R2m - kmi * tanh(kmi * h)) +
                        ((Rsn - Rsm) * (-Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) /
                            (R2m - kmi * tanh(kmi * h));
            double AA = 0.5 * (s->A[i] * g / oi) * (s->A[m] * g / om);
            double BB = (Dp / (oi + om));
            double chp = cosh(kpl * (zz + h)) / cosh(kpl * h);
            if (want & 1) us += AA * BB * (ki * cos(thi) + km * cos(thm)) * cos(phi_i + phi_m) * chp;
            if (want & 2) vs += AA * BB * (ki * sin(thi) + km * sin(thm)) * cos(phi_i + phi_m) * chp;
            if (want & 4) ws += AA * BB * kpl * sin(phi_i + phi_m) * (sinh(kpl * (zz + h)) / cosh(kpl * h));
            if (want & 8) {
                ps += AA * BB * (oi + om) * cos(phi_i + phi_m) * chp;
                ps -= (g * g * (ki * cos(thi) * km * cos(thm) + ki * sin(thi) * km * sin(thm)) *
                       profX(s, i, zz) * profX(s, m, zz)) / (oi * om);
                ps += (g * g * (ki * km) * profZ(s, i, zz) * profZ(s, m, zz)) / (oi * om);
            }
            if (ki != km) {
                double CC = (Dm / (oi - om));
                double chm = cosh(kmi * (zz + h)) / cosh(kmi * h);
                if (want & 1) us += AA * CC * (ki * cos(thi) - km * cos(thm)) * cos(phi_i - phi_m) * chm;
                if (want & 2) vs += AA * CC * (ki * sin(thi) - km * sin(thm)) * cos(phi_i - phi_m) * chm;
                if (want & 4) ws += AA * CC * kmi * sin(phi_i - phi_m) * (sinh(kmi * (zz + h)) / cosh(kmi * h));
                if (want & 8) ps += AA * CC * (oi - om) * cos(phi_i - phi_m) * chm;
            }
        }
        double r = framp(s, i, t);
        ut += us * r; vt += vs * r; wt += ws * r; pt += ps * r;
    }
    out[0] = ut; out[1] = vt; out[2] = wt; out[3] = s->rho * pt;
}

/* --- uvw2 from the pair cache, the s-grid variant (Irregular.cpp:975-1102) --- */
void orc_uvw2(const orc_sea *s, double t, double xx, double yy, double zz, double out[4]) {
    int N = s->n;
    double dxp = xx - s->fx, dyp = yy - s->fy, zpd = zz + s->depth, gg = s->g * s->g;
    double us = 0, vs = 0, ws = 0, ps = 0;
    double *buf = (double *)malloc(sizeof(double) * 5 * (size_t)(N > 0 ? N : 1));
    double *cphi = buf, *sphi = buf + N, *ramp = buf + 2 * N, *px = buf + 3 * N, *pz = buf + 4 * N;
    for (int i = 0; i < N; ++i) {
        double ph = s->k[i] * (s->cth[i] * dxp + s->sth[i] * dyp) - s->omega[i] * t + s->phase0[i];
        cphi[i] = cos(ph); sphi[i] = sin(ph);
        ramp[i] = framp(s, i, t);
        px[i] = profX(s, i, zz); pz[i] = profZ(s, i, zz);
    }
    for (int i = 0; i < N; ++i) {
        if (s->omega[i] > s->dw_cutoff) continue;
        double ki = s->k[i], oi = s->omega[i], cti = s->cth[i], sti = s->sth[i];
        double Rni = s->R[i], Rsni = s->Rs[i], agi = s->agw[i];
        double Dnn = (6.0 * Rsni * Rsni * (ki * ki - Rni * Rni)) /
                     (2.0 * Rsni * Rsni - ki * tanh(2.0 * ki * s->depth));
        double AAd = 0.25 * agi * agi * (Dnn / (2.0 * oi));
        double c2 = cphi[i] * cphi[i] - sphi[i] * sphi[i];
        double s2 = 2.0 * sphi[i] * cphi[i];
        double chd = cosh(2.0 * ki * zpd) / s->cosh2kd[i];
        double shd = sinh(2.0 * ki * zpd) / s->cosh2kd[i];
        double u = 0, v = 0, w = 0, p = 0;
        u += AAd * (2.0 * ki * cti) * c2 * chd;
        v += AAd * (2.0 * ki * sti) * c2 * chd;
        w += AAd * (2.0 * ki) * s2 * shd;
        p += AAd * (2.0 * oi) * c2 * chd;
        p -= (gg * (2.0 * ki * cti + 2.0 * ki * sti) * 2.0 * px[i]) / (2.0 * oi);
        p += (gg * (2.0 * ki) * 2.0 * pz[i]) / (2.0 * oi);
        double ri = ramp[i];
        us += u * ri; vs += v * ri; ws += w * ri; ps += p * ri;
    }
    for (long q = 0; q < s->np; q++) {
        int i = s->pi[q], m = s->pm[q];
        double ki = s->k[i], km = s->k[m], oi = s->omega[i], om = s->omega[m];
        double cti = s->cth[i], sti = s->sth[i], ctm = s->cth[m], stm = s->sth[m];
        double ri = ramp[i];
        double AA = 0.5 * s->agw[i] * s->agw[m];
        if (s->hp[q]) {
            double BB = s->Dp[q] / (oi + om);
            double cp = cphi[i] * cphi[m] - sphi[i] * sphi[m];
            double sp = sphi[i] * cphi[m] + cphi[i] * sphi[m];
            double den = cosh(s->kp[q] * s->depth);
            double ch = cosh(s->kp[q] * zpd) / den, sh = sinh(s->kp[q] * zpd) / den;
            us += AA * BB * (ki * cti + km * ctm) * cp * ch * ri;
            vs += AA * BB * (ki * sti + km * stm) * cp * ch * ri;
            ws += AA * BB * s->kp[q] * sp * sh * ri;
            ps += AA * BB * (oi + om) * cp * ch * ri;
            ps -= (gg * (ki * cti * km * ctm + ki * sti * km * stm) * px[i] * px[m]) / (oi * om) * ri;
            ps += (gg * (ki * km) * pz[i] * pz[m]) / (oi * om) * ri;
        }
        if (s->hm[q]) {
            double CC = s->Dm[q] / (oi - om);
            double cm = cphi[i] * cphi[m] + sphi[i] * sphi[m];
            double sm = sphi[i] * cphi[m] - cphi[i] * sphi[m];
            double den = cosh(s->km[q] * s->depth);
            double ch = cosh(s->km[q] * zpd) / den, sh = sinh(s->km[q] * zpd) / den;
            us += AA * CC * (ki * cti - km * ctm) * cm * ch * ri;
            vs += AA * CC * (ki * sti - km * stm) * cm * ch * ri;
            ws += AA * CC * s->km[q] * sm * sh * ri;
            ps += AA * CC * (oi - om) * cm * ch * ri;
        }
    }
    free(buf);
    out[0] = us; out[1] = vs; out[2] = ws; out[3] = ps;
}

/* --- Smit et al. (2017) s-coordinate second order, vertical_theory smit
 *     (u_smit, v_smit, w_smit, dp_smit, Irregular.cpp:1622-2027) --- */

/* Wheeler-stretched profiles, Irregular.cpp:121-138: the height is mapped to
 * sf = h (h + z) / (h + eta) in [0, h]. */
static double prof_s(double k, double depth, double z, double eta, int sinh_) {
    double sf = depth * (depth + z) / (depth + eta);
    return (sinh_ ? sinh(k * sf) : cosh(k * sf)) / cosh(k * depth);
}

/* H coefficient of the pair cache (Irregular.cpp:924-930, 951-958): the
 * inversion of Smit's Eq. 10 with the Sharma-Dean alpha. */
static double smit_h(double g, double om12, double oi, double om, double alpha, double k1dk2, double sgn) {
    return -g / om12 * (alpha / 2.0 - (oi * oi + om * om + sgn * oi * om) / (2.0 * g) + g * k1dk2 / (2.0 * oi * om));
}

/* out = u, v, w, dp; 0 above the surface (eta1 + eta2 + swl). */
void orc_smit(const orc_sea *s, double t, double xx, double yy, double zz, double out[4]) {
    const int N = s->n;
    const double h = s->depth, g = s->g, rho = s->rho;
    double eta = orc_eta1(s, t, xx, yy);
    if (s->order >= 1) eta += orc_eta2(s, t, xx, yy);
    out[0] = out[1] = out[2] = out[3] = 0.0;
    if (zz > eta + s->swl) return;
    zz = dmax(-h, zz - s->swl);
    double *buf = (double *)malloc(sizeof(double) * 4 * (size_t)(N > 0 ? N : 1));
    double *ph = buf, *fr = buf + N, *Ch = buf + 2 * N, *Sh = buf + 3 * N;
    for (int i = 0; i < N; i++) {
        ph[i] = s->k[i] * (s->cth[i] * (xx - s->fx) + s->sth[i] * (yy - s->fy)) - s->omega[i] * t + s->phase0[i];
        fr[i] = framp(s, i, t);
        Ch[i] = prof_s(s->k[i], h, zz, eta, 0);
        Sh[i] = prof_s(s->k[i], h, zz, eta, 1);
    }
    double u1 = 0, v1 = 0, w1 = 0, p1 = 0;
    for (int i = 0; i < N; i++) {
        double agk = s->A[i] * g * s->k[i] / s->omega[i];
        u1 += agk * Ch[i] * s->cth[i] * cos(ph[i]) * fr[i];
        v1 += agk * Ch[i] * s->sth[i] * cos(ph[i]) * fr[i];
        w1 += agk * Sh[i] * sin(ph[i]) * fr[i];
        p1 += s->A[i] * rho * g * Ch[i] * cos(ph[i]) * fr[i];
    }
    double u2 = 0, v2 = 0, w2 = 0, p2 = 0;
    if (s->order >= 1) {
        const double sp1 = (h + zz) / (h + eta), g1s = g * sp1;
        double dphi2ds = 0.0;
        for (int i = 0; i < N; i++) {          /* diagonal terms, no filter */
            double ki = s->k[i], oi = s->omega[i];
            double AA = s->A[i] * s->A[i] * fr[i] * fr[i];
            double k2 = 2.0 * ki, om2 = 2.0 * oi;
            double Rn = s->R[i], Rs = s->Rs[i];
            double Dnn = (6.0 * Rs * Rs * (ki * ki - Rn * Rn)) / (2.0 * Rs * Rs - ki * tanh(2.0 * ki * h));
            double ann = (Dnn - (ki * ki - Rn * Rn)) / Rn + 2.0 * Rn;
            double H = -g / om2 * (ann / 2.0 - (3.0 * oi * oi) / (2.0 * g) + g * ki * ki / (2.0 * oi * oi));
            double Ch2 = prof_s(k2, h, zz, eta, 0), Sh2 = prof_s(k2, h, zz, eta, 1);
            double c2 = cos(2.0 * ph[i]), s2 = sin(2.0 * ph[i]);
            double kx2 = 2.0 * ki * s->cth[i], ky2 = 2.0 * ki * s->sth[i];
            u2 += 0.5 * AA * H * kx2 * (-c2) * Ch2;
            u2 += 0.5 * AA * kx2 * g1s * (ki * Sh[i] / oi) * c2;
            dphi2ds += -0.5 * AA * H * (k2 * h * Sh2) * s2;
            dphi2ds += 0.5 * AA * g * (ki * Sh[i] / oi + sp1 * ki * (ki * h * Ch[i]) / oi) * s2;
            v2 += 0.5 * AA * H * ky2 * (-c2) * Ch2;
            w2 += 0.5 * AA * H * k2 * (-s2) * Sh2;
            p2 += 0.5 * AA * rho * om2 * H * (-c2) * Ch2;
            p2 -= 0.5 * AA * rho * g * g * ki * ki * (Ch[i] * Ch[i] - Sh[i] * Sh[i]) / (oi * oi) * c2;
        }
        for (long q = 0; q < s->np; q++) {     /* pair cache */
            int i = s->pi[q], m = s->pm[q];
            double ki = s->k[i], km = s->k[m], oi = s->omega[i], om = s->omega[m];
            double AA = s->A[i] * s->A[m] * fr[i] * fr[m];
            double gam = s->cth[i] * s->cth[m] + s->sth[i] * s->sth[m];
            double k1dk2 = ki * km * gam;
            double ai = ki * Sh[i] / oi, am_ = km * Sh[m] / om;
            double bi = ki * (ki * h * Ch[i]) / oi, bm = km * (km * h * Ch[m]) / om;
            if (s->hp[q]) {
                double H = smit_h(g, oi + om, oi, om, s->ap[q], k1dk2, 1.0);
                double pp = ph[i] + ph[m], c = cos(pp), sn = sin(pp);
                double kx12 = ki * s->cth[i] + km * s->cth[m], ky12 = ki * s->sth[i] + km * s->sth[m];
                double Ch12 = prof_s(s->kp[q], h, zz, eta, 0), Sh12 = prof_s(s->kp[q], h, zz, eta, 1);
                u2 += AA * H * kx12 * (-c) * Ch12;
                u2 += AA * kx12 * g1s * (ai + am_) * c;
                dphi2ds += -AA * H * (s->kp[q] * h * Sh12) * sn;
                dphi2ds += AA * g * ((ai + am_) + sp1 * (bi + bm)) * sn;
                v2 += AA * H * ky12 * (-c) * Ch12;
                w2 += AA * H * s->kp[q] * (-sn) * Sh12;
                p2 += AA * rho * (oi + om) * H * (-c) * Ch12;
                p2 -= AA * rho * g * g * k1dk2 * (Ch[i] * Ch[m] - Sh[i] * Sh[m]) / (oi * om) * c;
            }
            if (s->hm[q]) {
                double om12 = oi - om;
                double H = fabs(om12) > ORC_SMALL ? smit_h(g, om12, oi, om, s->am[q], k1dk2, -1.0) : 0.0;
                double pm_ = ph[i] - ph[m], c = cos(pm_), sn = sin(pm_);
                double kx12 = ki * s->cth[i] - km * s->cth[m], ky12 = ki * s->sth[i] - km * s->sth[m];
                double Ch12 = prof_s(s->km[q], h, zz, eta, 0), Sh12 = prof_s(s->km[q], h, zz, eta, 1);
                u2 += AA * H * kx12 * (-c) * Ch12;
                u2 += AA * kx12 * g1s * (ai - am_) * c;
                dphi2ds += -AA * H * (s->km[q] * h * Sh12) * sn;
                dphi2ds += AA * g * ((ai - am_) + sp1 * (bi - bm)) * sn;
                v2 += AA * H * ky12 * (-c) * Ch12;
                w2 += AA * H * s->km[q] * (-sn) * Sh12;
                p2 += AA * rho * om12 * H * (-c) * Ch12;
                p2 -= AA * rho * g * g * k1dk2 * (Ch[i] * Ch[m] + Sh[i] * Sh[m]) / (oi * om) * c;
            }
        }
        /* Lagrangian-to-Eulerian chain term of u (Irregular.cpp:1750-1768) */
        double eta_x = 0.0, phi_s = 0.0;
        for (int n = 0; n < N; n++) {
            double sn = sin(ph[n]);
            eta_x += -s->A[n] * s->k[n] * s->cth[n] * sn * fr[n];
            phi_s += (g * s->A[n] / s->omega[n]) * s->k[n] * h * Sh[n] * sn * fr[n];
        }
        phi_s += dphi2ds;
        u2 += -(h + zz) / ((h + eta) * (h + eta)) * eta_x * phi_s;
    }
    free(buf);
    out[0] = u1 + u2; out[1] = v1 + v2; out[2] = w1 + w2; out[3] = p1 + p2;
}

void orc_smit_batch(const orc_sea *s, long n, const double *x, const double *y, const double *z,
                    const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) orc_smit(s, t[p], x[p], y[p], z[p], out + 4 * p);
    (void)nthreads;
}

/* --- dispatch on order with the Taylor layer (Irregular.cpp:9-157) --- */
double orc_eta(const orc_sea *s, double t, double x, double y) {
    if (s->order == 2) return s->swl + orc_eta1(s, t, x, y) + orc_eta2(s, t, x, y);
    return s->swl + orc_eta1(s, t, x, y);
}

static double vel_common(const orc_sea *s, int comp, double t, double x, double y, double z) {
    double o[4];
    if (s->order == 2) {
        double z0 = dmin(0., z - s->swl), za = dmax(0., z - s->swl);
        point_second_order(s, t, x, y, z0, 1 << comp, o);
        if (comp == 0) return u1(s, t, x, y, z0) + o[0] + phi1_dxdz(s, t, x, y) * za;
        if (comp == 1) return v1(s, t, x, y, z0) + o[1] + phi1_dydz(s, t, x, y) * za;
        if (comp == 2) return w1(s, t, x, y, z0) + o[2] + phi1_dzdz(s, t, x, y) * za;
        return dp1(s, t, x, y, z0) + o[3] + dp1_dz(s, t, x, y) * za;
    }
    if (s->order == 1) {
        double zc = dmin(0., z - s->swl);
        point_second_order(s, t, x, y, zc, 1 << comp, o);
        if (comp == 0) return u1(s, t, x, y, zc) + o[0];
        if (comp == 1) return v1(s, t, x, y, zc) + o[1];
        if (comp == 2) return w1(s, t, x, y, zc) + o[2];
        return dp1(s, t, x, y, zc) + o[3];
    }
    if (comp == 0) return u1(s, t, x, y, z - s->swl);
    if (comp == 1) return v1(s, t, x, y, z - s->swl);
    if (comp == 2) return w1(s, t, x, y, z - s->swl);
    return dp1(s, t, x, y, z - s->swl);
}
double orc_u(const orc_sea *s, double t, double x, double y, double z) { return vel_common(s, 0, t, x, y, z); }
double orc_v(const orc_sea *s, double t, double x, double y, double z) { return vel_common(s, 1, t, x, y, z); }
double orc_w(const orc_sea *s, double t, double x, double y, double z) { return vel_common(s, 2, t, x, y, z); }
double orc_dp(const orc_sea *s, double t, double x, double y, double z) { return vel_common(s, 3, t, x, y, z); }

void orc_irregular_batch(const orc_sea *s, long n, const double *x, const double *y,
                         const double *z, const double *t, int fields, double *out,
                         int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) {
        double *o = out + 5 * p;
        o[0] = (fields & 1) ? orc_eta(s, t[p], x[p], y[p]) : 0.0;
        o[1] = (fields & 2) ? orc_u(s, t[p], x[p], y[p], z[p]) : 0.0;
        o[2] = (fields & 4) ? orc_v(s, t[p], x[p], y[p], z[p]) : 0.0;
        o[3] = (fields & 8) ? orc_w(s, t[p], x[p], y[p], z[p]) : 0.0;
        o[4] = (fields & 16) ? orc_dp(s, t[p], x[p], y[p], z[p]) : 0.0;
    }
    (void)nthreads;
}

void orc_uvw2_batch(const orc_sea *s, long n, const double *x, const double *y,
                    const double *z, const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) orc_uvw2(s, t[p], x[p], y[p], z[p], out + 4 * p);
    (void)nthreads;
}

/* Ramp::ramp and ramp1d, Utils.cpp:26-68 */
static double ramp1d(double x, double xs, double xe, int inv) {
    if (inv) return dmax(dmin(1. - ((x - xs) / (xe - xs)), 1.), 0.);
    return dmax(dmin(((x - xs) / (xe - xs)), 1.), 0.);
}
double orc_ramp(int init, int flags, const double lim[12], double t, double x, double y) {
    if (!init) return 1.0;
    double r[6] = {1, 1, 1, 1, 1, 1};
    double v[6] = {t, t, x, x, y, y};
    for (int i = 0; i < 6; i++)
        if (flags & (1 << i)) r[i] = ramp1d(v[i], lim[2 * i], lim[2 * i + 1], i & 1);
    double m = r[0];
    for (int i = 1; i < 6; i++) if (r[i] < m) m = r[i];
    return m;
}

/* internal hooks used by the grid oracle */
double orc__eta1(const orc_sea *s, double t, double x, double y) { return orc_eta1(s, t, x, y); }
double orc__u1(const orc_sea *s, double t, double x, double y, double z) { return u1(s, t, x, y, z); }
double orc__v1(const orc_sea *s, double t, double x, double y, double z) { return v1(s, t, x, y, z); }
double orc__w1(const orc_sea *s, double t, double x, double y, double z) { return w1(s, t, x, y, z); }
double orc__phi1_dxdz(const orc_sea *s, double t, double x, double y) { return phi1_dxdz(s, t, x, y); }
double orc__phi1_dydz(const orc_sea *s, double t, double x, double y) { return phi1_dydz(s, t, x, y); }
double orc__phi1_dzdz(const orc_sea *s, double t, double x, double y) { return phi1_dzdz(s, t, x, y); }
double orc__swl(const orc_sea *s) { return s->swl; }
double orc__dp1(const orc_sea *s, double t, double x, double y, double z) { return dp1(s, t, x, y, z); }
double orc__dp1_dz(const orc_sea *s, double t, double x, double y) { return dp1_dz(s, t, x, y); }
double orc__rho(const orc_sea *s) { return s->rho; }
