/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY): FP64 restatement of the reference's
 * regular-wave theories, oystelan/CFDwavemaker v3.1.0 src/Stokes5.cpp and
 * src/FentonStream.cpp.  The product never links this file; see oracle.h.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Stokes5.h:4-7 and FentonStream.h:6-8 use the full-precision PI. */
#define ORC_PI 3.14159265358979323846

/* ---------------- dispersion, Stokes5.cpp:187-229 ---------------- */
double orc_wavenumber_from_period(double T, double depth, double gravity) {
    if (T <= 0.0 || depth <= 0.0 || gravity <= 0.0) return -1.0;
    double omega = 2.0 * ORC_PI / T;
    double kd = omega * omega / gravity, ks = omega / sqrt(gravity * depth);
    double kk = 0.5 * (kd + ks);
    for (int it = 0; it < 40; ++it) {
        double th = tanh(kk * depth);
        double f = gravity * kk * th - omega * omega;
        if (fabs(f) < 1e-14) break;
        double df = gravity * (th + kk * depth * (1.0 - th * th));
        if (fabs(df) < 1e-14) break;
        double dk = -f / df;
        kk += dk;
        if (kk < 1e-12) kk = 1e-12;
        if (fabs(dk) < 1e-12 * kk) break;
    }
    return kk;
}
double orc_wavelength_from_period(double T, double depth, double g) {
    double kk = orc_wavenumber_from_period(T, depth, g);
    return (kk > 0.0) ? 2.0 * ORC_PI / kk : 0.0;
}
double orc_period_from_length(double L, double depth, double g) {
    if (L <= 0.0 || depth <= 0.0 || g <= 0.0) return -1.0;
    double kk = 2.0 * ORC_PI / L;
    return 2.0 * ORC_PI / sqrt(g * kk * tanh(kk * depth));
}

/* ---------------- Stokes 5th, Stokes5.cpp:10-181 ---------------- */
struct orc_stokes5 {
    double A11, A22, A31, A33, A42, A44, A51, A53, A55, B22, B31, B42, B44, B53, B55;
    double C0, C2, C4, D2, D4, E2, E4, S, eps, k, kd, kH, c, cs, u_mean, Q, R;
    double wave_length, wave_height, depth, current, gravity, rho, x0, y0, z0, t0, theta;
};

orc_stokes5 *orc_stokes5_create(double wave_length, double wave_height, double depth,
                                double current, double gravity, double rho, double x0,
                                double y0, double z0, double t0, double theta) {
    orc_stokes5 *s = (orc_stokes5 *)calloc(1, sizeof(orc_stokes5));
    s->wave_length = wave_length; s->wave_height = wave_height; s->depth = depth;
    s->current = current; s->gravity = gravity; s->rho = rho;
    s->x0 = x0; s->y0 = y0; s->z0 = z0; s->t0 = t0; s->theta = theta;
    /* set_stokes5_properties, Stokes5.cpp:10-23 */
    double k = 2. * ORC_PI / wave_length, kd = k * depth, S = 1. / cosh(2. * kd);
    s->k = k; s->kd = kd; s->eps = k * wave_height / 2.; s->S = S; s->kH = k * wave_height;
    /* calculate_stokes_coefficients, Stokes5.cpp:26-61 */
    double sh = sinh(kd), ct = cosh(kd) / sinh(kd), th = tanh(kd), g = gravity, eps = s->eps;
    s->A11 = 1 / sh;
    s->A22 = 3 * pow(S, 2) / (2 * pow(1 - S, 2));
    s->A31 = (-4 - 20 * S + 10 * pow(S, 2) - 13 * pow(S, 3)) / (8 * sh * pow(1 - S, 3));
    s->A33 = (-2 * pow(S, 2) + 11 * pow(S, 3)) / (8 * sh * pow(1 - S, 3));
    s->A42 = (12 * S - 14 * pow(S, 2) - 264 * pow(S, 3) - 45 * pow(S, 4) - 13 * pow(S, 5)) / (24 * pow(1 - S, 5));
    s->A44 = (10 * pow(S, 3) - 174 * pow(S, 4) + 291 * pow(S, 5) + 278 * pow(S, 6)) / (48 * (3 + 2 * S) * pow(1 - S, 5));
    s->A51 = (-1184 + 32 * S + 13232 * pow(S, 2) + 21712 * pow(S, 3) + 20940 * pow(S, 4) + 12554 * pow(S, 5) -
              500 * pow(S, 6) - 3341 * pow(S, 7) - 670 * pow(S, 8)) /
             (64 * sh * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    s->A53 = (4 * S + 105 * pow(S, 2) + 198 * pow(S, 3) - 1376 * pow(S, 4) - 1302 * pow(S, 5) - 117 * pow(S, 6) +
              58 * pow(S, 7)) / (32 * sh * (3 + 2 * S) * (pow(1 - S, 6)));
    s->A55 = (-6 * pow(S, 3) + 272 * pow(S, 4) - 1552 * pow(S, 5) + 852 * pow(S, 6) + 2029 * pow(S, 7) +
              430 * pow(S, 8)) / (64 * sh * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    s->B22 = ct * (1 + 2 * S) / (2 * (1 - S));
    s->B31 = -3 * (1 + 3 * S + 3 * pow(S, 2) + 2 * pow(S, 3)) / (8 * pow(1 - S, 3));
    s->B42 = ct * (6 - 26 * S - 182 * pow(S, 2) - 204 * pow(S, 3) - 25 * pow(S, 4) + 26 * pow(S, 5)) /
             (6 * (3 + 2 * S) * pow(1 - S, 4));
    s->B44 = ct * (24 + 92 * S + 122 * pow(S, 2) + 66 * pow(S, 3) + 67 * pow(S, 4) + 34 * pow(S, 5)) /
             (24 * (3 + 2 * S) * pow(1 - S, 4));
    s->B53 = 9 * (132 + 17 * S - 2216 * pow(S, 2) - 5897 * pow(S, 3) - 6292 * pow(S, 4) - 2687 * pow(S, 5) +
                  194 * pow(S, 6) + 467 * pow(S, 7) + 82 * pow(S, 8)) /
             (128 * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    s->B55 = 5 * (300 + 1579 * S + 3176 * pow(S, 2) + 2949 * pow(S, 3) + 1188 * pow(S, 4) + 675 * pow(S, 5) +
                  1326 * pow(S, 6) + 827 * pow(S, 7) + 130 * pow(S, 8)) /
             (384 * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    s->C0 = pow(th, 0.5);
    s->C2 = pow(th, 0.5) * (2 + 7 * pow(S, 2)) / (4 * pow(1 - S, 2));
    s->C4 = pow(th, 0.5) * (4 + 32 * S - 116 * pow(S, 2) - 400 * pow(S, 3) - 71 * pow(S, 4) + 146 * pow(S, 5)) /
            (32 * pow(1 - S, 5));
    s->D2 = -pow(ct, 0.5) / 2;
    s->D4 = pow(ct, 0.5) * (2 + 4 * S + pow(S, 2) + 2 * pow(S, 3)) / (8 * pow(1 - S, 3));
    s->E2 = th * (2 + 2 * S + 5 * pow(S, 2)) / (4 * pow(1 - S, 2));
    s->E4 = th * (8 + 12 * S - 152 * pow(S, 2) - 308 * pow(S, 3) - 42 * pow(S, 4) + 77 * pow(S, 5)) /
            (32 * pow(1 - S, 5));
    s->u_mean = (s->C0 + pow(eps, 2) * s->C2 + pow(eps, 4) * s->C4) / sqrt(k / g);
    s->c = s->u_mean + current;
    s->Q = s->u_mean * depth + (s->D2 * pow(eps, 2) + s->D4 * pow(eps, 4)) / sqrt(pow(k, 3) / g);
    s->cs = s->c - s->Q / depth;
    s->R = (g / k) * (0.5 * pow(s->C0, 2) + kd + s->E2 * pow(eps, 2) + s->E4 * pow(eps, 4));
    return s;
}
void orc_stokes5_free(orc_stokes5 *s) { free(s); }

void orc_stokes5_coeffs(const orc_stokes5 *s, double *d) {
    double v[32] = {s->A11, s->A22, s->A31, s->A33, s->A42, s->A44, s->A51, s->A53, s->A55,
                    s->B22, s->B31, s->B42, s->B44, s->B53, s->B55, s->C0, s->C2, s->C4,
                    s->D2, s->D4, s->E2, s->E4, s->S, s->eps, s->k, s->kd, s->kH, s->c,
                    s->cs, s->u_mean, s->Q, s->R};
    memcpy(d, v, sizeof(v));
}

static double st_eta(const orc_stokes5 *s, double t, double X, double Y) {
    double k = s->k, eps = s->eps;
    double kx = k * (cos(s->theta * ORC_PI / 180.) * (X - s->x0) + sin(s->theta * ORC_PI / 180.) * (Y - s->y0) - s->c * (t - s->t0));
    double keta = s->kd + eps * cos(kx) + pow(eps, 2) * s->B22 * cos(2 * kx) +
                  pow(eps, 3) * s->B31 * (cos(kx) - cos(3 * kx)) +
                  pow(eps, 4) * (s->B42 * cos(2 * kx) + s->B44 * cos(4 * kx)) +
                  pow(eps, 5) * (-(s->B53 + s->B55) * cos(kx) + s->B53 * cos(3 * kx) + s->B55 * cos(5 * kx));
    return keta / k - s->depth + s->z0;
}
/* Fourier sums shared by u/v/w/dp (Stokes5.cpp:83-181). */
static void st_sums(const orc_stokes5 *s, double t, double X, double Y, double Z, double *uo, double *wo) {
    double k = s->k, eps = s->eps;
    double kx = k * (cos(s->theta * ORC_PI / 180.) * (X - s->x0) + sin(s->theta * ORC_PI / 180.) * (Y - s->y0) - s->c * (t - s->t0));
    double ky = k * (Z + s->depth - s->z0);
    double pre = s->C0 * sqrt(s->gravity / pow(k, 3));
    *uo = pre * (pow(eps, 1) * (1 * k * s->A11 * cosh(1 * ky) * cos(1 * kx)) +
                 pow(eps, 2) * (2 * k * s->A22 * cosh(2 * ky) * cos(2 * kx)) +
                 pow(eps, 3) * (1 * k * s->A31 * cosh(1 * ky) * cos(1 * kx) + 3 * k * s->A33 * cosh(3 * ky) * cos(3 * kx)) +
                 pow(eps, 4) * (2 * k * s->A42 * cosh(2 * ky) * cos(2 * kx) + 4 * k * s->A44 * cosh(4 * ky) * cos(4 * kx)) +
                 pow(eps, 5) * (1 * k * s->A51 * cosh(1 * ky) * cos(1 * kx) + 3 * k * s->A53 * cosh(3 * ky) * cos(3 * kx) +
                                5 * k * s->A55 * cosh(5 * ky) * cos(5 * kx)));
    *wo = pre * (pow(eps, 1) * (1 * k * s->A11 * sinh(1 * ky) * sin(1 * kx)) +
                 pow(eps, 2) * (2 * k * s->A22 * sinh(2 * ky) * sin(2 * kx)) +
                 pow(eps, 3) * (1 * k * s->A31 * sinh(1 * ky) * sin(1 * kx) + 3 * k * s->A33 * sinh(3 * ky) * sin(3 * kx)) +
                 pow(eps, 4) * (2 * k * s->A42 * sinh(2 * ky) * sin(2 * kx) + 4 * k * s->A44 * sinh(4 * ky) * sin(4 * kx)) +
                 pow(eps, 5) * (1 * k * s->A51 * sinh(1 * ky) * sin(1 * kx) + 3 * k * s->A53 * sinh(3 * ky) * sin(3 * kx) +
                                5 * k * s->A55 * sinh(5 * ky) * sin(5 * kx)));
}

void orc_stokes5_batch(const orc_stokes5 *s, long n, const double *x, const double *y,
                       const double *z, const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) {
        double uo, wo;
        st_sums(s, t[p], x[p], y[p], z[p], &uo, &wo);
        double eta = st_eta(s, t[p], x[p], y[p]);
        double *o = out + 5 * p;
        o[0] = eta;
        o[1] = cos(s->theta * ORC_PI / 180.) * (s->c - s->u_mean + uo);
        o[2] = sin(s->theta * ORC_PI / 180.) * (s->c - s->u_mean + uo);
        o[3] = wo;
        double up = uo - s->u_mean, q2 = up * up + wo * wo;
        o[4] = s->rho * (s->R - s->gravity * (eta + s->depth - s->z0) - 0.5 * q2);
    }
    (void)nthreads;
}

/* ---------------- Fenton stream function, FentonStream.cpp ---------------- */
struct orc_fenton {
    int N, nstep, finite, case_wavelength, current_euler;
    double height, hoverd, height_full, hoverd_full, value;
    double *B, *Y, *coshjkd, *cosa, *sina;
    double ubar, Rc, wave_length, wave_height, wave_period, current, depth, gravity, rho;
    double x0, y0, z0, t0, theta, k, c;
};

/* gauss_solve, FentonStream.cpp:11-39 (1-indexed, row-major n+1 square) */
static int gauss_solve(double *A, double *b, int n) {
    int ld = n + 1;
    for (int col = 1; col <= n; ++col) {
        int piv = col;
        double best = fabs(A[col * ld + col]);
        for (int r = col + 1; r <= n; ++r)
            if (fabs(A[r * ld + col]) > best) { best = fabs(A[r * ld + col]); piv = r; }
        if (best < 1e-300) return 0;
        if (piv != col) {
            for (int cc = 0; cc <= n; cc++) { double tmp = A[piv * ld + cc]; A[piv * ld + cc] = A[col * ld + cc]; A[col * ld + cc] = tmp; }
            double tb = b[piv]; b[piv] = b[col]; b[col] = tb;
        }
        double dinv = 1.0 / A[col * ld + col];
        for (int r = col + 1; r <= n; ++r) {
            double f = A[r * ld + col] * dinv;
            if (f != 0.0) {
                for (int cc = col; cc <= n; ++cc) A[r * ld + cc] -= f * A[col * ld + cc];
                b[r] -= f * b[col];
            }
        }
    }
    for (int r = n; r >= 1; --r) {
        double sm = b[r];
        for (int cc = r + 1; cc <= n; ++cc) sm -= A[r * ld + cc] * b[cc];
        b[r] = sm / A[r * ld + r];
    }
    return 1;
}

/* init, FentonStream.cpp:45-81 */
static void fen_init(orc_fenton *f, double *z) {
    int n = f->N;
    if (f->finite) {
        if (!f->case_wavelength) {
            double a = 4.0 * ORC_PI * ORC_PI * f->height / f->hoverd;
            double b = a / sqrt(tanh(a));
            double t = tanh(b);
            z[1] = b + (a - b * t) / (t + b * (1.0 - t * t));
        } else {
            z[1] = 2.0 * ORC_PI * f->height / f->hoverd;
        }
        z[2] = z[1] * f->hoverd;
        z[4] = sqrt(tanh(z[1]));
    } else {
        z[1] = -1.0; z[4] = 1.0;
        z[2] = f->case_wavelength ? (2.0 * ORC_PI * f->height) : (4.0 * ORC_PI * ORC_PI * f->height);
    }
    z[3] = 2.0 * ORC_PI / z[4];
    if (f->current_euler) { z[5] = f->value * sqrt(z[2]); z[6] = 0.0; }
    else { z[6] = f->value * sqrt(z[2]); z[5] = 0.0; }
    z[7] = z[4]; z[8] = 0.0; z[9] = 0.5 * z[7] * z[7];
    f->cosa[0] = 1.0; f->sina[0] = 0.0;
    z[10] = 0.5 * z[2];
    for (int i = 1; i <= n; ++i) {
        f->cosa[i] = cos(i * ORC_PI / n); f->cosa[i + n] = cos((i + n) * ORC_PI / n);
        f->sina[i] = sin(i * ORC_PI / n); f->sina[i + n] = sin((i + n) * ORC_PI / n);
        z[n + i + 10] = 0.0;
        z[i + 10] = 0.5 * z[2] * f->cosa[i];
    }
    z[n + 11] = 0.5 * z[2] / z[7];
}

/* eqns, FentonStream.cpp:86-136 */
static void fen_eqns(const orc_fenton *f, const double *z, double *rhs, double *coeff) {
    int n = f->N;
    rhs[1] = f->finite ? (z[2] - z[1] * f->hoverd) : (z[1] + 1.0);
    rhs[2] = f->case_wavelength ? (z[2] - 2.0 * ORC_PI * f->height) : (z[2] - f->height * z[3] * z[3]);
    rhs[3] = z[4] * z[3] - 2.0 * ORC_PI;
    rhs[4] = z[5] + z[7] - z[4];
    rhs[5] = z[6] + z[7] - z[4];
    if (f->finite) rhs[5] -= z[8] / z[1];
    for (int i = 0; i <= n; i++) coeff[i] = 0.0;
    if (f->finite) for (int i = 1; i <= n; ++i) coeff[i] = z[n + i + 10] / cosh(i * z[1]);
    int it = f->current_euler ? 5 : 6;
    rhs[6] = z[it] - f->value * sqrt(z[2]);
    rhs[7] = z[10] + z[n + 10];
    for (int i = 1; i <= n - 1; ++i) rhs[7] += z[10 + i] + z[10 + i];
    rhs[8] = z[10] - z[n + 10] - z[2];
    for (int m = 0; m <= n; ++m) {
        double psi = 0.0, uu = 0.0, vv = 0.0;
        if (f->finite) {
            for (int j = 1; j <= n; ++j) {
                int nm = (m * j) % (2 * n);
                double e = exp(j * (z[1] + z[10 + m]));
                double s = 0.5 * (e - 1.0 / e), cc = 0.5 * (e + 1.0 / e);
                psi += coeff[j] * s * f->cosa[nm];
                uu += j * coeff[j] * cc * f->cosa[nm];
                vv += j * coeff[j] * s * f->sina[nm];
            }
        } else {
            for (int j = 1; j <= n; ++j) {
                int nm = (m * j) % (2 * n);
                double e = exp(j * z[10 + m]);
                psi += z[n + j + 10] * e * f->cosa[nm];
                uu += j * z[n + j + 10] * e * f->cosa[nm];
                vv += j * z[n + j + 10] * e * f->sina[nm];
            }
        }
        rhs[9 + m] = psi - z[7] * z[10 + m] - z[8];
        double uw = -z[7] + uu;
        rhs[n + 10 + m] = 0.5 * (uw * uw + vv * vv) + z[10 + m] - z[9];
    }
}

/* set_stream_properties, FentonStream.cpp:141-239 */
orc_fenton *orc_fenton_create(double wave_height, double wave_length, double wave_period,
                              int specify_length, int current_type, int n_fourier,
                              int n_steps, double depth, double current, double gravity,
                              double rho, double x0, double y0, double z0, double t0,
                              double theta, int *status) {
    *status = 0;
    orc_fenton *f = (orc_fenton *)calloc(1, sizeof(orc_fenton));
    f->depth = depth; f->current = current; f->gravity = gravity; f->rho = rho;
    f->x0 = x0; f->y0 = y0; f->z0 = z0; f->t0 = t0; f->theta = theta;
    f->wave_height = wave_height;
    f->N = (n_fourier > 0) ? n_fourier : 16;
    f->nstep = (n_steps > 0) ? n_steps : 5;
    f->case_wavelength = specify_length;
    f->current_euler = (current_type == 0);
    f->finite = (depth > 0.0 && depth < 1e8);
    if (wave_height <= 0.0) { *status = 1; free(f); return NULL; }
    if (specify_length) {
        if (wave_length <= 0.0) { *status = 1; free(f); return NULL; }
        f->wave_length = wave_length;
        f->height_full = wave_height / wave_length;
    } else {
        if (wave_period <= 0.0) { *status = 1; free(f); return NULL; }
        f->wave_period = wave_period;
        f->height_full = wave_height / (gravity * wave_period * wave_period);
    }
    f->hoverd_full = f->finite ? (wave_height / depth) : 0.0;
    f->value = current / sqrt(gravity * wave_height);
    int N = f->N, num = 2 * N + 10;
    f->cosa = (double *)calloc(2 * N + 1, sizeof(double));
    f->sina = (double *)calloc(2 * N + 1, sizeof(double));
    double *z = calloc(num + 1, sizeof(double)), *s1 = calloc(num + 1, sizeof(double)),
           *s2 = calloc(num + 1, sizeof(double)), *r1 = calloc(num + 1, sizeof(double)),
           *r2 = calloc(num + 1, sizeof(double)), *b = calloc(num + 1, sizeof(double)),
           *coeff = calloc(N + 1, sizeof(double)),
           *A = calloc((size_t)(num + 1) * (num + 1), sizeof(double));
    double dhc = f->height_full / f->nstep, dho = f->hoverd_full / f->nstep, crit = 1e-3;
    int ok = 1;
    for (int ns = 1; ns <= f->nstep && ok; ++ns) {
        f->height = ns * dhc;
        f->hoverd = ns * dho;
        if (ns == 1) fen_init(f, z);
        else for (int i = 1; i <= num; ++i) z[i] = 2.0 * s2[i] - s1[i];
        int maxit = (f->nstep == 1) ? 20 : 9, conv = 0;
        for (int iter = 0; iter < maxit; ++iter) {
            fen_eqns(f, z, r1, coeff);
            memset(A, 0, sizeof(double) * (size_t)(num + 1) * (num + 1));
            for (int i = 1; i <= num; ++i) {
                double hh = (fabs(z[i]) > 1e-4) ? 0.01 * z[i] : 1e-5;
                double zi = z[i];
                z[i] = zi + hh;
                fen_eqns(f, z, r2, coeff);
                z[i] = zi;
                for (int j = 1; j <= num; ++j) A[j * (num + 1) + i] = (r2[j] - r1[j]) / hh;
            }
            for (int j = 1; j <= num; ++j) b[j] = -r1[j];
            if (!gauss_solve(A, b, num)) { ok = 0; *status = 2; break; }
            double sum = 0.0;
            for (int i = 1; i <= num; ++i) { z[i] += b[i]; sum += fabs(b[i]); }
            double criter = (ns == f->nstep) ? 0.01 * crit : crit;
            if (sum < criter) { conv = 1; break; }
        }
        if (ok && !conv && ns == f->nstep) *status = 3;
        for (int i = 1; i <= num; ++i) { s1[i] = s2[i]; s2[i] = z[i]; }
    }
    if (ok) {
        f->k = f->finite ? (z[1] / depth) : (z[2] / wave_height);
        f->c = z[4] * sqrt(gravity / f->k);
        f->ubar = z[7] * sqrt(gravity / f->k);
        f->wave_length = 2.0 * ORC_PI / f->k;
        f->wave_period = z[3] / sqrt(gravity * f->k);
        f->Rc = z[9] * gravity / f->k + (f->finite ? gravity * depth : 0.0);
        f->B = calloc(N + 1, sizeof(double));
        f->Y = calloc(N + 1, sizeof(double));
        f->coshjkd = calloc(N + 1, sizeof(double));
        for (int j = 1; j <= N; ++j) {
            f->B[j] = z[N + 10 + j];
            f->coshjkd[j] = f->finite ? cosh(j * f->k * depth) : 1.0;
        }
        for (int j = 1; j <= N; ++j) {
            double sm = 0.5 * (z[10] + z[N + 10] * ((j % 2 == 0) ? 1.0 : -1.0));
            for (int m = 1; m <= N - 1; ++m) sm += z[10 + m] * f->cosa[(m * j) % (2 * N)];
            f->Y[j] = 2.0 * sm / N;
        }
    }
    free(z); free(s1); free(s2); free(r1); free(r2); free(b); free(coeff); free(A);
    if (!ok) { free(f->cosa); free(f->sina); free(f); return NULL; }
    return f;
}

void orc_fenton_free(orc_fenton *f) {
    if (!f) return;
    free(f->B); free(f->Y); free(f->coshjkd); free(f->cosa); free(f->sina); free(f);
}

int orc_fenton_solution(const orc_fenton *f, double *d) {
    int q = 0;
    d[q++] = f->k; d[q++] = f->c; d[q++] = f->ubar; d[q++] = f->Rc;
    d[q++] = f->wave_length; d[q++] = f->wave_period;
    for (int j = 1; j <= f->N; j++) d[q++] = f->B[j];
    for (int j = 1; j <= f->N; j++) d[q++] = f->Y[j];
    return q;
}

/* eta/velocity_sums/u/v/w/dp, FentonStream.cpp:243-314 */
static double fen_kx(const orc_fenton *f, double t, double X, double Y) {
    double th = f->theta * ORC_PI / 180.0;
    return f->k * (cos(th) * (X - f->x0) + sin(th) * (Y - f->y0) - f->c * (t - f->t0));
}
static double fen_eta(const orc_fenton *f, double t, double X, double Y) {
    double kx = fen_kx(f, t, X, Y);
    double keta = 0.5 * f->Y[f->N] * cos(f->N * kx);
    for (int j = 1; j <= f->N - 1; ++j) keta += f->Y[j] * cos(j * kx);
    return keta / f->k + f->z0;
}
static void fen_sums(const orc_fenton *f, double kx, double Z, double *su, double *sw) {
    *su = 0.0; *sw = 0.0;
    if (f->finite) {
        double ky = f->k * (Z + f->depth - f->z0);
        for (int j = 1; j <= f->N; ++j) {
            double bj = f->B[j] / f->coshjkd[j];
            *su += j * bj * cosh(j * ky) * cos(j * kx);
            *sw += j * bj * sinh(j * ky) * sin(j * kx);
        }
    } else {
        double ky = f->k * (Z - f->z0);
        for (int j = 1; j <= f->N; ++j) {
            double e = f->B[j] * exp(j * ky);
            *su += j * e * cos(j * kx);
            *sw += j * e * sin(j * kx);
        }
    }
}

void orc_fenton_batch(const orc_fenton *f, long n, const double *x, const double *y,
                      const double *z, const double *t, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long p = 0; p < n; p++) {
        double kx = fen_kx(f, t[p], x[p], y[p]), su, sw;
        fen_sums(f, kx, z[p], &su, &sw);
        double sg = sqrt(f->gravity / f->k);
        double U = f->c - f->ubar + sg * su;
        double eta = fen_eta(f, t[p], x[p], y[p]);
        double *o = out + 5 * p;
        o[0] = eta;
        o[1] = cos(f->theta * ORC_PI / 180.0) * U;
        o[2] = sin(f->theta * ORC_PI / 180.0) * U;
        o[3] = sg * sw;
        double uw = -f->ubar + sg * su, wv = sg * sw;
        o[4] = f->rho * (f->Rc - f->gravity * (eta + f->depth - f->z0) - 0.5 * (uw * uw + wv * wv));
    }
    (void)nthreads;
}
