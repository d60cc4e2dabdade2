// Regular waves: Stokes 5th order and the Fenton stream function.
//
// Reference (oystelan/CFDwavemaker v3.1.0):
//   Stokes5::set_stokes5_properties / calculate_stokes_coefficients  Stokes5.cpp:10-61
//   Stokes5::eta/u/v/w/dp                                           Stokes5.cpp:64-181
//   FentonStream::set_stream_properties (+ init, eqns, gauss_solve)  FentonStream.cpp:11-239
//   FentonStream::eta/velocity_sums/u/v/w/dp                        FentonStream.cpp:243-314
//
// GB300 design: the coefficient setup runs in FP64 on the device (a single
// thread for Stokes, one CTA for the Fenton Newton iteration: the finite-
// difference Jacobian columns are evaluated by one thread each and the dense
// pivoted elimination runs in shared memory).  Every loop has a fixed cap
// (the reference's own iteration limits); the solver writes a status word.
// Evaluation is FP32 with the phase formed in FP64: the harmonics are
// generated by complex recurrence from one sincos, the depth ratios
// cosh(j k y)/cosh(j k d) from two exponentials raised to the j-th power.
#include "cfdwm.h"
#include "ffmath.cuh"
#include "ramp.cuh"

#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <vector>

namespace cfdwm {

#define CK(x)                                                  \
    do {                                                       \
        cudaError_t e_ = (x);                                  \
        if (e_ != cudaSuccess) {                               \
            std::fprintf(stderr, "cfdwm: CUDA error %s at %s:%d\n", \
                         cudaGetErrorString(e_), __FILE__, __LINE__); \
            return E_CUDA;                                     \
        }                                                      \
    } while (0)

constexpr int MAXN = 64;                 // largest Fourier order accepted
constexpr int MAXNUM = 2 * MAXN + 10;    // unknowns of the Newton system

// Solution block layout (FP64, device):
//   [0] k  [1] c  [2] ubar  [3] R  [4] L  [5] T  [6] status  [7] N
//   [8]  phase constants: cos(theta), sin(theta)
//   [16 .. 16+MAXN)        harmonic coefficient of the horizontal velocity sum
//   [16+MAXN .. +2MAXN)    harmonic coefficient of the vertical velocity sum
//   [16+2MAXN .. +3MAXN)   elevation harmonic coefficient (of cos(j kx))
//   [16+3MAXN .. +4MAXN)   1/(1+exp(-2 j k d))
//   [16+4MAXN]             elevation offset, [+1] u offset (c - ubar or c - u_mean),
//                          [+2] R' = R - g (d - z0), [+3] u_mean (Stokes)
//   [OFF_B .. OFF_B+MAXN)  the dimensionless Fourier coefficients B_j (Fenton)
constexpr int OFF_U = 16, OFF_W = 16 + MAXN, OFF_E = 16 + 2 * MAXN, OFF_Q = 16 + 3 * MAXN,
              OFF_S = 16 + 4 * MAXN, OFF_B = 16 + 4 * MAXN + 8;
constexpr int SOL = OFF_B + MAXN;

struct RegIn {
    double H, L, T, d, cur, g, rho, x0, y0, z0, t0, theta_deg;
    int specify_length, N, nstep;
};

// ----------------------------- Stokes 5th ----------------------------------
__global__ void k_stokes_setup(RegIn in, double *sol) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double PI = 3.14159265358979323846;
    double k = 2. * PI / in.L, kd = k * in.d, eps = k * in.H / 2., S = 1. / cosh(2. * kd);
    double sh = sinh(kd), ct = cosh(kd) / sinh(kd), th = tanh(kd), g = in.g;
    double A11 = 1 / sh;
    double A22 = 3 * pow(S, 2) / (2 * pow(1 - S, 2));
    double A31 = (-4 - 20 * S + 10 * pow(S, 2) - 13 * pow(S, 3)) / (8 * sh * pow(1 - S, 3));
    double A33 = (-2 * pow(S, 2) + 11 * pow(S, 3)) / (8 * sh * pow(1 - S, 3));
    double A42 = (12 * S - 14 * pow(S, 2) - 264 * pow(S, 3) - 45 * pow(S, 4) - 13 * pow(S, 5)) / (24 * pow(1 - S, 5));
    double A44 = (10 * pow(S, 3) - 174 * pow(S, 4) + 291 * pow(S, 5) + 278 * pow(S, 6)) / (48 * (3 + 2 * S) * pow(1 - S, 5));
    double A51 = (-1184 + 32 * S + 13232 * pow(S, 2) + 21712 * pow(S, 3) + 20940 * pow(S, 4) + 12554 * pow(S, 5) -
                  500 * pow(S, 6) - 3341 * pow(S, 7) - 670 * pow(S, 8)) /
                 (64 * sh * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    double A53 = (4 * S + 105 * pow(S, 2) + 198 * pow(S, 3) - 1376 * pow(S, 4) - 1302 * pow(S, 5) - 117 * pow(S, 6) +
                  58 * pow(S, 7)) / (32 * sh * (3 + 2 * S) * pow(1 - S, 6));
    double A55 = (-6 * pow(S, 3) + 272 * pow(S, 4) - 1552 * pow(S, 5) + 852 * pow(S, 6) + 2029 * pow(S, 7) +
                  430 * pow(S, 8)) / (64 * sh * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    double B22 = ct * (1 + 2 * S) / (2 * (1 - S));
    double B31 = -3 * (1 + 3 * S + 3 * pow(S, 2) + 2 * pow(S, 3)) / (8 * pow(1 - S, 3));
    double B42 = ct * (6 - 26 * S - 182 * pow(S, 2) - 204 * pow(S, 3) - 25 * pow(S, 4) + 26 * pow(S, 5)) /
                 (6 * (3 + 2 * S) * pow(1 - S, 4));
    double B44 = ct * (24 + 92 * S + 122 * pow(S, 2) + 66 * pow(S, 3) + 67 * pow(S, 4) + 34 * pow(S, 5)) /
                 (24 * (3 + 2 * S) * pow(1 - S, 4));
    double B53 = 9 * (132 + 17 * S - 2216 * pow(S, 2) - 5897 * pow(S, 3) - 6292 * pow(S, 4) - 2687 * pow(S, 5) +
                      194 * pow(S, 6) + 467 * pow(S, 7) + 82 * pow(S, 8)) /
                 (128 * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    double B55 = 5 * (300 + 1579 * S + 3176 * pow(S, 2) + 2949 * pow(S, 3) + 1188 * pow(S, 4) + 675 * pow(S, 5) +
                      1326 * pow(S, 6) + 827 * pow(S, 7) + 130 * pow(S, 8)) /
                 (384 * (3 + 2 * S) * (4 + S) * pow(1 - S, 6));
    double C0 = pow(th, 0.5);
    double C2 = pow(th, 0.5) * (2 + 7 * pow(S, 2)) / (4 * pow(1 - S, 2));
    double C4 = pow(th, 0.5) * (4 + 32 * S - 116 * pow(S, 2) - 400 * pow(S, 3) - 71 * pow(S, 4) + 146 * pow(S, 5)) /
                (32 * pow(1 - S, 5));
    double D2 = -pow(ct, 0.5) / 2;
    double D4 = pow(ct, 0.5) * (2 + 4 * S + pow(S, 2) + 2 * pow(S, 3)) / (8 * pow(1 - S, 3));
    double E2 = th * (2 + 2 * S + 5 * pow(S, 2)) / (4 * pow(1 - S, 2));
    double E4 = th * (8 + 12 * S - 152 * pow(S, 2) - 308 * pow(S, 3) - 42 * pow(S, 4) + 77 * pow(S, 5)) /
                (32 * pow(1 - S, 5));
    double u_mean = (C0 + pow(eps, 2) * C2 + pow(eps, 4) * C4) / sqrt(k / g);
    double c = u_mean + in.cur;
    double R = (g / k) * (0.5 * pow(C0, 2) + kd + E2 * pow(eps, 2) + E4 * pow(eps, 4));
    (void)D2; (void)D4;
    for (int q = 0; q < SOL; q++) sol[q] = 0.0;
    sol[0] = k; sol[1] = c; sol[2] = u_mean; sol[3] = R; sol[4] = in.L;
    sol[5] = in.T;
    sol[6] = 0; sol[7] = 5;
    sol[8] = cos(in.theta_deg * PI / 180.); sol[9] = sin(in.theta_deg * PI / 180.);
    // velocity harmonics grouped per j (Stokes5.cpp:83-97): the sum over
    // orders of eps^m j k A_jm, times C0 sqrt(g/k^3) cosh(j k d)
    double pre = C0 * sqrt(g / pow(k, 3));
    double Uj[6] = {0, eps * A11 + pow(eps, 3) * A31 + pow(eps, 5) * A51, pow(eps, 2) * A22 + pow(eps, 4) * A42,
                    pow(eps, 3) * A33 + pow(eps, 5) * A53, pow(eps, 4) * A44, pow(eps, 5) * A55};
    double Ej[6] = {0, eps + pow(eps, 3) * B31 - pow(eps, 5) * (B53 + B55), pow(eps, 2) * B22 + pow(eps, 4) * B42,
                    -pow(eps, 3) * B31 + pow(eps, 5) * B53, pow(eps, 4) * B44, pow(eps, 5) * B55};
    for (int j = 1; j <= 5; j++) {
        double cj = cosh(j * kd);
        sol[OFF_U + j - 1] = pre * j * k * Uj[j] * cj;
        sol[OFF_W + j - 1] = pre * j * k * Uj[j] * cj;
        sol[OFF_E + j - 1] = Ej[j] / k;
        sol[OFF_Q + j - 1] = 1.0 / (1.0 + exp(-2.0 * j * kd));
    }
    sol[OFF_S + 0] = kd / k - in.d + in.z0;          // elevation offset
    sol[OFF_S + 1] = c - u_mean;                      // horizontal velocity offset
    sol[OFF_S + 2] = R - g * (in.d - in.z0);          // R - g (d - z0)
    sol[OFF_S + 3] = u_mean;
}

// ----------------------------- Fenton ------------------------------------
struct FenState {
    int N, finite, case_wavelength, current_euler;
    double height, hoverd, value;
};

// eqns (FentonStream.cpp:86-136), z and rhs 1-indexed, length 2N+11
__device__ void fen_eqns(const FenState &f, const double *z, double *rhs, const double *cosa,
                         const double *sina) {
    const double PI = 3.14159265358979323846;
    int n = f.N;
    rhs[1] = f.finite ? (z[2] - z[1] * f.hoverd) : (z[1] + 1.0);
    rhs[2] = f.case_wavelength ? (z[2] - 2.0 * PI * f.height) : (z[2] - f.height * z[3] * z[3]);
    rhs[3] = z[4] * z[3] - 2.0 * PI;
    rhs[4] = z[5] + z[7] - z[4];
    rhs[5] = z[6] + z[7] - z[4];
    if (f.finite) rhs[5] -= z[8] / z[1];
    double coeff[MAXN + 1];
    for (int i = 0; i <= n; i++) coeff[i] = 0.0;
    if (f.finite) for (int i = 1; i <= n; ++i) coeff[i] = z[n + i + 10] / cosh(i * z[1]);
    int it = f.current_euler ? 5 : 6;
    rhs[6] = z[it] - f.value * sqrt(z[2]);
    rhs[7] = z[10] + z[n + 10];
    for (int i = 1; i <= n - 1; ++i) rhs[7] += z[10 + i] + z[10 + i];
    rhs[8] = z[10] - z[n + 10] - z[2];
    for (int m = 0; m <= n; ++m) {
        double psi = 0.0, uu = 0.0, vv = 0.0;
        for (int j = 1; j <= n; ++j) {
            int nm = (m * j) % (2 * n);
            if (f.finite) {
                double e = exp(j * (z[1] + z[10 + m]));
                double s = 0.5 * (e - 1.0 / e), cc = 0.5 * (e + 1.0 / e);
                psi += coeff[j] * s * cosa[nm];
                uu += j * coeff[j] * cc * cosa[nm];
                vv += j * coeff[j] * s * sina[nm];
            } else {
                double e = exp(j * z[10 + m]);
                psi += z[n + j + 10] * e * cosa[nm];
                uu += j * z[n + j + 10] * e * cosa[nm];
                vv += j * z[n + j + 10] * e * sina[nm];
            }
        }
        rhs[9 + m] = psi - z[7] * z[10 + m] - z[8];
        double uw = -z[7] + uu;
        rhs[n + 10 + m] = 0.5 * (uw * uw + vv * vv) + z[10 + m] - z[9];
    }
}

// One CTA of 128 threads.  Status: 0 converged, 2 singular Jacobian,
// 3 not fully converged after the last continuation step (the reference
// only warns in that case and keeps the iterate).
__global__ void __launch_bounds__(128) k_fenton_solve(RegIn in, double *sol, double *work) {
    const double PI = 3.14159265358979323846;
    __shared__ double cosa[2 * MAXN + 1], sina[2 * MAXN + 1];
    __shared__ double z[MAXNUM + 1], s1[MAXNUM + 1], s2[MAXNUM + 1], r1[MAXNUM + 1], b[MAXNUM + 1];
    __shared__ double red[128];
    __shared__ int piv_s, fail_s, conv_s;
    __shared__ FenState f;
    const int tid = threadIdx.x;
    const int N = in.N, num = 2 * N + 10, ld = num + 1;
    double *A = work;                                   // (num+1)^2
    double *zl = work + (size_t)ld * ld + (size_t)tid * 2 * ld;   // per-thread z copy
    double *rl = zl + ld;                                          // per-thread rhs
    if (tid == 0) {
        f.N = N;
        f.finite = (in.d > 0.0 && in.d < 1e8);
        f.case_wavelength = in.specify_length;
        f.current_euler = 1;
        f.value = in.cur / sqrt(in.g * in.H);
        fail_s = 0;
    }
    __syncthreads();
    const double height_full = in.specify_length ? in.H / in.L : in.H / (in.g * in.T * in.T);
    const double hoverd_full = f.finite ? (in.H / in.d) : 0.0;
    const double dhc = height_full / in.nstep, dho = hoverd_full / in.nstep, crit = 1e-3;
    for (int i = tid; i <= num; i += blockDim.x) { z[i] = 0.0; s1[i] = 0.0; s2[i] = 0.0; }
    __syncthreads();
    int status = 0;
    for (int ns = 1; ns <= in.nstep; ++ns) {
        if (tid == 0) {
            f.height = ns * dhc;
            f.hoverd = ns * dho;
            if (ns == 1) {
                // init (FentonStream.cpp:45-81)
                int n = N;
                if (f.finite) {
                    if (!f.case_wavelength) {
                        double a = 4.0 * PI * PI * f.height / f.hoverd;
                        double bb = a / sqrt(tanh(a));
                        double t = tanh(bb);
                        z[1] = bb + (a - bb * t) / (t + bb * (1.0 - t * t));
                    } else {
                        z[1] = 2.0 * PI * f.height / f.hoverd;
                    }
                    z[2] = z[1] * f.hoverd;
                    z[4] = sqrt(tanh(z[1]));
                } else {
                    z[1] = -1.0; z[4] = 1.0;
                    z[2] = f.case_wavelength ? (2.0 * PI * f.height) : (4.0 * PI * PI * f.height);
                }
                z[3] = 2.0 * PI / z[4];
                z[5] = f.value * sqrt(z[2]); z[6] = 0.0;
                z[7] = z[4]; z[8] = 0.0; z[9] = 0.5 * z[7] * z[7];
                cosa[0] = 1.0; sina[0] = 0.0;
                z[10] = 0.5 * z[2];
                for (int i = 1; i <= n; ++i) {
                    cosa[i] = cos(i * PI / n); cosa[i + n] = cos((i + n) * PI / n);
                    sina[i] = sin(i * PI / n); sina[i + n] = sin((i + n) * PI / n);
                    z[n + i + 10] = 0.0;
                    z[i + 10] = 0.5 * z[2] * cosa[i];
                }
                z[n + 11] = 0.5 * z[2] / z[7];
            } else {
                for (int i = 1; i <= num; ++i) z[i] = 2.0 * s2[i] - s1[i];
            }
            conv_s = 0;
        }
        __syncthreads();
        const int maxit = (in.nstep == 1) ? 20 : 9;
        for (int iter = 0; iter < maxit; ++iter) {
            if (tid == 0) fen_eqns(f, z, r1, cosa, sina);
            __syncthreads();
            // finite-difference Jacobian: column i by thread i-1
            for (int i = tid + 1; i <= num; i += blockDim.x) {
                for (int q = 0; q <= num; q++) zl[q] = z[q];
                double hh = (fabs(z[i]) > 1e-4) ? 0.01 * z[i] : 1e-5;
                zl[i] = z[i] + hh;
                fen_eqns(f, zl, rl, cosa, sina);
                for (int j = 1; j <= num; ++j) A[j * ld + i] = (rl[j] - r1[j]) / hh;
            }
            for (int j = tid + 1; j <= num; j += blockDim.x) b[j] = -r1[j];
            __syncthreads();
            // Gaussian elimination with partial pivoting (FentonStream.cpp:11-39)
            for (int col = 1; col <= num; ++col) {
                if (tid == 0) {
                    int piv = col;
                    double best = fabs(A[col * ld + col]);
                    for (int r = col + 1; r <= num; ++r)
                        if (fabs(A[r * ld + col]) > best) { best = fabs(A[r * ld + col]); piv = r; }
                    piv_s = piv;
                    if (best < 1e-300) fail_s = 1;
                }
                __syncthreads();
                if (fail_s) break;
                int piv = piv_s;
                if (piv != col) {
                    for (int cc = tid; cc <= num; cc += blockDim.x) {
                        double t = A[piv * ld + cc]; A[piv * ld + cc] = A[col * ld + cc]; A[col * ld + cc] = t;
                    }
                    if (tid == 0) { double t = b[piv]; b[piv] = b[col]; b[col] = t; }
                }
                __syncthreads();
                const double dinv = 1.0 / A[col * ld + col];
                for (int r = col + 1 + tid; r <= num; r += blockDim.x) {
                    double fct = A[r * ld + col] * dinv;
                    if (fct != 0.0) {
                        for (int cc = col; cc <= num; ++cc) A[r * ld + cc] -= fct * A[col * ld + cc];
                        b[r] -= fct * b[col];
                    }
                }
                __syncthreads();
            }
            if (fail_s) { status = 2; break; }
            if (tid == 0) {
                for (int r = num; r >= 1; --r) {
                    double sm = b[r];
                    for (int cc = r + 1; cc <= num; ++cc) sm -= A[r * ld + cc] * b[cc];
                    b[r] = sm / A[r * ld + r];
                }
                double sum = 0.0;
                for (int i = 1; i <= num; ++i) { z[i] += b[i]; sum += fabs(b[i]); }
                double criter = (ns == in.nstep) ? 0.01 * crit : crit;
                conv_s = (sum < criter) ? 1 : 0;
            }
            __syncthreads();
            if (conv_s) break;
        }
        if (status == 2) break;
        if (tid == 0) {
            if (!conv_s && ns == in.nstep) status = 3;
            for (int i = 1; i <= num; ++i) { s1[i] = s2[i]; s2[i] = z[i]; }
            red[0] = status;
        }
        __syncthreads();
        status = (int)red[0];
    }
    if (tid != 0) return;
    // a Newton iterate that left the finite numbers (a wave beyond the
    // highest one: the reference warns and serves NaN coefficients) is a
    // failure here, status 4
    if (status != 2)
        for (int i = 1; i <= num; ++i)
            if (!isfinite(z[i])) { status = 4; break; }
    for (int q = 0; q < SOL; q++) sol[q] = 0.0;
    sol[6] = status;
    sol[7] = N;
    if (status == 2 || status == 4) return;
    // dimensional results and the output coefficients (FentonStream.cpp:213-239)
    double g = in.g, d = in.d;
    double k = f.finite ? (z[1] / d) : (z[2] / in.H);
    double c = z[4] * sqrt(g / k), ubar = z[7] * sqrt(g / k);
    double Rc = z[9] * g / k + (f.finite ? g * d : 0.0);
    sol[0] = k; sol[1] = c; sol[2] = ubar; sol[3] = Rc; sol[4] = 2.0 * PI / k;
    sol[5] = z[3] / sqrt(g * k);
    sol[8] = cos(in.theta_deg * PI / 180.0); sol[9] = sin(in.theta_deg * PI / 180.0);
    double sg = sqrt(g / k);
    for (int j = 1; j <= N; ++j) {
        double Bj = z[N + 10 + j];
        sol[OFF_B + j - 1] = Bj;
        sol[OFF_U + j - 1] = sg * j * Bj;            // times cosh(jky)/cosh(jkd) cos(jkx)
        sol[OFF_W + j - 1] = sg * j * Bj;            // times sinh(jky)/cosh(jkd) sin(jkx)
        double sm = 0.5 * (z[10] + z[N + 10] * ((j % 2 == 0) ? 1.0 : -1.0));
        for (int m = 1; m <= N - 1; ++m) sm += z[10 + m] * cosa[(m * j) % (2 * N)];
        double Y = 2.0 * sm / N;
        sol[OFF_E + j - 1] = (j == N ? 0.5 * Y : Y) / k;
        sol[OFF_Q + j - 1] = f.finite ? 1.0 / (1.0 + exp(-2.0 * j * k * d)) : 1.0;
    }
    sol[OFF_S + 0] = in.z0;
    sol[OFF_S + 1] = c - ubar;
    sol[OFF_S + 2] = Rc - g * (d - in.z0);
    sol[OFF_S + 3] = ubar;
}

// ----------------------------- evaluation --------------------------------
struct EvalArgs {
    long n;
    const double *x, *y, *z, *t;
    double *rows;       // [6][n] API rows (wave_SurfElev .. wave_nhPres), or null
    double *kin;        // [n][4] wave_Kinematics records, or null
    RampDev ramp;
    float2 nd;          // -depth as a float pair (the z clamp)
    const float *cf;    // [4][MAXN]: U, W, E, Q harmonic coefficients in FP32
    int N, finite;
    float2 P[6];        // k cos th, k sin th, -k c, -x0, -y0, -t0 as float pairs
    float F[12];        // k, cos th, sin th, k d, d - z0, -z0, eta offset, u offset,
                        // R - g (d - z0), ubar, g, rho
};

// One thread per point.  FP64 runs at a small fraction of the FP32 rate on
// this GPU, and a kernel with an FP64 phase, FP64 outputs and per-block FP64
// to FP32 conversions of the coefficients kept the FP64 pipe 85-88% busy
// (14% of DRAM).  So the coefficients and constants arrive in FP32 (converted
// once on the host), the coordinates are split into float pairs by integer
// operations, the phase is formed in float-float and reduced, the sums are
// FP32, and the outputs are widened to double exactly by integer operations.
// e^x through the SFU's base-2 exponential (relative error a few 1e-7; the
// arguments here are at most 0 and at least -2kh - a few)
__device__ __forceinline__ float reg_exp(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
    return y;
}

__global__ void __launch_bounds__(128) k_regular_eval(EvalArgs a) {
    __shared__ float cU[MAXN], cW[MAXN], cE[MAXN], cQ[MAXN];
    for (int j = threadIdx.x; j < MAXN; j += blockDim.x) {
        cU[j] = a.cf[j];
        cW[j] = a.cf[MAXN + j];
        cE[j] = a.cf[2 * MAXN + j];
        cQ[j] = a.cf[3 * MAXN + j];
    }
    __syncthreads();
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    // kx = k (cos th (X - x0) + sin th (Y - y0) - c (t - t0)) in float-float
    const float2 dx = ff_add(ff_from_double(a.x[p]), a.P[3]);
    const float2 dy = ff_add(ff_from_double(a.y[p]), a.P[4]);
    const float2 dt = ff_add(ff_from_double(a.t[p]), a.P[5]);
    float2 kx = ff_add(ff_mul(a.P[0].x, a.P[0].y, dx.x, dx.y), ff_mul(a.P[1].x, a.P[1].y, dy.x, dy.y));
    kx = ff_add(kx, ff_mul(a.P[2].x, a.P[2].y, dt.x, dt.y));
    float s1, c1;
    ff_sincos_poly(ff_reduce_2pi(kx), s1, c1);
    const int N = a.N;
    // elevation: sum_j E_j cos(j kx)
    float cj = c1, sj = s1, eta = 0.f;
    for (int j = 0; j < N; j++) {
        eta = fmaf(cE[j], cj, eta);
        float cn = cj * c1 - sj * s1, sn = sj * c1 + cj * s1;
        cj = cn; sj = sn;
    }
    const float etao = eta + a.F[6];
    // velocity sums with depth ratios, z clamped at the seabed (max(-d, z))
    float2 zf = ff_from_double(a.z[p]);
    if (zf.x < a.nd.x || (zf.x == a.nd.x && zf.y < a.nd.y)) zf = a.nd;
    float su = 0.f, sw = 0.f;
    if (a.finite) {
        const float kd = a.F[3];
        const float ky = a.F[0] * ((zf.x + a.F[4]) + zf.y);
        const float e1 = reg_exp(ky - kd), e2 = reg_exp(-2.f * ky);
        float p1 = 1.f, p2 = 1.f;
        cj = c1; sj = s1;
        for (int j = 0; j < N; j++) {
            p1 *= e1; p2 *= e2;
            // cosh(j ky)/cosh(j kd) = e^{j(ky-kd)} (1 + e^{-2 j ky}) q_j, q_j = 1/(1+e^{-2 j kd})
            float ch = p1 * (1.f + p2) * cQ[j];
            float shh = p1 * (1.f - p2) * cQ[j];
            su = fmaf(cU[j] * ch, cj, su);
            sw = fmaf(cW[j] * shh, sj, sw);
            float cn = cj * c1 - sj * s1, sn = sj * c1 + cj * s1;
            cj = cn; sj = sn;
        }
    } else {
        const float ky = a.F[0] * ((zf.x + a.F[5]) + zf.y);
        const float e1 = reg_exp(ky);
        float p1 = 1.f;
        cj = c1; sj = s1;
        for (int j = 0; j < N; j++) {
            p1 *= e1;
            su = fmaf(cU[j] * p1, cj, su);
            sw = fmaf(cW[j] * p1, sj, sw);
            float cn = cj * c1 - sj * s1, sn = sj * c1 + cj * s1;
            cj = cn; sj = sn;
        }
    }
    const float U = a.F[7] + su;
    // p_nh = rho (R - g (eta + d - z0) - q'^2 / 2), q'^2 = (U_osc - ubar)^2 + w^2;
    // F[8] = R - g (d - z0), and the elevation includes z0
    const float up = su - a.F[9];
    const float q2 = fmaf(up, up, sw * sw);
    // the API rows: eta, u, v, w, the dynamic pressure (0.0 for regular
    // waves, as in the reference) and p_nh, times the ramp where one is set
    // (FP64 multiplies only then: the FP64 rate is a small fraction of FP32's)
    double v[6] = {d_from_float(etao), d_from_float(a.F[1] * U), d_from_float(a.F[2] * U), d_from_float(sw), 0.0,
                   d_from_float(a.F[11] * (fmaf(-a.F[10], etao, a.F[8]) - 0.5f * q2))};
    if (a.ramp.init) {
        const double rr = d_ramp(a.ramp, a.t[p], a.x[p], a.y[p]);
        for (int q = 0; q < 6; q++) v[q] *= rr;
    }
    if (a.rows)
        for (int q = 0; q < 6; q++) a.rows[q * a.n + p] = v[q];
    if (a.kin)
        for (int q = 0; q < 4; q++) a.kin[4 * p + q] = v[q];
}

// ----------------------------- host side ---------------------------------
int regular_build(const Config &cfg, DevRegular &r, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    regular_free(r);
    RegIn in;
    in.H = cfg.wave_height; in.L = cfg.wave_length; in.T = cfg.wave_period; in.d = cfg.depth;
    in.cur = cfg.current; in.g = cfg.gravity; in.rho = cfg.rho; in.x0 = cfg.x_pos;
    in.y0 = cfg.y_pos; in.z0 = cfg.swl; in.t0 = cfg.tofmax; in.theta_deg = cfg.mtheta;
    in.specify_length = cfg.regular_specify_length ? 1 : 0;
    in.N = (cfg.wave_order > 0) ? cfg.wave_order : 16;
    in.nstep = 5;
    r.theory = cfg.regular_theory;
    CK(cudaMalloc(&r.d_sol, sizeof(double) * SOL));
    if (r.theory == 0) {
        if (in.L <= 0 || in.d <= 0) return E_BAD_ARGUMENT;
        k_stokes_setup<<<1, 32, 0, stream>>>(in, r.d_sol);
        note_launch();
        CK(cudaGetLastError());
        r.N = 5;
    } else {
        if (in.N > MAXN) return E_TOO_LARGE;
        if (in.H <= 0.0 || (in.specify_length && in.L <= 0.0) || (!in.specify_length && in.T <= 0.0))
            return E_BAD_ARGUMENT;
        int num = 2 * in.N + 10, ld = num + 1;
        double *work = nullptr;
        CK(cudaMalloc(&work, sizeof(double) * ((size_t)ld * ld + 128 * 2 * (size_t)ld)));
        CK(cudaMemsetAsync(work, 0, sizeof(double) * (size_t)ld * ld, stream));
        k_fenton_solve<<<1, 128, 0, stream>>>(in, r.d_sol, work);
        note_launch();
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream));
        cudaFree(work);
        r.N = in.N;
    }
    double h[SOL];
    CK(cudaMemcpyAsync(h, r.d_sol, sizeof(double) * SOL, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    r.status = (int)h[6];
    r.k = h[0]; r.c = h[1]; r.wave_length = h[4]; r.wave_period = h[5];
    for (int q = 0; q < 10; q++) r.head[q] = h[q];
    for (int q = 0; q < 4; q++) r.soff[q] = h[OFF_S + q];
    // the harmonic coefficients in FP32 for the evaluation kernel
    float cf[4 * MAXN];
    for (int j = 0; j < MAXN; j++) {
        cf[j] = (float)h[OFF_U + j];
        cf[MAXN + j] = (float)h[OFF_W + j];
        cf[2 * MAXN + j] = (float)h[OFF_E + j];
        cf[3 * MAXN + j] = (float)h[OFF_Q + j];
    }
    CK(cudaMalloc(&r.d_cf, sizeof cf));
    CK(cudaMemcpyAsync(r.d_cf, cf, sizeof cf, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    if (r.status == 2 || r.status == 4) return E_SOLVER;
    return OK;
}

void regular_free(DevRegular &r) {
    if (r.d_sol) cudaFree(r.d_sol);
    if (r.d_cf) cudaFree(r.d_cf);
    r.d_sol = nullptr;
    r.d_cf = nullptr;
}

int regular_eval(const DevRegular &r, const Config &cfg, long n, const double *x, const double *y,
                 const double *z, const double *t, const RampDev &ramp, double *rows, double *kin,
                 void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (n <= 0) return OK;
    if (!r.d_cf) return E_NOT_INITIALIZED;
    EvalArgs a;
    a.n = n; a.x = x; a.y = y; a.z = z; a.t = t; a.rows = rows; a.kin = kin; a.cf = r.d_cf;
    a.ramp = ramp;
    ff_split(-cfg.depth, a.nd.x, a.nd.y);
    a.N = r.N;
    a.finite = (cfg.depth > 0.0 && cfg.depth < 1e8) ? 1 : 0;
    const double k = r.head[0], c = r.head[1], cth = r.head[8], sth = r.head[9];
    const double pv[6] = {k * cth, k * sth, -k * c, -cfg.x_pos, -cfg.y_pos, -cfg.tofmax};
    for (int q = 0; q < 6; q++) ff_split(pv[q], a.P[q].x, a.P[q].y);
    const double fv[12] = {k, cth, sth, k * cfg.depth, cfg.depth - cfg.swl, -cfg.swl,
                           r.soff[0], r.soff[1], r.soff[2], r.soff[3], cfg.gravity, cfg.rho};
    for (int q = 0; q < 12; q++) a.F[q] = (float)fv[q];
    prof_begin(PK_REGULAR, stream);
    k_regular_eval<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(a);
    note_launch();
    prof_end(PK_REGULAR, stream);
    CK(cudaGetLastError());
    return OK;
}

int regular_solution(const DevRegular &r, double *dst, int cap, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    double h[SOL];
    CK(cudaMemcpyAsync(h, r.d_sol, sizeof(double) * SOL, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    int q = 0;
    for (int i = 0; i < 6 && q < cap; i++) dst[q++] = h[i];
    if (r.theory == 1)
        for (int j = 0; j < r.N && q < cap; j++) dst[q++] = h[OFF_B + j];
    return q;
}

}  // namespace cfdwm
