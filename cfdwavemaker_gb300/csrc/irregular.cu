// Irregular second-order (Sharma & Dean) kinematics on the GPU.
//
// What is computed follows the reference (oystelan/CFDwavemaker v3.1.0):
//   first-order sums     Irregular.cpp:178-198, 394-447, 1107-1192
//   eta2 (pair cache)    Irregular.cpp:223-293
//   u2/v2/w2/dp2         Irregular.cpp:450-803   (point API, unfiltered pairs)
//   uvw2 (pair cache)    Irregular.cpp:975-1102  (s-grid)
//   pair cache filters   Irregular.cpp:840-967
//   order dispatch       Irregular.cpp:9-157     (Taylor layer above swl)
//
// How it is computed (GB300 design):
//  * The per-pair transfer functions (D+-, alpha+-) are evaluated ONCE, in FP64
//    on the device, and stored as FP32 coefficients in tiles of the upper
//    triangle of the N x N pair matrix (build kernels below).  Each pair
//    record already folds the amplitudes, 1/(omega_i +- omega_m), the
//    direction factors and the depth normaliser 1/(1+exp(-2 k+- h)).
//  * Phases are formed in FP64 (k.x - omega t + phase0 can reach 1e4 rad) and
//    reduced to [-pi, pi] before an FP32 sincos; the phasors of every
//    (component, point) are written once to a scratch workspace.
//  * The pair sums run on FP32 CUDA cores: each thread owns one point (or one
//    s-grid column with LV levels in registers); the coefficient tile and the
//    phasors of the streamed component tile are staged in shared memory and
//    read as warp-wide broadcasts / conflict-free rows.  The depth factors
//    cosh(k(z+h))/cosh(kh) and sinh(k(z+h))/cosh(kh) use two MUFU ex2 per
//    wavenumber, exp(kz) and exp(-2k(z+h)), both <= 1 below the surface.
//  * Accumulation is compensated: a tile row is summed in FP32, then added to
//    a Kahan (sum, carry) pair per output.
#include "cfdwm.h"
#include "ffmath.cuh"
#include "ramp.cuh"

#include <cuda_runtime.h>
#include <algorithm>
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

constexpr int EATA_NC = 2;    // eta table: A (cc coefficient), B (ss coefficient)
constexpr int GRIDV_NC = 8;   // uvw table: Pu, Mu, Pv, Mv, Pw, Mw, kp, km
// s-grid pressure tables (grid mask, rho folded): Pp, Mp of the phase terms,
// and X, Z of the phase-free terms (products of the first-order profiles for
// a pair, the linear diagonal terms on the diagonal entry)
constexpr int GRIDP_NC = 2;
constexpr int POINTV_NC = 12; // point table: Pu, Mu, Pv, Mv, Pw, Mw, Pp, Mp, kp, km, Xpp, Xzz
constexpr float LOG2E_F = 1.4426950408889634f;
constexpr long SPLIT_TARGET_BLOCKS = 4 * 152;   // blocks a column-pair launch aims for
// batches of at most this many points take the few-point kernels (a block
// per point, the components or pair rows over its threads).  Measured on the
// 128-component point sea, a velocity and an elevation batch: at 256 points
// 133 us against 191 us with the per-thread kernels, at 512 166 against 187,
// at 1024 226 against 196.
constexpr long FEW_POINTS = 512;
// the phasors alone: the few-point kernel up to 1024 points (a velocity and
// an elevation batch of 1024 points 159 us against 193 us; 2048 points 210
// against 205)
constexpr long PH_FEW_POINTS = 1024;

__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// Irregular::freq_ramp, Irregular.cpp:200-204 (FP64, as the reference).
__device__ __forceinline__ double d_freq_ramp(double t, double rt, double ts, double du) {
    double rampdown = fmax(fmin(1. - ((t - ts - du + rt) / (rt + SMALL)), 1.), 0.);
    double rampup = fmax(fmin(((t - ts) / (rt + SMALL)), 1.), 0.);
    return rampup * rampdown;
}

__host__ __device__ inline long tile_index(int I, int M, int nt) {
    return (long)I * nt - (long)I * (I - 1) / 2 + (M - I);
}

// ---------------------------------------------------------------------------
// Setup: FP64 component data and pair tables (on device)
// ---------------------------------------------------------------------------
struct CompIn {
    int n, npad;
    const double *omega, *A, *k, *theta;   // device copies (FP64), length n
    double depth, g, rho, mtheta_rad, cutoff, bandwidth, kmax;
};

// ki^2 + km^2 + 2 ki km gam, each product rounded separately (as the
// reference's FP64 expression without contraction)
__device__ __forceinline__ double pair_k2(double ki, double km, double gam) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ki, ki), __dmul_rn(km, km)), __dmul_rn(__dmul_rn(2.0 * ki, km), gam));
}

// One record per (tile, entry).  mode 0: grid mask (eta + uvw tables, and
// the pressure tables tab_gp / tab_gk), mode 1: point-API mask
// (u2/v2/w2/dp2 table).
__global__ void k_build_tables(CompIn c, int TT, int nt, int mode, float *tab_eta,
                               float *tab_v, float *tab_gp, float *tab_gk) {
    long t = blockIdx.x;
    int I = 0;
    while (tile_index(I, nt - 1, nt) < t) I++;
    int M = (int)(t - tile_index(I, I, nt)) + I;
    for (int e = threadIdx.x; e < TT * TT; e += blockDim.x) {
        int ii = e / TT, mm = e % TT;
        int i = I * TT + ii, m = M * TT + mm;
        double out[12], pr[4] = {0.0, 0.0, 0.0, 0.0};   // pr: Pp, Mp, X, Z (mode 0)
        for (int q = 0; q < 12; q++) out[q] = 0.0;
        double eA = 0.0, eB = 0.0;
        const double h = c.depth, g = c.g, gg = c.g * c.g;
        if (i < c.n && m < c.n && i <= m) {
            double ki = c.k[i], oi = c.omega[i], Ai = c.A[i];
            double thi = c.theta[i] + c.mtheta_rad;
            double cti = cos(thi), sti = sin(thi);
            double Rn = ki * tanh(ki * h), Rsn = sqrt(Rn);
            double agi = Ai * g / oi;
            if (i == m) {
                bool keep = (mode == 1) || (oi <= c.cutoff);
                if (keep) {
                    double Dnn = (6.0 * Rsn * Rsn * (ki * ki - Rn * Rn)) /
                                 (2.0 * Rsn * Rsn - ki * tanh(2.0 * ki * h));
                    double AAd = 0.25 * agi * agi * (Dnn / (2.0 * oi));
                    double q2 = 1.0 / (1.0 + exp(-4.0 * ki * h));
                    out[0] = AAd * (2.0 * ki * cti) * q2;
                    out[2] = AAd * (2.0 * ki * sti) * q2;
                    out[4] = AAd * (2.0 * ki) * q2;
                    if (mode == 1) {
                        out[6] = c.rho * AAd * (2.0 * oi) * q2;
                        out[8] = 2.0 * ki;
                    } else {
                        out[6] = 2.0 * ki;
                        // uvw2 pressure, diagonal (Irregular.cpp:1034-1037): the
                        // 2-phi term and the two terms linear in the profiles
                        pr[0] = c.rho * AAd * (2.0 * oi) * q2;
                        pr[2] = -c.rho * (gg * (2.0 * ki * cti + 2.0 * ki * sti) * 2.0) / (2.0 * oi);
                        pr[3] = c.rho * (gg * (2.0 * ki) * 2.0) / (2.0 * oi);
                        if (2.0 * ki <= c.kmax) {
                            double ann = (Dnn - (ki * ki - Rn * Rn)) / Rn + 2.0 * Rn;
                            double pe = 0.25 * Ai * Ai * ann;
                            eA = pe;
                            eB = -pe;
                        }
                    }
                }
            } else {
                double km = c.k[m], om = c.omega[m], Am = c.A[m];
                double thm = c.theta[m] + c.mtheta_rad;
                double ctm = cos(thm), stm = sin(thm);
                double Rm = km * tanh(km * h), Rsm = sqrt(Rm);
                double agm = Am * g / om;
                bool keep = true, hp = true, hm = (ki != km);
                double gam;
                if (mode == 0) {
                    keep = (oi <= c.cutoff) && (om <= c.cutoff) && (fabs(oi - om) <= c.bandwidth);
                    hp = (ki + km) <= c.kmax;
                    // Irregular.cpp:870, rounded as the reference rounds it (no FMA)
                    gam = __dadd_rn(__dmul_rn(cti, ctm), __dmul_rn(sti, stm));
                } else {
                    gam = cos(thi - thm);               // Irregular.cpp:470
                }
                if (keep && (hp || hm)) {
                    // |k_i +- k_m|; for opposite (equal) directions of equal k the
                    // radicand is 0 up to rounding: clamped so that a -1e-16 does
                    // not turn the whole table into NaN
                    double kp = sqrt(fmax(0.0, pair_k2(ki, km, gam)));
                    double kq = sqrt(fmax(0.0, pair_k2(ki, km, -gam)));
                    double sp = Rsn + Rsm, sm = Rsn - Rsm;
                    double R2p = sp * sp, R2m = sm * sm;
                    double AA = 0.5 * agi * agm;
                    if (hp) {
                        double den = R2p - kp * tanh(kp * h);
                        double Dp = (2.0 * R2p * (ki * km * gam - Rn * Rm)) / den +
                                    (sp * (Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
                        double BB = Dp / (oi + om);
                        double qp = 1.0 / (1.0 + exp(-2.0 * kp * h));
                        out[0] = AA * BB * (ki * cti + km * ctm) * qp;
                        out[2] = AA * BB * (ki * sti + km * stm) * qp;
                        out[4] = AA * BB * kp * qp;
                        if (mode == 1) {
                            out[6] = c.rho * AA * BB * (oi + om) * qp;
                            out[8] = kp;
                        } else {
                            out[6] = kp;
                            // uvw2 pressure, sum term and the phase-free
                            // products of the profiles (Irregular.cpp:1074-1077)
                            pr[0] = c.rho * AA * BB * (oi + om) * qp;
                            pr[2] = -c.rho * (gg * (ki * cti * km * ctm + ki * sti * km * stm)) / (oi * om);
                            pr[3] = c.rho * (gg * (ki * km)) / (oi * om);
                            double ap = (Dp - (ki * km * gam - Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
                            double pe = 0.5 * Ai * Am * ap;
                            eA += pe;
                            eB -= pe;
                        }
                    }
                    if (hm) {
                        double den = R2m - kq * tanh(kq * h);
                        double Dm = (2.0 * R2m * (ki * km * gam + Rn * Rm)) / den +
                                    (sm * (-Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
                        double CC = Dm / (oi - om);
                        double qm = 1.0 / (1.0 + exp(-2.0 * kq * h));
                        out[1] = AA * CC * (ki * cti - km * ctm) * qm;
                        out[3] = AA * CC * (ki * sti - km * stm) * qm;
                        out[5] = AA * CC * kq * qm;
                        if (mode == 1) {
                            out[7] = c.rho * AA * CC * (oi - om) * qm;
                            out[9] = kq;
                        } else {
                            out[7] = kq;
                            pr[1] = c.rho * AA * CC * (oi - om) * qm;   // Irregular.cpp:1093
                            double am = (Dm - (ki * km * gam + Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
                            double pe = 0.5 * Ai * Am * am;
                            eA += pe;
                            eB += pe;
                        }
                    }
                    if (mode == 1) {
                        // the phase-free products of the first-order profiles
                        // in dp2 (Irregular.cpp:786-787)
                        out[10] = -c.rho * (gg * (ki * cti * km * ctm + ki * sti * km * stm)) / (oi * om);
                        out[11] = c.rho * (gg * (ki * km)) / (oi * om);
                    }
                }
            }
        }
        long base = t * (long)TT * TT + e;
        if (mode == 0) {
            tab_eta[base * EATA_NC + 0] = (float)eA;
            tab_eta[base * EATA_NC + 1] = (float)eB;
            for (int q = 0; q < GRIDV_NC; q++) tab_v[base * GRIDV_NC + q] = (float)out[q];
            tab_gp[base * GRIDP_NC + 0] = (float)pr[0];
            tab_gp[base * GRIDP_NC + 1] = (float)pr[1];
            tab_gk[base * GRIDP_NC + 0] = (float)pr[2];
            tab_gk[base * GRIDP_NC + 1] = (float)pr[3];
        } else {
            for (int q = 0; q < POINTV_NC; q++) tab_v[base * POINTV_NC + q] = (float)out[q];
        }
    }
}

// Count of pairs kept by the reference's pair cache (Irregular.cpp:840-967).
__global__ void k_count_pairs(CompIn c, unsigned long long *cnt) {
    long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long tot = (long)c.n * c.n;
    unsigned long long local = 0;
    for (; idx < tot; idx += (long)gridDim.x * blockDim.x) {
        int i = (int)(idx / c.n), m = (int)(idx % c.n);
        if (m <= i) continue;
        double oi = c.omega[i], om = c.omega[m];
        if (oi > c.cutoff || om > c.cutoff || fabs(oi - om) > c.bandwidth) continue;
        bool hp = (c.k[i] + c.k[m]) <= c.kmax, hm = c.k[i] != c.k[m];
        if (hp || hm) local++;
    }
    if (local) atomicAdd(cnt, local);
}

__global__ void k_component_coefs(CompIn c, int npad, double fx, double fy, double tofmax,
                                  const double *phase, const double *rt, const double *st,
                                  const double *du, double *ph_out, float *cf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    double v[NCF];
    for (int q = 0; q < NCF; q++) v[q] = 0.0;
    double kx = 0, ky = 0, om = 0, p0 = 0, r0 = 0, r1 = -SMALL, r2 = HUGE_;
    if (i < c.n) {
        double k = c.k[i], w = c.omega[i], A = c.A[i], h = c.depth, g = c.g, gg = g * g;
        double th = c.theta[i] + c.mtheta_rad, ct = cos(th), st_ = sin(th);
        kx = k * ct; ky = k * st_; om = w; p0 = w * tofmax + phase[i];
        r0 = rt[i]; r1 = st[i]; r2 = du[i];
        v[CF_A] = A;
        v[CF_AU] = A * g * k / w;
        v[CF_CT] = ct;
        v[CF_ST] = st_;
        v[CF_K] = k;
        v[CF_Q] = 1.0 / (1.0 + exp(-2.0 * k * h));
        v[CF_AP] = A * c.rho * g;
        v[CF_GX] = ct * A * w * k;
        v[CF_GY] = st_ * A * w * k;
        v[CF_GZ] = A * w * k * (cosh(k * h) / sinh(k * h));
        v[CF_GP] = A * c.rho * g * k;
        v[CF_X1] = -c.rho * (gg * (2 * k * ct + 2 * k * st_) * 2) / (2 * w);
        v[CF_Z1] = c.rho * (gg * (2 * k) * 2) / (2 * w);
        v[CF_KW] = w > 0.0 ? k / w : 0.0;
    }
    ph_out[0 * npad + i] = kx;
    ph_out[1 * npad + i] = ky;
    ph_out[2 * npad + i] = om;
    ph_out[3 * npad + i] = p0;
    ph_out[4 * npad + i] = r0;
    ph_out[5 * npad + i] = r1;
    ph_out[6 * npad + i] = r2;
    for (int q = 0; q < NCF; q++) cf[q * npad + i] = (float)v[q];
}

constexpr int PH_REC = 13;       // floats of a phasor record
constexpr int PH_CHUNK = 128;    // records per shared-memory chunk

// The phasor records of all components (time-independent, built once with the sea).
__global__ void k_phasor_records(int n, int npad, const double *phase, const float *cf, int cs, float *rec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    float *o = rec + (long)i * PH_REC;
    if (i >= n) {
        for (int q = 0; q < PH_REC; q++) o[q] = 0.f;
        return;
    }
    ff_split(phase[i], o[0], o[1]);
    ff_split(phase[cs + i], o[2], o[3]);
    ff_split(-phase[2 * cs + i], o[4], o[5]);
    ff_split(phase[3 * cs + i], o[6], o[7]);
    o[8] = cf[CF_A * cs + i];
    o[9] = cf[CF_GX * cs + i];
    o[10] = cf[CF_GY * cs + i];
    o[11] = cf[CF_GZ * cs + i];
    o[12] = cf[CF_GP * cs + i];
}

int sea_build(const Config &cfg, DevSea &sea, bool point_table, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    sea_free(sea);
    int n = (int)cfg.omega.size();
    sea.n = n;
    sea.depth = cfg.depth; sea.swl = cfg.swl; sea.g = cfg.gravity; sea.rho = cfg.rho;
    sea.fx = cfg.x_pos; sea.fy = cfg.y_pos; sea.order = cfg.order;
    sea.npad_g = ((n + GRID_TILE - 1) / GRID_TILE) * GRID_TILE;
    sea.npad_p = ((n + POINT_TILE - 1) / POINT_TILE) * POINT_TILE;
    if (sea.npad_g == 0) sea.npad_g = GRID_TILE;
    if (sea.npad_p == 0) sea.npad_p = POINT_TILE;
    sea.ntile_g = sea.npad_g / GRID_TILE;
    sea.ntile_p = sea.npad_p / POINT_TILE;
    sea.trivial_ramp = true;
    for (int i = 1; i < n; i++)
        if (cfg.ramptime[i] != cfg.ramptime[0] || cfg.starttime[i] != cfg.starttime[0] ||
            cfg.duration[i] != cfg.duration[0])
            sea.trivial_ramp = false;
    double kmax = 0.0;   // Irregular.cpp:833-835
    for (int i = 0; i < n; i++) kmax = std::max(kmax, cfg.k[i]);
    sea.kmax = kmax;

    // FP64 component inputs on the device
    double *d_in = nullptr;
    size_t nn = (size_t)(n > 0 ? n : 1);
    CK(cudaMalloc(&d_in, sizeof(double) * nn * 8));
    const std::vector<double> *src[8] = {&cfg.omega, &cfg.A, &cfg.k, &cfg.theta, &cfg.phase,
                                         &cfg.ramptime, &cfg.starttime, &cfg.duration};
    for (int q = 0; q < 8; q++)
        if (n) CK(cudaMemcpyAsync(d_in + q * nn, src[q]->data(), sizeof(double) * n,
                                  cudaMemcpyHostToDevice, stream));
    CompIn ci;
    ci.n = n; ci.npad = sea.npad_g;
    ci.omega = d_in; ci.A = d_in + nn; ci.k = d_in + 2 * nn; ci.theta = d_in + 3 * nn;
    ci.depth = cfg.depth; ci.g = cfg.gravity; ci.rho = cfg.rho;
    ci.mtheta_rad = cfg.mtheta * PI_IRR / 180.0;
    ci.cutoff = cfg.dw_cutoff; ci.bandwidth = cfg.dw_bandwidth; ci.kmax = kmax;

    CK(cudaMalloc(&sea.d_phase, sizeof(double) * 7 * sea.npad_g));
    CK(cudaMalloc(&sea.d_cf, sizeof(float) * NCF * sea.npad_g));
    CK(cudaMalloc(&sea.d_dfcomp, sizeof(float) * DF_COMP_FLOATS * 3 * sea.npad_g));
    // records for up to the next multiple of 256 components (the plain
    // precision form pads to 256), zero past the last component
    const int nrec_cap = ((sea.npad_g + 255) / 256) * 256;
    CK(cudaMalloc(&sea.d_phrec, sizeof(float) * PH_REC * nrec_cap));
    k_component_coefs<<<(sea.npad_g + 127) / 128, 128, 0, stream>>>(
        ci, sea.npad_g, cfg.x_pos, cfg.y_pos, cfg.tofmax, d_in + 4 * nn, d_in + 5 * nn,
        d_in + 6 * nn, d_in + 7 * nn, sea.d_phase, sea.d_cf);
    note_launch();
    CK(cudaGetLastError());
    k_phasor_records<<<(nrec_cap + 127) / 128, 128, 0, stream>>>(n, nrec_cap, sea.d_phase, sea.d_cf,
                                                                 sea.npad_g, sea.d_phrec);
    note_launch();
    CK(cudaGetLastError());

    if (cfg.order == 2) {
        long ntiles = tile_index(sea.ntile_g - 1, sea.ntile_g - 1, sea.ntile_g) + 1;
        size_t ent = (size_t)ntiles * GRID_TILE * GRID_TILE;
        CK(cudaMalloc(&sea.d_tab_eta, sizeof(float) * ent * EATA_NC));
        CK(cudaMalloc(&sea.d_tab_grid, sizeof(float) * ent * GRIDV_NC));
        CK(cudaMalloc(&sea.d_tab_gp, sizeof(float) * ent * GRIDP_NC));
        CK(cudaMalloc(&sea.d_tab_gk, sizeof(float) * ent * GRIDP_NC));
        k_build_tables<<<(unsigned)ntiles, 256, 0, stream>>>(ci, GRID_TILE, sea.ntile_g, 0,
                                                             sea.d_tab_eta, sea.d_tab_grid, sea.d_tab_gp,
                                                             sea.d_tab_gk);
        note_launch();
        CK(cudaGetLastError());
        if (point_table) {
            long ntp = tile_index(sea.ntile_p - 1, sea.ntile_p - 1, sea.ntile_p) + 1;
            size_t entp = (size_t)ntp * POINT_TILE * POINT_TILE;
            CK(cudaMalloc(&sea.d_tab_point, sizeof(float) * entp * POINTV_NC));
            k_build_tables<<<(unsigned)ntp, 256, 0, stream>>>(ci, POINT_TILE, sea.ntile_p, 1,
                                                              nullptr, sea.d_tab_point, nullptr, nullptr);
            note_launch();
            CK(cudaGetLastError());
        }
        if (cfg.vertical_theory == 1) {
            SmitIn si;
            si.n = n; si.omega = ci.omega; si.A = ci.A; si.k = ci.k; si.theta = ci.theta;
            si.depth = ci.depth; si.g = ci.g; si.rho = ci.rho; si.mtheta_rad = ci.mtheta_rad;
            si.cutoff = ci.cutoff; si.bandwidth = ci.bandwidth; si.kmax = ci.kmax;
            int rc = smit_build(si, sea, stream);
            if (rc) return rc;
            sea.smit = true;
        }
        unsigned long long *d_cnt = nullptr, h_cnt = 0;
        CK(cudaMalloc(&d_cnt, sizeof(unsigned long long)));
        CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), stream));
        k_count_pairs<<<256, 256, 0, stream>>>(ci, d_cnt);
        note_launch();
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&h_cnt, d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        cudaFree(d_cnt);
        sea.npairs_grid = (long)h_cnt;
    }
    CK(cudaStreamSynchronize(stream));
    cudaFree(d_in);
    return OK;
}

void sea_free(DevSea &sea) {
    if (sea.d_phase) cudaFree(sea.d_phase);
    if (sea.d_cf) cudaFree(sea.d_cf);
    if (sea.d_tab_eta) cudaFree(sea.d_tab_eta);
    if (sea.d_tab_grid) cudaFree(sea.d_tab_grid);
    if (sea.d_tab_point) cudaFree(sea.d_tab_point);
    if (sea.d_tab_gp) cudaFree(sea.d_tab_gp);
    if (sea.d_tab_gk) cudaFree(sea.d_tab_gk);
    if (sea.d_tab_smit) cudaFree(sea.d_tab_smit);
    if (sea.d_dfcomp) cudaFree(sea.d_dfcomp);
    if (sea.d_phrec) cudaFree(sea.d_phrec);
    sea.d_tab_smit = nullptr;
    sea.d_dfcomp = nullptr;
    sea.d_phrec = nullptr;
    sea.smit = false;
    sea.d_phase = nullptr; sea.d_cf = nullptr; sea.d_tab_eta = nullptr;
    sea.d_tab_grid = nullptr; sea.d_tab_point = nullptr; sea.d_tab_gp = nullptr; sea.d_tab_gk = nullptr;
}

int workspace_reserve(Workspace &ws, size_t bytes) {
    if (ws.bytes >= bytes) return OK;
    if (ws.base) cudaFree(ws.base);
    ws.base = nullptr;
    ws.bytes = 0;
    CK(cudaMalloc(&ws.base, bytes));
    ws.bytes = bytes;
    return OK;
}
void workspace_free(Workspace &ws) {
    if (ws.base) cudaFree(ws.base);
    ws.base = nullptr;
    ws.bytes = 0;
}

// ---------------------------------------------------------------------------
// Phasor pass: one thread per point/column, all components.
// ---------------------------------------------------------------------------
struct PhArgs {
    long n;
    const double *x, *y, *t;
    long sx, sy, st;        // element strides of x, y, t (0 broadcasts one value)
    int ncomp, npad;
    const double *phase;    // [7][npad_g]
    const float *cf;        // [NCF][npad_g]
    int cstride;            // npad_g
    double fx, fy;
    int trivial_ramp;
    const float *rec;       // [npad_g][PH_REC] phasor records
    float2 *ph;             // [npad][n]
    float *rr;              // [npad][n]
    double *first;          // [5][n]: eta1, gx, gy, gz, gp
};

__device__ __forceinline__ void ph_kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// One thread per point: the phasors (cos, sin) and ramps of every component
// and the first-order sums eta1 and the Taylor gradients.  The phase
// kx (x - fx) + ky (y - fy) - omega t + phase0 is formed in float-float from
// the records (the point's coordinates split by integer operations) and
// reduced, then sine and cosine by polynomial (within 1e-7; the SFU's few
// 1e-7 raised the plain form's error against FP64 tenfold); the sums are FP32
// with Kahan compensation.  FP64 per (point, component) -- phase, reduction and FP64
// sums -- kept the FP64 pipe the bound on this GPU.  Only non-trivial
// component ramps are evaluated in FP64 (Irregular.cpp:200-204).
__global__ void __launch_bounds__(128) k_phasors(PhArgs a) {
    __shared__ float s_rec[PH_CHUNK * PH_REC];
    __shared__ float2 s_off[2];
    const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const bool valid = p < a.n;
    const long pc = valid ? p : 0;
    if (threadIdx.x == 0) {
        ff_split(-a.fx, s_off[0].x, s_off[0].y);
        ff_split(-a.fy, s_off[1].x, s_off[1].y);
    }
    __syncthreads();
    const double tp = a.t[pc * a.st];
    const float2 dx = ff_add(ff_from_double(a.x[pc * a.sx]), s_off[0]);
    const float2 dy = ff_add(ff_from_double(a.y[pc * a.sy]), s_off[1]);
    const float2 tt = ff_from_double(tp);
    const double *P = a.phase;
    const int cs = a.cstride;
    const float rconst = a.trivial_ramp ? (float)d_freq_ramp(tp, P[4 * cs], P[5 * cs], P[6 * cs]) : 0.f;
    float sm[5] = {0, 0, 0, 0, 0}, cm[5] = {0, 0, 0, 0, 0};
    for (int i0 = 0; i0 < a.npad; i0 += PH_CHUNK) {
        const int nrec = min(PH_CHUNK, a.npad - i0);
        __syncthreads();
        for (int e = threadIdx.x; e < nrec * PH_REC; e += blockDim.x) s_rec[e] = a.rec[(long)i0 * PH_REC + e];
        __syncthreads();
        if (!valid) continue;
        for (int ii = 0; ii < nrec; ii++) {
            const int i = i0 + ii;
            const float *R = s_rec + ii * PH_REC;
            float c = 0.f, s = 0.f, r = 0.f;
            if (i < a.ncomp) {
                float2 ph = ff_add(ff_mul(R[0], R[1], dx.x, dx.y), ff_mul(R[2], R[3], dy.x, dy.y));
                ph = ff_add(ph, ff_mul(R[4], R[5], tt.x, tt.y));
                ph = ff_add(ph, make_float2(R[6], R[7]));
                ff_sincos_poly(ff_reduce_2pi(ph), s, c);
                r = a.trivial_ramp ? rconst
                                   : (float)d_freq_ramp(tp, P[4 * cs + i], P[5 * cs + i], P[6 * cs + i]);
                const float rc = r * c, rs = r * s;
                ph_kahan(sm[0], cm[0], rc * R[8]);
                ph_kahan(sm[1], cm[1], rc * R[9]);
                ph_kahan(sm[2], cm[2], rc * R[10]);
                ph_kahan(sm[3], cm[3], rs * R[11]);
                ph_kahan(sm[4], cm[4], rc * R[12]);
            }
            a.ph[(long)i * a.n + p] = make_float2(c, s);
            a.rr[(long)i * a.n + p] = r;
        }
    }
    if (!valid) return;
    for (int q = 0; q < 5; q++) a.first[q * a.n + p] = (double)sm[q] - (double)cm[q];
}

// Few points (a scalar call, a short batch): one block per point, the
// components spread over the threads, so that a point's N phasors are formed
// in parallel instead of by one thread in turn.  The same records and
// arithmetic per (point, component) as k_phasors; each thread's share of the
// five first-order sums is Kahan-compensated in FP32 and the 128 shares are
// added in FP64 (per point, not per component).
__global__ void __launch_bounds__(128) k_phasors_few(PhArgs a) {
    __shared__ double s_red[4][5];
    const long p = blockIdx.x;
    float2 off[2];
    ff_split(-a.fx, off[0].x, off[0].y);
    ff_split(-a.fy, off[1].x, off[1].y);
    const double tp = a.t[p * a.st];
    const float2 dx = ff_add(ff_from_double(a.x[p * a.sx]), off[0]);
    const float2 dy = ff_add(ff_from_double(a.y[p * a.sy]), off[1]);
    const float2 tt = ff_from_double(tp);
    const double *P = a.phase;
    const int cs = a.cstride;
    const float rconst = a.trivial_ramp ? (float)d_freq_ramp(tp, P[4 * cs], P[5 * cs], P[6 * cs]) : 0.f;
    float sm[5] = {0, 0, 0, 0, 0}, cm[5] = {0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < a.npad; i += blockDim.x) {
        const float *R = a.rec + (long)i * PH_REC;
        float c = 0.f, sn = 0.f, r = 0.f;
        if (i < a.ncomp) {
            float2 ph = ff_add(ff_mul(R[0], R[1], dx.x, dx.y), ff_mul(R[2], R[3], dy.x, dy.y));
            ph = ff_add(ph, ff_mul(R[4], R[5], tt.x, tt.y));
            ph = ff_add(ph, make_float2(R[6], R[7]));
            ff_sincos_poly(ff_reduce_2pi(ph), sn, c);
            r = a.trivial_ramp ? rconst : (float)d_freq_ramp(tp, P[4 * cs + i], P[5 * cs + i], P[6 * cs + i]);
            const float rc = r * c, rs = r * sn;
            ph_kahan(sm[0], cm[0], rc * R[8]);
            ph_kahan(sm[1], cm[1], rc * R[9]);
            ph_kahan(sm[2], cm[2], rc * R[10]);
            ph_kahan(sm[3], cm[3], rs * R[11]);
            ph_kahan(sm[4], cm[4], rc * R[12]);
        }
        a.ph[(long)i * a.n + p] = make_float2(c, sn);
        a.rr[(long)i * a.n + p] = r;
    }
    double v[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
        v[q] = (double)sm[q] - (double)cm[q];
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int q = 0; q < 5; q++) s_red[warp][q] = v[q];
    __syncthreads();
    if (threadIdx.x < 5)
        a.first[threadIdx.x * a.n + p] = ((s_red[0][threadIdx.x] + s_red[1][threadIdx.x]) + s_red[2][threadIdx.x]) +
                                         s_red[3][threadIdx.x];
}

// ---------------------------------------------------------------------------
// Pair-sum kernels
// ---------------------------------------------------------------------------
struct PairArgs {
    long ncol;           // points / columns
    int nl;              // levels per column
    int nlg;             // level groups per column (power of two, <= 16)
    int ntile;           // component tiles of the table
    const float *tab;    // pair tiles
    const float2 *tabp;  // pressure pair tiles (Pp, Mp), column kernel with pressure
    const float2 *ph;    // [npad][ncol]
    const float *rr;     // [npad][ncol]
    const float *cf;     // [NCF][cstride]
    int cstride;
    const float *z0;     // [ncol*nl] evaluation heights (z0 <= 0 below the surface)
    float depth;
    float *out;          // [nf][ncol*nl]
    int pairs;           // 0: first-order z-dependent sums only
    int first;           // 1: add first-order z-dependent sums
    int tp_per;          // tile pairs per blockIdx.y (split of the pair loop; partial sums
                         // of slice y go to out + y * nf * ncol * nl)
};

// Depth factors with the normaliser folded into the coefficients:
//   F = exp(kz) (1 + exp(-2k(z+h))),  G = exp(kz) (1 - exp(-2k(z+h))).
__device__ __forceinline__ void depth_fg(float k, float zk, float zetak, float &F, float &G) {
    const float e1 = ex2(k * zk);
    const float e2 = ex2(k * zetak);
    F = fmaf(e1, e2, e1);       // e1 (1 + e2), one rounding
    G = fmaf(-e1, e2, e1);      // e1 (1 - e2)
}

// Column mode: u, v, w (PR: and the phase terms of the pressure, with the
// first-order dp1) at LV levels per thread, grid (pair-cache) mask.
template <int TT, int LV, bool PR>
__global__ void __launch_bounds__(128) k_pairs_columns(PairArgs a) {
    extern __shared__ float4 smem4[];
    constexpr int NF = PR ? 4 : 3;
    float *s_tab = reinterpret_cast<float *>(smem4);                       // TT*TT*8
    float2 *s_tp = reinterpret_cast<float2 *>(s_tab + TT * TT * GRIDV_NC); // TT*TT (PR)
    float2 *s_ph = s_tp + (PR ? TT * TT : 0);                             // TT*cols
    const int cols = 128 / a.nlg;
    const int lg = threadIdx.x / cols, cl = threadIdx.x % cols;
    const long col = (long)blockIdx.x * cols + cl;
    const bool valid = col < a.ncol;
    const long colc = valid ? col : 0;
    const long npts = a.ncol * a.nl;
    static_assert(LV % 2 == 0, "levels are processed in pairs");
    constexpr int LP = LV / 2;
    float zk[LV], zetak[LV], yk[LV];   // z log2(e), -2(z + h) log2(e), -(z + 2h) log2(e)
    float2 zk2[LP], yk2[LP];
    float su[LV], cu[LV], sv[LV], cv[LV], sw[LV], cw[LV];
    float sp[PR ? LV : 1], cq[PR ? LV : 1];     // pressure sum and carry
#pragma unroll
    for (int l = 0; l < LV; l++) {
        int lev = lg * LV + l;
        float z = (valid && lev < a.nl) ? a.z0[colc * a.nl + lev] : 0.f;
        zk[l] = z * LOG2E_F;
        zetak[l] = -2.f * (z + a.depth) * LOG2E_F;
        yk[l] = -(z + 2.f * a.depth) * LOG2E_F;
        su[l] = cu[l] = sv[l] = cv[l] = sw[l] = cw[l] = 0.f;
        if (PR) sp[l] = cq[l] = 0.f;
    }
#pragma unroll
    for (int j = 0; j < LP; j++) {
        zk2[j] = make_float2(zk[2 * j], zk[2 * j + 1]);
        yk2[j] = make_float2(yk[2 * j], yk[2 * j + 1]);
    }
    // slice of the tile-pair loop owned by this blockIdx.y (block-uniform)
    const int tp_lo = blockIdx.y * a.tp_per, tp_hi = tp_lo + a.tp_per;
    int tp = -1;
    for (int I = 0; I < a.ntile; I++) {
        for (int M = I; M < a.ntile; M++) {
            if (!a.pairs && M != I) continue;
            tp++;
            if (tp < tp_lo || tp >= tp_hi) continue;
            __syncthreads();
            if (a.pairs) {
                const float4 *src = reinterpret_cast<const float4 *>(
                    a.tab + tile_index(I, M, a.ntile) * (long)TT * TT * GRIDV_NC);
                float4 *dst = reinterpret_cast<float4 *>(s_tab);
                for (int e = threadIdx.x; e < TT * TT * GRIDV_NC / 4; e += blockDim.x) dst[e] = src[e];
                if (PR) {
                    const float2 *srp = a.tabp + tile_index(I, M, a.ntile) * (long)TT * TT;
                    for (int e = threadIdx.x; e < TT * TT; e += blockDim.x) s_tp[e] = srp[e];
                }
            }
            for (int e = threadIdx.x; e < TT * cols; e += blockDim.x) {
                int mm = e / cols, c2 = e % cols;
                long cc = (long)blockIdx.x * cols + c2;
                s_ph[e] = (cc < a.ncol) ? a.ph[(long)(M * TT + mm) * a.ncol + cc] : make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (!valid) continue;
            if (a.pairs) {
                for (int ii = 0; ii < TT; ii++) {
                    const int i = I * TT + ii;
                    const float2 pi = a.ph[(long)i * a.ncol + col];
                    const float ri = a.rr[(long)i * a.ncol + col];
                    // packed FP32x2 over level pairs: per pair and level,
                    // E = exp(k z), Y = exp(-k(z + 2h)) = E exp(-2k(z+h)),
                    // F = E + Y, G = E - Y (the normaliser is in the record)
                    float2 au[LP], av[LP], aw[LP], apr[PR ? LP : 1];
#pragma unroll
                    for (int j = 0; j < LP; j++) au[j] = av[j] = aw[j] = make_float2(0.f, 0.f);
#pragma unroll
                    for (int j = 0; j < (PR ? LP : 1); j++) apr[j] = make_float2(0.f, 0.f);
                    const float2 neg1 = make_float2(-1.f, -1.f);
                    const int m0 = (M == I) ? ii : 0;
                    for (int mm = m0; mm < TT; mm++) {
                        const float4 c0 = *reinterpret_cast<const float4 *>(s_tab + (ii * TT + mm) * GRIDV_NC);
                        const float4 c1 = *reinterpret_cast<const float4 *>(s_tab + (ii * TT + mm) * GRIDV_NC + 4);
                        const float2 pm = s_ph[mm * cols + cl];
                        const float cc = pi.x * pm.x, ss = pi.y * pm.y;
                        const float sc = pi.y * pm.x, cs = pi.x * pm.y;
                        const float cp = cc - ss, cmn = cc + ss, sp = sc + cs, smn = sc - cs;
                        const float up = c0.x * cp, um = c0.y * cmn, vp = c0.z * cp, vm = c0.w * cmn;
                        const float wp = c1.x * sp, wm = c1.y * smn;
                        const float2 up2 = make_float2(up, up), um2 = make_float2(um, um);
                        const float2 vp2 = make_float2(vp, vp), vm2 = make_float2(vm, vm);
                        const float2 wp2 = make_float2(wp, wp), wm2 = make_float2(wm, wm);
                        const float2 kp2 = make_float2(c1.z, c1.z), km2 = make_float2(c1.w, c1.w);
                        float2 pp2 = make_float2(0.f, 0.f), pm2 = pp2;
                        if (PR) {
                            const float2 tp = s_tp[ii * TT + mm];
                            const float pp = tp.x * cp, pm_ = tp.y * cmn;
                            pp2 = make_float2(pp, pp);
                            pm2 = make_float2(pm_, pm_);
                        }
#pragma unroll
                        for (int j = 0; j < LP; j++) {
                            const float2 ap = __fmul2_rn(kp2, zk2[j]), bp = __fmul2_rn(kp2, yk2[j]);
                            const float2 am = __fmul2_rn(km2, zk2[j]), bm = __fmul2_rn(km2, yk2[j]);
                            const float2 Ep = make_float2(ex2(ap.x), ex2(ap.y));
                            const float2 Yp = make_float2(ex2(bp.x), ex2(bp.y));
                            const float2 Em = make_float2(ex2(am.x), ex2(am.y));
                            const float2 Ym = make_float2(ex2(bm.x), ex2(bm.y));
                            const float2 Fp = __fadd2_rn(Ep, Yp), Gp = __ffma2_rn(Yp, neg1, Ep);
                            const float2 Fm = __fadd2_rn(Em, Ym), Gm = __ffma2_rn(Ym, neg1, Em);
                            au[j] = __ffma2_rn(up2, Fp, __ffma2_rn(um2, Fm, au[j]));
                            av[j] = __ffma2_rn(vp2, Fp, __ffma2_rn(vm2, Fm, av[j]));
                            aw[j] = __ffma2_rn(wp2, Gp, __ffma2_rn(wm2, Gm, aw[j]));
                            if (PR) apr[j] = __ffma2_rn(pp2, Fp, __ffma2_rn(pm2, Fm, apr[j]));
                        }
                    }
#pragma unroll
                    for (int j = 0; j < LP; j++) {
                        kahan(su[2 * j], cu[2 * j], ri * au[j].x);
                        kahan(su[2 * j + 1], cu[2 * j + 1], ri * au[j].y);
                        kahan(sv[2 * j], cv[2 * j], ri * av[j].x);
                        kahan(sv[2 * j + 1], cv[2 * j + 1], ri * av[j].y);
                        kahan(sw[2 * j], cw[2 * j], ri * aw[j].x);
                        kahan(sw[2 * j + 1], cw[2 * j + 1], ri * aw[j].y);
                        if (PR) {
                            kahan(sp[2 * j], cq[2 * j], ri * apr[j].x);
                            kahan(sp[2 * j + 1], cq[2 * j + 1], ri * apr[j].y);
                        }
                    }
                }
            }
            if (a.first && M == I) {
                // first-order u1, v1, w1 at the level heights (Irregular.cpp:394-447)
                for (int mm = 0; mm < TT; mm++) {
                    const int m = M * TT + mm;
                    const float2 pm = s_ph[mm * cols + cl];
                    const float rm = a.rr[(long)m * a.ncol + col];
                    const float k = a.cf[CF_K * a.cstride + m], q = a.cf[CF_Q * a.cstride + m];
                    const float au_ = a.cf[CF_AU * a.cstride + m] * q * rm;
                    const float cu_ = au_ * a.cf[CF_CT * a.cstride + m] * pm.x;
                    const float cv_ = au_ * a.cf[CF_ST * a.cstride + m] * pm.x;
                    const float cw_ = au_ * pm.y;
                    // dp1 (Irregular.cpp:1107-1120)
                    const float cp_ = PR ? a.cf[CF_AP * a.cstride + m] * q * rm * pm.x : 0.f;
#pragma unroll
                    for (int l = 0; l < LV; l++) {
                        float F, G;
                        depth_fg(k, zk[l], zetak[l], F, G);
                        kahan(su[l], cu[l], cu_ * F);
                        kahan(sv[l], cv[l], cv_ * F);
                        kahan(sw[l], cw[l], cw_ * G);
                        if (PR) kahan(sp[l], cq[l], cp_ * F);
                    }
                }
            }
        }
    }
    if (!valid) return;
    float *out = a.out + (long)blockIdx.y * NF * npts;
#pragma unroll
    for (int l = 0; l < LV; l++) {
        int lev = lg * LV + l;
        if (lev < a.nl) {
            long o = col * a.nl + lev;
            out[0 * npts + o] = su[l];
            out[1 * npts + o] = sv[l];
            out[2 * npts + o] = sw[l];
            if (PR) out[3 * npts + o] = sp[l];
        }
    }
}

// Sum of the split slices of the column kernel, in slice order.
__global__ void k_sum_slices(long n, int nslice, const float *part, float *out) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= n) return;
    float s = 0.f, c = 0.f;
    for (int k = 0; k < nslice; k++) kahan(s, c, part[(long)k * n + e]);
    out[e] = s;
}

// Point mode: u, v, w, dp at one height per thread, point-API mask
// (u2/v2/w2/dp2 of the reference, with rho folded into the p records).
// VEL: the velocity sums, PR: the pressure sums (a call that asks for one of
// them does not pay for the other; rows not computed are 0).
template <int TT, bool VEL, bool PR>
__global__ void __launch_bounds__(128) k_pairs_points(PairArgs a) {
    extern __shared__ float4 smem4[];
    float *s_tab = reinterpret_cast<float *>(smem4);                        // TT*TT*12
    float2 *s_ph = reinterpret_cast<float2 *>(s_tab + TT * TT * POINTV_NC); // TT*128
    float2 *s_pz = s_ph + TT * 128;                                         // TT*128
    const long p = (long)blockIdx.x * 128 + threadIdx.x;
    const bool valid = p < a.ncol;
    const long pc = valid ? p : 0;
    const float z = valid ? a.z0[pc] : 0.f;
    const float zk = z * LOG2E_F, zetak = -2.f * (z + a.depth) * LOG2E_F;
    float su = 0, cu = 0, sv = 0, cv = 0, sw = 0, cw = 0, sq = 0, cq = 0;
    // slice of the tile-pair loop owned by this blockIdx.y (block-uniform)
    const int tp_lo = blockIdx.y * a.tp_per, tp_hi = tp_lo + a.tp_per;
    int tp = -1;
    for (int I = 0; I < a.ntile; I++) {
        for (int M = I; M < a.ntile; M++) {
            if (!a.pairs && M != I) continue;
            tp++;
            if (tp < tp_lo || tp >= tp_hi) continue;
            __syncthreads();
            if (a.pairs) {
                const float4 *src = reinterpret_cast<const float4 *>(
                    a.tab + tile_index(I, M, a.ntile) * (long)TT * TT * POINTV_NC);
                float4 *dst = reinterpret_cast<float4 *>(s_tab);
                for (int e = threadIdx.x; e < TT * TT * POINTV_NC / 4; e += blockDim.x) dst[e] = src[e];
            }
            for (int mm = 0; mm < TT; mm++) {
                const int m = M * TT + mm;
                float2 pm = a.ph[(long)m * a.ncol + pc];
                float F, G;
                depth_fg(a.cf[CF_K * a.cstride + m], zk, zetak, F, G);
                const float q = a.cf[CF_Q * a.cstride + m];
                s_ph[mm * 128 + threadIdx.x] = pm;
                s_pz[mm * 128 + threadIdx.x] = make_float2(q * F, q * G);   // px_m, pz_m
            }
            __syncthreads();
            if (!valid) continue;
            if (a.pairs) {
                for (int ii = 0; ii < TT; ii++) {
                    const int i = I * TT + ii;
                    const float2 pi = a.ph[(long)i * a.ncol + p];
                    const float ri = a.rr[(long)i * a.ncol + p];
                    const float2 pxi = (M == I) ? s_pz[ii * 128 + threadIdx.x] : make_float2(0.f, 0.f);
                    float2 pxz_i = pxi;
                    if (M != I) {
                        float F, G;
                        depth_fg(a.cf[CF_K * a.cstride + i], zk, zetak, F, G);
                        const float q = a.cf[CF_Q * a.cstride + i];
                        pxz_i = make_float2(q * F, q * G);
                    }
                    float au = 0, av = 0, aw = 0, ap = 0, ax = 0, az = 0;
                    const int m0 = (M == I) ? ii : 0;
                    for (int mm = m0; mm < TT; mm++) {
                        const float *e = s_tab + (ii * TT + mm) * POINTV_NC;
                        const float4 c0 = *reinterpret_cast<const float4 *>(e);
                        const float4 c1 = *reinterpret_cast<const float4 *>(e + 4);
                        const float4 c2 = *reinterpret_cast<const float4 *>(e + 8);
                        const float2 pm = s_ph[mm * 128 + threadIdx.x];
                        const float2 xm = s_pz[mm * 128 + threadIdx.x];
                        const float cc = pi.x * pm.x, ss = pi.y * pm.y;
                        const float sc = pi.y * pm.x, cs = pi.x * pm.y;
                        const float cp = cc - ss, cmn = cc + ss, sp = sc + cs, smn = sc - cs;
                        float Fp, Gp, Fm, Gm;
                        depth_fg(c2.x, zk, zetak, Fp, Gp);
                        depth_fg(c2.y, zk, zetak, Fm, Gm);
                        // the phase-and-depth products once, then one FMA per coefficient
                        const float A = cp * Fp, B = cmn * Fm;
                        if (VEL) {
                            const float Cq = sp * Gp, D = smn * Gm;
                            au = fmaf(c0.x, A, fmaf(c0.y, B, au));
                            av = fmaf(c0.z, A, fmaf(c0.w, B, av));
                            aw = fmaf(c1.x, Cq, fmaf(c1.y, D, aw));
                        }
                        if (PR) {
                            ap = fmaf(c1.z, A, fmaf(c1.w, B, ap));
                            ax = fmaf(c2.z, xm.x, ax);
                            az = fmaf(c2.w, xm.y, az);
                        }
                    }
                    if (VEL) {
                        kahan(su, cu, ri * au);
                        kahan(sv, cv, ri * av);
                        kahan(sw, cw, ri * aw);
                    }
                    if (PR) {
                        ap = fmaf(pxz_i.x, ax, fmaf(pxz_i.y, az, ap));
                        kahan(sq, cq, ri * ap);
                    }
                }
            }
            if (a.first && M == I) {
                // first-order u1, v1, w1, dp1 and the linear dp2 diagonal terms
                for (int mm = 0; mm < TT; mm++) {
                    const int m = M * TT + mm;
                    const float2 pm = s_ph[mm * 128 + threadIdx.x];
                    const float2 xm = s_pz[mm * 128 + threadIdx.x];
                    const float rm = a.rr[(long)m * a.ncol + p];
                    if (VEL) {
                        const float au_ = a.cf[CF_AU * a.cstride + m] * rm;
                        kahan(su, cu, au_ * xm.x * a.cf[CF_CT * a.cstride + m] * pm.x);
                        kahan(sv, cv, au_ * xm.x * a.cf[CF_ST * a.cstride + m] * pm.x);
                        kahan(sw, cw, au_ * xm.y * pm.y);
                    }
                    if (PR) {
                        float pp = a.cf[CF_AP * a.cstride + m] * xm.x * pm.x;
                        if (a.pairs)
                            pp += a.cf[CF_X1 * a.cstride + m] * xm.x + a.cf[CF_Z1 * a.cstride + m] * xm.y;
                        kahan(sq, cq, rm * pp);
                    }
                }
            }
        }
    }
    if (!valid) return;
    float *out = a.out + (long)blockIdx.y * 4 * a.ncol;
    out[0 * a.ncol + p] = su;
    out[1 * a.ncol + p] = sv;
    out[2 * a.ncol + p] = sw;
    out[3 * a.ncol + p] = sq;
}

// Few points, point mode: block (point p, slice y); thread t takes row
// ii = t % TT of tile pair 8 g + t / TT for g = y, y + nslice, ... (TT = 16: 8
// tile pairs a pass).  A row is summed over its mm as in k_pairs_points (the
// depth factors of component m formed per term here, since no other point
// shares them), diagonal tile pairs add the first-order term of component
// I TT + ii, each thread's rows are Kahan-summed, and the block's 128 sums
// are added in FP32 into slice y's partial sums ([nslice][4][n], summed in
// order by k_sum_slices).
template <int TT>
__global__ void __launch_bounds__(128) k_pairs_points_few(PairArgs a, int ntp, int nslice) {
    __shared__ float s_red[4][4];
    const long p = blockIdx.x;
    const float z = a.z0[p];
    const float zk = z * LOG2E_F, zetak = -2.f * (z + a.depth) * LOG2E_F;
    const int ii = threadIdx.x % TT;
    constexpr int PER = 128 / TT;           // tile pairs a pass
    float su = 0, cu = 0, sv = 0, cv = 0, sw = 0, cw = 0, sq = 0, cq = 0;
    for (int g = blockIdx.y; g * PER < ntp; g += nslice) {
        int tp = g * PER + threadIdx.x / TT;
        if (tp >= ntp) continue;
        int I = 0, M = 0;
        if (a.pairs) {
            while (tp >= a.ntile - I) { tp -= a.ntile - I; I++; }
            M = I + tp;
        } else {
            I = M = tp;
        }
        const int i = I * TT + ii;
        const float2 pi = a.ph[(long)i * a.ncol + p];
        const float ri = a.rr[(long)i * a.ncol + p];
        float Fi, Gi;
        depth_fg(a.cf[CF_K * a.cstride + i], zk, zetak, Fi, Gi);
        const float qi = a.cf[CF_Q * a.cstride + i];
        const float2 pxz_i = make_float2(qi * Fi, qi * Gi);
        if (a.pairs) {
            const float *T = a.tab + tile_index(I, M, a.ntile) * (long)TT * TT * POINTV_NC;
            float au = 0, av = 0, aw = 0, ap = 0, ax = 0, az = 0;
            for (int mm = (M == I) ? ii : 0; mm < TT; mm++) {
                const int m = M * TT + mm;
                const float *e = T + (ii * TT + mm) * POINTV_NC;
                const float4 c0 = *reinterpret_cast<const float4 *>(e);
                const float4 c1 = *reinterpret_cast<const float4 *>(e + 4);
                const float4 c2 = *reinterpret_cast<const float4 *>(e + 8);
                const float2 pm = a.ph[(long)m * a.ncol + p];
                float Fm_, Gm_;
                depth_fg(a.cf[CF_K * a.cstride + m], zk, zetak, Fm_, Gm_);
                const float qm = a.cf[CF_Q * a.cstride + m];
                const float2 xm = make_float2(qm * Fm_, qm * Gm_);
                const float cc = pi.x * pm.x, ss = pi.y * pm.y;
                const float sc = pi.y * pm.x, cs = pi.x * pm.y;
                const float cp = cc - ss, cmn = cc + ss, sp = sc + cs, smn = sc - cs;
                float Fp, Gp, Fm, Gm;
                depth_fg(c2.x, zk, zetak, Fp, Gp);
                depth_fg(c2.y, zk, zetak, Fm, Gm);
                const float A = cp * Fp, B = cmn * Fm, Cq = sp * Gp, D = smn * Gm;
                au = fmaf(c0.x, A, fmaf(c0.y, B, au));
                av = fmaf(c0.z, A, fmaf(c0.w, B, av));
                aw = fmaf(c1.x, Cq, fmaf(c1.y, D, aw));
                ap = fmaf(c1.z, A, fmaf(c1.w, B, ap));
                ax = fmaf(c2.z, xm.x, ax);
                az = fmaf(c2.w, xm.y, az);
            }
            ap = fmaf(pxz_i.x, ax, fmaf(pxz_i.y, az, ap));
            kahan(su, cu, ri * au);
            kahan(sv, cv, ri * av);
            kahan(sw, cw, ri * aw);
            kahan(sq, cq, ri * ap);
        }
        if (a.first && M == I) {
            // first-order u1, v1, w1, dp1 and the linear dp2 diagonal terms of component i
            const float au_ = a.cf[CF_AU * a.cstride + i] * ri;
            kahan(su, cu, au_ * pxz_i.x * a.cf[CF_CT * a.cstride + i] * pi.x);
            kahan(sv, cv, au_ * pxz_i.x * a.cf[CF_ST * a.cstride + i] * pi.x);
            kahan(sw, cw, au_ * pxz_i.y * pi.y);
            float pp = a.cf[CF_AP * a.cstride + i] * pxz_i.x * pi.x;
            if (a.pairs)
                pp += a.cf[CF_X1 * a.cstride + i] * pxz_i.x + a.cf[CF_Z1 * a.cstride + i] * pxz_i.y;
            kahan(sq, cq, ri * pp);
        }
    }
    float v[4] = {su - cu, sv - cv, sw - cw, sq - cq};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        for (int o = 16; o > 0; o >>= 1) v[f] += __shfl_down_sync(0xffffffffu, v[f], o);
        if (lane == 0) s_red[warp][f] = v[f];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int f = threadIdx.x;
        a.out[((long)blockIdx.y * 4 + f) * a.ncol + p] = ((s_red[0][f] + s_red[1][f]) + s_red[2][f]) + s_red[3][f];
    }
}

// Elevation mode: eta2 from the pair cache (Irregular.cpp:223-293).  The
// record holds A = P+M and B = M-P so that a pair contributes
// c_i (A c_m) + s_i (B s_m); a row is c_i sum(A c_m) + s_i sum(B s_m).
template <int TT>
__global__ void __launch_bounds__(128) k_pairs_eta(PairArgs a) {
    extern __shared__ float4 smem4[];
    float2 *s_tab = reinterpret_cast<float2 *>(smem4);        // TT*TT
    float2 *s_ph = s_tab + TT * TT;                            // TT*128
    const long p = (long)blockIdx.x * 128 + threadIdx.x;
    const bool valid = p < a.ncol;
    const long pc = valid ? p : 0;
    float se = 0, ce = 0;
    const int tp_lo = blockIdx.y * a.tp_per, tp_hi = tp_lo + a.tp_per;
    int tp = -1;
    for (int I = 0; I < a.ntile; I++) {
        for (int M = I; M < a.ntile; M++) {
            tp++;
            if (tp < tp_lo || tp >= tp_hi) continue;   // block-uniform
            __syncthreads();
            const float4 *src = reinterpret_cast<const float4 *>(
                a.tab + tile_index(I, M, a.ntile) * (long)TT * TT * 2);
            float4 *dst = reinterpret_cast<float4 *>(s_tab);
            for (int e = threadIdx.x; e < TT * TT / 2; e += blockDim.x) dst[e] = src[e];
            for (int mm = 0; mm < TT; mm++)
                s_ph[mm * 128 + threadIdx.x] = a.ph[(long)(M * TT + mm) * a.ncol + pc];
            __syncthreads();
            if (!valid) continue;
            for (int ii = 0; ii < TT; ii++) {
                const int i = I * TT + ii;
                const float2 pi = a.ph[(long)i * a.ncol + p];
                const float ri = a.rr[(long)i * a.ncol + p];
                float ac = 0.f, as = 0.f;
                const int m0 = (M == I) ? ii : 0;
                for (int mm = m0; mm < TT; mm++) {
                    const float2 cab = s_tab[ii * TT + mm];
                    const float2 pm = s_ph[mm * 128 + threadIdx.x];
                    ac = fmaf(cab.x, pm.x, ac);
                    as = fmaf(cab.y, pm.y, as);
                }
                kahan(se, ce, ri * fmaf(pi.x, ac, pi.y * as));
            }
        }
    }
    if (valid) a.out[(long)blockIdx.y * a.ncol + p] = se;
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
namespace {

struct WsLayout {
    float2 *ph;
    float *rr;
    double *first;
    float *z0;
    float *sec;
    float *split;         // partial sums of a split point-pair launch
    long split_cap;       // its floats
    size_t bytes;
};

// Slices of the tile-pair loop for a launch of nblk blocks (per slice) on a
// GPU with `slots` resident blocks: the fewest slices (at most maxs, and at
// most one per tile pair) whose blocks fill the waves they start to 85 %, or
// else the best filling.  A launch of 512 point blocks on 760 slots fills
// 67 % of its one wave; 4 slices fill 90 % of three.
static int wave_slices(long nblk, int ntp, long slots, long maxs) {
    const long top = std::max<long>(1, std::min<long>(ntp, maxs));
    int best = 1;
    double beste = -1.0;
    for (long ns = 1; ns <= top; ns++) {
        const double w = (double)(nblk * ns) / (double)slots;
        const double eff = w / std::ceil(w);
        if (eff > beste + 1e-9) {
            beste = eff;
            best = (int)ns;
        }
        if (eff >= 0.85) break;
    }
    return best;
}

// Resident blocks of a kernel on the current device (0 where the query fails).
template <typename K>
static long resident_slots(K kernel, int threads, size_t smem) {
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (long)per * nsm;
}
// floats of the split region: room for 7 partial rows per slice and point at
// slices x points = 256 SPLIT_TARGET_BLOCKS; the launches take no more
// slices than the region holds for their batch.  It has that fixed size,
// whatever the batch (a batch's last, short chunk may split while its first
// does not).
static long point_split_floats(long n) {
    (void)n;
    return 7L * 128 * 2 * SPLIT_TARGET_BLOCKS;
}

WsLayout layout(long n, int npad, void *base) {
    WsLayout L;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off += (b + 255) & ~size_t(255); return o; };
    size_t o_ph = take(sizeof(float2) * (size_t)npad * n);
    size_t o_rr = take(sizeof(float) * (size_t)npad * n);
    size_t o_first = take(sizeof(double) * 5 * (size_t)n);
    size_t o_z = take(sizeof(float) * (size_t)n);
    size_t o_sec = take(sizeof(float) * 5 * (size_t)n);
    const long scap = point_split_floats(n);
    size_t o_split = take(sizeof(float) * (size_t)std::max<long>(scap, 1));
    char *b = (char *)base;
    L.ph = (float2 *)(b + o_ph);
    L.rr = (float *)(b + o_rr);
    L.first = (double *)(b + o_first);
    L.z0 = (float *)(b + o_z);
    L.sec = (float *)(b + o_sec);
    L.split = (float *)(b + o_split);
    L.split_cap = scap;
    L.bytes = off;
    return L;
}

// z0 = min(0, z - swl) (order 2/1) or z - swl (order 0), as float
// clamp: the seabed clamp of the wave_* calls (z below -depth evaluated at
// -depth), or 0 for the unclamped sums of cfdwm_irregular_fields
__global__ void k_prep_z(long n, const double *z, double swl, int order, int clamp, double depth, float *z0) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double zz = (clamp ? fmax(-depth, z[p]) : z[p]) - swl;
    z0[p] = (float)(order == 0 ? zz : fmin(0.0, zz));
}

// Irregular::eta/u/v/w/dp assembled from the pieces (Irregular.cpp:9-157).
// out has row stride ldo (the full batch length).
// With api.rows or api.kin set, the API rows and records are written here
// (the finishing pass folded in) instead of out.
__global__ void k_combine(long n, long ldo, int order, double swl, const double *z,
                          const double *first, const float *sec, const float *eta2, int mask,
                          double *out, ApiRows api) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double za = (order == 2) ? fmax(0.0, z[p] - swl) : 0.0;
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (mask & 1) v[0] = swl + first[0 * n + p] + (eta2 ? (double)eta2[p] : 0.0);
    if (mask & 2) v[1] = (double)sec[0 * n + p] + first[1 * n + p] * za;
    if (mask & 4) v[2] = (double)sec[1 * n + p] + first[2 * n + p] * za;
    if (mask & 8) v[3] = (double)sec[2 * n + p] + first[3 * n + p] * za;
    if (mask & 16) v[4] = (double)sec[3 * n + p] + first[4 * n + p] * za;
    if (!api.rows && !api.kin) {
        for (int q = 0; q < 5; q++)
            if (mask & (1 << q)) out[q * ldo + p] = v[q];
        return;
    }
    v[5] = v[4] - api.rho * api.g * v[0];
    if (api.ramp.init) {
        const double rr = d_ramp(api.ramp, api.t[p], api.x[p], api.y[p]);
        for (int q = 0; q < 6; q++) v[q] *= rr;
    }
    if (api.rows)
        for (int q = 0; q < 6; q++) api.rows[q * ldo + p] = v[q];
    if (api.kin)
        for (int q = 0; q < 4; q++) api.kin[4 * p + q] = v[q];
}

}  // namespace

static int launch_phasors(const DevSea &sea, long n, const double *x, const double *y,
                          const double *t, long sx, long sy, long st, int npad, float2 *ph,
                          float *rr, double *first, cudaStream_t stream) {
    PhArgs a;
    a.n = n; a.x = x; a.y = y; a.t = t; a.sx = sx; a.sy = sy; a.st = st;
    a.ncomp = sea.n; a.npad = npad; a.phase = sea.d_phase; a.cf = sea.d_cf;
    a.cstride = sea.npad_g; a.fx = sea.fx; a.fy = sea.fy;
    a.trivial_ramp = sea.trivial_ramp ? 1 : 0;
    a.ph = ph; a.rr = rr; a.first = first; a.rec = sea.d_phrec;
    if (!sea.d_phrec || npad > ((sea.npad_g + 255) / 256) * 256) return E_BAD_ARGUMENT;
    prof_begin(PK_PHASORS, stream);
    if (n <= PH_FEW_POINTS)
        k_phasors_few<<<(unsigned)n, 128, 0, stream>>>(a);
    else
        k_phasors<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(a);
    note_launch();
    prof_end(PK_PHASORS, stream);
    CK(cudaGetLastError());
    return OK;
}

int launch_phasors_public(const DevSea &sea, long n, const double *x, const double *y,
                          const double *t, long sx, long sy, long st, int npad, float2 *ph,
                          float *rr, double *first, cudaStream_t stream) {
    return launch_phasors(sea, n, x, y, t, sx, sy, st, npad, ph, rr, first, stream);
}

int launch_eta_pairs(const DevSea &sea, long n, const float2 *ph, const float *rr, float *out,
                     cudaStream_t stream, float *split_buf = nullptr, long split_cap = 0) {
    PairArgs a{};
    a.ncol = n; a.nl = 1; a.nlg = 1; a.ntile = sea.ntile_g; a.tab = sea.d_tab_eta;
    a.ph = ph; a.rr = rr; a.cf = sea.d_cf; a.cstride = sea.npad_g; a.out = out;
    a.pairs = 1; a.first = 0;
    const long nblk = (n + 127) / 128;
    const int ntp = sea.ntile_g * (sea.ntile_g + 1) / 2;
    const size_t smem = sizeof(float2) * (GRID_TILE * GRID_TILE + GRID_TILE * 128);
    // set once per process (thread-safe static initialisation)
    static const cudaError_t attr = cudaFuncSetAttribute(k_pairs_eta<GRID_TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
    CK(attr);
    static const long slots = [&] {
        const long v = resident_slots(k_pairs_eta<GRID_TILE>, 128, smem);
        return v > 0 ? v : SPLIT_TARGET_BLOCKS;
    }();
    // the tile-pair loop split over blockIdx.y where the columns alone do
    // not fill whole waves of the resident blocks (slices summed in order)
    int nslice = wave_slices(nblk, ntp, slots, split_buf ? split_cap / std::max<long>(1, n) : 1);
    a.tp_per = (ntp + nslice - 1) / nslice;
    nslice = (ntp + a.tp_per - 1) / a.tp_per;
    if (nslice > 1) a.out = split_buf;
    prof_begin(PK_ETA_PAIRS, stream);
    k_pairs_eta<GRID_TILE><<<dim3((unsigned)nblk, (unsigned)nslice), 128, smem, stream>>>(a);
    note_launch();
    prof_end(PK_ETA_PAIRS, stream);
    CK(cudaGetLastError());
    if (nslice > 1) {
        k_sum_slices<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, nslice, split_buf, out);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

long column_pairs_split_floats(int nl) {
    constexpr int LV = 8;
    int nlg = 1;
    while (nlg * LV < nl) nlg *= 2;
    long cols = 128 / nlg;
    return 4L * nl * cols * 2 * SPLIT_TARGET_BLOCKS;
}

template <bool PR>
static int column_pairs_t(const PairArgs &a, long nblk, int nslice, int cols, cudaStream_t stream) {
    constexpr int LV = 8;
    auto bytes = [](int c) {
        return sizeof(float) * GRID_TILE * GRID_TILE * GRIDV_NC + (PR ? sizeof(float2) * GRID_TILE * GRID_TILE : 0) +
               sizeof(float2) * GRID_TILE * c;
    };
    // set once per process (thread-safe static initialisation)
    static const cudaError_t attr = cudaFuncSetAttribute(k_pairs_columns<GRID_TILE, LV, PR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes(128));
    CK(attr);
    prof_begin(PK_COLUMN_PAIRS, stream);
    k_pairs_columns<GRID_TILE, LV, PR><<<dim3((unsigned)nblk, (unsigned)nslice), 128, bytes(cols), stream>>>(a);
    note_launch();
    prof_end(PK_COLUMN_PAIRS, stream);
    CK(cudaGetLastError());
    return OK;
}

// u, v, w (pressure: and p) sums of the columns at their levels, out [nf][ncol nl]
int launch_column_pairs(const DevSea &sea, long ncol, int nl, const float2 *ph, const float *rr,
                        const float *z0, float *out, int pairs, cudaStream_t stream, float *split_buf,
                        long split_cap, bool pressure) {
    constexpr int LV = 8;
    int nlg = 1;
    while (nlg * LV < nl) nlg *= 2;
    if (nlg > 16) return E_TOO_LARGE;
    if (pressure && !sea.d_tab_gp) return E_NOT_INITIALIZED;
    const int nf = pressure ? 4 : 3;
    PairArgs a{};
    a.ncol = ncol; a.nl = nl; a.nlg = nlg; a.ntile = sea.ntile_g; a.tab = sea.d_tab_grid;
    a.tabp = reinterpret_cast<const float2 *>(sea.d_tab_gp);
    a.ph = ph; a.rr = rr; a.cf = sea.d_cf; a.cstride = sea.npad_g; a.z0 = z0;
    a.depth = (float)sea.depth; a.out = out; a.pairs = pairs; a.first = 1;
    int cols = 128 / nlg;
    // Few columns (a small grid, a column sample): split the tile-pair loop
    // over blockIdx.y so that the launch still fills the GPU, and sum the
    // slices in a fixed order afterwards.
    const long nblk = (ncol + cols - 1) / cols;
    const int ntp = pairs ? sea.ntile_g * (sea.ntile_g + 1) / 2 : sea.ntile_g;
    int nslice = 1;
    a.tp_per = ntp;
    if (pairs && split_buf && nblk < SPLIT_TARGET_BLOCKS) {
        int want = (int)std::min<long>(ntp, (SPLIT_TARGET_BLOCKS + nblk - 1) / nblk);
        int per = (ntp + want - 1) / want;
        int ns = (ntp + per - 1) / per;
        if ((long)ns * nf * ncol * nl <= split_cap && ns > 1) {
            nslice = ns;
            a.tp_per = per;
            a.out = split_buf;
        }
    }
    int rc = pressure ? column_pairs_t<true>(a, nblk, nslice, cols, stream)
                      : column_pairs_t<false>(a, nblk, nslice, cols, stream);
    if (rc) return rc;
    if (nslice > 1) {
        long n = (long)nf * ncol * nl;
        k_sum_slices<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, nslice, split_buf, out);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

// ---------------------------------------------------------------------------
// Phase-free part of the s-grid pressure (uvw2, Irregular.cpp:1036-1037 and
// 1076-1077): at the evaluation height z0 in [-h, 0] and time t
//   K(z) = sum_pairs r_i [X px_i(z) px_m(z) + Z pz_i(z) pz_m(z)]
//        + sum_diag  r_i [X px_i(z) + Z pz_i(z)],
// px = cosh(k(z+h))/cosh(kh), pz = sinh(k(z+h))/cosh(kh), rho folded into X, Z.
// K does not depend on the column, so one ring step needs one table of K and
// dK/dz on nz uniform heights (read by cubic Hermite interpolation) instead
// of a second pass over the pairs per node.
// ---------------------------------------------------------------------------
struct KinArgs {
    const float2 *tabk;        // grid-mask pair tiles (X, Z)
    int ntile, ncomp, npad, trivial_ramp, zb;
    const double *phase;       // [7][npad]: ramp parameters in rows 4..6
    const float *cf;           // [NCF][npad]
    double t, depth, dz;
    int nz;
    double *kin;               // [nz][2]: K, dK/dz
};

constexpr int KIN_ZB = 4;      // heights per block (upper bound)

__global__ void __launch_bounds__(256) k_pressure_kin(KinArgs a) {
    extern __shared__ float smk[];
    const int np = a.npad, zb = a.zb;
    float *s_k = smk, *s_r = smk + np, *s_px = smk + 2 * np, *s_pz = s_px + (long)zb * np;
    const int j0 = blockIdx.x * zb;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        double k = 0.0, r = 0.0;
        if (i < a.ncomp) {
            k = a.cf[CF_K * np + i];
            const int ir = a.trivial_ramp ? 0 : i;
            r = d_freq_ramp(a.t, a.phase[4 * np + ir], a.phase[5 * np + ir], a.phase[6 * np + ir]);
        }
        s_k[i] = (float)k;
        s_r[i] = (float)r;
        for (int q = 0; q < zb; q++) {
            const double z = fmin(0.0, -a.depth + a.dz * min(j0 + q, a.nz - 1));
            // cosh(k(z+h))/cosh(kh) and sinh(k(z+h))/cosh(kh), both bounded by 1
            const double qn = 1.0 / (1.0 + exp(-2.0 * k * a.depth));
            const double E = exp(k * z), Y = exp(-k * (z + 2.0 * a.depth));
            s_px[q * np + i] = (float)(qn * (E + Y));
            s_pz[q * np + i] = (float)(qn * (E - Y));
        }
    }
    __syncthreads();
    float sK[KIN_ZB], cK[KIN_ZB], sD[KIN_ZB], cD[KIN_ZB];
#pragma unroll
    for (int q = 0; q < KIN_ZB; q++) sK[q] = cK[q] = sD[q] = cD[q] = 0.f;
    constexpr int TT = GRID_TILE;
    int I = 0, M = 0;
    const long ntiles = tile_index(a.ntile - 1, a.ntile - 1, a.ntile) + 1;
    for (long t = 0; t < ntiles; t++) {
        const float2 *tk = a.tabk + t * (long)TT * TT;
        for (int e = threadIdx.x; e < TT * TT; e += blockDim.x) {
            const float2 c = tk[e];
            if (c.x == 0.f && c.y == 0.f) continue;     // filtered pair or padding
            const int i = I * TT + e / TT, m = M * TT + e % TT;
            const float ri = s_r[i], ki = s_k[i], km = s_k[m];
#pragma unroll
            for (int q = 0; q < KIN_ZB; q++) {
                if (q >= zb) break;
                const float pxi = s_px[q * np + i], pzi = s_pz[q * np + i];
                float v, dv;
                if (i == m) {
                    v = c.x * pxi + c.y * pzi;
                    dv = ki * (c.x * pzi + c.y * pxi);
                } else {
                    const float pxm = s_px[q * np + m], pzm = s_pz[q * np + m];
                    v = c.x * pxi * pxm + c.y * pzi * pzm;
                    dv = c.x * (ki * pzi * pxm + km * pxi * pzm) + c.y * (ki * pxi * pzm + km * pzi * pxm);
                }
                kahan(sK[q], cK[q], ri * v);
                kahan(sD[q], cD[q], ri * dv);
            }
        }
        if (++M == a.ntile) { ++I; M = I; }
    }
    // block reduction in FP64, in a fixed order
    __shared__ double red[2][256];
    for (int q = 0; q < zb; q++) {
        __syncthreads();
        red[0][threadIdx.x] = (double)sK[q] - (double)cK[q];
        red[1][threadIdx.x] = (double)sD[q] - (double)cD[q];
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                red[0][threadIdx.x] += red[0][threadIdx.x + w];
                red[1][threadIdx.x] += red[1][threadIdx.x + w];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0 && j0 + q < a.nz) {
            a.kin[2 * (j0 + q)] = red[0][0];
            a.kin[2 * (j0 + q) + 1] = red[1][0];
        }
    }
}

int launch_pressure_kin(const DevSea &sea, double t, int nz, double *kin, cudaStream_t stream) {
    if (!sea.d_tab_gk || nz < 2) return E_NOT_INITIALIZED;
    const int np = sea.npad_g;
    // shared memory: k, ramp and zb rows of px, pz per component
    const size_t cap = 200 * 1024;
    int zb = KIN_ZB;
    while (zb > 1 && sizeof(float) * (size_t)np * (2 + 2 * zb) > cap) zb--;
    const size_t smem = sizeof(float) * (size_t)np * (2 + 2 * zb);
    if (smem > cap) return E_TOO_LARGE;
    // set once per process (thread-safe static initialisation)
    static const cudaError_t attr = cudaFuncSetAttribute(k_pressure_kin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    CK(attr);
    KinArgs a;
    a.tabk = reinterpret_cast<const float2 *>(sea.d_tab_gk);
    a.ntile = sea.ntile_g; a.ncomp = sea.n; a.npad = np; a.trivial_ramp = sea.trivial_ramp ? 1 : 0; a.zb = zb;
    a.phase = sea.d_phase; a.cf = sea.d_cf;
    a.t = t; a.depth = sea.depth; a.dz = sea.depth / (nz - 1); a.nz = nz; a.kin = kin;
    k_pressure_kin<<<(unsigned)((nz + zb - 1) / zb), 256, smem, stream>>>(a);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

static int launch_point_pairs(const DevSea &sea, long n, const float2 *ph, const float *rr,
                              const float *z0, float *out, int pairs, int mask, cudaStream_t stream,
                              float *split_buf, long split_cap) {
    PairArgs a{};
    a.ncol = n; a.nl = 1; a.nlg = 1; a.ntile = sea.ntile_p; a.tab = sea.d_tab_point;
    a.ph = ph; a.rr = rr; a.cf = sea.d_cf; a.cstride = sea.npad_g; a.z0 = z0;
    a.depth = (float)sea.depth; a.out = out; a.pairs = pairs; a.first = 1;
    // few points: the tile-pair loop split over blockIdx.y, slices summed in order
    const int ntp = pairs ? sea.ntile_p * (sea.ntile_p + 1) / 2 : sea.ntile_p;
    if (n <= FEW_POINTS && split_buf) {
        // a block per (point, slice), the rows of 8 tile pairs over its threads
        constexpr int PER = 128 / POINT_TILE;
        const int npass = (ntp + PER - 1) / PER;
        int nslice = (int)std::min<long>(npass, std::max<long>(1, split_cap / (4L * n)));
        nslice = std::min(nslice, 65535);
        a.out = split_buf;
        prof_begin(PK_POINT_PAIRS, stream);
        k_pairs_points_few<POINT_TILE><<<dim3((unsigned)n, (unsigned)nslice), 128, 0, stream>>>(a, ntp, nslice);
        note_launch();
        prof_end(PK_POINT_PAIRS, stream);
        CK(cudaGetLastError());
        k_sum_slices<<<(unsigned)((4 * n + 255) / 256), 256, 0, stream>>>(4 * n, nslice, split_buf, out);
        note_launch();
        CK(cudaGetLastError());
        return OK;
    }
    const size_t smem = sizeof(float) * POINT_TILE * POINT_TILE * POINTV_NC + 2 * sizeof(float2) * POINT_TILE * 128;
    // the same shared memory in every variant: resident blocks once per process
    static const long slots = [&] {
        cudaFuncSetAttribute(k_pairs_points<POINT_TILE, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        const long v = resident_slots(k_pairs_points<POINT_TILE, true, true>, 128, smem);
        return v > 0 ? v : SPLIT_TARGET_BLOCKS;
    }();
    const long nblk = (n + 127) / 128;
    int nslice = wave_slices(nblk, ntp, slots, split_buf ? split_cap / (4L * n) : 1);
    a.tp_per = (ntp + nslice - 1) / nslice;
    nslice = (ntp + a.tp_per - 1) / a.tp_per;
    if (nslice > 1) a.out = split_buf;
    // set once per process (thread-safe static initialisation)
    static const cudaError_t attr = [&] {
        cudaError_t e = cudaFuncSetAttribute(k_pairs_points<POINT_TILE, true, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_pairs_points<POINT_TILE, true, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_pairs_points<POINT_TILE, false, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e;
    }();
    CK(attr);
    // the velocity sums only where u, v or w is asked for, the pressure sums
    // only where dp is
    const bool vel = (mask & 14) != 0, pr = (mask & 16) != 0;
    const dim3 grid((unsigned)((n + 127) / 128), (unsigned)nslice);
    prof_begin(PK_POINT_PAIRS, stream);
    if (vel && pr)
        k_pairs_points<POINT_TILE, true, true><<<grid, 128, smem, stream>>>(a);
    else if (vel)
        k_pairs_points<POINT_TILE, true, false><<<grid, 128, smem, stream>>>(a);
    else
        k_pairs_points<POINT_TILE, false, true><<<grid, 128, smem, stream>>>(a);
    note_launch();
    prof_end(PK_POINT_PAIRS, stream);
    CK(cudaGetLastError());
    if (nslice > 1) {
        k_sum_slices<<<(unsigned)((4 * n + 255) / 256), 256, 0, stream>>>(4 * n, nslice, split_buf, out);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

// Phasor layout used by the pair kernels: the point kernel reads tiles of
// POINT_TILE, the grid kernels tiles of GRID_TILE; the workspace is sized for
// npad_g >= npad_p so both fit.
int irregular_eval(const DevSea &sea, long n, const double *x, const double *y, const double *z,
                   const double *t, int mask, double *out, Workspace &ws, void *stream_, const ApiRows *api) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (n <= 0) return OK;
    const long chunk = 1L << 18;
    const int npad = sea.npad_g;
    WsLayout L0 = layout(std::min(n, chunk), npad, nullptr);
    int rc = workspace_reserve(ws, L0.bytes);
    if (rc) return rc;
    for (long b = 0; b < n; b += chunk) {
        long m = std::min(chunk, n - b);
        WsLayout L = layout(m, npad, ws.base);
        rc = launch_phasors(sea, m, x + b, y + b, t + b, 1, 1, 1, npad, L.ph, L.rr, L.first, stream);
        if (rc) return rc;
        // vertical_theory smit: u, v, w, dp need eta at the point first
        const bool smit = sea.smit && (mask & 30);
        float *eta2 = nullptr;
        if (((mask & 1) || smit) && sea.order == 2) {
            eta2 = L.sec + 4 * m;
            rc = launch_eta_pairs(sea, m, L.ph, L.rr, eta2, stream, L.split, L.split_cap);
            if (rc) return rc;
        }
        if (smit) {
            rc = smit_eval(sea, m, z + b, L.ph, L.rr, L.first, eta2, L.sec, L.split, L.split_cap, n, out + b,
                           mask, stream);
            if (rc) return rc;
        } else if (mask & 30) {
            k_prep_z<<<(unsigned)((m + 255) / 256), 256, 0, stream>>>(m, z + b, sea.swl, sea.order, api ? 1 : 0,
                                                                  sea.depth, L.z0);
            note_launch();
            CK(cudaGetLastError());
            // the point table is padded to POINT_TILE; the phasor rows beyond
            // npad_p are never read by the point kernel
            rc = launch_point_pairs(sea, m, L.ph, L.rr, L.z0, L.sec, sea.order != 0 ? 1 : 0, mask, stream,
                                    L.split, L.split_cap);
            if (rc) return rc;
        }
        ApiRows ar{};
        if (api && !smit) {
            ar = *api;
            ar.x = api->x + b; ar.y = api->y + b; ar.t = api->t + b;
            ar.rows = api->rows ? api->rows + b : nullptr;
            ar.kin = api->kin ? api->kin + 4 * b : nullptr;
        }
        k_combine<<<(unsigned)((m + 255) / 256), 256, 0, stream>>>(m, n, sea.order, sea.swl, z + b,
                                                                   L.first, L.sec, eta2, smit ? (mask & 1) : mask,
                                                                   out ? out + b : nullptr, ar);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

size_t irregular_eval_scratch_bytes(const DevSea &sea, long n) {
    const long chunk = 1L << 18;
    return layout(std::min(n, chunk), sea.npad_g, nullptr).bytes;
}

}  // namespace cfdwm
