// Smit et al. (2017) s-coordinate second-order kinematics on the GPU
// (vertical_theory smit, the reference's experimental theory).
//
// What is computed follows oystelan/CFDwavemaker v3.1.0 src/Irregular.cpp:
//   u_smit :1622-1771, v_smit :1773-1850, w_smit :1852-1927, dp_smit :1929-2027,
//   the pair cache's H coefficients :924-930, 951-958 (Eq. 10 inverted with the
//   Sharma-Dean alpha), the Wheeler-stretched profiles :121-138.
// At a point below the surface, with eta = eta1 + eta2 there and
// sf = h (h + z) / (h + eta), every profile is the ordinary one at the
// stretched height z* = sf - h in [-h, 0]:
//   cosh(k sf)/cosh(kh) = q(k) (e^{k z*} + e^{-k(z* + 2h)}),
// so the sums have the shape of the Sharma-Dean point sums (one thread per
// point, pair tiles in shared memory, two ex2 per wavenumber) with Smit's
// terms per pair: the bound wave H (u, v, w, p), the particular-solution
// velocity and its s-derivative (u), the Bernoulli products (p), and the
// Lagrangian-to-Eulerian chain term of u from first-order sums.
// Ramps enter as r_i r_m per pair (the theory's AA), and every diagonal term
// is kept (its loops have no filter); the pairs are those of the pair cache.
#include "cfdwm.h"

#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>

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

namespace {

constexpr int ST = SMIT_TILE;     // components per tile side
constexpr int SNC = 16;           // floats per pair record
constexpr float L2E = 1.4426950408889634f;

__device__ __forceinline__ float sx2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void skahan(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}
__host__ __device__ inline long stile(int I, int M, int nt) { return (long)I * nt - (long)I * (I - 1) / 2 + (M - I); }

// e^{kz} (1 +- e^{-2k(z+h)}): the profiles with the normaliser left out
__device__ __forceinline__ void sfg(float k, float zk, float zetak, float &F, float &G) {
    const float e1 = sx2(k * zk), e2 = sx2(k * zetak);
    F = fmaf(e1, e2, e1);       // e1 (1 + e2), one rounding
    G = fmaf(-e1, e2, e1);      // e1 (1 - e2)
}

// Eq. 10 inverted for H with the Sharma-Dean alpha (Irregular.cpp:926-929, 954-957)
__device__ __forceinline__ double smit_h(double g, double om12, double oi, double om, double alpha, double k1dk2,
                                         double sgn) {
    return -g / om12 * (alpha / 2.0 - (oi * oi + om * om + sgn * oi * om) / (2.0 * g) + g * k1dk2 / (2.0 * oi * om));
}

__device__ __forceinline__ double k2_rounded(double ki, double km, double gam) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ki, ki), __dmul_rn(km, km)), __dmul_rn(__dmul_rn(2.0 * ki, km), gam));
}

// One record per (tile, entry) of the upper triangle, FP64 -> FP32:
//  0 Hp q+ A_i A_m      1 Hm q- A_i A_m       (diagonal: 0.5 A^2 H q(2k))
//  2 k+                 3 k-
//  4 kx+  5 kx-  6 ky+  7 ky-                 (k_i cos th_i +- k_m cos th_m, ...)
//  8 rho (w_i + w_m)    9 rho (w_i - w_m)
// 10 -rho g^2 k_i.k_m / (w_i w_m) A_i A_m [+]  11 the same [-]   (diagonal: 0.5 A^2 ...)
// 12 g kx+ A_i A_m     13 g kx- A_i A_m      (diagonal: 0.25 A^2 g 2k cos th)
// 14 g A_i A_m [+]     15 g A_i A_m [-]      (diagonal: 0.25 A^2 g)
__global__ void k_build_smit(SmitIn c, int nt, float *tab) {
    const long t = blockIdx.x;
    int I = 0;
    while (stile(I, nt - 1, nt) < t) I++;
    const int M = (int)(t - stile(I, I, nt)) + I;
    const double h = c.depth, g = c.g, gg = g * g, rho = c.rho;
    for (int e = threadIdx.x; e < ST * ST; e += blockDim.x) {
        const int i = I * ST + e / ST, m = M * ST + e % ST;
        double r[SNC];
        for (int q = 0; q < SNC; q++) r[q] = 0.0;
        if (i < c.n && m < c.n && i <= m) {
            const double ki = c.k[i], oi = c.omega[i], Ai = c.A[i];
            const double thi = c.theta[i] + c.mtheta_rad, cti = cos(thi), sti = sin(thi);
            const double Rn = ki * tanh(ki * h), Rsn = sqrt(Rn);
            if (i == m) {
                const double Dnn = (6.0 * Rsn * Rsn * (ki * ki - Rn * Rn)) / (2.0 * Rsn * Rsn - ki * tanh(2.0 * ki * h));
                const double ann = (Dnn - (ki * ki - Rn * Rn)) / Rn + 2.0 * Rn;
                const double om2 = 2.0 * oi;
                const double H = -g / om2 * (ann / 2.0 - (3.0 * oi * oi) / (2.0 * g) + g * ki * ki / (2.0 * oi * oi));
                const double q2 = 1.0 / (1.0 + exp(-4.0 * ki * h));
                const double a2 = Ai * Ai;
                r[0] = 0.5 * a2 * H * q2;
                r[2] = 2.0 * ki;
                r[4] = 2.0 * ki * cti;
                r[6] = 2.0 * ki * sti;
                r[8] = rho * om2;
                r[10] = -0.5 * a2 * rho * gg * ki * ki / (oi * oi);
                r[12] = 0.25 * a2 * g * 2.0 * ki * cti;
                r[14] = 0.25 * a2 * g;
            } else {
                const double km = c.k[m], om = c.omega[m], Am = c.A[m];
                const double thm = c.theta[m] + c.mtheta_rad, ctm = cos(thm), stm = sin(thm);
                const double Rm = km * tanh(km * h), Rsm = sqrt(Rm);
                const bool keep = (oi <= c.cutoff) && (om <= c.cutoff) && (fabs(oi - om) <= c.bandwidth);
                const bool hp = keep && (ki + km) <= c.kmax, hm = keep && (ki != km);
                const double gam = __dadd_rn(__dmul_rn(cti, ctm), __dmul_rn(sti, stm));   // Irregular.cpp:869-871
                const double k1dk2 = ki * km * gam;
                const double AA = Ai * Am;
                const double sp = Rsn + Rsm, sm = Rsn - Rsm, R2p = sp * sp, R2m = sm * sm;
                r[4] = ki * cti + km * ctm;
                r[5] = ki * cti - km * ctm;
                r[6] = ki * sti + km * stm;
                r[7] = ki * sti - km * stm;
                r[8] = rho * (oi + om);
                r[9] = rho * (oi - om);
                if (hp) {
                    const double kp = sqrt(fmax(0.0, k2_rounded(ki, km, gam)));
                    const double den = R2p - kp * tanh(kp * h);
                    const double Dp = (2.0 * R2p * (ki * km * gam - Rn * Rm)) / den +
                                      (sp * (Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
                    const double ap = (Dp - (ki * km * gam - Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
                    const double H = smit_h(g, oi + om, oi, om, ap, k1dk2, 1.0);
                    r[0] = AA * H / (1.0 + exp(-2.0 * kp * h));
                    r[2] = kp;
                    r[10] = -AA * rho * gg * k1dk2 / (oi * om);
                    r[12] = AA * g * r[4];
                    r[14] = AA * g;
                }
                if (hm) {
                    const double kq = sqrt(fmax(0.0, k2_rounded(ki, km, -gam)));
                    const double den = R2m - kq * tanh(kq * h);
                    const double Dm = (2.0 * R2m * (ki * km * gam + Rn * Rm)) / den +
                                      (sm * (-Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
                    const double am = (Dm - (ki * km * gam + Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
                    const double om12 = oi - om;
                    const double H = fabs(om12) > SMALL ? smit_h(g, om12, oi, om, am, k1dk2, -1.0) : 0.0;
                    r[1] = AA * H / (1.0 + exp(-2.0 * kq * h));
                    r[3] = kq;
                    r[11] = -AA * rho * gg * k1dk2 / (oi * om);
                    r[13] = AA * g * r[5];
                    r[15] = AA * g;
                }
            }
        }
        float *o = tab + (t * ST * ST + e) * SNC;
        for (int q = 0; q < SNC; q++) o[q] = (float)r[q];
    }
}

// Per point: eta = eta1 + eta2; zero output above eta + swl; the stretched
// height z*, (1 + s) = (h + z)/(h + eta) and the chain factor -(h + z)/(h + eta)^2.
__global__ void k_smit_prep(long n, const double *z, const double *first, const float *eta2, double depth, double swl,
                            float *zs, float *sp1, float *chain, float *above) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double eta = first[p] + (double)eta2[p];
    const double zz = fmax(-depth, z[p] - swl);
    const double D = depth + eta;
    above[p] = (z[p] > eta + swl) ? 1.f : 0.f;
    zs[p] = (float)(depth * (depth + zz) / D - depth);
    sp1[p] = (float)((depth + zz) / D);
    chain[p] = (float)(-(depth + zz) / (D * D));
}

struct SmitArgs {
    long n;
    int ntile, cstride;
    const float *tab;
    const float2 *ph;          // [npad][n] phasors of the point phases
    const float *rr;           // [npad][n] ramps
    const float *cf;           // [NCF][cstride]
    const double *phase;       // [7][cstride]: omega in row 2
    const float *zs, *sp1, *chain, *above;
    float depth;
    int tp_per;                // tile pairs per blockIdx.y
    float *part;               // [slices][7][n] partial sums (split launches), or null
    long ldo;
    double *out;               // rows 1..4: u, v, w, dp
};

constexpr int SMIT_PARTS = 7;  // u, v, w, dp, d phi2/ds, eta_x, d phi1/ds
// batches of at most this many points take k_smit_points_few
constexpr long SMIT_FEW_POINTS = 512;

// VEL: the velocity sums (u with its chain term, v, w), PR: the pressure sum;
// a call that asks for one of them does not pay for the other (rows not
// computed are 0).
template <int TT, bool VEL, bool PR>
__global__ void __launch_bounds__(128) k_smit_points(SmitArgs a) {
    extern __shared__ float4 smem4[];
    float *s_tab = reinterpret_cast<float *>(smem4);                  // TT*TT*SNC
    float2 *s_ph = reinterpret_cast<float2 *>(s_tab + TT * TT * SNC); // TT*128: phasors of the m tile
    float2 *s_pf = s_ph + TT * 128;                                   // TT*128: Ch_m, Sh_m
    float *s_r = reinterpret_cast<float *>(s_pf + TT * 128);          // TT*128: ramps
    __shared__ float s_k[TT], s_a[TT];                                // k_m, k_m / w_m
    const long p = (long)blockIdx.x * 128 + threadIdx.x;
    const bool valid = p < a.n;
    const long pc = valid ? p : 0;
    const float h = a.depth;
    const float zs = a.zs[pc], sp1 = a.sp1[pc];
    const float zk = zs * L2E, zetak = -2.f * (zs + h) * L2E;
    float su = 0, cu = 0, sv = 0, cv = 0, sw = 0, cw = 0, sq = 0, cq = 0, sd = 0, cd = 0;
    float ex = 0, cex = 0, ps = 0, cps = 0;   // first-order eta_x and d phi1 / ds of the chain term
    const int tp_lo = blockIdx.y * a.tp_per, tp_hi = tp_lo + a.tp_per;   // this block's tile pairs
    int tp = -1;
    for (int I = 0; I < a.ntile; I++) {
        for (int M = I; M < a.ntile; M++) {
            tp++;
            if (tp < tp_lo || tp >= tp_hi) continue;      // block-uniform
            __syncthreads();
            {
                const float4 *src = reinterpret_cast<const float4 *>(a.tab + stile(I, M, a.ntile) * (long)TT * TT * SNC);
                float4 *dst = reinterpret_cast<float4 *>(s_tab);
                for (int e = threadIdx.x; e < TT * TT * SNC / 4; e += blockDim.x) dst[e] = src[e];
            }
            if (threadIdx.x < TT) {
                const int m = M * TT + threadIdx.x;
                s_k[threadIdx.x] = a.cf[CF_K * a.cstride + m];
                s_a[threadIdx.x] = a.cf[CF_KW * a.cstride + m];
            }
            for (int mm = 0; mm < TT; mm++) {
                const int m = M * TT + mm;
                float F, G;
                sfg(a.cf[CF_K * a.cstride + m], zk, zetak, F, G);
                const float q = a.cf[CF_Q * a.cstride + m];
                s_ph[mm * 128 + threadIdx.x] = a.ph[(long)m * a.n + pc];
                s_pf[mm * 128 + threadIdx.x] = make_float2(q * F, q * G);
                s_r[mm * 128 + threadIdx.x] = a.rr[(long)m * a.n + pc];
            }
            __syncthreads();
            if (!valid) continue;
            for (int ii = 0; ii < TT; ii++) {
                const int i = I * TT + ii;
                const float2 pi = a.ph[(long)i * a.n + p];
                const float ri = a.rr[(long)i * a.n + p];
                float2 pfi;
                if (M == I) {
                    pfi = s_pf[ii * 128 + threadIdx.x];
                } else {
                    float F, G;
                    sfg(a.cf[CF_K * a.cstride + i], zk, zetak, F, G);
                    const float q = a.cf[CF_Q * a.cstride + i];
                    pfi = make_float2(q * F, q * G);
                }
                // k_i / omega_i from the coefficient rows: an FP64 division here,
                // per (point, component, tile pair), kept the FP64 pipe 31% busy
                const float ki = a.cf[CF_K * a.cstride + i];
                const float ai = a.cf[CF_KW * a.cstride + i];
                const float A1 = ai * pfi.y, B1 = ai * ki * h * pfi.x;
                float au = 0, av = 0, aw = 0, ap = 0, ad = 0;
                const int m0 = (M == I) ? ii : 0;
                for (int mm = m0; mm < TT; mm++) {
                    const float *rec = s_tab + (ii * TT + mm) * SNC;
                    const float4 c0 = *reinterpret_cast<const float4 *>(rec);
                    const float4 c1 = *reinterpret_cast<const float4 *>(rec + 4);
                    const float4 c2 = *reinterpret_cast<const float4 *>(rec + 8);
                    const float4 c3 = *reinterpret_cast<const float4 *>(rec + 12);
                    const float2 pm = s_ph[mm * 128 + threadIdx.x];
                    const float2 pfm = s_pf[mm * 128 + threadIdx.x];
                    const float rm = s_r[mm * 128 + threadIdx.x];
                    const float cc = pi.x * pm.x, ss = pi.y * pm.y, sc = pi.y * pm.x, cs = pi.x * pm.y;
                    const float cp = cc - ss, cmn = cc + ss, sp = sc + cs, smn = sc - cs;
                    float Fp, Gp, Fm, Gm;
                    sfg(c0.z, zk, zetak, Fp, Gp);
                    sfg(c0.w, zk, zetak, Fm, Gm);
                    const float hpc = -c0.x * cp * Fp, hmc = -c0.y * cmn * Fm;   // bound wave, cos part
                    if (VEL) {
                        const float A2 = s_a[mm] * pfm.y, B2 = s_a[mm] * s_k[mm] * h * pfm.x;
                        const float hps = c0.x * c0.z * Gp, hms = c0.y * c0.w * Gm;  // bound wave, k Sh part
                        float tu = c1.x * hpc + c1.y * hmc + sp1 * (c3.x * (A1 + A2) * cp + c3.y * (A1 - A2) * cmn);
                        float tv = c1.z * hpc + c1.w * hmc;
                        float tw = -(hps * sp + hms * smn);
                        float td = -h * (hps * sp + hms * smn) + c3.z * ((A1 + A2) + sp1 * (B1 + B2)) * sp +
                                   c3.w * ((A1 - A2) + sp1 * (B1 - B2)) * smn;
                        au = fmaf(rm, tu, au);
                        av = fmaf(rm, tv, av);
                        aw = fmaf(rm, tw, aw);
                        ad = fmaf(rm, td, ad);
                    }
                    if (PR) {
                        const float chch = pfi.x * pfm.x, shsh = pfi.y * pfm.y;
                        float tp = c2.x * hpc + c2.y * hmc + c2.z * (chch - shsh) * cp + c2.w * (chch + shsh) * cmn;
                        ap = fmaf(rm, tp, ap);
                    }
                }
                if (VEL) {
                    skahan(su, cu, ri * au);
                    skahan(sv, cv, ri * av);
                    skahan(sw, cw, ri * aw);
                    skahan(sd, cd, ri * ad);
                }
                if (PR) skahan(sq, cq, ri * ap);
            }
            if (M == I) {
                // first order with the stretched profiles and the first-order
                // sums of the chain term (Irregular.cpp:1638-1645, 1750-1760)
                for (int mm = 0; mm < TT; mm++) {
                    const int m = M * TT + mm;
                    const float2 pm = s_ph[mm * 128 + threadIdx.x];
                    const float2 pfm = s_pf[mm * 128 + threadIdx.x];
                    const float rm = s_r[mm * 128 + threadIdx.x];
                    if (VEL) {
                        const float agk = a.cf[CF_AU * a.cstride + m] * rm;     // A g k / w
                        const float ct = a.cf[CF_CT * a.cstride + m];
                        skahan(su, cu, agk * pfm.x * ct * pm.x);
                        skahan(sv, cv, agk * pfm.x * a.cf[CF_ST * a.cstride + m] * pm.x);
                        skahan(sw, cw, agk * pfm.y * pm.y);
                        skahan(ex, cex, -a.cf[CF_A * a.cstride + m] * s_k[mm] * ct * pm.y * rm);
                        skahan(ps, cps, agk * h * pfm.y * pm.y);
                    }
                    if (PR) skahan(sq, cq, a.cf[CF_AP * a.cstride + m] * rm * pfm.x * pm.x);
                }
            }
        }
    }
    if (!valid) return;
    if (a.part) {
        float *o = a.part + (long)blockIdx.y * SMIT_PARTS * a.n + p;
        const float v[SMIT_PARTS] = {su - cu, sv - cv, sw - cw, sq - cq, sd - cd, ex - cex, ps - cps};
        for (int q = 0; q < SMIT_PARTS; q++) o[(long)q * a.n] = v[q];
        return;
    }
    const bool up = a.above[p] != 0.f;
    const double chain = (double)a.chain[p] * ((double)ex - cex) * (((double)ps - cps) + ((double)sd - cd));
    a.out[1 * a.ldo + p] = up ? 0.0 : ((double)su - cu) + chain;
    a.out[2 * a.ldo + p] = up ? 0.0 : (double)sv - cv;
    a.out[3 * a.ldo + p] = up ? 0.0 : (double)sw - cw;
    a.out[4 * a.ldo + p] = up ? 0.0 : (double)sq - cq;
}

// Few points (a scalar call, a short batch): block (point p, slice y), thread
// t takes row ii = t % TT of tile pair 8 g + t / TT for g = y, y + nslice, ...
// (TT = 16).  A row is the inner loop of k_smit_points for one point, with the
// m tile's depth factors, phasors and ramps read per term (no other point
// shares them); diagonal tile pairs add the first-order terms of component
// I TT + ii.  Each thread's rows are Kahan-summed, the block's 128 sums added
// in FP32 into slice y's seven partial sums, and k_smit_finish adds the
// slices in order and forms the chain term.
template <int TT>
__global__ void __launch_bounds__(128) k_smit_points_few(SmitArgs a, int ntp, int nslice) {
    __shared__ float s_red[4][SMIT_PARTS];
    const long p = blockIdx.x;
    const float h = a.depth;
    const float zs = a.zs[p], sp1 = a.sp1[p];
    const float zk = zs * L2E, zetak = -2.f * (zs + h) * L2E;
    const int ii = threadIdx.x % TT;
    constexpr int PER = 128 / TT;
    float su = 0, cu = 0, sv = 0, cv = 0, sw = 0, cw = 0, sq = 0, cq = 0, sd = 0, cd = 0;
    float ex = 0, cex = 0, ps = 0, cps = 0;
    for (int g = blockIdx.y; g * PER < ntp; g += nslice) {
        int tp = g * PER + threadIdx.x / TT;
        if (tp >= ntp) continue;
        int I = 0;
        while (tp >= a.ntile - I) { tp -= a.ntile - I; I++; }
        const int M = I + tp;
        const int i = I * TT + ii;
        const float2 pi = a.ph[(long)i * a.n + p];
        const float ri = a.rr[(long)i * a.n + p];
        float F, G;
        sfg(a.cf[CF_K * a.cstride + i], zk, zetak, F, G);
        const float qi = a.cf[CF_Q * a.cstride + i];
        const float2 pfi = make_float2(qi * F, qi * G);
        const float ki = a.cf[CF_K * a.cstride + i];
        const float ai = a.cf[CF_KW * a.cstride + i];
        const float A1 = ai * pfi.y, B1 = ai * ki * h * pfi.x;
        const float *T = a.tab + stile(I, M, a.ntile) * (long)TT * TT * SNC;
        float au = 0, av = 0, aw = 0, ap = 0, ad = 0;
        for (int mm = (M == I) ? ii : 0; mm < TT; mm++) {
            const int m = M * TT + mm;
            const float *rec = T + (ii * TT + mm) * SNC;
            const float4 c0 = *reinterpret_cast<const float4 *>(rec);
            const float4 c1 = *reinterpret_cast<const float4 *>(rec + 4);
            const float4 c2 = *reinterpret_cast<const float4 *>(rec + 8);
            const float4 c3 = *reinterpret_cast<const float4 *>(rec + 12);
            const float2 pm = a.ph[(long)m * a.n + p];
            const float rm = a.rr[(long)m * a.n + p];
            const float km = a.cf[CF_K * a.cstride + m], am = a.cf[CF_KW * a.cstride + m];
            float Fm_, Gm_;
            sfg(km, zk, zetak, Fm_, Gm_);
            const float qm = a.cf[CF_Q * a.cstride + m];
            const float2 pfm = make_float2(qm * Fm_, qm * Gm_);
            const float cc = pi.x * pm.x, ss = pi.y * pm.y, sc = pi.y * pm.x, cs = pi.x * pm.y;
            const float cp = cc - ss, cmn = cc + ss, sp = sc + cs, smn = sc - cs;
            float Fp, Gp, Fm, Gm;
            sfg(c0.z, zk, zetak, Fp, Gp);
            sfg(c0.w, zk, zetak, Fm, Gm);
            const float A2 = am * pfm.y, B2 = am * km * h * pfm.x;
            const float hpc = -c0.x * cp * Fp, hmc = -c0.y * cmn * Fm;
            const float hps = c0.x * c0.z * Gp, hms = c0.y * c0.w * Gm;
            float tu = c1.x * hpc + c1.y * hmc + sp1 * (c3.x * (A1 + A2) * cp + c3.y * (A1 - A2) * cmn);
            float tv = c1.z * hpc + c1.w * hmc;
            float tw = -(hps * sp + hms * smn);
            const float chch = pfi.x * pfm.x, shsh = pfi.y * pfm.y;
            float tq = c2.x * hpc + c2.y * hmc + c2.z * (chch - shsh) * cp + c2.w * (chch + shsh) * cmn;
            float td = -h * (hps * sp + hms * smn) + c3.z * ((A1 + A2) + sp1 * (B1 + B2)) * sp +
                       c3.w * ((A1 - A2) + sp1 * (B1 - B2)) * smn;
            au = fmaf(rm, tu, au);
            av = fmaf(rm, tv, av);
            aw = fmaf(rm, tw, aw);
            ap = fmaf(rm, tq, ap);
            ad = fmaf(rm, td, ad);
        }
        skahan(su, cu, ri * au);
        skahan(sv, cv, ri * av);
        skahan(sw, cw, ri * aw);
        skahan(sq, cq, ri * ap);
        skahan(sd, cd, ri * ad);
        if (M == I) {
            // first order of component i with the stretched profiles and the
            // first-order sums of the chain term (Irregular.cpp:1638-1645, 1750-1760)
            const float agk = a.cf[CF_AU * a.cstride + i] * ri;
            const float ct = a.cf[CF_CT * a.cstride + i];
            skahan(su, cu, agk * pfi.x * ct * pi.x);
            skahan(sv, cv, agk * pfi.x * a.cf[CF_ST * a.cstride + i] * pi.x);
            skahan(sw, cw, agk * pfi.y * pi.y);
            skahan(sq, cq, a.cf[CF_AP * a.cstride + i] * ri * pfi.x * pi.x);
            skahan(ex, cex, -a.cf[CF_A * a.cstride + i] * ki * ct * pi.y * ri);
            skahan(ps, cps, agk * h * pfi.y * pi.y);
        }
    }
    float v[SMIT_PARTS] = {su - cu, sv - cv, sw - cw, sq - cq, sd - cd, ex - cex, ps - cps};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int f = 0; f < SMIT_PARTS; f++) {
        for (int o = 16; o > 0; o >>= 1) v[f] += __shfl_down_sync(0xffffffffu, v[f], o);
        if (lane == 0) s_red[warp][f] = v[f];
    }
    __syncthreads();
    if (threadIdx.x < SMIT_PARTS) {
        const int f = threadIdx.x;
        a.part[((long)blockIdx.y * SMIT_PARTS + f) * a.n + p] = ((s_red[0][f] + s_red[1][f]) + s_red[2][f]) + s_red[3][f];
    }
}

// The slices of a split launch summed in order, then the chain term.
__global__ void k_smit_finish(long n, int nslice, const float *part, const float *chain, const float *above,
                              long ldo, double *out) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double v[SMIT_PARTS];
    for (int q = 0; q < SMIT_PARTS; q++) {
        float s = 0.f, c = 0.f;
        for (int k = 0; k < nslice; k++) skahan(s, c, part[((long)k * SMIT_PARTS + q) * n + p]);
        v[q] = (double)s - c;
    }
    const bool up = above[p] != 0.f;
    out[1 * ldo + p] = up ? 0.0 : v[0] + (double)chain[p] * v[5] * (v[6] + v[4]);
    out[2 * ldo + p] = up ? 0.0 : v[1];
    out[3 * ldo + p] = up ? 0.0 : v[2];
    out[4 * ldo + p] = up ? 0.0 : v[3];
}

}  // namespace

int smit_build(const SmitIn &c, DevSea &sea, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (sea.d_tab_smit) cudaFree(sea.d_tab_smit);
    sea.d_tab_smit = nullptr;
    sea.npad_s = ((c.n + ST - 1) / ST) * ST;
    if (sea.npad_s == 0) sea.npad_s = ST;
    sea.ntile_s = sea.npad_s / ST;
    if (sea.npad_s > sea.npad_g) return E_BAD_ARGUMENT;
    const long ntiles = stile(sea.ntile_s - 1, sea.ntile_s - 1, sea.ntile_s) + 1;
    CK(cudaMalloc(&sea.d_tab_smit, sizeof(float) * (size_t)ntiles * ST * ST * SNC));
    k_build_smit<<<(unsigned)ntiles, 256, 0, stream>>>(c, sea.ntile_s, sea.d_tab_smit);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

int smit_eval(const DevSea &sea, long n, const double *z, const void *ph, const float *rr, const double *first,
              const float *eta2, float *scratch, float *split_buf, long split_cap, long ldo, double *out,
              int mask, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!sea.d_tab_smit) return E_NOT_INITIALIZED;
    if (n <= 0) return OK;
    float *zs = scratch, *sp1 = scratch + n, *chain = scratch + 2 * n, *above = scratch + 3 * n;
    k_smit_prep<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, z, first, eta2, sea.depth, sea.swl, zs, sp1, chain,
                                                                 above);
    note_launch();
    CK(cudaGetLastError());
    SmitArgs a;
    a.n = n; a.ntile = sea.ntile_s; a.cstride = sea.npad_g; a.tab = sea.d_tab_smit;
    a.ph = static_cast<const float2 *>(ph); a.rr = rr; a.cf = sea.d_cf; a.phase = sea.d_phase;
    a.zs = zs; a.sp1 = sp1; a.chain = chain; a.above = above;
    a.depth = (float)sea.depth; a.ldo = ldo; a.out = out;
    const int ntp = sea.ntile_s * (sea.ntile_s + 1) / 2;
    if (n <= SMIT_FEW_POINTS && split_buf) {
        // a block per (point, slice), the rows of 8 tile pairs over its threads
        constexpr int PER = 128 / ST;
        const int npass = (ntp + PER - 1) / PER;
        int nslice = (int)std::min<long>(npass, std::max<long>(1, split_cap / ((long)SMIT_PARTS * n)));
        nslice = std::min(nslice, 65535);
        a.part = split_buf;
        prof_begin(PK_POINT_PAIRS, stream);
        k_smit_points_few<ST><<<dim3((unsigned)n, (unsigned)nslice), 128, 0, stream>>>(a, ntp, nslice);
        note_launch();
        prof_end(PK_POINT_PAIRS, stream);
        CK(cudaGetLastError());
        k_smit_finish<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, nslice, split_buf, chain, above, ldo, out);
        note_launch();
        CK(cudaGetLastError());
        return OK;
    }
    // few points: the tile-pair loop split over blockIdx.y (as many blocks as
    // fill the GPU), the slices summed in order by k_smit_finish
    const long nblk = (n + 127) / 128;
    const long target = 4L * 152;
    int nslice = nblk >= target ? 1 : (int)std::min<long>(ntp, (target + nblk - 1) / nblk);
    a.tp_per = (ntp + nslice - 1) / nslice;
    nslice = (ntp + a.tp_per - 1) / a.tp_per;
    if (nslice > 1 && (!split_buf || (long)SMIT_PARTS * n * nslice > split_cap)) {
        nslice = 1;
        a.tp_per = ntp;
    }
    a.part = nslice > 1 ? split_buf : nullptr;
    const size_t smem = sizeof(float) * ST * ST * SNC + 2 * sizeof(float2) * ST * 128 + sizeof(float) * ST * 128;
    // set once per process (thread-safe static initialisation)
    static const cudaError_t attr = [&] {
        cudaError_t e = cudaFuncSetAttribute(k_smit_points<ST, true, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_smit_points<ST, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_smit_points<ST, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        return e;
    }();
    CK(attr);
    // the velocity sums only where u, v or w is asked for, the pressure sum
    // only where dp is
    const bool vel = (mask & 14) != 0, pr = (mask & 16) != 0;
    prof_begin(PK_POINT_PAIRS, stream);
    const dim3 grid((unsigned)nblk, (unsigned)nslice);
    if (vel && pr)
        k_smit_points<ST, true, true><<<grid, 128, smem, stream>>>(a);
    else if (vel)
        k_smit_points<ST, true, false><<<grid, 128, smem, stream>>>(a);
    else
        k_smit_points<ST, false, true><<<grid, 128, smem, stream>>>(a);
    note_launch();
    prof_end(PK_POINT_PAIRS, stream);
    CK(cudaGetLastError());
    if (nslice > 1) {
        k_smit_finish<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, nslice, split_buf, chain, above, ldo, out);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

}  // namespace cfdwm
