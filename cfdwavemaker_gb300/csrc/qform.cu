// Precision form: the second-order sums at z = 0 (the surface elevation and
// the Taylor-layer velocities above the still-water level) as quadratic
// forms over each point's phasor vector, evaluated on the tcgen05 tensor
// cores with split 16-bit operands.
//
// What is computed: for each point p with phasors c_i = cos(phi_i),
// s_i = sin(phi_i) and ramps r_i,
//   eta2 = sum_{i<=m} r_i [A_e c_i c_m + B_e s_i s_m]             (Irregular.cpp:223-293)
//   u2, v2 at z0 = 0: the same form with A_u = Pu + Mu, B_u = Mu - Pu
//   w2 at z0 = 0:     sum r_i [C_w s_i c_m + D_w c_i s_m], C,D = Pw' +- Mw'
// with the uvw2 pair-cache coefficients (Irregular.cpp:975-1102) at z = 0,
// where cosh(k(z+h))/cosh(kh) = 1 and sinh(k(z+h))/cosh(kh) = tanh(kh).
// These are the second-order parts the reference evaluates for every point
// at or above the still-water level (Irregular.cpp:24-39, lsgrid_spline.cpp:890-897).
//
// As a GEMM: X = [r c | r s] (rows = points, K = 2N), W = the eight N x N
// upper-triangular coefficient blocks (eta, u, v, w) x (cos, sin half),
// T = X W, and each output is the row-wise dot of a T block with c or s.
//
// GB300 design:
//  * X is split into hi + lo 16-bit parts (bf16 or fp16) by a prep kernel
//    that writes one chunk of rows to a scratch buffer; W is split once at
//    set-up (stored transposed, K-major, as the B operand).
//  * k_qform_tc: warp-specialised persistent tcgen05 GEMM on CTA pairs
//    (cta_group::2), one 256 x 256 output tile per pair: warp 0 of each CTA
//    issues TMA loads (128B swizzle) of its 128 rows of X and its half of
//    the W tile into a stage ring, one thread of CTA 0 issues tcgen05.mma
//    (M=256, N=256, K=16) for the three split products Xh Wh + Xh Wl + Xl Wh
//    into FP32 TMEM accumulators (fp16: one accumulator over K segments of
//    512 terms, two TMEM buffers so that a unit's epilogue runs under the
//    next unit's MMAs; or a second accumulator for the cross products, with
//    the lo parts scaled by 2^11, over the whole K range), warps 2-9 read TMEM with
//    tcgen05.ld, multiply by the right-hand phasors (column-major, loaded
//    before the accumulator is ready) and reduce the row, one atomic add per
//    (row, tile).  Tiles are ordered in groups so that the X and W tiles in
//    flight stay L2-resident.  Only the K blocks of the upper triangle are
//    visited.  Every mbarrier wait is bounded; a timeout sets an error word.
//  * k_qform_plain: the same sums on FP32 CUDA cores (the plain form).
#include "cfdwm.h"
#include "ffmath.cuh"
#include "tc05.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
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

constexpr int QT = 32;          // tile of the plain table (components)
constexpr int QNC = 8;          // plain record: Ae, Be, Au, Bu, Av, Bv, Cw, Dw

__host__ __device__ inline long qtile_index(int I, int M, int nt) {
    return (long)I * nt - (long)I * (I - 1) / 2 + (M - I);
}

__device__ __forceinline__ double q_freq_ramp(double t, double rt, double ts, double du) {
    double rampdown = fmax(fmin(1. - ((t - ts - du + rt) / (rt + SMALL)), 1.), 0.);
    double rampup = fmax(fmin(((t - ts) / (rt + SMALL)), 1.), 0.);
    return rampup * rampdown;
}

// ---------------------------------------------------------------------------
// Coefficients at z = 0 from the pair-cache transfer functions (FP64)
// ---------------------------------------------------------------------------
struct QIn {
    int n;
    const double *omega, *A, *k, *theta;
    double depth, g, mtheta_rad, cutoff, bandwidth, kmax;
};

// value of the eight coefficients of entry (i, m), i <= m
__device__ void q_coefs(const QIn &c, int i, int m, double out[QNC]) {
    for (int q = 0; q < QNC; q++) out[q] = 0.0;
    if (i >= c.n || m >= c.n || i > m) return;
    const double h = c.depth, g = c.g;
    double ki = c.k[i], oi = c.omega[i], Ai = c.A[i];
    double thi = c.theta[i] + c.mtheta_rad, cti = cos(thi), sti = sin(thi);
    double Rn = ki * tanh(ki * h), Rsn = sqrt(Rn), agi = Ai * g / oi;
    if (i == m) {
        if (oi > c.cutoff) return;
        double Dnn = (6.0 * Rsn * Rsn * (ki * ki - Rn * Rn)) / (2.0 * Rsn * Rsn - ki * tanh(2.0 * ki * h));
        double AAd = 0.25 * agi * agi * (Dnn / (2.0 * oi));
        if (2.0 * ki <= c.kmax) {
            double ann = (Dnn - (ki * ki - Rn * Rn)) / Rn + 2.0 * Rn;
            double pe = 0.25 * Ai * Ai * ann;
            out[0] = pe; out[1] = -pe;                       // cos(2 phi) = c^2 - s^2
        }
        double pu = AAd * 2.0 * ki * cti, pv = AAd * 2.0 * ki * sti;
        out[2] = pu; out[3] = -pu;
        out[4] = pv; out[5] = -pv;
        double pw = AAd * 2.0 * ki * tanh(2.0 * ki * h);    // sin(2 phi) = 2 s c
        out[6] = pw; out[7] = pw;
        return;
    }
    double km = c.k[m], om = c.omega[m], Am = c.A[m];
    double thm = c.theta[m] + c.mtheta_rad, ctm = cos(thm), stm = sin(thm);
    double Rm = km * tanh(km * h), Rsm = sqrt(Rm), agm = Am * g / om;
    if (oi > c.cutoff || om > c.cutoff || fabs(oi - om) > c.bandwidth) return;
    bool hp = (ki + km) <= c.kmax, hm = (ki != km);
    // rounded as the reference rounds it; radicands clamped at 0 (opposite
    // directions of equal k give 0 up to rounding)
    double gam = __dadd_rn(__dmul_rn(cti, ctm), __dmul_rn(sti, stm));
    double kp = sqrt(fmax(0.0, __dadd_rn(__dadd_rn(__dmul_rn(ki, ki), __dmul_rn(km, km)),
                                          __dmul_rn(__dmul_rn(2.0 * ki, km), gam))));
    double kq = sqrt(fmax(0.0, __dadd_rn(__dadd_rn(__dmul_rn(ki, ki), __dmul_rn(km, km)),
                                          -__dmul_rn(__dmul_rn(2.0 * ki, km), gam))));
    double sp = Rsn + Rsm, sm = Rsn - Rsm, R2p = sp * sp, R2m = sm * sm;
    double AA = 0.5 * agi * agm;
    double Pe = 0, Me = 0, Pu = 0, Mu = 0, Pv = 0, Mv = 0, Pw = 0, Mw = 0;
    if (hp) {
        double den = R2p - kp * tanh(kp * h);
        double Dp = (2.0 * R2p * (ki * km * gam - Rn * Rm)) / den +
                    (sp * (Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
        double ap = (Dp - (ki * km * gam - Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
        double BB = Dp / (oi + om);
        Pe = 0.5 * Ai * Am * ap;
        Pu = AA * BB * (ki * cti + km * ctm);
        Pv = AA * BB * (ki * sti + km * stm);
        Pw = AA * BB * kp * tanh(kp * h);
    }
    if (hm) {
        double den = R2m - kq * tanh(kq * h);
        double Dm = (2.0 * R2m * (ki * km * gam + Rn * Rm)) / den +
                    (sm * (-Rsn * (km * km - Rm * Rm) + Rsm * (ki * ki - Rn * Rn))) / den;
        double am = (Dm - (ki * km * gam + Rn * Rm)) / sqrt(Rn * Rm) + (Rn + Rm);
        double CC = Dm / (oi - om);
        Me = 0.5 * Ai * Am * am;
        Mu = AA * CC * (ki * cti - km * ctm);
        Mv = AA * CC * (ki * sti - km * stm);
        Mw = AA * CC * kq * tanh(kq * h);
    }
    // cos(a+b) = cc - ss, cos(a-b) = cc + ss, sin(a+b) = sc + cs, sin(a-b) = sc - cs
    out[0] = Pe + Me; out[1] = Me - Pe;
    out[2] = Pu + Mu; out[3] = Mu - Pu;
    out[4] = Pv + Mv; out[5] = Mv - Pv;
    out[6] = Pw + Mw; out[7] = Pw - Mw;
}

// FP64 coefficients of every pair, once: coef[b][m][i] (W^T layout) for the
// eight GEMM blocks.  Block b: field (b & 3) -- eta, u, v, w -- and left
// half (b >> 2): 0 uses X = r c, 1 uses X = r s; the record index of block b
// is {A_e, A_u, A_v, D_w, B_e, B_u, B_v, C_w}.
__global__ void k_qform_coef64(QIn c, int npad, double *coef) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long tot = (long)npad * npad;
    if (e >= tot) return;
    int m = (int)(e / npad), i = (int)(e % npad);
    static const int idx[8] = {0, 2, 4, 7, 1, 3, 5, 6};
    double rec[QNC];
    q_coefs(c, i, m, rec);
    for (int b = 0; b < 8; b++) coef[((long)b * npad + m) * npad + i] = rec[idx[b]];
}

// plain table tiles from the FP64 coefficients
__global__ void k_qform_plain_from64(int npad, int nt, const double *coef, float *tab) {
    long t = blockIdx.x;
    int I = 0;
    while (qtile_index(I, nt - 1, nt) < t) I++;
    int M = (int)(t - qtile_index(I, I, nt)) + I;
    static const int rec_of_block[8] = {0, 2, 4, 7, 1, 3, 5, 6};
    for (int e = threadIdx.x; e < QT * QT; e += blockDim.x) {
        int ii = e / QT, mm = e % QT, i = I * QT + ii, m = M * QT + mm;
        long base = (t * QT * QT + e) * QNC;
        for (int b = 0; b < 8; b++)
            tab[base + rec_of_block[b]] = (float)coef[((long)b * npad + m) * npad + i];
    }
}

// B operand of the tensor-core form, split into hi and lo 16-bit parts.
// For fp16 each column m is scaled by 2^e_m (column maximum near 2^14);
// colscale[b][m] holds 2^-e_m (1 for bf16).  The lo part is scaled by a
// further lo_scale: 2^11 where the fp16 cross products go to their own
// accumulator, 1 where they share the hi accumulator.  Sharing it over a long
// K range loses their low bits (the tensor cores' FP32 accumulation keeps few
// guard bits: 1.5e-5 at N = 4096 over whole column tiles); over K segments of
// 512 terms it does not (3.3e-6, against 5.1e-6 with the second accumulator).
template <typename T16>
__global__ void k_qform_split(int npad, int fp16, double lo_scale, const double *coef, T16 *Whi, T16 *Wlo,
                              float *colscale) {
    const int b = blockIdx.y, m = blockIdx.x;
    const double *row = coef + ((long)b * npad + m) * npad;
    __shared__ double red[32];
    __shared__ double smax;
    double lmax = 0.0;
    for (int i = threadIdx.x; i < npad; i += blockDim.x) lmax = fmax(lmax, fabs(row[i]));
    for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) mx = fmax(mx, red[w]);
        smax = mx;
    }
    __syncthreads();
    double scale = 1.0;
    if (fp16 && smax > 0.0) {
        int ex;
        frexp(smax, &ex);               // smax = f 2^ex, f in [0.5, 1)
        scale = ldexp(1.0, 14 - ex);
    }
    if (threadIdx.x == 0) colscale[(long)b * npad + m] = (float)(1.0 / scale);
    for (int i = threadIdx.x; i < npad; i += blockDim.x) {
        double v = row[i] * scale;
        T16 hi, lo;
        if (fp16) {
            __half h = __float2half_rn((float)v);
            __half l = __float2half_rn((float)((v - (double)__half2float(h)) * lo_scale));
            hi = *reinterpret_cast<T16 *>(&h);
            lo = *reinterpret_cast<T16 *>(&l);
        } else {
            __nv_bfloat16 h = __float2bfloat16_rn((float)v);
            __nv_bfloat16 l = __float2bfloat16_rn((float)(v - (double)__bfloat162float(h)));
            hi = *reinterpret_cast<T16 *>(&h);
            lo = *reinterpret_cast<T16 *>(&l);
        }
        long o = ((long)b * npad + m) * npad + i;
        Whi[o] = hi;
        Wlo[o] = lo;
    }
}

// ---------------------------------------------------------------------------
// Phasor prep for a chunk of rows: X hi/lo (16-bit, [rows][2 npad]) and the
// right-hand phasors Y (FP32, [rows][2 npad]).
//
// The phase k.x - omega t + phase0 reaches 1e3-1e4 rad, so it is formed in
// float-float arithmetic (Dekker's exact product via FMA and Knuth's
// two-sum) from per-component (hi, lo) coefficient pairs and per-row (hi,
// lo) coordinates, then reduced by a three-part 2 pi (Cody-Waite) before the
// FP32 sincos.  Error: a few 1e-7 rad at |phase| ~ 1e4.
// ---------------------------------------------------------------------------
struct QRow {     // per row: dx, dy, t as float pairs and the ramp (trivial ramps)
    float dxh, dxl, dyh, dyl, th, tl, ramp, pad;
};
struct QComp {    // per component: kx, ky, -omega, phase0 as float pairs
    float kxh, kxl, kyh, kyl, wh, wl, ph, pl;
};

__global__ void k_qform_rows(long rows, const double *x, const double *y, const double *t, long st, double fx,
                             double fy, const double *phase, int cstride, QRow *out) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= rows) return;
    double dx = x[p] - fx, dy = y[p] - fy, tt = t[p * st];
    QRow r;
    r.dxh = (float)dx; r.dxl = (float)(dx - (double)r.dxh);
    r.dyh = (float)dy; r.dyl = (float)(dy - (double)r.dyh);
    r.th = (float)tt; r.tl = (float)(tt - (double)r.th);
    r.ramp = (float)q_freq_ramp(tt, phase[4 * cstride], phase[5 * cstride], phase[6 * cstride]);
    r.pad = 0.f;
    out[p] = r;
}

__global__ void k_qform_comps(int n, int npad, const double *phase, int cstride, QComp *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    QComp c = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
        double v[4] = {phase[i], phase[cstride + i], -phase[2 * cstride + i], phase[3 * cstride + i]};
        float h[4], l[4];
        for (int q = 0; q < 4; q++) { h[q] = (float)v[q]; l[q] = (float)(v[q] - (double)h[q]); }
        c = {h[0], l[0], h[1], l[1], h[2], l[2], h[3], l[3]};
    }
    out[i] = c;
}

struct QPrep {
    long rows;
    const QRow *row;
    const QComp *comp;
    const double *phase;       // [7][cstride] (ramp parameters for non-trivial ramps)
    const double *t;
    long st;                   // element stride of t
    int cstride, ncomp, npad;
    int trivial_ramp, fp16;
    float lo_scale;          // fp16: factor of the lo parts (2^11 with a cross accumulator, else 1)
    void *Xhi, *Xlo;           // [rows][2 npad]
    float *Y;                  // [2 npad][ldy], column-major: rows adjacent
    long ldy;                  // >= rows rounded up to PREP_ROWS
};

constexpr int PREP_ROWS = 16;      // rows per block of the operand preparation

// blockDim 128: thread t owns components i = 256 blockIdx.x + 2t and i + 1
// (their float-float coefficients stay in registers); blockIdx.y: a group of
// PREP_ROWS rows.  Per (row, component): the float-float phase, its cos and
// sin (Y), and r cos, r sin split into hi and lo 16-bit parts (X).  X rows are
// written as 16-bit pairs; Y is staged in shared memory and written
// column-major, each column's 16 rows (64 B) by 16 adjacent threads (rows
// past the last are zero).
__global__ void __launch_bounds__(128) k_qform_prep(QPrep a) {
    __shared__ float s_y[512][PREP_ROWS + 1];     // [cos 256 | sin 256][row]
    const int i = blockIdx.x * 256 + 2 * threadIdx.x;
    QComp K[2];
    bool on[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        on[q] = i + q < a.ncomp;
        K[q] = on[q] ? a.comp[i + q] : QComp{0, 0, 0, 0, 0, 0, 0, 0};
    }
    const long p0 = (long)blockIdx.y * PREP_ROWS;
    for (int rr = 0; rr < PREP_ROWS; rr++) {
        const long p = p0 + rr;
        float c[2] = {0.f, 0.f}, s[2] = {0.f, 0.f}, r[2] = {0.f, 0.f};
        if (p < a.rows) {
            const QRow R = a.row[p];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (!on[q]) continue;
                float2 ph = ff_add(ff_mul(K[q].kxh, K[q].kxl, R.dxh, R.dxl), ff_mul(K[q].kyh, K[q].kyl, R.dyh, R.dyl));
                ph = ff_add(ph, ff_mul(K[q].wh, K[q].wl, R.th, R.tl));
                ph = ff_add(ph, make_float2(K[q].ph, K[q].pl));
                __sincosf(ff_reduce_2pi(ph), &s[q], &c[q]);
                r[q] = a.trivial_ramp ? R.ramp
                                      : (float)q_freq_ramp(a.t[p * a.st], a.phase[4 * a.cstride + i + q],
                                                           a.phase[5 * a.cstride + i + q],
                                                           a.phase[6 * a.cstride + i + q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            s_y[2 * threadIdx.x + q][rr] = c[q];
            s_y[256 + 2 * threadIdx.x + q][rr] = s[q];
        }
        if (p >= a.rows) continue;
        const long o = p * 2 * a.npad + i;
        const float xc0 = r[0] * c[0], xc1 = r[1] * c[1], xs0 = r[0] * s[0], xs1 = r[1] * s[1];
        if (a.fp16) {
            const __half2 hc = __floats2half2_rn(xc0, xc1), hs = __floats2half2_rn(xs0, xs1);
            const float2 fc = __half22float2(hc), fs = __half22float2(hs);
            __half2 *H = reinterpret_cast<__half2 *>((__half *)a.Xhi + o);
            __half2 *L = reinterpret_cast<__half2 *>((__half *)a.Xlo + o);
            H[0] = hc;
            H[a.npad / 2] = hs;
            L[0] = __floats2half2_rn((xc0 - fc.x) * a.lo_scale, (xc1 - fc.y) * a.lo_scale);
            L[a.npad / 2] = __floats2half2_rn((xs0 - fs.x) * a.lo_scale, (xs1 - fs.y) * a.lo_scale);
        } else {
            const __nv_bfloat162 hc = __floats2bfloat162_rn(xc0, xc1), hs = __floats2bfloat162_rn(xs0, xs1);
            const float2 fc = __bfloat1622float2(hc), fs = __bfloat1622float2(hs);
            __nv_bfloat162 *H = reinterpret_cast<__nv_bfloat162 *>((__nv_bfloat16 *)a.Xhi + o);
            __nv_bfloat162 *L = reinterpret_cast<__nv_bfloat162 *>((__nv_bfloat16 *)a.Xlo + o);
            H[0] = hc;
            H[a.npad / 2] = hs;
            L[0] = __floats2bfloat162_rn(xc0 - fc.x, xc1 - fc.y);
            L[a.npad / 2] = __floats2bfloat162_rn(xs0 - fs.x, xs1 - fs.y);
        }
    }
    __syncthreads();
    // Y: warp w writes columns 2 k + (lane >> 4), k = w, w + 4, ..., rows lane & 15
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = lane & (PREP_ROWS - 1);
    const int i0 = blockIdx.x * 256;
    for (int col = 2 * warp + (lane >> 4); col < 512; col += 8) {
        const long gcol = col < 256 ? (long)i0 + col : (long)a.npad + i0 + (col - 256);
        a.Y[gcol * a.ldy + p0 + rr] = s_y[col][rr];
    }
}

// ---------------------------------------------------------------------------
// Plain FP32 form (CUDA cores), register-blocked.
//
// Block of 128 threads over 256 rows: thread t owns rows p and p + 128.  The
// pair matrix is walked column tile by column tile (M outer, I = 0..M inner).
// For the column tile M each thread keeps its two rows' 32 phasors (c, s) of
// that tile in registers, packed as row pairs, so one coefficient read -- a
// warp broadcast from shared memory -- feeds both rows through packed FP32x2
// FMAs: per (pair, row pair) 8 FFMA2 against one 32-byte record read.  The
// coefficient tiles (32 x 32 records of 8 floats, 32 KB) stream through two
// shared-memory stages with cp.async, the next tile landing while the current
// one is used.  The row phasor of component i is prefetched one i ahead.
// Accumulation: the 32 terms of a tile row in FP32, then a Kahan pair per
// (row, field), as before.  The lower triangle of the diagonal tiles holds
// zeros, so every tile runs the full 32 x 32 loop.
// ---------------------------------------------------------------------------
constexpr int QPL_MAXSEG = 32;

struct QPlain {
    long rows;
    int ntile;
    const float *tab;        // plain tiles
    const float2 *ph;        // [npad][rows] (c, s)
    const float *rr;         // [npad][rows]
    int nseg;                // segments of the tile walk (units per row block)
    int mb[QPL_MAXSEG + 1];  // segment g walks the column tiles M in [mb[g], mb[g + 1])
    float *part;             // [nseg][rows][4]: each segment's sums
};

constexpr int QPL_ROWS = 256;                              // rows per block
constexpr int QPL_TILE4 = QT * QT * QNC / 4;               // float4 per tile
constexpr int QPLAIN_SMEM = 2 * QPL_TILE4 * 16;            // two stages, 64 KB

__device__ __forceinline__ void qpl_cp16(void *smem, const void *gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void qpl_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void qpl_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ void qpl_kahan(float &S, float &C, float y) {
    y -= C;
    float t = S + y;
    C = (t - S) - y;
    S = t;
}

__global__ void __launch_bounds__(128, 2) k_qform_plain(QPlain a) {
    extern __shared__ float4 q_smem[];
    const int tid = threadIdx.x;
    // unit = (segment, row block), segments outermost: the units in flight
    // together walk the same few column tiles, whose records stay in L2
    const long nrb = (a.rows + QPL_ROWS - 1) / QPL_ROWS;
    const int seg = (int)(blockIdx.x / nrb);
    const long rb = blockIdx.x % nrb;
    const long p0 = rb * QPL_ROWS + tid, p1 = p0 + 128;
    const long q0 = p0 < a.rows ? p0 : 0, q1 = p1 < a.rows ? p1 : 0;   // clamped reads
    const int nt = a.ntile;
    const int mlo = a.mb[seg], mhi = a.mb[seg + 1];
    const long ntiles = ((long)mhi * (mhi + 1) - (long)mlo * (mlo + 1)) / 2;
    const float4 *tab4 = reinterpret_cast<const float4 *>(a.tab);
    float S0[4] = {0, 0, 0, 0}, C0[4] = {0, 0, 0, 0}, S1[4] = {0, 0, 0, 0}, C1[4] = {0, 0, 0, 0};
    float2 pm0[QT], pm1[QT];     // (c, s) of the 32 components of tile M, rows p and p + 128

    // stage k of the walk: tile (I, M) with M outer, M in [mlo, mhi)
    int lI = 0, lM = mlo;        // next tile to load
    auto issue = [&](long k) {
        if (k < ntiles) {
            const float4 *src = tab4 + qtile_index(lI, lM, nt) * (long)QPL_TILE4;
            float4 *dst = q_smem + (k & 1) * QPL_TILE4;
#pragma unroll 4
            for (int e = tid; e < QPL_TILE4; e += 128) qpl_cp16(dst + e, src + e);
            if (++lI > lM) { lI = 0; lM++; }
        }
        qpl_commit();
    };
    issue(0);
    int I = 0, M = mlo;
    for (long k = 0; k < ntiles; k++) {
        issue(k + 1);
        if (I == 0) {
#pragma unroll
            for (int mm = 0; mm < QT; mm++) {
                const long r = (long)(M * QT + mm) * a.rows;
                pm0[mm] = a.ph[r + q0];
                pm1[mm] = a.ph[r + q1];
            }
        }
        qpl_wait1();
        __syncthreads();
        const float4 *st = q_smem + (k & 1) * QPL_TILE4;
        // row phasors of component i, prefetched two components ahead (the
        // ones past the tile re-read its last component)
        const long rbase = (long)(I * QT) * a.rows;
        float2 pa0 = a.ph[rbase + q0], pa1 = a.ph[rbase + q1];
        float ra0 = a.rr[rbase + q0], ra1 = a.rr[rbase + q1];
        float2 pb0 = a.ph[rbase + a.rows + q0], pb1 = a.ph[rbase + a.rows + q1];
        float rb0 = a.rr[rbase + a.rows + q0], rb1 = a.rr[rbase + a.rows + q1];
        for (int ii = 0; ii < QT; ii++) {
            const long rn = rbase + (long)(ii + 2 < QT ? ii + 2 : QT - 1) * a.rows;
            const float2 n0 = a.ph[rn + q0], n1 = a.ph[rn + q1];
            const float nr0 = a.rr[rn + q0], nr1 = a.rr[rn + q1];
            // (A_cos, A_sin) of each field times (c_m, s_m): the record's
            // float pairs and the phasor are the two lanes of each FFMA2
            float2 e0 = {0, 0}, u0 = {0, 0}, v0 = {0, 0}, w0 = {0, 0};
            float2 e1 = {0, 0}, u1 = {0, 0}, v1 = {0, 0}, w1 = {0, 0};
            const float4 *rec = st + ii * QT * 2;
#pragma unroll
            for (int mm = 0; mm < QT; mm++) {
                const float4 c0 = rec[2 * mm], c1 = rec[2 * mm + 1];
                const float2 ce = make_float2(c0.x, c0.y), cu = make_float2(c0.z, c0.w);
                const float2 cv = make_float2(c1.x, c1.y), cw = make_float2(c1.z, c1.w);
                e0 = __ffma2_rn(ce, pm0[mm], e0); e1 = __ffma2_rn(ce, pm1[mm], e1);
                u0 = __ffma2_rn(cu, pm0[mm], u0); u1 = __ffma2_rn(cu, pm1[mm], u1);
                v0 = __ffma2_rn(cv, pm0[mm], v0); v1 = __ffma2_rn(cv, pm1[mm], v1);
                w0 = __ffma2_rn(cw, pm0[mm], w0); w1 = __ffma2_rn(cw, pm1[mm], w1);
            }
            // eta, u, v: c_i (A_c . c) + s_i (A_s . s); w: s_i (C . c) + c_i (D . s)
            qpl_kahan(S0[0], C0[0], ra0 * fmaf(pa0.x, e0.x, pa0.y * e0.y));
            qpl_kahan(S0[1], C0[1], ra0 * fmaf(pa0.x, u0.x, pa0.y * u0.y));
            qpl_kahan(S0[2], C0[2], ra0 * fmaf(pa0.x, v0.x, pa0.y * v0.y));
            qpl_kahan(S0[3], C0[3], ra0 * fmaf(pa0.y, w0.x, pa0.x * w0.y));
            qpl_kahan(S1[0], C1[0], ra1 * fmaf(pa1.x, e1.x, pa1.y * e1.y));
            qpl_kahan(S1[1], C1[1], ra1 * fmaf(pa1.x, u1.x, pa1.y * u1.y));
            qpl_kahan(S1[2], C1[2], ra1 * fmaf(pa1.x, v1.x, pa1.y * v1.y));
            qpl_kahan(S1[3], C1[3], ra1 * fmaf(pa1.y, w1.x, pa1.x * w1.y));
            pa0 = pb0; pa1 = pb1; ra0 = rb0; ra1 = rb1;
            pb0 = n0; pb1 = n1; rb0 = nr0; rb1 = nr1;
        }
        __syncthreads();     // the stage is refilled by the next issue
        if (++I > M) { I = 0; M++; }
    }
    // the segment's compensated sums
    float *P = a.part + (long)seg * a.rows * 4;
    if (p0 < a.rows)
        for (int f = 0; f < 4; f++) P[p0 * 4 + f] = S0[f] - C0[f];
    if (p1 < a.rows)
        for (int f = 0; f < 4; f++) P[p1 * 4 + f] = S1[f] - C1[f];
}

// out[row][f] = the segments' sums added in segment order (Kahan)
__global__ void k_qform_plain_sum(long rows, int nseg, const float *part, float *out) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= rows * 4) return;
    float S = 0.f, C = 0.f;
    for (int g = 0; g < nseg; g++) qpl_kahan(S, C, part[(long)g * rows * 4 + e]);
    out[e] = S - C;
}

// ---------------------------------------------------------------------------
// tcgen05 tensor-core form
// ---------------------------------------------------------------------------
constexpr int TBM = 128, TBK = 64;
// variants (TMEM holds 512 FP32 columns), all with N = 256 MMAs (measured:
// M = 128, N = 128 MMAs kept the tensor pipe about 60% busy, N = 256 about 80%):
//   one accumulator, two accumulator buffers, so that the epilogue of one
//   tile unit hides behind the next unit's MMAs (bf16, and fp16 with the
//   cross products in the hi accumulator);
//   fp16 with hi and cross accumulators filling TMEM, one buffer (TWO);
// each on one SM (M = 128) or on a CTA pair (M = 256, cta_group::2: each CTA
// holds its 128 rows of X and half of the W tile, so each SM stages and reads
// half the W bytes; measured 3-10% faster than the one-SM form).
constexpr int TBN = 256;                  // component padding unit
constexpr int A_TILE = TBM * TBK * 2;     // 16 KiB
template <int BN, bool TWO, bool PAIR> struct TcCfg {
    static constexpr int BROWS = PAIR ? BN / 2 : BN;     // W rows held by one CTA
    static constexpr int B_TILE = BROWS * TBK * 2;
    static constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;   // one CTA's share of a stage
    static constexpr int STAGES = 196608 / STAGE_BYTES < 4 ? 196608 / STAGE_BYTES : 4;
    static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 256;
    static constexpr int ACOLS = TWO ? 2 * BN : BN;     // TMEM columns of one tile
    static constexpr int NBUF = 512 / ACOLS;             // accumulator buffers
};

__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *m, uint64_t *bar, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
                 ::"r"(su32(dst)), "l"(m), "r"(su32(bar)), "r"(x), "r"(y) : "memory");
}
// CTA-pair forms (cta_group::2).  The load lands in this CTA's shared memory
// and signals the mbarrier at cluster address `bar`, which may be the peer's.
__device__ __forceinline__ void tma_2d_pair(void *dst, const CUtensorMap *m, uint32_t bar, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%3, %4}], [%2];"
                 ::"r"(su32(dst)), "l"(m), "r"(bar), "r"(x), "r"(y) : "memory");
}
// one MMA of the pair: M = 256 (128 rows from each CTA's shared memory at the
// same offsets), N columns (the first half of B from this CTA, the second from
// the peer); each CTA's TMEM receives its own 128 rows
__device__ __forceinline__ void umma_pair(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}"
                 ::"r"(dt), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// arrives once on the mbarrier at this offset in both CTAs of the pair when the
// pair's MMAs issued so far have completed
__device__ __forceinline__ void umma_pair_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(su32(bar)), "h"((uint16_t)3) : "memory");
}
// cluster address of the same shared-memory location in CTA `rank`
__device__ __forceinline__ uint32_t mapa_rank(const void *p, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(su32(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_cluster(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
                 "selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(su32(b)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t ncluster_x() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
constexpr int QTC_MAXCU = 256;

struct QTC {
    long rows;               // rows of this chunk
    int npad;                // components (multiple of 256)
    int ntn;                 // column tiles per block (npad / N)
    int group_m;             // row blocks per tile group
    int nblk;                // coefficient blocks of W
    int nout;                // outputs per row
    const int *bmap;         // per block: X half, Y half, output column
    const float *Y;          // [2 npad][ldy], column-major
    long ldy;
    const float *colscale;   // [nblk][npad] (1 for bf16)
    float *out;              // [rows][nout] accumulated with atomics
    int fp16;
    int *err;
    // column units per block: with seg = 0 unit u is column tile u over its
    // whole upper-triangle K range; with seg = 1 it is column tile cu_tn[u]
    // over the K blocks [cu_kb0[u], cu_kb1[u]) (a long K range cut into
    // segments, each with its own accumulation and epilogue)
    int ncu, seg;
    unsigned short cu_tn[QTC_MAXCU], cu_kb0[QTC_MAXCU], cu_kb1[QTC_MAXCU];
};

// bounded wait that also gives up as soon as another role has set the error word
__device__ __forceinline__ bool mbar_wait_e(uint64_t *b, uint32_t parity, int *err, int code) {
    long long t0 = clock64();
    int n = 0;
    while (!mbar_try(b, parity)) {
        if ((++n & 255) == 0 && *(volatile int *)err != 0) return false;
        if (clock64() - t0 > WAIT_LIMIT) {
            atomicExch(err, code);
            return false;
        }
    }
    return true;
}

// the same with cluster-scope acquire: the arrivals come from both CTAs of a pair
__device__ __forceinline__ bool mbar_wait_ec(uint64_t *b, uint32_t parity, int *err, int code) {
    long long t0 = clock64();
    int n = 0;
    while (!mbar_try_cluster(b, parity)) {
        if ((++n & 255) == 0 && *(volatile int *)err != 0) return false;
        if (clock64() - t0 > WAIT_LIMIT) {
            atomicExch(err, code);
            return false;
        }
    }
    return true;
}

struct TileInfo {
    long rb;
    int blk, tn, kb0, kb1;
};

// grouped tile order: a group of group_m row units sweeps all column tiles.
// A row unit is CS consecutive row blocks, one per CTA of a cluster (CTA rank
// r takes block CS u + r; a block past the last row reads zeros through TMA
// and stores nothing), so that the CTAs of a cluster share every W tile.
// Validity depends on the unit only: the CTAs of a cluster walk the same
// tile sequence.
template <int BN, int CS>
__device__ __forceinline__ bool tile_of(const QTC &a, long nru, long t, int crank, TileInfo &ti) {
    const int ncol = a.nblk * a.ncu;
    const long gm = a.group_m / CS > 0 ? a.group_m / CS : 1;
    const long per_group = gm * ncol;
    long grp = t / per_group, in = t % per_group;
    long gm0 = grp * gm;
    long gsz = nru - gm0 < gm ? nru - gm0 : gm;
    if (gsz <= 0) return false;
    long ru = gm0 + in % gsz;
    int ct = (int)(in / gsz);
    if (ru >= nru || ct >= ncol) return false;
    ti.rb = ru * CS + crank;
    ti.blk = ct / a.ncu;
    const int cu = ct % a.ncu;
    if (a.seg) {
        ti.tn = a.cu_tn[cu];
        ti.kb0 = a.cu_kb0[cu];
        ti.kb1 = a.cu_kb1[cu];
    } else {
        ti.tn = cu;
        ti.kb0 = 0;
        ti.kb1 = (cu * BN + BN) / TBK;          // upper triangle: i < m0 + BN
    }
    return true;
}

// Persistent: CTA (or CTA pair) c takes tile units c, c + (number of units
// in flight), ...  Warp 0 streams the operand tiles through the stage ring
// (continuously across tiles), one thread of warp 1 issues the MMAs into TMEM
// accumulator buffer j % NBUF of its j-th tile, warps 2-9 drain it when its
// MMAs complete: with two buffers (one accumulator) the epilogue of tile j
// overlaps the MMAs of tile j + 1.
// Epilogue warp w reads TMEM lane quarter w % 4 (its 32 rows) and column half
// (w - 2) / 4; it loads its rows' right-hand phasors Y, scaled by the column
// scales, before it waits for the accumulator, so those loads (coalesced: Y is
// column-major) overlap the tile's MMAs.
//
// PAIR: a cluster of two CTAs computes a 256-row tile with cta_group::2 MMAs.
// Both CTAs load their own 128 rows of X and their half of the W tile into
// their own shared memory; every load signals the full barrier of CTA 0,
// whose one thread issues the pair's MMAs.  Its commits arrive on the empty,
// accumulator-full and done barriers of both CTAs; the epilogue warps of both
// CTAs arrive on CTA 0's drained barrier (count 8).  Before it exits, each
// producer waits for the last release of its stages, so no commit is still
// on its way to a CTA that has left.
constexpr int TC_THREADS = 320;            // producer, MMA and 8 epilogue warps
constexpr int TC_EPI_WARPS = 8;

template <int BN, bool TWO, bool PAIR>
__global__ void __launch_bounds__(TC_THREADS, 1) k_qform_tc(const __grid_constant__ CUtensorMap mXh,
                                                     const __grid_constant__ CUtensorMap mXl,
                                                     const __grid_constant__ CUtensorMap mWh,
                                                     const __grid_constant__ CUtensorMap mWl,
                                                     const __grid_constant__ QTC a) {
    using CF = TcCfg<BN, TWO, PAIR>;
    constexpr int CS = PAIR ? 2 : 1;
    constexpr int TSTAGES = CF::STAGES, STAGE_BYTES = CF::STAGE_BYTES, B_TILE = CF::B_TILE;
    constexpr int BROWS = CF::BROWS, ACOLS = CF::ACOLS, NBUF = CF::NBUF;
    static_assert((BROWS * 128) % 1024 == 0, "W halves keep the 1024 B swizzle atom");
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + TSTAGES * STAGE_BYTES);
    uint64_t *empty = full + TSTAGES;
    uint64_t *accf = empty + TSTAGES;         // [2] accumulator buffer full
    uint64_t *acce = accf + 2;                // [2] accumulator buffer drained
    uint64_t *mdone = acce + 2;               // all MMAs into this CTA's TMEM complete
    uint32_t *tmem_slot = (uint32_t *)(mdone + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int crank = PAIR ? (int)cluster_ctarank() : 0;
    const bool leader = crank == 0;
    const long cid = PAIR ? (long)cluster_id_x() : (long)blockIdx.x;
    const long ncl = PAIR ? (long)ncluster_x() : (long)gridDim.x;
    const long nrb = (a.rows + TBM - 1) / TBM;
    const long nru = (nrb + CS - 1) / CS;
    const long ntiles = nru * (long)a.nblk * a.ncu;
    // (a pair does not return early: its CTAs address each other until the end)
    if (!PAIR && *(volatile int *)a.err != 0) return;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TSTAGES; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; b++) { mbar_init(&accf[b], 1); mbar_init(&acce[b], TC_EPI_WARPS * CS); }
        mbar_init(mdone, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const uint32_t ncols_tmem = 512;          // two buffers of 256 FP32 columns (one or two accumulators)
    if (warp == 1) {
        if (PAIR) {
            asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                         "r"(ncols_tmem));
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
        } else {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                         "r"(ncols_tmem));
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        }
    }
    __syncthreads();
    // the peer's barriers are initialised (and its TMEM allocated) before any
    // load or MMA of the pair addresses them
    if (PAIR) cluster_sync_all();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    __shared__ long issued_s, consumed_s;
    if (threadIdx.x == 0) { issued_s = 0; consumed_s = 0; }
    __syncthreads();
    if (warp == 0) {
        if (lane == 0) {
            // the full barriers every load of the pair signals: CTA 0's
            const uint32_t full0 = PAIR ? mapa_rank(full, 0) : 0u;
            long g = 0;
            bool ok = true;
            for (long t = cid; t < ntiles && ok; t += ncl) {
                TileInfo ti;
                if (!tile_of<BN, CS>(a, nru, t, crank, ti)) continue;
                const int khalf = a.bmap[3 * ti.blk];
                const int m0 = ti.tn * BN;
                for (int kb = ti.kb0; kb < ti.kb1; kb++, g++) {
                    int s = (int)(g % TSTAGES);
                    uint32_t ph = (uint32_t)((g / TSTAGES) & 1);
                    if (!mbar_wait_e(&empty[s], ph ^ 1, a.err, 1)) { ok = false; break; }
                    uint8_t *st = smem + s * STAGE_BYTES;
                    // CTA 0 expects the bytes of both CTAs' shares
                    if (leader) mbar_expect_tx(&full[s], CS * STAGE_BYTES);
                    int kx = khalf * a.npad + kb * TBK;
                    int ky = (int)(ti.rb * TBM);
                    int wy = ti.blk * a.npad + m0 + crank * BROWS;
                    if (PAIR) {
                        const uint32_t fb = full0 + (uint32_t)(s * 8);
                        tma_2d_pair(st, &mXh, fb, kx, ky);
                        tma_2d_pair(st + A_TILE, &mXl, fb, kx, ky);
                        tma_2d_pair(st + 2 * A_TILE, &mWh, fb, kb * TBK, wy);
                        tma_2d_pair(st + 2 * A_TILE + B_TILE, &mWl, fb, kb * TBK, wy);
                    } else {
                        tma_2d(st, &mXh, &full[s], kx, ky);
                        tma_2d(st + A_TILE, &mXl, &full[s], kx, ky);
                        tma_2d(st + 2 * A_TILE, &mWh, &full[s], kb * TBK, wy);
                        tma_2d(st + 2 * A_TILE + B_TILE, &mWl, &full[s], kb * TBK, wy);
                    }
                    issued_s = g + 1;
                }
            }
            // the last release of each stage (pair: CTA 0's commit, which also
            // arrives here), so nothing is on its way to this CTA after it exits
            if (ok && PAIR)
                for (long h = g - TSTAGES > 0 ? g - TSTAGES : 0; h < g; h++)
                    if (!mbar_wait_e(&empty[h % TSTAGES], (uint32_t)((h / TSTAGES) & 1), a.err, 7)) break;
        }
    } else if (warp == 1) {
        if (lane == 0 && leader) {
            // kind::f16, D = F32, A/B = bf16 (1) or f16 (0), both K-major, N = BN, M = 128 CS
            const uint32_t fmt = a.fp16 ? 0u : 1u;
            const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(BN >> 3) << 17) |
                                   ((uint32_t)((CS * TBM) >> 4) << 24);
            long g = 0;
            int j = 0;
            bool ok = true;
            for (long t = cid; t < ntiles && ok; t += ncl) {
                TileInfo ti;
                if (!tile_of<BN, CS>(a, nru, t, crank, ti)) continue;
                const int buf = j % NBUF;
                const uint32_t use = (uint32_t)(j / NBUF);
                // the epilogues (of both CTAs) have drained this buffer's previous tile
                const bool drained = PAIR ? mbar_wait_ec(&acce[buf], (use & 1) ^ 1, a.err, 5)
                                          : mbar_wait_e(&acce[buf], (use & 1) ^ 1, a.err, 5);
                if (!drained) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(buf * ACOLS);
                const uint32_t acc2 = TWO ? acc + BN : acc;     // fp16: cross products
                for (int kb = ti.kb0; kb < ti.kb1; kb++, g++) {
                    int s = (int)(g % TSTAGES);
                    uint32_t ph = (uint32_t)((g / TSTAGES) & 1);
                    if (!mbar_wait_e(&full[s], ph, a.err, 2)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    uint32_t base = su32(smem + s * STAGE_BYTES);
                    uint64_t dXh = sdesc(base), dXl = sdesc(base + A_TILE);
                    uint64_t dWh = sdesc(base + 2 * A_TILE), dWl = sdesc(base + 2 * A_TILE + B_TILE);
                    for (int k = 0; k < TBK / 16; k++) {
                        uint64_t o = (uint64_t)(k * 32) >> 4;     // 16 elements = 32 bytes per step
                        uint32_t first = (kb == ti.kb0 && k == 0) ? 0u : 1u;
                        if (PAIR) {
                            umma_pair(acc, dXh + o, dWh + o, idesc, first);
                            umma_pair(acc2, dXh + o, dWl + o, idesc, TWO ? first : 1u);
                            umma_pair(acc2, dXl + o, dWh + o, idesc, 1u);
                        } else {
                            umma(acc, dXh + o, dWh + o, idesc, first);
                            umma(acc2, dXh + o, dWl + o, idesc, TWO ? first : 1u);
                            umma(acc2, dXl + o, dWh + o, idesc, 1u);
                        }
                    }
                    if (PAIR) umma_pair_commit(&empty[s]);
                    else umma_commit(&empty[s]);
                    consumed_s = g + 1;
                }
                if (!ok) break;
                if (PAIR) umma_pair_commit(&accf[buf]);
                else umma_commit(&accf[buf]);
                j++;
            }
            if (PAIR) umma_pair_commit(mdone);
            else umma_commit(mdone);
        }
    } else {
        // epilogue: warps 2..9, lane quarter q, column half hc
        constexpr int HC = BN / 2, NCH = HC / 32;
        const int q = warp & 3, hc = (warp - 2) >> 2;
        const uint32_t acce0 = PAIR ? mapa_rank(acce, 0) : 0u;
        int j = 0;
        for (long t = cid; t < ntiles; t += ncl) {
            TileInfo ti;
            if (!tile_of<BN, CS>(a, nru, t, crank, ti)) continue;
            const int buf = j % NBUF;
            const uint32_t use = (uint32_t)(j / NBUF);
            const int yhalf = a.bmap[3 * ti.blk + 1], outcol = a.bmap[3 * ti.blk + 2];
            const int c0 = ti.tn * BN + hc * HC;       // first column of this warp
            const long row = ti.rb * TBM + q * 32 + lane;
            const bool live = row < a.rows;
            const float *Yc = a.Y + ((long)yhalf * a.npad + c0) * a.ldy + (live ? row : 0);
            const float *cs = a.colscale + (long)ti.blk * a.npad + c0;
            if (TWO) {
                // hi and cross accumulators, one buffer: read this warp's TMEM rows first
                // (hi + cross / 2^11, HC values a thread), release the buffer to
                // the next tile's MMAs, then load Y (column-major: the warp's 32
                // rows of a column are adjacent) and reduce meanwhile
                bool ok = mbar_wait_e(&accf[buf], use & 1, a.err, 3);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc =
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * ACOLS) + (uint32_t)(hc * HC);
                float tv[NCH][32];
#pragma unroll
                for (int c = 0; c < NCH; c++) {
                    tmem_ld32(acc + c * 32, tv[c]);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        float w[16];
                        tmem_ld16(acc + BN + c * 32 + h * 16, w);
#pragma unroll
                        for (int jj = 0; jj < 16; jj++)
                            tv[c][h * 16 + jj] = fmaf(w[jj], 1.0f / 2048.0f, tv[c][h * 16 + jj]);
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    if (PAIR) mbar_arrive_remote(acce0 + (uint32_t)(buf * 8));
                    else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&acce[buf])) : "memory");
                }
                float part = 0.f;
                if (live) {
#pragma unroll
                    for (int c = 0; c < NCH; c++)
#pragma unroll
                        for (int jj = 0; jj < 32; jj += 4) {
                            const float4 s4 = __ldg(reinterpret_cast<const float4 *>(cs + c * 32 + jj));
                            const float y0 = __ldg(Yc + (long)(c * 32 + jj) * a.ldy);
                            const float y1 = __ldg(Yc + (long)(c * 32 + jj + 1) * a.ldy);
                            const float y2 = __ldg(Yc + (long)(c * 32 + jj + 2) * a.ldy);
                            const float y3 = __ldg(Yc + (long)(c * 32 + jj + 3) * a.ldy);
                            part = fmaf(tv[c][jj] * s4.x, y0, part);
                            part = fmaf(tv[c][jj + 1] * s4.y, y1, part);
                            part = fmaf(tv[c][jj + 2] * s4.z, y2, part);
                            part = fmaf(tv[c][jj + 3] * s4.w, y3, part);
                        }
                    atomicAdd(a.out + row * a.nout + outcol, part);
                }
                j++;
                continue;
            }
            // one accumulator, two buffers: Y times the column scales; the
            // first NSL chunks of 32 columns are loaded before the accumulator
            // is ready, the others one chunk ahead
            constexpr int NSL = NCH < 2 ? NCH : 2;
            float ys[NSL][32];
#pragma unroll
            for (int c = 0; c < NSL; c++)
#pragma unroll
                for (int jj = 0; jj < 32; jj++) ys[c][jj] = live ? __ldg(Yc + (long)(c * 32 + jj) * a.ldy) : 0.f;
#pragma unroll
            for (int c = 0; c < NSL; c++)
#pragma unroll
                for (int jj = 0; jj < 32; jj += 4) {
                    const float4 s4 = __ldg(reinterpret_cast<const float4 *>(cs + c * 32 + jj));
                    ys[c][jj] *= s4.x;
                    ys[c][jj + 1] *= s4.y;
                    ys[c][jj + 2] *= s4.z;
                    ys[c][jj + 3] *= s4.w;
                }
            bool ok = mbar_wait_e(&accf[buf], use & 1, a.err, 3);
            // tcgen05.ld is warp-collective (.sync.aligned): decide per warp
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * ACOLS) + (uint32_t)(hc * HC);
            float part = 0.f;
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                const int sl = c % NSL;
                if (c >= NSL) {
                    // loaded while chunk c - NSL was reduced
#pragma unroll
                    for (int jj = 0; jj < 32; jj += 4) {
                        const float4 s4 = __ldg(reinterpret_cast<const float4 *>(cs + c * 32 + jj));
                        ys[sl][jj] *= s4.x;
                        ys[sl][jj + 1] *= s4.y;
                        ys[sl][jj + 2] *= s4.z;
                        ys[sl][jj + 3] *= s4.w;
                    }
                }
                float v[32];
                tmem_ld32(acc + c * 32, v);
#pragma unroll
                for (int jj = 0; jj < 32; jj++) part = fmaf(v[jj], ys[sl][jj], part);
                if (TWO) {
                    // cross products: lo parts carry a factor 2^11
                    float w[32];
                    tmem_ld32(acc + BN + c * 32, w);
                    float pw = 0.f;
#pragma unroll
                    for (int jj = 0; jj < 32; jj++) pw = fmaf(w[jj], ys[sl][jj], pw);
                    part = fmaf(pw, 1.0f / 2048.0f, part);
                }
                if (c + NSL < NCH) {
#pragma unroll
                    for (int jj = 0; jj < 32; jj++)
                        ys[sl][jj] = live ? __ldg(Yc + (long)((c + NSL) * 32 + jj) * a.ldy) : 0.f;
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                if (PAIR) mbar_arrive_remote(acce0 + (uint32_t)(buf * 8));
                else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&acce[buf])) : "memory");
            }
            if (live) atomicAdd(a.out + row * a.nout + outcol, part);
            j++;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // every MMA into this CTA's TMEM has completed before it is freed
        mbar_wait(mdone, 0, a.err, 6);
        // error path only: wait (bounded) for the copies still in flight
        if (leader)
            for (long g = consumed_s; g < issued_s; g++)
                mbar_wait(&full[g % TSTAGES], (uint32_t)((g / TSTAGES) & 1), a.err, 4);
    }
    __syncthreads();
    // neither CTA of a pair leaves while the other may still address it
    if (PAIR) cluster_sync_all();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (PAIR)
            asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem));
        else
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem));
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled get_encode() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
    }
    return fn;
}

// 2-D K-major map of a [rows][cols] 16-bit matrix, box {64, box_rows}, 128B swizzle
static int make_map(CUtensorMap *m, const void *base, long rows, long cols, int box_rows, bool fp16) {
    EncodeTiled enc = get_encode();
    if (!enc) return E_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)TBK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                     const_cast<void *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? OK : E_CUDA;
}

// ---------------------------------------------------------------------------
// A quadratic form on the tensor cores: the split W operand of nblk blocks
// and the per-block map (X half, Y half, output column).
// ---------------------------------------------------------------------------
int launch_phasors_public(const DevSea &sea, long n, const double *x, const double *y, const double *t,
                          long sx, long sy, long st, int npad, float2 *ph, float *rr, double *first,
                          cudaStream_t stream);

void tcform_free(TcForm &f) {
    void *q[] = {f.Whi, f.Wlo, f.colscale, f.bmap, f.err, f.scratch};
    for (void *p : q) if (p) cudaFree(p);
    for (void *e : f.ev) if (e) cudaEventDestroy((cudaEvent_t)e);
    if (f.aux) cudaStreamDestroy((cudaStream_t)f.aux);
    f = TcForm();
}

// coef64: [nblk][npad (output column m)][npad (K index i)] FP64, W transposed.
int tcform_split(TcForm &f, const double *coef64, const int *bmap_host, int nblk, int nout, int npad, bool fp16,
                 void *stream_, bool one_acc) {
    cudaStream_t stream = (cudaStream_t)stream_;
    tcform_free(f);
    if (npad % TBN != 0 || nblk < 1) return E_BAD_ARGUMENT;
    f.npad = npad; f.nblk = nblk; f.nout = nout; f.fp16 = fp16; f.one_acc = fp16 && one_acc;
    size_t wel = (size_t)nblk * npad * npad;
    CK(cudaMalloc(&f.Whi, 2 * wel));
    CK(cudaMalloc(&f.Wlo, 2 * wel));
    CK(cudaMalloc(&f.colscale, sizeof(float) * nblk * npad));
    CK(cudaMalloc(&f.bmap, sizeof(int) * 3 * nblk));
    CK(cudaMemcpyAsync(f.bmap, bmap_host, sizeof(int) * 3 * nblk, cudaMemcpyHostToDevice, stream));
    dim3 gt((unsigned)npad, (unsigned)nblk);
    if (fp16)
        k_qform_split<__half><<<gt, 256, 0, stream>>>(npad, 1, f.one_acc ? 1.0 : 2048.0, coef64, (__half *)f.Whi,
                                                      (__half *)f.Wlo, f.colscale);
    else
        k_qform_split<__nv_bfloat16><<<gt, 256, 0, stream>>>(npad, 0, 1.0, coef64, (__nv_bfloat16 *)f.Whi,
                                                             (__nv_bfloat16 *)f.Wlo, f.colscale);
    note_launch();
    CK(cudaGetLastError());
    CK(cudaMalloc(&f.err, sizeof(int)));
    CK(cudaMemsetAsync(f.err, 0, sizeof(int), stream));
    CK(cudaStreamSynchronize(stream));
    f.built = true;
    return OK;
}

// Launches the GEMM of one chunk: as many CTAs (or CTA pairs) as fit on the
// device at once (one CTA per SM), at most one per tile unit.
// CTAs (or CTA pairs) of this form that fit on the device at once; set and
// queried once per process (thread-safe static initialisation); <= 0: none.
// Row blocks per tile group of the tile walk (the group sweeps every column
// tile while its rows of X and Y stay in L2); CFDWM_TC_GROUP overrides it.
static int tc_group_m() {
    static const int g = [] {
        const char *e = std::getenv("CFDWM_TC_GROUP");
        int v = e ? std::atoi(e) : 8;
        return v >= 2 && v <= 512 ? v : 8;
    }();
    return g;
}

template <int BN, bool TWO, bool PAIR>
static int tc_max_units() {
    using CF = TcCfg<BN, TWO, PAIR>;
    // computed on the device current at the first call and kept for the
    // process (the library serves one device: the model's)
    static const int maxunits = [] {
        if (cudaFuncSetAttribute(k_qform_tc<BN, TWO, PAIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM) !=
            cudaSuccess) {
            cudaGetLastError();     // a failure here only selects the other form
            return -1;
        }
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        if (!PAIR) return nsm;
        cudaLaunchConfig_t c = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        c.gridDim = dim3((unsigned)(2 * (nsm / 2)));
        c.blockDim = dim3(TC_THREADS);
        c.dynamicSmemBytes = CF::SMEM;
        c.attrs = at;
        c.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_qform_tc<BN, TWO, PAIR>, &c) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        return n;
    }();
    return maxunits;
}

template <int BN, bool TWO, bool PAIR>
static int launch_tc(const CUtensorMap &mXh, const CUtensorMap &mXl, const CUtensorMap &mWh, const CUtensorMap &mWl,
                     const QTC &q, long nunits, cudaStream_t stream) {
    using CF = TcCfg<BN, TWO, PAIR>;
    const int maxunits = tc_max_units<BN, TWO, PAIR>();
    if (maxunits <= 0) {
        std::fprintf(stderr, "cfdwm: the tensor-core form (pair %d) does not fit on this device\n", (int)PAIR);
        return E_CUDA;
    }
    const long nu = std::min<long>(nunits, maxunits);
    if (!PAIR) {
        k_qform_tc<BN, TWO, false><<<(unsigned)nu, TC_THREADS, CF::SMEM, stream>>>(mXh, mXl, mWh, mWl, q);
    } else {
        cudaLaunchConfig_t c = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        c.gridDim = dim3((unsigned)(nu * 2));
        c.blockDim = dim3(TC_THREADS);
        c.dynamicSmemBytes = CF::SMEM;
        c.stream = stream;
        c.attrs = at;
        c.numAttrs = 1;
        CK(cudaLaunchKernelEx(&c, k_qform_tc<BN, TWO, true>, mXh, mXl, mWh, mWl, q));
    }
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

// The GEMM on CTA pairs (cta_group::2) or on single CTAs; CFDWM_TC_PAIR=0 or 1
// overrides the default.  The results do not depend on it beyond the order of
// the epilogue's atomic adds.
static bool tc_pair() {
    const char *e = std::getenv("CFDWM_TC_PAIR");
    if (e && (e[0] == '0' || e[0] == '1') && e[1] == 0) return e[0] == '1';
    return true;
}

static int tc_reserve(TcForm &f, size_t bytes) {
    if (f.scratch_bytes >= bytes) return OK;
    if (f.scratch) cudaFree(f.scratch);
    f.scratch = nullptr;
    f.scratch_bytes = 0;
    CK(cudaMalloc(&f.scratch, bytes));
    f.scratch_bytes = bytes;
    return OK;
}

// out [n][nout] FP32 (zeroed here, then accumulated): the nout quadratic forms
// of the points (x, y, t[p * st]).
int tcform_eval(TcForm &f, const DevSea &sea, long n, const double *x, const double *y, const double *t, long st,
                float *out, void *stream_, int *tc_error) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!f.built) return E_NOT_INITIALIZED;
    if (n <= 0) return OK;
    const int npad = f.npad;
    if (npad < sea.n) return E_BAD_ARGUMENT;
    CK(cudaMemsetAsync(out, 0, sizeof(float) * f.nout * n, stream));
    const long chunk = 1L << 16;
    long m = std::min(n, chunk);
    long mpad = ((m + TBM - 1) / TBM) * TBM;
    size_t xb = (size_t)mpad * 2 * npad * 2;     // one 16-bit matrix
    size_t yb = (size_t)mpad * 2 * npad * 4;
    // several chunks: two operand buffers, the next chunk's operands prepared
    // on a second stream, so that preparation and GEMM of neighbouring chunks
    // overlap where the SMs have room (measured: 1277 against 1323 ms per step
    // of 4e6 points)
    const int nbuf = n > chunk ? 2 : 1;
    const size_t bufb = ((2 * xb + yb + sizeof(QRow) * chunk + sizeof(QComp) * npad + 4095) / 4096) * 4096;
    int rc = tc_reserve(f, nbuf * bufb);
    if (rc) return rc;
    cudaStream_t pst = stream;
    cudaEvent_t *ev = (cudaEvent_t *)f.ev;
    if (nbuf == 2) {
        if (!f.aux) {
            cudaStream_t a2;
            CK(cudaStreamCreateWithFlags(&a2, cudaStreamNonBlocking));
            f.aux = a2;
            for (int e = 0; e < 5; e++) CK(cudaEventCreateWithFlags(&ev[e], cudaEventDisableTiming));
        }
        pst = (cudaStream_t)f.aux;
        CK(cudaEventRecord(ev[0], stream));          // inputs and the zeroed output are ordered before
        CK(cudaStreamWaitEvent(pst, ev[0], 0));
    }
    const int BN = 256;
    // CTA pairs where two-CTA clusters fit on the device, else single CTAs
    // two accumulators (hi, cross) for the fp16 split unless the form keeps
    // the cross products in the hi accumulator
    const bool two = f.fp16 && !f.one_acc;
    const bool pair = tc_pair() && (two ? tc_max_units<256, true, true>() : tc_max_units<256, false, true>()) > 0;
    const int CSZ = pair ? 2 : 1;
    int j = 0;
    for (long b = 0; b < n; b += chunk, j++) {
        long mm = std::min(chunk, n - b);
        const int buf = j % nbuf;
        char *base = (char *)f.scratch + buf * bufb;
        // this buffer's previous GEMM has finished reading it
        if (nbuf == 2 && j >= 2) CK(cudaStreamWaitEvent(pst, ev[3 + buf], 0));
        void *Xh = base, *Xl = base + xb;
        float *Y = (float *)(base + 2 * xb);
        QRow *rowrec = (QRow *)(base + 2 * xb + yb);
        QComp *comprec = (QComp *)(base + 2 * xb + yb + sizeof(QRow) * chunk);
        k_qform_rows<<<(unsigned)((mm + 255) / 256), 256, 0, pst>>>(mm, x + b, y + b, t + b * st, st, sea.fx,
                                                                    sea.fy, sea.d_phase, sea.npad_g, rowrec);
        note_launch();
        k_qform_comps<<<(unsigned)((npad + 255) / 256), 256, 0, pst>>>(sea.n, npad, sea.d_phase, sea.npad_g,
                                                                       comprec);
        note_launch();
        QPrep pp;
        pp.rows = mm; pp.row = rowrec; pp.comp = comprec; pp.phase = sea.d_phase; pp.t = t + b * st; pp.st = st;
        pp.cstride = sea.npad_g; pp.ncomp = sea.n; pp.npad = npad;
        pp.trivial_ramp = sea.trivial_ramp ? 1 : 0; pp.fp16 = f.fp16 ? 1 : 0;
        pp.lo_scale = two ? 2048.0f : 1.0f;
        pp.Xhi = Xh; pp.Xlo = Xl; pp.Y = Y; pp.ldy = mpad;
        // a full grid: with two blocks per SM beside the GEMM the preparation
        // ran latency-bound at a tenth of its speed and became the bottleneck
        k_qform_prep<<<dim3((unsigned)(npad / 256), (unsigned)((mm + PREP_ROWS - 1) / PREP_ROWS)), 128, 0, pst>>>(pp);
        note_launch();
        CK(cudaGetLastError());
        if (nbuf == 2) {
            CK(cudaEventRecord(ev[1 + buf], pst));
            CK(cudaStreamWaitEvent(stream, ev[1 + buf], 0));
        }
        CUtensorMap mXh, mXl, mWh, mWl;
        if (make_map(&mXh, Xh, mm, 2L * npad, TBM, f.fp16) || make_map(&mXl, Xl, mm, 2L * npad, TBM, f.fp16) ||
            make_map(&mWh, f.Whi, (long)f.nblk * npad, npad, BN / CSZ, f.fp16) ||
            make_map(&mWl, f.Wlo, (long)f.nblk * npad, npad, BN / CSZ, f.fp16))
            return E_CUDA;
        QTC q;
        q.rows = mm; q.npad = npad; q.ntn = npad / BN; q.group_m = tc_group_m(); q.nblk = f.nblk; q.nout = f.nout;
        q.bmap = f.bmap; q.Y = Y; q.ldy = mpad; q.colscale = f.colscale;
        q.out = out + (long)f.nout * b; q.fp16 = f.fp16 ? 1 : 0; q.err = f.err;
        // column units: each column tile's upper-triangle K range, cut into
        // segments of at most f.kseg K blocks when the form asks for it
        // (a column tile keeps its whole range where its segments would not
        // fit the table: at most QTC_MAXCU / ntn segments per tile)
        q.ncu = q.ntn;
        q.seg = 0;
        if (f.kseg > 0 && q.ntn <= QTC_MAXCU) {
            q.ncu = 0;
            q.seg = 1;
            for (int tn = 0; tn < q.ntn; tn++) {
                const int nkb = (tn * BN + BN) / TBK;
                int nseg = (nkb + f.kseg - 1) / f.kseg;
                if (q.ntn * nseg > QTC_MAXCU) nseg = 1;
                for (int sg = 0; sg < nseg; sg++) {
                    q.cu_tn[q.ncu] = (unsigned short)tn;
                    q.cu_kb0[q.ncu] = (unsigned short)(nkb * sg / nseg);
                    q.cu_kb1[q.ncu] = (unsigned short)(nkb * (sg + 1) / nseg);
                    q.ncu++;
                }
            }
        }
        long nrb = (mm + TBM - 1) / TBM;
        long nunits = (nrb + CSZ - 1) / CSZ * (long)f.nblk * q.ncu;
        prof_begin(PK_QFORM, stream);
        if (!two)
            rc = pair ? launch_tc<256, false, true>(mXh, mXl, mWh, mWl, q, nunits, stream)
                      : launch_tc<256, false, false>(mXh, mXl, mWh, mWl, q, nunits, stream);
        else
            rc = pair ? launch_tc<256, true, true>(mXh, mXl, mWh, mWl, q, nunits, stream)
                      : launch_tc<256, true, false>(mXh, mXl, mWh, mWl, q, nunits, stream);
        prof_end(PK_QFORM, stream);
        if (rc) return rc;
        if (nbuf == 2) CK(cudaEventRecord(ev[3 + buf], stream));
    }
    if (tc_error) {
        int h = 0;
        CK(cudaMemcpyAsync(&h, f.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        *tc_error = h;
    }
    return OK;
}

// ---------------------------------------------------------------------------
// The precision form of the API: eight blocks (eta, u, v, w) x (cos, sin half)
// ---------------------------------------------------------------------------
struct QformState {
    bool built = false;
    int n = 0, npad = 0, ntile_plain = 0;
    float *plain_tab = nullptr;
    TcForm tc;
    void *scratch = nullptr;   // plain-form chunk buffers
    size_t scratch_bytes = 0;
};
static QformState g_q;

int qform_build(const Config &cfg, const DevSea &sea, bool fp16, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    qform_free();
    int n = (int)cfg.omega.size();
    int npad = ((n + TBN - 1) / TBN) * TBN;
    if (npad == 0) npad = TBN;
    g_q.n = n;
    g_q.npad = npad;
    double kmax = 0;
    for (double k : cfg.k) kmax = std::max(kmax, k);
    double *d_in = nullptr;
    size_t nn = (size_t)std::max(n, 1);
    CK(cudaMalloc(&d_in, sizeof(double) * nn * 4));
    const std::vector<double> *src[4] = {&cfg.omega, &cfg.A, &cfg.k, &cfg.theta};
    for (int q = 0; q < 4; q++)
        CK(cudaMemcpyAsync(d_in + q * nn, src[q]->data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream));
    QIn qi;
    qi.n = n; qi.omega = d_in; qi.A = d_in + nn; qi.k = d_in + 2 * nn; qi.theta = d_in + 3 * nn;
    qi.depth = cfg.depth; qi.g = cfg.gravity; qi.mtheta_rad = cfg.mtheta * PI_IRR / 180.0;
    qi.cutoff = cfg.dw_cutoff; qi.bandwidth = cfg.dw_bandwidth; qi.kmax = kmax;
    // FP64 coefficients of all pairs (temporary), then the plain tiles and
    // the split tensor-core operand from them
    size_t wel = (size_t)8 * npad * npad;
    double *coef = nullptr;
    CK(cudaMalloc(&coef, sizeof(double) * wel));
    long tot = (long)npad * npad;
    k_qform_coef64<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(qi, npad, coef);
    note_launch();
    CK(cudaGetLastError());
    int nt = npad / QT;
    g_q.ntile_plain = nt;
    long ntiles = qtile_index(nt - 1, nt - 1, nt) + 1;
    CK(cudaMalloc(&g_q.plain_tab, sizeof(float) * ntiles * QT * QT * QNC));
    k_qform_plain_from64<<<(unsigned)ntiles, 256, 0, stream>>>(npad, nt, coef, g_q.plain_tab);
    note_launch();
    CK(cudaGetLastError());
    // block b: field (b & 3) -- eta, u, v, w -- X half (b >> 2); the w blocks
    // take the other half of Y (sin(a +- b) = s c +- c s)
    int bmap[24];
    for (int b = 0; b < 8; b++) {
        int field = b & 3, kh = b >> 2;
        bmap[3 * b] = kh;
        bmap[3 * b + 1] = field == 3 ? 1 - kh : kh;
        bmap[3 * b + 2] = field;
    }
    // fp16: the cross products in the hi accumulator over K segments of at
    // most 8 blocks (512 terms), so that the FP32 accumulation keeps their
    // bits, and two TMEM buffers that hide each unit's epilogue (4096
    // components at 1e6 points: the same cycles per step with 8, 16, 32 or 64
    // blocks, the largest error against FP64 3.3e-6, 4.3e-6, 6.4e-6, 1.3e-5;
    // the second accumulator over the whole K range, 5.1e-6 and 7 % more
    // cycles).  CFDWM_QFORM_TWO_ACC=1 restores that arrangement,
    // CFDWM_QFORM_KSEG sets the segment length.
    const char *e2 = std::getenv("CFDWM_QFORM_TWO_ACC");
    const bool one_acc = fp16 && !(e2 && e2[0] == '1');
    int rc = tcform_split(g_q.tc, coef, bmap, 8, 4, npad, fp16, stream, one_acc);
    if (one_acc) {
        const char *ek = std::getenv("CFDWM_QFORM_KSEG");
        g_q.tc.kseg = ek ? std::atoi(ek) : 8;
    }
    cudaFree(coef);
    cudaFree(d_in);
    if (rc) return rc;
    g_q.built = true;
    (void)sea;
    return OK;
}

void qform_free() {
    if (g_q.plain_tab) cudaFree(g_q.plain_tab);
    if (g_q.scratch) cudaFree(g_q.scratch);
    tcform_free(g_q.tc);
    g_q = QformState();
}

static int reserve_scratch(size_t bytes) {
    if (g_q.scratch_bytes >= bytes) return OK;
    if (g_q.scratch) cudaFree(g_q.scratch);
    g_q.scratch = nullptr;
    g_q.scratch_bytes = 0;
    CK(cudaMalloc(&g_q.scratch, bytes));
    g_q.scratch_bytes = bytes;
    return OK;
}

// out [rows][4] FP32: eta2, u2, v2, w2 at z0 = 0 (no ramp of the API, no
// first order).  method 0 plain FP32, 1 tensor cores.
int qform_eval(const DevSea &sea, long n, const double *x, const double *y, const double *t, int method,
               float *out, void *stream_, int *tc_error) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!g_q.built) return E_NOT_INITIALIZED;
    if (n <= 0) return OK;
    const int npad = g_q.npad;
    if (method == 1) return tcform_eval(g_q.tc, sea, n, x, y, t, 1, out, stream, tc_error);
    CK(cudaMemsetAsync(out, 0, sizeof(float) * 4 * n, stream));
    const long chunk = 1L << 16;
    // one-time, thread-safe (static initialisation)
    static const cudaError_t pattr =
        cudaFuncSetAttribute(k_qform_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, QPLAIN_SMEM);
    CK(pattr);
    // two blocks of the kernel fit an SM (registers, shared memory)
    static const int slots = [] {
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return 2 * 148;
        }
        return 2 * nsm;
    }();
    const int nt = g_q.ntile_plain;
    long m = std::min(n, chunk);
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    const size_t b_ph = up(sizeof(float2) * npad * m), b_rr = up(sizeof(float) * npad * m),
                 b_first = up(sizeof(double) * 5 * m);
    int rc = reserve_scratch(b_ph + b_rr + b_first + sizeof(float) * 4 * (size_t)QPL_MAXSEG * m);
    if (rc) return rc;
    for (long b = 0; b < n; b += chunk) {
        long mm = std::min(chunk, n - b);
        float2 *ph = (float2 *)g_q.scratch;
        float *rr = (float *)((char *)g_q.scratch + b_ph);
        double *first = (double *)((char *)rr + b_rr);
        float *part = (float *)((char *)first + b_first);
        rc = launch_phasors_public(sea, mm, x + b, y + b, t + b, 1, 1, 1, npad, ph, rr, first, stream);
        if (rc) return rc;
        // The tile walk of a row block is cut into nseg segments of about equal
        // work (at column-tile boundaries), so that the units -- row blocks x
        // segments -- fill whole waves of the SMs' two block slots: nseg is the
        // count in [4, 32] (at most one per column tile) whose waves are fullest.
        const long nrb = (mm + QPL_ROWS - 1) / QPL_ROWS;
        int nseg = 1;
        double best = 0.0;
        for (int g = 4; g <= std::min(QPL_MAXSEG, nt); g++) {
            const long units = nrb * g;
            const double fill = (double)units / (double)(((units + slots - 1) / slots) * slots);
            if (fill > best + 1e-9) { best = fill; nseg = g; }
        }
        QPlain q;
        q.rows = mm; q.ntile = nt; q.tab = g_q.plain_tab; q.ph = ph; q.rr = rr; q.part = part;
        q.nseg = nseg;
        const long total = (long)nt * (nt + 1) / 2;
        q.mb[0] = 0;
        int M = 0;
        long acc = 0;
        for (int g = 1; g < nseg; g++) {
            const long target = total * g / nseg;
            while (M < nt && acc + (M + 1) <= target) { acc += M + 1; M++; }
            q.mb[g] = std::max(M, q.mb[g - 1]);
        }
        q.mb[nseg] = nt;
        prof_begin(PK_QFORM, stream);
        k_qform_plain<<<(unsigned)(nrb * nseg), 128, QPLAIN_SMEM, stream>>>(q);
        note_launch();
        k_qform_plain_sum<<<(unsigned)((mm * 4 + 255) / 256), 256, 0, stream>>>(mm, nseg, part, out + 4 * b);
        note_launch();
        prof_end(PK_QFORM, stream);
        CK(cudaGetLastError());
    }
    return OK;
}

}  // namespace cfdwm
