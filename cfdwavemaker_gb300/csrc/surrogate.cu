// Learned s-grid update: a small convolutional operator over the grid's
// columns that predicts the second-order part of a ring slot from first-order
// channels, with the plain second-order method as its fallback and judge.
//
// The plain ring update (lsgrid_spline.cpp:847-931, columns :880-903) fills a
// slot with eta = eta1 + eta2 + swl and, at 16 stretched levels placed under
// that eta, U = first order + second order (uvw2, Irregular.cpp:975-1102) +
// the Taylor term above swl.  Its cost is the second-order pair sum
// (P ~ N^2 / 2 pairs per node).  This file replaces that sum, between full
// plain updates, by
//
//   features  first-order channels of every column on a grid extended by a
//             4-column halo: at the 16 levels placed under eta1 alone,
//             u, v, w and the hydrodynamic pressure head, each as the in-phase
//             sum (cos of the component phase) and its quadrature (the phase
//             shifted by -pi/2), scaled by the sea's first-order scales.
//             Products of in-phase and quadrature channels give exactly the
//             cos(phi_i +- phi_m) terms of the Sharma-Dean sums.
//   network   4 valid 3x3 convolutions (8 nl -> 32 -> 32 -> 32 -> 1 + 3 nl),
//             SiLU between them, BF16 weights, FP32 accumulation; the halo
//             makes the output exactly the grid's nx x ny columns.
//   output    eta2 and U - U1(levels under eta1) per level, scaled by the
//             second-order scales k sigma^2 and k sigma^2 omega.
//
// Training (forward, backward, Adam) runs on these kernels too; the training
// pairs are ring slots that the plain method filled.  Every surrogate step can
// be checked against the plain method on a sample of columns; when the
// sampled error exceeds the tolerance the plain method fills the slot.
//
// GB300 notes: the convolutions (forward, data and weight gradients) run as
// implicit GEMMs on the tcgen05 tensor cores (convtc.cu), with the FP32
// activations split into BF16 hi + lo parts and FP32 accumulation in TMEM.
// The features form their phases in float-float arithmetic in the kernel (no
// FP64 phasor table of the halo grid).
#include "cfdwm.h"
#include "ffmath.cuh"
#include "sgrid_geom.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
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

GridGeom grid_geom(const DevGrid &g);

// convtc.cu: valid 3x3 convolutions on the tcgen05 tensor cores
int conv_tc_forward(const float *x, long xbs, const int *idx, const __nv_bfloat16 *w, const float *bias, int B,
                    int C, int O, int H, int W, float *y, float *pre, int act, void *stream);
int conv_tc_data_grad(const float *dy, const __nv_bfloat16 *w, const float *pre, int B, int C, int O, int H, int W,
                      float *dx, void *stream);
long conv_tc_wgt_slabs(int B, int H, int W, int *kslab, int *per_img);
int conv_tc_weight_grad(const float *x, long xbs, const int *idx, const float *dy, int B, int C, int O, int H, int W,
                        float *part, void *stream);
int conv_tc_error(void *stream);

namespace {

constexpr int SH = 4;        // halo columns per side: 4 valid 3x3 convolutions
constexpr int NQ = 8;        // first-order channels per level
constexpr int HID = 32;      // hidden channels
constexpr float LOG2E = 1.4426950408889634f;


__device__ __forceinline__ float ex2f(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---------------------------------------------------------------------------
// First-order channels
// ---------------------------------------------------------------------------
struct FeatArgs {
    GridGeom g;
    int nxh, nyh;
    long ncolh;
    const double *xy;      // [2][ncolh] coordinates of the halo columns
    double t, fx, fy;
    const double *phase;   // [7][cstride]: kx, ky, omega, phase0, ramp parameters
    int trivial_ramp;
    const double *first;   // [5][ncolh]: eta1, phi1_dxdz, phi1_dydz, phi1_dzdz, dp1_dz
    const float *cf;
    int cstride, ncomp;
    float inv_su, inv_sp;  // 1 / (sigma omega_m), 1 / sigma
    float *feat;           // [NQ nl][ncolh]
    float *base;           // [3][nx ny nl] first order with the Taylor term (interior), or null
    float *eta1;           // [nx ny] (interior), or null
    const void *recs;      // this launch's component records (SurrRec, ncomp of them)
};

constexpr int FC = 128;      // components per shared-memory chunk

// a component's record: float-pair phase coefficients and ramp at the
// launch's time, then k, cu, cv, cw, cp
struct SurrRec {
    FfComp f;
    float c[5];
};
static_assert(sizeof(SurrRec) == DF_COMP_FLOATS * sizeof(float), "component record size");

// The records of all components, one thread each: the FP64 phase rows and
// ramps converted once per launch instead of in every block (FP64 runs at a
// small fraction of the FP32 rate on this GPU).
__global__ void k_surr_recs(FeatArgs a, SurrRec *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.ncomp) return;
    const int cs = a.cstride;
    SurrRec d;
    d.f = ff_component(a.phase, cs, i, a.trivial_ramp, a.t);
    const float q = a.cf[CF_Q * cs + i];
    const float au = a.cf[CF_AU * cs + i] * q;
    d.c[0] = a.cf[CF_K * cs + i];
    d.c[1] = au * a.cf[CF_CT * cs + i];
    d.c[2] = au * a.cf[CF_ST * cs + i];
    d.c[3] = au;
    d.c[4] = a.cf[CF_A * cs + i] * q;
    out[i] = d;
}

// blockDim = 32 columns x ceil(nl / 4) level groups of 4 levels.  The warps
// hold the same 32 columns: each forms the float-float phasors of every
// nw-th component of a chunk into shared memory, and all of them read the
// whole chunk, so a (column, component) phasor is formed once per block.
__global__ void __launch_bounds__(256) k_surr_features(FeatArgs a) {
    __shared__ FfComp s_f[FC];
    __shared__ float s_c[5][FC];         // k, cu, cv, cw, cp of the chunk's components
    __shared__ float2 s_ph[FC][32];      // (r cos, r sin) of (component, column)
    const int cl = threadIdx.x & 31, lg = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long p = (long)blockIdx.x * 32 + cl;
    const bool valid = p < a.ncolh;
    const long pc = valid ? p : 0;
    const GridGeom &g = a.g;
    float dxh, dxl, dyh, dyl, th, tl;
    ff_split(a.xy[pc] - a.fx, dxh, dxl);
    ff_split(a.xy[a.ncolh + pc] - a.fy, dyh, dyl);
    ff_split(a.t, th, tl);
    const double e1 = a.first[pc];
    float zk[4], yk[4], za[4];
#pragma unroll
    for (int l = 0; l < 4; l++) {
        int m = lg * 4 + l;
        double z = d_sigmaS2cart(g, m < g.nl ? m : g.nl - 1, e1 + g.swl);
        double z0 = fmin(0.0, z);
        za[l] = (float)fmax(0.0, z - g.swl);
        zk[l] = (float)z0 * LOG2E;
        yk[l] = -((float)z0 + 2.f * (float)g.depth) * LOG2E;
    }
    float acc[4][NQ];
#pragma unroll
    for (int l = 0; l < 4; l++)
#pragma unroll
        for (int q = 0; q < NQ; q++) acc[l][q] = 0.f;
    for (int i0 = 0; i0 < a.ncomp; i0 += FC) {
        __syncthreads();
        for (int e = threadIdx.x; e < FC; e += blockDim.x) {
            const int i = i0 + e;
            SurrRec d = {};
            if (i < a.ncomp) d = reinterpret_cast<const SurrRec *>(a.recs)[i];
            s_f[e] = d.f;
            s_c[0][e] = d.c[0]; s_c[1][e] = d.c[1]; s_c[2][e] = d.c[2]; s_c[3][e] = d.c[3]; s_c[4][e] = d.c[4];
        }
        __syncthreads();
        const int iend = min(FC, a.ncomp - i0);
        for (int ii = lg; ii < iend; ii += nw) {
            float c, sn;
            ff_phasor(s_f[ii], dxh, dxl, dyh, dyl, th, tl, c, sn);
            s_ph[ii][cl] = make_float2(s_f[ii].r * c, s_f[ii].r * sn);
        }
        __syncthreads();
        for (int ii = 0; ii < iend; ii++) {
            const float2 pv = s_ph[ii][cl];
            const float rc = pv.x, rs = pv.y;
            const float k = s_c[0][ii];
            const float q0 = s_c[1][ii] * rc, q1 = s_c[1][ii] * rs;
            const float q2 = s_c[2][ii] * rc, q3 = s_c[2][ii] * rs;
            const float q4 = s_c[3][ii] * rs, q5 = -s_c[3][ii] * rc;
            const float q6 = s_c[4][ii] * rc, q7 = s_c[4][ii] * rs;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                // profile factors with the normaliser in the coefficient:
                // cosh(k(z+h))/cosh(kh) = q (E + Y), sinh(k(z+h))/cosh(kh) = q (E - Y)
                const float E = ex2f(k * zk[l]), Y = ex2f(k * yk[l]);
                const float F = E + Y, G = E - Y;
                acc[l][0] = fmaf(q0, F, acc[l][0]);
                acc[l][1] = fmaf(q1, F, acc[l][1]);
                acc[l][2] = fmaf(q2, F, acc[l][2]);
                acc[l][3] = fmaf(q3, F, acc[l][3]);
                acc[l][4] = fmaf(q4, G, acc[l][4]);
                acc[l][5] = fmaf(q5, G, acc[l][5]);
                acc[l][6] = fmaf(q6, F, acc[l][6]);
                acc[l][7] = fmaf(q7, F, acc[l][7]);
            }
        }
    }
    if (!valid) return;
    const int ih = (int)(p / a.nyh), jh = (int)(p % a.nyh);
    const int i = ih - SH, j = jh - SH;
    const bool inner = i >= 0 && i < g.nx && j >= 0 && j < g.ny;
    const long c = (long)i * g.ny + j;
    const long nxy = (long)g.nx * g.ny;
#pragma unroll
    for (int l = 0; l < 4; l++) {
        int m = lg * 4 + l;
        if (m >= g.nl) continue;
#pragma unroll
        for (int q = 0; q < NQ; q++)
            a.feat[(long)(m * NQ + q) * a.ncolh + p] = acc[l][q] * (q < 6 ? a.inv_su : a.inv_sp);
        if (inner && a.base) {
            for (int f = 0; f < 3; f++)
                a.base[(long)f * nxy * g.nl + c * g.nl + m] =
                    acc[l][2 * f] + (float)a.first[(long)(1 + f) * a.ncolh + p] * za[l];
        }
    }
    if (inner && a.eta1 && lg == 0) a.eta1[c] = (float)e1;
}

__global__ void k_halo_coords(GridGeom g, int nxh, int nyh, double *xy) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long n = (long)nxh * nyh;
    if (p >= n) return;
    int ih = (int)(p / nyh), jh = (int)(p % nyh);
    xy[p] = g.d0 + g.dx * (ih - SH);
    xy[n + p] = g.d2 + g.dy * (jh - SH);
}

// grad[e] = sum over slabs of part[slab][e], in slab order
__global__ void k_sum_slabs(long per, int nslab, const float *part, float *gw, float *gb, long nw) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= per) return;
    float s = 0.f;
    for (int k = 0; k < nslab; k++) s += part[(long)k * per + e];
    if (e < nw) gw[e] = s;
    else gb[e - nw] = s;
}

// Weighted mean-square loss and its gradient:
//   L = sum_{b,o,p} w_o (y - t)^2 / (B P sum_o w_o),  dy = 2 w_o (y - t) / (B P sum w)
__global__ void __launch_bounds__(256) k_surr_loss(const float *y, const float *tg, long tbs, const int *idx,
                                                   int B, int O, long P, float w0, float inv_norm, float *dy,
                                                   float *lpart) {
    __shared__ float red[256];
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long n = (long)B * O * P;
    float l = 0.f;
    if (e < n) {
        int b = (int)(e / ((long)O * P));
        long r = e % ((long)O * P);
        int o = (int)(r / P);
        float wo = (o == 0) ? w0 : 1.f;
        float t = tg[(long)(idx ? idx[b] : b) * tbs + r];
        float d = y[e] - t;
        l = wo * d * d * inv_norm;
        if (dy) dy[e] = 2.f * wo * d * inv_norm;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) lpart[blockIdx.x] = red[0];
}

__global__ void k_adam(long n, float lr, float b1, float b2, float eps, float c1, float c2, const float *g,
                       float *w, float *m, float *v, __nv_bfloat16 *wbf, long nweights_bf) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= n) return;
    float gg = g[e];
    float mm = b1 * m[e] + (1.f - b1) * gg;
    float vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    float ww = w[e] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
    w[e] = ww;
    if (e < nweights_bf) wbf[e] = __float2bfloat16_rn(ww);
}

__global__ void k_to_bf16(long n, const float *w, __nv_bfloat16 *wbf) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e < n) wbf[e] = __float2bfloat16_rn(w[e]);
}

// ---------------------------------------------------------------------------
// Slot-side kernels
// ---------------------------------------------------------------------------
// Normalised training targets of ring slot `slot` (all columns):
//   t[0][c] = (ETA - swl - eta1) / s_eta,  t[1 + f nl + m][c] = (U_f - base_f) / s_u
__global__ void k_surr_targets(int nx, int ny, int nl, int slot, float swl, const float *ETA, const float *U0,
                               const float *U1, const float *U2, const float *eta1, const float *base,
                               float inv_eta, float inv_u, float *tg) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long nxy = (long)nx * ny, n = nxy * nl;
    if (e >= n) return;
    long c = e / nl;
    int m = (int)(e % nl);
    const float *U[3] = {U0, U1, U2};
    for (int f = 0; f < 3; f++) {
        float v = U[f][(long)slot * n + e] - base[(long)f * n + e];
        tg[(long)(1 + f * nl + m) * nxy + c] = v * inv_u;
    }
    if (m == 0) tg[c] = (ETA[(long)slot * nxy + c] - swl - eta1[c]) * inv_eta;
}

// Writes the predicted slot for the live columns.
// Writes the predicted slot for the live columns: first order + (network
// output + carried residual R of the last plain slot, when given).
__global__ void k_surr_apply(long nlive, const int *live, int nx, int ny, int nl, int slot, float swl,
                             const float *eta1, const float *base, const float *pred, const float *R,
                             float s_eta, float s_u, float *ETA, float *U0, float *U1, float *U2) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= nlive * nl) return;
    long q = e / nl;
    int m = (int)(e % nl);
    long c = live[q];
    long nxy = (long)nx * ny, n = nxy * nl;
    float *U[3] = {U0, U1, U2};
    for (int f = 0; f < 3; f++) {
        long o = (long)(1 + f * nl + m) * nxy + c;
        float v = pred[o] + (R ? R[o] : 0.f);
        U[f][(long)slot * n + c * nl + m] = base[(long)f * n + c * nl + m] + v * s_u;
    }
    if (m == 0) ETA[(long)slot * nxy + c] = eta1[c] + swl + (pred[c] + (R ? R[c] : 0.f)) * s_eta;
}

// Gaussian low-pass along one grid direction (dir 0: i, 1: j) of [C][nx][ny]
// planes, weights renormalised at the grid edges.
__global__ void k_blur(int C, int nx, int ny, int dir, float inv2s2, int rad, const float *in, float *out) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long nxy = (long)nx * ny;
    if (e >= (long)C * nxy) return;
    long ch = e / nxy, c = e % nxy;
    int i = (int)(c / ny), j = (int)(c % ny);
    const float *pl = in + ch * nxy;
    float acc = 0.f, wsum = 0.f;
    for (int d = -rad; d <= rad; d++) {
        int ii = dir == 0 ? i + d : i, jj = dir == 0 ? j : j + d;
        if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;
        float w = __expf(-(float)(d * d) * inv2s2);
        acc += w * pl[(long)ii * ny + jj];
        wsum += w;
    }
    out[e] = acc / wsum;
}

__global__ void k_sub(long n, const float *b, float *a) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e < n) a[e] -= b[e];
}

__device__ __forceinline__ void atomic_max_pos(unsigned *p, float v) {
    if (!(v >= 0.f)) v = 3.0e38f;   // NaN counts as a failed check
    atomicMax(p, __float_as_uint(v));
}

// Max |slot - reference| over the columns col[0..n) (reference: slot 0 of the
// scratch arrays), eta and each velocity field, normalised.  err: [4] uint.
__global__ void k_surr_compare(long n, const int *col, int nx, int ny, int nl, int slot, const float *ETA,
                               const float *U0, const float *U1, const float *U2, const float *rETA,
                               const float *rU0, const float *rU1, const float *rU2, float inv_eta, float inv_u,
                               unsigned *err) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= n * nl) return;
    long q = e / nl;
    int m = (int)(e % nl);
    long c = col ? col[q] : q;
    long nxy = (long)nx * ny, nn = nxy * nl;
    const float *U[3] = {U0, U1, U2}, *R[3] = {rU0, rU1, rU2};
    for (int f = 0; f < 3; f++)
        atomic_max_pos(err + 1 + f, fabsf(U[f][(long)slot * nn + c * nl + m] - R[f][c * nl + m]) * inv_u);
    if (m == 0) atomic_max_pos(err, fabsf(ETA[(long)slot * nxy + c] - rETA[c]) * inv_eta);
}

// max |ETA - swl| and max |U| over one slot (or slot-0 scratch arrays)
__global__ void k_slot_max(long nxy, int nl, float swl, const float *ETA, const float *U0, const float *U1,
                           const float *U2, unsigned *mx) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long n = nxy * nl;
    if (e >= n) return;
    float u = fmaxf(fabsf(U0[e]), fmaxf(fabsf(U1[e]), fabsf(U2[e])));
    atomic_max_pos(mx + 1, u);
    if (e < nxy) atomic_max_pos(mx, fabsf(ETA[e] - swl));
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct Surrogate {
    bool ready = false;
    int nl = 0, cin = 0, cout = 0;
    int ch[5] = {0, 0, 0, 0, 0};
    long off_w[4] = {0, 0, 0, 0}, off_b[4] = {0, 0, 0, 0}, nparams = 0;
    float *w32 = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
    __nv_bfloat16 *wbf = nullptr;
    long adam_step = 0;
    // training / gradient scratch
    void *tr = nullptr;
    size_t tr_bytes = 0;
    int *d_idx = nullptr;
    int idx_cap = 0;
    // grid-side buffers
    int gnx = 0, gny = 0, gnl = 0;
    const float *g_eta = nullptr;      // identity of the attached grid
    double g_dx = 0, g_dy = 0, g_dom[4] = {0, 0, 0, 0}, g_ign[4] = {0, 0, 0, 0};
    double *xyh = nullptr;
    float *feat = nullptr, *base = nullptr, *eta1 = nullptr, *pred = nullptr, *hbuf = nullptr;
    float *R = nullptr;        // residual (plain - network) of the last plain slot, [cout][nx ny]
    float *Rtmp = nullptr;
    bool have_res = false;
    double carry_lw = 0.0;     // low-pass scale of the carried residual, in mean wavelengths (0: none)
    float *rETA = nullptr, *rU[3] = {nullptr, nullptr, nullptr};
    int *d_sample = nullptr;
    unsigned *d_err = nullptr;
    std::vector<int> live;
    float fmax_eta = 0.f, fmax_u = 0.f;
    unsigned long long rng = 0x2545F4914F6CDD1DULL;
    long steps = 0, fallbacks = 0, plain_steps = 0;
};

static Surrogate g_s;

static void free_grid_side(Surrogate &s) {
    void *q[] = {s.xyh, s.feat, s.base, s.eta1, s.pred, s.hbuf, s.rETA, s.rU[0], s.rU[1], s.rU[2],
                 s.d_sample, s.d_err, s.R, s.Rtmp};
    for (void *p : q) if (p) cudaFree(p);
    s.xyh = nullptr; s.feat = s.base = s.eta1 = s.pred = s.hbuf = s.rETA = s.R = nullptr;
    s.Rtmp = nullptr;
    s.have_res = false;
    s.rU[0] = s.rU[1] = s.rU[2] = nullptr;
    s.d_sample = nullptr; s.d_err = nullptr;
    s.gnx = s.gny = s.gnl = 0;
    s.g_eta = nullptr;
    s.live.clear();
}

static void free_all(Surrogate &s) {
    free_grid_side(s);
    void *q[] = {s.w32, s.m1, s.m2, s.grad, s.wbf, s.tr, s.d_idx};
    for (void *p : q) if (p) cudaFree(p);
    s = Surrogate();
}

// splitmix64 + Box-Muller: the same initial weights on every host
static double rnd_unit(unsigned long long &st) {
    st += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

int surrogate_create(int nl, unsigned long long seed, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (nl < 1 || nl > 32) return E_BAD_ARGUMENT;
    free_all(g_s);
    Surrogate &s = g_s;
    s.nl = nl;
    s.cin = NQ * nl;
    s.cout = 1 + 3 * nl;
    int ch[5] = {s.cin, HID, HID, HID, s.cout};
    std::memcpy(s.ch, ch, sizeof(ch));
    long off = 0;
    // all weight blocks first (they have BF16 copies), then the biases
    for (int l = 0; l < 4; l++) { s.off_w[l] = off; off += (long)ch[l + 1] * ch[l] * 9; }
    for (int l = 0; l < 4; l++) { s.off_b[l] = off; off += ch[l + 1]; }
    s.nparams = off;
    std::vector<float> w(off, 0.f);
    unsigned long long st = seed;
    for (int l = 0; l < 4; l++) {
        double sd = std::sqrt(2.0 / (ch[l] * 9.0)) * (l == 3 ? 0.1 : 1.0);
        for (long e = 0; e < (long)ch[l + 1] * ch[l] * 9; e++) {
            double u1 = rnd_unit(st), u2 = rnd_unit(st);
            w[s.off_w[l] + e] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    CK(cudaMalloc(&s.w32, sizeof(float) * off));
    CK(cudaMalloc(&s.m1, sizeof(float) * off));
    CK(cudaMalloc(&s.m2, sizeof(float) * off));
    CK(cudaMalloc(&s.grad, sizeof(float) * off));
    CK(cudaMalloc(&s.wbf, sizeof(__nv_bfloat16) * s.off_b[0]));
    CK(cudaMemcpyAsync(s.w32, w.data(), sizeof(float) * off, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(s.m1, 0, sizeof(float) * off, stream));
    CK(cudaMemsetAsync(s.m2, 0, sizeof(float) * off, stream));
    k_to_bf16<<<(unsigned)((s.off_b[0] + 255) / 256), 256, 0, stream>>>(s.off_b[0], s.w32, s.wbf);
    note_launch();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    s.ready = true;
    return OK;
}

void surrogate_destroy() { free_all(g_s); }

long surrogate_nparams() { return g_s.ready ? g_s.nparams : 0; }
int surrogate_levels() { return g_s.ready ? g_s.nl : 0; }

int surrogate_get_params(float *dst, long n, void *stream) {
    if (!g_s.ready) return E_NOT_INITIALIZED;
    if (n < g_s.nparams || !dst) return E_BAD_ARGUMENT;
    CK(cudaMemcpyAsync(dst, g_s.w32, sizeof(float) * g_s.nparams, cudaMemcpyDefault, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return OK;
}

int surrogate_set_params(const float *src, long n, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!g_s.ready) return E_NOT_INITIALIZED;
    if (n != g_s.nparams || !src) return E_BAD_ARGUMENT;
    CK(cudaMemcpyAsync(g_s.w32, src, sizeof(float) * n, cudaMemcpyDefault, stream));
    CK(cudaMemsetAsync(g_s.m1, 0, sizeof(float) * n, stream));
    CK(cudaMemsetAsync(g_s.m2, 0, sizeof(float) * n, stream));
    g_s.adam_step = 0;
    k_to_bf16<<<(unsigned)((g_s.off_b[0] + 255) / 256), 256, 0, stream>>>(g_s.off_b[0], g_s.w32, g_s.wbf);
    note_launch();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    return OK;
}

// ---- layer launchers ------------------------------------------------------
// The convolutions run as implicit GEMMs on the tcgen05 tensor cores
// (convtc.cu); the error word of their bounded waits is read where a call
// synchronises anyway.
static int conv_fwd(const Surrogate &s, int l, const float *x, long xbs, const int *idx, int B, int H, int W,
                    float *y, float *pre, int act, cudaStream_t st) {
    return conv_tc_forward(x, xbs, idx, s.wbf + s.off_w[l], s.w32 + s.off_b[l], B, s.ch[l], s.ch[l + 1], H, W, y,
                           pre, act, st);
}

static int conv_bwd_data(const Surrogate &s, int l, const float *dy, const float *pre, int B, int H, int W,
                         float *dx, cudaStream_t st) {
    return conv_tc_data_grad(dy, s.wbf + s.off_w[l], pre, B, s.ch[l], s.ch[l + 1], H, W, dx, st);
}

static long wgt_slabs(int B, int H, int W) { return conv_tc_wgt_slabs(B, H, W, nullptr, nullptr); }

static int conv_bwd_wgt(Surrogate &s, int l, const float *x, long xbs, const int *idx, const float *dy, int B,
                        int H, int W, float *part, cudaStream_t st) {
    const int C = s.ch[l], O = s.ch[l + 1];
    int rc = conv_tc_weight_grad(x, xbs, idx, dy, B, C, O, H, W, part, st);
    if (rc) return rc;
    const long nslab = wgt_slabs(B, H, W);
    long nw = (long)O * C * 9, per = nw + O;
    k_sum_slabs<<<(unsigned)((per + 255) / 256), 256, 0, st>>>(per, (int)nslab, part, s.grad + s.off_w[l],
                                                                s.grad + s.off_b[l], nw);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

static int conv_check(cudaStream_t st) {
    int e = conv_tc_error(st);
    if (e == 0) return OK;
    std::fprintf(stderr, "cfdwm: a bounded wait of the tensor-core convolutions expired (code %d)\n", e);
    return E_CUDA;
}

static int reserve_tr(Surrogate &s, size_t bytes) {
    if (s.tr_bytes >= bytes) return OK;
    if (s.tr) cudaFree(s.tr);
    s.tr = nullptr;
    s.tr_bytes = 0;
    CK(cudaMalloc(&s.tr, bytes));
    s.tr_bytes = bytes;
    return OK;
}

// Forward + loss + backward into s.grad.  x: [*][cin][H][W], tg: [*][cout][H-8][W-8],
// batch entries idx[0..B) (device) or 0..B-1.
static int loss_grad(Surrogate &s, const float *x, const float *tg, const int *idx, int B, int H, int W,
                     double *loss, cudaStream_t st) {
    if (H < 9 || W < 9 || B < 1) return E_BAD_ARGUMENT;
    const long P1 = (long)(H - 2) * (W - 2), P2 = (long)(H - 4) * (W - 4), P3 = (long)(H - 6) * (W - 6),
               P4 = (long)(H - 8) * (W - 8);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t n1 = up(sizeof(float) * B * HID * P1), n2 = up(sizeof(float) * B * HID * P2),
           n3 = up(sizeof(float) * B * HID * P3), n4 = up(sizeof(float) * B * s.cout * P4);
    long maxpart = 0;
    int HH[4] = {H, H - 2, H - 4, H - 6}, WW[4] = {W, W - 2, W - 4, W - 6};
    for (int l = 0; l < 4; l++)
        maxpart = std::max(maxpart, wgt_slabs(B, HH[l], WW[l]) * ((long)s.ch[l + 1] * s.ch[l] * 9 + s.ch[l + 1]));
    long nl4 = ((long)B * s.cout * P4 + 255) / 256;
    size_t npart = up(sizeof(float) * maxpart), nloss = up(sizeof(float) * nl4);
    // a1 h1 a2 h2 a3 h3 y dy da3 da2 da1 part lpart
    size_t bytes = 2 * n1 + 2 * n2 + 2 * n3 + 2 * n4 + n3 + n2 + n1 + npart + nloss;
    int rc = reserve_tr(s, bytes);
    if (rc) return rc;
    char *p = (char *)s.tr;
    float *a1 = (float *)p; p += n1;
    float *h1 = (float *)p; p += n1;
    float *a2 = (float *)p; p += n2;
    float *h2 = (float *)p; p += n2;
    float *a3 = (float *)p; p += n3;
    float *h3 = (float *)p; p += n3;
    float *y = (float *)p; p += n4;
    float *dy = (float *)p; p += n4;
    float *da3 = (float *)p; p += n3;
    float *da2 = (float *)p; p += n2;
    float *da1 = (float *)p; p += n1;
    float *part = (float *)p; p += npart;
    float *lpart = (float *)p;
    const long xbs = (long)s.cin * H * W, tbs = (long)s.cout * P4;
    if ((rc = conv_fwd(s, 0, x, xbs, idx, B, H, W, h1, a1, 1, st))) return rc;
    if ((rc = conv_fwd(s, 1, h1, (long)HID * P1, nullptr, B, H - 2, W - 2, h2, a2, 1, st))) return rc;
    if ((rc = conv_fwd(s, 2, h2, (long)HID * P2, nullptr, B, H - 4, W - 4, h3, a3, 1, st))) return rc;
    if ((rc = conv_fwd(s, 3, h3, (long)HID * P3, nullptr, B, H - 6, W - 6, y, nullptr, 0, st))) return rc;
    const float w0 = (float)s.nl;
    const float inv_norm = (float)(1.0 / ((double)B * P4 * (w0 + (s.cout - 1))));
    k_surr_loss<<<(unsigned)nl4, 256, 0, st>>>(y, tg, tbs, idx, B, s.cout, P4, w0, inv_norm, dy, lpart);
    note_launch();
    CK(cudaGetLastError());
    if ((rc = conv_bwd_wgt(s, 3, h3, (long)HID * P3, nullptr, dy, B, H - 6, W - 6, part, st))) return rc;
    if ((rc = conv_bwd_data(s, 3, dy, a3, B, H - 6, W - 6, da3, st))) return rc;
    if ((rc = conv_bwd_wgt(s, 2, h2, (long)HID * P2, nullptr, da3, B, H - 4, W - 4, part, st))) return rc;
    if ((rc = conv_bwd_data(s, 2, da3, a2, B, H - 4, W - 4, da2, st))) return rc;
    if ((rc = conv_bwd_wgt(s, 1, h1, (long)HID * P1, nullptr, da2, B, H - 2, W - 2, part, st))) return rc;
    if ((rc = conv_bwd_data(s, 1, da2, a1, B, H - 2, W - 2, da1, st))) return rc;
    if ((rc = conv_bwd_wgt(s, 0, x, xbs, idx, da1, B, H, W, part, st))) return rc;
    if (loss) {
        std::vector<float> lp(nl4);
        CK(cudaMemcpyAsync(lp.data(), lpart, sizeof(float) * nl4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        double L = 0.0;
        for (float v : lp) L += v;
        *loss = L;
        return conv_check(st);
    }
    return OK;
}

static int put_idx(Surrogate &s, const int *idx_host, int B, cudaStream_t st) {
    if (s.idx_cap < B) {
        if (s.d_idx) cudaFree(s.d_idx);
        s.d_idx = nullptr;
        CK(cudaMalloc(&s.d_idx, sizeof(int) * B));
        s.idx_cap = B;
    }
    CK(cudaMemcpyAsync(s.d_idx, idx_host, sizeof(int) * B, cudaMemcpyHostToDevice, st));
    return OK;
}

int surrogate_loss_grad(const float *x, const float *tg, int B, int H, int W, double *loss, float *grad,
                        void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    if (!g_s.ready) return E_NOT_INITIALIZED;
    int rc = loss_grad(g_s, x, tg, nullptr, B, H, W, loss, st);
    if (rc) return rc;
    if (grad) CK(cudaMemcpyAsync(grad, g_s.grad, sizeof(float) * g_s.nparams, cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    return OK;
}

int surrogate_train_step(const float *xs, const float *ts, long nsamples, const int *idx_host, int B, int H, int W,
                         float lr, double *loss, void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    if (!s.ready) return E_NOT_INITIALIZED;
    if (!idx_host || B < 1) return E_BAD_ARGUMENT;
    for (int b = 0; b < B; b++)
        if (idx_host[b] < 0 || idx_host[b] >= nsamples) return E_BAD_ARGUMENT;
    int rc = put_idx(s, idx_host, B, st);
    if (rc) return rc;
    rc = loss_grad(s, xs, ts, s.d_idx, B, H, W, loss, st);
    if (rc) return rc;
    s.adam_step++;
    const double b1 = 0.9, b2 = 0.999;
    float c1 = (float)(1.0 / (1.0 - std::pow(b1, (double)s.adam_step)));
    float c2 = (float)(1.0 / (1.0 - std::pow(b2, (double)s.adam_step)));
    k_adam<<<(unsigned)((s.nparams + 255) / 256), 256, 0, st>>>(s.nparams, lr, (float)b1, (float)b2, 1e-8f, c1, c2,
                                                                s.grad, s.w32, s.m1, s.m2, s.wbf, s.off_b[0]);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

int surrogate_check(void *stream) { return conv_check((cudaStream_t)stream); }

int surrogate_forward(const float *x, int B, int H, int W, float *y, void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    if (!s.ready) return E_NOT_INITIALIZED;
    if (H < 9 || W < 9 || B < 1) return E_BAD_ARGUMENT;
    const long P1 = (long)(H - 2) * (W - 2), P2 = (long)(H - 4) * (W - 4), P3 = (long)(H - 6) * (W - 6);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t n1 = up(sizeof(float) * B * HID * P1), n2 = up(sizeof(float) * B * HID * P2),
           n3 = up(sizeof(float) * B * HID * P3);
    int rc = reserve_tr(s, n1 + n2 + n3);
    if (rc) return rc;
    float *h1 = (float *)s.tr, *h2 = (float *)((char *)s.tr + n1), *h3 = (float *)((char *)s.tr + n1 + n2);
    prof_begin(PK_SURR_NET, st);
    if ((rc = conv_fwd(s, 0, x, (long)s.cin * H * W, nullptr, B, H, W, h1, nullptr, 1, st))) return rc;
    if ((rc = conv_fwd(s, 1, h1, (long)HID * P1, nullptr, B, H - 2, W - 2, h2, nullptr, 1, st))) return rc;
    if ((rc = conv_fwd(s, 2, h2, (long)HID * P2, nullptr, B, H - 4, W - 4, h3, nullptr, 1, st))) return rc;
    rc = conv_fwd(s, 3, h3, (long)HID * P3, nullptr, B, H - 6, W - 6, y, nullptr, 0, st);
    prof_end(PK_SURR_NET, st);
    return rc;
}

// ---- grid side ------------------------------------------------------------
// Sea-state scales: sigma^2 = sum A^2 / 2, omega_m and k_m the A^2-weighted means.
static void sea_scales(const Config &cfg, double &sigma, double &om, double &km) {
    double s2 = 0, so = 0, sk = 0;
    for (size_t i = 0; i < cfg.A.size(); i++) {
        double a2 = cfg.A[i] * cfg.A[i];
        s2 += a2;
        so += a2 * cfg.omega[i];
        sk += a2 * cfg.k[i];
    }
    sigma = std::sqrt(0.5 * s2);
    om = s2 > 0 ? so / s2 : 1.0;
    km = s2 > 0 ? sk / s2 : 1.0;
    if (sigma <= 0) sigma = 1.0;
}

// The grid-side buffers follow the grid: their sizes its dimensions, the
// halo coordinates and the live-column list its placement and ignore area.
static bool same_grid(const Surrogate &s, const DevGrid &g) {
    if (!(s.gnx == g.nx && s.gny == g.ny && s.gnl == g.nl && s.feat)) return false;
    if (s.g_eta != g.ETA || s.g_dx != g.dx || s.g_dy != g.dy) return false;
    for (int q = 0; q < 4; q++)
        if (s.g_dom[q] != g.cfg.domain[q] || s.g_ign[q] != g.cfg.domain_ignore[q]) return false;
    return true;
}

static int attach_grid(Surrogate &s, DevGrid &g, cudaStream_t st) {
    if (g.nl != s.nl) return E_BAD_ARGUMENT;
    if (same_grid(s, g)) return OK;
    free_grid_side(s);
    const int nxh = g.nx + 2 * SH, nyh = g.ny + 2 * SH;
    const long nh = (long)nxh * nyh, nxy = (long)g.nx * g.ny, n = nxy * g.nl;
    CK(cudaMalloc(&s.xyh, sizeof(double) * 2 * nh));
    CK(cudaMalloc(&s.feat, sizeof(float) * s.cin * nh));
    CK(cudaMalloc(&s.base, sizeof(float) * 3 * n));
    CK(cudaMalloc(&s.eta1, sizeof(float) * nxy));
    CK(cudaMalloc(&s.pred, sizeof(float) * s.cout * nxy));
    CK(cudaMalloc(&s.R, sizeof(float) * s.cout * nxy));
    CK(cudaMalloc(&s.Rtmp, sizeof(float) * s.cout * nxy));
    CK(cudaMalloc(&s.rETA, sizeof(float) * nxy));
    for (int f = 0; f < 3; f++) CK(cudaMalloc(&s.rU[f], sizeof(float) * n));
    CK(cudaMalloc(&s.d_err, sizeof(unsigned) * 8));
    CK(cudaMalloc(&s.d_sample, sizeof(int) * 4096));
    GridGeom G = grid_geom(g);
    k_halo_coords<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(G, nxh, nyh, s.xyh);
    note_launch();
    CK(cudaGetLastError());
    const int *act;
    long nlive;
    grid_live_columns(g, &act, &nlive);
    s.live.resize(nlive);
    if (nlive) CK(cudaMemcpyAsync(s.live.data(), act, sizeof(int) * nlive, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    s.gnx = g.nx; s.gny = g.ny; s.gnl = g.nl;
    s.g_eta = g.ETA; s.g_dx = g.dx; s.g_dy = g.dy;
    for (int q = 0; q < 4; q++) { s.g_dom[q] = g.cfg.domain[q]; s.g_ign[q] = g.cfg.domain_ignore[q]; }
    s.fmax_eta = s.fmax_u = 0.f;
    s.have_res = false;
    return OK;
}

// First-order channels of the attached grid at time t into s.feat/s.base/s.eta1
// (or the given outputs).
static int features(Surrogate &s, const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, double t,
                    float *feat, float *base, float *eta1, cudaStream_t st) {
    const int nxh = g.nx + 2 * SH, nyh = g.ny + 2 * SH;
    const long nh = (long)nxh * nyh;
    int rc = workspace_reserve(ws, sizeof(double) * 5 * nh);
    if (rc) return rc;
    double *first = (double *)ws.base;
    // eta1 and the Taylor gradients of the halo columns (float-float phases)
    rc = depthform_first(sea, nh, g.nl, s.xyh, t, nullptr, first, nullptr, 3, st);
    if (rc) return rc;
    double sigma, om, km;
    sea_scales(cfg, sigma, om, km);
    FeatArgs a;
    a.g = grid_geom(g);
    a.nxh = nxh; a.nyh = nyh; a.ncolh = nh;
    a.xy = s.xyh; a.t = t; a.fx = sea.fx; a.fy = sea.fy; a.phase = sea.d_phase;
    a.trivial_ramp = sea.trivial_ramp ? 1 : 0;
    a.first = first; a.cf = sea.d_cf; a.cstride = sea.npad_g; a.ncomp = sea.n;
    a.inv_su = (float)(1.0 / (sigma * om));
    a.inv_sp = (float)(1.0 / sigma);
    a.feat = feat; a.base = base; a.eta1 = eta1;
    if (!sea.d_dfcomp) return E_NOT_INITIALIZED;
    SurrRec *recs = reinterpret_cast<SurrRec *>(sea.d_dfcomp) + 2L * sea.npad_g;
    k_surr_recs<<<(unsigned)((sea.n + 127) / 128), 128, 0, st>>>(a, recs);
    note_launch();
    a.recs = recs;
    int ngrp = (g.nl + 3) / 4;
    prof_begin(PK_SURR_FEATURES, st);
    k_surr_features<<<(unsigned)((nh + 31) / 32), 32 * ngrp, 0, st>>>(a);
    note_launch();
    prof_end(PK_SURR_FEATURES, st);
    CK(cudaGetLastError());
    return OK;
}

int surrogate_features(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, double t, float *feat,
                       float *base, float *eta1, void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    if (!s.ready) return E_NOT_INITIALIZED;
    int rc = attach_grid(s, g, st);
    if (rc) return rc;
    return features(s, cfg, sea, g, ws, t, feat ? feat : s.feat, base ? base : s.base, eta1 ? eta1 : s.eta1, st);
}

int surrogate_targets(const Config &cfg, DevGrid &g, int slot, const float *base, const float *eta1, float *tg,
                      void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    if (!s.ready) return E_NOT_INITIALIZED;
    if (slot < 0 || slot > 3 || g.nl != s.nl) return E_BAD_ARGUMENT;
    double sigma, om, km;
    sea_scales(cfg, sigma, om, km);
    const double s_eta = km * sigma * sigma, s_u = s_eta * om;
    long n = (long)g.nx * g.ny * g.nl;
    k_surr_targets<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        g.nx, g.ny, g.nl, slot, (float)g.swl, g.ETA, g.U[0], g.U[1], g.U[2], eta1 ? eta1 : s.eta1,
        base ? base : s.base, (float)(1.0 / s_eta), (float)(1.0 / s_u), tg);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

static int slot_max(Surrogate &s, DevGrid &g, const float *ETA, float *const U[3], cudaStream_t st, float *me,
                    float *mu) {
    long nxy = (long)g.nx * g.ny;
    CK(cudaMemsetAsync(s.d_err, 0, sizeof(unsigned) * 8, st));
    k_slot_max<<<(unsigned)((nxy * g.nl + 255) / 256), 256, 0, st>>>(nxy, g.nl, (float)g.swl, ETA, U[0], U[1], U[2],
                                                                      s.d_err + 4);
    note_launch();
    CK(cudaGetLastError());
    unsigned h[2];
    CK(cudaMemcpyAsync(h, s.d_err + 4, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(me, &h[0], 4);
    std::memcpy(mu, &h[1], 4);
    return OK;
}

// Predicts slot `slot` at time t for the live columns.
static int predict_slot(Surrogate &s, const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, int slot,
                        double t, bool carry, cudaStream_t st) {
    int rc = features(s, cfg, sea, g, ws, t, s.feat, s.base, s.eta1, st);
    if (rc) return rc;
    const int nxh = g.nx + 2 * SH, nyh = g.ny + 2 * SH;
    rc = surrogate_forward(s.feat, 1, nxh, nyh, s.pred, st);
    if (rc) return rc;
    double sigma, om, km;
    sea_scales(cfg, sigma, om, km);
    const double s_eta = km * sigma * sigma, s_u = s_eta * om;
    long nlive = (long)s.live.size();
    if (nlive == 0) return OK;
    const int *act;
    long nl2;
    grid_live_columns(g, &act, &nl2);
    k_surr_apply<<<(unsigned)((nlive * g.nl + 255) / 256), 256, 0, st>>>(
        nlive, act, g.nx, g.ny, g.nl, slot, (float)g.swl, s.eta1, s.base, s.pred, (carry && s.have_res) ? s.R : nullptr,
        (float)s_eta, (float)s_u, g.ETA, g.U[0], g.U[1], g.U[2]);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

// err[0..3]: max |eta - eta_ref| / max|eta_ref - swl|, and the same for u, v, w
// against max |U_ref| (the plain reference of the compared columns comes from
// the scratch arrays; col null: all columns).
static int compare(Surrogate &s, DevGrid &g, int slot, const int *col, long n, float inv_eta, float inv_u,
                   double err[4], cudaStream_t st) {
    CK(cudaMemsetAsync(s.d_err, 0, sizeof(unsigned) * 4, st));
    k_surr_compare<<<(unsigned)((n * g.nl + 255) / 256), 256, 0, st>>>(
        n, col, g.nx, g.ny, g.nl, slot, g.ETA, g.U[0], g.U[1], g.U[2], s.rETA, s.rU[0], s.rU[1], s.rU[2], inv_eta,
        inv_u, s.d_err);
    note_launch();
    CK(cudaGetLastError());
    unsigned h[4];
    CK(cudaMemcpyAsync(h, s.d_err, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int rc = conv_check(st);
    if (rc) return rc;
    for (int q = 0; q < 4; q++) {
        float v;
        std::memcpy(&v, &h[q], 4);
        err[q] = v;
    }
    return OK;
}

// R = (plain slot - first order) - network, normalised, for a slot the plain
// method filled at time t.  have_pred: s.pred/s.base/s.eta1 already hold the
// network's output and the first order at t.
static int refresh_residual(Surrogate &s, const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws,
                            int slot, double t, bool have_pred, cudaStream_t st) {
    int rc;
    if (!have_pred) {
        rc = features(s, cfg, sea, g, ws, t, s.feat, s.base, s.eta1, st);
        if (rc) return rc;
        rc = surrogate_forward(s.feat, 1, g.nx + 2 * SH, g.ny + 2 * SH, s.pred, st);
        if (rc) return rc;
    }
    rc = surrogate_targets(cfg, g, slot, s.base, s.eta1, s.R, st);
    if (rc) return rc;
    long n = (long)s.cout * g.nx * g.ny;
    k_sub<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, s.pred, s.R);
    note_launch();
    CK(cudaGetLastError());
    // keep the slowly varying part: a Gaussian of carry_lw mean wavelengths
    // (the sum-frequency part of the residual oscillates on half a wavelength
    // and in time at twice the wave frequency; the long-wave part persists)
    double sigma, om, km;
    sea_scales(cfg, sigma, om, km);
    const double lam = 2.0 * 3.141592653589793 / std::max(km, 1e-12);
    if (s.carry_lw > 0) {
        for (int dir = 0; dir < 2; dir++) {
            double sd = s.carry_lw * lam / (dir == 0 ? g.dx : g.dy);
            int rad = (int)std::min(3.0 * sd, (double)(dir == 0 ? g.nx : g.ny));
            float inv2s2 = (float)(0.5 / std::max(sd * sd, 1e-12));
            const float *src = dir == 0 ? s.R : s.Rtmp;
            float *dst = dir == 0 ? s.Rtmp : s.R;
            k_blur<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s.cout, g.nx, g.ny, dir, inv2s2, rad, src, dst);
            note_launch();
            CK(cudaGetLastError());
        }
    } else {
        CK(cudaMemsetAsync(s.R, 0, sizeof(float) * n, st));
    }
    s.have_res = true;
    return OK;
}

void surrogate_set_carry(double wavelengths) {
    g_s.carry_lw = wavelengths;
    g_s.have_res = false;
}

static unsigned long long lcg(unsigned long long &st) {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    return st >> 33;
}

// One ring step of the grid (lsgrid_spline.cpp:847-931 order: advance, fill
// the newest slot, gradients).  mode 0 plain; 1 surrogate with a check of
// nsample plain columns (fallback to plain above tol); 2 surrogate unchecked.
int surrogate_step(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, int mode, double tol,
                   int nsample, int *fell_back, double *err_out, void *stream_) {
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    const bool carry = (mode & 4) == 0;
    mode &= 3;
    if (mode != 0 && !s.ready) return E_NOT_INITIALIZED;
    if (mode > 2 || nsample < 0 || nsample > 4096) return E_BAD_ARGUMENT;
    if (mode != 0 && g.nf != 3) return E_UNSUPPORTED;   // the network predicts no pressure
    if (mode != 0) {
        int rc = attach_grid(s, g, st);
        if (rc) return rc;
        if (carry && !s.have_res) {
            // the newest slot is a plain one (initialisation or a plain step)
            rc = refresh_residual(s, cfg, sea, g, ws, (g.tstep + 3) % 4, g.t0 + 2 * g.dt, false, st);
            if (rc) return rc;
        }
    }
    g.tstep++;
    g.t0 += g.dt;
    const double t2 = g.t0 + 2 * g.dt;
    const int slot = (g.tstep + 3) % 4;
    int fb = 0;
    double err[4] = {0, 0, 0, 0};
    int rc = OK;
    if (mode == 0) {
        rc = grid_fill_slot(g, sea, ws, slot, t2, st);
        if (rc) return rc;
        s.plain_steps++;
        if (s.ready && same_grid(s, g)) {
            long nxy = (long)g.nx * g.ny;
            float *U[3] = {g.U[0] + (long)slot * nxy * g.nl, g.U[1] + (long)slot * nxy * g.nl,
                           g.U[2] + (long)slot * nxy * g.nl};
            rc = slot_max(s, g, g.ETA + (long)slot * nxy, U, st, &s.fmax_eta, &s.fmax_u);
            if (rc) return rc;
            if (carry) {
                rc = refresh_residual(s, cfg, sea, g, ws, slot, t2, false, st);
                if (rc) return rc;
            }
        }
    } else {
        if (s.fmax_eta <= 0.f || s.fmax_u <= 0.f) {
            // scales of the check: the slot the plain method filled last
            long nxy = (long)g.nx * g.ny;
            int prev = (g.tstep + 2) % 4;
            float *U[3] = {g.U[0] + (long)prev * nxy * g.nl, g.U[1] + (long)prev * nxy * g.nl,
                           g.U[2] + (long)prev * nxy * g.nl};
            rc = slot_max(s, g, g.ETA + (long)prev * nxy, U, st, &s.fmax_eta, &s.fmax_u);
            if (rc) return rc;
        }
        long ns = std::min<long>(nsample, (long)s.live.size());
        if (mode == 1 && ns > 0) {
            std::vector<int> pick(ns);
            for (long q = 0; q < ns; q++) pick[q] = s.live[lcg(s.rng) % s.live.size()];
            CK(cudaMemcpyAsync(s.d_sample, pick.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
            float *rU[3] = {s.rU[0], s.rU[1], s.rU[2]};
            rc = grid_fill_columns(g, sea, ws, s.d_sample, ns, t2, s.rETA, rU, 0, st);
            if (rc) return rc;
        }
        rc = predict_slot(s, cfg, sea, g, ws, slot, t2, carry, st);
        if (rc) return rc;
        s.steps++;
        if (mode == 1 && ns > 0) {
            rc = compare(s, g, slot, s.d_sample, ns, 1.f / std::max(s.fmax_eta, 1e-30f),
                         1.f / std::max(s.fmax_u, 1e-30f), err, st);
            if (rc) return rc;
            double e = std::max(std::max(err[0], err[1]), std::max(err[2], err[3]));
            if (!(e <= tol)) {
                rc = grid_fill_slot(g, sea, ws, slot, t2, st);
                if (rc) return rc;
                fb = 1;
                s.fallbacks++;
                if (carry) {
                    rc = refresh_residual(s, cfg, sea, g, ws, slot, t2, true, st);
                    if (rc) return rc;
                }
            }
        }
    }
    if (fell_back) *fell_back = fb;
    if (err_out) for (int q = 0; q < 4; q++) err_out[q] = err[q];
    return grid_gradients(g, st);
}

// Plain fill of the newest slot's time into the scratch arrays and the
// normalised max errors of the grid's newest slot against it (all columns).
int surrogate_compare_newest(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, double *err,
                             void *stream_) {
    (void)cfg;
    cudaStream_t st = (cudaStream_t)stream_;
    Surrogate &s = g_s;
    if (!s.ready) return E_NOT_INITIALIZED;
    int rc = attach_grid(s, g, st);
    if (rc) return rc;
    const int slot = (g.tstep + 3) % 4;
    const double t2 = g.t0 + 2 * g.dt;
    float *rU[3] = {s.rU[0], s.rU[1], s.rU[2]};
    const int *act;
    long nlive;
    grid_live_columns(g, &act, &nlive);
    const long nxy = (long)g.nx * g.ny;
    CK(cudaMemsetAsync(s.rETA, 0, sizeof(float) * nxy, st));
    for (int f = 0; f < 3; f++) CK(cudaMemsetAsync(s.rU[f], 0, sizeof(float) * nxy * g.nl, st));
    rc = grid_fill_columns(g, sea, ws, act, nlive, t2, s.rETA, rU, 0, st);
    if (rc) return rc;
    float me, mu;
    rc = slot_max(s, g, s.rETA, rU, st, &me, &mu);
    if (rc) return rc;
    return compare(s, g, slot, act, nlive, 1.f / std::max(me, 1e-30f), 1.f / std::max(mu, 1e-30f), err, st);
}

void surrogate_stats(long *steps, long *fallbacks, long *plain_steps) {
    if (steps) *steps = g_s.steps;
    if (fallbacks) *fallbacks = g_s.fallbacks;
    if (plain_steps) *plain_steps = g_s.plain_steps;
}

void surrogate_reset_stats() {
    g_s.steps = g_s.fallbacks = g_s.plain_steps = 0;
    g_s.fmax_eta = g_s.fmax_u = 0.f;
}

}  // namespace cfdwm
