// Lagrangian stretched s-grid with 4-D cubic-Hermite query, on the GPU.
//
// Behaviour follows the reference's lsGridSpline (oystelan/CFDwavemaker
// v3.1.0, src/lsgrid_spline.cpp):
//   storage and ring of 4 time slots     :35-61, 847-931
//   sigma maps z2s/s2z/cart2sigmaS/...   :91-122
//   column body (eta, levels, uvw2)      :695-720, 880-903
//   finite-difference gradients          :124-366
//   spline query                         :368-605
//
// GB300 design: the whole grid lives in one device allocation (FP32 fields in
// the reference's [slot][i][j][m] layout), so the reference's MPI column
// partition and MPI_Allgatherv disappear.  A ring step is
//   phasors of the active columns  ->  eta2 pair sums  ->  level heights
//   ->  column pair sums (u, v, w at all levels of a column in registers)
//   ->  scatter into the slot  ->  one fused finite-difference pass.
// The query kernel gathers the 2x2(x2) stencils of the two bracketing slots
// and reduces x -> y -> s -> t exactly in the reference's order.
#include "cfdwm.h"
#include "sgrid_geom.cuh"
#include "ffmath.cuh"

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

// launchers shared with irregular.cu
int launch_eta_pairs(const DevSea &sea, long n, const float2 *ph, const float *rr, float *out,
                     cudaStream_t stream, float *split_buf, long split_cap);
int launch_column_pairs(const DevSea &sea, long ncol, int nl, const float2 *ph, const float *rr,
                        const float *z0, float *out, int pairs, cudaStream_t stream, float *split_buf,
                        long split_cap, bool pressure);
long column_pairs_split_floats(int nl);
int launch_pressure_kin(const DevSea &sea, double t, int nz, double *kin, cudaStream_t stream);

// heights of the table of the phase-free pressure terms over [-h, 0]
constexpr int KIN_NZ = 2049;
int launch_phasors_public(const DevSea &sea, long n, const double *x, const double *y,
                          const double *t, long sx, long sy, long st, int npad, float2 *ph,
                          float *rr, double *first, cudaStream_t stream);

__global__ void k_column_coords(GridGeom g, long nact, const int *act, double *xy) {
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= nact) return;
    int c = act[q], i = c / g.ny, j = c % g.ny;
    xy[q] = g.d0 + g.dx * i;
    xy[nact + q] = g.d2 + g.dy * j;
}

// ETA of the slot, the level heights and the level offsets above swl.
// blockDim 128; the stretched coordinate of each level (which depends on the
// level only) is formed once per block
__global__ void k_levels(GridGeom g, long nact, const int *act, const double *first,
                         const float *eta2, int slot, float *ETA, float *zmin, float *zmax) {
    __shared__ double s_sig[128];
    for (int m = threadIdx.x; m < g.nl; m += blockDim.x) s_sig[m] = d_sigma_level(g, m);
    __syncthreads();
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= nact) return;
    int c = act[q];
    double e = first[q] + (double)eta2[q] + g.swl;     // eta1 + eta2 + swl
    float ef = (float)e;
    ETA[(long)slot * g.nx * g.ny + c] = ef;
    for (int m = 0; m < g.nl; m++) {
        // the reference evaluates the levels from the stored value; the FP32
        // store is the value the query sees, so use it here too
        double z = d_s2z(g, s_sig[m], (double)ef);
        zmin[q * g.nl + m] = (float)fmin(0.0, z);
        zmax[q * g.nl + m] = (float)fmax(0.0, z - g.swl);
    }
}

// The level sums into the slot, with the Taylor terms above swl
// (lsgrid_spline.cpp:892-897).  With UP: the dynamic pressure
//   dp1(z0) + rho uvw2.p(z0) + dp1_dz max(0, z - swl),
// the phase-free part of uvw2.p from the height table kin (cubic Hermite).
__global__ void k_scatter_levels(GridGeom g, long nact, const int *act, const double *first,
                                 const float *sec, const float *zmin, const float *zmax, int slot,
                                 float *UX, float *UY, float *UZ, float *UP, const double *kin, int nkz) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long tot = nact * g.nl;
    if (e >= tot) return;
    long q = e / g.nl;
    int m = (int)(e % g.nl);
    long c = act[q];
    float za = zmax[e];
    long o = (long)slot * g.nx * g.ny * g.nl + c * g.nl + m;
    UX[o] = sec[0 * tot + e] + (float)first[1 * nact + q] * za;
    UY[o] = sec[1 * tot + e] + (float)first[2 * nact + q] * za;
    UZ[o] = sec[2 * tot + e] + (float)first[3 * nact + q] * za;
    if (UP) {
        const double dz = g.depth / (nkz - 1);
        double t = ((double)zmin[e] + g.depth) / dz;
        t = fmin(fmax(t, 0.0), (double)(nkz - 1));
        int i = min((int)t, nkz - 2);
        double r = t - i;
        double f0 = kin[2 * i], f1 = kin[2 * i + 2], d0 = kin[2 * i + 1], d1 = kin[2 * i + 3];
        double a = dz * d0 - (f1 - f0), b = -dz * d1 + (f1 - f0);
        double K = f0 * (1.0 - r) + f1 * r + r * (1.0 - r) * (a * (1.0 - r) + b * r);
        UP[o] = (float)((double)sec[3 * tot + e] + K) + (float)first[4 * nact + q] * za;
    }
}

// All finite differences of lsgrid_spline.cpp:124-366 in one pass over the
// nodes: x/y/s gradients of slots (tstep+1)%4, (tstep+2)%4 into gradient
// slots 0/1 and the time gradient of the slot(s) the reference writes.
struct GradArgs {
    GridGeom g;
    int tstep;
    const float *F[5];      // ETA, UX, UY, UZ (and the pressure)
    float *Fx[5], *Fy[5], *Fs[5], *Ft[5];
    float rdx, rdy, rds, rdt;   // reciprocal spacings
};

__global__ void k_gradients(GradArgs a) {
    const GridGeom &g = a.g;
    long nodes = (long)g.nx * g.ny * g.nl, cols = (long)g.nx * g.ny;
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    int field = blockIdx.y;                  // 0 ETA (column nodes), 1..3 U, V, W, 4 P
    int nl = field == 0 ? 1 : g.nl;
    long S = field == 0 ? cols : nodes;
    if (e >= S) return;
    int m = (int)(e % nl);
    long c = e / nl;
    int i = (int)(c / g.ny), j = (int)(c % g.ny);
    const float *D = a.F[field];
    int tids[2] = {(a.tstep + 1) % 4, (a.tstep + 2) % 4};
    long sx = (long)g.ny * nl, sy = nl;
    // FP32 differences of the FP32 node values times the reciprocal spacings
    // (one-sided at the boundaries, central inside)
    const float rdx = a.rdx, rdy = a.rdy, rds = a.rds, rdt = a.rdt;
    for (int q = 0; q < 2; q++) {
        const float *d = D + tids[q] * S;
        float gx, gy;
        if (g.nx == 1) gx = 0.f;
        else if (i == 0) gx = (d[e + sx] - d[e]) * rdx;
        else if (i == g.nx - 1) gx = (d[e] - d[e - sx]) * rdx;
        else gx = (d[e + sx] - d[e - sx]) * (0.5f * rdx);
        if (g.ny == 1) gy = 0.f;
        else if (j == 0) gy = (d[e + sy] - d[e]) * rdy;
        else if (j == g.ny - 1) gy = (d[e] - d[e - sy]) * rdy;
        else gy = (d[e + sy] - d[e - sy]) * (0.5f * rdy);
        a.Fx[field][q * S + e] = gx;
        a.Fy[field][q * S + e] = gy;
        if (field > 0) {
            float gs;
            if (nl == 1) gs = 0.f;
            else if (m == 0) gs = (d[e + 1] - d[e]) * rds;
            else if (m == nl - 1) gs = (d[e] - d[e - 1]) * rds;
            else gs = (d[e + 1] - d[e - 1]) * (0.5f * rds);
            a.Fs[field][q * S + e] = gs;
        }
    }
    float *T = a.Ft[field];
    if (a.tstep > 0) {
        int tid = (a.tstep + 2) % 4, tid1 = (a.tstep + 3) % 4, tid0 = (a.tstep + 1) % 4;
        T[tid * S + e] = (D[tid1 * S + e] - D[tid0 * S + e]) * (0.5f * rdt);
    } else {
        T[1 * S + e] = (D[2 * S + e] - D[1 * S + e]) * rdt;
        T[2 * S + e] = (D[3 * S + e] - D[1 * S + e]) * (0.5f * rdt);
    }
}

// ---------------------------------------------------------------------------
// Query
// ---------------------------------------------------------------------------
struct QueryArgs {
    GridGeom g;
    int tid1, tid2;
    double t0;
    const float *ETA, *ETAdt, *ETAdx, *ETAdy;
    const float4 *img;      // query image: [2][nodes][5] (U, U_t, U_x, U_y, U_s over the fields)
    int nf;
    long n;
    const double *x, *y, *z, *t;
    double *out;    // [1 + nf][n]
    double inv_dx, inv_dy, inv_dt;   // reciprocals of the spacings (host-computed)
    float tanab;                     // tan(a)^b of the stretching
};

__device__ __forceinline__ float herm(float f0, float f1, float d0, float d1, float h, float r) {
    float a = h * d0 - (f1 - f0), b = -h * d1 + (f1 - f0);
    return f0 * (1.f - r) + f1 * r + r * (1.f - r) * (a * (1.f - r) + b * r);
}
__device__ __forceinline__ float lin(float f0, float f1, float r) { return f0 * (1.f - r) + f1 * r; }

// cart2sigmaS (lsgrid_spline.cpp:109-113).  The reference takes pow() of a
// negative base (NaN, then an out-of-range index) for eta - swl < z <= eta
// when swl != 0; here the base is clamped at zero, i.e. such points are
// evaluated at the surface level.
__device__ __forceinline__ float cart2sigmaS(const GridGeom &g, float tanab, float zpt, float e) {
    float z = fminf(zpt, e);
    float es = e - (float)g.swl;
    float sigma = fmaxf((z - es) / ((float)g.depth + es), -1.f);
    float base = fmaxf(-sigma * tanab, 0.f);
    return 1.f - atanf(powf(base, 1.f / (float)g.tan_b)) / (float)g.tan_a;
}

__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ float4 herm4(float4 f0, float4 f1, float4 d0, float4 d1, float h, float r) {
    return make_float4(herm(f0.x, f1.x, d0.x, d1.x, h, r), herm(f0.y, f1.y, d0.y, d1.y, h, r),
                       herm(f0.z, f1.z, d0.z, d1.z, h, r), herm(f0.w, f1.w, d0.w, d1.w, h, r));
}
__device__ __forceinline__ float4 lin4(float4 f0, float4 f1, float r) {
    return make_float4(lin(f0.x, f1.x, r), lin(f0.y, f1.y, r), lin(f0.z, f1.z, r), lin(f0.w, f1.w, r));
}

// spline_interp_velo (lsgrid_spline.cpp:386-502) of every velocity field at
// once: the eight corners of each of the two bracketing slots are read as
// records of the query image, and the reductions x -> y -> s -> t run on the
// fields as float4 lanes (the reference's order, per field).
__device__ float4 spline_velo4(const QueryArgs &a, int xp, int yp, int s0, int s1, float xd, float yd, float sd0,
                               float sd1, float td) {
    const GridGeom &g = a.g;
    const long nn = (long)g.nx * g.ny * g.nl;
    const int x1 = iclamp(xp + 1, 0, g.nx - 1), y1 = iclamp(yp + 1, 0, g.ny - 1);
    const int ls[2] = {s0, s1};
    const float dx = (float)g.dx, dy = (float)g.dy, ds = (float)g.ds;
    float4 red[2], redt[2];
    for (int q = 0; q < 2; q++) {            // q = 0: slot (tstep+1)%4 at s0; q = 1: slot (tstep+2)%4 at s1
        const int l0 = ls[q], l1 = iclamp(ls[q] + 1, 0, g.nl - 1);
        const float4 *base = a.img + (long)q * nn * 5;
        // corners: x-pairs (xp, x1) at (yp, l0), (y1, l0), (yp, l1), (y1, l1)
        const int ys[4] = {yp, y1, yp, y1}, zs[4] = {l0, l0, l1, l1};
        float4 v[4], yv[4], tv[4], sv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float4 *ra = base + (((long)xp * g.ny + ys[k]) * g.nl + zs[k]) * 5;
            const float4 *rb = base + (((long)x1 * g.ny + ys[k]) * g.nl + zs[k]) * 5;
            const float4 aU = __ldg(ra), aT = __ldg(ra + 1), aX = __ldg(ra + 2), aY = __ldg(ra + 3), aS = __ldg(ra + 4);
            const float4 bU = __ldg(rb), bT = __ldg(rb + 1), bX = __ldg(rb + 2), bY = __ldg(rb + 3), bS = __ldg(rb + 4);
            v[k] = herm4(aU, bU, aX, bX, dx, xd);
            yv[k] = lin4(aY, bY, xd);
            tv[k] = lin4(aT, bT, xd);
            sv[k] = lin4(aS, bS, xd);
        }
        const float4 c0 = herm4(v[0], v[1], yv[0], yv[1], dy, yd), c1 = herm4(v[2], v[3], yv[2], yv[3], dy, yd);
        const float4 c0s = lin4(sv[0], sv[1], yd), c1s = lin4(sv[2], sv[3], yd);
        const float4 c0t = lin4(tv[0], tv[1], yd), c1t = lin4(tv[2], tv[3], yd);
        const float sd = q == 0 ? sd0 : sd1;
        red[q] = herm4(c0, c1, c0s, c1s, ds, sd);
        redt[q] = lin4(c0t, c1t, sd);
    }
    return herm4(red[0], red[1], redt[0], redt[1], (float)g.dt, td);
}

__global__ void __launch_bounds__(128) k_query(QueryArgs a) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const GridGeom &g = a.g;
    const double xpt = a.x[p], ypt = a.y[p], zpt = a.z[p], tpt = a.t[p];
    // std::modf with a float* argument selects the float overload in the
    // reference (lsgrid_spline.cpp:515-520): the fractions are float.
    float xi, yi;
    // (FP64 divisions per query replaced by products with the reciprocals:
    // FP64 runs at a small fraction of the FP32 rate on this GPU)
    float xd = modff((float)fmax(0.0, fmin((xpt - g.d0) * a.inv_dx, g.nx - 1.0)), &xi);
    float yd = modff((float)fmax(0.0, fmin((ypt - g.d2) * a.inv_dy, g.ny - 1.0)), &yi);
    float td = (float)fmin(1.0, fmax(0.0, (tpt - a.t0) * a.inv_dt));
    int xp = (int)xi, yp = (int)yi;
    const long nc = (long)g.nx * g.ny;
    const int x1 = iclamp(xp + 1, 0, g.nx - 1), y1 = iclamp(yp + 1, 0, g.ny - 1);
    long cid[4] = {(long)xp * g.ny + yp, (long)xp * g.ny + y1, (long)x1 * g.ny + yp, (long)x1 * g.ny + y1};
    float C[4], D[4], Ct[4], Dt[4], Cx[4], Dx[4], Cy[4], Dy[4];
    for (int k = 0; k < 4; k++) {
        C[k] = __ldg(a.ETA + a.tid1 * nc + cid[k]);
        D[k] = __ldg(a.ETA + a.tid2 * nc + cid[k]);
        Ct[k] = __ldg(a.ETAdt + a.tid1 * nc + cid[k]);
        Dt[k] = __ldg(a.ETAdt + a.tid2 * nc + cid[k]);
        Cx[k] = __ldg(a.ETAdx + cid[k]);
        Dx[k] = __ldg(a.ETAdx + nc + cid[k]);
        Cy[k] = __ldg(a.ETAdy + cid[k]);
        Dy[k] = __ldg(a.ETAdy + nc + cid[k]);
    }
    const float dx = (float)g.dx, dy = (float)g.dy;
    float C0 = herm(C[0], C[2], Cx[0], Cx[2], dx, xd), C1 = herm(C[1], C[3], Cx[1], Cx[3], dx, xd);
    float D0 = herm(D[0], D[2], Dx[0], Dx[2], dx, xd), D1 = herm(D[1], D[3], Dx[1], Dx[3], dx, xd);
    float C0y = lin(Cy[0], Cy[2], xd), C1y = lin(Cy[1], Cy[3], xd);
    float D0y = lin(Dy[0], Dy[2], xd), D1y = lin(Dy[1], Dy[3], xd);
    float C0t = lin(Ct[0], Ct[2], xd), C1t = lin(Ct[1], Ct[3], xd);
    float D0t = lin(Dt[0], Dt[2], xd), D1t = lin(Dt[1], Dt[3], xd);
    float e0 = herm(C0, C1, C0y, C1y, dy, yd), e1 = herm(D0, D1, D0y, D1y, dy, yd);
    float CCt = lin(C0t, C1t, yd), DDt = lin(D0t, D1t, yd);
    float eta = herm(e0, e1, CCt, DDt, (float)g.dt, td);
    const float tanab = a.tanab;
    float n0 = cart2sigmaS(g, tanab, (float)zpt, e0) / (float)g.ds;
    float n1 = cart2sigmaS(g, tanab, (float)zpt, e1) / (float)g.ds;
    float s0i, s1i;
    float sd0 = modff(n0, &s0i), sd1 = modff(n1, &s1i);
    int s0 = iclamp((int)s0i, 0, g.nl - 1), s1 = iclamp((int)s1i, 0, g.nl - 1);
    a.out[p] = d_from_float(eta);
    const float4 u = spline_velo4(a, xp, yp, s0, s1, xd, yd, sd0, sd1, td);
    a.out[1 * a.n + p] = d_from_float(u.x);
    a.out[2 * a.n + p] = d_from_float(u.y);
    a.out[3 * a.n + p] = d_from_float(u.z);
    if (a.nf == 4) a.out[4 * a.n + p] = d_from_float(u.w);
}

// The query image of the two slots the queries read, (tstep+1)%4 and
// (tstep+2)%4: per node one record of five float4, U, U_t, U_x, U_y, U_s, each
// over the velocity fields (and the pressure; lane 3 is 0 without it).  A
// query corner is then one 80-byte record instead of 5 nf separate loads.
struct QImgArgs {
    const float *U[4], *Ut[4], *Ux[4], *Uy[4], *Us[4];
    int nf, tstep;
    long nodes;
    float4 *img;
};
__global__ void k_query_image(QImgArgs a) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= a.nodes) return;
    const int q = blockIdx.y;
    const long S = a.nodes;
    const long ts = (long)((a.tstep + 1 + q) % 4) * S + e, gs = (long)q * S + e;
    float r[5][4];
#pragma unroll
    for (int f = 0; f < 4; f++) {
        const bool on = f < a.nf;
        r[0][f] = on ? a.U[f][ts] : 0.f;
        r[1][f] = on ? a.Ut[f][ts] : 0.f;
        r[2][f] = on ? a.Ux[f][gs] : 0.f;
        r[3][f] = on ? a.Uy[f][gs] : 0.f;
        r[4][f] = on ? a.Us[f][gs] : 0.f;
    }
    float4 *o = a.img + ((long)q * S + e) * 5;
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = make_float4(r[k][0], r[k][1], r[k][2], r[k][3]);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static GridGeom geom(const DevGrid &g) {
    GridGeom G;
    G.nx = g.nx; G.ny = g.ny; G.nl = g.nl;
    G.d0 = g.cfg.domain[0]; G.d2 = g.cfg.domain[2];
    G.dx = g.dx; G.dy = g.dy; G.ds = g.ds; G.depth = g.depth; G.swl = g.swl;
    G.tan_a = g.cfg.tan_a; G.tan_b = g.cfg.tan_b; G.dt = g.dt;
    return G;
}

// Extra per-grid device scratch kept alongside DevGrid (keyed by the grid).
struct GridExtra {
    int *act_all = nullptr, *act_live = nullptr;
    long n_all = 0, n_live = 0;
    double *xy = nullptr;      // [2][ncol]
    float *zmin = nullptr, *zmax = nullptr, *sec = nullptr;
    float *eta2 = nullptr;
    double *tdev = nullptr;    // the slot time, read with stride 0 by the phasor pass
    float *split = nullptr;    // slices of a split column-pair launch
    long split_cap = 0;
    double *kin = nullptr;     // [KIN_NZ][2] phase-free pressure terms of the slot being written
    // the table depends on t only through the component ramps: the ramps it
    // was built with, and the ramp parameters (ramptime, starttime, duration)
    std::vector<double> kin_r, ramp_par;
    bool kin_valid = false;
    DepthForm df;              // tensor-core form of the column sums (method 1)
    // live columns before row i (act_live is ascending in i ny + j):
    // the live columns of rows [i0, i1) are act_live[row_live[i0] .. row_live[i1])
    std::vector<long> row_live;
};
static std::vector<std::pair<const DevGrid *, GridExtra>> g_extra;
static GridExtra *extra(const DevGrid &g) {
    for (auto &e : g_extra) if (e.first == &g) return &e.second;
    g_extra.push_back({&g, GridExtra{}});
    return &g_extra.back().second;
}

int grid_create(const Config &cfg, DevGrid &g, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    grid_free(g);
    g.cfg = cfg.lsgrid;
    g.nx = cfg.lsgrid.nx; g.ny = cfg.lsgrid.ny; g.nl = cfg.lsgrid.nl;
    if (g.nx < 1 || g.ny < 1 || g.nl < 1) return E_BAD_ARGUMENT;
    if (g.nl > 128) return E_TOO_LARGE;
    // initialize_kinematics (lsgrid_spline.cpp:673-677) and set_ignore (:1406)
    g.dx = (g.cfg.domain[1] - g.cfg.domain[0]) / std::max(1., double(g.nx - 1));
    g.dy = (g.cfg.domain[3] - g.cfg.domain[2]) / std::max(1., double(g.ny - 1));
    g.ds = 1. / std::max(1., double(g.nl - 1));
    g.t0 = g.cfg.t0; g.dt = g.cfg.dt; g.depth = cfg.depth; g.swl = cfg.swl; g.tstep = 0;
    long c = (long)g.nx * g.ny, v = c * g.nl;
    CK(cudaMalloc(&g.ETA, sizeof(float) * 4 * c));
    CK(cudaMalloc(&g.ETAdt, sizeof(float) * 4 * c));
    CK(cudaMalloc(&g.ETAdx, sizeof(float) * 2 * c));
    CK(cudaMalloc(&g.ETAdy, sizeof(float) * 2 * c));
    CK(cudaMemsetAsync(g.ETA, 0, sizeof(float) * 4 * c, stream));
    CK(cudaMemsetAsync(g.ETAdt, 0, sizeof(float) * 4 * c, stream));
    for (int f = 0; f < 3; f++) {
        CK(cudaMalloc(&g.U[f], sizeof(float) * 4 * v));
        CK(cudaMalloc(&g.Ut[f], sizeof(float) * 4 * v));
        CK(cudaMalloc(&g.Ux[f], sizeof(float) * 2 * v));
        CK(cudaMalloc(&g.Uy[f], sizeof(float) * 2 * v));
        CK(cudaMalloc(&g.Us[f], sizeof(float) * 2 * v));
        CK(cudaMemsetAsync(g.U[f], 0, sizeof(float) * 4 * v, stream));
        CK(cudaMemsetAsync(g.Ut[f], 0, sizeof(float) * 4 * v, stream));
    }
    std::vector<int> ign(c), all, live;
    GridExtra *xr = extra(g);
    xr->row_live.assign(g.nx + 1, 0);
    for (int i = 0; i < g.nx; i++) {
        xr->row_live[i] = (long)live.size();
        double xp = g.cfg.domain[0] + g.dx * i;
        for (int j = 0; j < g.ny; j++) {
            double yp = g.cfg.domain[2] + g.dy * j;
            const double *di = g.cfg.domain_ignore;
            int ig = (xp >= di[0] && xp <= di[1] && yp >= di[2] && yp <= di[3]) ? 1 : 0;
            ign[(long)i * g.ny + j] = ig;
            all.push_back(i * g.ny + j);
            if (!ig) live.push_back(i * g.ny + j);
        }
    }
    xr->row_live[g.nx] = (long)live.size();
    CK(cudaMalloc(&g.IGNORE, sizeof(int) * c));
    CK(cudaMemcpyAsync(g.IGNORE, ign.data(), sizeof(int) * c, cudaMemcpyHostToDevice, stream));
    GridExtra *x = extra(g);
    x->n_all = (long)all.size();
    x->n_live = (long)live.size();
    CK(cudaMalloc(&x->act_all, sizeof(int) * std::max<long>(1, x->n_all)));
    CK(cudaMalloc(&x->act_live, sizeof(int) * std::max<long>(1, x->n_live)));
    CK(cudaMemcpyAsync(x->act_all, all.data(), sizeof(int) * x->n_all, cudaMemcpyHostToDevice, stream));
    if (x->n_live)
        CK(cudaMemcpyAsync(x->act_live, live.data(), sizeof(int) * x->n_live, cudaMemcpyHostToDevice, stream));
    CK(cudaMalloc(&x->xy, sizeof(double) * 2 * c));
    CK(cudaMalloc(&x->zmin, sizeof(float) * v));
    CK(cudaMalloc(&x->zmax, sizeof(float) * v));
    CK(cudaMalloc(&x->sec, sizeof(float) * 4 * v));
    CK(cudaMalloc(&x->eta2, sizeof(float) * c));
    CK(cudaMalloc(&x->tdev, sizeof(double)));
    x->split_cap = column_pairs_split_floats(g.nl);
    CK(cudaMalloc(&x->split, sizeof(float) * x->split_cap));
    CK(cudaMalloc(&g.QIMG, sizeof(float4) * 10 * v));
    CK(cudaStreamSynchronize(stream));
    return OK;
}

void grid_free(DevGrid &g) {
    float *ptrs[] = {g.ETA, g.ETAdx, g.ETAdy, g.ETAdt};
    for (float *p : ptrs) if (p) cudaFree(p);
    for (int f = 0; f < 4; f++) {
        float *q[] = {g.U[f], g.Ut[f], g.Ux[f], g.Uy[f], g.Us[f]};
        for (float *p : q) if (p) cudaFree(p);
        g.U[f] = g.Ut[f] = g.Ux[f] = g.Uy[f] = g.Us[f] = nullptr;
    }
    g.nf = 3;
    if (g.IGNORE) cudaFree(g.IGNORE);
    if (g.QIMG) cudaFree(g.QIMG);
    g.ETA = g.ETAdx = g.ETAdy = g.ETAdt = nullptr;
    g.IGNORE = nullptr;
    g.QIMG = nullptr;
    for (auto it = g_extra.begin(); it != g_extra.end(); ++it)
        if (it->first == &g) {
            GridExtra &x = it->second;
            void *q[] = {x.act_all, x.act_live, x.xy, x.zmin, x.zmax, x.sec, x.eta2, x.tdev, x.split, x.kin};
            for (void *p : q) if (p) cudaFree(p);
            depthform_free(x.df);
            g_extra.erase(it);
            break;
        }
}

// Plain second-order fill of the columns act[0..nact) at time t into ring
// slot `slot` of the arrays ETA ([slot][nx*ny]) and U[f] ([slot][nx*ny*nl]);
// P (or null): the pressure field, when the grid holds one.
static int fill_cols(DevGrid &g, const DevSea &sea, Workspace &ws, const int *act, long nact, double t,
                     float *ETA, float *const U[3], float *P, int slot, cudaStream_t stream) {
    GridExtra *x = extra(g);
    if (nact == 0) return OK;
    const bool pres = P != nullptr && g.nf == 4;
    GridGeom G = geom(g);
    const int npad = sea.npad_g;
    const bool tc = g.method == 1 && x->df.built;
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    // workspace: plain: phasors [npad][nact], ramps [npad][nact], first-order
    // sums [5][nact]; tensor-core: the first-order sums only
    size_t b_ph = tc ? 0 : up(sizeof(float2) * (size_t)npad * nact);
    size_t b_rr = tc ? 0 : up(sizeof(float) * (size_t)npad * nact);
    int rc = workspace_reserve(ws, b_ph + b_rr + sizeof(double) * 5 * nact);
    if (rc) return rc;
    char *b = (char *)ws.base;
    float2 *ph = (float2 *)b;
    float *rr = (float *)(b + b_ph);
    double *first = (double *)(b + b_ph + b_rr);
    k_column_coords<<<(unsigned)((nact + 255) / 256), 256, 0, stream>>>(G, nact, act, x->xy);
    note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(x->tdev, &t, sizeof(double), cudaMemcpyHostToDevice, stream));
    if (tc) {
        // eta1 and the Taylor gradients (float-float phases), then eta2 and the
        // 3R depth-separated quadratic forms of every column in one GEMM
        rc = depthform_first(sea, nact, g.nl, x->xy, t, nullptr, first, nullptr, 3, stream);
        if (!rc) rc = depthform_columns(x->df, sea, nact, x->xy, x->xy + nact, x->tdev, x->eta2, stream);
    } else {
        rc = launch_phasors_public(sea, nact, x->xy, x->xy + nact, x->tdev, 1, 1, 0, npad, ph, rr, first, stream);
        if (!rc) rc = launch_eta_pairs(sea, nact, ph, rr, x->eta2, stream, x->split, x->split_cap);
    }
    if (rc) return rc;
    k_levels<<<(unsigned)((nact + 127) / 128), 128, 0, stream>>>(G, nact, act, first, x->eta2, slot, ETA,
                                                                 x->zmin, x->zmax);
    note_launch();
    CK(cudaGetLastError());
    if (tc) {
        // first order at the level heights, then the second order from the R
        // basis functions of the level heights
        // (the form holds the pressure blocks when the grid holds pressure;
        // a fill without P leaves them unused)
        if (pres && x->df.nf != 4) return E_NOT_INITIALIZED;
        rc = depthform_first(sea, nact, g.nl, x->xy, t, x->zmin, nullptr, x->sec, x->df.nf, stream);
        if (!rc) rc = depthform_combine(x->df, nact, g.nl, x->zmin, x->sec, stream);
    } else {
        // first and second order per (pair, level)
        rc = launch_column_pairs(sea, nact, g.nl, ph, rr, x->zmin, x->sec, 1, stream, x->split, x->split_cap,
                                 pres);
    }
    if (rc) return rc;
    if (pres) {
        // rebuild the height table only when a component ramp changed (once
        // every ramp has reached 1, the table stays valid)
        const size_t nc = x->ramp_par.size() / 3;
        std::vector<double> r(nc);
        for (size_t i = 0; i < nc; i++) {
            const double rt = x->ramp_par[3 * i], ts = x->ramp_par[3 * i + 1], du = x->ramp_par[3 * i + 2];
            const double down = std::max(std::min(1. - ((t - ts - du + rt) / (rt + SMALL)), 1.), 0.);
            const double up = std::max(std::min((t - ts) / (rt + SMALL), 1.), 0.);
            r[i] = up * down;
        }
        if (!x->kin_valid || r != x->kin_r) {
            rc = launch_pressure_kin(sea, t, KIN_NZ, x->kin, stream);
            if (rc) return rc;
            x->kin_r = r;
            x->kin_valid = true;
        }
    }
    long tot = nact * g.nl;
    k_scatter_levels<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(
        G, nact, act, first, x->sec, x->zmin, x->zmax, slot, U[0], U[1], U[2], pres ? P : nullptr, x->kin, KIN_NZ);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

// Fill one ring slot at time t for the given column set.
static int fill_slot(DevGrid &g, const DevSea &sea, Workspace &ws, int slot, double t, bool live_only,
                     cudaStream_t stream) {
    GridExtra *x = extra(g);
    long nact = live_only ? x->n_live : x->n_all;
    const int *act = live_only ? x->act_live : x->act_all;
    return fill_cols(g, sea, ws, act, nact, t, g.ETA, g.U, g.nf == 4 ? g.U[3] : nullptr, slot, stream);
}

int grid_fill_columns(DevGrid &g, const DevSea &sea, Workspace &ws, const int *act, long nact, double t,
                      float *ETA, float *const U[3], int slot, void *stream) {
    if (nact < 0 || nact > (long)g.nx * g.ny) return E_BAD_ARGUMENT;
    return fill_cols(g, sea, ws, act, nact, t, ETA, U, nullptr, slot, (cudaStream_t)stream);
}

int grid_fill_slot(DevGrid &g, const DevSea &sea, Workspace &ws, int slot, double t, void *stream) {
    return fill_slot(g, sea, ws, slot, t, true, (cudaStream_t)stream);
}

void grid_live_columns(DevGrid &g, const int **act, long *n) {
    GridExtra *x = extra(g);
    *act = x->act_live;
    *n = x->n_live;
}

GridGeom grid_geom(const DevGrid &g) { return geom(g); }

static int gradients(DevGrid &g, cudaStream_t stream) {
    GradArgs a;
    a.g = geom(g);
    a.tstep = g.tstep;
    a.rdx = (float)(1.0 / g.dx); a.rdy = (float)(1.0 / g.dy); a.rds = (float)(1.0 / g.ds); a.rdt = (float)(1.0 / g.dt);
    a.F[0] = g.ETA; a.Fx[0] = g.ETAdx; a.Fy[0] = g.ETAdy; a.Fs[0] = nullptr; a.Ft[0] = g.ETAdt;
    for (int f = 0; f < 4; f++) {
        a.F[f + 1] = g.U[f]; a.Fx[f + 1] = g.Ux[f]; a.Fy[f + 1] = g.Uy[f];
        a.Fs[f + 1] = g.Us[f]; a.Ft[f + 1] = g.Ut[f];
    }
    long nodes = (long)g.nx * g.ny * g.nl;
    dim3 grid((unsigned)((nodes + 255) / 256), (unsigned)(1 + g.nf));
    prof_begin(PK_GRADIENTS, stream);
    k_gradients<<<grid, 256, 0, stream>>>(a);
    note_launch();
    CK(cudaGetLastError());
    QImgArgs qa;
    for (int f = 0; f < 4; f++) {
        qa.U[f] = g.U[f]; qa.Ut[f] = g.Ut[f]; qa.Ux[f] = g.Ux[f]; qa.Uy[f] = g.Uy[f]; qa.Us[f] = g.Us[f];
    }
    qa.nf = g.nf; qa.tstep = g.tstep; qa.nodes = nodes; qa.img = reinterpret_cast<float4 *>(g.QIMG);
    k_query_image<<<dim3((unsigned)((nodes + 255) / 256), 2), 256, 0, stream>>>(qa);
    note_launch();
    prof_end(PK_GRADIENTS, stream);
    CK(cudaGetLastError());
    return OK;
}

int grid_initialize(DevGrid &g, const DevSea &sea, Workspace &ws, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    bool wi = g.cfg.ignore_at_init;
    // initialize_kinematics[_with_ignore] (lsgrid_spline.cpp:679, 758)
    double tt0[4] = {wi ? g.t0 : g.t0 - g.dt, g.t0, g.t0 + g.dt, g.t0 + 2 * g.dt};
    g.tstep = 0;
    for (int tt = 0; tt < 4; tt++) {
        int rc = fill_slot(g, sea, ws, tt, tt0[tt], wi, stream);
        if (rc) return rc;
    }
    int rc = gradients(g, stream);
    if (rc) return rc;
    CK(cudaStreamSynchronize(stream));
    return OK;
}

int grid_gradients(DevGrid &g, void *stream) { return gradients(g, (cudaStream_t)stream); }

int grid_set_method(DevGrid &g, const Config &cfg, const DevSea &sea, int method, void *stream) {
    if (method != 0 && method != 1) return E_BAD_ARGUMENT;
    GridExtra *x = extra(g);
    if (method == 1 && (!x->df.built || x->df.nf != g.nf)) {
        int rc = depthform_build(cfg, sea, x->df, g.nf, stream);
        if (rc) return rc;
    }
    g.method = method;
    return OK;
}

int grid_set_pressure(DevGrid &g, const Config &cfg, const DevSea &sea, bool on, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    GridExtra *x = extra(g);
    const int nf = on ? 4 : 3;
    if (on && (!sea.d_tab_gp || !sea.d_tab_gk)) return E_UNSUPPORTED;   // first-order sea
    if (nf == g.nf) return OK;
    long v = (long)g.nx * g.ny * g.nl;
    if (on) {
        CK(cudaMalloc(&g.U[3], sizeof(float) * 4 * v));
        CK(cudaMalloc(&g.Ut[3], sizeof(float) * 4 * v));
        CK(cudaMalloc(&g.Ux[3], sizeof(float) * 2 * v));
        CK(cudaMalloc(&g.Uy[3], sizeof(float) * 2 * v));
        CK(cudaMalloc(&g.Us[3], sizeof(float) * 2 * v));
        CK(cudaMemsetAsync(g.U[3], 0, sizeof(float) * 4 * v, stream));
        CK(cudaMemsetAsync(g.Ut[3], 0, sizeof(float) * 4 * v, stream));
        if (!x->kin) CK(cudaMalloc(&x->kin, sizeof(double) * 2 * KIN_NZ));
        x->ramp_par.resize(3 * cfg.omega.size());
        for (size_t i = 0; i < cfg.omega.size(); i++) {
            x->ramp_par[3 * i] = cfg.ramptime[i];
            x->ramp_par[3 * i + 1] = cfg.starttime[i];
            x->ramp_par[3 * i + 2] = cfg.duration[i];
        }
        x->kin_valid = false;
    } else {
        float *q[] = {g.U[3], g.Ut[3], g.Ux[3], g.Uy[3], g.Us[3]};
        for (float *p : q) if (p) cudaFree(p);
        g.U[3] = g.Ut[3] = g.Ux[3] = g.Uy[3] = g.Us[3] = nullptr;
    }
    g.nf = nf;
    // the tensor-core form carries the pressure blocks only when asked to
    if (g.method == 1) {
        int rc = depthform_build(cfg, sea, x->df, nf, stream);
        if (rc) return rc;
    } else if (x->df.built) {
        depthform_free(x->df);
    }
    CK(cudaStreamSynchronize(stream));
    return OK;
}

int grid_tc_error(DevGrid &g, void *stream) { return depthform_error(extra(g)->df, stream); }

int depthform_rank(DevGrid &g) { return extra(g)->df.built ? extra(g)->df.R : 0; }

int grid_update(DevGrid &g, const DevSea &sea, Workspace &ws, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    // update (lsgrid_spline.cpp:847-931)
    g.tstep++;
    g.t0 += g.dt;
    double t2 = g.t0 + 2 * g.dt;
    int slot = (g.tstep + 3) % 4;
    int rc = fill_slot(g, sea, ws, slot, t2, true, stream);
    if (rc) return rc;
    return gradients(g, stream);
}

bool grid_check_time(const DevGrid &g, double t) { return t > g.t0 + g.dt; }

// ---------------------------------------------------------------------------
// Column shard.  The reference's MPI build splits the grid's rows of columns
// (index i) over the ranks by a work-balanced contiguous partition weighted
// by the live columns of each row (lsgrid_spline.cpp:652-664,
// mpi_utils.h:46-64); each rank fills its rows of the new slot and the slot's
// ETA, UX, UY, UZ are all-gathered (lsgrid_spline.cpp:907-910) before every
// rank recomputes the gradients.  A rank's rows [i0, i1) of a slot are
// contiguous in every field ([slot][i][j] and [slot][i][j][m]), so a block is
// one copy per field.
// ---------------------------------------------------------------------------
void grid_row_weights(const DevGrid &g, std::vector<long> &w) {
    GridExtra *x = extra(g);
    w.resize(g.nx);
    for (int i = 0; i < g.nx; i++) w[i] = x->row_live[i + 1] - x->row_live[i];
}

int grid_step_block(DevGrid &g, const DevSea &sea, Workspace &ws, int i0, int i1, void *stream_) {
    if (i0 < 0 || i1 > g.nx || i0 > i1) return E_BAD_ARGUMENT;
    cudaStream_t stream = (cudaStream_t)stream_;
    g.tstep++;
    g.t0 += g.dt;
    const double t2 = g.t0 + 2 * g.dt;
    const int slot = (g.tstep + 3) % 4;
    GridExtra *x = extra(g);
    const long a = x->row_live[i0], b = x->row_live[i1];
    return fill_cols(g, sea, ws, x->act_live + a, b - a, t2, g.ETA, g.U, g.nf == 4 ? g.U[3] : nullptr, slot, stream);
}

// rows [i0, i1) of field f (0 ETA, 1 + q the velocity / pressure field q) of
// the newest slot to or from buf (device or host memory); returns the count
long grid_block_elems(const DevGrid &g, int f, int i0, int i1) {
    return (long)(i1 - i0) * g.ny * (f == 0 ? 1 : g.nl);
}

int grid_block_copy(DevGrid &g, int f, int i0, int i1, float *buf, bool into_grid, void *stream_) {
    if (i0 < 0 || i1 > g.nx || i0 > i1 || f < 0 || f > g.nf || !buf) return E_BAD_ARGUMENT;
    cudaStream_t stream = (cudaStream_t)stream_;
    const int slot = (g.tstep + 3) % 4;
    const long c = (long)g.nx * g.ny;
    float *base = f == 0 ? g.ETA + (long)slot * c + (long)i0 * g.ny
                         : g.U[f - 1] + ((long)slot * c + (long)i0 * g.ny) * g.nl;
    const size_t bytes = sizeof(float) * grid_block_elems(g, f, i0, i1);
    if (bytes == 0) return OK;
    CK(cudaMemcpyAsync(into_grid ? base : buf, into_grid ? buf : base, bytes, cudaMemcpyDefault, stream));
    return OK;
}

int grid_query(const DevGrid &g, long n, const double *x, const double *y, const double *z,
               const double *t, double *out, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (n <= 0) return OK;
    QueryArgs a;
    a.g = geom(g);
    a.tid1 = (g.tstep + 1) % 4; a.tid2 = (g.tstep + 2) % 4; a.t0 = g.t0;
    a.ETA = g.ETA; a.ETAdt = g.ETAdt; a.ETAdx = g.ETAdx; a.ETAdy = g.ETAdy;
    a.img = reinterpret_cast<const float4 *>(g.QIMG);
    a.nf = g.nf;
    a.n = n; a.x = x; a.y = y; a.z = z; a.t = t; a.out = out;
    a.inv_dx = 1.0 / a.g.dx; a.inv_dy = 1.0 / a.g.dy; a.inv_dt = 1.0 / a.g.dt;
    a.tanab = powf(tanf((float)a.g.tan_a), (float)a.g.tan_b);
    prof_begin(PK_QUERY, stream);
    k_query<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(a);
    note_launch();
    prof_end(PK_QUERY, stream);
    CK(cudaGetLastError());
    return OK;
}

int grid_download(const DevGrid &g, int which, double *dst, long cap, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    long c = (long)g.nx * g.ny, v = c * g.nl;
    const float *src = nullptr;
    long n = 0;
    switch (which) {
    case 0: src = g.ETA; n = 4 * c; break;
    case 1: case 2: case 3: src = g.U[which - 1]; n = 4 * v; break;
    case 4: src = g.ETAdx; n = 2 * c; break;
    case 5: src = g.ETAdy; n = 2 * c; break;
    case 6: src = g.ETAdt; n = 4 * c; break;
    case 23:
        if (g.nf != 4) return E_UNSUPPORTED;
        src = g.U[3]; n = 4 * v; break;
    default:
        if (which >= 19 && which <= 22 && g.nf != 4) return E_UNSUPPORTED;
        if (which >= 7 && which <= 22) {
            int f = (which - 7) / 4, k = (which - 7) % 4;
            const float *arr[4] = {g.Ut[f], g.Ux[f], g.Uy[f], g.Us[f]};
            src = arr[k];
            n = (k == 0 ? 4 : 2) * v;
        } else {
            return E_BAD_ARGUMENT;
        }
    }
    if (!dst) return (int)std::min<long>(n, 0x7fffffff);
    if (cap < n) return E_TOO_LARGE;
    std::vector<float> h(n);
    CK(cudaMemcpyAsync(h.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    for (long i = 0; i < n; i++) dst[i] = h[i];
    return (int)n;
}

}  // namespace cfdwm
