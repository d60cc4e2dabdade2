// Depth-separable form of the s-grid column pair sums, on the tensor cores.
//
// The column update (lsgrid_spline.cpp:880-903 -> Irregular::uvw2,
// Irregular.cpp:975-1102) sums, at every level height z of a column,
//   u2(z) = sum_pairs r_i [Pu F(k+, z) cos(phi_i + phi_m) + Mu F(k-, z) cos(phi_i - phi_m)]
// (and v2 alike, w2 with G and sines), with the depth profiles
//   F(k, z) = q(k) (e^{kz} + e^{-k(z + 2h)}),  G(k, z) = q(k) (e^{kz} - e^{-k(z + 2h)}),
// q folded into the pair coefficients.  F and G do not factor into a part of
// the pair and a part of the level, which is why the plain form evaluates
// them per (pair, level).  Over k in [0, K] and z in [-h, 0] the two
// exponential families have a low numerical rank, though: with an
// orthonormal basis b_r(z) of their span (the eigenfunctions of the kernel
//   C(z, z') = int_0^K [e^{k(z+z')} + e^{-k(z+z'+4h)}] dk ),
//   e^{kz} + e^{-k(z+2h)} = sum_r f_r(k) b_r(z),  e^{kz} - e^{-k(z+2h)} = sum_r g_r(k) b_r(z)
// to 1e-8 with R of about 16 terms (a Karhunen-Loeve expansion).  Then
//   u2(z) = sum_r b_r(z) Q^u_r,   Q^u_r = sum_pairs r_i [Pu f_r(k+) cos(.+.) + Mu f_r(k-) cos(.-.)],
// and every Q_r is a quadratic form in the column's phasor vector -- the
// same shape as the precision form at z = 0 -- so the 3R forms and eta2 run
// as one tcgen05 GEMM over all columns (qform.cu), and the levels only
// combine R numbers per field.  The first-order sums stay exact
// (k_pairs_columns with pairs = 0).
//
// Set-up (host, FP64): Gauss-Legendre nodes on [-h, 0], the weighted kernel
// matrix, its eigenvectors by cyclic Jacobi rotations, b_r on a fine z table
// (barycentric interpolation through the nodes), f_r and g_r on a fine k
// table (quadrature).  The rank is the smallest R whose reconstruction error
// over a test set of (k, z) is below 4e-6 of max F: the profile error then
// stays at the level of the fp16x3 split's own error on the second-order sums
// (about 5e-6 of their maximum), and the whole field (first order included)
// differs from the plain form by a few 1e-7.
#include "cfdwm.h"
#include "ffmath.cuh"
#include "sgrid_geom.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace cfdwm {

// the cross products of the fp16 split in the hi accumulator (default) or in
// a second one (CFDWM_DF_TWO_ACC=1, the precision form's arrangement)
static bool df_one_acc() {
    const char *e = std::getenv("CFDWM_DF_TWO_ACC");
    return !(e && e[0] == '1');
}

#define CK(x)                                                  \
    do {                                                       \
        cudaError_t e_ = (x);                                  \
        if (e_ != cudaSuccess) {                               \
            std::fprintf(stderr, "cfdwm: CUDA error %s at %s:%d\n", \
                         cudaGetErrorString(e_), __FILE__, __LINE__); \
            return E_CUDA;                                     \
        }                                                      \
    } while (0)

constexpr int DF_RMAX = 32;
constexpr int DF_NK = 4097;      // k table points over [0, K]
constexpr int DF_NZ = 8193;      // z table points over [-h, 0]
constexpr int DF_TT = 32;        // pair-table tile of the grid tables (GRID_TILE)
constexpr int GRIDV_NC_DF = 8;   // grid uvw record: Pu, Mu, Pv, Mv, Pw, Mw, kp, km
constexpr int EATA_NC_DF = 2;    // grid eta record: A, B

// ---------------------------------------------------------------------------
// Host: basis construction
// ---------------------------------------------------------------------------
static void gauss_legendre(int n, double a, double b, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; i++) {
        double t = std::cos(3.141592653589793 * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = t;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (t * p1 - p0) / (t * t - 1.0);
            double dt = p1 / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-16) break;
        }
        {
            double p0 = 1.0, p1 = t;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (t * p1 - p0) / (t * t - 1.0);
        }
        x[i] = 0.5 * (a + b) + 0.5 * (b - a) * t;
        w[i] = (b - a) / ((1.0 - t * t) * dp * dp);
    }
}

// One-sided (Hestenes) Jacobi SVD of an m x n matrix G (column-major): the
// columns are rotated until mutually orthogonal.  On return sv holds the
// column norms (the singular values) and V (n x n, column-major) the right
// singular vectors.  It resolves small singular values to relative
// accuracy, which a Gram-matrix eigen-decomposition (squared condition)
// does not.
static void jacobi_svd(int m, int n, std::vector<double> &G, std::vector<double> &sv, std::vector<double> &V) {
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 80; sweep++) {
        bool rotated = false;
        for (int p = 0; p < n; p++) {
            double *gp = &G[(size_t)p * m];
            for (int q = p + 1; q < n; q++) {
                double *gq = &G[(size_t)q * m];
                double al = 0, be = 0, ga = 0;
                for (int i = 0; i < m; i++) {
                    al += gp[i] * gp[i];
                    be += gq[i] * gq[i];
                    ga += gp[i] * gq[i];
                }
                if (std::fabs(ga) <= 1e-15 * std::sqrt(al * be) || ga == 0.0) continue;
                rotated = true;
                double ze = (be - al) / (2.0 * ga);
                double t = (ze >= 0 ? 1.0 : -1.0) / (std::fabs(ze) + std::sqrt(1.0 + ze * ze));
                double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < m; i++) {
                    double a1 = gp[i], a2 = gq[i];
                    gp[i] = c * a1 - s * a2;
                    gq[i] = s * a1 + c * a2;
                }
                double *vp = &V[(size_t)p * n], *vq = &V[(size_t)q * n];
                for (int i = 0; i < n; i++) {
                    double a1 = vp[i], a2 = vq[i];
                    vp[i] = c * a1 - s * a2;
                    vq[i] = s * a1 + c * a2;
                }
            }
        }
        if (!rotated) break;
    }
    sv.assign(n, 0.0);
    for (int j = 0; j < n; j++) {
        double a = 0;
        for (int i = 0; i < m; i++) a += G[(size_t)j * m + i] * G[(size_t)j * m + i];
        sv[j] = std::sqrt(a);
    }
}

struct DfBasis {
    int R = 0, nz = 0;
    double K = 0, h = 0, err = 0;
    std::vector<double> zj, wj, b;   // b[r][j] = b_r(z_j)
};

// Barycentric interpolation weights of Gauss-Legendre nodes on [a, b]
// (monotone order): (-1)^j sqrt((1 - t_j^2) W_j), t_j the nodes and W_j the
// weights on [-1, 1] (Wang and Xiang, 2012), free of the over- and underflow
// of the product formula.
static std::vector<double> bary_weights(const std::vector<double> &x, const std::vector<double> &w, double a,
                                        double b) {
    int n = (int)x.size();
    std::vector<double> lw(n);
    for (int j = 0; j < n; j++) {
        double t = (2.0 * x[j] - (a + b)) / (b - a);
        double W = w[j] * 2.0 / (b - a);
        lw[j] = ((j & 1) ? -1.0 : 1.0) * std::sqrt((1.0 - t * t) * W);
    }
    return lw;
}

static double bary_eval(const std::vector<double> &x, const std::vector<double> &lw, const double *f, double z) {
    int n = (int)x.size();
    double num = 0.0, den = 0.0;
    for (int j = 0; j < n; j++) {
        double dz = z - x[j];
        if (dz == 0.0) return f[j];
        double t = lw[j] / dz;
        num += t * f[j];
        den += t;
    }
    return num / den;
}

static int build_basis(double K, double h, DfBasis &B) {
    const int nz = std::min(512, std::max(96, (int)std::ceil(0.75 * K * h) + 64));
    std::vector<double> z, w, kq, wq;
    gauss_legendre(nz, -h, 0.0, z, w);
    const int nk = 64;
    gauss_legendre(nk, 0.0, K, kq, wq);
    // rows: the two exponential families at the k nodes, columns: the z nodes,
    // both with the square roots of their quadrature weights
    const int m = 2 * nk;
    std::vector<double> G((size_t)m * nz);
    for (int j = 0; j < nz; j++)
        for (int a = 0; a < nk; a++) {
            double sw = std::sqrt(wq[a] * w[j]);
            G[(size_t)j * m + a] = sw * std::exp(kq[a] * z[j]);
            G[(size_t)j * m + nk + a] = sw * std::exp(-kq[a] * (z[j] + 2.0 * h));
        }
    std::vector<double> d, V;
    jacobi_svd(m, nz, G, d, V);
    std::vector<int> ord(nz);
    for (int i = 0; i < nz; i++) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return d[a] > d[b]; });
    // candidate basis (descending), b_r(z_j) = V_jr / sqrt(w_j)
    std::vector<double> bb((size_t)DF_RMAX * nz);
    for (int r = 0; r < DF_RMAX && r < nz; r++)
        for (int j = 0; j < nz; j++) bb[(size_t)r * nz + j] = V[(size_t)ord[r] * nz + j] / std::sqrt(w[j]);
    // smallest R with max |F - sum_r f_r b_r| <= 4e-6 * 2 over a test set
    std::vector<double> lw = bary_weights(z, w, -h, 0.0);
    const int nkt = 48, nzt = 160;
    const int rmax = std::min(DF_RMAX, nz);
    std::vector<double> zt(nzt), bt((size_t)rmax * nzt), ft((size_t)nkt * rmax), Ft((size_t)nkt * nzt);
    for (int c = 0; c < nzt; c++) zt[c] = -h + h * std::sqrt((double)c / (nzt - 1));   // dense near z = 0
    for (int r = 0; r < rmax; r++)
        for (int c = 0; c < nzt; c++) bt[(size_t)r * nzt + c] = bary_eval(z, lw, &bb[(size_t)r * nz], zt[c]);
    for (int a = 0; a < nkt; a++) {
        double k = K * a / (nkt - 1);
        for (int r = 0; r < rmax; r++) {
            double acc = 0.0;
            for (int j = 0; j < nz; j++)
                acc += w[j] * (std::exp(k * z[j]) + std::exp(-k * (z[j] + 2.0 * h))) * bb[(size_t)r * nz + j];
            ft[(size_t)a * rmax + r] = acc;
        }
        for (int c = 0; c < nzt; c++) Ft[(size_t)a * nzt + c] = std::exp(k * zt[c]) + std::exp(-k * (zt[c] + 2.0 * h));
    }
    int R = 0;
    double e_at_R = 0.0;
    for (int Rt = 8; Rt <= rmax; Rt += 2) {
        double emax = 0.0;
        for (int a = 0; a < nkt; a++)
            for (int c = 0; c < nzt; c++) {
                double Fa = 0.0;
                for (int r = 0; r < Rt; r++) Fa += ft[(size_t)a * rmax + r] * bt[(size_t)r * nzt + c];
                emax = std::max(emax, std::fabs(Ft[(size_t)a * nzt + c] - Fa));
            }
        if (emax <= 8e-6) {
            R = Rt;
            e_at_R = emax;
            break;
        }
    }
    if (R == 0) return E_UNSUPPORTED;
    B.err = e_at_R;
    B.R = R;
    B.nz = nz;
    B.K = K;
    B.h = h;
    B.zj = z;
    B.wj = w;
    B.b.assign(bb.begin(), bb.begin() + (size_t)R * nz);
    return OK;
}

// ---------------------------------------------------------------------------
// Device
// ---------------------------------------------------------------------------
__device__ __forceinline__ long df_tile_index(int I, int M, int nt) {
    return (long)I * nt - (long)I * (I - 1) / 2 + (M - I);
}

// cubic Lagrange interpolation on a uniform table (4 points, clamped)
__device__ __forceinline__ void cubic_w(double t, int n, int &i0, double wt[4]) {
    int i = (int)floor(t);
    i = max(1, min(n - 3, i));
    double u = t - i;              // in [0, 1] between points i and i+1
    i0 = i - 1;
    wt[0] = -u * (u - 1.0) * (u - 2.0) / 6.0;
    wt[1] = (u + 1.0) * (u - 1.0) * (u - 2.0) / 2.0;
    wt[2] = -(u + 1.0) * u * (u - 2.0) / 2.0;
    wt[3] = (u + 1.0) * u * (u - 1.0) / 6.0;
}

struct DfCoefArgs {
    int n, npad, ntile, R, nf;
    const float *tab_grid, *tab_eta, *tab_gp;
    const double *fk, *gk;    // [R][DF_NK]
    double inv_dk;
    double *coef;             // [2 + 2 nf R][npad][npad]
};

// One thread per (m, i): the coefficient of every block at W^T[m][i].
__global__ void k_depth_coef(DfCoefArgs a) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long tot = (long)a.npad * a.npad;
    if (e >= tot) return;
    const int m = (int)(e / a.npad), i = (int)(e % a.npad);
    const long nn = tot;
    const int nb = 2 + 2 * a.nf * a.R;
    if (i > m || i >= a.n || m >= a.n) {
        for (int b = 0; b < nb; b++) a.coef[(long)b * nn + e] = 0.0;
        return;
    }
    const int I = i / DF_TT, M = m / DF_TT, ii = i % DF_TT, mm = m % DF_TT;
    const long rec = df_tile_index(I, M, a.ntile) * DF_TT * DF_TT + ii * DF_TT + mm;
    const float *g = a.tab_grid + rec * GRIDV_NC_DF;
    const double Pu = g[0], Mu = g[1], Pv = g[2], Mv = g[3], Pw = g[4], Mw = g[5];
    const double kp = g[6], km = g[7];
    const double Pp = a.nf == 4 ? a.tab_gp[rec * 2] : 0.0, Mp = a.nf == 4 ? a.tab_gp[rec * 2 + 1] : 0.0;
    a.coef[e] = a.tab_eta[rec * EATA_NC_DF + 0];
    a.coef[nn + e] = a.tab_eta[rec * EATA_NC_DF + 1];
    int ip, im;
    double wp[4], wm[4];
    cubic_w(kp * a.inv_dk, DF_NK, ip, wp);
    cubic_w(km * a.inv_dk, DF_NK, im, wm);
    for (int r = 0; r < a.R; r++) {
        const double *fr = a.fk + (long)r * DF_NK, *gr = a.gk + (long)r * DF_NK;
        double fp = 0, fm = 0, gp = 0, gm = 0;
        for (int q = 0; q < 4; q++) {
            fp += wp[q] * fr[ip + q];
            gp += wp[q] * gr[ip + q];
            fm += wm[q] * fr[im + q];
            gm += wm[q] * gr[im + q];
        }
        double *c = a.coef + (long)(2 + 2 * a.nf * r) * nn + e;
        c[0] = Pu * fp + Mu * fm;          // u, c c
        c[nn] = Mu * fm - Pu * fp;         // u, s s
        c[2 * nn] = Pv * fp + Mv * fm;     // v, c c
        c[3 * nn] = Mv * fm - Pv * fp;     // v, s s
        c[4 * nn] = Pw * gp - Mw * gm;     // w, c s
        c[5 * nn] = Pw * gp + Mw * gm;     // w, s c
        if (a.nf == 4) {
            c[6 * nn] = Pp * fp + Mp * fm; // p, c c
            c[7 * nn] = Mp * fm - Pp * fp; // p, s s
        }
    }
}

// ---------------------------------------------------------------------------
// First-order sums of the columns for the tensor-core path, with float-float
// phases (the plain path's FP64 phasor pass and its per-(component, column)
// phasor table are not needed here):
//   mode 0: eta1 and the Taylor gradients phi1_dxdz, phi1_dydz, phi1_dzdz,
//           dp1_dz per column (Irregular.cpp:178-198, 1107-1192) into first[5][n];
//   mode 1: u1, v1, w1 (nf = 4: and dp1) at the level heights z0
//           (Irregular.cpp:394-447, 1107-1120) into sec[nf][n nl].
// Sums are FP32 with Kahan compensation.
// ---------------------------------------------------------------------------
struct DfFirstArgs {
    long n;
    const double *xy;          // [2][n]
    double t, fx, fy;
    const double *phase;       // [7][cstride]: kx, ky, omega, phase0, ramp parameters
    const float *cf;           // [NCF][cstride]
    int cstride, ncomp, trivial_ramp;
    int nl, nf;
    const float *z0;           // [n nl] (mode 1)
    float depth;
    double *first;             // [5][n] (mode 0)
    float *sec;                // [nf][n nl] (mode 1)
    const void *comps;         // this launch's component records (DfComp, ncomp of them)
};

constexpr int DFC = 128;       // components per shared-memory chunk
constexpr float LOG2E_DF = 1.4426950408889634f;

__device__ __forceinline__ float df_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void df_kahan(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// shared record of a component: phase coefficients as float pairs, ramp, 5 coefficients
struct DfComp {
    FfComp f;
    float c[5];
};

static_assert(sizeof(DfComp) == DF_COMP_FLOATS * sizeof(float), "component record size");

// The records of all components at this launch's time, one thread each:
// converting the FP64 phase rows and evaluating the FP64 ramp once here, not
// in every block (FP64 runs at a small fraction of the FP32 rate on this GPU;
// done per block it kept the FP64 pipe 71% busy in the level kernel).
template <int MODE>
__global__ void k_df_comps(DfFirstArgs a, DfComp *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.ncomp) return;
    const int cs = a.cstride;
    DfComp d;
    d.f = ff_component(a.phase, cs, i, a.trivial_ramp, a.t);
    if (MODE == 0) {
        d.c[0] = a.cf[CF_A * cs + i];
        d.c[1] = a.cf[CF_GX * cs + i];
        d.c[2] = a.cf[CF_GY * cs + i];
        d.c[3] = a.cf[CF_GZ * cs + i];
        d.c[4] = a.cf[CF_GP * cs + i];
    } else {
        const float au = a.cf[CF_AU * cs + i] * a.cf[CF_Q * cs + i];
        d.c[0] = a.cf[CF_K * cs + i];
        d.c[1] = au * a.cf[CF_CT * cs + i];
        d.c[2] = au * a.cf[CF_ST * cs + i];
        d.c[3] = au;
        d.c[4] = a.cf[CF_AP * cs + i] * a.cf[CF_Q * cs + i];
    }
    out[i] = d;
}

// a chunk of DFC records into shared memory (zero past the last component)
__device__ __forceinline__ void df_stage(const DfFirstArgs &a, int i0, DfComp *sc) {
    const float *src = reinterpret_cast<const float *>(a.comps) + (long)i0 * DF_COMP_FLOATS;
    float *dst = reinterpret_cast<float *>(sc);
    const int nrec = min(DFC, a.ncomp - i0);
    for (int e = threadIdx.x; e < DFC * DF_COMP_FLOATS; e += blockDim.x)
        dst[e] = e < nrec * DF_COMP_FLOATS ? src[e] : 0.f;
}

__global__ void __launch_bounds__(128) k_df_first_surface(DfFirstArgs a) {
    __shared__ DfComp sc[DFC];
    const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const bool valid = p < a.n;
    const long pc = valid ? p : 0;
    float dxh, dxl, dyh, dyl, th, tl;
    ff_split(a.xy[pc] - a.fx, dxh, dxl);
    ff_split(a.xy[a.n + pc] - a.fy, dyh, dyl);
    ff_split(a.t, th, tl);
    float s[5] = {0, 0, 0, 0, 0}, k[5] = {0, 0, 0, 0, 0};
    for (int i0 = 0; i0 < a.ncomp; i0 += DFC) {
        __syncthreads();
        df_stage(a, i0, sc);
        __syncthreads();
        const int iend = min(DFC, a.ncomp - i0);
        for (int ii = 0; ii < iend; ii++) {
            const DfComp &d = sc[ii];
            float c, sn;
            ff_phasor(d.f, dxh, dxl, dyh, dyl, th, tl, c, sn);
            const float rc = d.f.r * c, rs = d.f.r * sn;
            df_kahan(s[0], k[0], rc * d.c[0]);
            df_kahan(s[1], k[1], rc * d.c[1]);
            df_kahan(s[2], k[2], rc * d.c[2]);
            df_kahan(s[3], k[3], rs * d.c[3]);
            df_kahan(s[4], k[4], rc * d.c[4]);
        }
    }
    if (!valid) return;
    for (int q = 0; q < 5; q++) a.first[q * a.n + p] = (double)s[q] - (double)k[q];
}

// blockDim = 32 columns x up to 8 level groups of 4 levels; blockIdx.y: further level groups.
// The warps of a block hold the same 32 columns: each computes the phasors of
// every nw-th component of a chunk into shared memory, and all of them read
// the whole chunk, so a (column, component) phasor is formed once per block.
// A chunk's terms are summed in FP32 and the chunk sum is added to a Kahan
// (sum, carry) pair per output.
__global__ void __launch_bounds__(256) k_df_first_levels(DfFirstArgs a) {
    __shared__ DfComp sc[DFC];
    __shared__ float2 s_ph[DFC][32];     // (r cos, r sin) of (component, column)
    const int cl = threadIdx.x & 31, wg = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int lg = blockIdx.y * nw + wg;
    const long p = (long)blockIdx.x * 32 + cl;
    const bool valid = p < a.n;
    const long pc = valid ? p : 0;
    float dxh, dxl, dyh, dyl, th, tl;
    ff_split(a.xy[pc] - a.fx, dxh, dxl);
    ff_split(a.xy[a.n + pc] - a.fy, dyh, dyl);
    ff_split(a.t, th, tl);
    float zk[4], yk[4];
#pragma unroll
    for (int l = 0; l < 4; l++) {
        const int m = lg * 4 + l;
        const float z = (valid && m < a.nl) ? a.z0[pc * a.nl + m] : 0.f;
        zk[l] = z * LOG2E_DF;
        yk[l] = -(z + 2.f * a.depth) * LOG2E_DF;
    }
    float su[4] = {0, 0, 0, 0}, sv[4] = {0, 0, 0, 0}, sw[4] = {0, 0, 0, 0}, sp[4] = {0, 0, 0, 0};
    float cu[4] = {0, 0, 0, 0}, cv[4] = {0, 0, 0, 0}, cw[4] = {0, 0, 0, 0}, cp[4] = {0, 0, 0, 0};
    const bool pres = a.nf == 4;
    for (int i0 = 0; i0 < a.ncomp; i0 += DFC) {
        __syncthreads();
        df_stage(a, i0, sc);
        __syncthreads();
        const int iend = min(DFC, a.ncomp - i0);
        for (int ii = wg; ii < iend; ii += nw) {
            float c, sn;
            ff_phasor(sc[ii].f, dxh, dxl, dyh, dyl, th, tl, c, sn);
            s_ph[ii][cl] = make_float2(sc[ii].f.r * c, sc[ii].f.r * sn);
        }
        __syncthreads();
        float tu[4] = {0, 0, 0, 0}, tv[4] = {0, 0, 0, 0}, tw[4] = {0, 0, 0, 0}, tp[4] = {0, 0, 0, 0};
        for (int ii = 0; ii < iend; ii++) {
            const DfComp &d = sc[ii];
            const float2 ph = s_ph[ii][cl];
            const float au = d.c[1] * ph.x, av = d.c[2] * ph.x, aw = d.c[3] * ph.y, k = d.c[0];
            const float ap = d.c[4] * ph.x;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                // cosh(k(z+h))/cosh(kh) = q (E + Y), sinh(k(z+h))/cosh(kh) = q (E - Y)
                const float E = df_ex2(k * zk[l]), Y = df_ex2(k * yk[l]);
                const float F = E + Y, G = E - Y;
                tu[l] = fmaf(au, F, tu[l]);
                tv[l] = fmaf(av, F, tv[l]);
                tw[l] = fmaf(aw, G, tw[l]);
                if (pres) tp[l] = fmaf(ap, F, tp[l]);
            }
        }
#pragma unroll
        for (int l = 0; l < 4; l++) {
            df_kahan(su[l], cu[l], tu[l]);
            df_kahan(sv[l], cv[l], tv[l]);
            df_kahan(sw[l], cw[l], tw[l]);
            if (pres) df_kahan(sp[l], cp[l], tp[l]);
        }
    }
    if (!valid) return;
    const long tot = a.n * a.nl;
#pragma unroll
    for (int l = 0; l < 4; l++) {
        const int m = lg * 4 + l;
        if (m >= a.nl) continue;
        const long o = p * a.nl + m;
        a.sec[o] = su[l];
        a.sec[tot + o] = sv[l];
        a.sec[2 * tot + o] = sw[l];
        if (pres) a.sec[3 * tot + o] = sp[l];
    }
}

// eta2 of the columns from output column 0
__global__ void k_df_take(long n, int nout, const float *out, float *eta2) {
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q < n) eta2[q] = out[q * nout];
}

// sec[f][e] += sum_r b_r(z0[e]) Q[q][1 + nf r + f], e = q nl + m
__global__ void k_df_combine(long nact, int nl, int R, int nf, int nout, const float *z0, const float *out,
                             const float *bz, float h, float inv_dz, float *sec) {
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long tot = nact * nl;
    if (e >= tot) return;
    long q = e / nl;
    float t = (z0[e] + h) * inv_dz;
    int i = (int)floorf(t);
    i = max(1, min(DF_NZ - 3, i));
    float u = t - i;
    float w0 = -u * (u - 1.f) * (u - 2.f) * (1.f / 6.f);
    float w1 = (u + 1.f) * (u - 1.f) * (u - 2.f) * 0.5f;
    float w2 = -(u + 1.f) * u * (u - 2.f) * 0.5f;
    float w3 = (u + 1.f) * u * (u - 1.f) * (1.f / 6.f);
    const float *Q = out + q * nout + 1;
    float su = 0.f, sv = 0.f, sw = 0.f, sp = 0.f;
    for (int r = 0; r < R; r++) {
        const float *b = bz + (long)r * DF_NZ + i - 1;
        float br = w0 * b[0] + w1 * b[1] + w2 * b[2] + w3 * b[3];
        su = fmaf(br, Q[nf * r], su);
        sv = fmaf(br, Q[nf * r + 1], sv);
        sw = fmaf(br, Q[nf * r + 2], sw);
        if (nf == 4) sp = fmaf(br, Q[nf * r + 3], sp);
    }
    sec[e] += su;
    sec[tot + e] += sv;
    sec[2 * tot + e] += sw;
    if (nf == 4) sec[3 * tot + e] += sp;
}

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
int depthform_build(const Config &cfg, const DevSea &sea, DepthForm &df, int nf, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    depthform_free(df);
    if (nf != 3 && nf != 4) return E_BAD_ARGUMENT;
    if (sea.n < 1 || !sea.d_tab_grid || !sea.d_tab_eta || (nf == 4 && !sea.d_tab_gp)) return E_NOT_INITIALIZED;
    double kmax = sea.kmax;
    for (double k : cfg.k) kmax = std::max(kmax, k);
    // the pair wavenumbers |k_i +- k_m| and the diagonal 2 k are <= 2 kmax
    const double K = 2.0 * kmax * (1.0 + 1e-9) + 1e-12;
    const double h = cfg.depth;
    DfBasis B;
    int rc = build_basis(K, h, B);
    if (rc) return rc;
    const int R = B.R, nz = B.nz;
    // k tables f_r(k), g_r(k) by quadrature; z table b_r(z) by barycentric interpolation
    std::vector<double> fk((size_t)R * DF_NK), gk((size_t)R * DF_NK);
    const double dk = K / (DF_NK - 1);
    for (int a = 0; a < DF_NK; a++) {
        double k = dk * a;
        std::vector<double> E(nz), Y(nz);
        for (int j = 0; j < nz; j++) {
            E[j] = std::exp(k * B.zj[j]);
            Y[j] = std::exp(-k * (B.zj[j] + 2.0 * h));
        }
        for (int r = 0; r < R; r++) {
            double f = 0.0, g = 0.0;
            for (int j = 0; j < nz; j++) {
                double wb = B.wj[j] * B.b[(size_t)r * nz + j];
                f += wb * (E[j] + Y[j]);
                g += wb * (E[j] - Y[j]);
            }
            fk[(size_t)r * DF_NK + a] = f;
            gk[(size_t)r * DF_NK + a] = g;
        }
    }
    std::vector<double> lw = bary_weights(B.zj, B.wj, -h, 0.0);
    std::vector<float> bz((size_t)R * DF_NZ);
    const double dz = h / (DF_NZ - 1);
    for (int r = 0; r < R; r++)
        for (int c = 0; c < DF_NZ; c++)
            bz[(size_t)r * DF_NZ + c] = (float)bary_eval(B.zj, lw, &B.b[(size_t)r * nz], -h + dz * c);
    df.R = R;
    df.K = K;
    df.h = h;
    df.nf = nf;
    df.nout = 1 + nf * R;
    CK(cudaMalloc(&df.bz, sizeof(float) * bz.size()));
    CK(cudaMemcpyAsync(df.bz, bz.data(), sizeof(float) * bz.size(), cudaMemcpyHostToDevice, stream));
    double *d_fk = nullptr, *d_gk = nullptr, *coef = nullptr;
    CK(cudaMalloc(&d_fk, sizeof(double) * fk.size()));
    CK(cudaMalloc(&d_gk, sizeof(double) * gk.size()));
    CK(cudaMemcpyAsync(d_fk, fk.data(), sizeof(double) * fk.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_gk, gk.data(), sizeof(double) * gk.size(), cudaMemcpyHostToDevice, stream));
    const int npad = ((sea.n + TC_NPAD - 1) / TC_NPAD) * TC_NPAD;
    const int nblk = 2 + 2 * nf * R;
    CK(cudaMalloc(&coef, sizeof(double) * (size_t)nblk * npad * npad));
    DfCoefArgs a;
    a.n = sea.n; a.npad = npad; a.ntile = sea.ntile_g; a.R = R; a.nf = nf;
    a.tab_grid = sea.d_tab_grid; a.tab_eta = sea.d_tab_eta; a.tab_gp = sea.d_tab_gp; a.fk = d_fk; a.gk = d_gk;
    a.inv_dk = 1.0 / dk; a.coef = coef;
    long tot = (long)npad * npad;
    k_depth_coef<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(a);
    note_launch();
    CK(cudaGetLastError());
    // blocks: eta (c c, s s), then per r: u (c c, s s), v (c c, s s), w (c s, s c)
    // and, nf = 4, p (c c, s s)
    std::vector<int> bmap(3 * nblk);
    auto setb = [&](int b, int kh, int yh, int col) { bmap[3 * b] = kh; bmap[3 * b + 1] = yh; bmap[3 * b + 2] = col; };
    setb(0, 0, 0, 0);
    setb(1, 1, 1, 0);
    for (int r = 0; r < R; r++) {
        int b = 2 + 2 * nf * r, o = 1 + nf * r;
        setb(b + 0, 0, 0, o);
        setb(b + 1, 1, 1, o);
        setb(b + 2, 0, 0, o + 1);
        setb(b + 3, 1, 1, o + 1);
        setb(b + 4, 0, 1, o + 2);
        setb(b + 5, 1, 0, o + 2);
        if (nf == 4) {
            setb(b + 6, 0, 0, o + 3);
            setb(b + 7, 1, 1, o + 3);
        }
    }
    // fp16 split with one accumulator: the K range of a tile is short here
    // (256-1024 components), so the cross products keep their bits in the hi
    // accumulator, and the two accumulator buffers hide each tile's epilogue
    rc = tcform_split(df.tc, coef, bmap.data(), nblk, df.nout, npad, true, stream, df_one_acc());
    cudaFree(coef);
    cudaFree(d_fk);
    cudaFree(d_gk);
    if (rc) return rc;
    df.built = true;
    return OK;
}

// Host-only check of the basis construction (no device work).
int depthform_basis_info(double K, double h, int *R, double *err) {
    if (!(K > 0) || !(h > 0)) return E_BAD_ARGUMENT;
    DfBasis B;
    int rc = build_basis(K, h, B);
    if (rc) return rc;
    if (R) *R = B.R;
    if (err) *err = B.err;
    return OK;
}

void depthform_free(DepthForm &df) {
    tcform_free(df.tc);
    if (df.bz) cudaFree(df.bz);
    if (df.qout) cudaFree(df.qout);
    df = DepthForm();
}

// second-order sums of the columns act[0..nact): eta2 [nact] and the basis
// coefficients of the level sums in qout (combined by depthform_combine)
int depthform_columns(DepthForm &df, const DevSea &sea, long nact, const double *x, const double *y,
                      const double *tdev, float *eta2, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (!df.built) return E_NOT_INITIALIZED;
    if (df.qcap < nact) {
        if (df.qout) cudaFree(df.qout);
        df.qout = nullptr;
        df.qcap = 0;
        CK(cudaMalloc(&df.qout, sizeof(float) * df.nout * nact));
        df.qcap = nact;
    }
    int rc = tcform_eval(df.tc, sea, nact, x, y, tdev, 0, df.qout, stream, nullptr);
    if (rc) return rc;
    k_df_take<<<(unsigned)((nact + 255) / 256), 256, 0, stream>>>(nact, df.nout, df.qout, eta2);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

int depthform_first(const DevSea &sea, long nact, int nl, const double *xy, double t, const float *z0,
                    double *first, float *sec, int nf, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (nact <= 0) return OK;
    DfFirstArgs a;
    a.n = nact; a.xy = xy; a.t = t; a.fx = sea.fx; a.fy = sea.fy;
    a.phase = sea.d_phase; a.cf = sea.d_cf; a.cstride = sea.npad_g; a.ncomp = sea.n;
    a.trivial_ramp = sea.trivial_ramp ? 1 : 0;
    a.nl = nl; a.nf = nf; a.z0 = z0; a.depth = (float)sea.depth; a.first = first; a.sec = sec;
    if (!sea.d_dfcomp) return E_NOT_INITIALIZED;
    DfComp *recs = reinterpret_cast<DfComp *>(sea.d_dfcomp);
    const unsigned cb = (unsigned)((sea.n + 127) / 128);
    if (first) {
        k_df_comps<0><<<cb, 128, 0, stream>>>(a, recs);
        note_launch();
        a.comps = recs;
        k_df_first_surface<<<(unsigned)((nact + 127) / 128), 128, 0, stream>>>(a);
        note_launch();
        CK(cudaGetLastError());
    }
    if (sec) {
        const int ngrp = (nl + 3) / 4;
        const int gpb = std::min(ngrp, 8);
        dim3 grid((unsigned)((nact + 31) / 32), (unsigned)((ngrp + gpb - 1) / gpb));
        k_df_comps<1><<<cb, 128, 0, stream>>>(a, recs + sea.npad_g);
        note_launch();
        a.comps = recs + sea.npad_g;
        k_df_first_levels<<<grid, 32 * gpb, 0, stream>>>(a);
        note_launch();
        CK(cudaGetLastError());
    }
    return OK;
}

int depthform_combine(DepthForm &df, long nact, int nl, const float *z0, float *sec, void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    long tot = nact * nl;
    k_df_combine<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(nact, nl, df.R, df.nf, df.nout, z0, df.qout,
                                                                    df.bz,
                                                                    (float)df.h,
                                                                    (float)((DF_NZ - 1) / df.h), sec);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

int depthform_error(DepthForm &df, void *stream_) {
    if (!df.built) return OK;
    int h = 0;
    CK(cudaMemcpyAsync(&h, df.tc.err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream_));
    CK(cudaStreamSynchronize((cudaStream_t)stream_));
    return h;
}

}  // namespace cfdwm
