// Valid 3x3 convolutions of the learned s-grid update as implicit GEMMs on
// the tcgen05 tensor cores (forward, data gradient and weight gradient).
//
// The network (surrogate.cu) keeps its activations as FP32 planes
// [B][C][H][W] and its weights as BF16 [O][C][9].  Each convolution is a GEMM
// whose operand tiles the CUDA cores gather from those planes straight into
// shared memory, in the K-major 128-byte swizzle layout the tensor cores read,
// one 64-wide K stage at a time; two stages are in flight, so the MMAs of one
// stage run while the threads gather the next:
//   forward      D[pixel][o]    = sum_{tap, c} x[c][pixel + tap] w[o][c][tap]
//   data grad    D[pixel][c]    = sum_{tap, o} dy[o][pixel - tap] w[o][c][tap]
//   weight grad  D[tap, c][o]   = sum_{pixel}  x[c][pixel + tap] dy[o][pixel]
//                                 (per slab of pixels; the slabs are summed in
//                                 order afterwards, so the result is
//                                 deterministic)
// M = 128 rows per CTA (two threads per row, each gathering half of a K
// stage), N = the channel count padded to 32 or 64, K = 16 per MMA; D is an
// FP32 accumulator in TMEM, read back with tcgen05.ld by the warps of its
// lane quarter.  The weights of a forward or data-gradient launch are packed
// once into the K-contiguous B layout, so a stage's B tile is one 16-byte
// copy per chunk.  The FP32 activations and
// gradients are split into BF16 hi + lo parts (16 significant bits, error
// <= 2^-17 of the value); the weights are BF16 already, so the forward and
// data-gradient GEMMs take two MMAs per K step (hi, lo) and the weight
// gradient, whose two operands are both split, three (hi hi, hi lo, lo hi).
// Every mbarrier wait is bounded and sets the error word when it gives up.
#include "cfdwm.h"
#include "tc05.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

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

constexpr int CT_M = 128;                 // GEMM rows per CTA, one per thread
constexpr int CT_K = 64;                  // K per stage: one 128-byte swizzled row of BF16
constexpr int CT_ATILE = CT_M * CT_K * 2; // 16 KiB, one split part of A

enum { CT_FWD = 0, CT_DATA = 1, CT_WGT = 2 };

struct TcConv {
    const float *x;              // FWD, WGT: input planes [*][C][H][W]
    long xbs;                    // batch stride of x
    const int *idx;              // sample index of batch entry b (null: b)
    const float *dy;             // DATA, WGT: output gradient [B][O][H-2][W-2]
    const __nv_bfloat16 *w;      // FWD, DATA: the packed B operand [NP][Kp] (k_ct_pack)
    const float *bias;           // FWD
    float *pre;                  // FWD: pre-activation copy (written, may be null);
                                 // DATA: pre-activation of the input (read, may be null)
    float *out;                  // FWD: y [B][O][H-2][W-2]; DATA: dx [B][C][H][W];
                                 // WGT: per-slab partial sums [slab][O C 9 + O]
    int B, C, O, H, W;
    int act;                     // FWD: SiLU
    int kslab;                   // WGT: output pixels per slab
    int slabs_per_img;           // WGT
    int *err;
};

__device__ __forceinline__ float ct_silu(float a) { return a / (1.f + expf(-a)); }
__device__ __forceinline__ float ct_silu_d(float a) {
    float s = 1.f / (1.f + expf(-a));
    return s * (1.f + a * (1.f - s));
}

// byte offset of the 16-byte chunk j (elements 8j..8j+7) of row r in a K-major
// tile of 128-byte rows with the 128-byte swizzle (8-row atoms of 1024 B)
__device__ __forceinline__ uint32_t swz(int r, int j) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((j ^ (r & 7)) << 4));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// eight values into the hi and lo tiles of row r, chunk j
__device__ __forceinline__ void put8_split(uint8_t *hi, uint8_t *lo, int r, int j, const float *v) {
    float h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        h[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
        l[e] = v[e] - h[e];
    }
    const uint32_t o = swz(r, j);
    *reinterpret_cast<uint4 *>(hi + o) =
        make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
    *reinterpret_cast<uint4 *>(lo + o) =
        make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]), pack_bf16(l[6], l[7]));
}

constexpr int CT_THREADS = 256;           // two threads per A row, each half of its K stage

template <int OP, int NP>
struct CtCfg {
    static constexpr int BTILE = NP * CT_K * 2;                  // B: NP rows of 128 B
    static constexpr int NBP = OP == CT_WGT ? 2 : 1;             // split parts of B
    static constexpr int STAGE = 2 * CT_ATILE + NBP * BTILE;     // a multiple of 1024
    static constexpr int SMEM = 2 * STAGE + 1024 + 64 + 8 * 64 * 4;
};

// B operand of the forward (op 0) and data-gradient (op 1) GEMMs, [NP][Kp]
// BF16, K contiguous: forward B[o][tap C + c] = w[o][c][tap]; data gradient
// B[c][tap O + o] = w[o][c][tap]; zero past O (C) and past 9 C (9 O).
__global__ void k_ct_pack(const __nv_bfloat16 *w, int C, int O, int op, int NP, int Kp, __nv_bfloat16 *out) {
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= (long)NP * Kp) return;
    const int n = (int)(e / Kp), k = (int)(e % Kp);
    __nv_bfloat16 v = __float2bfloat16_rn(0.f);
    if (op == CT_FWD) {
        const int tap = k / C, c = k % C;
        if (n < O && tap < 9) v = w[((long)n * C + c) * 9 + tap];
    } else {
        const int tap = k / O, o = k % O;
        if (n < C && tap < 9) v = w[((long)o * C + n) * 9 + tap];
    }
    out[e] = v;
}

template <int OP, int NP>
__global__ void __launch_bounds__(CT_THREADS, 2) k_conv_tc(TcConv a) {
    using CF = CtCfg<OP, NP>;
    constexpr int BTILE = CF::BTILE, STAGE = CF::STAGE;
    extern __shared__ __align__(1024) uint8_t ct_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)ct_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bar = (uint64_t *)(smem + 2 * STAGE);      // [0, 1] stage released, [2] all MMAs done
    uint32_t *tslot = (uint32_t *)(bar + 4);
    float *red = (float *)(bar + 8);                     // WGT: bias partial sums [8][64]
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & (CT_M - 1), half = tid >> 7;     // A row, and which half of its K stage
    const int Ho = a.H - 2, Wo = a.W - 2;
    const long plane = (long)a.H * a.W, oplane = (long)Ho * Wo;

    // this CTA's rows and K extent
    int b, slab = 0;
    long row = 0, q0 = 0, q1 = 0, K;
    bool live;
    if (OP == CT_WGT) {
        slab = blockIdx.x;
        b = slab / a.slabs_per_img;
        q0 = (long)(slab % a.slabs_per_img) * a.kslab;
        q1 = q0 + a.kslab < oplane ? q0 + a.kslab : oplane;
        row = (long)blockIdx.y * CT_M + r;               // (tap, c) = (row / C, row % C)
        live = row < 9L * a.C;
        K = q1 - q0;
    } else {
        b = blockIdx.y;
        row = (long)blockIdx.x * CT_M + r;               // pixel of the output (FWD) or input (DATA) plane
        live = row < (OP == CT_FWD ? oplane : plane);
        K = 9L * (OP == CT_FWD ? a.C : a.O);
    }
    const int nst = (int)((K + CT_K - 1) / CT_K);
    const long Kp = (long)nst * CT_K;
    const float *X = (OP != CT_DATA) ? a.x + (long)(a.idx ? a.idx[b] : b) * a.xbs : nullptr;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    constexpr uint32_t TCOLS = NP < 32 ? 32 : NP;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    // per-thread constants of the A row
    int ay = 0, ax = 0, wc = 0, wtap = 0;
    if (OP == CT_WGT) {
        wtap = live ? (int)(row / a.C) : 0;
        wc = live ? (int)(row % a.C) : 0;
    } else if (live) {
        const int pw = OP == CT_FWD ? Wo : a.W;
        ay = (int)(row / pw);
        ax = (int)(row % pw);
    }
    // B chunks of a stage: NP rows x 8 chunks of 16 B; chunk id = tid + 256 q
    constexpr int BCH = NP * 8 / CT_THREADS;             // 1 (NP = 32) or 2 (NP = 64)
    float bsum[BCH];
#pragma unroll
    for (int q = 0; q < BCH; q++) bsum[q] = 0.f;

    bool failed = false;
    for (int s = 0; s < nst; s++) {
        const int buf = s & 1;
        uint8_t *st = smem + buf * STAGE;
        uint8_t *Ahi = st, *Alo = st + CT_ATILE, *Bhi = st + 2 * CT_ATILE, *Blo = Bhi + BTILE;
        bool ok = true;
        if (s >= 2) ok = mbar_wait(&bar[buf], (uint32_t)(((s >> 1) - 1) & 1), a.err, 11);
        if (__syncthreads_or(!ok)) { failed = true; break; }
        const long k0 = (long)s * CT_K + half * (CT_K / 2);
        // ---- half of the A row of this thread: 32 K values, gathered with all
        // loads in flight, the K index walked incrementally
        float v[32];
        if (OP == CT_WGT) {
            long q = q0 + k0;
            int oy = (int)(q / Wo), ox = (int)(q - (long)oy * Wo);
            const float *xr = X + (long)wc * plane + (long)(wtap / 3) * a.W + wtap % 3;
#pragma unroll
            for (int e = 0; e < 32; e++) {
                v[e] = (live && k0 + e < K) ? xr[(long)oy * a.W + ox] : 0.f;
                if (++ox == Wo) { ox = 0; oy++; }
            }
        } else {
            const int cdim = OP == CT_FWD ? a.C : a.O;
            int tap = (int)(k0 / cdim), c = (int)(k0 - (long)tap * cdim);
#pragma unroll
            for (int e = 0; e < 32; e++) {
                float val = 0.f;
                if (live && k0 + e < K) {
                    if (OP == CT_FWD) {
                        val = X[(long)c * plane + (long)(ay + tap / 3) * a.W + ax + tap % 3];
                    } else {
                        const int yy = ay - tap / 3, xx = ax - tap % 3;
                        if (yy >= 0 && yy < Ho && xx >= 0 && xx < Wo)
                            val = a.dy[((long)b * a.O + c) * oplane + (long)yy * Wo + xx];
                    }
                }
                v[e] = val;
                if (++c == cdim) { c = 0; tap++; }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) put8_split(Ahi, Alo, r, half * 4 + j, v + 8 * j);
        // ---- B chunks
#pragma unroll
        for (int q = 0; q < BCH; q++) {
            const int id = tid + CT_THREADS * q, n = id >> 3, j = id & 7;
            const long kc = (long)s * CT_K + j * 8;
            if (OP == CT_WGT) {
                float bv[8];
                const float *dr = a.dy + ((long)b * a.O + n) * oplane + q0;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const float val = (n < a.O && kc + e < K) ? dr[kc + e] : 0.f;
                    bsum[q] += val;
                    bv[e] = val;
                }
                put8_split(Bhi, Blo, n, j, bv);
            } else {
                // the packed weights: one 16-byte chunk
                const uint4 c4 = *reinterpret_cast<const uint4 *>(a.w + (long)n * Kp + kc);
                *reinterpret_cast<uint4 *>(Bhi + swz(n, j)) = c4;
            }
        }
        // the generic-proxy writes become visible to the tensor cores' reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NP >> 3) << 17) |
                                   ((uint32_t)(CT_M >> 4) << 24);
            const uint64_t dAh = sdesc(su32(Ahi)), dAl = sdesc(su32(Alo)), dBh = sdesc(su32(Bhi));
            const uint64_t dBl = sdesc(su32(Blo));
#pragma unroll
            for (int k = 0; k < CT_K / 16; k++) {
                const uint64_t o = (uint64_t)(k * 32) >> 4;        // 16 BF16 = 32 bytes per step
                const uint32_t first = (s == 0 && k == 0) ? 0u : 1u;
                umma(tmem, dAh + o, dBh + o, idesc, first);
                umma(tmem, dAl + o, dBh + o, idesc, 1u);
                if (OP == CT_WGT) umma(tmem, dAh + o, dBl + o, idesc, 1u);
            }
            umma_commit(&bar[buf]);
        }
    }
    if (tid == 0 && !failed) umma_commit(&bar[2]);
    bool ok = !failed && nst > 0 && mbar_wait(&bar[2], 0u, a.err, 12);
    ok = !__syncthreads_or(!ok);
    if (ok) {
        // warp w reads TMEM lane quarter w % 4, column half w / 4
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        constexpr int HC = NP / 2;
        const int c0 = half * HC;
        const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0;
        float d[HC];
        if constexpr (HC == 32) tmem_ld32(ta, d);
        else tmem_ld16(ta, d);
        if (live) {
#pragma unroll
            for (int n = 0; n < HC; n++) {
                const int ch = c0 + n;
                if (OP == CT_FWD) {
                    if (ch >= a.O) break;
                    const long off = ((long)b * a.O + ch) * oplane + row;
                    const float val = d[n] + a.bias[ch];
                    if (a.pre) a.pre[off] = val;
                    a.out[off] = a.act ? ct_silu(val) : val;
                } else if (OP == CT_DATA) {
                    if (ch >= a.C) break;
                    const long off = ((long)b * a.C + ch) * plane + row;
                    a.out[off] = a.pre ? d[n] * ct_silu_d(a.pre[off]) : d[n];
                } else {
                    if (ch >= a.O) break;
                    const long per = (long)a.O * a.C * 9 + a.O;
                    a.out[(long)slab * per + ((long)ch * a.C + wc) * 9 + wtap] = d[n];
                }
            }
        }
    }
    if (OP == CT_WGT && blockIdx.y == 0) {
        // bias gradient of the slab: the sum of dy over its pixels, the eight
        // chunks of a row added in a fixed order
#pragma unroll
        for (int q = 0; q < BCH; q++) {
            const int id = tid + CT_THREADS * q;
            red[(id & 7) * 64 + (id >> 3)] = bsum[q];
        }
        __syncthreads();
        if (tid < NP && tid < a.O) {
            float t = 0.f;
            for (int j = 0; j < 8; j++) t += red[j * 64 + tid];
            const long per = (long)a.O * a.C * 9 + a.O;
            a.out[(long)slab * per + (long)a.O * a.C * 9 + tid] = t;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
}

template <int OP, int NP>
int launch_ct(const TcConv &a, dim3 grid, cudaStream_t st) {
    using CF = CtCfg<OP, NP>;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_conv_tc<OP, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM);
    CK(attr);
    k_conv_tc<OP, NP><<<grid, CT_THREADS, CF::SMEM, st>>>(a);
    note_launch();
    CK(cudaGetLastError());
    return OK;
}

int *g_ct_err = nullptr;      // error word of the bounded waits (device)
std::mutex g_ct_mtx;          // serialises the lazy allocations of this file

int ct_err_word(int **p) {
    std::lock_guard<std::mutex> lk(g_ct_mtx);
    if (!g_ct_err) {
        CK(cudaMalloc(&g_ct_err, sizeof(int)));
        CK(cudaMemset(g_ct_err, 0, sizeof(int)));
    }
    *p = g_ct_err;
    return OK;
}

// The B operand of a forward or data-gradient launch, packed by k_ct_pack into
// one device buffer that the launches reuse in turn.  The network is a
// process-wide singleton driven from one stream (surrogate.cu); the buffer
// follows the same rule, and its (re)allocation is serialised.
__nv_bfloat16 *g_ct_w = nullptr;
long g_ct_w_cap = 0;

int ct_pack(const __nv_bfloat16 *w, int C, int O, int op, int NP, long Kp, cudaStream_t st,
            const __nv_bfloat16 **out) {
    std::lock_guard<std::mutex> lk(g_ct_mtx);
    const long n = (long)NP * Kp;
    if (n > g_ct_w_cap) {
        if (g_ct_w) cudaFree(g_ct_w);
        g_ct_w = nullptr;
        g_ct_w_cap = 0;
        CK(cudaMalloc(&g_ct_w, sizeof(__nv_bfloat16) * n));
        g_ct_w_cap = n;
    }
    k_ct_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(w, C, O, op, NP, (int)Kp, g_ct_w);
    note_launch();
    CK(cudaGetLastError());
    *out = g_ct_w;
    return OK;
}

}  // namespace

// y[b][o] = act(conv3x3(x[b]) + bias), with the pre-activation copied to pre.
int conv_tc_forward(const float *x, long xbs, const int *idx, const __nv_bfloat16 *w, const float *bias, int B,
                    int C, int O, int H, int W, float *y, float *pre, int act, void *stream) {
    if (O < 1 || O > 64 || C < 1 || H < 3 || W < 3 || B < 1) return E_BAD_ARGUMENT;
    TcConv a = {};
    a.x = x; a.xbs = xbs; a.idx = idx; a.bias = bias; a.pre = pre; a.out = y;
    a.B = B; a.C = C; a.O = O; a.H = H; a.W = W; a.act = act;
    int rc = ct_err_word(&a.err);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int NP = O <= 32 ? 32 : 64;
    const long Kp = (9L * C + CT_K - 1) / CT_K * CT_K;
    if ((rc = ct_pack(w, C, O, CT_FWD, NP, Kp, st, &a.w))) return rc;
    const long opl = (long)(H - 2) * (W - 2);
    dim3 grid((unsigned)((opl + CT_M - 1) / CT_M), (unsigned)B);
    return NP == 32 ? launch_ct<CT_FWD, 32>(a, grid, st) : launch_ct<CT_FWD, 64>(a, grid, st);
}

// dx[b][c] = conv3x3^T(dy[b]) times silu'(pre) when pre is given.
int conv_tc_data_grad(const float *dy, const __nv_bfloat16 *w, const float *pre, int B, int C, int O, int H, int W,
                      float *dx, void *stream) {
    if (C < 1 || C > 64 || O < 1 || H < 3 || W < 3 || B < 1) return E_BAD_ARGUMENT;
    TcConv a = {};
    a.dy = dy; a.pre = const_cast<float *>(pre); a.out = dx;
    a.B = B; a.C = C; a.O = O; a.H = H; a.W = W;
    int rc = ct_err_word(&a.err);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int NP = C <= 32 ? 32 : 64;
    const long Kp = (9L * O + CT_K - 1) / CT_K * CT_K;
    if ((rc = ct_pack(w, C, O, CT_DATA, NP, Kp, st, &a.w))) return rc;
    dim3 grid((unsigned)(((long)H * W + CT_M - 1) / CT_M), (unsigned)B);
    return NP == 32 ? launch_ct<CT_DATA, 32>(a, grid, st) : launch_ct<CT_DATA, 64>(a, grid, st);
}

// Slabs of the weight gradient for a batch of B (H x W) inputs.
long conv_tc_wgt_slabs(int B, int H, int W, int *kslab, int *per_img) {
    const long opl = (long)(H - 2) * (W - 2);
    const int ks = 1024;
    const int spi = (int)((opl + ks - 1) / ks);
    if (kslab) *kslab = ks;
    if (per_img) *per_img = spi;
    return (long)B * spi;
}

// part[slab][O C 9 + O]: the weight and bias gradients of each slab.
int conv_tc_weight_grad(const float *x, long xbs, const int *idx, const float *dy, int B, int C, int O, int H, int W,
                        float *part, void *stream) {
    if (O < 1 || O > 64 || C < 1 || H < 3 || W < 3 || B < 1) return E_BAD_ARGUMENT;
    TcConv a = {};
    a.x = x; a.xbs = xbs; a.idx = idx; a.dy = dy; a.out = part;
    a.B = B; a.C = C; a.O = O; a.H = H; a.W = W;
    int rc = ct_err_word(&a.err);
    if (rc) return rc;
    const long nslab = conv_tc_wgt_slabs(B, H, W, &a.kslab, &a.slabs_per_img);
    dim3 grid((unsigned)nslab, (unsigned)((9L * C + CT_M - 1) / CT_M));
    cudaStream_t st = (cudaStream_t)stream;
    return O <= 32 ? launch_ct<CT_WGT, 32>(a, grid, st) : launch_ct<CT_WGT, 64>(a, grid, st);
}

// The error word of the bounded waits (0: none expired); reading clears it.
int conv_tc_error(void *stream) {
    if (!g_ct_err) return 0;
    int h = 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(&h, g_ct_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (h) cudaMemsetAsync(g_ct_err, 0, sizeof(int), st);
    return h;
}

}  // namespace cfdwm
