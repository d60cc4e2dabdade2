// The exported C ABI (include/cfdwavemaker_gb300.h).
//
// Global model: like the reference's singletons (CFDwavemaker.cpp:129-163)
// the library keeps one loaded wave model per process: the parsed input, the
// device-resident irregular sea tables, the s-grid ring or the regular-wave
// solution.  Every query goes through one device pipeline; the scalar
// wave_* functions are batches of one point.
//
// Dispatch, clamping and ramps follow CFDwavemaker.cpp:1543-2009: z is
// clamped to the seabed for the velocity/pressure queries, every output is
// multiplied by Ramp::ramp(t, x, y), the non-hydrostatic pressure of the
// irregular sea is ramp * (dp - rho g eta).
#include "cfdwm.h"
#include "ramp.cuh"
#include "../../include/cfdwavemaker_gb300.h"

#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <atomic>

namespace cfdwm {

static std::atomic<long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static void note_launches(long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(); }

// Per-kernel event profiler (single-threaded use: benchmarks and tests).
static bool g_prof = false;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof_ev[PK_COUNT];
static cudaEvent_t g_prof_open[PK_COUNT];
bool prof_on() { return g_prof; }
void prof_begin(int k, void *stream) {
    if (!g_prof) return;
    cudaEventCreate(&g_prof_open[k]);
    cudaEventRecord(g_prof_open[k], (cudaStream_t)stream);
}
void prof_end(int k, void *stream) {
    if (!g_prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, (cudaStream_t)stream);
    g_prof_ev[k].push_back({g_prof_open[k], e});
}

#define CKR(x)                                                 \
    do {                                                       \
        cudaError_t e_ = (x);                                  \
        if (e_ != cudaSuccess) {                               \
            set_error(std::string("CUDA: ") + cudaGetErrorString(e_)); \
            return E_CUDA;                                     \
        }                                                      \
    } while (0)

namespace {

struct Model {
    bool init = false;
    int device = -1;          // the device current at initialisation: tables live there
    Config cfg;
    DevSea sea;
    DevGrid grid;
    DevRegular reg;
    Workspace grid_ws;
};
Model g_model;
std::mutex g_model_mtx;
// changes whenever the model is freed or rebuilt (scalar-call graphs compare it)
std::atomic<long> g_model_gen{0};
// status word of the last regular-wave set-up (cfdwm_regular_status)
int g_last_reg_status = -1;

}  // namespace
int noalloc_prepare();     // noalloc.cu
namespace {

// Ring updates through the learned update (cfdwm_surrogate_enable): every
// plain_every-th update is plain, the others are predicted and checked.
struct SurrUse {
    bool on = false;
    int plain_every = 20;
    double tol = 1e-3;
    int nsample = 64;
    long count = 0;
};
SurrUse g_surr_use;

// A scalar call's pipeline captured as a CUDA graph (one per thread and
// quantity): the point is read from and the result written to a small pinned
// buffer in place, so a call is one graph launch and one synchronisation.
struct ScalarGraph {
    cudaGraphExec_t exec = nullptr;
    long gen = -1;                 // model generation at capture
    const void *ws[2] = {nullptr, nullptr};   // workspace bases at capture
    long launches = 0;             // kernels in the graph
    // s-grid: the ring state the query's arguments hold (slots, time, fields, arrays)
    int tstep = -1, nf = 0;
    double t0 = 0.0;
    const void *ring[2] = {nullptr, nullptr};
};

// whether graph g was captured for the current s-grid ring state (always true
// for the other wave types)
bool ring_matches(const ScalarGraph &g) {
    const Model &M = g_model;
    if (M.cfg.wavetype != WT_IRR_SGRID) return true;
    return g.tstep == M.grid.tstep && g.t0 == M.grid.t0 && g.nf == M.grid.nf && g.ring[0] == M.grid.QIMG &&
           g.ring[1] == M.grid.ETA;
}

// Per-thread execution context: stream, workspace and staging buffers.
struct ThreadCtx {
    cudaStream_t own = nullptr;
    cudaStream_t user = nullptr;
    bool user_set = false;
    Workspace ws;
    double *d_in = nullptr;   // staging of x, y, z, t  [4][cap]
    double *d_out = nullptr;  // pipeline outputs       [6][cap]
    double *h_pin = nullptr;  // pinned host staging    [10][cap]
    long cap = 0;
    double kin[4] = {0, 0, 0, 0};
    std::string err;
    Workspace api_ws;         // eval_api's scratch (clamped z, model outputs)
    Workspace qf_stage;       // the precision form's staging of host arrays
    double *h_pt = nullptr;   // pinned [16]: x, y, z, t of a scalar call, then its rows
    ScalarGraph sg[7];        // quantities 0-5 (wave_SurfElev ... wave_nhPres), 6: wave_Kinematics
    bool sg_off = false;      // capture failed once on this thread: launch by launch
    ~ThreadCtx() {
        for (auto &g : sg)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        if (h_pt) cudaFreeHost(h_pt);
        workspace_free(qf_stage);
        workspace_free(api_ws);
        if (d_in) cudaFree(d_in);
        if (d_out) cudaFree(d_out);
        if (h_pin) cudaFreeHost(h_pin);
        workspace_free(ws);
        if (own) cudaStreamDestroy(own);
    }
};
thread_local ThreadCtx t_ctx;

void set_error(const std::string &s) { t_ctx.err = s; }

cudaStream_t stream_of() {
    if (t_ctx.user_set) return t_ctx.user;
    if (!t_ctx.own) cudaStreamCreateWithFlags(&t_ctx.own, cudaStreamNonBlocking);
    return t_ctx.own;
}

int ensure_cap(long n) {
    if (t_ctx.cap >= n) return OK;
    long cap = std::max<long>(n, 1024);
    if (t_ctx.d_in) cudaFree(t_ctx.d_in);
    if (t_ctx.d_out) cudaFree(t_ctx.d_out);
    if (t_ctx.h_pin) cudaFreeHost(t_ctx.h_pin);
    t_ctx.d_in = t_ctx.d_out = t_ctx.h_pin = nullptr;
    t_ctx.cap = 0;
    CKR(cudaMalloc(&t_ctx.d_in, sizeof(double) * 4 * cap));
    CKR(cudaMalloc(&t_ctx.d_out, sizeof(double) * 6 * cap));
    CKR(cudaMallocHost(&t_ctx.h_pin, sizeof(double) * 10 * cap));
    t_ctx.cap = cap;
    return OK;
}

bool is_device(const void *p) {
    if (!p) return true;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Whether kernels may read and write the caller's pageable host arrays
// directly: the device accesses pageable memory through the host's page
// tables (Grace-Blackwell address translation over the coherent chip-to-chip
// link).  Queried once; CFDWM_HOST_STAGING=1 keeps the staged copies.
bool direct_host_access() {
    static const bool supported = [] {
        int dev = 0, a = 0, b = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return false;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
        if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
            return false;
        return a != 0 && b != 0;
    }();
    const char *e = std::getenv("CFDWM_HOST_STAGING");
    return supported && !(e && e[0] == '1');
}

// ---------------------------------------------------------------------------
// small kernels of the API layer
// ---------------------------------------------------------------------------
__global__ void k_copy_row(long n, const double *src, double *dst) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p < n) dst[p] = src[p];
}
__global__ void k_clamp_z(long n, const double *z, double depth, double *zc) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p < n) zc[p] = fmax(-depth, z[p]);
}

// Irregular wave types 1 and 5 finish here: out rows
// 0 SurfElev, 1 VeloX, 2 VeloY, 3 VeloZ, 4 DynPres, 5 nhPres.  sgp: the
// s-grid holds the dynamic pressure (row 4 of its query).
// The API rows of the model outputs: out[6][n] (eta, u, v, w, dp, nhpres;
// or null) and/or the wave_Kinematics records kin[n][4] (eta, u, v, w; or
// null), written in one pass.  Without a ramp the factor is not applied: FP64
// multiplies run at a small fraction of the FP32 rate on this GPU.
__global__ void k_finish(long n, int wavetype, int sgp, RampDev r, double rho, double g, const double *x,
                         const double *y, const double *t, const double *f, const double *fe,
                         double *out, double *kin) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const bool ramped = r.init;
    const double rr = ramped ? d_ramp(r, t[p], x[p], y[p]) : 1.0;
    double v[6];
    if (wavetype == WT_IRREGULAR) {
        // f = [5][n] eta, u, v, w, dp of Irregular::*
        for (int q = 0; q < 5; q++) v[q] = f[q * n + p];
        v[5] = f[4 * n + p] - rho * g * f[0 * n + p];
    } else {
        // WT_IRR_SGRID (regular waves write their rows in their own kernel)
        // f = [4][n] query at the clamped z (sgp: [5][n] with the pressure),
        // fe = [4][n] query at z = 0.  Without a pressure field the
        // reference's 0.0 (CFDwavemaker.cpp:1808-1812, 1815-1891); with one,
        // the irregular sea's forms (:1807-1808, 1826-1830) on the grid.
        v[0] = fe[0 * n + p];
        v[1] = f[1 * n + p];
        v[2] = f[2 * n + p];
        v[3] = f[3 * n + p];
        v[4] = sgp ? f[4 * n + p] : 0.0;
        v[5] = sgp ? f[4 * n + p] - rho * g * f[0 * n + p] : 0.0;
    }
    if (ramped)
        for (int q = 0; q < 6; q++) v[q] *= rr;
    if (out)
        for (int q = 0; q < 6; q++) out[q * n + p] = v[q];
    if (kin)
        for (int q = 0; q < 4; q++) kin[4 * p + q] = v[q];
}

// wave_VFrac (CFDwavemaker.cpp:1990-2009) from the ramped elevation.
__global__ void k_vfrac(long n, const double *z, const double *eta, double dcell, double *out) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double w = eta[p], zp = z[p];
    double v;
    if (w < zp - (dcell / 2.)) v = 0.0;
    else if (w > zp + (dcell / 2.)) v = 1.0;
    else v = (w - (zp - (dcell / 2.))) / dcell;
    out[p] = v;
}

// [4][n] rows -> [n][4] records (wave_Kinematics layout)
__global__ void k_interleave4(long n, const double *rows, double *rec) {
    long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    for (int q = 0; q < 4; q++) rec[4 * p + q] = rows[(long)q * n + p];
}

RampDev ramp_dev(const RampCfg &r) {
    RampDev d;
    d.init = r.init ? 1 : 0;
    d.flags = r.flags;
    for (int q = 0; q < 12; q++) d.lim[q] = r.lim[q];
    return d;
}

// The device pipeline: out[6][n] of the reference's wave_* functions for
// the points (x, y, z, t), all device pointers.  want: bit q = output q.
int eval_api(long n, const double *x, const double *y, const double *z, const double *t, int want,
             double *out, cudaStream_t s, double *kin = nullptr) {
    Model &M = g_model;
    if (!M.init) return E_NOT_INITIALIZED;
    if (n <= 0) return OK;
    int wt = M.cfg.wavetype;
    RampDev rd = ramp_dev(M.cfg.ramp);
    // regular waves: one kernel clamps z, evaluates, applies the ramp and
    // writes the rows and records
    if (wt == WT_REGULAR) return regular_eval(M.reg, M.cfg, n, x, y, z, t, rd, out, kin, s);
    Workspace &ws = t_ctx.ws;
    int mask = 0;
    if (wt == WT_IRREGULAR) {
        if (want & (1 | 32)) mask |= 1;
        if (want & 2) mask |= 2;
        if (want & 4) mask |= 4;
        if (want & 8) mask |= 8;
        if (want & (16 | 32)) mask |= 16;
        // irregular waves: the seabed clamp in the height pass and the API
        // rows written by the combining pass (no clamp or finishing pass),
        // except where the Smit theory's kernels write the velocity rows
        if ((out || kin) && !(M.sea.smit && (mask & 30))) {
            const ApiRows ar{rd, M.cfg.rho, M.cfg.gravity, x, y, t, out, kin};
            return irregular_eval(M.sea, n, x, y, z, t, mask, nullptr, ws, s, &ar);
        }
    }
    // scratch: clamped z [n], model outputs [5][n] and [4][n]
    size_t need = sizeof(double) * (size_t)n * 10;
    // irregular_eval uses the same thread workspace; keep a separate buffer
    Workspace &api_ws = t_ctx.api_ws;
    int rc = workspace_reserve(api_ws, need);
    if (rc) return rc;
    double *zc = (double *)api_ws.base, *f = zc + n, *fe = f + 5 * n;
    k_clamp_z<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, z, M.cfg.depth, zc);
    note_launch();
    CKR(cudaGetLastError());
    if (wt == WT_IRREGULAR) {
        CKR(cudaMemsetAsync(f, 0, sizeof(double) * 5 * n, s));
        rc = irregular_eval(M.sea, n, x, y, zc, t, mask, f, ws, s);
        if (rc) return rc;
    } else if (wt == WT_IRR_SGRID) {
        // get_kinematics_at_point forms eta before it looks at z
        // (lsgrid_spline.cpp:505-571), so one query serves wave_SurfElev
        // (queried at z = 0) and the velocities (queried at the clamped z)
        rc = grid_query(M.grid, n, x, y, zc, t, f, s);
        if (rc) return rc;
        fe = f;
    } else {
        return E_UNSUPPORTED;
    }
    const int sgp = (wt == WT_IRR_SGRID && M.grid.nf == 4) ? 1 : 0;
    k_finish<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, wt, sgp, rd, M.cfg.rho, M.cfg.gravity, x, y, t,
                                                         f, fe, out, kin);
    note_launch();
    CKR(cudaGetLastError());
    return OK;
}

// Copies n doubles between pageable and pinned host memory on up to 16 host
// threads (a single core moves about 10 GB/s; the copies were most of the
// host-buffer calls' time beside the GPU work).
static void host_copy(double *dst, const double *src, long n) {
    const long per = 1L << 18;                       // 2 MB a thread at least
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const long nt = std::min<long>(std::min<long>(hw, 16), std::max<long>(1, n / per));
    if (nt <= 1) {
        std::memcpy(dst, src, sizeof(double) * n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (long k = 1; k < nt; k++) {
        const long lo = n * k / nt, hi = n * (k + 1) / nt;
        th.emplace_back([=] { std::memcpy(dst + lo, src + lo, sizeof(double) * (hi - lo)); });
    }
    std::memcpy(dst, src, sizeof(double) * (n / nt));
    for (auto &t : th) t.join();
}

// Runs eval_api on user arrays, staging host memory as needed.  outs[q]
// receives row q of the pipeline output (NULL: not wanted).  For VFrac the
// caller post-processes row 0.
int run_batch(const double *x, const double *y, const double *z, const double *t, long n,
              double *const outs[6], int want, double vf_dcell, double *vf_out,
              double *kin_out = nullptr) {
    if (!g_model.init) return E_NOT_INITIALIZED;
    if (n < 0) return E_BAD_ARGUMENT;
    if (n == 0) return OK;
    if (!x || !y || !t || (!z && (want & ~1))) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    bool dev = is_device(x) && is_device(y) && is_device(t) && (!z || is_device(z));
    for (int q = 0; q < 6; q++) if (outs[q] && !is_device(outs[q])) dev = false;
    if (vf_out && !is_device(vf_out)) dev = false;
    if (kin_out && !is_device(kin_out)) dev = false;
    // host arrays that the kernels can address directly: no staging, the
    // outputs written by a copy kernel, and the call completes before it
    // returns.  Up to 4M points: for a point batch (65,536) e2e went from
    // 2.17e7 to 2.62e7 points/s and for 1e6 s-grid queries from 6.87e7 to
    // 7.22e7 nodes/s; 1e7 points (640 MB) moved faster staged (4.05e8 against
    // 3.73e8 points/s).
    const bool direct = !dev && n <= (1L << 22) && direct_host_access();
    if (dev || direct) {
        double *out = nullptr;
        Workspace &ws = t_ctx.ws;
        (void)ws;
        static thread_local Workspace dev_out;
        int rc = workspace_reserve(dev_out, sizeof(double) * 6 * (size_t)n);
        if (rc) return rc;
        out = (double *)dev_out.base;
        const double *zz = z ? z : t;   // z unused for SurfElev only
        bool rows = vf_out != nullptr;
        for (int q = 0; q < 6; q++) rows = rows || outs[q] != nullptr;
        // the Kinematics records come straight from the finishing pass
        rc = eval_api(n, x, y, zz, t, want, rows ? out : nullptr, s, kin_out);
        if (rc) return rc;
        for (int q = 0; q < 6; q++) {
            if (!outs[q]) continue;
            if (direct) {
                k_copy_row<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, out + (long)q * n, outs[q]);
                note_launch();
                CKR(cudaGetLastError());
            } else {
                CKR(cudaMemcpyAsync(outs[q], out + (long)q * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            }
        }
        if (vf_out) {
            k_vfrac<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, z, out, vf_dcell, vf_out);
            note_launch();
            CKR(cudaGetLastError());
        }
        if (!t_ctx.user_set || direct) CKR(cudaStreamSynchronize(s));
        return OK;
    }
    // host path: stage in chunks through pinned buffers
    const long chunk = 1L << 20;
    int rc = ensure_cap(std::min(n, chunk));
    if (rc) return rc;
    for (long b = 0; b < n; b += chunk) {
        long m = std::min(chunk, n - b);
        double *hp = t_ctx.h_pin, *din = t_ctx.d_in, *dout = t_ctx.d_out;
        const double *src[4] = {x, y, z ? z : t, t};
        for (int q = 0; q < 4; q++) {
            if (is_device(src[q])) {
                CKR(cudaMemcpyAsync(din + (long)q * m, src[q] + b, sizeof(double) * m,
                                    cudaMemcpyDeviceToDevice, s));
            } else {
                host_copy(hp + (long)q * m, src[q] + b, m);
                CKR(cudaMemcpyAsync(din + (long)q * m, hp + (long)q * m, sizeof(double) * m,
                                    cudaMemcpyHostToDevice, s));
            }
        }
        rc = eval_api(m, din, din + m, din + 2 * m, din + 3 * m, want, dout, s);
        if (rc) return rc;
        if (vf_out) {
            k_vfrac<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, din + 2 * m, dout, vf_dcell, dout + 5 * m);
            note_launch();
            CKR(cudaGetLastError());
        }
        // only the rows asked for come back: row q of dout to hp + (4 + q) m;
        // the Kinematics records are interleaved on the device (into din,
        // whose inputs are consumed) and come back as one block
        for (int q = 0; q < 6; q++)
            if (outs[q])
                CKR(cudaMemcpyAsync(hp + (4 + q) * m, dout + (long)q * m, sizeof(double) * m,
                                    cudaMemcpyDeviceToHost, s));
        if (vf_out)
            CKR(cudaMemcpyAsync(hp + 9 * m, dout + 5 * m, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
        if (kin_out) {
            k_interleave4<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, dout, din);
            note_launch();
            CKR(cudaGetLastError());
            CKR(cudaMemcpyAsync(hp, din, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost, s));
        }
        CKR(cudaStreamSynchronize(s));
        for (int q = 0; q < 6; q++)
            if (outs[q]) host_copy(outs[q] + b, hp + (4 + q) * m, m);
        if (vf_out) host_copy(vf_out + b, hp + 9 * m, m);
        if (kin_out) host_copy(kin_out + 4 * b, hp, 4 * m);
    }
    return OK;
}

void free_model() {
    Model &M = g_model;
    g_model_gen.fetch_add(1);
    qform_free();
    sea_free(M.sea);
    grid_free(M.grid);
    regular_free(M.reg);
    workspace_free(M.grid_ws);
    M.cfg = Config();
    M.init = false;
}

int initialize_from_text(const std::string &text) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    free_model();
    Model &M = g_model;
    Config cfg;
    int rc = parse_waveinput_text(text, cfg);
    if (rc) {
        set_error("waveinput.dat: " + cfg.error);
        std::fprintf(stderr, "cfdwavemaker_gb300: INPUTFILE ERROR: %s\n", cfg.error.c_str());
        return rc;
    }
    int wt = cfg.wavetype;
    if (wt != WT_IRREGULAR && wt != WT_IRR_SGRID && wt != WT_REGULAR) {
        set_error("wave type not served by this build (piston, swd, vtk and slope are not)");
        std::fprintf(stderr, "cfdwavemaker_gb300: %s\n", t_ctx.err.c_str());
        return E_UNSUPPORTED;
    }
    // vertical_theory smit changes only Irregular::u/v/w/dp (Irregular.cpp:25, 53, 77,
    // 143): the point API of wave type 1.  The s-grid update calls u1/uvw2 directly
    // (lsgrid_spline.cpp:880-903), so wave type 5 is the same with either theory.
    if (wt == WT_IRREGULAR && cfg.vertical_theory == 1 && cfg.order != 2) {
        set_error("vertical_theory smit is served with second order (kinematics_surf_extrap 2) only");
        std::fprintf(stderr, "cfdwavemaker_gb300: %s\n", t_ctx.err.c_str());
        return E_UNSUPPORTED;
    }
    cudaStream_t s = stream_of();
    M.cfg = cfg;
    if (cudaGetDevice(&M.device) != cudaSuccess) M.device = -1;
    if (wt == WT_IRREGULAR || wt == WT_IRR_SGRID) {
        dump_spectral_components(cfg);
        rc = sea_build(cfg, M.sea, wt == WT_IRREGULAR, s);
        if (rc) { free_model(); return rc; }
        // the fixed workspace of the allocation-free entry point is committed
        // here, while the caller may still allocate (its module loads lazily)
        noalloc_prepare();
        if (wt == WT_IRR_SGRID) {
            rc = grid_create(cfg, M.grid, s);
            // column sums: the depth-separable tensor-core form unless
            // CFDWM_SGRID_METHOD=0 asks for the plain form (or the depth basis
            // cannot be built for this sea, in which case the plain form is kept)
            const char *env = std::getenv("CFDWM_SGRID_METHOD");
            int method = (env && env[0] == '0') ? 0 : 1;
            if (!rc && method == 1 && grid_set_method(M.grid, cfg, M.sea, 1, s) != OK) {
                cudaGetLastError();
                grid_set_method(M.grid, cfg, M.sea, 0, s);
            }
            if (!rc) rc = grid_initialize(M.grid, M.sea, M.grid_ws, s);
            if (rc) { free_model(); return rc; }
            // [lsgrid2vtk]: the initial ring (lsgrid_spline.cpp:746-748, 837-839)
            if (cfg.lsgrid.dump_vtk && grid_dump_vtu(M.grid, false, s) != OK)
                std::fprintf(stderr, "cfdwavemaker_gb300: could not write the .vtu file\n");
        }
    } else {
        rc = regular_build(cfg, M.reg, s);
        g_last_reg_status = (rc == OK || rc == E_SOLVER) ? M.reg.status : -1;
        if (rc) {
            if (rc == E_SOLVER && M.reg.status == 2)
                set_error("FentonStream: singular Jacobian in the Newton solve");
            else if (rc == E_SOLVER)
                set_error("FentonStream: the Newton iteration left the finite numbers (no solution for this "
                          "wave height)");
            else
                set_error("regular-wave setup failed");
            free_model();
            return rc;
        }
        if (M.reg.status == 3)
            std::fprintf(stderr, "FentonStream: warning - Newton iteration did not fully converge.\n");
    }
    M.init = true;
    g_model_gen.fetch_add(1);
    return OK;
}

// The one-point pipeline of quantity q on the thread's pinned point buffer:
// eval_api reads x, y, z, t from its first four elements and writes the six
// API rows of the point (one value each) into the next six, where row q is
// read back (q = 6: the eta, u, v, w record of wave_Kinematics there).
int scalar_pipeline(int q, cudaStream_t s) {
    double *in = t_ctx.h_pt;
    if (q == 6) return eval_api(1, in, in + 1, in + 2, in + 3, 15, nullptr, s, in + 4);
    return eval_api(1, in, in + 1, in + 2, in + 3, 1 << q, in + 4, s);
}

// Scalar calls replay a graph of scalar_pipeline.  The graph is captured
// after one plain run of the pipeline (which reserves the workspaces) and
// captured again when the model was rebuilt, a workspace has moved, or (wave
// type 5) the ring has moved on: its query takes the ring's slots and time as
// arguments, so a graph serves the calls between two ring updates.
int scalar_graph(int q, double x, double y, double z, double t, double *v) {
    const int nv = q == 6 ? 4 : 1;          // values of the result
    const int r0 = q == 6 ? 4 : 4 + q;      // where they are in the pinned buffer
    ThreadCtx &c = t_ctx;
    if (!c.h_pt) CKR(cudaMallocHost(&c.h_pt, sizeof(double) * 16));
    cudaStream_t s = stream_of();
    ScalarGraph &g = c.sg[q];
    const long gen = g_model_gen.load();
    double *in = c.h_pt;
    in[0] = x; in[1] = y; in[2] = z; in[3] = t;
    if (g.exec && g.gen == gen && g.ws[0] == c.ws.base && g.ws[1] == c.api_ws.base && ring_matches(g)) {
        CKR(cudaGraphLaunch(g.exec, s));
        CKR(cudaStreamSynchronize(s));
        note_launches(g.launches);
        for (int k = 0; k < nv; k++) v[k] = in[r0 + k];
        return OK;
    }
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    // the plain run: its result is this call's, and it reserves the workspaces
    int rc = scalar_pipeline(q, s);
    if (rc) return rc;
    CKR(cudaStreamSynchronize(s));
    for (int k = 0; k < nv; k++) v[k] = in[r0 + k];
    cudaGraph_t graph = nullptr;
    bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        const int prc = scalar_pipeline(q, s);
        ok = cudaStreamEndCapture(s, &graph) == cudaSuccess && prc == OK && graph;
    }
    // the kernels of the graph: counted by the launch counter at capture,
    // though not launched then, and at every replay
    long captured = 0;
    if (ok) {
        size_t nn = 0;
        ok = cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess;
        std::vector<cudaGraphNode_t> nodes(nn);
        if (ok && nn) ok = cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess;
        for (size_t k = 0; ok && k < nn; k++) {
            cudaGraphNodeType ty;
            if (cudaGraphNodeGetType(nodes[k], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) captured++;
        }
        note_launches(-captured);
    }
    if (ok) ok = cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
        cudaGetLastError();
        g.exec = nullptr;
        c.sg_off = true;
        return OK;
    }
    g.gen = gen;
    g.ws[0] = c.ws.base; g.ws[1] = c.api_ws.base;
    g.launches = captured;
    g.tstep = g_model.grid.tstep; g.t0 = g_model.grid.t0; g.nf = g_model.grid.nf;
    g.ring[0] = g_model.grid.QIMG; g.ring[1] = g_model.grid.ETA;
    return OK;
}

double scalar(int q, double x, double y, double z, double t) {
    if (!g_model.init) return 0.0;
    if (!t_ctx.user_set && !prof_on() && !t_ctx.sg_off) {
        double v = 0.0;
        return scalar_graph(q, x, y, z, t, &v) == OK ? v : 0.0;
    }
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double v = 0.0;
    outs[q] = &v;
    int rc = run_batch(&x, &y, &z, &t, 1, outs, 1 << q, 0.0, nullptr);
    return rc ? 0.0 : v;
}

}  // namespace

// Accessors for entry points defined in other translation units.
const DevSea *api_loaded_sea(int *wavetype) {
    if (wavetype) *wavetype = g_model.init ? g_model.cfg.wavetype : 0;
    return g_model.init ? &g_model.sea : nullptr;
}
int api_model_device() { return g_model.init ? g_model.device : -1; }
void api_set_error(const char *msg) { set_error(msg); }
void *api_user_stream() { return t_ctx.user_set ? (void *)t_ctx.user : nullptr; }

}  // namespace cfdwm

using namespace cfdwm;

extern "C" {

int CFDwavemaker_is_initialized(void) { return g_model.init ? 1 : 0; }

int wave_Initialize(void) {
    std::string text, where;
    if (read_waveinput_file(text, where) != OK) {
        std::fprintf(stderr, "Could not open file (is it really there?) \n");
        set_error("waveinput.dat not found");
        return -1;
    }
    return initialize_from_text(text);
}

int cfdwm_initialize_text(const char *text) {
    if (!text) return E_BAD_ARGUMENT;
    return initialize_from_text(std::string(text));
}

int wave_Cleanup(void) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    // the reference's grid writes the slot after the base slot when it is
    // destroyed (lsgrid_spline.h:25-28)
    Model &M = g_model;
    if (M.init && M.cfg.wavetype == WT_IRR_SGRID && M.cfg.lsgrid.dump_vtk)
        grid_dump_vtu(M.grid, true, stream_of());
    free_model();
    return 0;
}

double wave_VeloX(double x, double y, double z, double t) { return scalar(1, x, y, z, t); }
double wave_VeloY(double x, double y, double z, double t) { return scalar(2, x, y, z, t); }
double wave_VeloZ(double x, double y, double z, double t) { return scalar(3, x, y, z, t); }
double wave_DynPres(double x, double y, double z, double t) { return scalar(4, x, y, z, t); }
double wave_nhPres(double x, double y, double z, double t) { return scalar(5, x, y, z, t); }
double wave_SurfElev(double x, double y, double t) { return scalar(0, x, y, 0.0, t); }

double wave_VFrac(double x, double y, double z, double t, double dcell) {
    double eta = wave_SurfElev(x, y, t);
    if (eta < z - (dcell / 2.)) return 0.0;
    if (eta > z + (dcell / 2.)) return 1.0;
    return (eta - (z - (dcell / 2.))) / dcell;
}

double wave_Seabed(double x, double y) {
    (void)x; (void)y;
    return -g_model.cfg.depth;
}

double *wave_Kinematics(double x, double y, double z, double t) {
    double *k = t_ctx.kin;
    k[0] = k[1] = k[2] = k[3] = 0.0;
    int wt = g_model.cfg.wavetype;
    if (!g_model.init || (wt != WT_IRR_SGRID && wt != WT_IRREGULAR)) return k;
    if (!t_ctx.user_set && !prof_on() && !t_ctx.sg_off) {
        double v[4];
        if (scalar_graph(6, x, y, z, t, v) == OK)
            for (int q = 0; q < 4; q++) k[q] = v[q];
        return k;
    }
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    run_batch(&x, &y, &z, &t, 1, outs, 15, 0.0, nullptr, k);
    return k;
}

double wave_piston_position(double t) {
    (void)t;
    return 0.;
}

void wave_force_update(double t) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!M.init || M.cfg.wavetype != WT_IRR_SGRID) return;
    cudaStream_t s = stream_of();
    while (grid_check_time(M.grid, t)) {
        if (g_surr_use.on && surrogate_levels() == M.grid.nl && M.grid.nf == 3) {
            int mode = (g_surr_use.count++ % g_surr_use.plain_every == 0) ? 0 : 1;
            if (surrogate_step(M.cfg, M.sea, M.grid, M.grid_ws, mode, g_surr_use.tol, g_surr_use.nsample,
                               nullptr, nullptr, s) != OK)
                break;
        } else if (grid_update(M.grid, M.sea, M.grid_ws, s) != OK) {
            break;
        }
        // [lsgrid2vtk]: every updated ring (lsgrid_spline.cpp:924-926)
        if (M.cfg.lsgrid.dump_vtk) grid_dump_vtu(M.grid, false, s);
    }
    cudaStreamSynchronize(s);
}

void wave_set_mpi_comm(int fortran_comm) { (void)fortran_comm; }
void update_probes(double t) { (void)t; }

double wave_phase_speed(int opt) {
    return g_model.cfg.wavetype == WT_IRREGULAR ? phase_speed(g_model.cfg, opt) : 0.;
}
double wave_mean_length(int opt) {
    if (g_model.cfg.wavetype == WT_IRREGULAR) return mean_wave_length(g_model.cfg, opt);
    if (g_model.cfg.wavetype == WT_REGULAR)
        return g_model.cfg.regular_theory == 1 ? g_model.reg.wave_length : g_model.cfg.wave_length;
    return 0.;
}
double wave_mean_period(int opt) {
    if (g_model.cfg.wavetype == WT_IRREGULAR) return mean_wave_period(g_model.cfg, opt);
    if (g_model.cfg.wavetype == WT_REGULAR)
        return g_model.cfg.regular_theory == 1 ? g_model.reg.wave_period : g_model.cfg.wave_period;
    return 0.;
}
double wave_water_depth(void) { return g_model.cfg.depth; }

double VelocityX(int, int, int, double x, double y, double z, double t) { return wave_VeloX(x, y, z, t); }
double VelocityY(int, int, int, double x, double y, double z, double t) { return wave_VeloY(x, y, z, t); }
double VelocityZ(int, int, int, double x, double y, double z, double t) { return wave_VeloZ(x, y, z, t); }
double DynamicPressure(int, int, int, double x, double y, double z, double t) { return wave_DynPres(x, y, z, t); }
double SurfaceElevation(int, int, double x, double y, double t) { return wave_SurfElev(x, y, t); }
double VolumeFraction(double x, double y, double z, double t, double d) { return wave_VFrac(x, y, z, t, d); }
int Init(void *) { return wave_Initialize(); }
int Prepare(double, int) { return 0; }
int Cleanup(void) { return wave_Cleanup(); }

int wave_SurfElev_batch(const double *x, const double *y, const double *t, long n, double *eta) {
    double *outs[6] = {eta, nullptr, nullptr, nullptr, nullptr, nullptr};
    return run_batch(x, y, nullptr, t, n, outs, 1, 0.0, nullptr);
}
int wave_VeloXYZ_batch(const double *x, const double *y, const double *z, const double *t, long n,
                       double *u, double *v, double *w) {
    double *outs[6] = {nullptr, u, v, w, nullptr, nullptr};
    int want = (u ? 2 : 0) | (v ? 4 : 0) | (w ? 8 : 0);
    return run_batch(x, y, z, t, n, outs, want, 0.0, nullptr);
}
int wave_DynPres_batch(const double *x, const double *y, const double *z, const double *t, long n,
                       double *p) {
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, p, nullptr};
    return run_batch(x, y, z, t, n, outs, 16, 0.0, nullptr);
}
int wave_nhPres_batch(const double *x, const double *y, const double *z, const double *t, long n,
                      double *p) {
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, p};
    return run_batch(x, y, z, t, n, outs, 32, 0.0, nullptr);
}
int wave_VFrac_batch(const double *x, const double *y, const double *z, const double *t, double dcell,
                     long n, double *vf) {
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return run_batch(x, y, z, t, n, outs, 1, dcell, vf);
}
int wave_Kinematics_batch(const double *x, const double *y, const double *z, const double *t, long n,
                          double *out) {
    double *outs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (n > 0 && !out) return E_BAD_ARGUMENT;
    return run_batch(x, y, z, t, n, outs, 15, 0.0, nullptr, out);
}

int cfdwm_set_stream(void *cuda_stream) {
    t_ctx.user = (cudaStream_t)cuda_stream;
    t_ctx.user_set = cuda_stream != nullptr;
    return OK;
}

int cfdwm_last_error(char *buf, int len) {
    int n = (int)t_ctx.err.size();
    if (buf && len > 0) {
        std::strncpy(buf, t_ctx.err.c_str(), (size_t)len - 1);
        buf[len - 1] = 0;
    }
    return n;
}

long cfdwm_kernel_launches(void) { return launch_count(); }

int cfdwm_profile_enable(int on) {
    g_prof = on != 0;
    return OK;
}

long cfdwm_profile_read(int kernel, double *total_ms) {
    if (kernel < 0 || kernel >= PK_COUNT) return E_BAD_ARGUMENT;
    double tot = 0.0;
    long n = 0;
    for (auto &pr : g_prof_ev[kernel]) {
        cudaEventSynchronize(pr.second);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) { tot += ms; n++; }
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    g_prof_ev[kernel].clear();
    if (total_ms) *total_ms = tot;
    return n;
}

int cfdwm_wavetype(void) { return g_model.init ? g_model.cfg.wavetype : 0; }

int cfdwm_irregular_fields(const double *x, const double *y, const double *z, const double *t, long n,
                           int mask, double *out) {
    Model &M = g_model;
    if (!M.init) return E_NOT_INITIALIZED;
    if (M.cfg.wavetype != WT_IRREGULAR && M.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    if (n <= 0) return n == 0 ? OK : E_BAD_ARGUMENT;
    if ((mask & 30) && !M.sea.d_tab_point && M.cfg.order == 2) {
        // the s-grid model has no point-API table; build it on demand
        int rc = sea_build(M.cfg, M.sea, true, stream_of());
        if (rc) return rc;
    }
    cudaStream_t s = stream_of();
    double *d = nullptr;
    CKR(cudaMalloc(&d, sizeof(double) * 9 * (size_t)n));
    const double *src[4] = {x, y, z ? z : t, t};
    for (int q = 0; q < 4; q++)
        CKR(cudaMemcpyAsync(d + (long)q * n, src[q], sizeof(double) * n, cudaMemcpyDefault, s));
    CKR(cudaMemsetAsync(d + 4 * n, 0, sizeof(double) * 5 * n, s));
    int rc = irregular_eval(M.sea, n, d, d + n, d + 2 * n, d + 3 * n, mask, d + 4 * n, t_ctx.ws, s);
    if (rc == OK) {
        CKR(cudaMemcpyAsync(out, d + 4 * n, sizeof(double) * 5 * n, cudaMemcpyDefault, s));
        CKR(cudaStreamSynchronize(s));
    }
    cudaFree(d);
    return rc;
}

long cfdwm_npairs(void) { return g_model.init ? g_model.sea.npairs_grid : 0; }

int cfdwm_components(double *dst) {
    const Config &c = g_model.cfg;
    int n = (int)c.omega.size();
    if (!dst) return n;
    const std::vector<double> *src[8] = {&c.omega, &c.A, &c.k, &c.phase, &c.theta, &c.ramptime,
                                         &c.starttime, &c.duration};
    for (int q = 0; q < 8; q++)
        for (int i = 0; i < n; i++) dst[(long)q * n + i] = (*src[q])[i];
    return n;
}

long cfdwm_sgrid_array(int which, double *dst, long cap) {
    if (!g_model.init || g_model.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    return grid_download(g_model.grid, which, dst, cap, stream_of());
}

int cfdwm_sgrid_state(double *t0, int *tstep) {
    if (!g_model.init || g_model.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    if (t0) *t0 = g_model.grid.t0;
    if (tstep) *tstep = g_model.grid.tstep;
    return OK;
}

int cfdwm_qform_build(int fp16) {
    Model &M = g_model;
    if (!M.init) return E_NOT_INITIALIZED;
    if (M.cfg.wavetype != WT_IRREGULAR && M.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    if (M.cfg.order != 2) return E_UNSUPPORTED;
    int rc = qform_build(M.cfg, M.sea, fp16 != 0, stream_of());
    if (rc) set_error("precision-form set-up failed");
    return rc;
}

int cfdwm_qform_eval(const double *x, const double *y, const double *t, long n, int method, float *out) {
    Model &M = g_model;
    if (!M.init) return E_NOT_INITIALIZED;
    if (n <= 0) return n == 0 ? OK : E_BAD_ARGUMENT;
    if (!x || !y || !t || !out) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    int err = 0;
    if (is_device(x) && is_device(y) && is_device(t) && is_device(out)) {
        int rc = qform_eval(M.sea, n, x, y, t, method, out, s, method == 1 ? &err : nullptr);
        if (rc) return rc;
        if (!t_ctx.user_set || method == 1) CKR(cudaStreamSynchronize(s));
    } else {
        // host arrays: staged through a device buffer of the thread in
        // chunks of 2^22 points (x, y, t in, out [m][4] back: 40 bytes a
        // point); any mix of host and device arrays is accepted
        const long chunk = 1L << 22;
        const long cap = std::min(n, chunk);
        int rc = workspace_reserve(t_ctx.qf_stage, (size_t)cap * (3 * sizeof(double) + 4 * sizeof(float)));
        if (rc) return rc;
        double *din = (double *)t_ctx.qf_stage.base;
        float *dout = reinterpret_cast<float *>(din + 3 * cap);
        const double *src[3] = {x, y, t};
        for (long b = 0; b < n; b += chunk) {
            const long m = std::min(chunk, n - b);
            for (int q = 0; q < 3; q++)
                CKR(cudaMemcpyAsync(din + q * cap, src[q] + b, sizeof(double) * m, cudaMemcpyDefault, s));
            int e = 0;
            rc = qform_eval(M.sea, m, din, din + cap, din + 2 * cap, method, dout, s, method == 1 ? &e : nullptr);
            if (rc) return rc;
            err = err ? err : e;
            CKR(cudaMemcpyAsync(out + 4 * b, dout, sizeof(float) * 4 * m, cudaMemcpyDefault, s));
        }
        CKR(cudaStreamSynchronize(s));
    }
    if (err) {
        set_error("tensor-core kernel: a bounded wait expired (code " + std::to_string(err) + ")");
        return E_CUDA;
    }
    return OK;
}

int cfdwm_parse_text(const char *text, double *scalars, double *comps, int cap) {
    if (!text) return E_BAD_ARGUMENT;
    Config c;
    int rc = parse_waveinput_text(std::string(text), c);
    if (rc) {
        set_error(c.error);
        return rc;
    }
    double v[16] = {(double)c.wavetype, (double)c.order, c.depth, c.mtheta, c.swl, c.gravity, c.rho,
                    c.tofmax, c.x_pos, c.y_pos, c.dw_cutoff, c.dw_bandwidth, c.wave_length,
                    c.wave_period, c.wave_height, (double)c.ndir};
    if (scalars) for (int q = 0; q < 16; q++) scalars[q] = v[q];
    int n = (int)c.omega.size();
    if (comps && n <= cap) {
        const std::vector<double> *src[8] = {&c.omega, &c.A, &c.k, &c.phase, &c.theta, &c.ramptime,
                                             &c.starttime, &c.duration};
        for (int q = 0; q < 8; q++)
            for (int i = 0; i < n; i++) comps[(long)q * n + i] = (*src[q])[i];
    }
    return n;
}

int cfdwm_regular_status(void) { return g_last_reg_status; }

// ---- column shard of the s-grid ring ---------------------------------------
int cfdwm_sgrid_partition(int nranks, int *bounds) {
    if (!g_model.init || g_model.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    if (nranks < 1 || !bounds) return E_BAD_ARGUMENT;
    std::vector<long> w;
    grid_row_weights(g_model.grid, w);
    partition_columns(w.data(), g_model.grid.nx, nranks, bounds);
    return OK;
}

int cfdwm_sgrid_due(double t) {
    if (!g_model.init || g_model.cfg.wavetype != WT_IRR_SGRID) return 0;
    return grid_check_time(g_model.grid, t) ? 1 : 0;
}

int cfdwm_sgrid_step_block(int i0, int i1) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!M.init || M.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    return grid_step_block(M.grid, M.sea, M.grid_ws, i0, i1, stream_of());
}

long cfdwm_sgrid_block_count(int field, int i0, int i1) {
    const DevGrid &g = g_model.grid;
    if (!g_model.init || g_model.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    if (i0 < 0 || i1 > g.nx || i0 > i1 || field < 0 || field > g.nf) return E_BAD_ARGUMENT;
    return grid_block_elems(g, field, i0, i1);
}

static int block_copy(int field, int i0, int i1, float *buf, bool into) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!M.init || M.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    cudaStream_t s = stream_of();
    int rc = grid_block_copy(M.grid, field, i0, i1, buf, into, s);
    if (rc) return rc;
    return cudaStreamSynchronize(s) == cudaSuccess ? OK : E_CUDA;
}

int cfdwm_sgrid_block_export(int field, int i0, int i1, float *dst) { return block_copy(field, i0, i1, dst, false); }

int cfdwm_sgrid_block_import(int field, int i0, int i1, const float *src) {
    return block_copy(field, i0, i1, const_cast<float *>(src), true);
}

int cfdwm_sgrid_step_finish(void) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!M.init || M.cfg.wavetype != WT_IRR_SGRID) return E_UNSUPPORTED;
    cudaStream_t s = stream_of();
    int rc = grid_gradients(M.grid, s);
    if (rc) return rc;
    // [lsgrid2vtk]: every updated ring (lsgrid_spline.cpp:924-926)
    if (M.cfg.lsgrid.dump_vtk) grid_dump_vtu(M.grid, false, s);
    return cudaStreamSynchronize(s) == cudaSuccess ? OK : E_CUDA;
}

int cfdwm_regular_solution(double *dst, int cap) {
    if (!g_model.init || g_model.cfg.wavetype != WT_REGULAR) return E_UNSUPPORTED;
    return regular_solution(g_model.reg, dst, cap, stream_of());
}

// ---- learned s-grid update ------------------------------------------------
static bool sgrid_loaded() { return g_model.init && g_model.cfg.wavetype == WT_IRR_SGRID; }

int cfdwm_surrogate_create(int nl, unsigned long long seed) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    int rc = surrogate_create(nl, seed, stream_of());
    if (rc) set_error("surrogate: create failed (levels must be 1..32)");
    return rc;
}

long cfdwm_surrogate_nparams(void) { return surrogate_nparams(); }

int cfdwm_surrogate_get_params(float *dst, long n) { return surrogate_get_params(dst, n, stream_of()); }

int cfdwm_surrogate_set_params(const float *src, long n) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    return surrogate_set_params(src, n, stream_of());
}

static const char SURR_MAGIC[8] = {'C', 'F', 'D', 'W', 'M', 'S', 'R', '1'};

int cfdwm_surrogate_save(const char *path) {
    long n = surrogate_nparams();
    if (n <= 0) return E_NOT_INITIALIZED;
    if (!path) return E_BAD_ARGUMENT;
    std::vector<float> w(n);
    int rc = surrogate_get_params(w.data(), n, stream_of());
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("surrogate: cannot write ") + path);
        return E_NO_FILE;
    }
    int32_t hdr[2] = {surrogate_levels(), 0};
    int64_t nn = n;
    bool ok = std::fwrite(SURR_MAGIC, 1, 8, f) == 8 && std::fwrite(hdr, 4, 2, f) == 2 &&
              std::fwrite(&nn, 8, 1, f) == 1 && std::fwrite(w.data(), 4, n, f) == (size_t)n;
    std::fclose(f);
    return ok ? OK : E_NO_FILE;
}

int cfdwm_surrogate_load(const char *path) {
    if (!path) return E_BAD_ARGUMENT;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("surrogate: cannot read ") + path);
        return E_NO_FILE;
    }
    char mg[8];
    int32_t hdr[2];
    int64_t nn = 0;
    bool ok = std::fread(mg, 1, 8, f) == 8 && std::memcmp(mg, SURR_MAGIC, 8) == 0 &&
              std::fread(hdr, 4, 2, f) == 2 && std::fread(&nn, 8, 1, f) == 1 && nn > 0 && nn < (1L << 28);
    std::vector<float> w(ok ? nn : 0);
    if (ok) ok = std::fread(w.data(), 4, nn, f) == (size_t)nn;
    std::fclose(f);
    if (!ok) {
        set_error(std::string("surrogate: not a weight file: ") + path);
        return E_PARSE;
    }
    std::lock_guard<std::mutex> lk(g_model_mtx);
    int rc = surrogate_levels() == hdr[0] ? OK : surrogate_create(hdr[0], 0, stream_of());
    if (rc) return rc;
    if (surrogate_nparams() != nn) {
        set_error("surrogate: weight file does not match the network shape");
        return E_PARSE;
    }
    return surrogate_set_params(w.data(), (long)nn, stream_of());
}

int cfdwm_surrogate_features(double t, float *feat, float *base, float *eta1) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    if (!is_device(feat) || !is_device(base) || !is_device(eta1)) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    int rc = surrogate_features(M.cfg, M.sea, M.grid, M.grid_ws, t, feat, base, eta1, s);
    if (!rc) CKR(cudaStreamSynchronize(s));
    return rc;
}

int cfdwm_surrogate_targets(int slot, const float *base, const float *eta1, float *tgt) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    if (!tgt || !is_device(tgt) || !is_device(base) || !is_device(eta1)) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    int rc = surrogate_targets(g_model.cfg, g_model.grid, slot, base, eta1, tgt, s);
    if (!rc) CKR(cudaStreamSynchronize(s));
    return rc;
}

int cfdwm_surrogate_forward(const float *x, int B, int H, int W, float *y) {
    if (!x || !y || !is_device(x) || !is_device(y)) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    int rc = surrogate_forward(x, B, H, W, y, s);
    if (!rc) CKR(cudaStreamSynchronize(s));
    if (!rc) rc = surrogate_check(s);
    return rc;
}

int cfdwm_surrogate_loss_grad(const float *x, const float *tgt, int B, int H, int W, double *loss, float *grad) {
    if (!x || !tgt || !is_device(x) || !is_device(tgt) || (grad && !is_device(grad))) return E_BAD_ARGUMENT;
    return surrogate_loss_grad(x, tgt, B, H, W, loss, grad, stream_of());
}

int cfdwm_surrogate_train_step(const float *xs, const float *ts, long nsamples, const int *idx, int B, int H, int W,
                               float lr, double *loss) {
    if (!xs || !ts || !is_device(xs) || !is_device(ts)) return E_BAD_ARGUMENT;
    return surrogate_train_step(xs, ts, nsamples, idx, B, H, W, lr, loss, stream_of());
}

int cfdwm_surrogate_step(int mode, double tol, int nsample, int *fell_back, double *err4) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    cudaStream_t s = stream_of();
    int rc = surrogate_step(M.cfg, M.sea, M.grid, M.grid_ws, mode, tol, nsample, fell_back, err4, s);
    if (rc) set_error("surrogate: ring step failed");
    return rc;
}

int cfdwm_surrogate_compare(double *err4) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    if (!err4) return E_BAD_ARGUMENT;
    return surrogate_compare_newest(M.cfg, M.sea, M.grid, M.grid_ws, err4, stream_of());
}

int cfdwm_surrogate_enable(int on, int plain_every, double tol, int nsample) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    if (on && sgrid_loaded() && g_model.grid.nf != 3) {
        set_error("surrogate: the learned update does not predict the pressure field");
        return E_UNSUPPORTED;
    }
    if (on && (surrogate_nparams() <= 0 || plain_every < 1 || nsample < 0 || nsample > 4096))
        return on && surrogate_nparams() <= 0 ? E_NOT_INITIALIZED : E_BAD_ARGUMENT;
    g_surr_use.on = on != 0;
    g_surr_use.plain_every = plain_every;
    g_surr_use.tol = tol;
    g_surr_use.nsample = nsample;
    g_surr_use.count = 0;
    surrogate_reset_stats();
    return OK;
}

int cfdwm_sgrid_method(int method, int *rank) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    cudaStream_t s = stream_of();
    int rc = grid_set_method(M.grid, M.cfg, M.sea, method, s);
    if (rc) {
        set_error("s-grid: the tensor-core form is not available for this sea (depth basis)");
        return rc;
    }
    // the ring is refilled at the current t0 with the selected method
    rc = grid_initialize(M.grid, M.sea, M.grid_ws, s);
    if (rc) return rc;
    if (rank) *rank = method == 1 ? depthform_rank(M.grid) : 0;
    return OK;
}

int cfdwm_depth_basis(double K, double h, int *rank, double *err) { return depthform_basis_info(K, h, rank, err); }

int cfdwm_spectrum_components(const double *params, int nfreq, int ndir, unsigned long long seed, double *comps) {
    if (!params || !comps || nfreq < 1 || ndir < 1) return E_BAD_ARGUMENT;
    cudaStream_t s = stream_of();
    const size_t bytes = sizeof(double) * 5 * (size_t)nfreq * ndir;
    double *d = nullptr;
    CKR(cudaMalloc(&d, bytes));
    int rc = spectrum_components(params, nfreq, ndir, seed, d, s);
    if (rc == OK) {
        if (cudaMemcpyAsync(comps, d, bytes, cudaMemcpyDefault, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = E_CUDA;
    }
    cudaFree(d);
    if (rc == E_BAD_ARGUMENT) set_error("spectrum: bad parameters");
    return rc;
}

int cfdwm_sgrid_write_vtu(const char *path, int last) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    if (!path) return E_BAD_ARGUMENT;
    const DevGrid &g = g_model.grid;
    int rc = grid_write_vtu(g, path, g.cfg.vtk_timelabel, last != 0, stream_of());
    if (rc) set_error(std::string("s-grid: cannot write ") + path);
    return rc;
}

int cfdwm_sgrid_pressure(int on) {
    std::lock_guard<std::mutex> lk(g_model_mtx);
    Model &M = g_model;
    if (!sgrid_loaded()) return E_UNSUPPORTED;
    if (on && g_surr_use.on) {
        set_error("s-grid: pressure and the learned update exclude each other");
        return E_UNSUPPORTED;
    }
    cudaStream_t s = stream_of();
    int rc = grid_set_pressure(M.grid, M.cfg, M.sea, on != 0, s);
    if (rc) {
        set_error(rc == E_UNSUPPORTED ? "s-grid: pressure needs a second-order sea" : "s-grid: pressure set-up failed");
        return rc;
    }
    // the ring is refilled at the current t0 with (or without) the pressure
    return grid_initialize(M.grid, M.sea, M.grid_ws, s);
}

int cfdwm_surrogate_set_carry(double wavelengths) {
    if (!(wavelengths >= 0.0)) return E_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_model_mtx);
    surrogate_set_carry(wavelengths);
    return OK;
}

int cfdwm_surrogate_stats(long *steps, long *fallbacks, long *plain_steps) {
    surrogate_stats(steps, fallbacks, plain_steps);
    return OK;
}

}  // extern "C"
