// Internal declarations of the GB300 build of CFDwavemaker's point-kinematics
// path: the parsed configuration, the device-resident wave models and the
// host-side launchers of the CUDA kernels.  Nothing here is exported; the
// C ABI lives in include/cfdwavemaker_gb300.h.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cfdwm {

// Wave-type numbering of the reference (CFDwavemaker.cpp:252-258).
enum WaveType {
    WT_NONE = 0,
    WT_IRREGULAR = 1,
    WT_IRR_SGRID = 5,
    WT_PISTON = 11,
    WT_REGULAR = 21,
    WT_SWD = 31,
    WT_SWD_SGRID = 34,
    WT_VTK = 41,
    WT_SLOPE = 51,
};

// Status codes of the batched entry points.
enum Status {
    OK = 0,
    E_NOT_INITIALIZED = -1,
    E_UNSUPPORTED = -2,
    E_BAD_ARGUMENT = -3,
    E_CUDA = -4,
    E_NO_FILE = -5,
    E_PARSE = -6,
    E_SOLVER = -7,
    E_TOO_LARGE = -8,
};

constexpr double SMALL = 1.e-12;   // Irregular.h:8
constexpr double HUGE_ = 1.e12;    // Irregular.h:11
constexpr double PI_IRR = 3.1415926535897;            // Irregular.h:14 (truncated)
constexpr double PI_FULL = 3.14159265358979323846;    // Stokes5.h:5

struct RampCfg {
    bool init = false;
    int flags = 0;        // bit q: time up, time down, x up, x down, y up, y down
    double lim[12] = {0};
};

struct LsgridCfg {
    bool present = false;
    double domain[4] = {0, 0, 0, 0};
    int nx = 5, ny = 0, nl = 4;
    double t0 = 0.0, dt = 0.1, tan_a = 0.0, tan_b = 0.0;
    double domain_ignore[4] = {1.e12, -1.e12, 1.e12, -1.e12};
    bool ignore_domain = false, ignore_at_init = false, init_only = false;
    // [lsgrid2vtk] (defaults of lsgrid_spline.h:58-61)
    bool dump_vtk = false;
    std::string vtk_path = "./", vtk_prefix = "kinematics", vtk_timelabel = "TimeValue";
};

struct Config {
    int wavetype = WT_NONE;
    double depth = 0.0, mtheta = 0.0, swl = 0.0, gravity = 9.81, rho = 1.0, ampl = 1.0;
    bool normalize = false, nhpres_kinetic = false;
    double tofmax = 0.0, x_pos = 0.0, y_pos = 0.0;
    RampCfg ramp;
    int extrapolation_met = 0, order = 2;
    double dw_cutoff = 100000.0, dw_bandwidth = 100.0;
    bool bw_auto = false, individual_ramp = false;
    int vertical_theory = 0;
    int nfreq = 0, ndir = 1;
    bool property_read = false;
    std::vector<double> omega, A, k, phase, theta, ramptime, starttime, duration;
    int regular_theory = 0, wave_order = 16;
    bool regular_specify_length = true;
    double wave_length = 0.0, wave_period = 0.0, wave_height = 0.0, current = 0.0;
    LsgridCfg lsgrid;
    std::string error;
};

// Count of kernel launches issued by the library (process-wide).
void note_launch();
long launch_count();

// Optional per-kernel timing with CUDA events recorded on the launching
// stream around the hot kernels.
enum ProfKernel { PK_COLUMN_PAIRS = 0, PK_ETA_PAIRS, PK_POINT_PAIRS, PK_PHASORS, PK_QUERY,
                  PK_GRADIENTS, PK_QFORM, PK_SURR_FEATURES, PK_SURR_NET, PK_REGULAR, PK_COUNT };
bool prof_on();
void prof_begin(int k, void *stream);
void prof_end(int k, void *stream);

// waveinput.dat reader (parser.cpp).  Returns OK or E_PARSE (cfg.error set).
int parse_waveinput_text(const std::string &text, Config &cfg);
// Search order of wave_Initialize (CFDwavemaker.cpp:2086-2111).
int read_waveinput_file(std::string &text, std::string &where);
// Host-side spectral helpers (Irregular.cpp:1336-1452).
void spectral_moments(const Config &c, double m[3]);
double phase_speed(const Config &c, int opt);
double mean_wave_length(const Config &c, int opt);
double mean_wave_period(const Config &c, int opt);
double wavenumber_from_period(double T, double depth, double g);
double wavelength_from_period(double T, double depth, double g);
double period_from_length(double L, double depth, double g);
void dump_spectral_components(const Config &c);

// ---------------------------------------------------------------------------
// Device-resident irregular sea (irregular.cu)
// ---------------------------------------------------------------------------
// Per-component FP32 coefficient rows (index * npad + component).
enum CompCoef {
    CF_A = 0,     // A                         eta1
    CF_AU,        // A g k / omega             u1, v1, w1
    CF_CT,        // cos(theta + mtheta)
    CF_ST,        // sin(theta + mtheta)
    CF_K,         // k
    CF_Q,         // 1 / (1 + exp(-2 k h))     depth-profile normaliser
    CF_AP,        // A rho g                   dp1
    CF_GX,        // cos(th) A omega k         phi1_dxdz
    CF_GY,        // sin(th) A omega k         phi1_dydz
    CF_GZ,        // A omega k coth(k h)       phi1_dzdz
    CF_GP,        // A rho g k                 dp1_dz
    CF_X1,        // rho * -g^2 (2k ct + 2k st) 2 / (2 omega)   dp2 diagonal, times px
    CF_Z1,        // rho *  g^2 (2k) 2 / (2 omega)              dp2 diagonal, times pz
    CF_KW,        // k / omega (0 for omega <= 0)               Smit theory
    NCF
};

// Pair-table tile geometry: the upper triangle of the N x N component pairs in
// square tiles of TILE x TILE, tile (I, M) with I <= M stored at
// tile_index(I, M), each entry a fixed-size coefficient record.
// Record sizes are defined with the kernels (irregular.cu).
constexpr int GRID_TILE = 32;
constexpr int POINT_TILE = 16;
constexpr int SMIT_TILE = 16;
constexpr int DF_COMP_FLOATS = 14;   // floats of one depthform.cu component record

struct DevSea {
    int n = 0;              // components
    int npad_g = 0;         // components padded to GRID_TILE
    int npad_p = 0;         // components padded to POINT_TILE
    double depth = 0, swl = 0, g = 9.81, rho = 1, fx = 0, fy = 0;
    int order = 2;
    bool trivial_ramp = true;
    long npairs_grid = 0;   // pairs kept by the reference's pair cache
    double kmax = 0;        // largest component wavenumber
    // FP64 phase data, length npad_g: kx, ky, omega, phase0, ramptime, starttime, duration
    double *d_phase = nullptr;   // [7][npad_g]
    float *d_cf = nullptr;       // [NCF][npad_g]
    float *d_tab_eta = nullptr;  // grid-mask pair tiles of eta2 (A, B per pair)
    float *d_tab_grid = nullptr; // grid-mask pair tiles of uvw2
    float *d_tab_point = nullptr;// point-API pair tiles (built on demand)
    float *d_tab_gp = nullptr;   // grid-mask pair tiles of the s-grid pressure: Pp, Mp (phase terms)
    float *d_tab_gk = nullptr;   // grid-mask pair tiles of the phase-free pressure terms: X, Z
    int ntile_g = 0, ntile_p = 0;
    // vertical_theory smit (Smit et al. 2017): its pair tiles (smit.cu)
    bool smit = false;
    float *d_tab_smit = nullptr;
    int npad_s = 0, ntile_s = 0;
    // per-launch component records of the first-order kernels: float-pair
    // phase coefficients, ramp, 5 coefficients; three regions of npad_g
    // records (depthform.cu surface and levels, surrogate.cu features)
    float *d_dfcomp = nullptr;
    // per-component records of the point phasor kernel (irregular.cu):
    // kx, ky, -omega, phase0 as float pairs, then A, GX, GY, GZ, GP
    float *d_phrec = nullptr;
};

// Seeded JONSWAP / cos-2s component columns [5][nfreq ndir] (omega, A, k,
// phase, theta) into device memory (spectrum.cu).  p: hs, tp, gamma, wmin,
// wmax, depth, spreading s, direction span, gravity.
int spectrum_components(const double *p, int nfreq, int ndir, unsigned long long seed, double *out_dev,
                        void *stream);

// FP64 component inputs (device pointers) of the Smit pair-table build.
struct SmitIn {
    int n;
    const double *omega, *A, *k, *theta;
    double depth, g, rho, mtheta_rad, cutoff, bandwidth, kmax;
};
// Builds sea.d_tab_smit (smit.cu).
int smit_build(const SmitIn &c, DevSea &sea, void *stream);
// u, v, w, dp of the Smit theory at n points into rows 1..4 of out (row
// stride ldo), from the point phasors (float2 (cos, sin), [npad_g][n]) and
// ramps, the first-order sums (first[0] = eta1) and eta2; scratch: 4 n floats;
// split_buf (split_cap floats, or null): partial sums when the pair loop is
// split over blocks for few points.
// mask: bits 2, 4, 8 (u, v, w) ask for the velocity sums, 16 (dp) for the
// pressure sum; rows not asked for are 0
int smit_eval(const DevSea &sea, long n, const double *z, const void *ph, const float *rr, const double *first,
              const float *eta2, float *scratch, float *split_buf, long split_cap, long ldo, double *out,
              int mask, void *stream);

// Builds the device tables (component coefficients and the FP64 transfer
// functions of the pair tables, computed on the device).  point_table: also
// build the unfiltered point-API table.
int sea_build(const Config &cfg, DevSea &sea, bool point_table, void *stream);
void sea_free(DevSea &sea);

// Scratch workspace for one batch: phasors and first-order sums.
struct Workspace {
    size_t bytes = 0;
    void *base = nullptr;
};
int workspace_reserve(Workspace &ws, size_t bytes);
void workspace_free(Workspace &ws);

// Evaluate irregular-sea kinematics at n points (device pointers, FP64 in).
// mask bits: 1 eta, 2 u, 4 v, 8 w, 16 dp.  out is [5][n] FP64 (no ramp, no
// clamp): the reference's Irregular::eta/u/v/w/dp.
struct ApiRows;
// api: when given (and the sea is not on the Smit theory), the combining pass
// writes the API rows and records of api instead of out (which may be null).
int irregular_eval(const DevSea &sea, long n, const double *x, const double *y,
                   const double *z, const double *t, int mask, double *out,
                   Workspace &ws, void *stream, const ApiRows *api = nullptr);

// Workspace bytes irregular_eval needs for a batch of n points.
size_t irregular_eval_scratch_bytes(const DevSea &sea, long n);


// ---------------------------------------------------------------------------
// Device-resident s-grid (sgrid.cu)
// ---------------------------------------------------------------------------
struct DevGrid {
    LsgridCfg cfg;
    int nx = 0, ny = 0, nl = 0;
    double dx = 0, dy = 0, ds = 0, t0 = 0, dt = 0, depth = 0, swl = 0;
    int tstep = 0;
    // FP32 fields, layouts of lsgrid_spline.cpp:35-61 ([slot][i][j][m]);
    // field 3 is the dynamic pressure, held only when nf = 4
    int nf = 3;
    float *ETA = nullptr, *ETAdx = nullptr, *ETAdy = nullptr, *ETAdt = nullptr;
    float *U[4] = {nullptr, nullptr, nullptr, nullptr};
    float *Ut[4] = {nullptr, nullptr, nullptr, nullptr};
    float *Ux[4] = {nullptr, nullptr, nullptr, nullptr};
    float *Uy[4] = {nullptr, nullptr, nullptr, nullptr};
    float *Us[4] = {nullptr, nullptr, nullptr, nullptr};
    int *IGNORE = nullptr;
    float *QIMG = nullptr;       // query image of the two slots a query reads ([2][nodes][5][4] floats)
    float *zlev = nullptr;       // scratch: level heights of the slot being written
    double *colpts = nullptr;    // scratch: column x, y, t (FP64)
    double *first = nullptr;     // scratch: eta1, gx, gy, gz per column
    float *second = nullptr;     // scratch: level sums [3][ncol*nl]
    float *eta2 = nullptr;       // scratch: eta2 per column
    int method = 0;              // 0 plain FP32 column sums, 1 depth-separable tensor-core form
};
// Selects the method of the column sums (builds the tensor-core form).
int grid_set_method(DevGrid &g, const Config &cfg, const DevSea &sea, int method, void *stream);
// Dynamic pressure on the ring (nf = 4) or not (nf = 3): allocates or frees
// the pressure fields and rebuilds the tensor-core form for the field count.
// The ring must be refilled afterwards (grid_initialize).
int grid_set_pressure(DevGrid &g, const Config &cfg, const DevSea &sea, bool on, void *stream);
// The error word of the tensor-core form (0: no bounded wait expired).
int grid_tc_error(DevGrid &g, void *stream);
int depthform_rank(DevGrid &g);
int grid_create(const Config &cfg, DevGrid &g, void *stream);
void grid_free(DevGrid &g);
int grid_initialize(DevGrid &g, const DevSea &sea, Workspace &ws, void *stream);
int grid_update(DevGrid &g, const DevSea &sea, Workspace &ws, void *stream);
bool grid_check_time(const DevGrid &g, double t);
// out [1 + nf][n] FP64: eta, u, v, w (and p when nf = 4), no ramp
int grid_query(const DevGrid &g, long n, const double *x, const double *y, const double *z,
               const double *t, double *out, void *stream);
int grid_download(const DevGrid &g, int which, double *dst, long cap, void *stream);
// .vtu export of the ring's base slot (last: the slot after it), as
// lsGridSpline::export_vtu (lsgrid_spline.cpp:1222-1403) writes it, to `path`.
int grid_write_vtu(const DevGrid &g, const std::string &path, const std::string &timelabel, bool last,
                   void *stream);
// The reference's write_vtk (lsgrid_spline.cpp:1200-1219): the file
// <vtk_path><vtk_prefix><tstep %05d>.vtu, creating the directory if needed.
int grid_dump_vtu(const DevGrid &g, bool last, void *stream);
// Plain fill of a column subset into ring slot `slot` of the given arrays
// (the grid's own ETA/U or a scratch copy with the same layout).
int grid_fill_columns(DevGrid &g, const DevSea &sea, Workspace &ws, const int *act, long nact, double t,
                      float *ETA, float *const U[3], int slot, void *stream);
// Plain fill of all live columns of slot `slot` of the grid at time t.
int grid_fill_slot(DevGrid &g, const DevSea &sea, Workspace &ws, int slot, double t, void *stream);
int grid_gradients(DevGrid &g, void *stream);
void grid_live_columns(DevGrid &g, const int **act, long *n);
// Column shard (sgrid.cu): live columns per row i; one ring step that fills
// only the rows [i0, i1) of the new slot (no gradients); copies of a block of
// rows of the newest slot; the host partition (shard.cpp).
void grid_row_weights(const DevGrid &g, std::vector<long> &w);
int grid_step_block(DevGrid &g, const DevSea &sea, Workspace &ws, int i0, int i1, void *stream);
long grid_block_elems(const DevGrid &g, int f, int i0, int i1);
int grid_block_copy(DevGrid &g, int f, int i0, int i1, float *buf, bool into_grid, void *stream);
void partition_columns(const long *w, int n, int nranks, int *bounds);

// ---------------------------------------------------------------------------
// Learned s-grid update (surrogate.cu)
// ---------------------------------------------------------------------------
int surrogate_create(int nl, unsigned long long seed, void *stream);
void surrogate_destroy();
long surrogate_nparams();
int surrogate_levels();
int surrogate_get_params(float *dst, long n, void *stream);
int surrogate_set_params(const float *src, long n, void *stream);
int surrogate_features(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, double t, float *feat,
                       float *base, float *eta1, void *stream);
int surrogate_targets(const Config &cfg, DevGrid &g, int slot, const float *base, const float *eta1, float *tg,
                      void *stream);
int surrogate_forward(const float *x, int B, int H, int W, float *y, void *stream);
// E_CUDA when a bounded wait of the network's tensor-core kernels expired
// since the last check (the stream is synchronised)
int surrogate_check(void *stream);
int surrogate_loss_grad(const float *x, const float *tg, int B, int H, int W, double *loss, float *grad,
                        void *stream);
int surrogate_train_step(const float *xs, const float *ts, long nsamples, const int *idx_host, int B, int H, int W,
                         float lr, double *loss, void *stream);
int surrogate_step(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, int mode, double tol,
                   int nsample, int *fell_back, double *err, void *stream);
int surrogate_compare_newest(const Config &cfg, const DevSea &sea, DevGrid &g, Workspace &ws, double *err,
                             void *stream);
void surrogate_stats(long *steps, long *fallbacks, long *plain_steps);
void surrogate_set_carry(double wavelengths);
void surrogate_reset_stats();

// ---------------------------------------------------------------------------
// Regular waves (regular.cu)
// ---------------------------------------------------------------------------
struct DevRegular {
    int theory = 0;         // 0 Stokes5, 1 Fenton
    int N = 0;
    double *d_sol = nullptr;  // FP64 solution block (coefficients), see regular.cu
    float *d_cf = nullptr;    // its harmonic coefficients in FP32, [4][64] (U, W, E, Q)
    int status = 0;           // Fenton: 0 converged, 3 not fully converged
    // host copies of the scalars
    double k = 0, c = 0, wave_length = 0, wave_period = 0;
    double head[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // solution words 0-9
    double soff[4] = {0, 0, 0, 0};                       // offsets: eta, u, R - g (d - z0), ubar
};
int regular_build(const Config &cfg, DevRegular &r, void *stream);
void regular_free(DevRegular &r);
// out [5][n] FP64: eta, u, v, w, nhpres (no ramp); z is used as given.
struct RampDev;
// The API rows ([6][n]: wave_SurfElev .. wave_nhPres) and/or the
// wave_Kinematics records ([n][4]) of regular waves in one pass: z clamped at
// the seabed, the ramp applied.
int regular_eval(const DevRegular &r, const Config &cfg, long n, const double *x,
                 const double *y, const double *z, const double *t, const RampDev &ramp, double *rows,
                 double *kin, void *stream);
int regular_solution(const DevRegular &r, double *dst, int cap, void *stream);

// ---------------------------------------------------------------------------
// Precision form (qform.cu): second-order sums at z = 0 as quadratic forms
// ---------------------------------------------------------------------------
// A quadratic form over each point's phasor vector on the tcgen05 tensor
// cores (qform.cu): nblk upper-triangular N x N coefficient blocks, split
// into 16-bit hi/lo parts, each block feeding one output column.
struct TcForm {
    bool built = false;
    int npad = 0, nblk = 0, nout = 0;
    bool fp16 = true;
    // fp16 split with the cross products in the hi accumulator (lo parts not
    // scaled): one accumulator, so the GEMM keeps two accumulator buffers and
    // a tile's epilogue runs under the next tile's MMAs
    bool one_acc = false;
    // K blocks (of 64) per accumulation segment of a column tile, 0: the whole
    // upper-triangle K range in one accumulation
    int kseg = 0;
    void *Whi = nullptr, *Wlo = nullptr;
    float *colscale = nullptr;
    int *bmap = nullptr;        // per block: X half, Y half, output column
    int *err = nullptr;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    void *aux = nullptr;        // stream of the operand preparation (several chunks)
    void *ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};
int tcform_split(TcForm &f, const double *coef64, const int *bmap_host, int nblk, int nout, int npad, bool fp16,
                 void *stream, bool one_acc = false);
int tcform_eval(TcForm &f, const DevSea &sea, long n, const double *x, const double *y, const double *t, long st,
                float *out, void *stream, int *tc_error);
void tcform_free(TcForm &f);
constexpr int TC_NPAD = 256;    // the component count of a TcForm is a multiple of this

// Depth-separable tensor-core form of the s-grid column sums (depthform.cu).
struct DepthForm {
    bool built = false;
    int R = 0, nout = 0;
    int nf = 3;                 // fields per basis function: u, v, w (and p)
    double K = 0, h = 0;
    TcForm tc;
    float *bz = nullptr;        // b_r(z) on a uniform table over [-h, 0]
    float *qout = nullptr;      // [ncol][1 + nf R] GEMM outputs
    long qcap = 0;
};
// nf = 3: u, v, w; nf = 4: and the phase terms of the pressure
int depthform_build(const Config &cfg, const DevSea &sea, DepthForm &df, int nf, void *stream);
void depthform_free(DepthForm &df);
int depthform_columns(DepthForm &df, const DevSea &sea, long nact, const double *x, const double *y,
                      const double *tdev, float *eta2, void *stream);
int depthform_combine(DepthForm &df, long nact, int nl, const float *z0, float *sec, void *stream);
// First-order sums of the tensor-core path (float-float phases): first [5][n]
// (eta1 and the Taylor gradients) and/or sec [nf][n nl] (u1, v1, w1, and dp1
// when nf = 4, at z0).
int depthform_first(const DevSea &sea, long nact, int nl, const double *xy, double t, const float *z0,
                    double *first, float *sec, int nf, void *stream);
int depthform_error(DepthForm &df, void *stream);
int depthform_basis_info(double K, double h, int *R, double *err);

int qform_build(const Config &cfg, const DevSea &sea, bool fp16, void *stream);
void qform_free();
// out [n][4] FP32: eta2, u2, v2, w2 at z0 = 0 (grid mask); method 0 plain
// FP32 CUDA cores, 1 tcgen05 tensor cores.  *tc_error: nonzero if a bounded
// wait of the tensor-core kernel expired.
int qform_eval(const DevSea &sea, long n, const double *x, const double *y, const double *t, int method,
               float *out, void *stream, int *tc_error);

// ---------------------------------------------------------------------------
// Post-processing shared by the API (api_kernels.cu)
// ---------------------------------------------------------------------------
// Ramp::ramp applied to [nf][n] fields in place (Utils.cpp:42-68).
int apply_ramp(const RampCfg &r, long n, const double *x, const double *y, const double *t,
               double *fields, int nf, void *stream);

}  // namespace cfdwm
