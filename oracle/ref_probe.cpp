// Reference probe (TEST INFRASTRUCTURE ONLY).
//
// A small C-ABI shim, written for this repository, that is linked against the
// reference's own objects (oystelan/CFDwavemaker v3.1.0 src/*.cpp, compiled
// from where they lie by oracle/Makefile into oracle/_ref/).  It lets
// tests/golden/make_golden.py drive the unmodified reference through its
// public API (CFDwavemaker.h) and read a few internal arrays of its global
// singletons (CFDwavemaker.cpp:129-163) to record golden vectors.  It is
// never linked into the product.
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <fcntl.h>
#include <vector>
#include "CFDwavemaker.h"
#include "Irregular.h"
#include "lsgrid_spline.h"
#include "FentonStream.h"

extern Irregular irregular;      // CFDwavemaker.cpp:141
extern lsGridSpline sgrids;      // CFDwavemaker.cpp:147
extern FentonStream fenton;      // CFDwavemaker.cpp:138

namespace {
int g_saved_stdout = -1;
void quiet_begin() {
    fflush(stdout);
    g_saved_stdout = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    dup2(devnull, 1);
    close(devnull);
}
void quiet_end() {
    fflush(stdout);
    dup2(g_saved_stdout, 1);
    close(g_saved_stdout);
}
}  // namespace

extern "C" {

int refp_init(const char *dir) {
    if (chdir(dir) != 0) return -2;
    quiet_begin();
    int rc = wave_Initialize();
    quiet_end();
    return rc;
}

// Public API, looped: which 0 SurfElev, 1 VeloX, 2 VeloY, 3 VeloZ, 4 DynPres,
// 5 nhPres, 6 VFrac (z is the cell centre, dcell = 0.1), 7 Kinematics (4 out).
void refp_api(int which, long n, const double *x, const double *y, const double *z,
              const double *t, double *out) {
    quiet_begin();
    for (long p = 0; p < n; p++) {
        switch (which) {
        case 0: out[p] = wave_SurfElev(x[p], y[p], t[p]); break;
        case 1: out[p] = wave_VeloX(x[p], y[p], z[p], t[p]); break;
        case 2: out[p] = wave_VeloY(x[p], y[p], z[p], t[p]); break;
        case 3: out[p] = wave_VeloZ(x[p], y[p], z[p], t[p]); break;
        case 4: out[p] = wave_DynPres(x[p], y[p], z[p], t[p]); break;
        case 5: out[p] = wave_nhPres(x[p], y[p], z[p], t[p]); break;
        case 6: out[p] = wave_VFrac(x[p], y[p], z[p], t[p], 0.1); break;
        case 7: {
            double *r = wave_Kinematics(x[p], y[p], z[p], t[p]);
            for (int q = 0; q < 4; q++) out[4 * p + q] = r[q];
            delete[] r;
            break;
        }
        }
    }
    quiet_end();
}

// Irregular methods called directly: 0 eta1, 1 eta2, 2 u2, 3 v2, 4 w2, 5 dp2,
// 6 uvw2 (4 outputs per point), 7 eta (dispatch), 8 u, 9 w, 10 dp.
void refp_irr(int which, long n, const double *x, const double *y, const double *z,
              const double *t, double *out) {
    for (long p = 0; p < n; p++) {
        switch (which) {
        case 0: out[p] = irregular.eta1(t[p], x[p], y[p]); break;
        case 1: out[p] = irregular.eta2(t[p], x[p], y[p]); break;
        case 2: out[p] = irregular.u2(t[p], x[p], y[p], z[p]); break;
        case 3: out[p] = irregular.v2(t[p], x[p], y[p], z[p]); break;
        case 4: out[p] = irregular.w2(t[p], x[p], y[p], z[p]); break;
        case 5: out[p] = irregular.dp2(t[p], x[p], y[p], z[p]); break;
        case 6: {
            UVWP r = irregular.uvw2(t[p], x[p], y[p], z[p]);
            out[4 * p + 0] = r.u; out[4 * p + 1] = r.v; out[4 * p + 2] = r.w; out[4 * p + 3] = r.p;
            break;
        }
        case 7: out[p] = irregular.eta(t[p], x[p], y[p]); break;
        case 8: out[p] = irregular.u(t[p], x[p], y[p], z[p]); break;
        case 9: out[p] = irregular.w(t[p], x[p], y[p], z[p]); break;
        case 10: out[p] = irregular.dp(t[p], x[p], y[p], z[p]); break;
        }
    }
}

// Component arrays after parsing, sorting and normalisation:
// omega, A, k, phase, theta, ramptime, starttime, duration ([8][n]).
int refp_components(double *dst) {
    int n = irregular.nfreq * irregular.ndir;
    if (!dst) return n;
    for (int i = 0; i < n; i++) {
        dst[0 * n + i] = irregular.omega[i];
        dst[1 * n + i] = irregular.A[i];
        dst[2 * n + i] = irregular.k[i];
        dst[3 * n + i] = irregular.phase[i];
        dst[4 * n + i] = irregular.theta[i];
        dst[5 * n + i] = irregular.freq_ramptime[i];
        dst[6 * n + i] = irregular.freq_starttime[i];
        dst[7 * n + i] = irregular.freq_duration[i];
    }
    return n;
}

long refp_npairs() { return (long)irregular.pair_cache.size(); }

void refp_force_update(double t) {
    quiet_begin();
    wave_force_update(t);
    quiet_end();
}

// lsGridSpline::export_vtu (lsgrid_spline.cpp:1222-1403) of the global grid into `path`.
int refp_sgrid_export_vtu(const char *path, int last) {
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    sgrids.export_vtu(fp, last != 0);
    fclose(fp);
    return 0;
}

void refp_sgrid_dims(int *dims, double *vals) {
    dims[0] = sgrids.nx; dims[1] = sgrids.ny; dims[2] = sgrids.nl; dims[3] = sgrids.tstep;
    vals[0] = sgrids.t0; vals[1] = sgrids.dt; vals[2] = sgrids.dx; vals[3] = sgrids.dy;
    vals[4] = sgrids.ds;
}

// Same numbering as orc_sgrid_array (oracle/oracle.h).
long refp_sgrid_array(int which, double *dst) {
    long c = (long)sgrids.nx * sgrids.ny, v = c * sgrids.nl;
    double *src = nullptr;
    long n = 0;
    switch (which) {
    case 0: src = sgrids.ETA; n = 4 * c; break;
    case 1: src = sgrids.UX; n = 4 * v; break;
    case 2: src = sgrids.UY; n = 4 * v; break;
    case 3: src = sgrids.UZ; n = 4 * v; break;
    case 4: src = sgrids.ETAdx; n = 2 * c; break;
    case 5: src = sgrids.ETAdy; n = 2 * c; break;
    case 6: src = sgrids.ETAdt; n = 4 * c; break;
    case 7: src = sgrids.Udt; n = 4 * v; break;
    case 8: src = sgrids.Udx; n = 2 * v; break;
    case 9: src = sgrids.Udy; n = 2 * v; break;
    case 10: src = sgrids.Uds; n = 2 * v; break;
    case 11: src = sgrids.Vdt; n = 4 * v; break;
    case 12: src = sgrids.Vdx; n = 2 * v; break;
    case 13: src = sgrids.Vdy; n = 2 * v; break;
    case 14: src = sgrids.Vds; n = 2 * v; break;
    case 15: src = sgrids.Wdt; n = 4 * v; break;
    case 16: src = sgrids.Wdx; n = 2 * v; break;
    case 17: src = sgrids.Wdy; n = 2 * v; break;
    case 18: src = sgrids.Wds; n = 2 * v; break;
    default: return -1;
    }
    if (dst) std::memcpy(dst, src, sizeof(double) * n);
    return n;
}

// Fenton solution: k, c, ubar, R, L, T, B[1..N]; returns the count.
int refp_fenton(double *dst) {
    int N = fenton.num_components(), q = 0;
    dst[q++] = fenton.k; dst[q++] = fenton.c; dst[q++] = fenton.mean_velocity();
    dst[q++] = fenton.bernoulli_R(); dst[q++] = fenton.wave_length; dst[q++] = fenton.wave_period;
    for (int j = 1; j <= N; j++) dst[q++] = fenton.coefficient(j);
    return q;
}

}  // extern "C"
