// Ramp::ramp (Utils.cpp:42-68): the minimum of up to six clamped linear
// ramps in t, x and y, shared by the finishing pass of the API rows and the
// kernels that write the API rows themselves (regular waves; the irregular
// sums' combining pass).
#pragma once

namespace cfdwm {

struct RampDev {
    int init, flags;
    double lim[12];
};

__device__ __forceinline__ double d_ramp(const RampDev &r, double t, double x, double y) {
    if (!r.init) return 1.0;
    double v[6] = {t, t, x, x, y, y};
    double m = 1.0;
    for (int q = 0; q < 6; q++) {
        double rq = 1.0;
        if (r.flags & (1 << q)) {
            double a = (v[q] - r.lim[2 * q]) / (r.lim[2 * q + 1] - r.lim[2 * q]);
            rq = (q & 1) ? fmax(fmin(1. - a, 1.), 0.) : fmax(fmin(a, 1.), 0.);
        }
        m = (q == 0) ? rq : fmin(m, rq);
    }
    return m;
}

// The API rows written by a kernel that ends the evaluation: rows [6][ldo]
// (wave_SurfElev .. wave_nhPres) and/or wave_Kinematics records [n][4], the
// ramp at (x, y, t) applied where one is set, p_nh = dp - rho g eta.
struct ApiRows {
    RampDev ramp;
    double rho, g;
    const double *x, *y, *t;
    double *rows;
    double *kin;
};

}  // namespace cfdwm
