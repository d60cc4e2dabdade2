// Geometry of the s-grid shared by the grid and the learned-update kernels.
#pragma once

#include <cuda_runtime.h>

namespace cfdwm {

struct GridGeom {
    int nx, ny, nl;
    double d0, d2, dx, dy, ds, depth, swl, tan_a, tan_b, dt;
};

// sigmaS2cart (lsgrid_spline.cpp:117-122) in FP64 for level m, s = m * ds.
// s and s - 1 are rounded explicitly: a fused m*ds - 1 leaves +5.6e-17 at the
// surface level (0.2 * 5 - 1) where the reference's separately rounded
// product gives exactly 0, and pow() of the then negative tangent is NaN.
__device__ __forceinline__ double d_sigma_level(const GridGeom &g, int m) {
    double s = __dmul_rn(g.ds, (double)m);
    double base = fmax(tan(-__dadd_rn(s, -1.0) * g.tan_a), 0.0);
    return -pow(base, g.tan_b) / pow(tan(g.tan_a), g.tan_b);
}
// s2z with the stretched coordinate of a level (lsgrid_spline.cpp:96-98)
__device__ __forceinline__ double d_s2z(const GridGeom &g, double sigma, double e) {
    return (e - g.swl) + sigma * (g.depth + (e - g.swl));
}
__device__ __forceinline__ double d_sigmaS2cart(const GridGeom &g, int m, double e) {
    return d_s2z(g, d_sigma_level(g, m), e);
}

}  // namespace cfdwm
