// Seeded JONSWAP sea states with cos-2s spreading, generated on the device.
//
// The reference reads its spectral components from waveinput.dat
// (CFDwavemaker.cpp:677-800) and leaves generating them to external tools.
// This builds the ndir-0 component columns (omega, A, k, phase, theta) of a
// sea state in one launch:
//   omega_f = linspace(wmin, wmax, nfreq), theta_d = linspace(-span, span, ndir)
//   S(w) = g^2 w^-5 exp(-1.25 (wp/w)^4) gamma^r(w), r = exp(-(w-wp)^2 / (2 s^2 wp^2)),
//          s = 0.07 (w <= wp) or 0.09, scaled so that 4 sqrt(sum S dw) = Hs
//   D_d  = cos(theta_d / 2)^(2 spread), normalised to sum 1 (D = 1 for ndir 1)
//   A    = sqrt(2 S(omega_f) dw D_d)
//   k    = FP64 Newton solve of w^2 = g k tanh(k h) (60 steps)
//   phase = 2 pi u, u = SplitMix64(seed + (c + 1) 0x9E3779B97F4A7C15) >> 11 / 2^53,
//           c = f ndir + d (Steele, Lea & Flood 2014, "Fast splittable
//           pseudorandom number generators"): one independent draw per component
// so the same (parameters, seed) give the same sea on any device.
#include "cfdwm.h"

#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>

namespace cfdwm {

namespace {

__host__ __device__ inline unsigned long long splitmix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct SpecArgs {
    double hs, tp, gamma, wmin, wmax, depth, spread, span, g;
    int nfreq, ndir;
    unsigned long long seed;
    double *out;     // [5][nfreq ndir]
};

// one block: the spectrum and spreading sums in a fixed order by thread 0,
// then one thread per component
__global__ void __launch_bounds__(256) k_spectrum(SpecArgs a) {
    __shared__ double s_m0, s_dsum;
    const int nf = a.nfreq, nd = a.ndir, n = nf * nd;
    const double dw = nf > 1 ? (a.wmax - a.wmin) / (nf - 1) : 1.0;
    const double wp = 2.0 * 3.14159265358979323846 / a.tp;
    auto omega = [&](int f) { return nf > 1 ? a.wmin + (a.wmax - a.wmin) * f / (nf - 1) : a.wmin; };
    auto spec = [&](double w) {
        const double sg = w <= wp ? 0.07 : 0.09;
        const double r = exp(-((w - wp) * (w - wp)) / (2.0 * sg * sg * wp * wp));
        return a.g * a.g * pow(w, -5.0) * exp(-1.25 * pow(wp / w, 4.0)) * pow(a.gamma, r);
    };
    auto theta = [&](int d) { return nd > 1 ? -a.span + 2.0 * a.span * d / (nd - 1) : 0.0; };
    auto dir = [&](int d) { return nd > 1 ? pow(cos(0.5 * theta(d)), 2.0 * a.spread) : 1.0; };
    if (threadIdx.x == 0) {
        double m0 = 0.0, ds = 0.0;
        for (int f = 0; f < nf; f++) m0 += spec(omega(f)) * dw;
        for (int d = 0; d < nd; d++) ds += dir(d);
        s_m0 = m0;
        s_dsum = ds;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const int f = c / nd, d = c % nd;
        const double w = omega(f);
        const double S = spec(w) * (a.hs * a.hs / 16.0) / s_m0;
        const double D = dir(d) / s_dsum;
        double k = fmax(w * w / a.g, w / sqrt(a.g * a.depth));
        for (int it = 0; it < 60; it++) {
            const double th = tanh(k * a.depth);
            const double fk = a.g * k * th - w * w, df = a.g * (th + k * a.depth * (1.0 - th * th));
            k = k - fk / df;
        }
        const unsigned long long z = splitmix64(a.seed + (unsigned long long)(c + 1) * 0x9E3779B97F4A7C15ULL);
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
        a.out[c] = w;
        a.out[n + c] = sqrt(2.0 * S * dw * D);
        a.out[2 * n + c] = k;
        a.out[3 * n + c] = 2.0 * 3.14159265358979323846 * u;
        a.out[4 * n + c] = theta(d);
    }
}

}  // namespace

int spectrum_components(const double *p, int nfreq, int ndir, unsigned long long seed, double *out_dev,
                        void *stream) {
    if (!p || nfreq < 1 || ndir < 1 || (long)nfreq * ndir > (1L << 22)) return E_BAD_ARGUMENT;
    SpecArgs a;
    a.hs = p[0]; a.tp = p[1]; a.gamma = p[2]; a.wmin = p[3]; a.wmax = p[4]; a.depth = p[5];
    a.spread = p[6]; a.span = p[7]; a.g = p[8];
    if (!(a.tp > 0) || !(a.wmin > 0) || !(a.wmax >= a.wmin) || !(a.depth > 0) || !(a.g > 0) || !(a.hs >= 0) ||
        !(a.gamma > 0))
        return E_BAD_ARGUMENT;
    a.nfreq = nfreq; a.ndir = ndir; a.seed = seed; a.out = out_dev;
    k_spectrum<<<1, 256, 0, (cudaStream_t)stream>>>(a);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? OK : E_CUDA;
}

}  // namespace cfdwm
