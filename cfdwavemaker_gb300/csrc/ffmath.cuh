// Float-float arithmetic for wave phases: k.x - omega t + phase0 reaches
// 1e3-1e4 rad, so it is formed from (hi, lo) float pairs with Dekker's exact
// product (via FMA) and Knuth's two-sum, and reduced by a three-part 2 pi
// (Cody-Waite) before an FP32 sincos.  Error: a few 1e-7 rad at 1e4 rad.
#pragma once

#include <cuda_runtime.h>

namespace cfdwm {

// a*b as an unevaluated float pair (products of the lo parts dropped)
__device__ __forceinline__ float2 ff_mul(float ah, float al, float bh, float bl) {
    float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    return make_float2(p, e);
}
// Knuth two-sum of the hi parts, error folded into the lo part
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    float s = a.x + b.x;
    float bb = s - a.x;
    float e = (a.x - (s - bb)) + (b.x - bb);
    return make_float2(s, e + a.y + b.y);
}
// the phase reduced to about [-pi, pi]
__device__ __forceinline__ float ff_reduce_2pi(float2 ph) {
    // 2 pi = P1 + P2 + P3: P1 = 201/32 has 8 significant bits, so n P1 is exact for |n| < 2^16
    const float P1 = 6.28125f, P2 = 1.9353071693331003e-3f, P3 = 1.0253376273028358e-11f;
    float n = rintf(ph.x * 0.15915494309189535f);
    float red = fmaf(-n, P1, ph.x);
    red = fmaf(-n, P2, red);
    red = fmaf(-n, P3, red);
    return red + ph.y;
}
__host__ __device__ __forceinline__ void ff_split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// v as an unevaluated float pair by integer operations on its bits only: FP64
// instructions, conversions included, run at a small fraction of the FP32
// rate on this GPU, and even a predicated-off FP64 fallback takes their issue
// slots.  For 2^-74 <= |v| < 2^127, hi keeps the leading 24 significant bits
// (truncated) and lo the next 29 rounded to 24, so hi + lo carries 48 bits;
// 2^-126 <= |v| < 2^-74 gives (hi, 0); smaller magnitudes give 0; larger,
// infinite and NaN inputs give an infinity or a NaN of v's sign.
__device__ __forceinline__ float2 ff_from_double(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7FFu);          // biased exponent
    if (e < 897) return make_float2(__uint_as_float(sign), 0.f);
    if (e > 1150) {
        const bool nan = e == 2047 && ((hw & 0xFFFFFu) | lw) != 0u;
        return make_float2(__uint_as_float(sign | (nan ? 0x7FC00000u : 0x7F800000u)), 0.f);
    }
    const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
    if (e < 949) return make_float2(hi, 0.f);
    // the low 29 mantissa bits have weight 2^(e - 1075): float exponent field e - 948
    const float scale = __uint_as_float((unsigned)(e - 948) << 23);
    const float lo = __uint_as_float(__float_as_uint(__uint2float_rn(lw & 0x1FFFFFFFu) * scale) | sign);
    return make_float2(hi, lo);
}

// f as a double, exactly, by integer operations only (all float classes)
__device__ __forceinline__ double d_from_float(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u, e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    unsigned hw, lw;
    if (e == 255u) {                                  // infinity, NaN (payload kept)
        hw = sign | 0x7FF00000u | (m >> 3);
        lw = (m & 7u) << 29;
    } else if (e == 0u) {
        if (m == 0u) {                                // signed zero
            hw = sign;
            lw = 0u;
        } else {                                      // subnormal: m 2^-149, normalised
            const int lz = __clz(m);                  // 9..31
            const unsigned mm = (m << (lz - 8)) & 0x7FFFFFu;
            hw = sign | ((unsigned)(905 - lz) << 20) | (mm >> 3);
            lw = (mm & 7u) << 29;
        }
    } else {
        hw = sign | ((e + 896u) << 20) | (m >> 3);
        lw = (m & 7u) << 29;
    }
    return __hiloint2double((int)hw, (int)lw);
}

// sin and cos of a reduced argument (|x| <= about 3.3) in FP32 FMAs only:
// quarter-period Cody-Waite reduction (pi/2 = A + B + C, A and B short enough
// that q A and q B are exact for |q| <= 2), then the Taylor series of sin to
// r^9 and of cos to r^10 on |r| <= pi/4 (truncation below 2e-9); measured
// against sin/cos at FP64 on a fine grid of [-3.3, 3.3]: below 1e-7 absolute.
__device__ __forceinline__ void ff_sincos_poly(float x, float &s, float &c) {
    const float q = rintf(x * 0.636619772f);
    float r = fmaf(-q, 1.5703125f, x);
    r = fmaf(-q, 4.837512969970703125e-4f, r);
    r = fmaf(-q, 7.549789948768648e-8f, r);
    const float r2 = r * r;
    const float ps = fmaf(r2, fmaf(r2, fmaf(r2, 2.7557319e-6f, -1.98412698e-4f), 8.33333333e-3f), -0.166666667f);
    const float pc =
        fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, -2.75573192e-7f, 2.48015873e-5f), -1.38888889e-3f), 4.16666667e-2f),
             -0.5f);
    const float sr = fmaf(r * r2, ps, r), cr = fmaf(r2, pc, 1.0f);
    const int qi = ((int)q) & 3;
    s = qi == 0 ? sr : qi == 1 ? cr : qi == 2 ? -sr : -cr;
    c = qi == 0 ? cr : qi == 1 ? -sr : qi == 2 ? -cr : sr;
}

// Irregular::freq_ramp (Irregular.cpp:200-204), FP64
__device__ __forceinline__ double ff_freq_ramp(double t, double rt, double ts, double du) {
    const double small = 1.e-12;   // Irregular.h:8
    double rampdown = fmax(fmin(1. - ((t - ts - du + rt) / (rt + small)), 1.), 0.);
    double rampup = fmax(fmin(((t - ts) / (rt + small)), 1.), 0.);
    return rampup * rampdown;
}

// One component's phase coefficients as float pairs and its ramp at time t.
struct FfComp {
    float kxh, kxl, kyh, kyl, wh, wl, ph, pl, r;
};
// Component i of the FP64 phase rows [7][cs] (kx, ky, omega, phase0, ramptime,
// starttime, duration); with trivial_ramp every component has component 0's ramp.
__device__ __forceinline__ FfComp ff_component(const double *phase, int cs, int i, int trivial_ramp, double t) {
    FfComp d;
    ff_split(phase[i], d.kxh, d.kxl);
    ff_split(phase[cs + i], d.kyh, d.kyl);
    ff_split(-phase[2 * cs + i], d.wh, d.wl);
    ff_split(phase[3 * cs + i], d.ph, d.pl);
    const int ir = trivial_ramp ? 0 : i;
    d.r = (float)ff_freq_ramp(t, phase[4 * cs + ir], phase[5 * cs + ir], phase[6 * cs + ir]);
    return d;
}
// cos and sin of kx (x - fx) + ky (y - fy) - omega t + phase0, the offsets and
// t given as float pairs.  The reduced argument lies in about [-pi, pi], where
// the SFU's sine and cosine are within a few 1e-7; the general sincosf kept
// the FP64 pipe busy in the per-(column, component) loops.
__device__ __forceinline__ void ff_phasor(const FfComp &d, float dxh, float dxl, float dyh, float dyl, float th,
                                          float tl, float &c, float &s) {
    float2 ph = ff_add(ff_mul(d.kxh, d.kxl, dxh, dxl), ff_mul(d.kyh, d.kyl, dyh, dyl));
    ph = ff_add(ph, ff_mul(d.wh, d.wl, th, tl));
    ph = ff_add(ph, make_float2(d.ph, d.pl));
    __sincosf(ff_reduce_2pi(ph), &s, &c);
}

}  // namespace cfdwm
