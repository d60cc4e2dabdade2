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

}  // namespace cfdwm
