// sincos_poly.cuh -- exp(i x) = (cos x, sin x) in single precision for the
// moderate arguments of the transmission function (|x| of a few radians: the
// phase sigma * v of a projected potential).
//
// Method (written here from the mathematics): x = k pi/2 + r with k the
// nearest integer to x * 2/pi and r = x - k pi/2 formed with fused
// multiply-adds against pi/2 split into three single-precision parts (Cody and
// Waite, "Software Manual for the Elementary Functions", 1980), so |r| <= pi/4
// with an absolute error of a few 1e-8 for |k| < 2^12; then the Taylor series
// of sin (to r^9) and cos (to r^10) on |r| <= pi/4 (truncation below 2e-11 and
// 3e-8 respectively), evaluated by Horner's rule; the quadrant k mod 4 rotates
// (cos r, sin r) by k quarter turns.  Accuracy: a few units in the last place
// (checked against double precision on the host, tests/test_sincos_poly.py).
// Arguments with |x| > kExpiMax go to the CUDA library's sincosf instead.
#pragma once

#include <cuda_runtime.h>

namespace msk {

constexpr float kExpiMax = 4096.0f;

__host__ __device__ __forceinline__ float2 expi_poly(float x)
{
    // pi/2 = kP1 + kP2 + kP3 (kP1 = pi/2 rounded to float, kP2 and kP3 the
    // rounded remainders)
    constexpr float kTwoOverPi = 0.636619772367581343f;
    constexpr float kP1 = 1.57079637050628662109375f;
    constexpr float kP2 = -4.37113882867379300296e-08f;
    constexpr float kP3 = -1.71512451000588190000e-15f;
    const float k = rintf(x * kTwoOverPi);
    float r = fmaf(-k, kP1, x);
    r = fmaf(-k, kP2, r);
    r = fmaf(-k, kP3, r);
    const float r2 = r * r;
    // sin r = r + r^3 (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 / 9!)))
    float ps = fmaf(r2, 2.75573192239858906526e-06f, -1.98412698412698412526e-04f);
    ps = fmaf(r2, ps, 8.33333333333333321769e-03f);
    ps = fmaf(r2, ps, -1.66666666666666657415e-01f);
    const float s = fmaf(r * r2, ps, r);
    // cos r = 1 + r^2 (-1/2! + r^2 (1/4! + r^2 (-1/6! + r^2 (1/8! - r^2 / 10!))))
    float pc = fmaf(r2, -2.75573192239858906526e-07f, 2.48015873015873015873e-05f);
    pc = fmaf(r2, pc, -1.38888888888888894189e-03f);
    pc = fmaf(r2, pc, 4.16666666666666643537e-02f);
    pc = fmaf(r2, pc, -0.5f);
    const float c = fmaf(r2, pc, 1.0f);
    // rotate by k quarter turns: q = 0 (c, s), 1 (-s, c), 2 (-c, -s), 3 (s, -c)
    const int q = (int)k;
    const float cq = (q & 1) ? s : c, sq = (q & 1) ? c : s;
    return make_float2((q + 1) & 2 ? -cq : cq, (q & 2) ? -sq : sq);
}

}  // namespace msk
