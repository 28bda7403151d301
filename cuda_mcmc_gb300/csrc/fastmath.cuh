// fastmath.cuh -- float32 helpers for the model inner loops.
//
// Polynomial coefficients come from gen_fastmath.py / gen_bessel_table.py
// (Chebyshev interpolants of float64 values); accuracies are a few float32
// ulps, stated in the generated headers.
#pragma once
#include <cuda_runtime.h>

#include "bessel_table.cuh"
#include "fastmath_coef.cuh"

namespace cmc {

// sin(pi t), cos(pi t): t = n + r with n = rint(t), |r| <= 1/2, and
// sin(pi (n + r)) = (-1)^n sin(pi r), cos(pi (n + r)) = (-1)^n cos(pi r).
__device__ __forceinline__ void sincospi_poly(float t, float *s, float *c)
{
  const float n = rintf(t);
  const float r = t - n;
  const float q = r * r;
  float ps = kSinPiS[5];
#pragma unroll
  for (int k = 4; k >= 0; --k) ps = fmaf(ps, q, kSinPiS[k]);
  float pc = kCosPiK[6];
#pragma unroll
  for (int k = 5; k >= 0; --k) pc = fmaf(pc, q, kCosPiK[k]);
  const float sg = (((int)n) & 1) ? -1.0f : 1.0f;
  *s = sg * (ps * r);
  *c = sg * pc;
}

// Single hardware approximations (PTX sin / cos / ex2 / rsqrt .approx.ftz):
// denormal inputs and results are flushed to zero, which the model's terms
// never depend on, so no denormal handling is wrapped around them.
__device__ __forceinline__ float sin_ftz(float x)
{
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float cos_ftz(float x)
{
  float y;
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// 2^x; 2^-inf = 0
__device__ __forceinline__ float ex2_ftz(float x)
{
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// 1/sqrt(x) for a positive normal x
__device__ __forceinline__ float rsqrt_ftz(float x)
{
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// sin(x), cos(x) as sin / cos(pi t), t = x / pi, from the polynomials above:
// rint, multiplies and explicit fmaf only, so that every kernel and call site
// rounds it identically (the per-proposal constants of the sweep and batch
// kernels must agree to the bit).  A few float32 ulps for |x| up to ~10^3.
__device__ __forceinline__ void sincos_fma(float x, float *s, float *c)
{
  sincospi_poly(x * 0.318309886183790672f, s, c);
}

#ifndef CMC_MUFU_SINCOS
#define CMC_MUFU_SINCOS 1
#endif

// sin(x), cos(x) for the model's arguments: the hardware approximations
// applied to x directly -- their absolute error stays below 2^-20.5 for
// |x| <= 100 pi (PTX ISA, sin.approx / cos.approx), and the arguments stay
// within a few pi (the ring shift 2 pi d U and the Gaussian offset phase, of
// a few units), so no explicit range reduction is needed.  With
// CMC_MUFU_SINCOS = 0, the polynomials of x / pi.
__device__ __forceinline__ void sincos_fast(float x, float *s, float *c)
{
#if CMC_MUFU_SINCOS
  *s = sin_ftz(x);
  *c = cos_ftz(x);
#else
  sincospi_poly(x * 0.318309886183790672f, s, c);
#endif
}

// atan2(y, x) in [-pi, pi]: a = min/max of |x|, |y| in [0, 1], atan(a) from
// the polynomial, then the octant.  atan2(0, 0) = 0.
__device__ __forceinline__ float atan2_poly(float y, float x)
{
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float a = (mx > 0.0f) ? __fdividef(mn, mx) : 0.0f;
  const float s = a * a;
  constexpr int kN = (int)(sizeof(kAtanP) / sizeof(kAtanP[0]));
  float p = kAtanP[kN - 1];
#pragma unroll
  for (int k = kN - 2; k >= 0; --k) p = fmaf(p, s, kAtanP[k]);
  // pi/2 - p a as an explicit fmaf: no multiply-add is left for the compiler
  // to contract differently in different kernels
  float r = (ay > ax) ? fmaf(-p, a, 1.57079632679489662f) : p * a;
  if (x < 0.0f) r = 3.14159265358979324f - r;
  return copysignf(r, y);
}

// F1, F2 as below, at the table coordinate t = kBesselSub |x| - 1/2, which
// the caller forms with one fmaf.  Interval i = rint(t) and offset
// d = t - i in [-1/2, 1/2] come from adding 1.5 * 2^23: the float sum is the
// integer nearest t, held in its low mantissa bits, so that no conversion
// instructions are needed.  BIG = false: the caller guarantees
// -1/2 <= t < kBesselIntervals - 1/2 (no index check).  BIG = true: any t,
// NaN and garbage included; the index is clamped to the table (unsigned
// min), and from x = 32 on (t >= kBesselIntervals - 1/2) F1, F2 come from
// CUDA's j0f / j1f as below.
template <bool BIG>
__device__ __forceinline__ void bessel_f12_at(const float4 *tab, float t, float &f1, float &f2)
{
  constexpr int kQ = (kBesselDeg + 1) / 2;
  constexpr float kMagic = 12582912.0f;   // 1.5 * 2^23
  const float a = __fadd_rn(t, kMagic);
  const float d = __fsub_rn(t, __fsub_rn(a, kMagic));
  unsigned i = (unsigned)(__float_as_int(a) - __float_as_int(kMagic));
  if (BIG) i = min(i, (unsigned)(kBesselIntervals - 1));
  const float4 *c = tab + i * kQ;
  float4 q = c[kQ - 1];
  float p1 = fmaf(q.z, d, q.x), p2 = fmaf(q.w, d, q.y);
#pragma unroll
  for (int m = kQ - 2; m >= 0; --m) {
    q = c[m];
    p1 = fmaf(fmaf(p1, d, q.z), d, q.x);
    p2 = fmaf(fmaf(p2, d, q.w), d, q.y);
  }
  f1 = p1;
  f2 = p2;
  if (BIG && t >= (float)kBesselIntervals - 0.5f) {
    const float x = fmaf(t, 1.0f / (float)kBesselSub, 0.5f / (float)kBesselSub);
    const float ix = 1.0f / x;
    const float j0 = j0f(x), j1 = j1f(x);
    f1 = j1 * ix;
    f2 = fmaf(2.0f, f1, -j0) * ix * ix;
  }
}

// F1(x) = J1(x)/x and F2(x) = J2(x)/x^2 (even in x) from the piecewise
// polynomial table `tab` (a shared-memory copy of kBesselTab: per interval of
// width 1/kBesselSub, (kBesselDeg + 1) / 2 float4 of coefficient pairs, in
// t = kBesselSub x - (i + 0.5)).  BIG = false: x is known to lie inside the
// table (straight-line code); BIG = true: beyond the table F1, F2 come from
// CUDA's j0f/j1f with J2 = 2 J1/x - J0.
template <bool BIG>
__device__ __forceinline__ void bessel_f12_tab(const float4 *tab, float x, float &f1, float &f2)
{
  constexpr int kQ = (kBesselDeg + 1) / 2;
  x = fabsf(x);
  const float xs = x * (float)kBesselSub;
  const int i = min((int)xs, kBesselIntervals - 1);
  const float d = xs - ((float)i + 0.5f);
  const float4 *c = tab + i * kQ;
  float4 a = c[kQ - 1];
  float p1 = fmaf(a.z, d, a.x), p2 = fmaf(a.w, d, a.y);
#pragma unroll
  for (int m = kQ - 2; m >= 0; --m) {
    a = c[m];
    p1 = fmaf(fmaf(p1, d, a.z), d, a.x);
    p2 = fmaf(fmaf(p2, d, a.w), d, a.y);
  }
  f1 = p1;
  f2 = p2;
  if (BIG && x >= (float)kBesselXmax) {
    const float ix = 1.0f / x;
    const float j0 = j0f(x), j1 = j1f(x);
    f1 = j1 * ix;
    f2 = fmaf(2.0f, f1, -j0) * ix * ix;
  }
}

}  // namespace cmc
