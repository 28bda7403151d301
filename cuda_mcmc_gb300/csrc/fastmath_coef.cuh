// fastmath_coef.cuh -- GENERATED by gen_fastmath.py; do not edit.
// Monomial coefficients (lowest degree first) of float32 polynomial fits:
//   kAtanP:  atan(a)/a in s = a^2, a in [0,1]       max |atan err| 1.53e-07
//   kSinPiS: sin(pi r)/r in s = r^2, |r| <= 1/2    max |sin err|  2.13e-07
//   kCosPiK: cos(pi r) in s = r^2, |r| <= 1/2      max |cos err|  1.49e-07
#pragma once
namespace cmc {
static __constant__ const float kAtanP[8] = {9.999998808e-01f, -3.333181143e-01f, 1.996696144e-01f, -1.400329024e-01f, 9.868865460e-02f, -5.882975459e-02f, 2.378051914e-02f, -4.559792113e-03f};
static __constant__ const float kSinPiS[6] = {3.141592741e+00f, -5.167712688e+00f, 2.550163269e+00f, -5.992521644e-01f, 8.205035329e-02f, -7.028304040e-03f};
static __constant__ const float kCosPiK[7] = {1.000000000e+00f, -4.934802055e+00f, 4.058712006e+00f, -1.335262299e+00f, 2.353254408e-01f, -2.577632107e-02f, 1.839996316e-03f};
}  // namespace cmc
