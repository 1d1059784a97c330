// Complex FP64 helpers on double2 (x = real, y = imaginary part), for the
// k-point path and the Hermitian eigensolver.
#pragma once
#include <cuda_runtime.h>

namespace hqcgb {

__host__ __device__ inline double2 zmk(double re, double im) { return make_double2(re, im); }
__host__ __device__ inline double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) b
__host__ __device__ inline double2 zcmul(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ inline double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ inline double2 zscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__host__ __device__ inline double zabs2(double2 a) { return a.x * a.x + a.y * a.y; }
// 1 / a (Smith's scaling against overflow)
__host__ __device__ inline double2 zrecip(double2 a) {
  if (fabs(a.x) >= fabs(a.y)) {
    double r = a.y / a.x, den = a.x + a.y * r;
    return make_double2(1.0 / den, -r / den);
  }
  double r = a.x / a.y, den = a.x * r + a.y;
  return make_double2(r / den, -1.0 / den);
}

}  // namespace hqcgb
