// Householder reduction of a symmetric matrix to tridiagonal form (lower
// variant), shared by the FP64 solver and the FP32 stage of the mixed solver.
// One thread block; A (n x n, row-major, global) is overwritten: the
// trailing matrix receives rank-2 updates and column k keeps the Householder
// vector v_k below the subdiagonal (v_k[0] = 1 implied).  On return d, e,
// tau hold the diagonal, subdiagonal and reflector scalars (shared or global
// memory); when hv is not null the vectors are also stored contiguously,
// hv[k * n + i] = v_k[i] for i < n - k - 1.
#pragma once
#include "common.cuh"

namespace hqcgb {

__device__ inline double e_sqrt(double x) { return sqrt(x); }
__device__ inline float e_sqrt(float x) { return sqrtf(x); }
__device__ inline double e_copysign(double a, double b) { return copysign(a, b); }
__device__ inline float e_copysign(float a, float b) { return copysignf(a, b); }

template <typename T>
__device__ void householder_tridiag(int n, T *__restrict__ A, T *__restrict__ d,
                                    T *__restrict__ e, T *__restrict__ tau, T *__restrict__ v,
                                    T *__restrict__ p, T *red, T *s_dbl, T *__restrict__ hv) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int k = 0; k < n - 2; ++k) {
    int m = n - k - 1;
    const T *col = A + (long long)(k + 1) * n + k;  // A[k+1+i][k] = col[i*n]
    T s2 = 0;
    for (int i = 1 + tid; i < m; i += nt) {
      T x = col[(long long)i * n];
      s2 += x * x;
    }
    s2 = block_sum(s2, red);
    if (tid == 0) {
      T x0 = col[0];
      if (s2 == T(0)) {
        tau[k] = T(0);
        e[k] = x0;
        s_dbl[0] = T(0);
      } else {
        T beta = -e_copysign(e_sqrt(x0 * x0 + s2), x0);
        tau[k] = (beta - x0) / beta;
        e[k] = beta;
        s_dbl[0] = T(1) / (x0 - beta);
      }
    }
    __syncthreads();
    T tk = tau[k];
    if (tk == T(0)) {
      for (int i = tid; i < m; i += nt) {
        v[i] = (i == 0) ? T(1) : T(0);
        if (hv) hv[(long long)k * n + i] = v[i];
      }
      __syncthreads();
      continue;
    }
    T sc = s_dbl[0];
    for (int i = tid; i < m; i += nt) {
      v[i] = (i == 0) ? T(1) : col[(long long)i * n] * sc;
      if (hv) hv[(long long)k * n + i] = v[i];
    }
    __syncthreads();
    // p = tau * A22 v  (one warp per row, coalesced over columns)
    T *A22 = A + (long long)(k + 1) * n + (k + 1);
    for (int i = warp; i < m; i += nw) {
      const T *row = A22 + (long long)i * n;
      T s = 0;
      for (int j = lane; j < m; j += 32) s += row[j] * v[j];
      s = warp_sum(s);
      if (lane == 0) p[i] = tk * s;
    }
    __syncthreads();
    T pv = 0;
    for (int i = tid; i < m; i += nt) pv += p[i] * v[i];
    pv = block_sum(pv, red);
    T alpha = T(-0.5) * tk * pv;
    for (int i = tid; i < m; i += nt) p[i] += alpha * v[i];  // p becomes w
    __syncthreads();
    for (long long idx = tid; idx < (long long)m * m; idx += nt) {
      int i = (int)(idx / m), j = (int)(idx % m);
      A22[(long long)i * n + j] -= v[i] * p[j] + p[i] * v[j];
    }
    // keep v below the subdiagonal of column k
    for (int i = 1 + tid; i < m; i += nt) A[(long long)(k + 1 + i) * n + k] = v[i];
    __syncthreads();
  }
  for (int i = tid; i < n; i += nt) d[i] = A[(long long)i * n + i];
  if (tid == 0) {
    if (n >= 2) e[n - 2] = A[(long long)(n - 1) * n + (n - 2)];
    e[n - 1] = T(0);
    if (n >= 2) tau[n - 2] = T(0);
    tau[n - 1] = T(0);
  }
  __syncthreads();
}

}  // namespace hqcgb
