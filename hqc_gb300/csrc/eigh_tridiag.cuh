// Householder reduction of a symmetric matrix to tridiagonal form (lower
// variant), shared by the FP64 solver and the FP32 stage of the mixed solver,
// and the implicit QL iteration on the tridiagonal, shared with the complex
// Hermitian solver (whose tridiagonal is real).
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

__device__ inline double e_hypot(double a, double b) { return hypot(a, b); }
__device__ inline float e_hypot(float a, float b) { return hypotf(a, b); }
template <typename T> struct EigEps;
template <> struct EigEps<double> { static constexpr double v = 1e-16; };
template <> struct EigEps<float> { static constexpr float v = 6e-8f; };

// a x + b y for a real scalar pair and a real or complex element
__device__ inline double lin2(double a, double x, double b, double y) { return a * x + b * y; }
__device__ inline float lin2(float a, float x, float b, float y) { return a * x + b * y; }
__device__ inline double2 lin2(double a, double2 x, double b, double2 y) {
  return make_double2(a * x.x + b * y.x, a * x.y + b * y.y);
}

// Implicit QL with Wilkinson-type shifts on the tridiagonal (d, e), one
// block.  Each sweep's Givens rotations are computed by thread 0 (rc, rs:
// shared, n each) and applied by all threads to the transposed eigenvector
// matrix Zt[c][r] (E = T, or double2 for complex eigenvectors with a real
// tridiagonal).  Returns nonzero when a sweep limit was hit.
template <typename T, typename E>
__device__ int tridiag_ql(int n, T *__restrict__ d, T *__restrict__ e, E *__restrict__ Zt,
                          T *__restrict__ rc, T *__restrict__ rs, int *s_int) {
  const int tid = threadIdx.x, nt = blockDim.x;
  int fail = 0;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; ++m) {
          T dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= EigEps<T>::v * dd) break;
        }
        int nrot = 0, lo = l;
        if (m != l) {
          if (iter++ >= 60) {
            fail = 1;
            m = l;
          } else {
            T g = (d[l + 1] - d[l]) / (T(2) * e[l]);
            T r = e_hypot(g, T(1));
            g = d[m] - d[l] + e[l] / (g + e_copysign(r, g));
            T s = T(1), c = T(1), pp = T(0);
            int i;
            bool early = false;
            for (i = m - 1; i >= l; --i) {
              T f = s * e[i], b = c * e[i];
              r = e_hypot(f, g);
              e[i + 1] = r;
              if (r == T(0)) {
                d[i + 1] -= pp;
                e[m] = T(0);
                early = true;
                break;
              }
              s = f / r;
              c = g / r;
              g = d[i + 1] - pp;
              r = (d[i] - g) * s + T(2) * c * b;
              pp = s * r;
              d[i + 1] = g + pp;
              g = c * r - b;
              rc[nrot] = c;
              rs[nrot] = s;
              ++nrot;
            }
            lo = early ? i + 1 : l;
            if (!early) {
              d[l] -= pp;
              e[l] = g;
              e[m] = T(0);
            }
          }
        }
        s_int[0] = m;
        s_int[1] = nrot;
        s_int[2] = lo;
        s_int[3] = fail;
      }
      __syncthreads();
      int m = s_int[0], nrot = s_int[1];
      fail = s_int[3];
      // apply the rotations of this sweep: rotation t acts on columns
      // (i, i+1) with i = m-1-t; thread k owns row k of Z
      if (nrot > 0) {
        // batches of RB rotations: the RB loads of a batch are independent
        // and issued together; the carried element stays in a register
        constexpr int RB = sizeof(E) == 4 ? 32 : 16;
        for (int k = tid; k < n; k += nt) {
          E cur = Zt[(long long)m * n + k];
          for (int t0 = 0; t0 < nrot; t0 += RB) {
            E z[RB];
#pragma unroll
            for (int u = 0; u < RB; ++u)
              if (t0 + u < nrot) z[u] = Zt[(long long)(m - 1 - t0 - u) * n + k];
#pragma unroll
            for (int u = 0; u < RB; ++u) {
              if (t0 + u < nrot) {
                int i = m - 1 - t0 - u;
                T c = rc[t0 + u], s = rs[t0 + u];
                Zt[(long long)(i + 1) * n + k] = lin2(s, z[u], c, cur);
                cur = lin2(c, z[u], -s, cur);
              }
            }
          }
          Zt[(long long)(m - nrot) * n + k] = cur;
        }
      }
      __syncthreads();
      if (m == l || fail) break;
    }
    if (fail) break;
  }
  return fail;
}

}  // namespace hqcgb
