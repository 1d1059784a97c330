// FP32 stage of the mixed-precision eigensolver: eigenpairs of a symmetric
// n x n matrix to single precision, for the FP64 refinement in
// eigh_mixed.cu.  Three kernels:
//
//  1. k_tridiag_f32 (one block): Householder reduction to tridiagonal
//     T = Q^T A Q (eigh_tridiag.cuh), reflectors stored contiguously.
//  2. k_tri_eig_f32 (one block, a thread per eigenvalue): the eigenvalues of
//     T by bisection on Sturm counts (W. Barth, R. S. Martin, J. H.
//     Wilkinson, "Calculation of the eigenvalues of a symmetric tridiagonal
//     matrix by the method of bisection", Numer. Math. 9 (1967) 386-393), all
//     in parallel; then the eigenvectors of T by inverse iteration with a
//     partial-pivoting LU of T - lambda I (J. H. Wilkinson, "The Algebraic
//     Eigenvalue Problem", 1965, ch. 5), eigenvalues closer than 1e-4 ||T||
//     treated as a cluster whose vectors one thread computes in turn,
//     orthogonalising each against the earlier ones (modified Gram-Schmidt).
//  3. k_backtransform_f32 (a block per 32 columns): V = Q Z, the reflectors
//     applied in reverse order to column tiles held in shared memory.
//
// The serial QL sweep of the FP64 solver (thousands of dependent Givens
// rotations generated by one thread) is replaced by work that is parallel
// over eigenvalues; the FP64 refinement then fixes what single precision
// leaves (inaccurate vectors within clusters included).
#include <cfloat>

#include "common.cuh"
#include "eigh_tridiag.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kTriThreads = 1024;

__global__ void __launch_bounds__(kTriThreads)
    k_tridiag_f32(int n, float *__restrict__ A, float *__restrict__ dg, float *__restrict__ eg,
                  float *__restrict__ taug, float *__restrict__ hv) {
  extern __shared__ __align__(16) float tsh[];
  float *d = tsh, *e = d + n, *tau = e + n, *v = tau + n, *p = v + n;
  __shared__ float red[32];
  __shared__ float s_dbl[4];
  householder_tridiag<float>(n, A, d, e, tau, v, p, red, s_dbl, hv);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    dg[i] = d[i];
    eg[i] = e[i];
    taug[i] = tau[i];
  }
}

// number of eigenvalues of the tridiagonal (d, e2 = e^2) below x
__device__ inline int sturm_count(int n, const float *__restrict__ d, const float *__restrict__ e2,
                                  float x, float pivmin) {
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  int c = q < 0.f;
  for (int k = 1; k < n; ++k) {
    q = (d[k] - x) - e2[k - 1] / q;
    if (fabsf(q) < pivmin) q = -pivmin;
    c += q < 0.f;
  }
  return c;
}

// Eigenpairs of the tridiagonal (d, e): w ascending, Z[r][c] column c the
// eigenvector of w[c].  scr: 6 n floats per cluster leader (LU and vector).
__global__ void __launch_bounds__(kTriThreads)
    k_tri_eig_f32(int n, const float *__restrict__ dg, const float *__restrict__ eg,
                  float *__restrict__ w, float *__restrict__ Z, float *__restrict__ scr) {
  extern __shared__ __align__(16) float ssh[];
  float *d = ssh, *e = d + n, *e2 = e + n, *lam = e2 + n;
  __shared__ float red[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  float lo = FLT_MAX, hi = -FLT_MAX, emax2 = 0.f;
  for (int i = tid; i < n; i += nt) {
    d[i] = dg[i];
    e[i] = i < n - 1 ? eg[i] : 0.f;
    e2[i] = e[i] * e[i];
    float r = (i > 0 ? fabsf(eg[i - 1]) : 0.f) + (i < n - 1 ? fabsf(eg[i]) : 0.f);
    lo = fminf(lo, dg[i] - r);
    hi = fmaxf(hi, dg[i] + r);
    emax2 = fmaxf(emax2, e2[i]);
  }
  lo = -block_max(-lo, red);
  hi = block_max(hi, red);
  emax2 = block_max(emax2, red);
  const float tnorm = fmaxf(fabsf(lo), fabsf(hi));
  const float pivmin = FLT_MIN * fmaxf(1.f, emax2);
  // widen the Gershgorin interval so that both ends are strict bounds
  const float pad = 2.f * FLT_EPSILON * tnorm + 4.f * pivmin;
  lo -= pad;
  hi += pad;

  // --- eigenvalue i by bisection: count(lo) <= i < count(hi)
  for (int i = tid; i < n; i += nt) {
    float a = lo, b = hi;
    for (int it = 0; it < 80; ++it) {
      float mid = 0.5f * (a + b);
      if (mid <= a || mid >= b) break;
      if (b - a <= 2.f * FLT_EPSILON * fmaxf(fabsf(a), fabsf(b)) + pivmin) break;
      if (sturm_count(n, d, e2, mid, pivmin) <= i) a = mid;
      else b = mid;
    }
    lam[i] = 0.5f * (a + b);
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) w[i] = lam[i];

  // --- eigenvectors by inverse iteration; the first member of each cluster
  // computes the cluster's vectors in order
  // clusters: eigenvalues within 1e-4 ||T||; vectors of eigenvalues further
  // apart are orthogonal to FP32 eps ||T|| / gap <= 1e-3, which the FP64
  // refinement removes
  const float sep = 1e-4f * tnorm;
  const float tiny = FLT_EPSILON * tnorm + pivmin;
  for (int i0 = tid; i0 < n; i0 += nt) {
    if (i0 > 0 && lam[i0] - lam[i0 - 1] <= sep) continue;
    int i1 = i0;
    while (i1 + 1 < n && lam[i1 + 1] - lam[i1] <= sep) ++i1;
    float *u1 = scr + (long long)i0 * 6 * n, *u2 = u1 + n, *u3 = u2 + n, *lm = u3 + n,
          *pv = lm + n, *x = pv + n;
    float shift_prev = 0.f;
    for (int j = i0; j <= i1; ++j) {
      // equal eigenvalues in a cluster are separated a little so that the
      // solves differ (the Gram-Schmidt step makes the vectors orthogonal)
      float lj = lam[j];
      if (j > i0 && lj - shift_prev < 10.f * tiny) lj = shift_prev + 10.f * tiny;
      shift_prev = lj;
      // LU with partial pivoting of T - lj I (rows k, k+1 swapped when the
      // subdiagonal entry is the larger pivot); U has two superdiagonals
      float b = d[0] - lj, c = n > 1 ? e[0] : 0.f;
      for (int k = 0; k < n - 1; ++k) {
        const float a = e[k], bn = d[k + 1] - lj, cn = k + 1 < n - 1 ? e[k + 1] : 0.f;
        if (fabsf(b) >= fabsf(a)) {
          if (b == 0.f) b = tiny;
          const float l = a / b;
          u1[k] = b; u2[k] = c; u3[k] = 0.f; lm[k] = l; pv[k] = 0.f;
          b = bn - l * c;
          c = cn;
        } else {
          const float l = b / a;
          u1[k] = a; u2[k] = bn; u3[k] = cn; lm[k] = l; pv[k] = 1.f;
          b = c - l * bn;
          c = -l * cn;
        }
      }
      u1[n - 1] = fabsf(b) < tiny ? (b < 0.f ? -tiny : tiny) : b;
      for (int k = 0; k < n - 1; ++k)
        if (fabsf(u1[k]) < tiny) u1[k] = u1[k] < 0.f ? -tiny : tiny;
      // start vector: deterministic, not orthogonal to any eigenvector in practice
      for (int k = 0; k < n; ++k) x[k] = 1.f + 0.37f * __sinf(0.7f * (float)k + 1.3f * (float)j);
      for (int it = 0; it < 3; ++it) {
        // L y = P x
        for (int k = 0; k < n - 1; ++k) {
          if (pv[k] != 0.f) {
            float t = x[k];
            x[k] = x[k + 1];
            x[k + 1] = t;
          }
          x[k + 1] -= lm[k] * x[k];
        }
        // U z = y
        x[n - 1] /= u1[n - 1];
        if (n > 1) x[n - 2] = (x[n - 2] - u2[n - 2] * x[n - 1]) / u1[n - 2];
        for (int k = n - 3; k >= 0; --k)
          x[k] = (x[k] - u2[k] * x[k + 1] - u3[k] * x[k + 2]) / u1[k];
        // orthogonalise against the cluster's earlier vectors, normalise
        for (int q = i0; q < j; ++q) {
          float s = 0.f;
          for (int k = 0; k < n; ++k) s += Z[(long long)k * n + q] * x[k];
          for (int k = 0; k < n; ++k) x[k] -= s * Z[(long long)k * n + q];
        }
        float nrm = 0.f;
        for (int k = 0; k < n; ++k) nrm += x[k] * x[k];
        nrm = nrm > 0.f ? rsqrtf(nrm) : 0.f;
        for (int k = 0; k < n; ++k) x[k] *= nrm;
      }
      for (int k = 0; k < n; ++k) Z[(long long)k * n + j] = x[k];
    }
  }
}

// V = Q Z for 32 columns per block: Z tile in shared memory, reflectors
// H_k = I - tau_k v_k v_k^T (rows k+1..n-1) applied for k = n-3 .. 0; eight
// threads (one warp quarter) own a column.
__global__ void __launch_bounds__(256)
    k_backtransform_f32(int n, const float *__restrict__ hv, const float *__restrict__ tau,
                        const float *__restrict__ Z, float *__restrict__ V) {
  extern __shared__ __align__(16) float zt[];  // [n][33]
  const int c0 = blockIdx.x * 32;
  const int tid = threadIdx.x, cc = tid >> 3, part = tid & 7;
  for (int idx = tid; idx < n * 32; idx += blockDim.x) {
    int r = idx >> 5, c = idx & 31;
    zt[r * 33 + c] = (c0 + c < n) ? Z[(long long)r * n + c0 + c] : 0.f;
  }
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const float tk = tau[k];
    if (tk == 0.f) continue;
    const int m = n - k - 1;
    const float *vk = hv + (long long)k * n;
    float s = 0.f;
    for (int i = part; i < m; i += 8) s += vk[i] * zt[(k + 1 + i) * 33 + cc];
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    s += __shfl_xor_sync(0xffffffffu, s, 4);
    s *= tk;
    for (int i = part; i < m; i += 8) zt[(k + 1 + i) * 33 + cc] -= s * vk[i];
    __syncwarp();
  }
  __syncthreads();
  for (int idx = tid; idx < n * 32; idx += blockDim.x) {
    int r = idx >> 5, c = idx & 31;
    if (c0 + c < n) V[(long long)r * n + c0 + c] = zt[r * 33 + c];
  }
}

size_t eigh_f32_scratch_floats(int n) { return (size_t)6 * n * n + (size_t)n * n + 4 * (size_t)n; }

// A (n x n, destroyed) -> w ascending, V columns.  scr: eigh_f32_scratch_floats(n).
void eigh_f32(int n, float *A, float *V, float *w, float *scr, cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  float *lu = scr, *hv = lu + (size_t)6 * n * n, *dg = hv + (size_t)n * n, *eg = dg + n,
        *taug = eg + n;
  size_t sm1 = (size_t)5 * n * sizeof(float);
  size_t sm2 = (size_t)4 * n * sizeof(float);
  size_t sm3 = (size_t)n * 33 * sizeof(float);
  HQ_REQUIRE(sm3 <= 200 * 1024, "matrix too large for the FP32 eigensolver");
  static size_t attr3 = 0;
  if (sm3 > 48 * 1024 && sm3 > attr3) {
    HQ_CUDA(cudaFuncSetAttribute(k_backtransform_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm3));
    attr3 = sm3;
  }
  k_tridiag_f32<<<1, kTriThreads, sm1, st>>>(n, A, dg, eg, taug, hv);
  HQ_LAUNCH_CHECK();
  // Z (tridiagonal eigenvectors) goes to V, then V = Q Z in place per tile
  k_tri_eig_f32<<<1, kTriThreads, sm2, st>>>(n, dg, eg, w, V, lu);
  HQ_LAUNCH_CHECK();
  k_backtransform_f32<<<ceil_div(n, 32), 256, sm3, st>>>(n, hv, taug, V, V);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
