// FP32 stage of the mixed-precision eigensolver: eigenpairs of a symmetric
// n x n matrix to single precision, for the FP64 refinement in
// eigh_mixed.cu.  Three kernels:
//
//  1. k_tridiag_f32_smem (one block): Householder reduction to tridiagonal
//     T = Q^T A Q with the matrix in shared memory (k_tridiag_f32, the
//     global-memory form of eigh_tridiag.cuh, above 310 AOs), reflectors
//     stored contiguously.
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
#include <cstdio>
#include <cstdlib>

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

// The same reduction with the matrix held in shared memory as a packed lower
// triangle (element (i, j), i >= j, at i (i + 1) / 2 + j): the symmetric
// matrix-vector product and the rank-2 update of each step touch only shared
// memory.  For n with n (n + 1) / 2 + 5 n floats within the shared-memory
// budget (n <= 310).
__device__ inline int tri_ix(int i, int j) { return i * (i + 1) / 2 + j; }

__global__ void __launch_bounds__(kTriThreads)
    k_tridiag_f32_smem(int n, const float *__restrict__ A, float *__restrict__ dg,
                       float *__restrict__ eg, float *__restrict__ taug, float *__restrict__ hv) {
  extern __shared__ __align__(16) float tsh[];
  float *L = tsh, *d = L + n * (n + 1) / 2, *e = d + n, *tau = e + n, *v = tau + n, *p = v + n;
  __shared__ float red[32];
  __shared__ float s_beta[2];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int idx = tid; idx < n * (n + 1) / 2; idx += nt) {
    // row i of the packed triangle: the largest i with i (i + 1) / 2 <= idx
    int i = (int)((sqrtf(8.f * (float)idx + 1.f) - 1.f) * 0.5f);
    while (i * (i + 1) / 2 > idx) --i;
    while ((i + 1) * (i + 2) / 2 <= idx) ++i;
    L[idx] = A[(long long)i * n + (idx - i * (i + 1) / 2)];
  }
  __syncthreads();
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;  // trailing rows k+1 .. n-1
    float s2 = 0.f;
    for (int i = 1 + tid; i < m; i += nt) {
      float x = L[tri_ix(k + 1 + i, k)];
      s2 += x * x;
    }
    s2 = block_sum(s2, red);
    if (tid == 0) {
      const float x0 = L[tri_ix(k + 1, k)];
      if (s2 == 0.f) {
        tau[k] = 0.f;
        e[k] = x0;
        s_beta[0] = 0.f;
      } else {
        const float beta = -copysignf(sqrtf(x0 * x0 + s2), x0);
        tau[k] = (beta - x0) / beta;
        e[k] = beta;
        s_beta[0] = 1.f / (x0 - beta);
      }
    }
    __syncthreads();
    const float tk = tau[k], sc = s_beta[0];
    for (int i = tid; i < m; i += nt) {
      v[i] = (i == 0) ? 1.f : (tk == 0.f ? 0.f : L[tri_ix(k + 1 + i, k)] * sc);
      hv[(long long)k * n + i] = v[i];
    }
    __syncthreads();
    if (tk == 0.f) continue;
    // p = tau A22 v, one warp per row i: sum over j <= i of L[i][j] v_j and
    // over j > i of L[j][i] v_j (trailing block indices)
    for (int i = warp; i < m; i += nw) {
      const int gi = k + 1 + i;
      float sum = 0.f;
      for (int j = lane; j < m; j += 32) {
        const int gj = k + 1 + j;
        sum += (j <= i ? L[tri_ix(gi, gj)] : L[tri_ix(gj, gi)]) * v[j];
      }
      sum = warp_sum(sum);
      if (lane == 0) p[i] = tk * sum;
    }
    __syncthreads();
    float pv = 0.f;
    for (int i = tid; i < m; i += nt) pv += p[i] * v[i];
    pv = block_sum(pv, red);
    const float alpha = -0.5f * tk * pv;
    for (int i = tid; i < m; i += nt) p[i] += alpha * v[i];  // p becomes w
    __syncthreads();
    // rank-2 update of the trailing lower triangle
    const int tri = m * (m + 1) / 2;
    for (int idx = tid; idx < tri; idx += nt) {
      int i = (int)((sqrtf(8.f * (float)idx + 1.f) - 1.f) * 0.5f);
      while (i * (i + 1) / 2 > idx) --i;
      while ((i + 1) * (i + 2) / 2 <= idx) ++i;
      const int j = idx - i * (i + 1) / 2;
      L[tri_ix(k + 1 + i, k + 1 + j)] -= v[i] * p[j] + p[i] * v[j];
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += nt) {
    dg[i] = L[tri_ix(i, i)];
    eg[i] = i < n - 2 ? e[i] : (i == n - 2 ? L[tri_ix(n - 1, n - 2)] : 0.f);
    taug[i] = i < n - 2 ? tau[i] : 0.f;
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
// eigenvector of w[c].  scr: 6 n x n floats (LU factors and the vector of
// each cluster leader, interleaved by leader).
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
    // per-leader arrays interleaved by leader (element k of leader i0 at
    // k * n + i0): the leaders step through k together, so a warp's accesses
    // are one coalesced line instead of 32 scattered ones
    float *u1 = scr + i0, *u2 = u1 + (long long)n * n, *u3 = u2 + (long long)n * n,
          *lm = u3 + (long long)n * n, *pv = lm + (long long)n * n, *x = pv + (long long)n * n;
#define U1(k) u1[(long long)(k) * n]
#define U2(k) u2[(long long)(k) * n]
#define U3(k) u3[(long long)(k) * n]
#define LM(k) lm[(long long)(k) * n]
#define PV(k) pv[(long long)(k) * n]
#define XX(k) x[(long long)(k) * n]
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
          U1(k) = b; U2(k) = c; U3(k) = 0.f; LM(k) = l; PV(k) = 0.f;
          b = bn - l * c;
          c = cn;
        } else {
          const float l = b / a;
          U1(k) = a; U2(k) = bn; U3(k) = cn; LM(k) = l; PV(k) = 1.f;
          b = c - l * bn;
          c = -l * cn;
        }
      }
      U1(n - 1) = fabsf(b) < tiny ? (b < 0.f ? -tiny : tiny) : b;
      for (int k = 0; k < n - 1; ++k)
        if (fabsf(U1(k)) < tiny) U1(k) = U1(k) < 0.f ? -tiny : tiny;
      // start vector: deterministic, not orthogonal to any eigenvector in practice
      for (int k = 0; k < n; ++k) XX(k) = 1.f + 0.37f * __sinf(0.7f * (float)k + 1.3f * (float)j);
      for (int it = 0; it < 3; ++it) {
        // L y = P x
        for (int k = 0; k < n - 1; ++k) {
          if (PV(k) != 0.f) {
            float t = XX(k);
            XX(k) = XX(k + 1);
            XX(k + 1) = t;
          }
          XX(k + 1) -= LM(k) * XX(k);
        }
        // U z = y
        XX(n - 1) /= U1(n - 1);
        if (n > 1) XX(n - 2) = (XX(n - 2) - U2(n - 2) * XX(n - 1)) / U1(n - 2);
        for (int k = n - 3; k >= 0; --k)
          XX(k) = (XX(k) - U2(k) * XX(k + 1) - U3(k) * XX(k + 2)) / U1(k);
        // orthogonalise against the cluster's earlier vectors, normalise
        for (int q = i0; q < j; ++q) {
          float s = 0.f;
          for (int k = 0; k < n; ++k) s += Z[(long long)k * n + q] * XX(k);
          for (int k = 0; k < n; ++k) XX(k) -= s * Z[(long long)k * n + q];
        }
        float nrm = 0.f;
        for (int k = 0; k < n; ++k) nrm += XX(k) * XX(k);
        nrm = nrm > 0.f ? rsqrtf(nrm) : 0.f;
        for (int k = 0; k < n; ++k) XX(k) *= nrm;
      }
      for (int k = 0; k < n; ++k) Z[(long long)k * n + j] = XX(k);
    }
#undef U1
#undef U2
#undef U3
#undef LM
#undef PV
#undef XX
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
  ensure_dyn_smem((const void *)k_backtransform_f32, sm3);
  const bool tr = std::getenv("HQCGB_TRACE") != nullptr;
  cudaEvent_t ev[4];
  if (tr)
    for (auto &x : ev) cudaEventCreate(&x);
  if (tr) cudaEventRecord(ev[0], st);
  const size_t smt = ((size_t)n * (n + 1) / 2 + 5 * (size_t)n) * sizeof(float);
  if (smt <= 200 * 1024) {
    ensure_dyn_smem((const void *)k_tridiag_f32_smem, smt);
    k_tridiag_f32_smem<<<1, kTriThreads, smt, st>>>(n, A, dg, eg, taug, hv);
  } else {
    k_tridiag_f32<<<1, kTriThreads, sm1, st>>>(n, A, dg, eg, taug, hv);
  }
  HQ_LAUNCH_CHECK();
  if (tr) cudaEventRecord(ev[1], st);
  // Z (tridiagonal eigenvectors) goes to V, then V = Q Z in place per tile
  k_tri_eig_f32<<<1, kTriThreads, sm2, st>>>(n, dg, eg, w, V, lu);
  HQ_LAUNCH_CHECK();
  if (tr) cudaEventRecord(ev[2], st);
  k_backtransform_f32<<<ceil_div(n, 32), 256, sm3, st>>>(n, hv, taug, V, V);
  HQ_LAUNCH_CHECK();
  if (tr) {
    cudaEventRecord(ev[3], st);
    cudaEventSynchronize(ev[3]);
    float t[3];
    for (int k = 0; k < 3; ++k) cudaEventElapsedTime(&t[k], ev[k], ev[k + 1]);
    fprintf(stderr, "  fp32 tridiag %.3f ms, bisection+inverse iteration %.3f ms, back %.3f ms\n", t[0],
            t[1], t[2]);
    for (auto &x : ev) cudaEventDestroy(x);
  }
}

}  // namespace hqcgb
