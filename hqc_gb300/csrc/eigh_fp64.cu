// Symmetric FP64 eigensolver for the SCF (one thread block per matrix).
//
// Stands in for jnp.linalg.eigh in hqc/pbc/solver.py:729,741 and
// hqc/pbc/scf.py:69,138,198 (ascending eigenvalues; eigenvectors equal up to
// sign / degenerate-subspace gauge).  Three stages, all FP64:
//   1. Householder reduction to tridiagonal form (lower variant), the
//      trailing matrix updated with a rank-2 correction per step;
//   2. implicit QL with Wilkinson-type shifts on the tridiagonal; each QL
//      sweep's Givens rotations are computed by one thread and then applied
//      by all threads to the transposed eigenvector matrix (coalesced);
//   3. back-transformation with the stored Householder vectors.
// GB300's FP64 rate makes every O(n^3) stage FP64-bound on one SM; a batch
// of matrices runs one block per SM.
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kEigThreads = 1024;

__global__ void __launch_bounds__(kEigThreads)
    k_eigh_tql(int n, double *__restrict__ Ab, double *__restrict__ Vb, double *__restrict__ wb,
               double *__restrict__ workb, int *__restrict__ status) {
  extern __shared__ double esh[];
  double *d = esh;             // [n]
  double *e = d + n;           // [n]
  double *tau = e + n;         // [n]
  double *v = tau + n;         // [n] current Householder vector
  double *p = v + n;           // [n]
  double *rc = p + n;          // [n] rotation cosines
  double *rs = rc + n;         // [n] rotation sines
  __shared__ double red[32];
  __shared__ int s_int[4];
  __shared__ double s_dbl[4];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double *A = Ab + (long long)blockIdx.x * n * n;
  double *V = Vb + (long long)blockIdx.x * n * n;  // receives eigenvectors (columns)
  double *w = wb + (long long)blockIdx.x * n;
  double *Zt = workb + (long long)blockIdx.x * n * n;  // Zt[c][r] = Z[r][c]
  int fail = 0;

  // ---------------- 1. tridiagonalisation ----------------
  for (int k = 0; k < n - 2; ++k) {
    int m = n - k - 1;
    const double *col = A + (long long)(k + 1) * n + k;  // A[k+1+i][k] = col[i*n]
    double s2 = 0;
    for (int i = 1 + tid; i < m; i += nt) {
      double x = col[(long long)i * n];
      s2 += x * x;
    }
    s2 = block_sum(s2, red);
    if (tid == 0) {
      double x0 = col[0];
      if (s2 == 0.0) {
        tau[k] = 0.0;
        e[k] = x0;
        s_dbl[0] = 0.0;
      } else {
        double beta = -copysign(sqrt(x0 * x0 + s2), x0);
        tau[k] = (beta - x0) / beta;
        e[k] = beta;
        s_dbl[0] = 1.0 / (x0 - beta);
      }
    }
    __syncthreads();
    double tk = tau[k];
    if (tk == 0.0) {
      for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? 1.0 : 0.0;
      __syncthreads();
      continue;
    }
    double sc = s_dbl[0];
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? 1.0 : col[(long long)i * n] * sc;
    __syncthreads();
    // p = tau * A22 v  (one warp per row, coalesced over columns)
    double *A22 = A + (long long)(k + 1) * n + (k + 1);
    for (int i = warp; i < m; i += nw) {
      const double *row = A22 + (long long)i * n;
      double s = 0;
      for (int j = lane; j < m; j += 32) s += row[j] * v[j];
      s = warp_sum(s);
      if (lane == 0) p[i] = tk * s;
    }
    __syncthreads();
    double pv = 0;
    for (int i = tid; i < m; i += nt) pv += p[i] * v[i];
    pv = block_sum(pv, red);
    double alpha = -0.5 * tk * pv;
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
    e[n - 1] = 0.0;
    if (n >= 2) tau[n - 2] = 0.0;
    tau[n - 1] = 0.0;
  }
  // Zt = I
  for (long long idx = tid; idx < (long long)n * n; idx += nt)
    Zt[idx] = ((int)(idx / n) == (int)(idx % n)) ? 1.0 : 0.0;
  __syncthreads();

  // ---------------- 2. implicit QL ----------------
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; ++m) {
          double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= 1e-16 * dd) break;
        }
        int nrot = 0, lo = l;
        if (m != l) {
          if (iter++ >= 60) {
            fail = 1;
            m = l;
          } else {
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + copysign(r, g));
            double s = 1.0, c = 1.0, pp = 0.0;
            int i;
            bool early = false;
            for (i = m - 1; i >= l; --i) {
              double f = s * e[i], b = c * e[i];
              r = hypot(f, g);
              e[i + 1] = r;
              if (r == 0.0) {
                d[i + 1] -= pp;
                e[m] = 0.0;
                early = true;
                break;
              }
              s = f / r;
              c = g / r;
              g = d[i + 1] - pp;
              r = (d[i] - g) * s + 2.0 * c * b;
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
              e[m] = 0.0;
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
        for (int k = tid; k < n; k += nt) {
          double cur = Zt[(long long)m * n + k];
          for (int t = 0; t < nrot; ++t) {
            int i = m - 1 - t;
            double zi = Zt[(long long)i * n + k];
            double c = rc[t], s = rs[t];
            Zt[(long long)(i + 1) * n + k] = s * zi + c * cur;
            cur = c * zi - s * cur;
          }
          Zt[(long long)(m - nrot) * n + k] = cur;
        }
      }
      __syncthreads();
      if (m == l || fail) break;
    }
    if (fail) break;
  }

  // ---------------- 3. back-transformation ----------------
  // Z <- H_k Z for k = n-3 .. 0 on rows k+1..n-1; Zt[c][r] layout.
  for (int k = n - 3; k >= 0 && !fail; --k) {
    __syncthreads();
    int m = n - k - 1;
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? 1.0 : A[(long long)(k + 1 + i) * n + k];
    double tk = tau[k];
    __syncthreads();
    if (tk == 0.0) continue;
    for (int c = warp; c < n; c += nw) {
      const double *zc = Zt + (long long)c * n + (k + 1);
      double s = 0;
      for (int i = lane; i < m; i += 32) s += v[i] * zc[i];
      s = warp_sum(s);
      if (lane == 0) p[c] = tk * s;
    }
    __syncthreads();
    for (long long idx = tid; idx < (long long)n * m; idx += nt) {
      int c = (int)(idx / m), i = (int)(idx % m);
      Zt[(long long)c * n + (k + 1) + i] -= v[i] * p[c];
    }
  }
  __syncthreads();

  // ---------------- 4. sort ascending, write V[r][rank] = Z[r][c] ----------------
  for (int c = tid; c < n; c += nt) {
    double lc = d[c];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      double lj = d[j];
      rank += (lj < lc) || (lj == lc && j < c);
    }
    w[rank] = lc;
    rc[c] = (double)rank;
  }
  __syncthreads();
  for (long long idx = tid; idx < (long long)n * n; idx += nt) {
    int c = (int)(idx / n), r = (int)(idx % n);
    int rank = (int)rc[c];
    V[(long long)r * n + rank] = Zt[idx];
  }
  if (tid == 0) status[blockIdx.x] = fail ? -1 : 0;
}

void eigh_tql(int n, int batch, double *A, double *V, double *w, double *work, int *status,
              cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  size_t smem = (size_t)7 * n * sizeof(double);
  HQ_REQUIRE(smem <= 200 * 1024, "matrix too large for the eigensolver");
  static size_t attr = 0;
  if (smem > attr) {
    HQ_CUDA(cudaFuncSetAttribute(k_eigh_tql, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  k_eigh_tql<<<batch, kEigThreads, smem, st>>>(n, A, V, w, work, status);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
