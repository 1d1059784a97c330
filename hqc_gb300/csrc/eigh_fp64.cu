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
#include "eigh_tridiag.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kEigThreads = 1024;


// T = double: the FP64 solver; T = float: the first stage of the mixed solver.
template <typename T>
__global__ void __launch_bounds__(kEigThreads)
    k_eigh_tql(int n, T *__restrict__ Ab, T *__restrict__ Vb, T *__restrict__ wb,
               T *__restrict__ workb, int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char esh_raw[];
  T *esh = reinterpret_cast<T *>(esh_raw);
  T *d = esh;             // [n]
  T *e = d + n;           // [n]
  T *tau = e + n;         // [n]
  T *v = tau + n;         // [n] current Householder vector
  T *p = v + n;           // [n]
  T *rc = p + n;          // [n] rotation cosines
  T *rs = rc + n;         // [n] rotation sines
  __shared__ T red[32];
  __shared__ int s_int[4];
  __shared__ T s_dbl[4];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  T *A = Ab + (long long)blockIdx.x * n * n;
  T *V = Vb + (long long)blockIdx.x * n * n;  // receives eigenvectors (columns)
  T *w = wb + (long long)blockIdx.x * n;
  T *Zt = workb + (long long)blockIdx.x * n * n;  // Zt[c][r] = Z[r][c]
  int fail = 0;

  // ---------------- 1. tridiagonalisation ----------------
  householder_tridiag<T>(n, A, d, e, tau, v, p, red, s_dbl, nullptr);
  // Zt = I
  for (long long idx = tid; idx < (long long)n * n; idx += nt)
    Zt[idx] = ((int)(idx / n) == (int)(idx % n)) ? T(1) : T(0);
  __syncthreads();

  // ---------------- 2. implicit QL ----------------
  fail = tridiag_ql<T, T>(n, d, e, Zt, rc, rs, s_int);

  // ---------------- 3. back-transformation ----------------
  // Z <- H_k Z for k = n-3 .. 0 on rows k+1..n-1; Zt[c][r] layout.
  for (int k = n - 3; k >= 0 && !fail; --k) {
    __syncthreads();
    int m = n - k - 1;
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? T(1) : A[(long long)(k + 1 + i) * n + k];
    T tk = tau[k];
    __syncthreads();
    if (tk == T(0)) continue;
    for (int c = warp; c < n; c += nw) {
      const T *zc = Zt + (long long)c * n + (k + 1);
      T s = 0;
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
    T lc = d[c];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      T lj = d[j];
      rank += (lj < lc) || (lj == lc && j < c);
    }
    w[rank] = lc;
    rc[c] = (T)rank;
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
  ensure_dyn_smem((const void *)k_eigh_tql<double>, smem);
  k_eigh_tql<double><<<batch, kEigThreads, smem, st>>>(n, A, V, w, work, status);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb

namespace hqcgb {

void eigh_tql_f32(int n, int batch, float *A, float *V, float *w, float *work, int *status,
                  cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  size_t smem = (size_t)7 * n * sizeof(float);
  HQ_REQUIRE(smem <= 200 * 1024, "matrix too large for the eigensolver");
  ensure_dyn_smem((const void *)k_eigh_tql<float>, smem);
  k_eigh_tql<float><<<batch, kEigThreads, smem, st>>>(n, A, V, w, work, status);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
