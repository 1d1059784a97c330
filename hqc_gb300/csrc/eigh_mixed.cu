// Mixed-precision symmetric eigensolver of the mixed SCF path.
//
// Stage 1 (FP32, one thread block): Householder tridiagonalisation, implicit
// QL and back-transformation -- the FP64 algorithm of eigh_fp64.cu run in
// FP32, 30-60x cheaper per operation on GB300.
// Stage 2 (FP64): two iterations of the Ogita-Aishima refinement
// (T. Ogita, K. Aishima, "Iterative refinement for symmetric eigenvalue
// decomposition", Japan J. Indust. Appl. Math. 35 (2018) 1007-1035):
//   R = I - X^T X,  S = X^T A X,  l_i = s_ii / (1 - r_ii),
//   E_ij = (s_ij + l_j r_ij) / (l_j - l_i)   for |l_i - l_j| > delta,
//   E_ij = r_ij / 2                            otherwise,
//   X <- X + X E,
// with delta = 2 (||S - diag(l)|| + ||A|| ||R||) (Frobenius norms).  Each
// iteration squares the error, so FP32-accurate vectors become FP64-accurate
// after two; all of it is FP64 GEMM work spread over many SMs.  The result
// stands in for jnp.linalg.eigh (hqc/pbc/scf.py:69,138,198).
#include <cstdlib>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

__global__ void k_f64_to_f32(long long n, const double *__restrict__ a, float *__restrict__ b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void k_f32_to_f64(long long n, const float *__restrict__ a, double *__restrict__ b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// One block: lambda, delta and the correction E from S and G = X^T X.
__global__ void __launch_bounds__(1024) k_oa_correction(int n, const double *__restrict__ A,
                                                        const double *__restrict__ S,
                                                        const double *__restrict__ G,
                                                        double *__restrict__ E,
                                                        double *__restrict__ lam,
                                                        double *__restrict__ emax) {
  __shared__ double red[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long nn = (long long)n * n;
  for (int i = tid; i < n; i += nt) lam[i] = S[(long long)i * n + i] / (G[(long long)i * n + i]);
  __syncthreads();
  double a2 = 0, s2 = 0, r2 = 0;
  for (long long k = tid; k < nn; k += nt) {
    int i = (int)(k / n), j = (int)(k % n);
    double a = A[k];
    a2 += a * a;
    double r = (i == j ? 1.0 : 0.0) - G[k];
    r2 += r * r;
    double sd = S[k] - (i == j ? lam[i] : 0.0);
    s2 += sd * sd;
  }
  a2 = block_sum(a2, red);
  s2 = block_sum(s2, red);
  r2 = block_sum(r2, red);
  double delta = 2.0 * (sqrt(s2) + sqrt(a2) * sqrt(r2));
  if (tid == 0 && emax) emax[1] = sqrt(s2) / fmax(sqrt(a2), 1e-300);  // relative off-diagonal
  double em = 0;
  for (long long k = tid; k < nn; k += nt) {
    int i = (int)(k / n), j = (int)(k % n);
    double r = (i == j ? 1.0 : 0.0) - G[k];
    double e;
    if (i != j && fabs(lam[i] - lam[j]) > delta) e = (S[k] + lam[j] * r) / (lam[j] - lam[i]);
    else e = 0.5 * r;
    E[k] = e;
    em = fmax(em, fabs(e));
  }
  // block max through the sum helper's shared buffer
  __shared__ double mx[32];
  for (int o = 16; o > 0; o >>= 1) em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
  if ((tid & 31) == 0) mx[tid >> 5] = em;
  __syncthreads();
  if (tid < 32) {
    em = (tid < (nt >> 5)) ? mx[tid] : 0.0;
    for (int o = 16; o > 0; o >>= 1) em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
    if (tid == 0 && emax) *emax = em;
  }
}

// Sort eigenpairs ascending (stable): w, and the columns of X via scratch T.
__global__ void __launch_bounds__(1024) k_sort_eigpairs(int n, double *__restrict__ w,
                                                        double *__restrict__ X,
                                                        double *__restrict__ T,
                                                        int *__restrict__ rank) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n; i += nt) {
    double li = w[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      double lj = w[j];
      r += (lj < li) || (lj == li && j < i);
    }
    rank[i] = r;
  }
  __syncthreads();
  for (long long k = tid; k < (long long)n * n; k += nt) {
    int row = (int)(k / n), col = (int)(k % n);
    T[(long long)row * n + rank[col]] = X[k];
  }
  __syncthreads();
  for (long long k = tid; k < (long long)n * n; k += nt) X[k] = T[k];
  __syncthreads();
  for (int i = tid; i < n; i += nt) T[rank[i]] = w[i];
  __syncthreads();
  for (int i = tid; i < n; i += nt) w[i] = T[i];
}

static void sort_eigpairs(int n, double *w, double *X, MixedEigWork &ws, cudaStream_t st) {
  k_sort_eigpairs<<<1, 1024, 0, st>>>(n, w, X, ws.T1, reinterpret_cast<int *>(ws.E));
  HQ_LAUNCH_CHECK();
}

static double oa_iteration(int n, const double *A, double *X, double *w, MixedEigWork &ws,
                           cudaStream_t st) {
  gemm(false, false, n, n, n, 1.0, A, n, X, n, nullptr, 0.0, ws.T1, n, st);    // A X
  gemm(true, false, n, n, n, 1.0, X, n, ws.T1, n, nullptr, 0.0, ws.S, n, st);  // X^T A X
  gemm(true, false, n, n, n, 1.0, X, n, X, n, nullptr, 0.0, ws.G, n, st);      // X^T X
  k_oa_correction<<<1, 1024, 0, st>>>(n, A, ws.S, ws.G, ws.E, w, ws.emax);
  HQ_LAUNCH_CHECK();
  gemm(false, false, n, n, n, 1.0, X, n, ws.E, n, nullptr, 0.0, ws.T1, n, st);  // X E
  axpby(n, 1.0, X, 1.0, ws.T1, false, X, st);                                  // X += X E
  double em[2] = {0, 0};
  HQ_CUDA(cudaMemcpyAsync(em, ws.emax, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  HQ_CUDA(cudaStreamSynchronize(st));
  return em[1];  // relative off-diagonal norm of X^T A X before this update
}

// Full solve: FP32 stage + two refinements.
void eigh_mixed(int n, const double *A, double *V, double *w, MixedEigWork &ws, cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  long long nn = (long long)n * n;
  k_f64_to_f32<<<ceil_div(nn, 256), 256, 0, st>>>(nn, A, ws.A32);
  HQ_LAUNCH_CHECK();
  eigh_tql_f32(n, 1, ws.A32, ws.V32, ws.w32, ws.work32, ws.status, st);
  k_f32_to_f64<<<ceil_div(nn, 256), 256, 0, st>>>(nn, ws.V32, V);
  HQ_LAUNCH_CHECK();
  for (int it = 0; it < 2; ++it) oa_iteration(n, A, V, w, ws, st);
  sort_eigpairs(n, w, V, ws, st);
}

// Warm start from eigenvectors X0 of a nearby matrix (the previous SCF
// iteration's Fock matrix): refinement only, while its corrections shrink
// quadratically.  Returns false (V untouched semantics not guaranteed) when
// the start is too far, so the caller runs the full solve.
bool eigh_mixed_warm(int n, const double *A, const double *X0, double *V, double *w,
                     MixedEigWork &ws, cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  HQ_CUDA(cudaMemcpyAsync(V, X0, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st));
  // off = ||X^T A X - diag|| / ||A|| of the start; the refinement converges
  // quadratically only when the start is close, so far starts fall back.
  double prev = 1e300;
  for (int it = 0; it < 6; ++it) {
    double off = oa_iteration(n, A, V, w, ws, st);
    if (std::getenv("HQCGB_TRACE")) fprintf(stderr, "  warm it %d off=%.3e\n", it, off);
    if (!(off < 2e-3) || (it > 0 && off > 0.25 * prev && off > 1e-12)) return false;
    if (off < 1e-11) {  // this update took it to rounding level
      sort_eigpairs(n, w, V, ws, st);
      return true;
    }
    prev = off;
  }
  return false;
}

}  // namespace hqcgb
