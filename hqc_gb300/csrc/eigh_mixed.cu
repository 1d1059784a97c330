// Mixed-precision symmetric eigensolver of the mixed SCF path.
//
// Stage 1 (FP32, eigh_f32.cu): Householder tridiagonalisation, bisection and
// inverse iteration on the tridiagonal, back-transformation -- single
// precision is 30-60x cheaper per operation than FP64 on GB300.
// Stage 2 (FP64): Ogita-Aishima refinement
// (T. Ogita, K. Aishima, "Iterative refinement for symmetric eigenvalue
// decomposition", Japan J. Indust. Appl. Math. 35 (2018) 1007-1035):
//   R = I - X^T X,  S = X^T A X,  l_i = s_ii / (1 - r_ii),
//   E_ij = (s_ij + l_j r_ij) / (l_j - l_i)   for |l_i - l_j| > delta,
//   E_ij = r_ij / 2                            otherwise,
//   X <- X + X E,
// with delta = 2 (||S - diag(l)|| + ||A|| ||R||) (Frobenius norms), and the
// clustered-eigenvalue extension of the same authors (below).  Each iteration
// squares the error, so FP32-accurate vectors become FP64-accurate after two
// or three; all of it is FP64 GEMM work spread over many SMs.  The result
// stands in for jnp.linalg.eigh (hqc/pbc/scf.py:69,138,198).
#include <algorithm>
#include <chrono>
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

// One block: lambda, delta, the clusters and the correction E from
// S = X^T A X and G = X^T X.
//
// Clusters (Ogita, Aishima, "Iterative refinement for symmetric eigenvalue
// decomposition II: clustered eigenvalues", Japan J. Indust. Appl. Math. 36
// (2019) 435-459): eigenvalue estimates closer than delta form a cluster,
// within which the basic update only re-orthogonalises.  Each cluster C is
// therefore rotated first by the eigenvectors W_C of its block S_CC (cyclic
// Jacobi, one thread per cluster): X_C <- X_C W_C, S <- W^T S W and
// G <- W^T G W, after which the cluster's Ritz values are separated and the
// next iteration converges quadratically again.  Clusters larger than
// kMaxCluster are left unrotated and flagged in emax[2].
// emax[0] = max |E|, emax[1] = ||S - diag(l)||_F / ||A||_F before the
// update, emax[2] = 1 when a cluster was too large, emax[3] = cluster count.
constexpr int kMaxCluster = 48;      // largest cluster rotated (wide spectra)
constexpr int kMaxClusterFock = 12;  // ... for Fock matrices (keeps the pass short)
constexpr int kShCluster = 12;       // clusters up to this size rotate in shared memory
constexpr int kOaThreads = 256;
constexpr int kOaJacobiThreads = 16;  // clusters rotated with their blocks in shared memory

// non-negative doubles compare like their bit patterns
__device__ inline void atomic_max_nonneg(double *a, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(a), (unsigned long long)__double_as_longlong(v));
}

// Pass 1 (grid): ||A||_F^2, ||S - diag(l)||_F^2, ||R||_F^2 and the largest
// coupling max_{i != j} |s_ij - l_j g_ij| into red[0..3] (zeroed by the host).
__global__ void __launch_bounds__(kOaThreads) k_oa_stats(int n, const double *__restrict__ A,
                                                         const double *__restrict__ S,
                                                         const double *__restrict__ G,
                                                         double *__restrict__ red) {
  __shared__ double sh[32];
  const long long nn = (long long)n * n;
  double a2 = 0, s2 = 0, r2 = 0, cm = 0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nn;
       k += (long long)gridDim.x * blockDim.x) {
    int i = (int)(k / n), j = (int)(k % n);
    double a = A[k];
    a2 += a * a;
    double g = G[k], r = (i == j ? 1.0 : 0.0) - g;
    r2 += r * r;
    double lj = S[(long long)j * n + j] / G[(long long)j * n + j];
    if (i == j) continue;
    double sv = S[k];
    s2 += sv * sv;
    cm = fmax(cm, fabs(sv - lj * g));
  }
  a2 = block_sum(a2, sh);
  s2 = block_sum(s2, sh);
  r2 = block_sum(r2, sh);
  cm = block_max(cm, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&red[0], a2);
    atomicAdd(&red[1], s2);
    atomicAdd(&red[2], r2);
    atomic_max_nonneg(&red[3], cm);
  }
}

// Pass 2 (one block): estimates, separation, clusters and the Jacobi
// rotations W_C of the cluster blocks.
//
// Clusters (Ogita, Aishima, "Iterative refinement for symmetric eigenvalue
// decomposition II: clustered eigenvalues", Japan J. Indust. Appl. Math. 36
// (2019) 435-459): estimates closer than delta form a cluster, within which
// the basic update only re-orthogonalises.  Each cluster C is rotated first
// by the eigenvectors W_C of its block S_CC (cyclic Jacobi, one thread per
// cluster): X_C <- X_C W_C, S <- W^T S W and G <- W^T G W (passes 3 and 4),
// after which the cluster's Ritz values are separated and the iteration
// converges quadratically again.  Clusters larger than kMaxCluster are left
// unrotated and flagged.
// Outputs: emax[1] = ||S - diag(l)||_F / ||A||_F, emax[2] = 1 when a cluster
// was too large, emax[3] = cluster count, emax[4] = delta; iwork = order,
// cluster id, cluster start / size / wbuf offset, then the count at 5n.
__global__ void __launch_bounds__(1024) k_oa_clusters(int n, const double *__restrict__ S,
                                                      const double *__restrict__ G,
                                                      const double *__restrict__ red,
                                                      double *__restrict__ lam,
                                                      double *__restrict__ emax,
                                                      int *__restrict__ iwork,
                                                      double *__restrict__ wbuf, int max_cluster) {
  __shared__ int s_nclus;
  const int tid = threadIdx.x, nt = blockDim.x;
  int *order = iwork, *cid = iwork + n, *cstart = iwork + 2 * n, *csize = iwork + 3 * n,
      *coff = iwork + 4 * n;
  for (int i = tid; i < n; i += nt) lam[i] = S[(long long)i * n + i] / G[(long long)i * n + i];
  __syncthreads();
  // off-diagonal part of ||S - diag(l)||: the diagonal of S - diag(l) is
  // s_ii (1 - 1/g_ii), negligible, and is left out
  const double a2 = red[0], s2 = red[1], cmax = red[3];
  // Separation: pairs closer than 10x the largest coupling would get
  // corrections |E_ij| > 0.1, outside the quadratic regime, so they are
  // clustered instead; the floor (1e-6 of the mean eigenvalue scale) keeps
  // pairs that are ill-determined at FP64 rounding in clusters as well.
  // (The paper's bound 2(||S - diag(l)||_F + ||A||_F ||R||_F) is rigorous but
  // lumps whole bands of a 270-AO Fock matrix into one cluster.)
  const double delta = fmax(10.0 * cmax, 1e-6 * sqrt(a2 / n));
  for (int i = tid; i < n; i += nt) {
    double li = lam[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      double lj = lam[j];
      r += (lj < li) || (lj == li && j < i);
    }
    order[r] = i;
  }
  __syncthreads();
  if (tid == 0) {
    int nclus = 0, bad = 0, off = 0;
    for (int i = 0; i < n;) {
      int j = i;
      while (j + 1 < n && lam[order[j + 1]] - lam[order[j]] <= delta) ++j;
      int k = j - i + 1;
      if (k >= 2 && k <= max_cluster) {
        cstart[nclus] = i;
        csize[nclus] = k;
        coff[nclus] = off;
        off += 2 * k * k;
        for (int m = i; m <= j; ++m) cid[order[m]] = nclus;
        ++nclus;
      } else {
        if (k > max_cluster) bad = 1;
        for (int m = i; m <= j; ++m) cid[order[m]] = -1;
      }
      i = j + 1;
    }
    s_nclus = nclus;
    iwork[5 * n] = nclus;
    emax[1] = sqrt(s2) / fmax(sqrt(a2), 1e-300);
    emax[2] = bad;
    emax[3] = nclus;
    emax[4] = delta;
  }
  __syncthreads();
  const int nclus = s_nclus;
  // cyclic Jacobi on each cluster block B = S_CC (in shared memory); W
  // accumulates the rotations and goes to wbuf for the rotation passes
  __shared__ double jb[kOaJacobiThreads][2 * kShCluster * kShCluster];
  for (int c = tid; c < nclus; c += nt) {
    const int k = csize[c], s0 = cstart[c];
    const bool in_sh = tid < kOaJacobiThreads && k <= kShCluster;
    double *B = in_sh ? jb[tid] : wbuf + coff[c];
    double *W = B + k * k;
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < k; ++b) {
        long long ia = order[s0 + a], ib = order[s0 + b];
        B[a * k + b] = 0.5 * (S[ia * n + ib] + S[ib * n + ia]);
        W[a * k + b] = (a == b) ? 1.0 : 0.0;
      }
    for (int sweep = 0; sweep < 40; ++sweep) {
      double offd = 0, diag = 0;
      for (int a = 0; a < k; ++a) {
        diag += B[a * k + a] * B[a * k + a];
        for (int b = a + 1; b < k; ++b) offd += B[a * k + b] * B[a * k + b];
      }
      // rounding level: off-diagonal entries ~1e-15 of the diagonal
      if (offd <= 1e-30 * diag || offd == 0.0) break;
      for (int a = 0; a < k - 1; ++a)
        for (int b = a + 1; b < k; ++b) {
          double bab = B[a * k + b];
          if (bab == 0.0) continue;
          double theta = (B[b * k + b] - B[a * k + a]) / (2.0 * bab);
          double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
          for (int m = 0; m < k; ++m) {  // B <- B J, W <- W J
            double x = B[m * k + a], y = B[m * k + b];
            B[m * k + a] = cs * x - sn * y;
            B[m * k + b] = sn * x + cs * y;
            x = W[m * k + a];
            y = W[m * k + b];
            W[m * k + a] = cs * x - sn * y;
            W[m * k + b] = sn * x + cs * y;
          }
          for (int m = 0; m < k; ++m) {  // B <- J^T B
            double x = B[a * k + m], y = B[b * k + m];
            B[a * k + m] = cs * x - sn * y;
            B[b * k + m] = sn * x + cs * y;
          }
        }
    }
    if (in_sh)
      for (int m = 0; m < k * k; ++m) wbuf[coff[c] + k * k + m] = W[m];
  }
}

// Pass 3 (grid): columns X_C <- X_C W_C, S_:C <- S_:C W_C, G_:C <- G_:C W_C.
__global__ void __launch_bounds__(kOaThreads) k_oa_rotate_cols(int n, double *__restrict__ X,
                                                               double *__restrict__ S,
                                                               double *__restrict__ G,
                                                               const int *__restrict__ iwork,
                                                               const double *__restrict__ wbuf) {
  const int nclus = iwork[5 * n];
  const int *order = iwork, *cstart = iwork + 2 * n, *csize = iwork + 3 * n, *coff = iwork + 4 * n;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < 3LL * n * nclus;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx % n), q = (int)((idx / n) % 3), c = (int)(idx / (3LL * n));
    const int k = csize[c], s0 = cstart[c];
    const double *W = wbuf + coff[c] + k * k;
    double *row = (q == 0 ? X : q == 1 ? S : G) + (long long)r * n;
    double tmp[kMaxCluster];
    for (int j = 0; j < k; ++j) {
      double acc = 0;
      for (int i = 0; i < k; ++i) acc += row[order[s0 + i]] * W[i * k + j];
      tmp[j] = acc;
    }
    for (int j = 0; j < k; ++j) row[order[s0 + j]] = tmp[j];
  }
}

// Pass 4 (grid): rows S_C: <- W_C^T S_C:, G_C: <- W_C^T G_C:.
__global__ void __launch_bounds__(kOaThreads) k_oa_rotate_rows(int n, double *__restrict__ S,
                                                               double *__restrict__ G,
                                                               const int *__restrict__ iwork,
                                                               const double *__restrict__ wbuf) {
  const int nclus = iwork[5 * n];
  const int *order = iwork, *cstart = iwork + 2 * n, *csize = iwork + 3 * n, *coff = iwork + 4 * n;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < 2LL * n * nclus;
       idx += (long long)gridDim.x * blockDim.x) {
    const int col = (int)(idx % n), q = (int)((idx / n) % 2), c = (int)(idx / (2LL * n));
    const int k = csize[c], s0 = cstart[c];
    const double *W = wbuf + coff[c] + k * k;
    double *m = q == 0 ? S : G;
    double tmp[kMaxCluster];
    for (int j = 0; j < k; ++j) {
      double acc = 0;
      for (int i = 0; i < k; ++i) acc += W[i * k + j] * m[(long long)order[s0 + i] * n + col];
      tmp[j] = acc;
    }
    for (int j = 0; j < k; ++j) m[(long long)order[s0 + j] * n + col] = tmp[j];
  }
}

// Pass 5 (grid): l_i = s_ii / g_ii of the rotated S, G and the correction
// E_ij = (s_ij + l_j r_ij) / (l_j - l_i) for separated pairs, r_ij / 2 within
// a cluster or closer than delta; max |E| into red[4] (zeroed by the host).
__global__ void __launch_bounds__(kOaThreads) k_oa_update(int n, const double *__restrict__ S,
                                                          const double *__restrict__ G,
                                                          const int *__restrict__ iwork,
                                                          const double *__restrict__ emax,
                                                          double *__restrict__ lam,
                                                          double *__restrict__ E,
                                                          double *__restrict__ red) {
  extern __shared__ double sl[];  // [n]
  __shared__ double sh[32];
  const int *cid = iwork + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    sl[i] = S[(long long)i * n + i] / G[(long long)i * n + i];
  __syncthreads();
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = sl[i];
  const double delta = emax[4];
  const long long nn = (long long)n * n;
  double em = 0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nn;
       k += (long long)gridDim.x * blockDim.x) {
    int i = (int)(k / n), j = (int)(k % n);
    double r = (i == j ? 1.0 : 0.0) - G[k];
    bool same = cid[i] >= 0 && cid[i] == cid[j];
    double e;
    if (i != j && !same && fabs(sl[i] - sl[j]) > delta) e = (S[k] + sl[j] * r) / (sl[j] - sl[i]);
    else e = 0.5 * r;
    E[k] = e;
    em = fmax(em, fabs(e));
  }
  em = block_max(em, sh);
  if (threadIdx.x == 0) atomic_max_nonneg(&red[4], em);
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

// Rayleigh quotients l_i = s_ii / g_ii (the eigenvalue estimates of a
// converged step, whose update is skipped).
__global__ void k_oa_lambda(int n, const double *__restrict__ S, const double *__restrict__ G,
                            double *__restrict__ lam) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lam[i] = S[(long long)i * n + i] / G[(long long)i * n + i];
}

// One refinement step; returns ||X^T A X - diag|| / ||A|| before the update.
// When that and ||I - X^T X|| are already at rounding level (< kOaConverged)
// the step stops after the statistics: X is kept and only the eigenvalue
// estimates are set.
constexpr double kOaConverged = 1e-12;
// An update whose largest correction |E_ij| is below this leaves an error of
// order |E|^2 (quadratic convergence outside clusters, which are rotated
// exactly): the solve ends after it without a confirming step.
constexpr double kOaFinalUpdate = 1e-7;
// Loose mode (eigenvectors that only feed the next SCF density, whose own
// noise is ~1e-7): converged at off < 1e-9, or after an update below 1e-4
// (error of order 1e-8).
constexpr double kOaConvergedLoose = 1e-9;
constexpr double kOaFinalUpdateLoose = 1e-4;
static double oa_iteration(int n, const double *A, double *X, double *w, MixedEigWork &ws,
                           cudaStream_t st, int max_cluster = kMaxClusterFock,
                           bool *final_update = nullptr, bool loose = false) {
  if (final_update) *final_update = false;
  const double conv = loose ? kOaConvergedLoose : kOaConverged;
  const double fin_thr = loose ? kOaFinalUpdateLoose : kOaFinalUpdate;
  const long long nn = (long long)n * n;
  const int grid = (int)std::min<long long>(ceil_div(nn, kOaThreads), 148);
  double *red = ws.emax + 8;  // [0..4] grid reductions
  gemm(false, false, n, n, n, 1.0, A, n, X, n, nullptr, 0.0, ws.T1, n, st);    // A X
  gemm(true, false, n, n, n, 1.0, X, n, ws.T1, n, nullptr, 0.0, ws.S, n, st);  // X^T A X
  gemm(true, false, n, n, n, 1.0, X, n, X, n, nullptr, 0.0, ws.G, n, st);      // X^T X
  HQ_CUDA(cudaMemsetAsync(red, 0, 5 * sizeof(double), st));
  k_oa_stats<<<grid, kOaThreads, 0, st>>>(n, A, ws.S, ws.G, red);
  HQ_LAUNCH_CHECK();
  double rs[4];
  HQ_CUDA(cudaMemcpyAsync(rs, red, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
  HQ_CUDA(cudaStreamSynchronize(st));
  const double off = std::sqrt(rs[1]) / std::max(std::sqrt(rs[0]), 1e-300);
  // converged: off-diagonal part and orthonormality residual ||I - X^T X||_F
  // both at rounding level (the update also re-normalises X)
  if (off < conv && std::sqrt(rs[2]) < conv) {
    k_oa_lambda<<<ceil_div(n, 256), 256, 0, st>>>(n, ws.S, ws.G, w);
    HQ_LAUNCH_CHECK();
    if (std::getenv("HQCGB_TRACE")) fprintf(stderr, "  oa off=%.3e (converged, no update)\n", off);
    return off;
  }
  k_oa_clusters<<<1, 1024, 0, st>>>(n, ws.S, ws.G, red, w, ws.emax, ws.iwork, ws.wbuf, max_cluster);
  HQ_LAUNCH_CHECK();
  k_oa_rotate_cols<<<grid, kOaThreads, 0, st>>>(n, X, ws.S, ws.G, ws.iwork, ws.wbuf);
  HQ_LAUNCH_CHECK();
  k_oa_rotate_rows<<<grid, kOaThreads, 0, st>>>(n, ws.S, ws.G, ws.iwork, ws.wbuf);
  HQ_LAUNCH_CHECK();
  k_oa_update<<<grid, kOaThreads, n * sizeof(double), st>>>(n, ws.S, ws.G, ws.iwork, ws.emax, w, ws.E,
                                                             red);
  HQ_LAUNCH_CHECK();
  gemm(false, false, n, n, n, 1.0, X, n, ws.E, n, nullptr, 0.0, ws.T1, n, st);  // X E
  axpby(n, 1.0, X, 1.0, ws.T1, false, X, st);                                  // X += X E
  if (final_update) {
    double em[13];
    HQ_CUDA(cudaMemcpyAsync(em, ws.emax, 13 * sizeof(double), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    *final_update = em[8 + 4] < fin_thr && em[2] == 0;
  }
  if (std::getenv("HQCGB_TRACE")) {
    double em[13];
    HQ_CUDA(cudaMemcpyAsync(em, ws.emax, 13 * sizeof(double), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    static thread_local auto t_last = std::chrono::steady_clock::now();
    auto now = std::chrono::steady_clock::now();
    fprintf(stderr, "  oa off=%.3e max|E|=%.3e clusters=%g%s (%.3f ms since last)\n", em[1], em[8 + 4],
            em[3], em[2] != 0 ? " (cluster too large)" : "",
            std::chrono::duration<double, std::milli>(now - t_last).count());
    t_last = now;
  }
  return off;
}

// Full solve: FP32 stage (eigh_f32.cu; the QL solver of eigh_fp64.cu when
// `wide`), then refinement until the relative
// off-diagonal norm measured before a step is at rounding level (1e-12).
// Returns false when the refinement does not get there within 8 steps (the
// caller then uses the FP64 solver).
bool eigh_mixed(int n, const double *A, double *V, double *w, MixedEigWork &ws, cudaStream_t st,
                bool wide, bool loose) {
  HQ_STAGE(ST_JACOBI, st);
  long long nn = (long long)n * n;
  k_f64_to_f32<<<ceil_div(nn, 256), 256, 0, st>>>(nn, A, ws.A32);
  HQ_LAUNCH_CHECK();
  if (wide) {
    // spectra spanning many orders of magnitude with dense near-degenerate
    // groups (the overlap matrix): the QL sweep's vectors refine reliably
    eigh_tql_f32(n, 1, ws.A32, ws.V32, ws.w32, ws.work32, ws.status, st);
    int hs = 0;
    HQ_CUDA(cudaMemcpyAsync(&hs, ws.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (hs < 0) return false;
  } else {
    const bool tr = std::getenv("HQCGB_TRACE") != nullptr;
    cudaEvent_t e0, e1;
    if (tr) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, st);
    }
    eigh_f32(n, ws.A32, ws.V32, ws.w32, ws.f32scr, st);
    if (tr) {
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      fprintf(stderr, "  fp32 stage %.3f ms\n", ms);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
  }
  k_f32_to_f64<<<ceil_div(nn, 256), 256, 0, st>>>(nn, ws.V32, V);
  HQ_LAUNCH_CHECK();
  for (int it = 0; it < 8; ++it) {
    bool fin = false;
    double off = oa_iteration(n, A, V, w, ws, st, wide ? kMaxCluster : kMaxClusterFock, &fin, loose);
    if (off < (loose ? kOaConvergedLoose : kOaConverged) || fin) {
      sort_eigpairs(n, w, V, ws, st);
      return true;
    }
  }
  return false;
}

// Warm start from eigenvectors X0 of a nearby matrix (the previous SCF
// iteration's orthogonalised Fock matrix): refinement only, accepted when it
// reaches rounding level while contracting.  Returns false when the start is
// too far (relative off-diagonal norm above 2e-3) or the iteration stalls; the
// caller then runs the full solve.
bool eigh_mixed_warm(int n, const double *A, const double *X0, double *V, double *w,
                     MixedEigWork &ws, cudaStream_t st, bool loose) {
  HQ_STAGE(ST_JACOBI, st);
  HQ_CUDA(cudaMemcpyAsync(V, X0, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st));
  double prev = 1e300;
  for (int it = 0; it < 8; ++it) {
    bool fin = false;
    double off = oa_iteration(n, A, V, w, ws, st, kMaxClusterFock, &fin, loose);
    if (!(off < 2e-3)) return false;
    if (off < (loose ? kOaConvergedLoose : kOaConverged) || fin) {
      sort_eigpairs(n, w, V, ws, st);
      return true;
    }
    if (it > 0 && off > 0.5 * prev) return false;
    prev = off;
  }
  return false;
}

}  // namespace hqcgb

// C ABI: the mixed-precision solver on one matrix (workspace allocated per call).
extern "C" int hqcgb_eigh_mixed(int n, const double *A, double *w, double *V, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(A && w && V && n >= 1 && n <= kMaxNao, "bad argument");
    size_t nn = (size_t)n * n;
    MixedEigWork ws{};
    size_t f32 = 3 * nn + 2 * (size_t)n + 64 + eigh_f32_scratch_floats(n), f64 = 6 * nn + 64,
           i32 = 5 * (size_t)n + 64;  // emax: 64
    StreamBuf blk(f64 * sizeof(double) + f32 * sizeof(float) + i32 * sizeof(int), st);
    double *d = blk.as<double>();
    ws.T1 = d; ws.S = d + nn; ws.G = d + 2 * nn; ws.E = d + 3 * nn; ws.wbuf = d + 4 * nn;
    ws.emax = d + 6 * nn;
    float *f = reinterpret_cast<float *>(d + f64);
    ws.A32 = f; ws.V32 = f + nn; ws.work32 = f + 2 * nn; ws.w32 = f + 3 * nn;
    ws.f32scr = f + 3 * nn + 2 * n + 64;
    ws.status = reinterpret_cast<int *>(f + f32);
    ws.iwork = ws.status + 64;
    HQ_CUDA(cudaMemsetAsync(ws.status, 0, sizeof(int), st));
    bool ok = eigh_mixed(n, A, V, w, ws, st);
    HQ_CUDA(cudaStreamSynchronize(st));
    int hs = ok ? 0 : -1;
    if (hs < 0) throw Error{HQCGB_EIG_FAIL, "eigensolver did not converge"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
