// Small dense FP64 linear algebra of the SCF loop (n_ao <= 1024).
//
//  * gemm: C = alpha op(A) diag(d) op(B) + beta C   (hqc/pbc/scf.py:68,137,197;
//    solver.py:575-577, 700); cuBLAS DGEMM without the diagonal
//  * jacobi_eigh: symmetric eigensolver, parallel cyclic Jacobi with
//    round-robin pair ordering, one block per matrix, ascending eigenvalues
//    (stands in for jnp.linalg.eigh; eigenvectors differ only by gauge)
//  * diis: Pulay matrix, regularised bordered solve and extrapolation
//    (hqc/pbc/scf.py:174-194)
//  * occupations: Fermi / Gauss smearing with the reference's bisection and
//    Newton chemical-potential searches, quirks kept (hqc/tools/smearing.py)
#include <cublas_v2.h>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

// ---------------------------------------------------------------------------
__global__ void k_gemm(int ta, int tb, int M, int N, int K, double alpha,
                       const double *__restrict__ A, int lda, const double *__restrict__ B, int ldb,
                       const double *__restrict__ d, double beta, double *__restrict__ C, int ldc) {
  __shared__ double As[32][33];
  __shared__ double Bs[32][33];
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  double acc[4] = {0, 0, 0, 0};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      // As[r][c] = opA(i0 + r, k0 + c) * d[k0 + c];  Bs[c][r] = opB(k0 + c, j0 + r)
      int i = i0 + r, k = k0 + tx;
      double a = 0;
      if (i < M && k < K) a = ta ? A[(long long)k * lda + i] : A[(long long)i * lda + k];
      if (d && k < K) a *= d[k];
      As[r][tx] = a;
      int j = j0 + r;
      double b = 0;
      if (j < N && k < K) b = tb ? B[(long long)j * ldb + k] : B[(long long)k * ldb + j];
      Bs[r][tx] = b;  // Bs[j][k]
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      double b = Bs[tx][kk];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] += As[ty + 8 * r][kk] * b;
    }
    __syncthreads();
  }
  for (int r = 0; r < 4; ++r) {
    int i = i0 + ty + 8 * r, j = j0 + tx;
    if (i < M && j < N) {
      double v = alpha * acc[r];
      C[(long long)i * ldc + j] = (beta == 0.0) ? v : v + beta * C[(long long)i * ldc + j];
    }
  }
}

// Plain FP64 GEMMs (no diagonal) go to cuBLAS: row-major C = op(A) op(B) is
// column-major C^T = op(B)^T op(A)^T.  One handle per host thread (batch
// workers run their own threads and streams).
static cublasHandle_t blas_handle() {
  static thread_local cublasHandle_t h = nullptr;
  if (!h) {
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS)
      throw Error{HQCGB_CUDA_ERROR, "cublasCreate failed"};
  }
  return h;
}

void gemm(bool ta, bool tb, int M, int N, int K, double alpha, const double *A, int lda,
          const double *B, int ldb, const double *d, double beta, double *C, int ldc,
          cudaStream_t st) {
  HQ_STAGE(ST_GEMM_SMALL, st);
  if (!d) {
    cublasHandle_t h = blas_handle();
    cublasSetStream(h, st);
    cublasStatus_t r = cublasDgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N,
                                   N, M, K, &alpha, B, ldb, A, lda, &beta, C, ldc);
    if (r != CUBLAS_STATUS_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cublasDgemm failed"};
    return;
  }
  dim3 grid(ceil_div(N, 32), ceil_div(M, 32));
  k_gemm<<<grid, 256, 0, st>>>(ta, tb, M, N, K, alpha, A, lda, B, ldb, d, beta, C, ldc);
  HQ_LAUNCH_CHECK();
}

// Row-major complex C = alpha op(A) op(B) + beta C, op 'N' (as is), 'T'
// (transpose) or 'C' (conjugate transpose): cuBLAS ZGEMM on the column-major
// view, where a row-major X reads as X^T and op carries over unchanged.
void zgemm(char opa, char opb, int M, int N, int K, double2 alpha, const double2 *A, int lda,
           const double2 *B, int ldb, double2 beta, double2 *C, int ldc, cudaStream_t st) {
  HQ_STAGE(ST_GEMM_SMALL, st);
  auto op = [](char c) { return c == 'T' ? CUBLAS_OP_T : (c == 'C' ? CUBLAS_OP_C : CUBLAS_OP_N); };
  cublasHandle_t h = blas_handle();
  cublasSetStream(h, st);
  cublasStatus_t r = cublasZgemm(h, op(opb), op(opa), N, M, K, &alpha, B, ldb, A, lda, &beta, C, ldc);
  if (r != CUBLAS_STATUS_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cublasZgemm failed"};
}

// C[b] = A[b] B[b] for row-major M x K and K x N blocks (strides in elements;
// stride 0 shares a block): cuBLAS strided-batched DGEMM, column-major view.
void gemm_batched_rowmajor(int M, int N, int K, const double *A, int lda, long long sa,
                           const double *B, int ldb, long long sb, double *C, int ldc, long long sc,
                           int batch, cudaStream_t st) {
  HQ_STAGE(ST_GEMM_SMALL, st);
  cublasHandle_t h = blas_handle();
  cublasSetStream(h, st);
  const double one = 1.0, zero = 0.0;
  cublasStatus_t r = cublasDgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one, B, ldb, sb,
                                               A, lda, sa, &zero, C, ldc, sc, batch);
  if (r != CUBLAS_STATUS_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cublasDgemmStridedBatched failed"};
}

// Complex C[b] = A[b] B[b] (row-major, strides in elements; stride 0 shares a
// block): cuBLAS strided-batched ZGEMM on the column-major view.
void zgemm_batched_rowmajor(int M, int N, int K, const double2 *A, int lda, long long sa,
                            const double2 *B, int ldb, long long sb, double2 *C, int ldc,
                            long long sc, int batch, cudaStream_t st) {
  HQ_STAGE(ST_GEMM_SMALL, st);
  cublasHandle_t h = blas_handle();
  cublasSetStream(h, st);
  const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0);
  cublasStatus_t r = cublasZgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one, B, ldb, sb,
                                               A, lda, sa, &zero, C, ldc, sc, batch);
  if (r != CUBLAS_STATUS_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cublasZgemmStridedBatched failed"};
}

// out = a*X + b*Y (+ c*Z^T): generic elementwise combos on n x n matrices.
__global__ void k_axpby(int n, double a, const double *__restrict__ X, double b,
                        const double *__restrict__ Y, int transY, double *__restrict__ out) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  int i = idx / n, j = idx % n;
  double y = Y ? (transY ? Y[j * n + i] : Y[idx]) : 0.0;
  out[idx] = (X ? a * X[idx] : 0.0) + b * y;
}

void axpby(int n, double a, const double *X, double b, const double *Y, bool transY, double *out,
           cudaStream_t st) {
  k_axpby<<<ceil_div((long long)n * n, 256), 256, 0, st>>>(n, a, X, b, Y, transY ? 1 : 0, out);
  HQ_LAUNCH_CHECK();
}

// out[slot] = scale * sum_ij A_ij B_ij   (= tr(A B) for symmetric B)
__global__ void k_dot(long long n, const double *__restrict__ A, const double *__restrict__ B,
                      double scale, double *__restrict__ out, int accumulate) {
  __shared__ double sh[32];
  double s = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += A[i] * (B ? B[i] : A[i]);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = accumulate ? *out + scale * s : scale * s;
}

void dot(long long n, const double *A, const double *B, double scale, double *out, bool accumulate,
         cudaStream_t st) {
  k_dot<<<1, 1024, 0, st>>>(n, A, B, scale, out, accumulate ? 1 : 0);
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Jacobi eigensolver.  A (n x n, overwritten), V (n x n eigenvectors as
// columns), w (n eigenvalues, ascending).  One block per matrix of a batch.
// status[b] = number of sweeps, or -1 when the sweep limit was hit.
// ---------------------------------------------------------------------------
__device__ inline int rr_player(int pos, int round, int m) {
  if (pos == 0) return 0;
  return 1 + ((pos - 1 + round) % (m - 1));
}

__global__ void __launch_bounds__(1024) k_jacobi(int n, double *__restrict__ Ab, double *__restrict__ Vb,
                                                 double *__restrict__ wb, double *__restrict__ tmpb,
                                                 int max_sweeps, double tol, int *__restrict__ status) {
  extern __shared__ double jsh[];
  int m = n + (n & 1);
  int npairs = m / 2;
  double *cs = jsh;
  double *sn = jsh + npairs;
  int *pp = (int *)(sn + npairs);
  int *qq = pp + npairs;
  __shared__ double red[32];
  __shared__ int done;
  double *A = Ab + (long long)blockIdx.x * n * n;
  double *V = Vb + (long long)blockIdx.x * n * n;
  double *w = wb + (long long)blockIdx.x * n;
  double *tmp = tmpb + (long long)blockIdx.x * n * n;
  int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n * n; i += nt) V[i] = (i / n == i % n) ? 1.0 : 0.0;
  int sweep = 0;
  if (tid == 0) done = 0;
  __syncthreads();
  for (sweep = 0; sweep < max_sweeps; ++sweep) {
    // convergence test: off-diagonal Frobenius norm vs the whole norm
    double off = 0, tot = 0;
    for (int i = tid; i < n * n; i += nt) {
      double a = A[i];
      tot += a * a;
      if (i / n != i % n) off += a * a;
    }
    off = block_sum(off, red);
    tot = block_sum(tot, red);
    if (tid == 0) done = (off <= tol * tol * tot) ? 1 : 0;
    __syncthreads();
    if (done) break;
    for (int round = 0; round < m - 1; ++round) {
      for (int t = tid; t < npairs; t += nt) {
        int a = rr_player(t, round, m), b = rr_player(m - 1 - t, round, m);
        int p = min(a, b), q = max(a, b);
        double c = 1.0, s = 0.0;
        if (q < n) {
          double apq = A[p * n + q];
          double app = A[p * n + p], aqq = A[q * n + q];
          if (fabs(apq) > 1e-300 && fabs(apq) > 1e-18 * sqrt(fabs(app * aqq))) {
            double tau = (aqq - app) / (2.0 * apq);
            double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + tt * tt);
            s = tt * c;
          }
        }
        cs[t] = c; sn[t] = s; pp[t] = p; qq[t] = q;
      }
      __syncthreads();
      // column rotations: A <- A J, V <- V J
      for (int it = tid; it < npairs * n; it += nt) {
        int t = it / n, r = it % n;
        int p = pp[t], q = qq[t];
        if (q >= n) continue;
        double c = cs[t], s = sn[t];
        if (s == 0.0) continue;
        double arp = A[r * n + p], arq = A[r * n + q];
        A[r * n + p] = c * arp - s * arq;
        A[r * n + q] = s * arp + c * arq;
        double vrp = V[r * n + p], vrq = V[r * n + q];
        V[r * n + p] = c * vrp - s * vrq;
        V[r * n + q] = s * vrp + c * vrq;
      }
      __syncthreads();
      // row rotations: A <- J^T A
      for (int it = tid; it < npairs * n; it += nt) {
        int t = it / n, r = it % n;
        int p = pp[t], q = qq[t];
        if (q >= n) continue;
        double c = cs[t], s = sn[t];
        if (s == 0.0) continue;
        double apr = A[p * n + r], aqr = A[q * n + r];
        A[p * n + r] = c * apr - s * aqr;
        A[q * n + r] = s * apr + c * aqr;
      }
      __syncthreads();
      for (int t = tid; t < npairs; t += nt) {
        int p = pp[t], q = qq[t];
        if (q < n && sn[t] != 0.0) { A[p * n + q] = 0.0; A[q * n + p] = 0.0; }
      }
      __syncthreads();
    }
  }
  // sort ascending: rank of each eigenvalue
  for (int i = tid; i < n; i += nt) tmp[i] = A[i * n + i];
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    double li = tmp[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      double lj = tmp[j];
      rank += (lj < li) || (lj == li && j < i);
    }
    w[rank] = li;
    for (int r = 0; r < n; ++r) A[r * n + rank] = V[r * n + i];  // reuse A as sorted vectors
  }
  __syncthreads();
  for (int i = tid; i < n * n; i += nt) V[i] = A[i];
  if (tid == 0) status[blockIdx.x] = (sweep >= max_sweeps) ? -1 : sweep;
}

void jacobi_eigh(int n, int batch, double *A, double *V, double *w, double *tmp, int *status,
                 cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  int m = n + (n & 1);
  size_t smem = (size_t)(m / 2) * (2 * sizeof(double) + 2 * sizeof(int));
  k_jacobi<<<batch, 1024, smem, st>>>(n, A, V, w, tmp, 60, 1e-14, status);
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// DIIS (scf.py:178-194).  ek/Fk: [space][n*n] ring; the extrapolation is
// invariant to the ring order.  B[i][j] = <e_i, e_j>.
// ---------------------------------------------------------------------------
__global__ void k_diis_B(int space, long long nn, const double *__restrict__ ek,
                         double *__restrict__ B) {
  __shared__ double sh[32];
  int i = blockIdx.x / space, j = blockIdx.x % space;
  if (j < i) return;
  double s = 0;
  for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += ek[i * nn + k] * ek[j * nn + k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) { B[i * space + j] = s; B[j * space + i] = s; }
}

__global__ void k_diis_solve(int space, const double *__restrict__ B, double *__restrict__ c) {
  if (threadIdx.x != 0) return;
  const int MAXS = 33;
  double h[MAXS][MAXS + 1];
  int m = space + 1;
  double tr = 0;
  for (int i = 0; i < space; ++i) tr += B[i * space + i];
  double eta = 1e-12 * (tr / space + 1.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j <= m; ++j) h[i][j] = 0.0;
  for (int i = 0; i < space; ++i) {
    for (int j = 0; j < space; ++j) h[i][j] = B[i * space + j] + (i == j ? eta : 0.0);
    h[i][space] = -1.0;
    h[space][i] = -1.0;
  }
  h[space][m] = -1.0;  // rhs g = (0,...,0,-1)
  // Gaussian elimination with partial pivoting (LU of jnp.linalg.solve)
  for (int k = 0; k < m; ++k) {
    int piv = k;
    for (int i = k + 1; i < m; ++i)
      if (fabs(h[i][k]) > fabs(h[piv][k])) piv = i;
    if (piv != k)
      for (int j = 0; j <= m; ++j) { double t = h[k][j]; h[k][j] = h[piv][j]; h[piv][j] = t; }
    double d = h[k][k];
    for (int i = k + 1; i < m; ++i) {
      double f = h[i][k] / d;
      for (int j = k; j <= m; ++j) h[i][j] -= f * h[k][j];
    }
  }
  double x[MAXS];
  for (int i = m - 1; i >= 0; --i) {
    double s = h[i][m];
    for (int j = i + 1; j < m; ++j) s -= h[i][j] * x[j];
    x[i] = s / h[i][i];
  }
  for (int i = 0; i < space; ++i) c[i] = x[i];
}

// F = (1 - damp) sum_k c_k F_k + damp F_last
__global__ void k_diis_extrapolate(int space, long long nn, const double *__restrict__ Fk,
                                   const double *__restrict__ c, int last, double damp,
                                   double *__restrict__ F) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nn) return;
  double s = 0;
  for (int k = 0; k < space; ++k) s += c[k] * Fk[k * nn + idx];
  F[idx] = (1.0 - damp) * s + damp * Fk[last * nn + idx];
}

void diis_extrapolate(int space, int n, const double *Fk, const double *ek, int last, double damp,
                      double *B, double *c, double *F, cudaStream_t st) {
  HQ_STAGE(ST_GEMM_SMALL, st);
  HQ_REQUIRE(space <= 32, "diis_space > 32");
  long long nn = (long long)n * n;
  k_diis_B<<<space * space, 256, 0, st>>>(space, nn, ek, B);
  HQ_LAUNCH_CHECK();
  k_diis_solve<<<1, 32, 0, st>>>(space, B, c);
  HQ_LAUNCH_CHECK();
  k_diis_extrapolate<<<ceil_div(nn, 256), 256, 0, st>>>(space, nn, Fk, c, last, damp, F);
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Occupations (smearing.py).  One warp.  w ascending eigenvalues (Hartree).
// ---------------------------------------------------------------------------
struct OccParams {
  int n_elec, nmo, smearing, method, search, cycle;
  double sigma, tol, shift;
};

__device__ inline double occ_f(const OccParams &P, double mu, double w) {
  if (P.method == HQCGB_SMEAR_FERMI) {
    double x = (w - mu) / P.sigma;
    x = fmin(fmax(x, -50.0), 50.0);
    return 2.0 / (exp(x) + 1.0);
  }
  return 0.5 * (1.0 + erf((mu - w) / P.sigma));
}

// N(mu) - n and derivatives, reduced over the warp
__device__ inline void occ_N(const OccParams &P, const double *w, double mu, double &N, double &d1,
                             double &d2) {
  double s0 = 0, s1 = 0, s2 = 0;
  for (int i = threadIdx.x; i < P.nmo; i += 32) {
    double s = P.sigma;
    if (P.method == HQCGB_SMEAR_FERMI) {
      double x = (w[i] - mu) / s;
      bool in = (x >= -50.0) && (x <= 50.0);
      double e = exp(fmin(fmax(x, -50.0), 50.0));
      s0 += 2.0 / (e + 1.0);
      if (in) {
        s1 += 2.0 * e / ((e + 1.0) * (e + 1.0)) / s;
        s2 += 2.0 * e * (e - 1.0) / ((e + 1.0) * (e + 1.0) * (e + 1.0)) / (s * s);
      }
    } else {
      double u = (mu - w[i]) / s;
      double g = exp(-u * u) * 0.56418958354775628;  // 1/sqrt(pi)
      s0 += 0.5 * (1.0 + erf(u));
      s1 += g / s;
      s2 += -2.0 * u * g / (s * s);
    }
  }
  N = warp_sum(s0) - P.n_elec;
  d1 = warp_sum(s1);
  d2 = warp_sum(s2);
}

__global__ void k_occupations(OccParams P, const double *__restrict__ w, double *__restrict__ f,
                              double *__restrict__ mu_out) {
  int n = P.nmo;
  if (!P.smearing) {
    for (int i = threadIdx.x; i < n; i += 32) f[i] = (i < P.n_elec / 2) ? 2.0 : 0.0;
    if (threadIdx.x == 0 && mu_out) *mu_out = 0.0;
    return;
  }
  double mu;
  if (P.search == HQCGB_SEARCH_BISECT) {
    // smearing.py:74-102 (w ascending: min = w[0], max = w[n-1])
    double lo = w[0] + P.shift, hi = w[n - 1] + P.shift;
    double ylo = -1.0, yhi = 1.0;
    int loop = 0;
    while ((ylo < -P.tol) && (yhi > P.tol) && (loop < P.cycle)) {
      double mid = 0.5 * (lo + hi), ym, d1, d2;
      occ_N(P, w, mid, ym, d1, d2);
      if (ym < 0) lo = mid; else hi = mid;
      occ_N(P, w, lo, ylo, d1, d2);
      occ_N(P, w, hi, yhi, d1, d2);
      ++loop;
    }
    mu = (lo > -P.tol ? lo : 0.0) + (hi < P.tol ? hi : 0.0) + (loop == P.cycle ? 0.5 * (lo + hi) : 0.0);
  } else {
    // smearing.py:106-138: Newton on N(mu)^2
    double mu0 = 1.0;
    mu = w[P.n_elec / 2];
    int loop = 0;
    while (fabs(mu - mu0) > P.tol && loop < P.cycle) {
      double N, d1, d2;
      occ_N(P, w, mu, N, d1, d2);
      double g1 = 2.0 * N * d1, g2 = 2.0 * d1 * d1 + 2.0 * N * d2;
      mu0 = mu;
      mu = mu - g1 / fabs(g2);
      ++loop;
    }
  }
  for (int i = threadIdx.x; i < n; i += 32) f[i] = occ_f(P, mu, w[i]);
  if (threadIdx.x == 0 && mu_out) *mu_out = mu;
}

void occupations(int n_elec, int nmo, int smearing, int method, double sigma, int search, int cycle,
                 double tol, double shift, const double *w, double *f, double *mu, cudaStream_t st) {
  HQ_STAGE(ST_OTHER, st);
  OccParams P{n_elec, nmo, smearing, method, search, cycle, sigma, tol, shift};
  k_occupations<<<1, 32, 0, st>>>(P, w, f, mu);
  HQ_LAUNCH_CHECK();
}

// Se = -2 sum [h ln h + (1-h) ln(1-h)], h = f/2, terms below 1e-15 dropped (solver.py:579-590)
__global__ void k_entropy(int n, const double *__restrict__ f, double *__restrict__ out) {
  __shared__ double sh[32];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double h = 0.5 * f[i];
    if (h > 1e-15) s += h * log(h);
    if (1.0 - h > 1e-15) s += (1.0 - h) * log(1.0 - h);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = -2.0 * s;
}

void entropy(int n, const double *f, double *out, cudaStream_t st) {
  k_entropy<<<1, 256, 0, st>>>(n, f, out);
  HQ_LAUNCH_CHECK();
}

// The entropy S that makes the smeared occupations stationary points of
// E - sigma S at fixed particle number: Fermi f = 2 / (e^x + 1) -> the Fermi
// formula above; Gaussian f = erfc(x) / 2 (capped at 1, smearing.py:52) ->
// S = sum_i exp(-x_i^2) / (2 sqrt(pi)), x_i = (w_i - mu) / sigma.
__global__ void k_entropy_gauss(int n, const double *__restrict__ w, const double *__restrict__ mu,
                                double sigma, double *__restrict__ out) {
  __shared__ double sh[32];
  double s = 0;
  const double m = *mu;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = (w[i] - m) / sigma;
    s += exp(-x * x);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s * 0.28209479177387814;  // 1 / (2 sqrt(pi))
}

void free_entropy(int n, int method, double sigma, const double *w, const double *mu, const double *f,
                  double *out, cudaStream_t st) {
  if (method == HQCGB_SMEAR_GAUSS) {
    k_entropy_gauss<<<1, 256, 0, st>>>(n, w, mu, sigma, out);
    HQ_LAUNCH_CHECK();
  } else {
    entropy(n, f, out, st);
  }
}

// v = U diag(w^-1/2)  (solver.py:729-730)
__global__ void k_inv_sqrt_cols(int n, const double *__restrict__ U, const double *__restrict__ w,
                                double *__restrict__ v, int *__restrict__ bad) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  int j = idx % n;
  double e = w[j];
  if (!(e > 1e-13)) { if (bad) *bad = 1; v[idx] = 0.0; return; }
  v[idx] = U[idx] / sqrt(e);
}

void inv_sqrt_cols(int n, const double *U, const double *w, double *v, int *bad, cudaStream_t st) {
  k_inv_sqrt_cols<<<ceil_div((long long)n * n, 256), 256, 0, st>>>(n, U, w, v, bad);
  HQ_LAUNCH_CHECK();
}

// ||X - X^T||_F for the DIIS error vector e = SDF - FDS = X - X^T with X = SDF.
__global__ void k_antisym(int n, const double *__restrict__ X, double *__restrict__ e) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  int i = idx / n, j = idx % n;
  e[idx] = X[idx] - X[j * n + i];
}

void antisym(int n, const double *X, double *e, cudaStream_t st) {
  k_antisym<<<ceil_div((long long)n * n, 256), 256, 0, st>>>(n, X, e);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb

namespace hqcgb {
// Y[p][k] = C[p][k] sqrt(occ[k]) for k < nuse (row stride nuse): D = Y Y^T.
__global__ void k_occ_block(const double *__restrict__ C, const double *__restrict__ occ, int n,
                            int nuse, double *__restrict__ Y) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nuse) return;
  const int p = idx / nuse, k = idx % nuse;
  Y[idx] = C[(long long)p * n + k] * sqrt(fmax(occ[k], 0.0));
}

void launch_occ_block(const double *C, const double *occ, int n, int nuse, double *Y, cudaStream_t st) {
  k_occ_block<<<ceil_div((long long)n * nuse, 256), 256, 0, st>>>(C, occ, n, nuse, Y);
  HQ_LAUNCH_CHECK();
}
}  // namespace hqcgb
