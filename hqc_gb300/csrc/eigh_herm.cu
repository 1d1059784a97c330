// Complex Hermitian FP64 eigensolver (one thread block per matrix), the
// k-point solver's jnp.linalg.eigh (hqc/pbc/solver.py:795, 812-813 and
// hqc/pbc/scf.py:69,138,198 on complex Fock matrices): ascending eigenvalues,
// eigenvectors equal up to a phase per column (degenerate subspaces: any
// unitary gauge).  Three stages:
//   1. Householder reduction with complex reflectors H_k = I - tau_k v v^H
//      chosen so that H_k^H x = beta e_1 with beta REAL (the zhetd2 / zlarfg
//      construction, lower variant): Q^H A Q = T is a real symmetric
//      tridiagonal; the trailing matrix takes the rank-2 update
//      A22 -= v w^H + w v^H, w = tau A22 v - 1/2 tau (x^H v) v;
//   2. the real implicit QL of eigh_tridiag.cuh, its rotations applied to
//      complex eigenvector rows;
//   3. back-transformation X <- H_k X, k = n-2 .. 0.
// Stage 1 reads both triangles, so the input must be Hermitian: the k-point
// solver passes (A + A^H) / 2, the input jnp.linalg.eigh symmetrises to.
#include <vector>

#include "common.cuh"
#include "eigh_tridiag.cuh"
#include "zmath.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kHermThreads = 1024;

__global__ void __launch_bounds__(kHermThreads)
    k_eigh_herm(int n, double2 *__restrict__ Ab, double2 *__restrict__ Vb, double *__restrict__ wb,
                double2 *__restrict__ workb, int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char hsh_raw[];
  double2 *tau = reinterpret_cast<double2 *>(hsh_raw);  // [n]
  double2 *v = tau + n;                                 // [n] current reflector
  double2 *p = v + n;                                   // [n]
  double *d = reinterpret_cast<double *>(p + n);        // [n]
  double *e = d + n;                                    // [n]
  double *rc = e + n;                                   // [n] rotation cosines / ranks
  double *rs = rc + n;                                  // [n] rotation sines
  __shared__ double red[32];
  __shared__ int s_int[4];
  __shared__ double2 s_sc;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double2 *A = Ab + (long long)blockIdx.x * n * n;
  double2 *V = Vb + (long long)blockIdx.x * n * n;  // receives eigenvectors (columns)
  double *w = wb + (long long)blockIdx.x * n;
  double2 *Zt = workb + (long long)blockIdx.x * n * n;  // Zt[c][r] = Z[r][c]

  // ---------------- 1. tridiagonalisation ----------------
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;
    double2 *col = A + (long long)(k + 1) * n + k;  // A[k+1+i][k] = col[i*n]
    double s2 = 0;
    for (int i = 1 + tid; i < m; i += nt) s2 += zabs2(col[(long long)i * n]);
    s2 = block_sum(s2, red);
    if (tid == 0) {
      const double2 a = col[0];
      if (s2 == 0.0 && a.y == 0.0) {
        tau[k] = zmk(0.0, 0.0);
        e[k] = a.x;
      } else {
        const double beta = -copysign(sqrt(a.x * a.x + a.y * a.y + s2), a.x);
        tau[k] = zmk((beta - a.x) / beta, -a.y / beta);
        e[k] = beta;
        s_sc = zrecip(zmk(a.x - beta, a.y));
      }
    }
    __syncthreads();
    const double2 tk = tau[k];
    if (tk.x == 0.0 && tk.y == 0.0) continue;
    const double2 sc = s_sc;
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? zmk(1.0, 0.0) : zmul(col[(long long)i * n], sc);
    __syncthreads();
    // p = tau A22 v  (one warp per row, coalesced over columns)
    double2 *A22 = A + (long long)(k + 1) * n + (k + 1);
    for (int i = warp; i < m; i += nw) {
      const double2 *row = A22 + (long long)i * n;
      double sr = 0, si = 0;
      for (int j = lane; j < m; j += 32) {
        const double2 t = zmul(row[j], v[j]);
        sr += t.x;
        si += t.y;
      }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (lane == 0) p[i] = zmul(tk, zmk(sr, si));
    }
    __syncthreads();
    double pr = 0, pi = 0;
    for (int i = tid; i < m; i += nt) {
      const double2 t = zcmul(p[i], v[i]);  // p^H v
      pr += t.x;
      pi += t.y;
    }
    pr = block_sum(pr, red);
    pi = block_sum(pi, red);
    const double2 alpha = zscale(-0.5, zmul(tk, zmk(pr, pi)));
    for (int i = tid; i < m; i += nt) p[i] = zadd(p[i], zmul(alpha, v[i]));  // p becomes w
    __syncthreads();
    for (long long idx = tid; idx < (long long)m * m; idx += nt) {
      const int i = (int)(idx / m), j = (int)(idx % m);
      const double2 t = zadd(zmul(v[i], zconj(p[j])), zmul(p[i], zconj(v[j])));
      A22[(long long)i * n + j] = zsub(A22[(long long)i * n + j], t);
    }
    // keep v below the subdiagonal of column k
    for (int i = 1 + tid; i < m; i += nt) col[(long long)i * n] = v[i];
    __syncthreads();
  }
  for (int i = tid; i < n; i += nt) d[i] = A[(long long)i * n + i].x;
  if (tid == 0) {
    e[n - 1] = 0.0;
    tau[n - 1] = zmk(0.0, 0.0);
  }
  for (long long idx = tid; idx < (long long)n * n; idx += nt)
    Zt[idx] = zmk(((int)(idx / n) == (int)(idx % n)) ? 1.0 : 0.0, 0.0);
  __syncthreads();

  // ---------------- 2. implicit QL (real tridiagonal) ----------------
  const int fail = tridiag_ql<double, double2>(n, d, e, Zt, rc, rs, s_int);

  // ---------------- 3. back-transformation ----------------
  for (int k = n - 2; k >= 0 && !fail; --k) {
    __syncthreads();
    const int m = n - k - 1;
    const double2 tk = tau[k];
    if (tk.x == 0.0 && tk.y == 0.0) continue;
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? zmk(1.0, 0.0) : A[(long long)(k + 1 + i) * n + k];
    __syncthreads();
    for (int c = warp; c < n; c += nw) {
      const double2 *zc = Zt + (long long)c * n + (k + 1);
      double sr = 0, si = 0;
      for (int i = lane; i < m; i += 32) {
        const double2 t = zcmul(v[i], zc[i]);  // v^H z
        sr += t.x;
        si += t.y;
      }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (lane == 0) p[c] = zmul(tk, zmk(sr, si));
    }
    __syncthreads();
    for (long long idx = tid; idx < (long long)n * m; idx += nt) {
      const int c = (int)(idx / m), i = (int)(idx % m);
      double2 *z = Zt + (long long)c * n + (k + 1) + i;
      *z = zsub(*z, zmul(v[i], p[c]));
    }
  }
  __syncthreads();

  // ---------------- 4. sort ascending, write V[r][rank] = Z[r][c] ----------------
  for (int c = tid; c < n; c += nt) {
    const double lc = d[c];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = d[j];
      rank += (lj < lc) || (lj == lc && j < c);
    }
    w[rank] = lc;
    rc[c] = (double)rank;
  }
  __syncthreads();
  for (long long idx = tid; idx < (long long)n * n; idx += nt) {
    const int c = (int)(idx / n), r = (int)(idx % n);
    V[(long long)r * n + (int)rc[c]] = Zt[idx];
  }
  if (tid == 0) status[blockIdx.x] = fail ? -1 : 0;
}

size_t eigh_herm_smem(int n) { return (size_t)n * (3 * sizeof(double2) + 4 * sizeof(double)); }

// A is overwritten; work holds batch * n * n complex.
void eigh_herm(int n, int batch, double2 *A, double2 *V, double *w, double2 *work, int *status,
               cudaStream_t st) {
  HQ_STAGE(ST_JACOBI, st);
  const size_t smem = eigh_herm_smem(n);
  HQ_REQUIRE(smem <= 200 * 1024, "matrix too large for the Hermitian eigensolver");
  ensure_dyn_smem((const void *)k_eigh_herm, smem);
  k_eigh_herm<<<batch, kHermThreads, smem, st>>>(n, A, V, w, work, status);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb

// C ABI: eigen-decomposition of batch complex Hermitian matrices A
// [batch][n][n] (interleaved re, im; device), eigenvalues ascending into w
// [batch][n] and eigenvectors as the columns of V [batch][n][n] (complex).
extern "C" int hqcgb_eigh_herm(int n, int batch, const double *A, double *w, double *V, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(A && w && V && n >= 1 && n <= kMaxNao && batch >= 1, "bad argument");
    const size_t nn = (size_t)n * n * batch;
    StreamBuf wbuf(nn * sizeof(double2), st), abuf(nn * sizeof(double2), st), sbuf(batch * sizeof(int), st);
    double2 *work = wbuf.as<double2>(), *Ac = abuf.as<double2>();
    int *stat = sbuf.as<int>();
    HQ_CUDA(cudaMemcpyAsync(Ac, A, nn * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    eigh_herm(n, batch, Ac, reinterpret_cast<double2 *>(V), w, work, stat, st);
    std::vector<int> hs(batch);
    HQ_CUDA(cudaMemcpyAsync(hs.data(), stat, batch * sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    for (int b = 0; b < batch; ++b)
      if (hs[b] < 0) throw Error{HQCGB_EIG_FAIL, "Hermitian eigensolver did not converge"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
