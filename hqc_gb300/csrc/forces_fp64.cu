// Grid parts of the exact exchange and of the nuclear gradient (FP64).
//
// The reference has no forces (doc/solver_algorithm.md:1210).  For the
// discrete, variational energy of hqc/pbc/solver.py, the grid contribution
// to dE/dR_A at fixed density matrix is
//   -2 dV sum_g sum_{p in A} grad phi_p(g) . [ V_eff(g) X_p(g) + ... ],
// X = D phi, with the GGA terms  X_p (u . hess phi_p) + grad phi_p (D Psi)_p
// (u = 2 v_sigma grad rho, Psi = u . grad phi) and, for Hartree-Fock, the
// orbital term  + dV sum_g grad phi_p(g) Z_p(g).  Grid tiles of grad phi and
// hess phi are recomputed from the 1D factor table, not stored.
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

// psi(g) = sum_p C[p][col] phi_p(g)
__global__ void k_psi(const double *__restrict__ C, int nao, int col, const double *__restrict__ phi,
                      long long N, double *__restrict__ psi) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  double s = 0;
  for (int p = 0; p < nao; ++p) s += C[(long long)p * nao + col] * phi[(long long)p * N + g];
  psi[g] = s;
}

void launch_psi(const double *C, int nao, int col, const double *phi, long long N, double *psi,
                cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  k_psi<<<ceil_div(N, 256), 256, 0, st>>>(C, nao, col, phi, N, psi);
  HQ_LAUNCH_CHECK();
}

// Z[i] += a * s[i % N] * X[i]
__global__ void k_axpy_grid(long long total, long long N, double a, const double *__restrict__ s,
                            const double *__restrict__ X, double *__restrict__ Z) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  Z[i] += a * (s ? s[i % N] : 1.0) * X[i];
}

void launch_axpy_grid(long long total, long long N, double a, const double *s, const double *X,
                      double *Z, cudaStream_t st) {
  k_axpy_grid<<<ceil_div(total, 256), 256, 0, st>>>(total, N, a, s, X, Z);
  HQ_LAUNCH_CHECK();
}

__global__ void k_add3(long long N, const double *__restrict__ a, const double *__restrict__ b,
                       const double *__restrict__ c, double *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  out[i] = (a ? a[i] : 0.0) + (b ? b[i] : 0.0) + (c ? c[i] : 0.0);
}

void launch_add3(long long N, const double *a, const double *b, const double *c, double *out,
                 cudaStream_t st) {
  k_add3<<<ceil_div(N, 256), 256, 0, st>>>(N, a, b, c, out);
  HQ_LAUNCH_CHECK();
}

// Psi_p(g) = sum_c u_c(g) dphi_c,p(g)
__global__ void k_gga_psi(const double *__restrict__ dphi, const double *__restrict__ u, int nao,
                          long long N, double *__restrict__ Psi) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long NN = (long long)nao * N;
  if (i >= NN) return;
  long long g = i % N;
  Psi[i] = u[g] * dphi[i] + u[N + g] * dphi[NN + i] + u[2 * N + g] * dphi[2 * NN + i];
}

void launch_gga_psi(const double *dphi, const double *u, int nao, long long N, double *Psi,
                    cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  k_gga_psi<<<ceil_div((long long)nao * N, 256), 256, 0, st>>>(dphi, u, nao, N, Psi);
  HQ_LAUNCH_CHECK();
}

__device__ inline double ao_eval_f(const double *__restrict__ F, const double *__restrict__ coef,
                                   int nprim, int ng, int A, int l, int cart, int ix, int iy, int iz,
                                   int c1, int c2) {
  int pw[3] = {0, 0, 0};
  if (l == 1) pw[cart] = 1;
  int kd[3] = {0, 0, 0};
  if (c1 >= 0) kd[c1] += 1;
  if (c2 >= 0) kd[c2] += 1;
  const double *fx = F + ((((long long)A * 3 + 0) * ng + ix) * nprim) * 6 + 3 * pw[0] + kd[0];
  const double *fy = F + ((((long long)A * 3 + 1) * ng + iy) * nprim) * 6 + 3 * pw[1] + kd[1];
  const double *fz = F + ((((long long)A * 3 + 2) * ng + iz) * nprim) * 6 + 3 * pw[2] + kd[2];
  double v = 0.0;
  for (int a = 0; a < nprim; ++a) v += coef[a] * fx[a * 6] * fy[a * 6] * fz[a * 6];
  return v;
}

// part[p][blk][c]: grid contribution of AO p to dE/dR_{A(p),c}.
__global__ void k_force_grid(const double *__restrict__ F1d, const double *__restrict__ coef,
                             const int *__restrict__ ao_l, const int *__restrict__ ao_cart,
                             int nao_atom, int nprim, int nao, int ng,
                             const double *__restrict__ veff, const double *__restrict__ X,
                             const double *__restrict__ u, const double *__restrict__ DPsi,
                             const double *__restrict__ Z, double dV, double *__restrict__ part) {
  __shared__ double sh[32];
  long long N = (long long)ng * ng * ng;
  int p = blockIdx.y;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double c3[3] = {0, 0, 0};
  if (g < N) {
    int iz = g % ng, iy = (g / ng) % ng, ix = (int)(g / ((long long)ng * ng));
    int A = p / nao_atom, k = p % nao_atom;
    const double *cf = coef + k * nprim;
    int l = ao_l[k], ca = ao_cart[k];
    double x = X[(long long)p * N + g];
    double dp[3];
    for (int c = 0; c < 3; ++c) dp[c] = ao_eval_f(F1d, cf, nprim, ng, A, l, ca, ix, iy, iz, c, -1);
    double ve = veff[g];
    for (int c = 0; c < 3; ++c) c3[c] = -2.0 * dV * ve * x * dp[c];
    if (u) {
      double ub[3] = {u[g], u[N + g], u[2 * N + g]};
      double dps = DPsi[(long long)p * N + g];
      for (int c = 0; c < 3; ++c) {
        double hs = 0;
        for (int b = 0; b < 3; ++b)
          hs += ub[b] * ao_eval_f(F1d, cf, nprim, ng, A, l, ca, ix, iy, iz, c, b);
        c3[c] += -2.0 * dV * (x * hs + dp[c] * dps);
      }
    }
    if (Z) {
      double z = Z[(long long)p * N + g];
      for (int c = 0; c < 3; ++c) c3[c] += dV * dp[c] * z;
    }
  }
  for (int c = 0; c < 3; ++c) {
    double s = block_sum(c3[c], sh);
    if (threadIdx.x == 0) part[((long long)p * gridDim.x + blockIdx.x) * 3 + c] = s;
  }
}

int force_grid_blocks(long long N) { return ceil_div(N, 256); }

void launch_force_grid(const double *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                       int nao_atom, int nprim, int nao, int ng, const double *veff,
                       const double *X, const double *u, const double *DPsi, const double *Z,
                       double dV, double *part, cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  long long N = (long long)ng * ng * ng;
  dim3 grid(force_grid_blocks(N), nao);
  k_force_grid<<<grid, 256, 0, st>>>(F1d, coef, ao_l, ao_cart, nao_atom, nprim, nao, ng, veff, X, u,
                                     DPsi, Z, dV, part);
  HQ_LAUNCH_CHECK();
}

__global__ void k_force_grid_reduce(const double *__restrict__ part, int nao_atom, int nblk,
                                    double *__restrict__ grad) {
  __shared__ double sh[32];
  int A = blockIdx.x;
  for (int c = 0; c < 3; ++c) {
    double s = 0;
    long long tot = (long long)nao_atom * nblk;
    for (long long k = threadIdx.x; k < tot; k += blockDim.x) {
      int pl = (int)(k / nblk);
      long long b = k % nblk;
      int p = A * nao_atom + pl;
      s += part[((long long)p * nblk + b) * 3 + c];
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) grad[A * 3 + c] += s;
    __syncthreads();
  }
}

void launch_force_grid_reduce(const double *part, int nao, int nao_atom, int nblk, double *grad,
                              cudaStream_t st) {
  k_force_grid_reduce<<<nao / nao_atom, 256, 0, st>>>(part, nao_atom, nblk, grad);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
