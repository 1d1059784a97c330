// Grid parts of the nuclear gradient at a single k-point (complex; FP64
// sums).
//
// The reference has no forces (doc/solver_algorithm.md:1210).  Its single-k
// energy (hf_kpt / dft_kpt, hqc/pbc/solver.py:769-962) uses the Bloch AOs
// phi^k; the k-point plan keeps phibar = conj(phi^k) on the grid.  With
// X = D phibar (D = C f C^H), the density rho = Re sum_p conj(phibar_p) X_p
// moves with atom A at fixed D by 2 Re sum_{p in A} dphi_p X_p, and
// dphi_p / dR_A = -grad phi_p = -conj(grad phibar_p).  So the grid term is
//   -2 dV sum_g V_eff(g) Re sum_{p in A} conj(grad phibar_p) X_p,
// with the GGA terms X_p (u . hess phi_p) + grad phi_p (D conj(u . grad phi))_p
// and, for Hartree-Fock, the Madelung term dV Re sum conj(grad phibar_p) Zm_p
// (Zm = c_M D S~ D phibar).  The exact-exchange term
//   dV sum_i f_i Re sum_{p in A} sum_r conj(grad phibar_p conj(psibar_i))
//                                     v_H[X_p conj(psibar_i)]
// is taken in G space by Parseval (coul = 4 pi / (G^2 N) with the
// unnormalised transforms of fft_fp64.cu): one forward transform of the four
// fields X_p conj(psibar_i), d_c phibar_p conj(psibar_i) per AO and orbital
// and no inverse transform (FP32 transforms with FP64 sums on the mixed
// plan, as the Gamma-point exchange gradient).  grad phibar and hess phibar
// are recomputed from the complex 1D factor table of the k-point plan, not
// stored.
#include "common.cuh"
#include "kernels.h"
#include "zmath.cuh"

namespace hqcgb {

// d^{k1} d^{k2} phibar_p at grid point (ix, iy, iz): c1, c2 in {-1, 0, 1, 2}
// (-1: no derivative).  F[A][d][i][a][s], s = 3 l + k (k-th derivative of
// u^l exp(-alpha u^2), each lattice term times exp(-i k_d t)).
__device__ inline double2 ao_eval2_kpt(const double2 *__restrict__ F, const double *__restrict__ coef,
                                       int nprim, int ng, int A, int l, int cart, int ix, int iy, int iz,
                                       int c1, int c2) {
  int pw[3] = {0, 0, 0};
  if (l == 1) pw[cart] = 1;
  int kd[3] = {0, 0, 0};
  if (c1 >= 0) kd[c1] += 1;
  if (c2 >= 0) kd[c2] += 1;
  const double2 *fx = F + ((((long long)A * 3 + 0) * ng + ix) * nprim) * 6 + 3 * pw[0] + kd[0];
  const double2 *fy = F + ((((long long)A * 3 + 1) * ng + iy) * nprim) * 6 + 3 * pw[1] + kd[1];
  const double2 *fz = F + ((((long long)A * 3 + 2) * ng + iz) * nprim) * 6 + 3 * pw[2] + kd[2];
  double2 v = make_double2(0.0, 0.0);
  for (int a = 0; a < nprim; ++a) {
    const double2 t = zmul(zmul(fx[a * 6], fy[a * 6]), fz[a * 6]);
    v.x += coef[a] * t.x;
    v.y += coef[a] * t.y;
  }
  return v;
}

// rho(g) = Re sum_p conj(phibar_p) X_p and, with dphi [3][nao][N],
// grad rho = 2 Re sum_p conj(d phibar_p) X_p.
__global__ void k_rho_from_x_kpt(const double2 *__restrict__ phi, const double2 *__restrict__ dphi,
                                 const double2 *__restrict__ X, int nao, long long N,
                                 double *__restrict__ rho, double *__restrict__ grho) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  const long long NN = (long long)nao * N;
  double r = 0, gx = 0, gy = 0, gz = 0;
  for (int p = 0; p < nao; ++p) {
    const double2 x = X[(long long)p * N + g];
    r += zcmul(phi[(long long)p * N + g], x).x;
    if (dphi) {
      gx += zcmul(dphi[(long long)p * N + g], x).x;
      gy += zcmul(dphi[NN + (long long)p * N + g], x).x;
      gz += zcmul(dphi[2 * NN + (long long)p * N + g], x).x;
    }
  }
  rho[g] = r;
  if (grho) {
    grho[g] = 2.0 * gx;
    grho[N + g] = 2.0 * gy;
    grho[2 * N + g] = 2.0 * gz;
  }
}

// out_p(g) = sum_c u_c(g) d_c phibar_p(g)  (= conj(u . grad phi_p))
__global__ void k_gga_zop_kpt(const double2 *__restrict__ dphi, const double *__restrict__ u, int nao,
                              long long N, double2 *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long NN = (long long)nao * N;
  if (i >= NN) return;
  const long long g = i % N;
  const double2 a = dphi[i], b = dphi[NN + i], c = dphi[2 * NN + i];
  const double u0 = u[g], u1 = u[N + g], u2 = u[2 * N + g];
  out[i] = make_double2(u0 * a.x + u1 * b.x + u2 * c.x, u0 * a.y + u1 * b.y + u2 * c.y);
}

// part[p][blk][c]: grid contribution of AO p to dE/dR_{A(p),c} (written).
__global__ void k_force_grid_kpt(const double2 *__restrict__ F1d, const double *__restrict__ coef,
                                 const int *__restrict__ ao_l, const int *__restrict__ ao_cart,
                                 int nao_atom, int nprim, int ng, const double *__restrict__ veff,
                                 const double2 *__restrict__ X, const double *__restrict__ u,
                                 const double2 *__restrict__ DPsi, const double2 *__restrict__ Zm,
                                 double dV, double *__restrict__ part) {
  __shared__ double sh[32];
  const long long N = (long long)ng * ng * ng;
  const int p = blockIdx.y;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double c3[3] = {0, 0, 0};
  if (g < N) {
    const int iz = (int)(g % ng), iy = (int)((g / ng) % ng), ix = (int)(g / ((long long)ng * ng));
    const int A = p / nao_atom, k = p % nao_atom;
    const double *cf = coef + k * nprim;
    const int l = ao_l[k], ca = ao_cart[k];
    const double2 x = X[(long long)p * N + g];
    double2 dp[3];
    for (int c = 0; c < 3; ++c) dp[c] = ao_eval2_kpt(F1d, cf, nprim, ng, A, l, ca, ix, iy, iz, c, -1);
    const double ve = veff[g];
    for (int c = 0; c < 3; ++c) c3[c] = -2.0 * dV * ve * zcmul(dp[c], x).x;
    if (u) {
      const double ub[3] = {u[g], u[N + g], u[2 * N + g]};
      const double2 dps = DPsi[(long long)p * N + g];
      for (int c = 0; c < 3; ++c) {
        double2 hs = make_double2(0.0, 0.0);
        for (int b = 0; b < 3; ++b) {
          const double2 h = ao_eval2_kpt(F1d, cf, nprim, ng, A, l, ca, ix, iy, iz, c, b);
          hs.x += ub[b] * h.x;
          hs.y += ub[b] * h.y;
        }
        c3[c] += -2.0 * dV * (zcmul(hs, x).x + zcmul(dp[c], dps).x);
      }
    }
    if (Zm) {
      const double2 z = Zm[(long long)p * N + g];
      for (int c = 0; c < 3; ++c) c3[c] += dV * zcmul(dp[c], z).x;
    }
  }
  for (int c = 0; c < 3; ++c) {
    const double s = block_sum(c3[c], sh);
    if (threadIdx.x == 0) part[((long long)p * gridDim.x + blockIdx.x) * 3 + c] = s;
  }
}

__device__ inline void store_c(double2 *p, double2 v) { *p = v; }
__device__ inline void store_c(float2 *p, double2 v) { *p = make_float2((float)v.x, (float)v.y); }
__device__ inline double2 load_c(const double2 *p) { return *p; }
__device__ inline double2 load_c(const float2 *p) {
  const float2 v = *p;
  return make_double2(v.x, v.y);
}

// The four exchange-gradient fields of orbital psibar (one per AO and field):
// out[f][p] = Y_f,p conj(psibar) with Y_0 = X, Y_{1+c} = d_c phibar (FP64, or
// FP32 for the mixed plan's FP32 transforms).
template <class C>
__global__ void k_kx_grad_fields(const double2 *__restrict__ F1d, const double *__restrict__ coef,
                                 const int *__restrict__ ao_l, const int *__restrict__ ao_cart,
                                 int nao_atom, int nprim, int nao, int ng, const double2 *__restrict__ X,
                                 const double2 *__restrict__ psi, C *__restrict__ out) {
  const long long N = (long long)ng * ng * ng;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long NN = (long long)nao * N;
  if (idx >= NN) return;
  const int p = (int)(idx / N);
  const long long g = idx - (long long)p * N;
  const int iz = (int)(g % ng), iy = (int)((g / ng) % ng), ix = (int)(g / ((long long)ng * ng));
  const int A = p / nao_atom, k = p % nao_atom;
  const double *cf = coef + k * nprim;
  const double2 pc = zconj(psi[g]);
  store_c(out + idx, zmul(X[idx], pc));
  for (int c = 0; c < 3; ++c)
    store_c(out + (long long)(1 + c) * NN + idx,
            zmul(ao_eval2_kpt(F1d, cf, nprim, ng, A, ao_l[k], ao_cart[k], ix, iy, iz, c, -1), pc));
}

// part[p][blk][c] += scale * sum_G coul(G) Re(conj(Fhat_{1+c,p}) Fhat_{0,p})  (FP64 sums)
template <class C>
__global__ void k_kx_grad_contract(const C *__restrict__ Fh, const double *__restrict__ coul,
                                   int nao, long long N, double scale, double *__restrict__ part) {
  __shared__ double sh[32];
  const int p = blockIdx.y;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long NN = (long long)nao * N;
  double c3[3] = {0, 0, 0};
  if (g < N) {
    const double w = coul[g];
    const double2 f0 = load_c(Fh + (long long)p * N + g);
    for (int c = 0; c < 3; ++c) c3[c] = w * zcmul(load_c(Fh + (long long)(1 + c) * NN + (long long)p * N + g), f0).x;
  }
  for (int c = 0; c < 3; ++c) {
    const double s = block_sum(c3[c], sh);
    if (threadIdx.x == 0) part[((long long)p * gridDim.x + blockIdx.x) * 3 + c] += scale * s;
  }
}

void launch_rho_from_x_kpt(const double2 *phi, const double2 *dphi, const double2 *X, int nao, long long N,
                           double *rho, double *grho, cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  k_rho_from_x_kpt<<<ceil_div(N, 256), 256, 0, st>>>(phi, dphi, X, nao, N, rho, grho);
  HQ_LAUNCH_CHECK();
}

void launch_gga_zop_kpt(const double2 *dphi, const double *u, int nao, long long N, double2 *out,
                        cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  k_gga_zop_kpt<<<ceil_div((long long)nao * N, 256), 256, 0, st>>>(dphi, u, nao, N, out);
  HQ_LAUNCH_CHECK();
}

void launch_force_grid_kpt(const double2 *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                           int nao_atom, int nprim, int nao, int ng, const double *veff, const double2 *X,
                           const double *u, const double2 *DPsi, const double2 *Zm, double dV, double *part,
                           cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  const long long N = (long long)ng * ng * ng;
  dim3 grid(force_grid_blocks(N), nao);
  k_force_grid_kpt<<<grid, 256, 0, st>>>(F1d, coef, ao_l, ao_cart, nao_atom, nprim, ng, veff, X, u, DPsi, Zm,
                                         dV, part);
  HQ_LAUNCH_CHECK();
}

template <class C>
void launch_kx_grad_fields(const double2 *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                           int nao_atom, int nprim, int nao, int ng, const double2 *X, const double2 *psi,
                           C *out, cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  const long long N = (long long)ng * ng * ng;
  k_kx_grad_fields<C><<<ceil_div((long long)nao * N, 256), 256, 0, st>>>(F1d, coef, ao_l, ao_cart, nao_atom,
                                                                         nprim, nao, ng, X, psi, out);
  HQ_LAUNCH_CHECK();
}
template void launch_kx_grad_fields<double2>(const double2 *, const double *, const int *, const int *, int,
                                             int, int, int, const double2 *, const double2 *, double2 *,
                                             cudaStream_t);
template void launch_kx_grad_fields<float2>(const double2 *, const double *, const int *, const int *, int,
                                            int, int, int, const double2 *, const double2 *, float2 *,
                                            cudaStream_t);

template <class C>
void launch_kx_grad_contract(const C *Fh, const double *coul, int nao, long long N, double scale, double *part,
                             cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  dim3 grid(force_grid_blocks(N), nao);
  k_kx_grad_contract<C><<<grid, 256, 0, st>>>(Fh, coul, nao, N, scale, part);
  HQ_LAUNCH_CHECK();
}
template void launch_kx_grad_contract<double2>(const double2 *, const double *, int, long long, double,
                                               double *, cudaStream_t);
template void launch_kx_grad_contract<float2>(const float2 *, const double *, int, long long, double,
                                              double *, cudaStream_t);

}  // namespace hqcgb
