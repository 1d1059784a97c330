// Grid part of the nuclear gradient in the mixed path (Kohn-Sham, no
// smearing): the FP64 formulation of forces_fp64.cu rewritten over the
// occupied orbitals on the grid, which the last SCF density pass leaves
// behind (psi_k = sum_q Y_qk phi_q and grad psi_k, Y = C_occ sqrt(f)):
//   X_p(g)        = sum_q D_pq phi_q(g)            = sum_k Y_pk psi_k(g)
//   (D Psi)_p(g)  = sum_q D_pq u(g).grad phi_q(g)  = sum_k Y_pk u(g).grad psi_k(g)
// so that the contribution of atom A,
//   -2 dV sum_g sum_{p in A} [ v_eff X_p grad phi_p
//                              + X_p (u . hess phi_p) + grad phi_p (D Psi)_p ],
// costs n_occ instead of n_ao multiply-adds per (AO, point) and needs no
// n_ao x N FP64 intermediates.  grad phi and hess phi are recomputed in FP32
// from the 1D factor table; per-thread sums are FP32, block and grid sums
// FP64.  The reference has no forces (doc/solver_algorithm.md:1210).
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kFgThreads = 256;
constexpr int kFgWarps = kFgThreads / 32;

__global__ void k_to_float(long long n, const double *__restrict__ a, float *__restrict__ b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// Y32[p][k] = C[p][k] sqrt(occ[k]) for k < nuse, 0 up to npsi.
__global__ void k_force_operand(const double *__restrict__ C, const double *__restrict__ occ,
                                int nao, int nuse, int npsi, float *__restrict__ Y32) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nao * npsi) return;
  int p = idx / npsi, k = idx % npsi;
  Y32[idx] = k < nuse ? (float)(C[(long long)p * nao + k] * sqrt(fmax(occ[k], 0.0))) : 0.f;
}

// One thread per grid point; the block loops over the atoms and writes
// part[block][atom][3].  psi: [4][NPSI][N] (value, d/dx, d/dy, d/dz) or
// [1][NPSI][N] without GGA.
template <int NPSI, bool GGA>
__global__ void __launch_bounds__(kFgThreads)
    k_force_grid_orb(const float *__restrict__ F, const double *__restrict__ coef,
                     const int *__restrict__ ao_l, const int *__restrict__ ao_cart, int n_atoms,
                     int nb, int nprim, int ng, const double *__restrict__ veff,
                     const double *__restrict__ u, const float *__restrict__ psi,
                     const float *__restrict__ Y, double dV, double *__restrict__ part) {
  extern __shared__ float fred[];  // [warps][n_atoms][3]
  const long long N = (long long)ng * ng * ng;
  const long long g = (long long)blockIdx.x * kFgThreads + threadIdx.x;
  const bool in = g < N;
  const long long gg = in ? g : 0;
  const int iz = (int)(gg % ng), iy = (int)((gg / ng) % ng), ix = (int)(gg / ((long long)ng * ng));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float ps[NPSI], t[NPSI];
  const float ve = (float)veff[gg];
  float u0 = 0.f, u1 = 0.f, u2 = 0.f;
  if (GGA) {
    u0 = (float)u[gg];
    u1 = (float)u[N + gg];
    u2 = (float)u[2 * N + gg];
  }
#pragma unroll
  for (int k = 0; k < NPSI; ++k) {
    ps[k] = psi[(long long)k * N + gg];
    if (GGA)
      t[k] = u0 * psi[(long long)(NPSI + k) * N + gg] + u1 * psi[(long long)(2 * NPSI + k) * N + gg] +
             u2 * psi[(long long)(3 * NPSI + k) * N + gg];
  }
  for (int A = 0; A < n_atoms; ++A) {
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    const float *fxb = F + (((long long)A * 3 + 0) * ng + ix) * nprim * 6;
    const float *fyb = F + (((long long)A * 3 + 1) * ng + iy) * nprim * 6;
    const float *fzb = F + (((long long)A * 3 + 2) * ng + iz) * nprim * 6;
    for (int j = 0; j < nb; ++j) {
      const int l = ao_l[j], ca = ao_cart[j];
      const int bx = (l == 1 && ca == 0) ? 3 : 0, by = (l == 1 && ca == 1) ? 3 : 0,
                bz = (l == 1 && ca == 2) ? 3 : 0;
      float d0 = 0.f, d1 = 0.f, d2 = 0.f, hxx = 0.f, hyy = 0.f, hzz = 0.f, hxy = 0.f, hxz = 0.f,
            hyz = 0.f;
      for (int a = 0; a < nprim; ++a) {
        const float cf = (float)coef[j * nprim + a];
        const float *fx = fxb + a * 6 + bx, *fy = fyb + a * 6 + by, *fz = fzb + a * 6 + bz;
        const float x0 = fx[0], x1 = fx[1], y0 = fy[0], y1 = fy[1], z0 = fz[0], z1 = fz[1];
        const float cy0z0 = cf * y0 * z0, cx0z0 = cf * x0 * z0, cx0y0 = cf * x0 * y0;
        d0 += x1 * cy0z0;
        d1 += y1 * cx0z0;
        d2 += z1 * cx0y0;
        if (GGA) {
          hxx += fx[2] * cy0z0;
          hyy += fy[2] * cx0z0;
          hzz += fz[2] * cx0y0;
          hxy += cf * x1 * y1 * z0;
          hxz += cf * x1 * y0 * z1;
          hyz += cf * x0 * y1 * z1;
        }
      }
      const float *yp = Y + (long long)(A * nb + j) * NPSI;
      float X = 0.f, DP = 0.f;
#pragma unroll
      for (int k = 0; k < NPSI; ++k) {
        X = fmaf(yp[k], ps[k], X);
        if (GGA) DP = fmaf(yp[k], t[k], DP);
      }
      const float vx = ve * X;
      f0 += vx * d0;
      f1 += vx * d1;
      f2 += vx * d2;
      if (GGA) {
        f0 += X * (u0 * hxx + u1 * hxy + u2 * hxz) + d0 * DP;
        f1 += X * (u0 * hxy + u1 * hyy + u2 * hyz) + d1 * DP;
        f2 += X * (u0 * hxz + u1 * hyz + u2 * hzz) + d2 * DP;
      }
    }
    if (!in) f0 = f1 = f2 = 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      f0 += __shfl_xor_sync(0xffffffffu, f0, o);
      f1 += __shfl_xor_sync(0xffffffffu, f1, o);
      f2 += __shfl_xor_sync(0xffffffffu, f2, o);
    }
    if (lane == 0) {
      float *r = fred + ((long long)warp * n_atoms + A) * 3;
      r[0] = f0;
      r[1] = f1;
      r[2] = f2;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_atoms * 3; i += kFgThreads) {
    double s = 0;
    for (int w = 0; w < kFgWarps; ++w) s += (double)fred[(long long)w * n_atoms * 3 + i];
    part[(long long)blockIdx.x * n_atoms * 3 + i] = -2.0 * dV * s;
  }
}

// grad[i] += sum_blocks part[block][i]
__global__ void k_force_orb_reduce(const double *__restrict__ part, int nblk, int nvals,
                                   double *__restrict__ grad) {
  __shared__ double sh[32];
  const int i = blockIdx.x;
  double s = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[(long long)b * nvals + i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) grad[i] += s;
}

int force_orb_blocks(long long N) { return ceil_div(N, kFgThreads); }

void launch_force_operand(const double *C, const double *occ, int nao, int nuse, int npsi,
                          float *Y32, cudaStream_t st) {
  k_force_operand<<<ceil_div(nao * npsi, 256), 256, 0, st>>>(C, occ, nao, nuse, npsi, Y32);
  HQ_LAUNCH_CHECK();
}

void launch_to_float(long long n, const double *a, float *b, cudaStream_t st) {
  k_to_float<<<ceil_div(n, 256), 256, 0, st>>>(n, a, b);
  HQ_LAUNCH_CHECK();
}

void launch_force_grid_orb(const float *F32, const double *coef, const int *ao_l, const int *ao_cart,
                           int n_atoms, int nb, int nprim, int ng, const double *veff,
                           const double *u, const float *psi, const float *Y32, int npsi, double dV,
                           double *part, double *grad, cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  const long long N = (long long)ng * ng * ng;
  const int nblk = force_orb_blocks(N);
  const size_t sm = (size_t)kFgWarps * n_atoms * 3 * sizeof(float);
  HQ_REQUIRE(sm <= 48 * 1024, "too many atoms for the force reduction buffer");
  const bool gga = u != nullptr;
#define HQ_FG(NP)                                                                                 \
  (gga ? k_force_grid_orb<NP, true><<<nblk, kFgThreads, sm, st>>>(F32, coef, ao_l, ao_cart,       \
                                                                   n_atoms, nb, nprim, ng, veff, u, \
                                                                   psi, Y32, dV, part)            \
       : k_force_grid_orb<NP, false><<<nblk, kFgThreads, sm, st>>>(F32, coef, ao_l, ao_cart,      \
                                                                    n_atoms, nb, nprim, ng, veff, \
                                                                    u, psi, Y32, dV, part))
  switch (npsi) {
    case 16: HQ_FG(16); break;
    case 32: HQ_FG(32); break;
    case 48: HQ_FG(48); break;
    case 64: HQ_FG(64); break;
    default: throw Error{HQCGB_BAD_ARG, "force grid: orbital width must be 16, 32, 48 or 64"};
  }
#undef HQ_FG
  HQ_LAUNCH_CHECK();
  k_force_orb_reduce<<<n_atoms * 3, 256, 0, st>>>(part, nblk, n_atoms * 3, grad);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
