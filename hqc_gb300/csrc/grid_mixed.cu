// Grid data of the mixed-precision path: FP32 AO values / gradients with a
// padded row stride (rows 256-byte aligned for vector loads; the padding is
// zero), and FP64 <-> FP32 conversions of grid vectors and small matrices.
// The 1D factor table and everything it is built from stay FP64
// (hqc/pbc/gto.py:326-369); only the stored AO grid is rounded to FP32.
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

__device__ inline double ao_eval_m(const double *__restrict__ F, const double *__restrict__ coef,
                                   int nprim, int ng, int A, int l, int cart, int ix, int iy, int iz,
                                   int c1) {
  int pw[3] = {0, 0, 0};
  if (l == 1) pw[cart] = 1;
  int kd[3] = {0, 0, 0};
  if (c1 >= 0) kd[c1] = 1;
  const double *fx = F + ((((long long)A * 3 + 0) * ng + ix) * nprim) * 6 + 3 * pw[0] + kd[0];
  const double *fy = F + ((((long long)A * 3 + 1) * ng + iy) * nprim) * 6 + 3 * pw[1] + kd[1];
  const double *fz = F + ((((long long)A * 3 + 2) * ng + iz) * nprim) * 6 + 3 * pw[2] + kd[2];
  double v = 0.0;
  for (int a = 0; a < nprim; ++a) v += coef[a] * fx[a * 6] * fy[a * 6] * fz[a * 6];
  return v;
}

// phi32[p][g] (row stride ld), dphi32[c][p][g] when requested; g in [N, ld) zeroed.
__global__ void k_phi32(const double *__restrict__ F, const double *__restrict__ coef,
                        const int *__restrict__ ao_l, const int *__restrict__ ao_cart, int nao_atom,
                        int nprim, int nao, int ng, long long ld, float *__restrict__ phi,
                        float *__restrict__ dphi) {
  long long N = (long long)ng * ng * ng;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nao * ld) return;
  int p = (int)(idx / ld);
  long long g = idx - (long long)p * ld;
  if (g >= N) {
    phi[idx] = 0.f;
    if (dphi)
      for (int d = 0; d < 3; ++d) dphi[(long long)d * nao * ld + idx] = 0.f;
    return;
  }
  int iz = g % ng, iy = (g / ng) % ng, ix = (int)(g / ((long long)ng * ng));
  int A = p / nao_atom, k = p % nao_atom;
  const double *c = coef + k * nprim;
  phi[idx] = (float)ao_eval_m(F, c, nprim, ng, A, ao_l[k], ao_cart[k], ix, iy, iz, -1);
  if (dphi)
    for (int d = 0; d < 3; ++d)
      dphi[(long long)d * nao * ld + idx] =
          (float)ao_eval_m(F, c, nprim, ng, A, ao_l[k], ao_cart[k], ix, iy, iz, d);
}

void launch_phi32(const double *F, const double *coef, const int *ao_l, const int *ao_cart,
                  int nao_atom, int nprim, int nao, int ng, long long ld, float *phi, float *dphi,
                  cudaStream_t st) {
  HQ_STAGE(ST_PHI, st);
  long long total = (long long)nao * ld;
  k_phi32<<<ceil_div(total, 256), 256, 0, st>>>(F, coef, ao_l, ao_cart, nao_atom, nprim, nao, ng, ld,
                                                 phi, dphi);
  HQ_LAUNCH_CHECK();
}

// out[r][g] (stride ldo) = scale * in[r][g] (stride ldi) for g < N, 0 for N <= g < ldo
__global__ void k_to_f32(const double *__restrict__ in, long long ldi, long long N, int rows,
                         double scale, float *__restrict__ out, long long ldo) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * ldo) return;
  int r = (int)(idx / ldo);
  long long g = idx - (long long)r * ldo;
  out[idx] = (g < N) ? (float)(scale * in[(long long)r * ldi + g]) : 0.f;
}

void launch_to_f32(const double *in, long long ldi, long long N, int rows, double scale, float *out,
                   long long ldo, cudaStream_t st) {
  long long total = (long long)rows * ldo;
  k_to_f32<<<ceil_div(total, 256), 256, 0, st>>>(in, ldi, N, rows, scale, out, ldo);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
