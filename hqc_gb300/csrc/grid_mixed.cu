// Grid data of the mixed-precision path: FP32 AO values / gradients with a
// padded row stride (rows 256-byte aligned for vector loads; the padding is
// zero), and FP64 <-> FP32 conversions of grid vectors and small matrices.
// The 1D factor table is built in FP64 (hqc/pbc/gto.py:326-369) and rounded
// to FP32 once per geometry for the AO grid evaluation.
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

// The same values in FP32 arithmetic from an FP32 copy of the factor table
// (FP64 arithmetic runs at 1/64 of the FP32 rate on GB300; the products of
// three rounded factors carry unbiased relative errors of a few 1e-7, the
// precision the grid is stored in anyway).  One thread per (AO, point):
// value and, when requested, the three derivatives share the factor loads.
__global__ void k_phi32_f(const float *__restrict__ F, const double *__restrict__ coef,
                          const int *__restrict__ ao_l, const int *__restrict__ ao_cart,
                          int nao_atom, int nprim, int nao, int ng, long long ld,
                          float *__restrict__ phi, float *__restrict__ dphi) {
  const long long N = (long long)ng * ng * ng;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nao * ld) return;
  const int p = (int)(idx / ld);
  const long long g = idx - (long long)p * ld;
  if (g >= N) {
    phi[idx] = 0.f;
    if (dphi)
      for (int d = 0; d < 3; ++d) dphi[(long long)d * nao * ld + idx] = 0.f;
    return;
  }
  const int iz = (int)(g % ng), iy = (int)((g / ng) % ng), ix = (int)(g / ((long long)ng * ng));
  const int A = p / nao_atom, k = p % nao_atom, l = ao_l[k], ca = ao_cart[k];
  const int bx = (l == 1 && ca == 0) ? 3 : 0, by = (l == 1 && ca == 1) ? 3 : 0,
            bz = (l == 1 && ca == 2) ? 3 : 0;
  const float *fxb = F + (((long long)A * 3 + 0) * ng + ix) * nprim * 6 + bx;
  const float *fyb = F + (((long long)A * 3 + 1) * ng + iy) * nprim * 6 + by;
  const float *fzb = F + (((long long)A * 3 + 2) * ng + iz) * nprim * 6 + bz;
  float v = 0.f, d0 = 0.f, d1 = 0.f, d2 = 0.f;
  for (int a = 0; a < nprim; ++a) {
    const float c = (float)coef[k * nprim + a];
    const float x0 = fxb[a * 6], y0 = fyb[a * 6], z0 = fzb[a * 6];
    const float cyz = c * y0 * z0;
    v = fmaf(x0, cyz, v);
    if (dphi) {
      d0 = fmaf(fxb[a * 6 + 1], cyz, d0);
      d1 = fmaf(fyb[a * 6 + 1], c * x0 * z0, d1);
      d2 = fmaf(fzb[a * 6 + 1], c * x0 * y0, d2);
    }
  }
  phi[idx] = v;
  if (dphi) {
    const long long s = (long long)nao * ld;
    dphi[idx] = d0;
    dphi[s + idx] = d1;
    dphi[2 * s + idx] = d2;
  }
}

void launch_phi32(const float *F32, const double *coef, const int *ao_l, const int *ao_cart,
                  int nao_atom, int nprim, int nao, int ng, long long ld, float *phi, float *dphi,
                  cudaStream_t st) {
  HQ_STAGE(ST_PHI, st);
  long long total = (long long)nao * ld;
  k_phi32_f<<<ceil_div(total, 256), 256, 0, st>>>(F32, coef, ao_l, ao_cart, nao_atom, nprim, nao, ng,
                                                   ld, phi, dphi);
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
