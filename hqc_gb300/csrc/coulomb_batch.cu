// Ewald energy of proton + electron configurations, batched over walkers:
// potential_energy of hqc/pbc/potential.py:69-101 (with psi, 35-67).  For
// each configuration x [n][dim] (rs units; the first n/2 particles are
// protons, Z = +1, the rest electrons, Z = -1) it returns
//   vpp =  2 rs / L sum_{i<j, pp} psi(r_ij),  vep = -2 rs / L sum_{ep} psi,
//   vee =  2 rs / L sum_{i<j, ee} psi,
//   psi(r) = erfc(kappa |r|) / |r|  (nearest image)  + sum_G g(G) cos(2 pi G.r) + g0,
// r_ij = (x_i - x_j) / L wrapped to the nearest image, G the caller's integer
// vectors (kpoints(dim, Gmax), potential.py:6-16).
//
// The reciprocal part is not summed pair by pair: with the species structure
// factors S_A(G) = sum_{i in A} exp(2 pi i G.x_i / L),
//   sum_{i<j in A} cos(2 pi G.r_ij) = (|S_A|^2 - n_A) / 2,
//   sum_{i in p, j in e} cos(2 pi G.r_ij) = Re(S_p conj(S_e)),
// so a configuration costs n N_G phase evaluations instead of n^2 N_G / 2
// (integer G makes the nearest-image shift irrelevant to the cosine).  The
// real-space erfc term stays pairwise (n^2 / 2, no G loop).
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kCbThreads = 256;
constexpr int kCbMaxParticles = 2048;

__device__ inline double coul_gk(int dim, double G2, double kappa) {
  if (dim == 3) return exp(-M_PI * M_PI * G2 / (kappa * kappa)) / (M_PI * G2);
  const double g = sqrt(G2);
  return erfc(M_PI * g / kappa) / g;
}

// Grid (B, ceil(nG / 256)); one thread per G vector of configuration b.
// part[b][blockIdx.y][3] = sum over this block's G of g(G) x {pp, ep, ee} cosine sums.
__global__ void __launch_bounds__(kCbThreads)
    k_coul_recip(int n, int dim, const double *__restrict__ x, double L, const int *__restrict__ G,
                 int nG, double kappa, double *__restrict__ part) {
  extern __shared__ double xs[];  // [n][dim] / L
  __shared__ double sh[32];
  const int b = blockIdx.x;
  const double *xb = x + (long long)b * n * dim;
  for (int k = threadIdx.x; k < n * dim; k += blockDim.x) xs[k] = xb[k] / L;
  __syncthreads();
  const int np = n / 2;
  const int gi = blockIdx.y * blockDim.x + threadIdx.x;
  double vpp = 0, vep = 0, vee = 0;
  if (gi < nG) {
    int g[3] = {0, 0, 0};
    double G2 = 0;
    for (int d = 0; d < dim; ++d) {
      g[d] = G[gi * dim + d];
      G2 += (double)g[d] * g[d];
    }
    double spr = 0, spi = 0, ser = 0, sei = 0;
    for (int i = 0; i < n; ++i) {
      double ph = 0;
      for (int d = 0; d < dim; ++d) ph += g[d] * xs[i * dim + d];
      double s, c;
      sincospi(2.0 * ph, &s, &c);
      if (i < np) {
        spr += c;
        spi += s;
      } else {
        ser += c;
        sei += s;
      }
    }
    const double gk = coul_gk(dim, G2, kappa);
    vpp = gk * 0.5 * (spr * spr + spi * spi - np);
    vee = gk * 0.5 * (ser * ser + sei * sei - (n - np));
    vep = gk * (spr * ser + spi * sei);
  }
  vpp = block_sum(vpp, sh);
  vep = block_sum(vep, sh);
  vee = block_sum(vee, sh);
  if (threadIdx.x == 0) {
    double *o = part + ((long long)b * gridDim.y + blockIdx.y) * 3;
    o[0] = vpp;
    o[1] = vep;
    o[2] = vee;
  }
}

// One block per configuration: the nearest-image erfc sums, then the total.
__global__ void __launch_bounds__(kCbThreads)
    k_coul_real_finish(int n, int dim, const double *__restrict__ x, double L, double rs, double kappa,
                       double g0, const double *__restrict__ part, int nblk, double *__restrict__ out) {
  extern __shared__ double xw[];  // [n][dim], wrapped into [0, L)
  __shared__ double sh[32];
  const int b = blockIdx.x;
  const double *xb = x + (long long)b * n * dim;
  for (int k = threadIdx.x; k < n * dim; k += blockDim.x) xw[k] = xb[k] - L * floor(xb[k] / L);
  __syncthreads();
  const int np = n / 2;
  double vpp = 0, vep = 0, vee = 0;
  for (long long k = threadIdx.x; k < (long long)n * n; k += blockDim.x) {
    const int i = (int)(k / n), j = (int)(k % n);
    if (j <= i) continue;
    double d2 = 0;
    for (int d = 0; d < dim; ++d) {
      double r = (xw[i * dim + d] - xw[j * dim + d]) / L;
      r -= rint(r);
      d2 += r * r;
    }
    const double dd = sqrt(d2);
    const double v = erfc(kappa * dd) / dd;
    if (j < np) vpp += v;
    else if (i >= np) vee += v;
    else vep += v;
  }
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
    const double *o = part + ((long long)b * nblk + k) * 3;
    vpp += o[0];
    vep += o[1];
    vee += o[2];
  }
  vpp = block_sum(vpp, sh);
  vep = block_sum(vep, sh);
  vee = block_sum(vee, sh);
  if (threadIdx.x == 0) {
    const double ne = n - np;
    const double f = 2.0 * rs / L;
    out[b * 3 + 0] = f * (vpp + 0.5 * np * (np - 1) * g0);
    out[b * 3 + 1] = -f * (vep + (double)np * ne * g0);
    out[b * 3 + 2] = f * (vee + 0.5 * ne * (ne - 1) * g0);
  }
}

}  // namespace hqcgb

// C ABI: potential_energy (hqc/pbc/potential.py:69-101) of B configurations
// x [B][n][dim] (device, rs units; first n/2 protons), box L (rs units), G
// [nG][dim] integer vectors (host), out [B][3] = (vpp, vep, vee) (device).
extern "C" int hqcgb_coulomb_energy(int B, int n, int dim, const double *x, double L, double rs,
                                    double kappa, int nG, const int *G, double *out, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(B >= 0 && n >= 2 && n % 2 == 0 && n <= kCbMaxParticles && (dim == 2 || dim == 3) &&
                   L > 0 && kappa > 0 && nG >= 0 && (nG == 0 || G) && x && out,
               "bad argument");
    for (long long k = 0; k < (long long)nG * dim; ++k) HQ_REQUIRE(G[k] > -100000 && G[k] < 100000, "bad G");
    for (int k = 0; k < nG; ++k) {
      bool zero = true;
      for (int d = 0; d < dim; ++d) zero = zero && G[k * dim + d] == 0;
      HQ_REQUIRE(!zero, "G = 0 is not part of the reciprocal sum");
    }
    if (B == 0) return HQCGB_OK;
    HQ_STAGE(ST_EWALD, st);
    const int nblk = nG > 0 ? ceil_div(nG, kCbThreads) : 0;
    const size_t gbytes = ((size_t)nG * dim * sizeof(int) + 15) / 16 * 16;
    StreamBuf blk(gbytes + (size_t)B * std::max(nblk, 1) * 3 * sizeof(double), st);
    int *Gd = blk.as<int>();
    double *part = blk.as<double>(gbytes);
    if (nG > 0) HQ_CUDA(cudaMemcpyAsync(Gd, G, (size_t)nG * dim * sizeof(int), cudaMemcpyHostToDevice, st));
    const size_t smem = (size_t)n * dim * sizeof(double);
    if (nblk > 0) {
      k_coul_recip<<<dim3(B, nblk), kCbThreads, smem, st>>>(n, dim, x, L, Gd, nG, kappa, part);
      HQ_LAUNCH_CHECK();
    }
    const double g0 = dim == 3 ? -M_PI / (kappa * kappa) : -2.0 * std::sqrt(M_PI) / kappa;
    k_coul_real_finish<<<B, kCbThreads, smem, st>>>(n, dim, x, L, rs, kappa, g0, part, nblk, out);
    HQ_LAUNCH_CHECK();
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
