// Standalone overlap (and kinetic) matrices without a plan: make_overlap of
// hqc/pbc/overlap.py:11-319 (Gamma: real S; k-point: complex Hermitian S^k
// with exp(-i k.t) lattice weights), for a batch of configurations.  The
// integrals are the lattice-summed Hermite forms of integrals_fp64.cu.
#include "common.cuh"
#include "kernels.h"

// xp [n_cfg][n_atoms][3] (device, Bohr); kpts [n_cfg][3] (host, 1/Bohr) or
// NULL for the Gamma point; S, T [n_cfg][nao][nao] (device; complex
// interleaved with kpts), T may be NULL.
extern "C" int hqcgb_overlap(int n_atoms, int nao_atom, int n_prim, const double *alpha,
                             const double *coef, const int *ao_l, const int *ao_cart, int n_lattice,
                             const double *lattice, int n_cfg, const double *xp, const double *kpts,
                             double *S, double *T, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(n_atoms >= 1 && nao_atom >= 1 && n_prim >= 1 && n_lattice >= 1 && n_cfg >= 0 && alpha &&
                   coef && ao_l && ao_cart && lattice && xp && S && n_atoms * nao_atom <= kMaxNao,
               "bad argument");
    for (int k = 0; k < nao_atom; ++k)
      HQ_REQUIRE((ao_l[k] == 0 || ao_l[k] == 1) && ao_cart[k] >= 0 && ao_cart[k] < 3,
                 "only s and p AOs are supported");
    if (n_cfg == 0) return HQCGB_OK;
    const bool kp = kpts != nullptr;
    const int nao = n_atoms * nao_atom;
    const size_t nn = (size_t)nao * nao, cw = kp ? 2 : 1;  // doubles per element
    const size_t nq = kp ? ovl_scratch_doubles_kpt(n_atoms, n_prim) : ovl_scratch_doubles(n_atoms, n_prim);
    const size_t nd = (size_t)n_prim + (size_t)nao_atom * n_prim + 3 * (size_t)n_lattice + 3 + nq +
                      (T ? 0 : cw * nn);
    StreamBuf blk(nd * sizeof(double) + 2 * (size_t)nao_atom * sizeof(int), st);
    double *d_alpha = blk.as<double>(), *d_coef = d_alpha + n_prim,
           *d_lat = d_coef + (size_t)nao_atom * n_prim, *d_k = d_lat + 3 * (size_t)n_lattice,
           *d_q = d_k + 3, *d_t = d_q + nq;
    int *d_l = reinterpret_cast<int *>(d_alpha + nd), *d_c = d_l + nao_atom;
    HQ_CUDA(cudaMemcpyAsync(d_alpha, alpha, n_prim * sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d_coef, coef, (size_t)nao_atom * n_prim * sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d_lat, lattice, 3 * (size_t)n_lattice * sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d_l, ao_l, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d_c, ao_cart, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    for (int b = 0; b < n_cfg; ++b) {
      const double *x = xp + (size_t)b * 3 * n_atoms;
      double *Sb = S + (size_t)b * cw * nn, *Tb = T ? T + (size_t)b * cw * nn : d_t;
      if (kp) {
        HQ_CUDA(cudaMemcpyAsync(d_k, kpts + 3 * (size_t)b, 3 * sizeof(double), cudaMemcpyHostToDevice, st));
        launch_overlap_kinetic_kpt(x, n_atoms, nao_atom, n_prim, d_alpha, d_coef, d_l, d_c, d_lat, n_lattice,
                                   d_k, reinterpret_cast<double2 *>(Sb), reinterpret_cast<double2 *>(Tb),
                                   d_q, st);
      } else {
        launch_overlap_kinetic(x, n_atoms, nao_atom, n_prim, d_alpha, d_coef, d_l, d_c, d_lat, n_lattice, Sb,
                               T ? Tb : nullptr, nullptr, nullptr, nullptr, nullptr, d_q, st);
      }
    }
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
