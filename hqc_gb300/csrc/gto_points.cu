// AO values at arbitrary points (electron positions), Gamma point: the
// reference's eval_pbc_ao (hqc/pbc/gto.py:326-369) -- per axis the 1D
// lattice sums  f_a^l(x) = sum_t (x - t L)^l exp(-alpha_a (x - t L)^2)  over
// t in [-tmax, tmax] (tmax = rcut // L), their product over the three axes
// and the contraction with the normalised coefficients (s: 1/sqrt(4 pi),
// p: sqrt(3 / (4 pi)) folded in).  Used by make_slater
// (hqc/pbc/slater.py:42-104) for walker batches.  FP64 throughout.  The
// k-point variant (eval_pbc_ao_kpt, gto.py:371-427) weights each lattice
// term with exp(i k_d t) and returns complex Bloch AO values.
#include "common.cuh"
#include "zmath.cuh"
#include "kernels.h"

namespace hqcgb {

constexpr int kPtMaxPrim = 16;

// One thread per (point, atom): out[pt][A * nb + j].
__global__ void k_ao_points(int n_atoms, int nb, int nprim, const double *__restrict__ alpha,
                            const double *__restrict__ coef, const int *__restrict__ ao_l,
                            const int *__restrict__ ao_cart, int nlat, const double *__restrict__ lat,
                            const double *__restrict__ xp, long long npts, int pts_per_group,
                            const double *__restrict__ xe, double *__restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npts * n_atoms) return;
  const int A = (int)(idx % n_atoms);
  const long long pt = idx / n_atoms;
  const long long grp = pt / pts_per_group;
  const double *xa = xp + (grp * n_atoms + A) * 3;
  const double *r = xe + pt * 3;
  // 1D factors f[d][a][l], l = 0, 1
  double f[3][kPtMaxPrim][2];
  for (int d = 0; d < 3; ++d) {
    const double x = r[d] - xa[d];
    for (int a = 0; a < nprim; ++a) {
      double s0 = 0, s1 = 0;
      for (int t = 0; t < nlat; ++t) {
        const double u = x - lat[t];
        const double g = exp(-alpha[a] * u * u);
        s0 += g;
        s1 += u * g;
      }
      f[d][a][0] = s0;
      f[d][a][1] = s1;
    }
  }
  const long long nao = (long long)n_atoms * nb;
  for (int j = 0; j < nb; ++j) {
    const int l = ao_l[j], ca = ao_cart[j];
    const int px = (l == 1 && ca == 0), py = (l == 1 && ca == 1), pz = (l == 1 && ca == 2);
    double v = 0;
    for (int a = 0; a < nprim; ++a)
      v += coef[j * nprim + a] * f[0][a][px] * f[1][a][py] * f[2][a][pz];
    out[pt * nao + (long long)A * nb + j] = v;
  }
}

}  // namespace hqcgb

// C ABI: AO values of n_atoms protons at npts points.  Basis tables as in
// the plan parameters (host pointers); xp [ngroups][n_atoms][3] and xe [npts][3]
// (device, Bohr), points grouped by pts_per_group per proton set; out
// [npts][n_atoms * nao_atom] (device).
extern "C" int hqcgb_ao_points(int n_atoms, int nao_atom, int n_prim, const double *alpha,
                               const double *coef, const int *ao_l, const int *ao_cart, int n_lat1d,
                               const double *lat1d, const double *xp, long long npts,
                               int pts_per_group, const double *xe, double *out, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(n_atoms >= 1 && nao_atom >= 1 && n_prim >= 1 && n_prim <= kPtMaxPrim && n_lat1d >= 1 &&
                   npts >= 0 && pts_per_group >= 1 && alpha && coef && ao_l && ao_cart && lat1d &&
                   xp && xe && out,
               "bad argument");
    for (int k = 0; k < nao_atom; ++k)
      HQ_REQUIRE((ao_l[k] == 0 || ao_l[k] == 1) && ao_cart[k] >= 0 && ao_cart[k] < 3,
                 "only s and p AOs are supported");
    if (npts == 0) return HQCGB_OK;
    const size_t nd = (size_t)n_prim + (size_t)nao_atom * n_prim + n_lat1d, ni = 2 * (size_t)nao_atom;
    StreamBuf blk(nd * sizeof(double) + ni * sizeof(int), st);
    double *d = blk.as<double>();
    int *iv = reinterpret_cast<int *>(d + nd);
    HQ_CUDA(cudaMemcpyAsync(d, alpha, n_prim * sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d + n_prim, coef, (size_t)nao_atom * n_prim * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d + n_prim + (size_t)nao_atom * n_prim, lat1d, n_lat1d * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(iv, ao_l, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(iv + nao_atom, ao_cart, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    const long long total = npts * n_atoms;
    k_ao_points<<<ceil_div(total, 128), 128, 0, st>>>(n_atoms, nao_atom, n_prim, d, d + n_prim, iv,
                                                      iv + nao_atom, n_lat1d,
                                                      d + n_prim + (size_t)nao_atom * n_prim, xp, npts,
                                                      pts_per_group, xe, out);
    HQ_LAUNCH_CHECK();
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

namespace hqcgb {
// M[p][k] = mo[p][idx[k]] for k < m (the Slater columns)
__global__ void k_gather_cols(const double *__restrict__ mo, int nao, int nmo,
                              const int *__restrict__ idx, int m, double *__restrict__ M) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nao * m) return;
  int p = i / m, k = i % m;
  M[i] = mo[(long long)p * nmo + idx[k]];
}
}  // namespace hqcgb

// C ABI: Slater matrices of W walkers (hqc/pbc/slater.py:42-70): up[w] =
// AO(xe[w][0:n/2]) mo[:, idx[0:n/2]], dn[w] = AO(xe[w][n/2:n]) mo[:, idx[n/2:n]].
// xp [xp_groups][n][3] with xp_groups 1 (shared protons) or W; xe [W][n][3]
// (device, Bohr); mo [nao][nmo] row-major (device); state_idx [n] (host);
// up, dn [W][n/2][n/2] (device).
extern "C" int hqcgb_slater(int n, int nao_atom, int n_prim, const double *alpha,
                            const double *coef, const int *ao_l, const int *ao_cart, int n_lat1d,
                            const double *lat1d, int W, int xp_groups, const double *xp,
                            const double *xe, const double *mo, int nmo, const int *state_idx,
                            double *up, double *dn, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(n >= 2 && n % 2 == 0 && W >= 1 && (xp_groups == 1 || xp_groups == W) && mo && up &&
                   dn && state_idx,
               "bad argument");
    const int n2 = n / 2, nao = n * nao_atom;
    for (int k = 0; k < n; ++k)
      HQ_REQUIRE(state_idx[k] >= 0 && state_idx[k] < nmo, "state index out of range");
    StreamBuf ao_buf((size_t)W * n * nao * sizeof(double), st), mu_buf((size_t)2 * nao * n2 * sizeof(double), st),
        idx_buf((size_t)n * sizeof(int), st);
    double *ao = ao_buf.as<double>(), *Mu = mu_buf.as<double>();
    int *idx = idx_buf.as<int>();
    HQ_CUDA(cudaMemcpyAsync(idx, state_idx, n * sizeof(int), cudaMemcpyHostToDevice, st));
    // AO values: with shared protons every point is in group 0
    const int ppg = xp_groups == 1 ? W * n : n;
    int s = hqcgb_ao_points(n, nao_atom, n_prim, alpha, coef, ao_l, ao_cart, n_lat1d, lat1d, xp,
                            (long long)W * n, ppg, xe, ao, stream);
    if (s != HQCGB_OK) throw Error{s, hqcgb_last_error()};
    k_gather_cols<<<ceil_div(nao * n2, 256), 256, 0, st>>>(mo, nao, nmo, idx, n2, Mu);
    HQ_LAUNCH_CHECK();
    k_gather_cols<<<ceil_div(nao * n2, 256), 256, 0, st>>>(mo, nao, nmo, idx + n2, n2,
                                                           Mu + (size_t)nao * n2);
    HQ_LAUNCH_CHECK();
    gemm_batched_rowmajor(n2, n2, nao, ao, nao, (long long)n * nao, Mu, n2, 0, up, n2,
                          (long long)n2 * n2, W, st);
    gemm_batched_rowmajor(n2, n2, nao, ao + (size_t)n2 * nao, nao, (long long)n * nao,
                          Mu + (size_t)nao * n2, n2, 0, dn, n2, (long long)n2 * n2, W, st);
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

namespace hqcgb {

// k-point AO values (complex): one thread per (point, atom), out[pt][A * nb + j].
__global__ void k_ao_points_kpt(int n_atoms, int nb, int nprim, const double *__restrict__ alpha,
                                const double *__restrict__ coef, const int *__restrict__ ao_l,
                                const int *__restrict__ ao_cart, int nlat,
                                const double *__restrict__ lat, double k0, double k1, double k2,
                                const double *__restrict__ xp, long long npts, int pts_per_group,
                                const double *__restrict__ xe, double2 *__restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npts * n_atoms) return;
  const int A = (int)(idx % n_atoms);
  const long long pt = idx / n_atoms;
  const long long grp = pt / pts_per_group;
  const double *xa = xp + (grp * n_atoms + A) * 3;
  const double *r = xe + pt * 3;
  const double kk[3] = {k0, k1, k2};
  double2 f[3][kPtMaxPrim][2];
  for (int d = 0; d < 3; ++d) {
    const double x = r[d] - xa[d];
    for (int a = 0; a < nprim; ++a) f[d][a][0] = f[d][a][1] = make_double2(0.0, 0.0);
    for (int t = 0; t < nlat; ++t) {
      const double u = x - lat[t];
      double sn, cs;
      sincos(kk[d] * lat[t], &sn, &cs);
      for (int a = 0; a < nprim; ++a) {
        const double g = exp(-alpha[a] * u * u);
        f[d][a][0].x += g * cs;
        f[d][a][0].y += g * sn;
        f[d][a][1].x += u * g * cs;
        f[d][a][1].y += u * g * sn;
      }
    }
  }
  const long long nao = (long long)n_atoms * nb;
  for (int j = 0; j < nb; ++j) {
    const int l = ao_l[j], ca = ao_cart[j];
    const int px = (l == 1 && ca == 0), py = (l == 1 && ca == 1), pz = (l == 1 && ca == 2);
    double2 v = make_double2(0.0, 0.0);
    for (int a = 0; a < nprim; ++a) {
      const double2 t = zmul(zmul(f[0][a][px], f[1][a][py]), f[2][a][pz]);
      v.x += coef[j * nprim + a] * t.x;
      v.y += coef[j * nprim + a] * t.y;
    }
    out[pt * nao + (long long)A * nb + j] = v;
  }
}

__global__ void k_gather_cols_z(const double2 *__restrict__ mo, int nao, int nmo,
                                const int *__restrict__ idx, int m, double2 *__restrict__ M) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nao * m) return;
  const int p = i / m, k = i % m;
  M[i] = mo[(long long)p * nmo + idx[k]];
}

}  // namespace hqcgb

// C ABI: k-point AO values (complex, interleaved) of n_atoms protons at npts
// points; arguments as hqcgb_ao_points plus kpt [3] (1/Bohr, host).
extern "C" int hqcgb_ao_points_kpt(int n_atoms, int nao_atom, int n_prim, const double *alpha,
                                   const double *coef, const int *ao_l, const int *ao_cart,
                                   int n_lat1d, const double *lat1d, const double *kpt,
                                   const double *xp, long long npts, int pts_per_group,
                                   const double *xe, double *out, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(n_atoms >= 1 && nao_atom >= 1 && n_prim >= 1 && n_prim <= kPtMaxPrim && n_lat1d >= 1 &&
                   npts >= 0 && pts_per_group >= 1 && alpha && coef && ao_l && ao_cart && lat1d &&
                   kpt && xp && xe && out,
               "bad argument");
    for (int k = 0; k < nao_atom; ++k)
      HQ_REQUIRE((ao_l[k] == 0 || ao_l[k] == 1) && ao_cart[k] >= 0 && ao_cart[k] < 3,
                 "only s and p AOs are supported");
    if (npts == 0) return HQCGB_OK;
    const size_t nd = (size_t)n_prim + (size_t)nao_atom * n_prim + n_lat1d, ni = 2 * (size_t)nao_atom;
    StreamBuf blk(nd * sizeof(double) + ni * sizeof(int), st);
    double *d = blk.as<double>();
    int *iv = reinterpret_cast<int *>(d + nd);
    HQ_CUDA(cudaMemcpyAsync(d, alpha, n_prim * sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d + n_prim, coef, (size_t)nao_atom * n_prim * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(d + n_prim + (size_t)nao_atom * n_prim, lat1d, n_lat1d * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(iv, ao_l, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaMemcpyAsync(iv + nao_atom, ao_cart, nao_atom * sizeof(int), cudaMemcpyHostToDevice, st));
    const long long total = npts * n_atoms;
    k_ao_points_kpt<<<ceil_div(total, 128), 128, 0, st>>>(
        n_atoms, nao_atom, n_prim, d, d + n_prim, iv, iv + nao_atom, n_lat1d,
        d + n_prim + (size_t)nao_atom * n_prim, kpt[0], kpt[1], kpt[2], xp, npts, pts_per_group, xe,
        reinterpret_cast<double2 *>(out));
    HQ_LAUNCH_CHECK();
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

// C ABI: k-point Slater matrices (hqc/pbc/slater.py:72-93): as hqcgb_slater
// with kpt [3] (host), complex mo [nao][nmo] and complex up, dn [W][n/2][n/2]
// (interleaved re, im).
extern "C" int hqcgb_slater_kpt(int n, int nao_atom, int n_prim, const double *alpha,
                                const double *coef, const int *ao_l, const int *ao_cart, int n_lat1d,
                                const double *lat1d, const double *kpt, int W, int xp_groups,
                                const double *xp, const double *xe, const double *mo, int nmo,
                                const int *state_idx, double *up, double *dn, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(n >= 2 && n % 2 == 0 && W >= 1 && (xp_groups == 1 || xp_groups == W) && mo && up &&
                   dn && state_idx && kpt,
               "bad argument");
    const int n2 = n / 2, nao = n * nao_atom;
    for (int k = 0; k < n; ++k)
      HQ_REQUIRE(state_idx[k] >= 0 && state_idx[k] < nmo, "state index out of range");
    StreamBuf ao_buf((size_t)W * n * nao * sizeof(double2), st),
        mu_buf((size_t)2 * nao * n2 * sizeof(double2), st), idx_buf((size_t)n * sizeof(int), st);
    double2 *ao = ao_buf.as<double2>(), *Mu = mu_buf.as<double2>();
    int *idx = idx_buf.as<int>();
    HQ_CUDA(cudaMemcpyAsync(idx, state_idx, n * sizeof(int), cudaMemcpyHostToDevice, st));
    const int ppg = xp_groups == 1 ? W * n : n;
    int s = hqcgb_ao_points_kpt(n, nao_atom, n_prim, alpha, coef, ao_l, ao_cart, n_lat1d, lat1d, kpt,
                                xp, (long long)W * n, ppg, xe, reinterpret_cast<double *>(ao), stream);
    if (s != HQCGB_OK) throw Error{s, hqcgb_last_error()};
    const double2 *moz = reinterpret_cast<const double2 *>(mo);
    k_gather_cols_z<<<ceil_div(nao * n2, 256), 256, 0, st>>>(moz, nao, nmo, idx, n2, Mu);
    HQ_LAUNCH_CHECK();
    k_gather_cols_z<<<ceil_div(nao * n2, 256), 256, 0, st>>>(moz, nao, nmo, idx + n2, n2,
                                                             Mu + (size_t)nao * n2);
    HQ_LAUNCH_CHECK();
    zgemm_batched_rowmajor(n2, n2, nao, ao, nao, (long long)n * nao, Mu, n2, 0,
                           reinterpret_cast<double2 *>(up), n2, (long long)n2 * n2, W, st);
    zgemm_batched_rowmajor(n2, n2, nao, ao + (size_t)n2 * nao, nao, (long long)n * nao,
                           Mu + (size_t)nao * n2, n2, 0, reinterpret_cast<double2 *>(dn), n2,
                           (long long)n2 * n2, W, st);
    HQ_CUDA(cudaStreamSynchronize(st));
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
