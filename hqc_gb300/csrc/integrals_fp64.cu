// Analytic lattice-summed overlap / kinetic integrals and the Ewald sum (FP64).
//
// S and T follow hqc/pbc/solver.py:240-389: primitive s-s integrals summed
// over the lattice sphere, p functions obtained as derivatives with respect
// to the centres (the reference uses jacfwd).  Here those derivatives are
// closed-form Hermite derivatives of exp(-mu |R+t|^2); T = -1/2 lap_R S for
// s primitives, so every kinetic derivative is a sum of overlap derivatives.
// With forces, one more derivative gives dS/dR and dT/dR.
//
// The Ewald energy follows hqc/pbc/potential.py:6-67,103-130 (nearest-image
// real space, reciprocal sphere |G| <= Gmax, Madelung self term, Rydberg).
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

// h[n] = (d^n/dx^n e^{-mu x^2}) / e^{-mu x^2}, n = 0..5
__device__ inline void hermite6(double mu, double x, double *h) {
  h[0] = 1.0;
  h[1] = -2.0 * mu * x;
  for (int k = 1; k < 5; ++k) h[k + 1] = -2.0 * mu * x * h[k] - 2.0 * k * mu * h[k - 1];
}

struct AOInfo {
  int l, cart;
};

// Two passes.  (1) One thread per (atom pair i, j; primitive pair a, b)
// accumulates over the lattice sphere the Hermite products
//   QS[m] = K_ab sum_t e_t h_m0(u_x) h_m1(u_y) h_m2(u_z),
//   QT[m] = K_ab sum_t e_t sum_d h_{m + 2 e_d}(u),   e_t = exp(-mu |R + t|^2),
// for every multi-index m an s/p pair needs: |m| <= 2 for S and T, |m| <= 3
// for their first derivatives (K_ab = (pi / (a + b))^(3/2)).  The exponential
// and the Hermite factors of a lattice term are computed once for all AO
// pairs.  (2) One thread per (i, j, p, q) contracts them with the
// coefficients: S_pq = sum_ab c'_pa c'_qb QS[m(p,q)], T = -1/2 (same with QT),
// and, with forces, the contribution D_pq dT/dR_i - W_pq dS/dR_i
// (R = R_i - R_j; the derivative with respect to R_j is its negative).
__constant__ int kMidx[20][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
                                 {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1},
                                 {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1},
                                 {1, 2, 0}, {0, 2, 1}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1}};
constexpr int kNq = 20;  // slots per (i, j, a, b): QS[20], QT[20]

__device__ inline int midx_of(int m0, int m1, int m2) {
  for (int k = 0; k < kNq; ++k)
    if (kMidx[k][0] == m0 && kMidx[k][1] == m1 && kMidx[k][2] == m2) return k;
  return 0;
}

// KPT: each lattice term also carries exp(-i k.t) (hqc/pbc/solver.py:257-274);
// the real and imaginary sums are stored side by side, Q[(i,j,a,b)][4][kNq] =
// {QS re, QT re, QS im, QT im}.
template <int NQ, bool KPT>
__global__ void k_ovl_lattice(const double *__restrict__ xp, int n, int nprim,
                              const double *__restrict__ alpha, const double *__restrict__ lattice,
                              int nlat, const double *__restrict__ kpt, double *__restrict__ Q) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int np2 = nprim * nprim;
  if (idx >= (long long)n * n * np2) return;
  // atom pairs fastest: a warp shares one primitive pair (one mu), so its
  // lanes skip the same far lattice terms
  const int ab = (int)(idx / ((long long)n * n)), a = ab / nprim, b = ab % nprim;
  const int ij = (int)(idx % ((long long)n * n)), i = ij / n, j = ij % n;
  double R[3];
  for (int d = 0; d < 3; ++d) R[d] = xp[i * 3 + d] - xp[j * 3 + d];
  const double asum = alpha[a] + alpha[b];
  const double mu = alpha[a] * alpha[b] / asum;
  const double K = pow(M_PI / asum, 1.5);
  double qs[NQ], qt[NQ], qsi[KPT ? NQ : 1], qti[KPT ? NQ : 1];
#pragma unroll
  for (int k = 0; k < NQ; ++k) qs[k] = qt[k] = 0.0;
  if (KPT)
#pragma unroll
    for (int k = 0; k < NQ; ++k) qsi[k] = qti[k] = 0.0;
  for (int t = 0; t < nlat; ++t) {
    double u[3], u2 = 0;
    for (int d = 0; d < 3; ++d) {
      u[d] = R[d] + lattice[t * 3 + d];
      u2 += u[d] * u[d];
    }
    double e = mu * u2;
    // exp(-60) times the largest Hermite factor (degree <= 5) is below 1e-18
    // of every matrix element: far images add nothing in FP64
    if (e > 60.0) continue;
    e = K * exp(-e);
    double ei = 0.0;
    if (KPT) {
      double sn, cs;
      sincos(-(kpt[0] * lattice[t * 3] + kpt[1] * lattice[t * 3 + 1] + kpt[2] * lattice[t * 3 + 2]),
             &sn, &cs);
      ei = e * sn;
      e *= cs;
    }
    double hx[6], hy[6], hz[6];
    hermite6(mu, u[0], hx);
    hermite6(mu, u[1], hy);
    hermite6(mu, u[2], hz);
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int m0 = kMidx[k][0], m1 = kMidx[k][1], m2 = kMidx[k][2];
      const double hs = hx[m0] * hy[m1] * hz[m2];
      const double ht = hx[m0 + 2] * hy[m1] * hz[m2] + hx[m0] * hy[m1 + 2] * hz[m2] +
                        hx[m0] * hy[m1] * hz[m2 + 2];
      qs[k] += e * hs;
      qt[k] += e * ht;
      if (KPT) {
        qsi[k] += ei * hs;
        qti[k] += ei * ht;
      }
    }
  }
  double *out = Q + (((long long)i * n + j) * np2 + ab) * ((KPT ? 4 : 2) * kNq);
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    out[k] = qs[k];
    out[kNq + k] = qt[k];
    if (KPT) {
      out[2 * kNq + k] = qsi[k];
      out[3 * kNq + k] = qti[k];
    }
  }
}

__global__ void k_ovl_contract(int n, int nb, int nprim, const double *__restrict__ alpha,
                               const double *__restrict__ coef, const int *__restrict__ ao_l,
                               const int *__restrict__ ao_cart, const double *__restrict__ Q,
                               double *__restrict__ S, double *__restrict__ T,
                               const double *__restrict__ D, const double *__restrict__ W,
                               double *__restrict__ gpart) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n * nb * nb) return;
  const int q = (int)(idx % nb), p = (int)((idx / nb) % nb);
  const int j = (int)((idx / ((long long)nb * nb)) % n), i = (int)(idx / ((long long)nb * nb * n));
  const int nao = n * nb, np2 = nprim * nprim;
  const int lp = ao_l[p], lq = ao_l[q];
  int mb[3] = {0, 0, 0};
  if (lp) mb[ao_cart[p]] += 1;
  if (lq) mb[ao_cart[q]] += 1;
  const bool grad = gpart != nullptr;
  const int ks = midx_of(mb[0], mb[1], mb[2]);
  int kc[3];
  for (int c = 0; c < 3; ++c) kc[c] = midx_of(mb[0] + (c == 0), mb[1] + (c == 1), mb[2] + (c == 2));
  double sS = 0, sT = 0, gS[3] = {0, 0, 0}, gT[3] = {0, 0, 0};
  const double *Qij = Q + ((long long)i * n + j) * np2 * (2 * kNq);
  for (int a = 0; a < nprim; ++a) {
    double ca = coef[p * nprim + a];
    if (ca == 0.0) continue;
    if (lp) ca *= 0.5 / alpha[a];
    for (int b = 0; b < nprim; ++b) {
      double cb = coef[q * nprim + b];
      if (cb == 0.0) continue;
      if (lq) cb *= -0.5 / alpha[b];
      const double cc = ca * cb;
      const double *qv = Qij + (long long)(a * nprim + b) * (2 * kNq);
      sS += cc * qv[ks];
      sT += cc * qv[kNq + ks];
      if (grad)
        for (int c = 0; c < 3; ++c) {
          gS[c] += cc * qv[kc[c]];
          gT[c] += cc * qv[kNq + kc[c]];
        }
    }
  }
  const long long pq = (long long)(i * nb + p) * nao + (j * nb + q);
  if (S) S[pq] = sS;
  if (T) T[pq] = -0.5 * sT;
  if (grad) {
    const double dd = D[pq], ww = W[pq];
    for (int c = 0; c < 3; ++c) gpart[idx * 3 + c] = (i == j) ? 0.0 : dd * (-0.5 * gT[c]) - ww * gS[c];
  }
}

// k-point contraction: complex S, T (interleaved) from the phase-weighted
// sums and, with gpart, Re[conj(D_pq) dT_pq - conj(W_pq) dS_pq] per (i, j, p, q)
// (Re tr(D dT) for Hermitian D: sum_pq D_qp dT_pq = sum_pq conj(D_pq) dT_pq).
__global__ void k_ovl_contract_kpt(int n, int nb, int nprim, const double *__restrict__ alpha,
                                   const double *__restrict__ coef, const int *__restrict__ ao_l,
                                   const int *__restrict__ ao_cart, const double *__restrict__ Q,
                                   double2 *__restrict__ S, double2 *__restrict__ T,
                                   const double2 *__restrict__ D, const double2 *__restrict__ W,
                                   double *__restrict__ gpart) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n * nb * nb) return;
  const int q = (int)(idx % nb), p = (int)((idx / nb) % nb);
  const int j = (int)((idx / ((long long)nb * nb)) % n), i = (int)(idx / ((long long)nb * nb * n));
  const int nao = n * nb, np2 = nprim * nprim;
  const int lp = ao_l[p], lq = ao_l[q];
  int mb[3] = {0, 0, 0};
  if (lp) mb[ao_cart[p]] += 1;
  if (lq) mb[ao_cart[q]] += 1;
  const int ks = midx_of(mb[0], mb[1], mb[2]);
  const bool grad = gpart != nullptr;
  int kc[3];
  for (int c = 0; c < 3; ++c) kc[c] = midx_of(mb[0] + (c == 0), mb[1] + (c == 1), mb[2] + (c == 2));
  double sS = 0, sT = 0, sSi = 0, sTi = 0;
  double gS[3] = {0, 0, 0}, gT[3] = {0, 0, 0}, gSi[3] = {0, 0, 0}, gTi[3] = {0, 0, 0};
  const double *Qij = Q + ((long long)i * n + j) * np2 * (4 * kNq);
  for (int a = 0; a < nprim; ++a) {
    double ca = coef[p * nprim + a];
    if (ca == 0.0) continue;
    if (lp) ca *= 0.5 / alpha[a];
    for (int b = 0; b < nprim; ++b) {
      double cb = coef[q * nprim + b];
      if (cb == 0.0) continue;
      if (lq) cb *= -0.5 / alpha[b];
      const double cc = ca * cb;
      const double *qv = Qij + (long long)(a * nprim + b) * (4 * kNq);
      sS += cc * qv[ks];
      sT += cc * qv[kNq + ks];
      sSi += cc * qv[2 * kNq + ks];
      sTi += cc * qv[3 * kNq + ks];
      if (grad)
        for (int c = 0; c < 3; ++c) {
          gS[c] += cc * qv[kc[c]];
          gT[c] += cc * qv[kNq + kc[c]];
          gSi[c] += cc * qv[2 * kNq + kc[c]];
          gTi[c] += cc * qv[3 * kNq + kc[c]];
        }
    }
  }
  const long long pq = (long long)(i * nb + p) * nao + (j * nb + q);
  if (S) S[pq] = make_double2(sS, sSi);
  if (T) T[pq] = make_double2(-0.5 * sT, -0.5 * sTi);
  if (grad) {
    const double2 dd = D[pq], ww = W[pq];
    for (int c = 0; c < 3; ++c)
      gpart[idx * 3 + c] = (i == j) ? 0.0
                                    : -0.5 * (dd.x * gT[c] + dd.y * gTi[c]) - (ww.x * gS[c] + ww.y * gSi[c]);
  }
}

size_t ovl_scratch_doubles(int n, int nprim) {
  return (size_t)n * n * nprim * nprim * 2 * kNq;
}
size_t ovl_scratch_doubles_kpt(int n, int nprim) {
  return (size_t)n * n * nprim * nprim * 4 * kNq;
}

// grad[A][c] += sum_{j,p,q} gpart(A,j,p,q) - sum_{i,p,q} gpart(i,A,p,q)
__global__ void k_reduce_pair_grad(const double *__restrict__ gpart, int n, int nb,
                                   double *__restrict__ grad) {
  __shared__ double sh[32];
  int A = blockIdx.x;
  long long per = (long long)nb * nb;
  for (int c = 0; c < 3; ++c) {
    double s = 0;
    for (long long k = threadIdx.x; k < (long long)n * per; k += blockDim.x) {
      int o = (int)(k / per);
      long long pq = k % per;
      s += gpart[(((long long)A * n + o) * per + pq) * 3 + c];
      s -= gpart[(((long long)o * n + A) * per + pq) * 3 + c];
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) grad[A * 3 + c] += s;
    __syncthreads();
  }
}

void launch_overlap_kinetic(const double *xp, int n, int nb, int nprim, const double *alpha,
                            const double *coef, const int *ao_l, const int *ao_cart,
                            const double *lattice, int nlat, double *S, double *T, const double *D,
                            const double *W, double *gpart, double *grad, double *Q,
                            cudaStream_t st) {
  HQ_STAGE(ST_OVERLAP, st);
  const long long terms = (long long)n * n * nprim * nprim;
  if (gpart)
    k_ovl_lattice<20, false><<<ceil_div(terms, 128), 128, 0, st>>>(xp, n, nprim, alpha, lattice, nlat,
                                                                   nullptr, Q);
  else
    k_ovl_lattice<10, false><<<ceil_div(terms, 128), 128, 0, st>>>(xp, n, nprim, alpha, lattice, nlat,
                                                                   nullptr, Q);
  HQ_LAUNCH_CHECK();
  const long long total = (long long)n * n * nb * nb;
  k_ovl_contract<<<ceil_div(total, 128), 128, 0, st>>>(n, nb, nprim, alpha, coef, ao_l, ao_cart, Q, S,
                                                      T, D, W, gpart);
  HQ_LAUNCH_CHECK();
  if (gpart) {
    k_reduce_pair_grad<<<n, 256, 0, st>>>(gpart, n, nb, grad);
    HQ_LAUNCH_CHECK();
  }
}

// S^k, T^k at k-point kpt (device, 1/Bohr): complex Hermitian, interleaved.
void launch_overlap_kinetic_kpt(const double *xp, int n, int nb, int nprim, const double *alpha,
                                const double *coef, const int *ao_l, const int *ao_cart,
                                const double *lattice, int nlat, const double *kpt, double2 *S,
                                double2 *T, double *Q, cudaStream_t st, const double2 *D,
                                const double2 *W, double *gpart, double *grad) {
  HQ_STAGE(ST_OVERLAP, st);
  const long long terms = (long long)n * n * nprim * nprim;
  if (gpart)
    k_ovl_lattice<20, true><<<ceil_div(terms, 128), 128, 0, st>>>(xp, n, nprim, alpha, lattice, nlat,
                                                                  kpt, Q);
  else
    k_ovl_lattice<10, true><<<ceil_div(terms, 128), 128, 0, st>>>(xp, n, nprim, alpha, lattice, nlat,
                                                                  kpt, Q);
  HQ_LAUNCH_CHECK();
  const long long total = (long long)n * n * nb * nb;
  k_ovl_contract_kpt<<<ceil_div(total, 128), 128, 0, st>>>(n, nb, nprim, alpha, coef, ao_l, ao_cart,
                                                          Q, S, T, D, W, gpart);
  HQ_LAUNCH_CHECK();
  if (gpart) {
    k_reduce_pair_grad<<<n, 256, 0, st>>>(gpart, n, nb, grad);
    HQ_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// Ewald (potential.py:103-130).  xp in rs units, L in rs units; energy in Ry,
// grad in Ry per rs unit.  psi(r) = erfc(kappa |r|)/|r| (nearest image) +
// sum_G g(G) cos(2 pi G.r) + g0 over 0 < |G|^2 <= Gmax^2 (L = 1 units).  The
// reciprocal part of sum_{i<j} psi(r_ij) is taken from the structure factor
// S(G) = sum_i exp(2 pi i G.x_i / L):  sum_{i<j} cos(2 pi G.r_ij) =
// (|S|^2 - n) / 2, and its derivative with respect to atom a is
// -2 pi G Im(conj(S) exp(2 pi i G.x_a / L)) -- n N_G phases instead of the
// pairwise n^2 N_G / 2.
// ---------------------------------------------------------------------------
constexpr int kEwThreads = 256;

__device__ inline bool ewald_g(long long k, int gmax, int &gx, int &gy, int &gz, int &G2) {
  const int side = 2 * gmax + 1;
  gx = (int)(k / ((long long)side * side)) - gmax;
  gy = (int)((k / side) % side) - gmax;
  gz = (int)(k % side) - gmax;
  G2 = gx * gx + gy * gy + gz * gz;
  return G2 != 0 && G2 <= gmax * gmax;
}

__device__ inline double ewald_gk(int G2, double kappa) {
  return exp(-M_PI * M_PI * G2 / (kappa * kappa)) / (M_PI * G2);
}

// S(G) per cube point (0 outside the sphere) and the reciprocal energy per block
__global__ void __launch_bounds__(kEwThreads)
    k_ewald_sf(const double *__restrict__ xp, int n, double L, double kappa, int gmax,
               double2 *__restrict__ S, double *__restrict__ part_e) {
  __shared__ double sh[32];
  const int side = 2 * gmax + 1;
  const long long nG = (long long)side * side * side;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0;
  if (k < nG) {
    int gx, gy, gz, G2;
    double sr = 0, si = 0;
    if (ewald_g(k, gmax, gx, gy, gz, G2)) {
      for (int i = 0; i < n; ++i) {
        const double ph = (gx * xp[i * 3] + gy * xp[i * 3 + 1] + gz * xp[i * 3 + 2]) / L;
        double sn, cs;
        sincospi(2.0 * ph, &sn, &cs);
        sr += cs;
        si += sn;
      }
      e = ewald_gk(G2, kappa) * 0.5 * (sr * sr + si * si - n);
    }
    S[k] = make_double2(sr, si);
  }
  e = block_sum(e, sh);
  if (threadIdx.x == 0) part_e[blockIdx.x] = e;
}

// reciprocal derivative of sum_{i<j} psi with respect to r_a (L = 1 units); one block per atom
__global__ void __launch_bounds__(kEwThreads)
    k_ewald_recip_grad(const double *__restrict__ xp, int n, double L, double kappa, int gmax,
                       const double2 *__restrict__ S, double *__restrict__ gr) {
  __shared__ double sh[32];
  const int a = blockIdx.x;
  const int side = 2 * gmax + 1;
  const long long nG = (long long)side * side * side;
  double g0 = 0, g1 = 0, g2 = 0;
  for (long long k = threadIdx.x; k < nG; k += blockDim.x) {
    int gx, gy, gz, G2;
    if (!ewald_g(k, gmax, gx, gy, gz, G2)) continue;
    const double ph = (gx * xp[a * 3] + gy * xp[a * 3 + 1] + gz * xp[a * 3 + 2]) / L;
    double sn, cs;
    sincospi(2.0 * ph, &sn, &cs);
    const double2 sk = S[k];
    const double f = -2.0 * M_PI * ewald_gk(G2, kappa) * (sk.x * sn - sk.y * cs);
    g0 += f * gx;
    g1 += f * gy;
    g2 += f * gz;
  }
  g0 = block_sum(g0, sh);
  g1 = block_sum(g1, sh);
  g2 = block_sum(g2, sh);
  if (threadIdx.x == 0) {
    gr[a * 3] = g0;
    gr[a * 3 + 1] = g1;
    gr[a * 3 + 2] = g2;
  }
}

// nearest-image real-space term and its derivative, one thread per pair (i < j)
__global__ void k_ewald_real(const double *__restrict__ xp, int n, double L, double kappa,
                             double *__restrict__ pair_e, double *__restrict__ pair_g) {
  const int npair = n * (n - 1) / 2;
  const int pidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (pidx >= npair) return;
  int i = 0, rem = pidx;
  while (rem >= n - 1 - i) {
    rem -= n - 1 - i;
    ++i;
  }
  const int j = i + 1 + rem;
  double r[3];
  for (int d = 0; d < 3; ++d) {
    const double a = xp[i * 3 + d] - L * floor(xp[i * 3 + d] / L);
    const double b = xp[j * 3 + d] - L * floor(xp[j * 3 + d] / L);
    const double x = (a - b) / L;
    r[d] = x - rint(x);
  }
  const double dd = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  const double sr = erfc(kappa * dd) / dd;
  const double dsr = -2.0 * kappa / sqrt(M_PI) * exp(-kappa * kappa * dd * dd) / dd - sr / dd;
  pair_e[pidx] = sr;
  for (int d = 0; d < 3; ++d) pair_g[pidx * 3 + d] = dsr * r[d] / dd;
}

__global__ void k_ewald_finish(const double *__restrict__ pair_e, const double *__restrict__ pair_g,
                               const double *__restrict__ part_e, int nblk, const double *__restrict__ gr,
                               int n, double L, double rs, double kappa, int gmax,
                               double *__restrict__ energy, double *__restrict__ grad) {
  __shared__ double sh[32];
  const int npair = n * (n - 1) / 2;
  double s = 0;
  for (int k = threadIdx.x; k < npair; k += blockDim.x) s += pair_e[k];
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) s += part_e[k];
  s = block_sum(s, sh);
  // Madelung constant of the unit simple-cubic lattice with this kappa / Gmax
  double m = 0;
  const int side = 2 * gmax + 1;
  const long long nG = (long long)side * side * side;
  for (long long k = threadIdx.x; k < nG; k += blockDim.x) {
    int gx, gy, gz, G2;
    if (ewald_g(k, gmax, gx, gy, gz, G2)) m += ewald_gk(G2, kappa);
  }
  m = block_sum(m, sh);
  if (threadIdx.x == 0) {
    const double g0 = -M_PI / (kappa * kappa);
    const double mad = m + g0 - 2.0 * kappa / sqrt(M_PI);
    *energy = 2.0 * (s + npair * g0) / L / rs + n * mad / L / rs;
  }
  if (grad) {
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
      double acc[3] = {gr[a * 3], gr[a * 3 + 1], gr[a * 3 + 2]};
      int k = 0;
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j, ++k) {
          const double sgn = (i == a) ? 1.0 : ((j == a) ? -1.0 : 0.0);
          if (sgn != 0.0)
            for (int d = 0; d < 3; ++d) acc[d] += sgn * pair_g[k * 3 + d];
        }
      for (int d = 0; d < 3; ++d) grad[a * 3 + d] = 2.0 * acc[d] / (L * L * rs);
    }
  }
}

size_t ewald_work_doubles(int n, int gmax) {
  const long long side = 2LL * gmax + 1, nG = side * side * side;
  const size_t npair = (size_t)n * (n - 1) / 2;
  return 4 * (npair + 1) + 2 * (size_t)nG + (size_t)ceil_div(nG, kEwThreads) + 3 * (size_t)n;
}

void launch_ewald(const double *xp, int n, double L, double rs, double kappa, int gmax, double *work,
                  double *energy, double *grad, cudaStream_t st) {
  HQ_STAGE(ST_EWALD, st);
  const int npair = n * (n - 1) / 2;
  const long long side = 2LL * gmax + 1, nG = side * side * side;
  const int nblk = ceil_div(nG, kEwThreads);
  double *pe = work, *pg = pe + (npair + 1), *Sd = pg + 3 * ((size_t)npair + 1);
  double *part = Sd + 2 * nG, *gr = part + nblk;
  double2 *S = reinterpret_cast<double2 *>(Sd);  // 16-byte aligned: 4 (npair + 1) doubles before it
  k_ewald_sf<<<nblk, kEwThreads, 0, st>>>(xp, n, L, kappa, gmax, S, part);
  HQ_LAUNCH_CHECK();
  if (grad) {
    k_ewald_recip_grad<<<n, kEwThreads, 0, st>>>(xp, n, L, kappa, gmax, S, gr);
    HQ_LAUNCH_CHECK();
  }
  if (npair > 0) {
    k_ewald_real<<<ceil_div(npair, 128), 128, 0, st>>>(xp, n, L, kappa, pe, pg);
    HQ_LAUNCH_CHECK();
  }
  k_ewald_finish<<<1, 256, 0, st>>>(pe, pg, part, nblk, gr, n, L, rs, kappa, gmax, energy, grad);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
