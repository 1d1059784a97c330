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
  const int ab = (int)(idx % np2), a = ab / nprim, b = ab % nprim;
  const int j = (int)((idx / np2) % n), i = (int)(idx / ((long long)np2 * n));
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
    if (e > 700.0) continue;
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
  double *out = Q + idx * ((KPT ? 4 : 2) * kNq);
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

// k-point contraction: complex S, T (interleaved) from the phase-weighted sums.
__global__ void k_ovl_contract_kpt(int n, int nb, int nprim, const double *__restrict__ alpha,
                                   const double *__restrict__ coef, const int *__restrict__ ao_l,
                                   const int *__restrict__ ao_cart, const double *__restrict__ Q,
                                   double2 *__restrict__ S, double2 *__restrict__ T) {
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
  double sS = 0, sT = 0, sSi = 0, sTi = 0;
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
    }
  }
  const long long pq = (long long)(i * nb + p) * nao + (j * nb + q);
  S[pq] = make_double2(sS, sSi);
  T[pq] = make_double2(-0.5 * sT, -0.5 * sTi);
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
                                double2 *T, double *Q, cudaStream_t st) {
  HQ_STAGE(ST_OVERLAP, st);
  const long long terms = (long long)n * n * nprim * nprim;
  k_ovl_lattice<10, true><<<ceil_div(terms, 128), 128, 0, st>>>(xp, n, nprim, alpha, lattice, nlat,
                                                                kpt, Q);
  HQ_LAUNCH_CHECK();
  const long long total = (long long)n * n * nb * nb;
  k_ovl_contract_kpt<<<ceil_div(total, 128), 128, 0, st>>>(n, nb, nprim, alpha, coef, ao_l, ao_cart,
                                                          Q, S, T);
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Ewald (potential.py:103-130).  xp in rs units, L in rs units.  One block per
// pair (i<j) accumulates psi and its gradient over G; the self term is added
// by block 0.  energy in Ry; grad in Ry per rs unit.
// ---------------------------------------------------------------------------
__global__ void k_ewald_pairs(const double *__restrict__ xp, int n, double L, double kappa,
                              int gmax, double *__restrict__ pair_e, double *__restrict__ pair_g) {
  __shared__ double sh[32];
  int pidx = blockIdx.x;
  // decode pair index -> (i, j), i < j (row-major over the upper triangle)
  int i = 0, rem = pidx;
  while (rem >= n - 1 - i) { rem -= n - 1 - i; ++i; }
  int j = i + 1 + rem;
  double r[3];
  for (int d = 0; d < 3; ++d) {
    double a = xp[i * 3 + d] - L * floor(xp[i * 3 + d] / L);
    double b = xp[j * 3 + d] - L * floor(xp[j * 3 + d] / L);
    double x = (a - b) / L;
    r[d] = x - rint(x);
  }
  int side = 2 * gmax + 1;
  long long nG = (long long)side * side * side;
  double v = 0, g[3] = {0, 0, 0};
  for (long long k = threadIdx.x; k < nG; k += blockDim.x) {
    int gx = (int)(k / (side * side)) - gmax, gy = (int)((k / side) % side) - gmax,
        gz = (int)(k % side) - gmax;
    int G2 = gx * gx + gy * gy + gz * gz;
    if (G2 == 0 || G2 > gmax * gmax) continue;
    double gk = exp(-M_PI * M_PI * G2 / (kappa * kappa)) / (M_PI * G2);
    double ph = 2.0 * M_PI * (gx * r[0] + gy * r[1] + gz * r[2]);
    double s, c;
    sincos(ph, &s, &c);
    v += gk * c;
    double f = -gk * s * 2.0 * M_PI;
    g[0] += f * gx; g[1] += f * gy; g[2] += f * gz;
  }
  v = block_sum(v, sh);
  for (int d = 0; d < 3; ++d) g[d] = block_sum(g[d], sh);
  if (threadIdx.x == 0) {
    double dd = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    double sr = erfc(kappa * dd) / dd;
    double dsr = -2.0 * kappa / sqrt(M_PI) * exp(-kappa * kappa * dd * dd) / dd - sr / dd;
    pair_e[pidx] = sr + v - M_PI / (kappa * kappa);
    for (int d = 0; d < 3; ++d) pair_g[pidx * 3 + d] = dsr * r[d] / dd + g[d];
  }
}

__global__ void k_ewald_finish(const double *__restrict__ pair_e, const double *__restrict__ pair_g,
                               int n, double L, double rs, double kappa, int gmax,
                               double *__restrict__ energy, double *__restrict__ grad) {
  __shared__ double sh[32];
  int npair = n * (n - 1) / 2;
  double s = 0;
  for (int k = threadIdx.x; k < npair; k += blockDim.x) s += pair_e[k];
  s = block_sum(s, sh);
  // Madelung constant of the unit simple-cubic lattice with this kappa / Gmax
  double m = 0;
  int side = 2 * gmax + 1;
  long long nG = (long long)side * side * side;
  for (long long k = threadIdx.x; k < nG; k += blockDim.x) {
    int gx = (int)(k / (side * side)) - gmax, gy = (int)((k / side) % side) - gmax,
        gz = (int)(k % side) - gmax;
    int G2 = gx * gx + gy * gy + gz * gz;
    if (G2 == 0 || G2 > gmax * gmax) continue;
    m += exp(-M_PI * M_PI * G2 / (kappa * kappa)) / (M_PI * G2);
  }
  m = block_sum(m, sh);
  if (threadIdx.x == 0) {
    double mad = m - M_PI / (kappa * kappa) - 2.0 * kappa / sqrt(M_PI);
    *energy = 2.0 * s / L / rs + n * mad / L / rs;
  }
  if (grad) {
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
      double acc[3] = {0, 0, 0};
      int k = 0;
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j, ++k) {
          double sgn = (i == a) ? 1.0 : ((j == a) ? -1.0 : 0.0);
          if (sgn != 0.0)
            for (int d = 0; d < 3; ++d) acc[d] += sgn * pair_g[k * 3 + d];
        }
      for (int d = 0; d < 3; ++d) grad[a * 3 + d] = 2.0 * acc[d] / (L * L * rs);
    }
  }
}

void launch_ewald(const double *xp, int n, double L, double rs, double kappa, int gmax,
                  double *pair_e, double *pair_g, double *energy, double *grad, cudaStream_t st) {
  HQ_STAGE(ST_EWALD, st);
  int npair = n * (n - 1) / 2;
  if (npair > 0) {
    k_ewald_pairs<<<npair, 256, 0, st>>>(xp, n, L, kappa, gmax, pair_e, pair_g);
    HQ_LAUNCH_CHECK();
  }
  k_ewald_finish<<<1, 256, 0, st>>>(pair_e, pair_g, n, L, rs, kappa, gmax, energy, grad);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
