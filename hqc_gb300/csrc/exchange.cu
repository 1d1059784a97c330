// Exact exchange of the Gamma-point Hartree-Fock Fock build and of its
// nuclear gradient, in the occupied-pair form with fused FFT stages.
//
// The reference builds the full ERI tensor (pr|sq) = sum_G V(G) rho_pr(G)
// rho_sq(G)* from AO pair densities in G space (hqc/pbc/solver.py:391-433) and
// contracts it with the density matrix (solver.py:604-614, 748-751):
//   K_pq = sum_rs D_rs (pr|sq),   V(G) = 4 pi / (Omega G^2), G = 0 dropped.
// With D = sum_j f_j c_j c_j^T this is, on the same odd grid and by Parseval,
//   K_pq = sum_j sum_G w(G) Re[ conj(P^_pj(G)) P^_qj(G) ],
//   P_pj(r) = phi_p(r) psi~_j(r),  psi~_j = sqrt(f_j) sum_p c_pj phi_p,
//   w(G) = dV * 4 pi / (G^2 N),  P^ = the (unnormalised) 3D DFT of P,
// (the occupied-pair-density exchange the reference sketches as exchange_rhoG,
// solver.py:631-666).  P is real, so only the half spectrum kz = 0..(n-1)/2
// is formed and the kz > 0 terms count twice.  Three stages per pair:
//
//   k_exx_plane   one x-plane of one pair: phi_p recomputed from the
//                 separable 1D GTO factors (no AO grid is read), the pair
//                 formed in shared memory, a real DFT along z (half
//                 spectrum; two real lines per complex transform) and a
//                 complex DFT along y;
//   k_exx_column  one ky-line of one pair: the DFT along x, then the
//                 frequency-stage multiply by sqrt(w(G) (1 or 2)); the store
//                 stage writes Q = sqrt(.) P^ as FP64, or as the TF32 hi/lo
//                 pieces the tensor-core Gram kernel reads (mixed path) --
//   K = Q Q^T     one symmetric Gram matrix over all pairs of a group of
//                 orbitals (tcgen05 3xTF32 on the mixed path, FP64 otherwise).
//
// Nuclear gradient (absent in the reference, doc/solver_algorithm.md:1210):
// the exchange part of dE/dR_A,c is
//   dV sum_{p in A} sum_j sum_g d_c phi_p(g) psi~_j(g) [v * (X_p psi~_j)](g),
// X = D phi, v the Coulomb kernel; by Parseval that is
//   sum_j sum_G w(G) Re[ conj(FFT(d_c phi_p psi~_j)) FFT(X_p psi~_j) ],
// which the column kernel's dot mode contracts in its store stage (no Q is
// written): four rows per AO (X_p and the three derivatives, recomputed from
// the 1D factors), three dot products per (pair, ky-line).
//
// Data: grid index g = (ix * n + iy) * n + iz (z fastest); T[pair][x][ky][kz]
// the plane-transformed pairs, n * nh complex per plane, nh = (n + 1) / 2.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {
namespace exx {

template <typename R> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };

// Twiddles w[k] = exp(-2 pi i k / n) rounded to R from the FP64 table.
template <typename R2>
__device__ inline void load_twiddles(R2 *w, const double2 *tw, int n) {
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    w[k].x = tw[k].x;
    w[k].y = tw[k].y;
  }
}

// Small DFTs in shared memory.  Every odd length pairs its outputs k and
// n - k, whose twiddles are complex conjugates: with C = sum_j x_j Re W^(jk)
// and S = sum_j x_j Im W^(jk) (complex sums),
//   X[k] = C + i S,   X[n - k] = C - i S,
// which halves the multiply-adds.  W = exp(-2 pi i / n), w[m] = W^m.
template <typename R2>
__device__ __forceinline__ R2 cmul(R2 a, R2 b) {
  R2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

constexpr int kMaxN1 = 16, kMaxN2 = 16;  // register-blocked factor sizes

// DFT along axis 0 of `in` [n][ncol] (columns contiguous), n odd.
// n = n1 n2 with n1 <= kMaxN1, n2 <= kMaxN2 (j = n2 j1 + j2, k = k1 + n1 k2):
//   y[j2 n1 + k1] = W^(j2 k1) sum_j1 x[n2 j1 + j2] W^(n2 j1 k1)   -> tmp
//   X[k1 + n1 k2] = sum_j2 y[j2 n1 + k1] W^(n1 j2 k2)               -> out
// each thread holding one (j2, col) input group (then one (k1, col)) in
// registers; otherwise (a prime n, n1 = 1, or a larger n2) the paired direct
// sum into tmp.  Returns the buffer holding the result; `in` may alias
// `out`.  Ends with a block barrier.
template <typename R, typename R2>
__device__ R2 *dft_axis0_any(const R2 *in, R2 *tmp, R2 *out, int n, int ncol, int n1, const R2 *w) {
  const int n2 = n1 > 1 ? n / n1 : n;
  if (n1 == 1 || n1 > kMaxN1 || n2 > kMaxN2) {
    const int nh = (n + 1) / 2;
    for (int idx = threadIdx.x; idx < nh * ncol; idx += blockDim.x) {
      const int k = idx / ncol, col = idx - k * ncol;
      R2 C = in[col], S;
      S.x = 0;
      S.y = 0;
      int t = 0;
      for (int j = 1; j < n; ++j) {
        t += k;
        if (t >= n) t -= n;
        const R2 x = in[j * ncol + col], ww = w[t];
        C.x += x.x * ww.x;
        C.y += x.y * ww.x;
        S.x += x.x * ww.y;
        S.y += x.y * ww.y;
      }
      R2 a, b;
      a.x = C.x - S.y;
      a.y = C.y + S.x;
      tmp[k * ncol + col] = a;
      if (k > 0) {
        b.x = C.x + S.y;
        b.y = C.y - S.x;
        tmp[(n - k) * ncol + col] = b;
      }
    }
    __syncthreads();
    return tmp;
  }
  for (int it = threadIdx.x; it < n2 * ncol; it += blockDim.x) {
    const int j2 = it / ncol, col = it - j2 * ncol;
    R2 x[kMaxN1];
#pragma unroll
    for (int j1 = 0; j1 < kMaxN1; ++j1)
      if (j1 < n1) x[j1] = in[(n2 * j1 + j2) * ncol + col];
    R2 s0 = x[0];
#pragma unroll
    for (int j1 = 1; j1 < kMaxN1; ++j1)
      if (j1 < n1) {
        s0.x += x[j1].x;
        s0.y += x[j1].y;
      }
    tmp[(j2 * n1) * ncol + col] = s0;
    for (int k1 = 1; 2 * k1 < n1; ++k1) {
      R2 C = x[0], S;
      S.x = 0;
      S.y = 0;
      int t = 0;
#pragma unroll
      for (int j1 = 1; j1 < kMaxN1; ++j1)
        if (j1 < n1) {
          t += k1;
          if (t >= n1) t -= n1;
          const R2 ww = w[n2 * t];
          C.x += x[j1].x * ww.x;
          C.y += x[j1].y * ww.x;
          S.x += x[j1].x * ww.y;
          S.y += x[j1].y * ww.y;
        }
      R2 a, b;
      a.x = C.x - S.y;
      a.y = C.y + S.x;
      b.x = C.x + S.y;
      b.y = C.y - S.x;
      tmp[(j2 * n1 + k1) * ncol + col] = cmul(a, w[(j2 * k1) % n]);
      tmp[(j2 * n1 + n1 - k1) * ncol + col] = cmul(b, w[(j2 * (n1 - k1)) % n]);
    }
  }
  __syncthreads();
  for (int it = threadIdx.x; it < n1 * ncol; it += blockDim.x) {
    const int k1 = it / ncol, col = it - k1 * ncol;
    R2 y[kMaxN2];
#pragma unroll
    for (int j2 = 0; j2 < kMaxN2; ++j2)
      if (j2 < n2) y[j2] = tmp[(j2 * n1 + k1) * ncol + col];
    R2 s0 = y[0];
#pragma unroll
    for (int j2 = 1; j2 < kMaxN2; ++j2)
      if (j2 < n2) {
        s0.x += y[j2].x;
        s0.y += y[j2].y;
      }
    out[k1 * ncol + col] = s0;
    for (int k2 = 1; 2 * k2 < n2; ++k2) {
      R2 C = y[0], S;
      S.x = 0;
      S.y = 0;
      int t = 0;
#pragma unroll
      for (int j2 = 1; j2 < kMaxN2; ++j2)
        if (j2 < n2) {
          t += k2;
          if (t >= n2) t -= n2;
          const R2 ww = w[n1 * t];
          C.x += y[j2].x * ww.x;
          C.y += y[j2].y * ww.x;
          S.x += y[j2].x * ww.y;
          S.y += y[j2].y * ww.y;
        }
      R2 a, b;
      a.x = C.x - S.y;
      a.y = C.y + S.x;
      b.x = C.x + S.y;
      b.y = C.y - S.x;
      out[(k1 + n1 * k2) * ncol + col] = a;
      out[(k1 + n1 * (n2 - k2)) * ncol + col] = b;
    }
  }
  __syncthreads();
  return out;
}

// The same two-factor transform for the grids of the benchmark
// configurations (n = N1 N2 at compile time): the inner transforms' twiddles
// live in registers and every index is a constant, which removes most of the
// integer work of the generic routine; work items advance without divisions.
template <typename R, typename R2, int N1, int N2>
__device__ R2 *dft_axis0_fixed(const R2 *in, R2 *tmp, R2 *out, int ncol, const R2 *w) {
  constexpr int n = N1 * N2;
  R2 w1[N1], w2[N2];  // W_N1^m = W^(N2 m), W_N2^m = W^(N1 m)
#pragma unroll
  for (int m = 0; m < N1; ++m) w1[m] = w[N2 * m];
#pragma unroll
  for (int m = 0; m < N2; ++m) w2[m] = w[N1 * m];
  const int step_r = (int)blockDim.x / ncol, step_c = (int)blockDim.x - step_r * ncol;
  {
    int j2 = (int)threadIdx.x / ncol, col = (int)threadIdx.x - j2 * ncol;
    while (j2 < N2) {
      R2 x[N1];
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) x[j1] = in[(N2 * j1 + j2) * ncol + col];
      R2 s0 = x[0];
#pragma unroll
      for (int j1 = 1; j1 < N1; ++j1) {
        s0.x += x[j1].x;
        s0.y += x[j1].y;
      }
      tmp[(j2 * N1) * ncol + col] = s0;
#pragma unroll
      for (int k1 = 1; 2 * k1 < N1; ++k1) {
        R2 C = x[0], S;
        S.x = 0;
        S.y = 0;
#pragma unroll
        for (int j1 = 1; j1 < N1; ++j1) {
          const R2 ww = w1[(j1 * k1) % N1];
          C.x += x[j1].x * ww.x;
          C.y += x[j1].y * ww.x;
          S.x += x[j1].x * ww.y;
          S.y += x[j1].y * ww.y;
        }
        R2 a, b;
        a.x = C.x - S.y;
        a.y = C.y + S.x;
        b.x = C.x + S.y;
        b.y = C.y - S.x;
        // j2 k1 < n: no reduction of the twiddle index
        tmp[(j2 * N1 + k1) * ncol + col] = cmul(a, w[j2 * k1]);
        tmp[(j2 * N1 + N1 - k1) * ncol + col] = cmul(b, w[j2 * (N1 - k1)]);
      }
      col += step_c;
      j2 += step_r;
      if (col >= ncol) {
        col -= ncol;
        ++j2;
      }
    }
  }
  __syncthreads();
  {
    int k1 = (int)threadIdx.x / ncol, col = (int)threadIdx.x - k1 * ncol;
    while (k1 < N1) {
      R2 y[N2];
#pragma unroll
      for (int j2 = 0; j2 < N2; ++j2) y[j2] = tmp[(j2 * N1 + k1) * ncol + col];
      R2 s0 = y[0];
#pragma unroll
      for (int j2 = 1; j2 < N2; ++j2) {
        s0.x += y[j2].x;
        s0.y += y[j2].y;
      }
      out[k1 * ncol + col] = s0;
#pragma unroll
      for (int k2 = 1; 2 * k2 < N2; ++k2) {
        R2 C = y[0], S;
        S.x = 0;
        S.y = 0;
#pragma unroll
        for (int j2 = 1; j2 < N2; ++j2) {
          const R2 ww = w2[(j2 * k2) % N2];
          C.x += y[j2].x * ww.x;
          C.y += y[j2].y * ww.x;
          S.x += y[j2].x * ww.y;
          S.y += y[j2].y * ww.y;
        }
        R2 a, b;
        a.x = C.x - S.y;
        a.y = C.y + S.x;
        b.x = C.x + S.y;
        b.y = C.y - S.x;
        out[(k1 + N1 * k2) * ncol + col] = a;
        out[(k1 + N1 * (N2 - k2)) * ncol + col] = b;
      }
      col += step_c;
      k1 += step_r;
      if (col >= ncol) {
        col -= ncol;
        ++k1;
      }
    }
  }
  __syncthreads();
  (void)n;
  return out;
}

// Dispatch: the fixed-size transforms for 25, 33, 49, 65 and 81 points,
// the generic routine otherwise.
template <typename R, typename R2>
__device__ R2 *dft_axis0(const R2 *in, R2 *tmp, R2 *out, int n, int ncol, int n1, const R2 *w) {
  switch (n) {
    case 25: return dft_axis0_fixed<R, R2, 5, 5>(in, tmp, out, ncol, w);
    case 33: return dft_axis0_fixed<R, R2, 3, 11>(in, tmp, out, ncol, w);
    case 49: return dft_axis0_fixed<R, R2, 7, 7>(in, tmp, out, ncol, w);
    case 65: return dft_axis0_fixed<R, R2, 5, 13>(in, tmp, out, ncol, w);
    case 81: return dft_axis0_fixed<R, R2, 9, 9>(in, tmp, out, ncol, w);
    default: return dft_axis0_any<R, R2>(in, tmp, out, n, ncol, n1, w);
  }
}

// dV * 4 pi / (G^2 N) (0 at G = 0), doubled for kz > 0 (the half spectrum
// stands for +G and -G).
__device__ inline double pair_weight(int kx, int ky, int kz, int n, double L, double dV) {
  const int mx = kx <= n / 2 ? kx : kx - n, my = ky <= n / 2 ? ky : ky - n;
  const double m2 = (double)mx * mx + (double)my * my + (double)kz * kz;
  if (m2 == 0.0) return 0.0;
  const double g = 2.0 * M_PI / L;
  const double N = (double)n * n * n;
  return dV * 4.0 * M_PI / (g * g * m2 * N) * (kz > 0 ? 2.0 : 1.0);
}

// wsq[kx][ky][kz] = sqrt(pair_weight), once per plan
template <typename R>
__global__ void k_pair_weights(int n, double L, double dV, R *__restrict__ wsq) {
  const int nh = (n + 1) / 2;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)n * n * nh) return;
  const int kz = (int)(i % nh), ky = (int)((i / nh) % n), kx = (int)(i / ((long long)n * nh));
  wsq[i] = (R)sqrt(pair_weight(kx, ky, kz, n, L, dV));
}

struct PlaneArgs {
  int n, nh, n1, nao, nb, nprim;
  int rows;                  // pair rows per orbital: nao (Fock), 4 nao (gradient)
  int xrows;                 // rows [0, xrows) read their field from X; the rest from the 1D factors
  const double2 *tw;
  const void *F1d;           // 1D factor table [atom][axis][grid][prim][6] (R)
  const double *coef;        // [nb][nprim]
  const int *ao_l, *ao_cart; // [nb]
  const double *X;           // [nao][ldx] FP64 (gradient mode), or null
  long long ldx;
  const void *psi;           // psi~ of the group's first orbital, rows ldpsi apart (R)
  long long ldpsi;
  void *T;                   // [g][rows][n][n][nh] complex R
};

// grid (n x-planes, rows, orbitals of the group)
// FP32: four CTAs of 256 threads per SM (64 registers); FP64 runs one
template <typename R>
constexpr int exx_min_blocks() { return sizeof(R) == 4 ? 4 : 1; }

template <typename R>
__global__ void __launch_bounds__(256, exx_min_blocks<R>()) k_exx_plane(PlaneArgs a) {
  using R2 = typename C2<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n = a.n, nh = a.nh, x = blockIdx.x, r = blockIdx.y, jl = blockIdx.z;
  const size_t bufc = (size_t)n * (n + 1) / 2 + 1;  // complex slots of one plane buffer (>= n^2 reals)
  R2 *w = reinterpret_cast<R2 *>(smraw);
  R2 *B0 = w + n;                  // plane buffers: the packed pair lines, the
  R2 *B1 = B0 + bufc;              // transforms' temporaries and the z-transformed plane
  R *fyz = reinterpret_cast<R *>(B1 + bufc);  // [2][nprim][n]: y and z factors
  load_twiddles(w, a.tw, n);
  const long long plane = (long long)x * n * n;
  const R *psi = reinterpret_cast<const R *>(a.psi) + (long long)jl * a.ldpsi + plane;
  const long long nn = (long long)n * n;
  // The pair plane goes straight into the packed layout of the z transform:
  // complex column pr of Z[z][pr] holds the real y-lines 2 pr (real part) and
  // 2 pr + 1 (imaginary part); the last column of an odd n has no partner.
  const int npair = (n + 1) / 2;
  R *Zr = reinterpret_cast<R *>(B0);  // Z[z][pr] as reals: [z][pr][2]
  auto put = [&](int i, R v) {
    const int y = i / n, z = i - y * n;
    Zr[2 * (z * npair + (y >> 1)) + (y & 1)] = v;
  };
  if (n & 1)
    for (int z = threadIdx.x; z < n; z += blockDim.x) Zr[2 * (z * npair + npair - 1) + 1] = 0;
  if (r < a.xrows) {
    const double *Xr = a.X + (long long)r * a.ldx + plane;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) put(i, (R)Xr[i] * psi[i]);
  } else {
    // Fock mode: row r is phi_p, p = r (c = -1: the value); gradient mode:
    // row nao (1 + c) + p is d_c phi_p
    const int rr = r - a.xrows;
    const int p = rr % a.nao, c = a.xrows > 0 ? rr / a.nao : -1;
    // AO p (or its derivative along c) = sum_a coef_a fx_a(x) fy_a(y) fz_a(z)
    const int A = p / a.nb, k = p % a.nb, l = a.ao_l[k], ca = a.ao_cart[k];
    int e[3];
    for (int d = 0; d < 3; ++d) e[d] = 3 * ((l == 1 && ca == d) ? 1 : 0) + (d == c ? 1 : 0);
    const R *F = reinterpret_cast<const R *>(a.F1d);
    for (int i = threadIdx.x; i < 2 * a.nprim * n; i += blockDim.x) {
      const int ax = i / (a.nprim * n), rem = i - ax * a.nprim * n, pr = rem / n, t = rem - pr * n;
      fyz[i] = F[((((long long)A * 3 + 1 + ax) * n + t) * a.nprim + pr) * 6 + e[1 + ax]];
    }
    __syncthreads();
    R fx[8];
    for (int pr = 0; pr < a.nprim; ++pr)
      fx[pr] = (R)a.coef[k * a.nprim + pr] * F[((((long long)A * 3 + 0) * n + x) * a.nprim + pr) * 6 + e[0]];
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int y = i / n, z = i - y * n;
      R v = 0;
      for (int pr = 0; pr < a.nprim; ++pr) v += fx[pr] * fyz[pr * n + y] * fyz[(a.nprim + pr) * n + z];
      put(i, v * psi[i]);
    }
  }
  __syncthreads();
  // z transform of the packed lines, then unpacked into C[y][kz], kz < nh:
  // A[k] = (Z[k] + conj Z[n-k]) / 2 (line 2 pr), B[k] = (Z[k] - conj Z[n-k]) / 2i
  R2 *Zt = dft_axis0<R, R2>(B0, B1, B0, n, npair, a.n1, w);
  R2 *Cb = (Zt == B0) ? B1 : B0;
  for (int i = threadIdx.x; i < npair * nh; i += blockDim.x) {
    const int pr = i / nh, kz = i - pr * nh;
    const R2 zk = Zt[kz * npair + pr], zm = Zt[(kz == 0 ? 0 : n - kz) * npair + pr];
    R2 u, v;
    u.x = (R)0.5 * (zk.x + zm.x);
    u.y = (R)0.5 * (zk.y - zm.y);
    v.x = (R)0.5 * (zk.y + zm.y);
    v.y = (R)0.5 * (zm.x - zk.x);
    Cb[(2 * pr) * nh + kz] = u;
    if (2 * pr + 1 < n) Cb[(2 * pr + 1) * nh + kz] = v;
  }
  __syncthreads();
  R2 *Ct = (Cb == B0) ? B1 : B0;
  const R2 *res = dft_axis0<R, R2>(Cb, Ct, Cb, n, nh, a.n1, w);
  R2 *T = reinterpret_cast<R2 *>(a.T) + (((long long)jl * a.rows + r) * n + x) * (long long)n * nh;
  for (int i = threadIdx.x; i < n * nh; i += blockDim.x) T[i] = res[i];
}

struct ColumnArgs {
  int n, nh, n1, nao, rows;
  const double2 *tw;
  const void *wsq;           // [n][n][nh] sqrt(pair_weight) (R)
  const void *T;             // [g][rows][n][n][nh] complex R
  // Fock mode: Q rows (one per AO), K index jl * 2 N_h + 2 ((kx n + ky) nh + kz) + {re, im}
  void *Q;                   // FP64 [rows][ldq], or the TF32 pieces [2][rows][ldq] (hi, then lo)
  long long ldq;
  // gradient mode: part[((jl * nao + p) * n + ky) * 3 + c]
  double *part;
};

__device__ inline uint32_t tf32_rna_x(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// OUT 0: FP64 Q;  OUT 1: TF32 hi/lo Q;  OUT 2: gradient dot products.
// grid (n ky-lines, AOs (OUT 2) or rows, orbitals of the group)
template <typename R, int OUT>
__global__ void __launch_bounds__(256, OUT == 2 ? 1 : exx_min_blocks<R>()) k_exx_column(ColumnArgs a) {
  using R2 = typename C2<R>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n = a.n, nh = a.nh, ky = blockIdx.x, r = blockIdx.y, jl = blockIdx.z;
  const size_t line = (size_t)n * nh;
  R2 *w = reinterpret_cast<R2 *>(smraw);
  R2 *B0 = w + n, *B1 = B0 + line, *B2 = B1 + line;
  load_twiddles(w, a.tw, n);
  const R2 *Tbase = reinterpret_cast<const R2 *>(a.T);
  const R *wsq = reinterpret_cast<const R *>(a.wsq) + (long long)ky * nh;  // + kx n nh + kz
  const long long plane = (long long)n * nh;
  auto load_line = [&](int row, R2 *dst) {
    const R2 *src = Tbase + ((long long)jl * a.rows + row) * n * plane + (long long)ky * nh;
    for (int i = threadIdx.x; i < n * nh; i += blockDim.x) {
      const int x = i / nh, kz = i - x * nh;
      dst[i] = src[(long long)x * plane + kz];
    }
    __syncthreads();
  };
  if (OUT != 2) {
    load_line(r, B0);
    const R2 *res = dft_axis0<R, R2>(B0, B1, B0, n, nh, a.n1, w);
    const long long K0 = (long long)jl * 2 * n * plane;
    for (int i = threadIdx.x; i < n * nh; i += blockDim.x) {
      const int kx = i / nh, kz = i - kx * nh;
      const R s = wsq[(long long)kx * n * nh + kz];
      const long long K = K0 + 2 * (((long long)kx * n + ky) * nh + kz);
      const R re = res[i].x * s, im = res[i].y * s;
      if (OUT == 0) {
        double *Q = reinterpret_cast<double *>(a.Q) + (long long)r * a.ldq + K;
        Q[0] = re;
        Q[1] = im;
      } else {
        float *Qh = reinterpret_cast<float *>(a.Q) + (long long)r * a.ldq + K;
        float *Ql = Qh + (long long)a.rows * a.ldq;
        const float hr = __uint_as_float(tf32_rna_x((float)re)), hi = __uint_as_float(tf32_rna_x((float)im));
        *reinterpret_cast<float2 *>(Qh) = make_float2(hr, hi);
        *reinterpret_cast<float2 *>(Ql) =
            make_float2(__uint_as_float(tf32_rna_x((float)re - hr)), __uint_as_float(tf32_rna_x((float)im - hi)));
      }
    }
  } else {
    // rows: X_p at p, d_c phi_p at nao (1 + c) + p
    const int p = r;
    __shared__ double red[3][8];
    load_line(p, B0);
    const R2 *xh = dft_axis0<R, R2>(B0, B1, B0, n, nh, a.n1, w);  // in B0 or B1
    R2 *spare = (xh == B0) ? B1 : B0;
    double acc[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
      load_line(a.nao * (1 + c) + p, B2);
      const R2 *dh = dft_axis0<R, R2>(B2, spare, B2, n, nh, a.n1, w);
      for (int i = threadIdx.x; i < n * nh; i += blockDim.x) {
        const int kx = i / nh, kz = i - kx * nh;
        const double s = (double)wsq[(long long)kx * n * nh + kz];
        acc[c] += s * s * ((double)xh[i].x * (double)dh[i].x + (double)xh[i].y * (double)dh[i].y);
      }
      __syncthreads();
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
      const double v = warp_sum(acc[c]);
      if (lane == 0) red[c][wp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      double s = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[threadIdx.x][k];
      a.part[(((long long)jl * a.nao + p) * n + ky) * 3 + threadIdx.x] = s;
    }
  }
}

// psi~_k(g) = sqrt(occ_k) sum_p C[p][k] phi_p(g) for k < nuse; 16 orbitals per
// block row, one grid point per thread.
template <typename R>
__global__ void __launch_bounds__(256) k_psi_all(const double *__restrict__ C, const double *__restrict__ occ,
                                                 int nao, int nmo, int nuse, const R *__restrict__ phi,
                                                 long long ldphi, long long N, R *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  R *Y = reinterpret_cast<R *>(smraw);  // [nao][16]
  const int k0 = blockIdx.y * 16;
  const int nk = min(16, nuse - k0);
  for (int i = threadIdx.x; i < nao * 16; i += blockDim.x) {
    const int p = i / 16, kk = i - p * 16;
    Y[i] = kk < nk ? (R)(C[(long long)p * nmo + k0 + kk] * sqrt(fmax(occ[k0 + kk], 0.0))) : (R)0;
  }
  __syncthreads();
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  R acc[16];
#pragma unroll
  for (int kk = 0; kk < 16; ++kk) acc[kk] = 0;
  for (int p = 0; p < nao; ++p) {
    const R v = phi[(long long)p * ldphi + g];
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) acc[kk] += Y[p * 16 + kk] * v;
  }
  for (int kk = 0; kk < nk; ++kk) out[(long long)(k0 + kk) * N + g] = acc[kk];
}

// grad[A][c] += sum_{p in A} sum_{jl < g, ky} part[((jl nao + p) n + ky)][c]
__global__ void k_exx_force_reduce(const double *__restrict__ part, int g, int nao, int nb, int n,
                                   double *__restrict__ grad) {
  __shared__ double sh[32];
  const int A = blockIdx.x;
  for (int c = 0; c < 3; ++c) {
    double s = 0;
    const int per = nb * n;
    for (int i = threadIdx.x; i < g * per; i += blockDim.x) {
      const int jl = i / per, rem = i - jl * per, pl = rem / n, ky = rem - pl * n;
      s += part[(((long long)jl * nao + A * nb + pl) * n + ky) * 3 + c];
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) grad[A * 3 + c] += s;
  }
}

}  // namespace exx

// ---------------------------------------------------------------------------
int exx_factor(int n) {
  int n1 = 1;
  for (int f = 2; f * f <= n; ++f)
    if (n % f == 0) n1 = f;
  return n1;
}

template <typename R>
static size_t plane_smem(int n, int nprim) {
  using R2 = typename exx::C2<R>::T;
  const size_t bufc = (size_t)n * (n + 1) / 2 + 1;
  return sizeof(R2) * ((size_t)n + 2 * bufc) + sizeof(R) * 2 * nprim * n;
}

template <typename R>
static size_t column_smem(int n) {
  using R2 = typename exx::C2<R>::T;
  return sizeof(R2) * ((size_t)n + 3 * (size_t)n * ((n + 1) / 2));
}

bool exx_fused_supported(int n, int nprim, bool fp64) {
  const size_t lim = 227 * 1024;
  if (nprim > 8) return false;
  return fp64 ? (plane_smem<double>(n, nprim) <= lim && column_smem<double>(n) <= lim)
              : (plane_smem<float>(n, nprim) <= lim && column_smem<float>(n) <= lim);
}

long long exx_pair_len(int n) { return 2LL * n * n * ((n + 1) / 2); }

template <typename R>
void launch_exx_weights(int n, double L, double dV, R *wsq, cudaStream_t st) {
  const long long tot = (long long)n * n * ((n + 1) / 2);
  exx::k_pair_weights<R><<<ceil_div(tot, 256), 256, 0, st>>>(n, L, dV, wsq);
  HQ_LAUNCH_CHECK();
}
template void launch_exx_weights<float>(int, double, double, float *, cudaStream_t);
template void launch_exx_weights<double>(int, double, double, double *, cudaStream_t);

template <typename R>
void launch_psi_all(const double *C, const double *occ, int nao, int nmo, int nuse, const R *phi,
                    long long ldphi, long long N, R *out, cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  HQ_REQUIRE(nao <= kMaxNao, "too many AOs");
  dim3 grid(ceil_div(N, 256), ceil_div(nuse, 16));
  const size_t smem = sizeof(R) * 16 * (size_t)nao;
  ensure_dyn_smem((const void *)exx::k_psi_all<R>, smem);
  exx::k_psi_all<R><<<grid, 256, smem, st>>>(C, occ, nao, nmo, nuse, phi, ldphi, N, out);
  HQ_LAUNCH_CHECK();
}
template void launch_psi_all<float>(const double *, const double *, int, int, int, const float *,
                                    long long, long long, float *, cudaStream_t);
template void launch_psi_all<double>(const double *, const double *, int, int, int, const double *,
                                     long long, long long, double *, cudaStream_t);

// Pair planes of `g` orbitals (psi~ rows from psi, ldpsi apart): rows = nao
// (Fock: phi_p psi~_j) or 4 nao with X (gradient: X_p psi~_j, then
// d_c phi_p psi~_j for c = x, y, z).
template <typename R>
void launch_exx_plane(const ExxGeom &G, const R *F1d, const double *X, long long ldx, const R *psi,
                      long long ldpsi, int g, void *T, cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  exx::PlaneArgs a;
  a.n = G.n;
  a.nh = (G.n + 1) / 2;
  a.n1 = exx_factor(G.n);
  a.nao = G.nao;
  a.nb = G.nb;
  a.nprim = G.nprim;
  a.rows = X ? 4 * G.nao : G.nao;
  a.xrows = X ? G.nao : 0;
  a.tw = G.tw;
  a.F1d = F1d;
  a.coef = G.coef;
  a.ao_l = G.ao_l;
  a.ao_cart = G.ao_cart;
  a.X = X;
  a.ldx = ldx;
  a.psi = psi;
  a.ldpsi = ldpsi;
  a.T = T;
  const size_t smem = plane_smem<R>(G.n, G.nprim);
  ensure_dyn_smem((const void *)exx::k_exx_plane<R>, smem);
  exx::k_exx_plane<R><<<dim3(G.n, a.rows, g), 256, smem, st>>>(a);
  HQ_LAUNCH_CHECK();
}

template <typename R, int OUT>
static void column(const ExxGeom &G, int rows, const void *T, int g, void *Q, long long ldq, double *part,
                   cudaStream_t st) {
  exx::ColumnArgs a;
  a.n = G.n;
  a.nh = (G.n + 1) / 2;
  a.n1 = exx_factor(G.n);
  a.nao = G.nao;
  a.rows = rows;
  a.tw = G.tw;
  a.wsq = G.wsq;
  a.T = T;
  a.Q = Q;
  a.ldq = ldq;
  a.part = part;
  const size_t smem = column_smem<R>(G.n);
  ensure_dyn_smem((const void *)exx::k_exx_column<R, OUT>, smem);
  exx::k_exx_column<R, OUT><<<dim3(G.n, OUT == 2 ? G.nao : rows, g), 256, smem, st>>>(a);
  HQ_LAUNCH_CHECK();
}

// Q rows of the Fock build: FP64 (split = false) or the TF32 hi/lo pieces.
template <typename R>
void launch_exx_column_q(const ExxGeom &G, const void *T, int g, void *Q, long long ldq, bool split,
                         cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  if (split) column<R, 1>(G, G.nao, T, g, Q, ldq, nullptr, st);
  else column<R, 0>(G, G.nao, T, g, Q, ldq, nullptr, st);
}

// Gradient dot products of a group, reduced into grad [n_atoms][3].
template <typename R>
void launch_exx_column_grad(const ExxGeom &G, const void *T, int g, double *part, double *grad,
                            cudaStream_t st) {
  HQ_STAGE(ST_EXCHANGE, st);
  column<R, 2>(G, 4 * G.nao, T, g, nullptr, 0, part, st);
  exx::k_exx_force_reduce<<<G.nao / G.nb, 256, 0, st>>>(part, g, G.nao, G.nb, G.n, grad);
  HQ_LAUNCH_CHECK();
}

template void launch_exx_plane<float>(const ExxGeom &, const float *, const double *, long long,
                                      const float *, long long, int, void *, cudaStream_t);
template void launch_exx_plane<double>(const ExxGeom &, const double *, const double *, long long,
                                       const double *, long long, int, void *, cudaStream_t);
template void launch_exx_column_q<float>(const ExxGeom &, const void *, int, void *, long long, bool,
                                         cudaStream_t);
template void launch_exx_column_q<double>(const ExxGeom &, const void *, int, void *, long long, bool,
                                          cudaStream_t);
template void launch_exx_column_grad<float>(const ExxGeom &, const void *, int, double *, double *,
                                            cudaStream_t);
template void launch_exx_column_grad<double>(const ExxGeom &, const void *, int, double *, double *,
                                             cudaStream_t);

}  // namespace hqcgb
