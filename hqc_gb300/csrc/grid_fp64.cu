// Real-space grid kernels of the FP64 path.
//
//  * gto1d: lattice-summed 1D Gaussian-power factors and their first two
//    derivatives (hqc/pbc/gto.py:326-339, evaluated on Rmesh_1d as in
//    hqc/pbc/solver.py:212-214);
//  * phi: AO values (and gradients) on the grid, the separable product of
//    those factors contracted over primitives (hqc/pbc/gto.py:341-369);
//  * density: rho(g) = sum_p phi_p(g) (D phi)_p(g)  (hqc/pbc/solver.py:690),
//    plus grad rho for GGA;
//  * gemm_nt_partial: split-K quadrature  M_pq = sum_g A_p(g) w(g) B_q(g)
//    (hqc/pbc/solver.py:693, the Vxc/J/Vep contractions);
//  * pointwise xc / energy kernels.
//
// Layouts: grid index g = (ix * n + iy) * n + iz with x_i = i L / n; AO-major
// arrays [p][g]; factor table F[A][d][i][a][s], s = 3*l + k with k = 0 value,
// 1 first, 2 second derivative of u^l exp(-alpha u^2).
#include "common.cuh"
#include "xc.cuh"
#include "kernels.h"

namespace hqcgb {

__global__ void k_gto1d(const double *__restrict__ xp, int n_atoms, int ng, double L,
                        const double *__restrict__ alpha, int nprim,
                        const double *__restrict__ lat1d, int nlat, double *__restrict__ F) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)n_atoms * 3 * ng * nprim;
  if (idx >= total) return;
  int a = idx % nprim;
  long long r = idx / nprim;
  int i = r % ng;
  r /= ng;
  int d = r % 3;
  int A = (int)(r / 3);
  double x = i * L / ng - xp[A * 3 + d];
  double al = alpha[a];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int t = 0; t < nlat; ++t) {
    double u = x - lat1d[t];
    double e = exp(-al * u * u);
    // l = 0: value, d/dx, d2/dx2
    s[0] += e;
    s[1] += -2.0 * al * u * e;
    s[2] += (4.0 * al * al * u * u - 2.0 * al) * e;
    // l = 1
    s[3] += u * e;
    s[4] += (1.0 - 2.0 * al * u * u) * e;
    s[5] += (4.0 * al * al * u * u * u - 6.0 * al * u) * e;
  }
  double *out = F + idx * 6;
#pragma unroll
  for (int k = 0; k < 6; ++k) out[k] = s[k];
}

void launch_gto1d(const double *xp, int n_atoms, int ng, double L, const double *alpha, int nprim,
                  const double *lat1d, int nlat, double *F, cudaStream_t st) {
  HQ_STAGE(ST_GTO, st);
  long long total = (long long)n_atoms * 3 * ng * nprim;
  k_gto1d<<<ceil_div(total, 256), 256, 0, st>>>(xp, n_atoms, ng, L, alpha, nprim, lat1d, nlat, F);
  HQ_LAUNCH_CHECK();
}

// AO value (deriv_dir < 0) or its derivative along deriv_dir (0..2), or the
// second derivative d_c d_e (hess >= 0: pair index xx yy zz xy xz yz).
__device__ inline double ao_eval(const double *__restrict__ F, const double *__restrict__ coef,
                                 int nprim, int ng, int A, int l, int cart, int ix, int iy, int iz,
                                 int c1, int c2) {
  int pw[3] = {0, 0, 0};
  if (l == 1) pw[cart] = 1;
  int kd[3] = {0, 0, 0};
  if (c1 >= 0) kd[c1] += 1;
  if (c2 >= 0) kd[c2] += 1;
  const double *fx = F + ((((long long)A * 3 + 0) * ng + ix) * nprim) * 6 + 3 * pw[0] + kd[0];
  const double *fy = F + ((((long long)A * 3 + 1) * ng + iy) * nprim) * 6 + 3 * pw[1] + kd[1];
  const double *fz = F + ((((long long)A * 3 + 2) * ng + iz) * nprim) * 6 + 3 * pw[2] + kd[2];
  double v = 0.0;
  for (int a = 0; a < nprim; ++a) v += coef[a] * fx[a * 6] * fy[a * 6] * fz[a * 6];
  return v;
}

__global__ void k_phi(const double *__restrict__ F, const double *__restrict__ coef,
                      const int *__restrict__ ao_l, const int *__restrict__ ao_cart, int nao_atom,
                      int nprim, int nao, int ng, double *__restrict__ phi,
                      double *__restrict__ dphi) {
  long long N = (long long)ng * ng * ng;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nao * N) return;
  int p = (int)(idx / N);
  long long g = idx - (long long)p * N;
  int iz = g % ng, iy = (g / ng) % ng, ix = (int)(g / ((long long)ng * ng));
  int A = p / nao_atom, k = p % nao_atom;
  const double *c = coef + k * nprim;
  phi[idx] = ao_eval(F, c, nprim, ng, A, ao_l[k], ao_cart[k], ix, iy, iz, -1, -1);
  if (dphi) {
    for (int d = 0; d < 3; ++d)
      dphi[(long long)d * nao * N + idx] =
          ao_eval(F, c, nprim, ng, A, ao_l[k], ao_cart[k], ix, iy, iz, d, -1);
  }
}

void launch_phi(const double *F, const double *coef, const int *ao_l, const int *ao_cart,
                int nao_atom, int nprim, int nao, int ng, double *phi, double *dphi,
                cudaStream_t st) {
  HQ_STAGE(ST_PHI, st);
  long long total = (long long)nao * ng * ng * ng;
  k_phi<<<ceil_div(total, 256), 256, 0, st>>>(F, coef, ao_l, ao_cart, nao_atom, nprim, nao, ng, phi,
                                               dphi);
  HQ_LAUNCH_CHECK();
}

// rho(g) = sum_p phi_p X_p, X = D phi; grad rho = 2 sum_p dphi_p X_p.
// One block: 32 grid points, 8 warps; phi tile of all AOs in shared memory.
__global__ void k_density(const double *__restrict__ phi, const double *__restrict__ dphi,
                          const double *__restrict__ D, int nao, long long N,
                          double *__restrict__ rho, double *__restrict__ grho,
                          double *__restrict__ Xout) {
  extern __shared__ double sh[];  // [nao][32] + reduction [8][4][32]
  double *tile = sh;
  double *red = sh + (size_t)nao * 32;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long g0 = (long long)blockIdx.x * 32;
  long long g = g0 + lane;
  bool ok = g < N;
  for (int p = w; p < nao; p += 8) tile[p * 32 + lane] = ok ? phi[(long long)p * N + g] : 0.0;
  __syncthreads();
  double acc = 0, ga0 = 0, ga1 = 0, ga2 = 0;
  for (int p = w; p < nao; p += 8) {
    const double *Drow = D + (long long)p * nao;
    double x = 0;
    for (int q = 0; q < nao; ++q) x += Drow[q] * tile[q * 32 + lane];
    acc += tile[p * 32 + lane] * x;
    if (ok) {
      if (Xout) Xout[(long long)p * N + g] = x;
      if (grho) {
        ga0 += dphi[(long long)p * N + g] * x;
        ga1 += dphi[(long long)(nao + p) * N + g] * x;
        ga2 += dphi[(long long)(2 * nao + p) * N + g] * x;
      }
    }
  }
  red[(w * 4 + 0) * 32 + lane] = acc;
  red[(w * 4 + 1) * 32 + lane] = ga0;
  red[(w * 4 + 2) * 32 + lane] = ga1;
  red[(w * 4 + 3) * 32 + lane] = ga2;
  __syncthreads();
  if (w < 4 && ok) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[(k * 4 + w) * 32 + lane];
    if (w == 0) rho[g] = s;
    else if (grho) grho[(long long)(w - 1) * N + g] = 2.0 * s;
  }
}

void launch_density(const double *phi, const double *dphi, const double *D, int nao, long long N,
                    double *rho, double *grho, double *Xout, cudaStream_t st) {
  HQ_STAGE(ST_DENSITY, st);
  size_t smem = ((size_t)nao * 32 + 8 * 4 * 32) * sizeof(double);
  HQ_REQUIRE(smem <= 227 * 1024, "too many AOs for the FP64 density tile");
  ensure_dyn_smem((const void *)k_density, smem);
  k_density<<<ceil_div(N, 32), 256, smem, st>>>(phi, dphi, D, nao, N, rho, grho, Xout);
  HQ_LAUNCH_CHECK();
}

// Split-K quadrature partials: P[c][p][q] = sum_{g in chunk c} A_p(g) w(g) B_q(g).
// 32x32 output tile per block (256 threads, 4 outputs each), K staged by 32.
constexpr int kQuadChunk = 2048;

__global__ void k_gemm_nt_partial(const double *__restrict__ A, const double *__restrict__ B,
                                  const double *__restrict__ w, int nao, long long N, int sym,
                                  double *__restrict__ P) {
  __shared__ double As[32][33];
  __shared__ double Bs[32][33];
  int pt = blockIdx.x, qt = blockIdx.y, chunk = blockIdx.z;
  if (sym && qt < pt) return;
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int p0 = pt * 32, q0 = qt * 32;
  long long k0 = (long long)chunk * kQuadChunk;
  long long k1 = k0 + kQuadChunk < N ? k0 + kQuadChunk : N;
  double acc[4] = {0, 0, 0, 0};
  for (long long kb = k0; kb < k1; kb += 32) {
    long long k = kb + tx;
    bool kin = k < k1;
    double wk = (w && kin) ? w[k] : 1.0;
    for (int r = ty; r < 32; r += 8) {
      int p = p0 + r, q = q0 + r;
      As[r][tx] = (kin && p < nao) ? A[(long long)p * N + k] * wk : 0.0;
      Bs[r][tx] = (kin && q < nao) ? B[(long long)q * N + k] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      double b = Bs[tx][kk];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] += As[ty + 8 * r][kk] * b;
    }
    __syncthreads();
  }
  for (int r = 0; r < 4; ++r) {
    int p = p0 + ty + 8 * r, q = q0 + tx;
    if (p < nao && q < nao) P[((long long)chunk * nao + p) * nao + q] = acc[r];
  }
}

// M[p][q] = scale * sum_c P[c][p][q] (+ mirror for the symmetric case).
__global__ void k_reduce_partials(const double *__restrict__ P, int nchunk, int nao, int sym,
                                  double scale, int accumulate, double *__restrict__ M) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nao * nao) return;
  int p = idx / nao, q = idx % nao;
  int pp = p, qq = q;
  if (sym && (q / 32) < (p / 32)) { pp = q; qq = p; }
  double s = 0;
  for (int c = 0; c < nchunk; ++c) s += P[((long long)c * nao + pp) * nao + qq];
  s *= scale;
  M[idx] = accumulate ? M[idx] + s : s;
}

int quad_chunks(long long N) { return ceil_div(N, kQuadChunk); }

void launch_quadrature(const double *A, const double *B, const double *w, int nao, long long N,
                       bool sym, double scale, bool accumulate, double *partial, double *M,
                       cudaStream_t st) {
  HQ_STAGE(ST_QUAD, st);
  int nt = ceil_div(nao, 32);
  int nchunk = quad_chunks(N);
  dim3 grid(nt, nt, nchunk);
  k_gemm_nt_partial<<<grid, 256, 0, st>>>(A, B, w, nao, N, sym ? 1 : 0, partial);
  HQ_LAUNCH_CHECK();
  k_reduce_partials<<<ceil_div((long long)nao * nao, 256), 256, 0, st>>>(
      partial, nchunk, nao, sym ? 1 : 0, scale, accumulate ? 1 : 0, M);
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// pointwise: exchange-correlation on the grid.
//   in : rho, grho (GGA), vh (Hartree potential)
//   out: w = dV (vh + v_rho) (quadrature weight), u = 2 v_sigma grad rho (GGA)
//   partial sums per block: [0] sum e_xc, [1] sum vh*rho
// F32 (mixed path): the functional and its derivatives are evaluated in FP32
// where rho > 1e-6 (FP64 below, where FP32 would lose range); per-point
// rounding of about 1e-7 averages out in the FP64 sums.
// ---------------------------------------------------------------------------
template <bool F32>
__global__ void k_xc_pointwise(int kind, const double *__restrict__ rho,
                               const double *__restrict__ grho, const double *__restrict__ vh,
                               long long N, double dV, double *__restrict__ w,
                               double *__restrict__ vxc_out, double *__restrict__ u,
                               double *__restrict__ part) {
  __shared__ double sh[32];
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double exc = 0, eh = 0;
  if (g < N) {
    double r = rho[g];
    double sig = 0, gx = 0, gy = 0, gz = 0;
    if (grho) {
      gx = grho[g]; gy = grho[N + g]; gz = grho[2 * N + g];
      sig = gx * gx + gy * gy + gz * gz;
    }
    double e = 0, vr = 0, vs = 0;
    if (kind >= 0) {
      if (F32 && r > 1e-6) {
        float ef, vrf, vsf;
        xc_point<float>(kind, (float)r, (float)sig, ef, vrf, vsf);
        e = ef;
        vr = vrf;
        vs = vsf;
      } else {
        xc_point<double>(kind, r, sig, e, vr, vs);
      }
    }
    double v = vh ? vh[g] : 0.0;
    if (w) w[g] = dV * (v + vr);
    if (vxc_out) vxc_out[g] = vr;
    if (u) {
      u[g] = 2.0 * vs * gx;
      u[N + g] = 2.0 * vs * gy;
      u[2 * N + g] = 2.0 * vs * gz;
    }
    exc = e;
    eh = v * r;
  }
  double s0 = block_sum(exc, sh);
  double s1 = block_sum(eh, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s0;
    part[2 * blockIdx.x + 1] = s1;
  }
}

int xc_blocks(long long N) { return ceil_div(N, 256); }

void launch_xc_pointwise(int kind, const double *rho, const double *grho, const double *vh,
                         long long N, double dV, double *w, double *vxc_out, double *u,
                         double *part, cudaStream_t st, bool fp32) {
  HQ_STAGE(ST_XC, st);
  if (fp32)
    k_xc_pointwise<true><<<xc_blocks(N), 256, 0, st>>>(kind, rho, grho, vh, N, dV, w, vxc_out, u, part);
  else
    k_xc_pointwise<false><<<xc_blocks(N), 256, 0, st>>>(kind, rho, grho, vh, N, dV, w, vxc_out, u, part);
  HQ_LAUNCH_CHECK();
}

// Z_p(g) = 0.5 w(g) phi_p(g) + dV sum_c u_c(g) dphi_c,p(g)   (GGA Fock operand;
// M = Z phi^T + phi Z^T reproduces v_rho phi phi + u.(grad phi phi + phi grad phi)).
__global__ void k_gga_operand(const double *__restrict__ phi, const double *__restrict__ dphi,
                              const double *__restrict__ w, const double *__restrict__ u,
                              int nao, long long N, double dV, double *__restrict__ Z) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nao * N) return;
  long long g = idx % N;
  long long NN = (long long)nao * N;
  Z[idx] = 0.5 * w[g] * phi[idx] +
           dV * (u[g] * dphi[idx] + u[N + g] * dphi[NN + idx] + u[2 * N + g] * dphi[2 * NN + idx]);
}

void launch_gga_operand(const double *phi, const double *dphi, const double *w, const double *u,
                        int nao, long long N, double dV, double *Z, cudaStream_t st) {
  HQ_STAGE(ST_XC, st);
  k_gga_operand<<<ceil_div((long long)nao * N, 256), 256, 0, st>>>(phi, dphi, w, u, nao, N, dV, Z);
  HQ_LAUNCH_CHECK();
}

// Generic sum over blocks of interleaved partial sums: out[j] = scale * sum_b part[b*stride+j].
__global__ void k_sum_partials(const double *__restrict__ part, int nblk, int stride, int nout,
                               double scale, double *__restrict__ out, int accumulate) {
  __shared__ double sh[32];
  for (int j = 0; j < nout; ++j) {
    double s = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[(long long)b * stride + j];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[j] = accumulate ? out[j] + scale * s : scale * s;
    __syncthreads();
  }
}

void launch_sum_partials(const double *part, int nblk, int stride, int nout, double scale,
                         double *out, bool accumulate, cudaStream_t st) {
  k_sum_partials<<<1, 256, 0, st>>>(part, nblk, stride, nout, scale, out, accumulate ? 1 : 0);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
