// Periodic Poisson solver on the odd real-space grid (FP64 path).
//
// The reference forms pair densities in G space with 1D FFTs and contracts
// them with V(G) = 4 pi / (Omega G^2), G = 0 dropped (hqc/pbc/solver.py:
// 187-207, 391-479).  On the same odd grid that is, by Parseval, a 3D DFT of
// the real-space product, a multiply by 4 pi / G^2 and an inverse DFT; this
// file implements those transforms as three axis passes of direct DFTs
// (any n, including the prime grids 41 and 73 of the benchmark configs).
//
// Data: complex double c[batch][N], g = (ix * n + iy) * n + iz.
#include "common.cuh"
#include "kernels.h"

namespace hqcgb {

// One axis pass over groups of 32 lines.  Line l of the group starts at
// base + l * line_stride; its elements are elem_stride apart.  When
// line_stride == 1 the group is loaded element-major (coalesced across lines),
// otherwise line-major (the lines are contiguous, elem_stride == 1).
// C = double2 (FP64 path) or float2 (mixed path; twiddles rounded from FP64).
// n1 > 1: two-factor Cooley-Tukey for ng = n1 n2 (j = n2 j1 + j2, k = k1 + n1 k2):
//   y[j2][k1]        = W^(j2 k1) sum_j1 x[n2 j1 + j2] W^(n2 j1 k1)
//   X[k1 + n1 k2]    = sum_j2 y[j2][k1] W^(n1 j2 k2),      W = exp(-2 pi i / ng),
// ng (n1 + n2) multiply-adds per line instead of ng^2; n1 = 1: the direct sum.
template <typename C>
__global__ void k_dft_pass(C *__restrict__ c, int ng, int axis, const double2 *__restrict__ tw,
                           int inverse, long long N, int n1) {
  using R = decltype(C::x);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  C *buf = reinterpret_cast<C *>(sm_raw);
  C *w = buf + (size_t)ng * 32;
  int tid = threadIdx.x;
  for (int k = tid; k < ng; k += blockDim.x) {
    double2 t = tw[k];
    C tt;
    tt.x = (R)t.x;
    tt.y = (R)(inverse ? -t.y : t.y);
    w[k] = tt;
  }
  C *data = c + (long long)blockIdx.y * N;
  long long base;
  long long line_stride, elem_stride;
  int nlines;
  int grp = blockIdx.x;
  int zb = (ng + 31) / 32;
  if (axis == 2) {  // lines (ix, iy) contiguous in z
    long long first = (long long)grp * 32;
    long long total = (long long)ng * ng;
    nlines = (int)min(32LL, total - first);
    base = first * ng;
    line_stride = ng;
    elem_stride = 1;
  } else {
    int outer = grp / zb, zblk = grp % zb;
    int z0 = zblk * 32;
    nlines = min(32, ng - z0);
    if (axis == 1) {  // lines (ix=outer, iz), stride n along y
      base = (long long)outer * ng * ng + z0;
      elem_stride = ng;
    } else {  // lines (iy=outer, iz), stride n^2 along x
      base = (long long)outer * ng + z0;
      elem_stride = (long long)ng * ng;
    }
    line_stride = 1;
  }
  C zero;
  zero.x = 0;
  zero.y = 0;
  int total = ng * 32;
  if (line_stride == 1) {
    for (int f = tid; f < total; f += blockDim.x) {
      int j = f / 32, l = f % 32;
      buf[j * 32 + l] = (l < nlines) ? data[base + l + (long long)j * elem_stride] : zero;
    }
  } else {
    for (int f = tid; f < total; f += blockDim.x) {
      int l = f / ng, j = f % ng;
      buf[j * 32 + l] = (l < nlines) ? data[base + (long long)l * line_stride + j] : zero;
    }
  }
  __syncthreads();
  // each thread: outputs (k, l) with l = tid % 32
  int l = tid & 31;
  C res[16];  // ng <= 256 with 16 warps
  int nk = 0;
  if (n1 > 1) {
    const int n2 = ng / n1;
    // stage A: m = j2 n1 + k1
    for (int m = tid >> 5; m < ng; m += (blockDim.x >> 5)) {
      const int j2 = m / n1, k1 = m - j2 * n1;
      const int step = (n2 * k1) % ng;
      R re = 0, im = 0;
      int idx = 0;
      for (int j1 = 0; j1 < n1; ++j1) {
        C x = buf[(n2 * j1 + j2) * 32 + l];
        C t = w[idx];
        re += x.x * t.x - x.y * t.y;
        im += x.x * t.y + x.y * t.x;
        idx += step;
        if (idx >= ng) idx -= ng;
      }
      C t = w[(j2 * k1) % ng];
      res[nk].x = re * t.x - im * t.y;
      res[nk].y = re * t.y + im * t.x;
      ++nk;
    }
    __syncthreads();
    nk = 0;
    for (int m = tid >> 5; m < ng; m += (blockDim.x >> 5)) buf[m * 32 + l] = res[nk++];
    __syncthreads();
    // stage B: output k = k1 + n1 k2 from y[j2][k1] at buf[(j2 n1 + k1) * 32 + l]
    nk = 0;
    for (int k = tid >> 5; k < ng; k += (blockDim.x >> 5)) {
      const int k2 = k / n1, k1 = k - k2 * n1;
      const int step = (n1 * k2) % ng;
      R re = 0, im = 0;
      int idx = 0;
      for (int j2 = 0; j2 < n2; ++j2) {
        C x = buf[(j2 * n1 + k1) * 32 + l];
        C t = w[idx];
        re += x.x * t.x - x.y * t.y;
        im += x.x * t.y + x.y * t.x;
        idx += step;
        if (idx >= ng) idx -= ng;
      }
      res[nk].x = re;
      res[nk].y = im;
      ++nk;
    }
  } else
  for (int k = tid >> 5; k < ng; k += (blockDim.x >> 5)) {
    R re = 0, im = 0;
    int idx = 0;
    for (int j = 0; j < ng; ++j) {
      C x = buf[j * 32 + l];
      C t = w[idx];
      re += x.x * t.x - x.y * t.y;
      im += x.x * t.y + x.y * t.x;
      idx += k;
      if (idx >= ng) idx -= ng;
    }
    res[nk].x = re;
    res[nk].y = im;
    ++nk;
  }
  __syncthreads();
  nk = 0;
  for (int k = tid >> 5; k < ng; k += (blockDim.x >> 5)) buf[k * 32 + l] = res[nk++];
  __syncthreads();
  if (line_stride == 1) {
    for (int f = tid; f < total; f += blockDim.x) {
      int j = f / 32, ll = f % 32;
      if (ll < nlines) data[base + ll + (long long)j * elem_stride] = buf[j * 32 + ll];
    }
  } else {
    for (int f = tid; f < total; f += blockDim.x) {
      int ll = f / ng, j = f % ng;
      if (ll < nlines) data[base + (long long)ll * line_stride + j] = buf[j * 32 + ll];
    }
  }
}

template <typename C>
static void fft3d_impl(C *c, int ng, int batch, const double2 *tw, bool inverse, cudaStream_t st) {
  HQ_REQUIRE(ng <= kMaxGrid, "grid too large for the direct DFT passes");
  long long N = (long long)ng * ng * ng;
  size_t smem = ((size_t)ng * 32 + ng) * sizeof(C);
  ensure_dyn_smem((const void *)k_dft_pass<C>, smem);
  int zb = (ng + 31) / 32;
  // largest factor n1 <= sqrt(ng) (1 for a prime size: the direct sum)
  int n1 = 1;
  for (int f = 2; f * f <= ng; ++f)
    if (ng % f == 0) n1 = f;
  for (int axis = 2; axis >= 0; --axis) {
    dim3 grid(axis == 2 ? ceil_div((long long)ng * ng, 32) : ng * zb, batch);
    k_dft_pass<C><<<grid, 512, smem, st>>>(c, ng, axis, tw, inverse ? 1 : 0, N, n1);
    HQ_LAUNCH_CHECK();
  }
}

void launch_fft3d(double2 *c, int ng, int batch, const double2 *tw, bool inverse, cudaStream_t st) {
  HQ_STAGE(ST_FFT, st);
  fft3d_impl(c, ng, batch, tw, inverse, st);
}

void launch_fft3d_f32(float2 *c, int ng, int batch, const double2 *tw, bool inverse,
                      cudaStream_t st) {
  HQ_STAGE(ST_FFT, st);
  fft3d_impl(c, ng, batch, tw, inverse, st);
}

// FP32 Poisson: out = ifft(kern * fft(src)), src/out FP64, transforms in FP32.
__global__ void k_r2c32(const double *__restrict__ a, long long N, float2 *__restrict__ c) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) c[i] = make_float2((float)a[i], 0.f);
}
__global__ void k_scale_c32(float2 *__restrict__ c, const double *__restrict__ k, long long N) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    float f = (float)k[i];
    float2 v = c[i];
    c[i] = make_float2(v.x * f, v.y * f);
  }
}
__global__ void k_c2r32(const float2 *__restrict__ c, long long N, double *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = (double)c[i].x;
}

void launch_poisson_f32(const double *src, double *dst, float2 *cbuf, const double *kern, int ng,
                        const double2 *tw, cudaStream_t st) {
  long long N = (long long)ng * ng * ng;
  k_r2c32<<<ceil_div(N, 256), 256, 0, st>>>(src, N, cbuf);
  HQ_LAUNCH_CHECK();
  launch_fft3d_f32(cbuf, ng, 1, tw, false, st);
  k_scale_c32<<<ceil_div(N, 256), 256, 0, st>>>(cbuf, kern, N);
  HQ_LAUNCH_CHECK();
  launch_fft3d_f32(cbuf, ng, 1, tw, true, st);
  k_c2r32<<<ceil_div(N, 256), 256, 0, st>>>(cbuf, N, dst);
  HQ_LAUNCH_CHECK();
}

// c[b][g] = (a[b][g] * (s ? s[g] : 1), 0)
__global__ void k_real_to_complex(const double *__restrict__ a, const double *__restrict__ s,
                                  long long N, long long total, double2 *__restrict__ c) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  double v = a[i];
  if (s) v *= s[i % N];
  c[i] = make_double2(v, 0.0);
}

void launch_real_to_complex(const double *a, const double *s, long long N, int batch, double2 *c,
                            cudaStream_t st) {
  long long total = N * batch;
  k_real_to_complex<<<ceil_div(total, 256), 256, 0, st>>>(a, s, N, total, c);
  HQ_LAUNCH_CHECK();
}

// c[b][g] *= k[g]
__global__ void k_scale_complex(double2 *__restrict__ c, const double *__restrict__ k, long long N,
                                long long total) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  double f = k[i % N];
  double2 v = c[i];
  c[i] = make_double2(v.x * f, v.y * f);
}

void launch_scale_complex(double2 *c, const double *k, long long N, int batch, cudaStream_t st) {
  long long total = N * batch;
  k_scale_complex<<<ceil_div(total, 256), 256, 0, st>>>(c, k, N, total);
  HQ_LAUNCH_CHECK();
}

__global__ void k_complex_real(const double2 *__restrict__ c, long long total, double scale,
                               double *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  out[i] = c[i].x * scale;
}

void launch_complex_real(const double2 *c, long long total, double scale, double *out,
                         cudaStream_t st) {
  k_complex_real<<<ceil_div(total, 256), 256, 0, st>>>(c, total, scale, out);
  HQ_LAUNCH_CHECK();
}

// Coulomb kernel 4 pi / G^2 / N (G = 0 -> 0) folded with the inverse-DFT 1/N.
__global__ void k_coulomb_table(int ng, double L, double *__restrict__ kern) {
  long long N = (long long)ng * ng * ng;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  int iz = g % ng, iy = (g / ng) % ng, ix = (int)(g / ((long long)ng * ng));
  int m[3] = {ix, iy, iz};
  double G2 = 0;
  for (int d = 0; d < 3; ++d) {
    int mm = m[d] <= ng / 2 ? m[d] : m[d] - ng;
    double G = 2.0 * M_PI * mm / L;
    G2 += G * G;
  }
  kern[g] = (g == 0) ? 0.0 : 4.0 * M_PI / G2 / (double)N;
}

void launch_coulomb_table(int ng, double L, double *kern, cudaStream_t st) {
  long long N = (long long)ng * ng * ng;
  k_coulomb_table<<<ceil_div(N, 256), 256, 0, st>>>(ng, L, kern);
  HQ_LAUNCH_CHECK();
}

// Per-atom phase factors ph[A][d][k] = exp(-i G_k R_Ad).
__global__ void k_phases(const double *__restrict__ xp, int n_atoms, int ng, double L,
                         double2 *__restrict__ ph) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_atoms * 3 * ng) return;
  int k = i % ng, d = (i / ng) % 3, A = i / (3 * ng);
  int mm = k <= ng / 2 ? k : k - ng;
  double G = 2.0 * M_PI * mm / L;
  double s, c;
  sincos(G * xp[A * 3 + d], &s, &c);
  ph[i] = make_double2(c, -s);
}

// vlocG(G) = -V(G) sum_A exp(-i G.R_A), V = 4 pi/(Omega G^2)   (solver.py:406-407)
__global__ void k_vloc_G(const double2 *__restrict__ ph, int n_atoms, int ng, double L,
                         double2 *__restrict__ out) {
  long long N = (long long)ng * ng * ng;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  int iz = g % ng, iy = (g / ng) % ng, ix = (int)(g / ((long long)ng * ng));
  double re = 0, im = 0;
  for (int A = 0; A < n_atoms; ++A) {
    double2 a = ph[(A * 3 + 0) * ng + ix], b = ph[(A * 3 + 1) * ng + iy],
            c = ph[(A * 3 + 2) * ng + iz];
    double abr = a.x * b.x - a.y * b.y, abi = a.x * b.y + a.y * b.x;
    re += abr * c.x - abi * c.y;
    im += abr * c.y + abi * c.x;
  }
  int m[3] = {ix, iy, iz};
  double G2 = 0;
  for (int d = 0; d < 3; ++d) {
    int mm = m[d] <= ng / 2 ? m[d] : m[d] - ng;
    double G = 2.0 * M_PI * mm / L;
    G2 += G * G;
  }
  double V = (g == 0) ? 0.0 : 4.0 * M_PI / (L * L * L) / G2;
  out[g] = make_double2(-V * re, -V * im);
}

void launch_vloc_G(const double *xp, int n_atoms, int ng, double L, double2 *ph, double2 *out,
                   cudaStream_t st) {
  HQ_STAGE(ST_OTHER, st);
  k_phases<<<ceil_div(n_atoms * 3 * ng, 128), 128, 0, st>>>(xp, n_atoms, ng, L, ph);
  HQ_LAUNCH_CHECK();
  long long N = (long long)ng * ng * ng;
  k_vloc_G<<<ceil_div(N, 256), 256, 0, st>>>(ph, n_atoms, ng, L, out);
  HQ_LAUNCH_CHECK();
}

// Structure-factor force term: part[b][A][c] = sum_{G in block} Re(i G_c V(G)
// e^{-iG.R_A} dV conj(F(G))), F = DFT(rho).
__global__ void k_vloc_force(const double2 *__restrict__ ph, const double2 *__restrict__ F,
                             int n_atoms, int ng, double L, double *__restrict__ part) {
  __shared__ double sh[32];
  long long N = (long long)ng * ng * ng;
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int ix = 0, iy = 0, iz = 0;
  double Gv[3] = {0, 0, 0}, V = 0;
  double2 Fc = make_double2(0, 0);
  if (g < N) {
    iz = g % ng; iy = (g / ng) % ng; ix = (int)(g / ((long long)ng * ng));
    int m[3] = {ix, iy, iz};
    double G2 = 0;
    for (int d = 0; d < 3; ++d) {
      int mm = m[d] <= ng / 2 ? m[d] : m[d] - ng;
      Gv[d] = 2.0 * M_PI * mm / L;
      G2 += Gv[d] * Gv[d];
    }
    double Omega = L * L * L;
    V = (g == 0) ? 0.0 : 4.0 * M_PI / Omega / G2;
    Fc = F[g];
    double dV = Omega / (double)N;
    Fc.x *= dV; Fc.y *= dV;
  }
  for (int A = 0; A < n_atoms; ++A) {
    double re = 0;
    if (g < N) {
      double2 a = ph[(A * 3 + 0) * ng + ix], b = ph[(A * 3 + 1) * ng + iy],
              c = ph[(A * 3 + 2) * ng + iz];
      double abr = a.x * b.x - a.y * b.y, abi = a.x * b.y + a.y * b.x;
      double er = abr * c.x - abi * c.y, ei = abr * c.y + abi * c.x;  // e^{-iG.R}
      // Re(i * e * conj(F)) = -Im(e * conj(F)) = -(ei*Fr - er*Fi)
      re = -(ei * Fc.x - er * Fc.y) * V;
    }
    for (int c = 0; c < 3; ++c) {
      double s = block_sum(re * Gv[c], sh);
      if (threadIdx.x == 0) part[((long long)blockIdx.x * n_atoms + A) * 3 + c] = s;
    }
  }
}

int vloc_force_blocks(long long N) { return ceil_div(N, 256); }

void launch_vloc_force(const double2 *ph, const double2 *F, int n_atoms, int ng, double L,
                       double *part, cudaStream_t st) {
  HQ_STAGE(ST_FORCE_GRID, st);
  long long N = (long long)ng * ng * ng;
  k_vloc_force<<<vloc_force_blocks(N), 256, 0, st>>>(ph, F, n_atoms, ng, L, part);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb
