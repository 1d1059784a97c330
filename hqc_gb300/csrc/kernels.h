// Host-side launchers of the hqcgb kernels (internal header).
#pragma once
#include <cuda_runtime.h>

namespace hqcgb {

// grid_fp64.cu
void launch_gto1d(const double *xp, int n_atoms, int ng, double L, const double *alpha, int nprim,
                  const double *lat1d, int nlat, double *F, cudaStream_t st);
void launch_phi(const double *F, const double *coef, const int *ao_l, const int *ao_cart,
                int nao_atom, int nprim, int nao, int ng, double *phi, double *dphi,
                cudaStream_t st);
void launch_density(const double *phi, const double *dphi, const double *D, int nao, long long N,
                    double *rho, double *grho, double *Xout, cudaStream_t st);
int quad_chunks(long long N);
void launch_quadrature(const double *A, const double *B, const double *w, int nao, long long N,
                       bool sym, double scale, bool accumulate, double *partial, double *M,
                       cudaStream_t st);
int xc_blocks(long long N);
void launch_xc_pointwise(int kind, const double *rho, const double *grho, const double *vh,
                         long long N, double dV, double *w, double *vxc_out, double *u,
                         double *part, cudaStream_t st, bool fp32 = false);
void launch_gga_operand(const double *phi, const double *dphi, const double *w, const double *u,
                        int nao, long long N, double dV, double *Z, cudaStream_t st);
void launch_sum_partials(const double *part, int nblk, int stride, int nout, double scale,
                         double *out, bool accumulate, cudaStream_t st);

// fft_fp64.cu
void launch_fft3d(double2 *c, int ng, int batch, const double2 *tw, bool inverse, cudaStream_t st);
void launch_real_to_complex(const double *a, const double *s, long long N, int batch, double2 *c,
                            cudaStream_t st);
void launch_scale_complex(double2 *c, const double *k, long long N, int batch, cudaStream_t st);
void launch_complex_real(const double2 *c, long long total, double scale, double *out,
                         cudaStream_t st);
void launch_coulomb_table(int ng, double L, double *kern, cudaStream_t st);
void launch_vloc_G(const double *xp, int n_atoms, int ng, double L, double2 *ph, double2 *out,
                   cudaStream_t st);
int vloc_force_blocks(long long N);
void launch_vloc_force(const double2 *ph, const double2 *F, int n_atoms, int ng, double L,
                       double *part, cudaStream_t st);

// linalg_fp64.cu
void gemm(bool ta, bool tb, int M, int N, int K, double alpha, const double *A, int lda,
          const double *B, int ldb, const double *d, double beta, double *C, int ldc,
          cudaStream_t st);
void axpby(int n, double a, const double *X, double b, const double *Y, bool transY, double *out,
           cudaStream_t st);
void dot(long long n, const double *A, const double *B, double scale, double *out, bool accumulate,
         cudaStream_t st);
void jacobi_eigh(int n, int batch, double *A, double *V, double *w, double *tmp, int *status,
                 cudaStream_t st);
void eigh_tql(int n, int batch, double *A, double *V, double *w, double *work, int *status,
              cudaStream_t st);
void diis_extrapolate(int space, int n, const double *Fk, const double *ek, int last, double damp,
                      double *B, double *c, double *F, cudaStream_t st);
void occupations(int n_elec, int nmo, int smearing, int method, double sigma, int search, int cycle,
                 double tol, double shift, const double *w, double *f, double *mu, cudaStream_t st);
void entropy(int n, const double *f, double *out, cudaStream_t st);
// entropy of the free energy E - sigma S whose gradient the forces are
void free_entropy(int n, int method, double sigma, const double *w, const double *mu, const double *f,
                  double *out, cudaStream_t st);
void launch_occ_block(const double *C, const double *occ, int n, int nuse, double *Y, cudaStream_t st);
void inv_sqrt_cols(int n, const double *U, const double *w, double *v, int *bad, cudaStream_t st);
void antisym(int n, const double *X, double *e, cudaStream_t st);

// integrals_fp64.cu
size_t ovl_scratch_doubles(int n, int nprim);
void launch_overlap_kinetic(const double *xp, int n, int nb, int nprim, const double *alpha,
                            const double *coef, const int *ao_l, const int *ao_cart,
                            const double *lattice, int nlat, double *S, double *T, const double *D,
                            const double *W, double *gpart, double *grad, double *Q,
                            cudaStream_t st);
size_t ewald_work_doubles(int n, int gmax);
void launch_ewald(const double *xp, int n, double L, double rs, double kappa, int gmax, double *work,
                  double *energy, double *grad, cudaStream_t st);

// forces_fp64.cu / exchange
void launch_psi(const double *C, int nao, int col, const double *phi, long long N, double *psi,
                cudaStream_t st);
void launch_axpy_grid(long long total, long long N, double a, const double *s, const double *X,
                      double *Z, cudaStream_t st);
int force_grid_blocks(long long N);
void launch_force_grid(const double *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                       int nao_atom, int nprim, int nao, int ng, const double *veff,
                       const double *X, const double *u, const double *DPsi, const double *Z,
                       double dV, double *part, cudaStream_t st);
void launch_force_grid_reduce(const double *part, int nao, int nao_atom, int nblk, double *grad,
                              cudaStream_t st);
void launch_gga_psi(const double *dphi, const double *u, int nao, long long N, double *Psi,
                    cudaStream_t st);
void launch_add3(long long N, const double *a, const double *b, const double *c, double *out,
                 cudaStream_t st);

void zgemm(char opa, char opb, int M, int N, int K, double2 alpha, const double2 *A, int lda,
           const double2 *B, int ldb, double2 beta, double2 *C, int ldc, cudaStream_t st);
void zgemm_batched_rowmajor(int M, int N, int K, const double2 *A, int lda, long long sa,
                            const double2 *B, int ldb, long long sb, double2 *C, int ldc,
                            long long sc, int batch, cudaStream_t st);
size_t ovl_scratch_doubles_kpt(int n, int nprim);
// With gpart (n*n*nb*nb*3 doubles) also grad[A][c] += Re tr(D dT/dR_A) - Re tr(W dS/dR_A)
// for Hermitian D, W (S and T may then be NULL).
void launch_overlap_kinetic_kpt(const double *xp, int n, int nb, int nprim, const double *alpha,
                                const double *coef, const int *ao_l, const int *ao_cart,
                                const double *lattice, int nlat, const double *kpt, double2 *S,
                                double2 *T, double *Q, cudaStream_t st, const double2 *D = nullptr,
                                const double2 *W = nullptr, double *gpart = nullptr,
                                double *grad = nullptr);
// forces_kpt.cu
void launch_rho_from_x_kpt(const double2 *phi, const double2 *dphi, const double2 *X, int nao, long long N,
                           double *rho, double *grho, cudaStream_t st);
void launch_gga_zop_kpt(const double2 *dphi, const double *u, int nao, long long N, double2 *out,
                        cudaStream_t st);
void launch_force_grid_kpt(const double2 *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                           int nao_atom, int nprim, int nao, int ng, const double *veff, const double2 *X,
                           const double *u, const double2 *DPsi, const double2 *Zm, double dV, double *part,
                           cudaStream_t st);
template <class C>  // C = double2 or float2
void launch_kx_grad_fields(const double2 *F1d, const double *coef, const int *ao_l, const int *ao_cart,
                           int nao_atom, int nprim, int nao, int ng, const double2 *X, const double2 *psi,
                           C *out, cudaStream_t st);
template <class C>
void launch_kx_grad_contract(const C *Fh, const double *coul, int nao, long long N, double scale, double *part,
                             cudaStream_t st);
// eigh_herm.cu
void eigh_herm(int n, int batch, double2 *A, double2 *V, double *w, double2 *work, int *status,
               cudaStream_t st);

void gemm_batched_rowmajor(int M, int N, int K, const double *A, int lda, long long sa,
                           const double *B, int ldb, long long sb, double *C, int ldc, long long sc,
                           int batch, cudaStream_t st);

// eigh_fp64.cu / eigh_mixed.cu
void eigh_tql_f32(int n, int batch, float *A, float *V, float *w, float *work, int *status,
                  cudaStream_t st);
size_t eigh_f32_scratch_floats(int n);
void eigh_f32(int n, float *A, float *V, float *w, float *scr, cudaStream_t st);
struct MixedEigWork {
  float *A32, *V32, *w32, *work32, *f32scr;
  double *T1, *S, *G, *E, *emax, *wbuf;  // wbuf: 2 n^2 (cluster blocks); emax: 16
  int *status, *iwork;                    // iwork: 5 n + 1
};
bool eigh_mixed_warm(int n, const double *A, const double *X0, double *V, double *w,
                     MixedEigWork &ws, cudaStream_t st, bool loose = false);
bool eigh_mixed(int n, const double *A, double *V, double *w, MixedEigWork &ws, cudaStream_t st,
                bool wide = false, bool loose = false);

// fft (FP32 transforms)
void launch_fft3d_f32(float2 *c, int ng, int batch, const double2 *tw, bool inverse,
                      cudaStream_t st);
void launch_poisson_f32(const double *src, double *dst, float2 *cbuf, const double *kern, int ng,
                        const double2 *tw, cudaStream_t st);

// grid_mixed.cu
void launch_phi32(const float *F32, const double *coef, const int *ao_l, const int *ao_cart,
                  int nao_atom, int nprim, int nao, int ng, long long ld, float *phi, float *dphi,
                  cudaStream_t st);
void launch_to_f32(const double *in, long long ldi, long long N, int rows, double scale, float *out,
                   long long ldo, cudaStream_t st);

// tc_gemm.cu (tcgen05, 3xTF32)
int tc_quad_chunk();
// kchunk: grid points per CTA along the contraction (0: tc_quad_chunk())
size_t tc_quad_partial_doubles(int nao, long long N, int kchunk = 0);
int tc_quad_tiles(int nao, bool sym);  // destination tiles of the tile plan (upper triangle if sym)
// blocked: the pieces are K-blocked [ld / 32][nao][32] (as launch_split_operand
// writes them); otherwise row-major [nao][ld]
void launch_tc_quad_split(const float *Ahl, const float *Bhl, int nao, long long N, long long ld,
                          bool sym, bool add_transpose, double scale, double *partial, double *M,
                          int *err, cudaStream_t st, int drain, int kchunk = 0, bool blocked = false);
void launch_split_operand(const float *phi, const float *dphi, const float *w, const float *u, int nao,
                          long long N, long long ldi, long long ldo, float a, float b, float *out,
                          cudaStream_t st);
void launch_tc_quadrature(const float *phi, const float *dphi, const float *phihl, const float *w,
                          const float *u, float dV, int nao, long long N, long long ld, bool gga,
                          double scale, double *partial, double *M, int *err, cudaStream_t st, int drain,
                          float *zhl);
size_t tc_density_partial_doubles(int nao, long long ld, bool gga);
int tc_ldk(int nao);
void launch_transpose_phi(const float *phi, int nao, long long N, long long ld, float *phiT,
                          cudaStream_t st);
int tc_psi_max(bool gga);
int tc_psi_width(int nuse);
void launch_psi_operand(const double *C, const double *occ, int nao, int nmo, int nuse, int ldk,
                        float *Yhl, cudaStream_t st);
void launch_tc_psi_density(const float *phiT, const float *dphiT, const float *Yhl, int npsi, int ldk,
                           long long N, double *rho, double *grho, int *err, cudaStream_t st,
                           float *psi_out = nullptr, int psi_drain = 1);
// forces_mixed.cu
int force_orb_blocks(long long N);
void launch_force_operand(const double *C, const double *occ, int nao, int nuse, int npsi,
                          float *Y32, cudaStream_t st);
void launch_to_float(long long n, const double *a, float *b, cudaStream_t st);
void launch_force_grid_orb(const float *F32, const double *coef, const int *ao_l, const int *ao_cart,
                           int n_atoms, int nb, int nprim, int ng, const double *veff,
                           const double *u, const float *psi, const float *Y32, int npsi, double dV,
                           double *part, double *grad, cudaStream_t st);
void launch_tc_density(const float *phi, const float *phiT, const float *dphi, const float *D32,
                       int nao, long long N, long long ld, double *part, double *rho, double *grho,
                       int *err, cudaStream_t st, int nsplit = 2, int drain = 3);

// exchange.cu: occupied-pair exact exchange with fused FFT stages
struct ExxGeom {
  int n, nao, nb, nprim;       // grid points per axis, AOs, AOs per atom, primitives
  const double2 *tw;           // FFT twiddles exp(-2 pi i k / n)
  const double *coef;          // [nb][nprim] contraction coefficients
  const int *ao_l, *ao_cart;   // [nb]
  const void *wsq;             // [n][n][(n+1)/2] square roots of the pair weights (R)
};
int exx_factor(int n);
bool exx_fused_supported(int n, int nprim, bool fp64);
long long exx_pair_len(int n);  // 2 n^2 (n+1)/2: reals of one pair's half spectrum
template <typename R>
void launch_exx_weights(int n, double L, double dV, R *wsq, cudaStream_t st);
template <typename R>
void launch_psi_all(const double *C, const double *occ, int nao, int nmo, int nuse, const R *phi,
                    long long ldphi, long long N, R *out, cudaStream_t st);
template <typename R>
void launch_exx_plane(const ExxGeom &G, const R *F1d, const double *X, long long ldx, const R *psi,
                      long long ldpsi, int g, void *T, cudaStream_t st);
template <typename R>
void launch_exx_column_q(const ExxGeom &G, const void *T, int g, void *Q, long long ldq, bool split,
                         cudaStream_t st);
template <typename R>
void launch_exx_column_grad(const ExxGeom &G, const void *T, int g, double *part, double *grad,
                            cudaStream_t st);

}  // namespace hqcgb
