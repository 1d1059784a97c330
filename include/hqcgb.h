/*
 * hqcgb.h -- C ABI of the GB300 (sm_103a) periodic GPW SCF engine.
 *
 * Drop-in boundary for the hot path of hqc (ZihangL/hqc v0.1.12), whose
 * public entry points are Python factories returning jitted closures:
 *
 *   make_solver(n, L, rs, basis, ...) -> solver(xp)      hqc/pbc/solver.py:14-32, 705-978
 *   make_lcao(...)  -> lcao(xp) = (mo_coeff, bands, E)   hqc/pbc/lcao.py:11-78
 *   make_pes(...)   -> pes(xp)  = E + Vpp                hqc/pbc/pes.py:10-152
 *   potential_energy_pp(xp, L, rs, kappa, Gmax)          hqc/pbc/potential.py:103-130
 *
 * The factory's table building is hqcgb_plan_create; one call of the jitted
 * closure is hqcgb_scf (+ hqcgb_ewald for make_pes).  Everything below works
 * on caller-owned DEVICE buffers and a caller stream; the plan owns its
 * workspace.  All functions return an hqcgb_status; a non-zero status leaves
 * a message for hqcgb_last_error().  Energies are in Hartree (the Python
 * layer converts to Rydberg like the reference), lengths in Bohr.
 */
#ifndef HQCGB_H
#define HQCGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  HQCGB_OK = 0,
  HQCGB_NOT_CONVERGED = 1,   /* SCF reached max_cycle (reference: converged=False) */
  HQCGB_BAD_ARG = 2,
  HQCGB_CUDA_ERROR = 3,
  HQCGB_EIG_FAIL = 4,        /* Jacobi sweep limit reached */
  HQCGB_NAN = 5,             /* non-finite energy or Fock matrix */
  HQCGB_NO_STATE = 6         /* forces requested before an SCF */
} hqcgb_status;

enum { HQCGB_XC_LDA_X = 0, HQCGB_XC_LDA_VWN = 1, HQCGB_XC_LDA_HL = 2, HQCGB_XC_LDA_BH = 3,
       HQCGB_XC_LDA_GL = 4, HQCGB_XC_PBE = 10 };
enum { HQCGB_SMEAR_FERMI = 0, HQCGB_SMEAR_GAUSS = 1 };
enum { HQCGB_SEARCH_BISECT = 0, HQCGB_SEARCH_NEWTON = 1 };
enum { HQCGB_PREC_FP64 = 0, HQCGB_PREC_MIXED = 1 };

typedef struct {
  /* system (hqc/pbc/solver.py:14-32, 153-176) */
  int n_atoms;
  int n_grid;              /* points per axis; odd for reference parity */
  double L;                /* box side, Bohr */
  /* basis, one hydrogen's AOs (hqc/pbc/solver.py:64-151, hqc/pbc/gto.py:72-300) */
  int nao_atom;
  int n_prim;
  const double *alpha;     /* [n_prim] primitive exponents */
  const double *coef;      /* [nao_atom][n_prim] contraction * cart2sph factor */
  const int *ao_l;         /* [nao_atom] 0 or 1 */
  const int *ao_cart;      /* [nao_atom] cartesian direction of a p AO */
  int n_lat1d;
  const double *lat1d;     /* [n_lat1d] 1D lattice translations of the grid GTOs */
  int n_lattice;
  const double *lattice;   /* [n_lattice][3] lattice sphere of the S/T sums */
  /* method */
  int dft;                 /* 0: Hartree-Fock, 1: Kohn-Sham */
  int xc;                  /* HQCGB_XC_* */
  int smearing;
  int smearing_method;     /* HQCGB_SMEAR_* */
  double smearing_sigma;   /* Hartree */
  int search_method;       /* HQCGB_SEARCH_* */
  int search_cycle;
  double search_tol;
  double tol;
  int max_cycle;
  int diis;
  int diis_space;
  int diis_start_cycle;
  double diis_damp;
  int precision;           /* HQCGB_PREC_* */
  double exx_occ_threshold;/* exchange skips orbitals with occupation <= max(this, 1e-14) */
  int want_forces;         /* keep derivative tables for hqcgb_forces */
} hqcgb_params;

typedef struct {
  double *mo_coeff;   /* [nao][nao], AO rows, MO columns (device) */
  double *dm;         /* [nao][nao] (device) */
  double *bands;      /* [nao] Hartree (device) */
  double *energies;   /* [5]: E, Ki, Vep, Vee (Hartree), Se (device) */
  int *converged;     /* [1] (device) */
  int *iterations;    /* [1] (device), may be NULL */
  /* [1] (device), may be NULL: the free energy E - sigma * S (Hartree) whose
   * gradient hqcgb_forces returns, S the entropy that makes the smearing's
   * occupations stationary -- Fermi: Se (the energies[4] slot); Gaussian:
   * sum_i exp(-x_i^2) / (2 sqrt(pi)), x_i = (eps_i - mu) / sigma; without
   * smearing it equals E.  No counterpart in the reference, whose E excludes
   * -sigma*S (hqc/pbc/scf.py:149,209). */
  double *free_energy;
} hqcgb_scf_out;

typedef struct hqcgb_plan hqcgb_plan;

/* Factory: validates the parameters and allocates the workspace.
 * Replaces the table-building part of make_solver (hqc/pbc/solver.py:61-231). */
int hqcgb_plan_create(const hqcgb_params *params, hqcgb_plan **plan);

/* Frees everything the plan owns. */
int hqcgb_plan_destroy(hqcgb_plan *plan);

/* One SCF at the proton positions xp [n_atoms][3] (Bohr, device).
 * Replaces hf_gamma / dft_gamma (hqc/pbc/solver.py:705-767, 839-899). */
int hqcgb_scf(hqcgb_plan *plan, const double *xp, const hqcgb_scf_out *out, void *stream);

/* Batched SCF over n_cfg configurations of the same plan: xp is
 * [n_cfg][n_atoms][3], every output pointer is strided by its per-config size.
 * The reference batches with jax.vmap (test/test.py:157). */
int hqcgb_scf_batch(hqcgb_plan *plan, int n_cfg, const double *xp, const hqcgb_scf_out *out,
                    void *stream);

/* Number of configurations a batch call runs concurrently (default 1:
 * sequentially on this plan).  With k > 1 the plan creates k - 1 clones of
 * its workspace (same parameters, own CUDA streams) on the first batch call;
 * each configuration of a batch runs on one of them, driven by its own host
 * thread.  Memory grows k-fold; results are identical to the sequential run. */
int hqcgb_plan_set_concurrency(hqcgb_plan *plan, int workers);

/* hqcgb_scf_batch plus, when grad is not NULL, the nuclear gradient of every
 * configuration into grad [n_cfg][n_atoms][3] (Hartree/Bohr, device) -- the
 * energy-and-force evaluation of a batch of configurations (the reference's
 * jax.vmap of make_pes with jax.grad, test/test.py:157, pes.py:78-115).
 * Returns the worst status over the batch; an error in any configuration is
 * reported with its index. */
int hqcgb_pes_batch(hqcgb_plan *plan, int n_cfg, const double *xp, const hqcgb_scf_out *out,
                    double *grad, void *stream);

/* ---- uneven batches --------------------------------------------------------
 * Energies (and gradients) of configurations that differ in atom count, box
 * and grid, in one call.  The reference batches with jax.vmap over
 * configurations of one shape (test/test.py:157,179); uneven sizes need one
 * vmapped call per shape there.  A batch groups configurations into size
 * classes (n_atoms, n_grid): each of `workers` host threads keeps one
 * workspace per size class (created on first use, kept until
 * hqcgb_batch_destroy) and resets its box-dependent tables per
 * configuration. */
typedef struct hqcgb_batch hqcgb_batch;

/* base: basis and method as for hqcgb_plan_create (n_atoms, n_grid, L and
 * the lattice fields are ignored: every configuration brings its own);
 * rcut (Bohr): the S/T lattice sphere (make_solver's rcut, solver.py:162-176;
 * the grid GTO sums use 24 Bohr as make_pbc_gto does). */
int hqcgb_batch_create(const hqcgb_params *base, double rcut, int workers, hqcgb_batch **batch);
int hqcgb_batch_destroy(hqcgb_batch *batch);

/* n_cfg configurations: n_atoms, n_grid, L [n_cfg] (HOST; L in Bohr); xp the
 * concatenation of every configuration's [n_atoms][3] positions (device,
 * Bohr).  Outputs are concatenated the same way (each may be NULL):
 * mo_coeff, dm [nao_c][nao_c] each; bands [nao_c] each; energies [n_cfg][5];
 * converged, iterations, free_energy [n_cfg]; grad (want_forces) [n_atoms_c][3]
 * each (Hartree/Bohr, the gradient of free_energy).  Returns the worst
 * status; an error names the configuration. */
int hqcgb_batch_run(hqcgb_batch *batch, int n_cfg, const int *n_atoms, const int *n_grid,
                    const double *L, const double *xp, const hqcgb_scf_out *out, double *grad,
                    void *stream);

/* AO values of n_atoms protons at npts points (electron positions), Gamma
 * point: the reference's eval_pbc_ao (hqc/pbc/gto.py:326-369) with the 1D
 * lattice lat1d of make_pbc_gto (tmax = rcut // L).  Basis tables as in the
 * plan parameters, host pointers; xp [ngroups][n_atoms][3], xe [npts][3] (device,
 * Bohr), pts_per_group consecutive points per proton set; out
 * [npts][n_atoms * nao_atom] (device). */
int hqcgb_ao_points(int n_atoms, int nao_atom, int n_prim, const double *alpha,
                    const double *coef, const int *ao_l, const int *ao_cart, int n_lat1d,
                    const double *lat1d, const double *xp, long long npts, int pts_per_group,
                    const double *xe, double *out, void *stream);

/* Slater matrices of W walkers (make_slater, hqc/pbc/slater.py:42-104,
 * Gamma): up[w] = AO(xe[w][0:n/2]) mo[:, state_idx[0:n/2]] and dn[w] the
 * same for electrons n/2..n-1 and state_idx[n/2:n].  xp [xp_groups][n][3]
 * (xp_groups 1 or W), xe [W][n][3] (device, Bohr); mo [nao][nmo] row-major
 * (device); state_idx [n] (host); up, dn [W][n/2][n/2] (device). */
int hqcgb_slater(int n, int nao_atom, int n_prim, const double *alpha, const double *coef,
                 const int *ao_l, const int *ao_cart, int n_lat1d, const double *lat1d, int W,
                 int xp_groups, const double *xp, const double *xe, const double *mo, int nmo,
                 const int *state_idx, double *up, double *dn, void *stream);

/* k-point variants (make_pbc_gto with gamma=False, eval_pbc_ao_kpt,
 * hqc/pbc/gto.py:371-427; make_slater's slater_kpt, hqc/pbc/slater.py:72-93):
 * every lattice term carries exp(i k.t), kpt [3] in 1/Bohr (HOST).  out,
 * mo, up and dn are complex, interleaved (re, im); other arguments as above. */
int hqcgb_ao_points_kpt(int n_atoms, int nao_atom, int n_prim, const double *alpha,
                        const double *coef, const int *ao_l, const int *ao_cart, int n_lat1d,
                        const double *lat1d, const double *kpt, const double *xp, long long npts,
                        int pts_per_group, const double *xe, double *out, void *stream);
int hqcgb_slater_kpt(int n, int nao_atom, int n_prim, const double *alpha, const double *coef,
                     const int *ao_l, const int *ao_cart, int n_lat1d, const double *lat1d,
                     const double *kpt, int W, int xp_groups, const double *xp, const double *xe,
                     const double *mo, int nmo, const int *state_idx, double *up, double *dn,
                     void *stream);

/* Overlap matrices without a plan: make_overlap (hqc/pbc/overlap.py:11-319)
 * for n_cfg configurations xp [n_cfg][n_atoms][3] (device, Bohr) over the
 * lattice sphere `lattice` [n_lattice][3] (host, Bohr; |t| <= rcut).  kpts
 * NULL: real S [n_cfg][nao][nao]; kpts [n_cfg][3] (host, 1/Bohr): complex
 * Hermitian S^k (interleaved).  T (kinetic, same layout) may be NULL. */
int hqcgb_overlap(int n_atoms, int nao_atom, int n_prim, const double *alpha, const double *coef,
                  const int *ao_l, const int *ao_cart, int n_lattice, const double *lattice,
                  int n_cfg, const double *xp, const double *kpts, double *S, double *T,
                  void *stream);

/* Ewald energies of proton + electron configurations, batched over walkers:
 * potential_energy (hqc/pbc/potential.py:69-101).  x [B][n][dim] (device, rs
 * units; the first n/2 particles are protons), L the box side (rs units),
 * G [nG][dim] the integer reciprocal vectors (host; kpoints(dim, Gmax));
 * out [B][3] = (vpp, vep, vee) (device), 2 rs / L times the pair sums as in
 * the reference (the Madelung constant is not included). */
int hqcgb_coulomb_energy(int B, int n, int dim, const double *x, double L, double rs, double kappa,
                         int nG, const int *G, double *out, void *stream);

/* Nuclear gradient dE/dR [n_atoms][3] (Hartree/Bohr, device) of the last SCF.
 * No counterpart in the reference (forces are absent there,
 * doc/solver_algorithm.md:1210); with Fermi smearing it is the gradient of
 * E - sigma*Se. */
int hqcgb_forces(hqcgb_plan *plan, double *grad, void *stream);

/* Proton-proton Ewald energy (Rydberg) and its gradient (Rydberg per rs unit).
 * xp [n][3] in rs units, L in rs units: hqc/pbc/potential.py:103-130.
 * grad may be NULL. */
int hqcgb_ewald(const double *xp, int n, double L, double rs, double kappa, int gmax,
                double *energy, double *grad, void *stream);

/* Copy an internal buffer of the last SCF into dst (device), for tests and
 * tools: "S", "T", "V", "phi", "rho", "vH", "vloc", "fock", "J", "K".
 * Returns the number of bytes copied (or needed when dst is NULL), < 0 on error. */
long long hqcgb_plan_query(hqcgb_plan *plan, const char *name, void *dst, size_t bytes,
                           void *stream);

/* (tools) Rebuild the exact-exchange matrix of a Hartree-Fock plan for the
 * density of its last SCF (the occupied-pair form with fused FFT stages), on
 * `stream`, and wait for it: for timing the exchange alone.  Returns the
 * number of AO-orbital pairs transformed, < 0 when the plan has no such
 * state (not Hartree-Fock, no SCF yet, or a grid beyond the fused kernels).
 * No counterpart in the reference (its exchange is an ERI contraction inside
 * the jitted SCF, hqc/pbc/solver.py:604-614). */
long long hqcgb_exchange_rebuild(hqcgb_plan *plan, void *stream);

/* The engine's FP64 symmetric eigensolver (Householder tridiagonalisation +
 * implicit QL, Jacobi fallback) on `batch` row-major n x n matrices A
 * (device, not modified): ascending eigenvalues w [batch][n] and eigenvectors
 * as the columns of V [batch][n][n].  Stands in for jnp.linalg.eigh as used
 * at hqc/pbc/solver.py:729,741 and hqc/pbc/scf.py:69,138,198. */
int hqcgb_eigh(int n, int batch, const double *A, double *w, double *V, void *stream);

/* The mixed-precision eigensolver of the mixed SCF path on one matrix: an
 * FP32 Householder + QL solve refined to FP64 accuracy by two Ogita-Aishima
 * iterations (FP64 GEMMs).  Same arguments and outputs as hqcgb_eigh with
 * batch = 1. */
int hqcgb_eigh_mixed(int n, const double *A, double *w, double *V, void *stream);

/* The tensor-core grid contractions of the mixed path as library calls
 * (device pointers; fp32 inputs with row stride ld >= N, ld % 4 == 0, zero
 * padding in [N, ld)).  nsplit = 2 (3xTF32; the only value accepted);
 * drain = number of K sub-chunks of 32 points summed in TMEM before a
 * compensated FP32 drain (1 = most accurate).
 *   quadrature: M[p][q] = sum_g phi[p][g] w[g] phi[q][g]  (hqc/pbc/solver.py:693)
 *   density:    rho[g]  = sum_pq D[p][q] phi[p][g] phi[q][g] (hqc/pbc/solver.py:690) */
int hqcgb_tc_quadrature(int nao, long long N, long long ld, const float *phi, const float *w,
                        int nsplit, int drain, double *M, void *stream);
int hqcgb_tc_density(int nao, long long N, long long ld, const float *phi, const float *D,
                     int nsplit, int drain, double *rho, void *stream);

/* The GGA (PBE) Fock quadrature of the mixed path: M = Z phi^T + phi Z^T with
 * Z = 0.5 w phi + dV u . grad phi (hqc/pbc/solver.py:680-694 plus the gradient
 * term); phi [nao][ld], dphi [3][nao][ld], w [ld], u [3][ld] fp32 (device),
 * ld % 32 == 0. */
int hqcgb_tc_quadrature_gga(int nao, long long N, long long ld, const float *phi,
                            const float *dphi, const float *w, const float *u, float dV, int drain,
                            double *M, void *stream);

/* Host only (no device work): the quadrature's tile plan for nao AOs in
 * 128-row blocks (sym: upper-triangle destination tiles only).  tiles
 * [cap][7] receives one row per product the kernels compute, {kind, mt, nt,
 * arow, brow, nb, swap}: kind 0 a full tile of the fused kernel, 1 a narrow
 * product carried by a fused diagonal CTA, 2 a tile of the tile-list kernel;
 * (mt, nt) the destination tile, arow / brow the first AO rows of the MMA's
 * A / B side (swap = 1: A side from the second operand, stored transposed),
 * nb the MMA N.  count = number of rows (only the first cap are written),
 * launches = quadrature kernel launches before the reduce.  Lets a caller
 * check that every destination tile is written exactly once. */
int hqcgb_tc_quad_tiles(int nao, int sym, int cap, int *tiles, int *count, int *launches);

/* Orbital form of the density: rho(g) = sum_k occ_k |psi_k(g)|^2 with
 * psi_k = sum_p C[p][k] phi_p over the first nuse (<= 64) orbitals, and
 * with dphi (3 x [nao][ld]) also grad rho (3 x N) -- the density of
 * D = C diag(occ) C^T (hqc/pbc/solver.py:566-577,690) at nuse/nao of the
 * work.  C is [nao][nmo] row-major FP64; phi/dphi fp32 as above; drain =
 * K blocks of 32 AOs accumulated in TMEM between compensated drains. */
int hqcgb_tc_orbital_density(int nao, long long N, long long ld, const float *phi,
                             const float *dphi, const double *C, const double *occ, int nmo,
                             int nuse, int drain, double *rho, double *grho, void *stream);

/* Largest n accepted by hqcgb_eigh_noalloc. */
#define HQCGB_EIGH_NOALLOC_MAX_N 320

/* hqcgb_eigh for one matrix (n <= HQCGB_EIGH_NOALLOC_MAX_N) that allocates
 * nothing: for callers that cannot allocate device memory, such as code
 * inside a framework that owns every device buffer (an XLA custom call in a
 * jitted program) or loops that must not wait on an allocation.  Its scratch
 * is a static device array of about 1.6 MB per GPU, shared by every call on
 * that device (calls whose device work overlaps race on it); the first call
 * on a device looks the array up and should precede any stream capture.
 * The call blocks the host: it synchronises the caller's stream once to read
 * the solver's status (twice more when the Jacobi fallback runs).
 * No counterpart in the reference. */
int hqcgb_eigh_noalloc(int n, const double *A, double *w, double *V, void *stream);

/* ---- single k-point solver (make_solver with gamma=False) ---------------- */

typedef struct hqcgb_kplan hqcgb_kplan;

/* Factory of the k-point solver: the same parameters as hqcgb_plan_create
 * (precision HQCGB_PREC_FP64, or HQCGB_PREC_MIXED for Hartree-Fock and LDA:
 * grid contractions on the tensor cores through the real embedding of the
 * complex AO grid, FP64 eigensolver; want_forces keeps what
 * hqcgb_forces_kpt needs).  Replaces the table-building part of
 * make_solver(gamma=False) (hqc/pbc/solver.py:209-231, 378-389). */
int hqcgb_kplan_create(const hqcgb_params *params, hqcgb_kplan **plan);
int hqcgb_kplan_destroy(hqcgb_kplan *plan);

/* One SCF at proton positions xp [n_atoms][3] (Bohr, device) and k-point
 * kpt [3] (1/Bohr, HOST).  Replaces hf_kpt / dft_kpt (hqc/pbc/solver.py:
 * 769-837, 901-962).  mo_coeff and dm are complex, interleaved (re, im):
 * 2 * nao * nao doubles each; the other outputs as in hqcgb_scf. */
int hqcgb_scf_kpt(hqcgb_kplan *plan, const double *xp, const double *kpt,
                  const hqcgb_scf_out *out, void *stream);

/* n_cfg k-point SCFs in sequence: xp [n_cfg][n_atoms][3] (device), kpts
 * [n_cfg][3] (host); outputs strided by their per-configuration sizes (the
 * reference's jax.vmap(solver) over (xp, kpt)).  Returns the worst status. */
int hqcgb_scf_kpt_batch(hqcgb_kplan *plan, int n_cfg, const double *xp, const double *kpts,
                        const hqcgb_scf_out *out, void *stream);

/* Nuclear gradient dE/dR [n_atoms][3] (Hartree/Bohr, device) of the last
 * k-point SCF at its fixed k-point: the gradient of E - sigma*Se of that
 * single-k energy (hf_kpt / dft_kpt, hqc/pbc/solver.py:769-962; pes_kpt,
 * hqc/pbc/pes.py:88-98, minus the proton Ewald term).  FP64 on both
 * precisions.  No counterpart in the reference (forces are absent there,
 * doc/solver_algorithm.md:1210). */
int hqcgb_forces_kpt(hqcgb_kplan *plan, double *grad, void *stream);

/* hqcgb_scf_kpt_batch plus, when grad is not NULL, each configuration's
 * gradient into grad [n_cfg][n_atoms][3] (Hartree/Bohr, device): the
 * energy-and-force evaluation of a k-mesh (the reference's jax.vmap of
 * pes_kpt over (xp, kpt), pes.py:88-98). */
int hqcgb_pes_kpt_batch(hqcgb_kplan *plan, int n_cfg, const double *xp, const double *kpts,
                        const hqcgb_scf_out *out, double *grad, void *stream);

/* Copy an internal buffer of the last k-point SCF into dst (device): "S",
 * "T", "V", "H", "D", "F", "K", "St" (complex nao x nao), "phi" (conjugated
 * Bloch AOs, complex nao x N), "rho", "vh", "vloc" (real N).  Bytes copied
 * (or needed when dst is NULL), < 0 on error. */
long long hqcgb_kplan_query(hqcgb_kplan *plan, const char *name, void *dst, size_t bytes,
                            void *stream);

/* The k-point solver's DIIS coefficients (host computation, no device
 * work): B [space][space] complex (interleaved, host) is the reference's
 * unconjugated error matrix sum_mn e_i e_j (hqc/pbc/scf.py:177-188); solves
 * [[B + eta I, -1], [-1, 0]] [c; lambda] = [0; -1] with
 * eta = 1e-12 (tr B / space + 1) by LU with partial pivoting; c [space]
 * complex (interleaved, host). */
int hqcgb_diis_coefficients(int space, const double *B, double *c);

/* Complex Hermitian FP64 eigensolver on `batch` row-major n x n matrices A
 * (complex, interleaved; device, not modified; both triangles are read, so A
 * must be Hermitian): ascending eigenvalues w [batch][n] and eigenvectors as
 * the columns of V [batch][n][n] (complex).  The k-point solver's
 * jnp.linalg.eigh (hqc/pbc/solver.py:795, 812; hqc/pbc/scf.py:69,138,198). */
int hqcgb_eigh_herm(int n, int batch, const double *A, double *w, double *V, void *stream);

/* Run-time tuning knobs, set by the autotuner (hqc_gb300/tune.py) from
 * measurements; each changes launch shapes only (results agree to rounding):
 *   "quad_kchunk"   grid points per CTA of the Fock quadrature (a multiple
 *                   of 2048; default 2048),
 *   "exx_group"     orbitals per exact-exchange group (read when a plan is
 *                   created; default from a 1.5 GB buffer budget),
 *   "exx_gram_ctas" CTAs of the exchange's tensor-core Gram (read when a
 *                   plan is created; default 304).
 * value <= 0 restores the default.  No counterpart in the reference (XLA
 * picks its own launch shapes). */
int hqcgb_tune_set(const char *name, long long value);
/* The value set for a knob, 0 when it runs with its default. */
long long hqcgb_tune_get(const char *name);

/* Human-readable description of the last error on this host thread. */
const char *hqcgb_last_error(void);

/* Kernel launches issued on behalf of the caller since the last reset. */
long long hqcgb_launch_count(int reset);

/* Stage timing: hqcgb_profile(1) clears the record and starts timing every
 * stage (grid build, density, quadrature, FFT, xc, eigensolver, ...) with
 * CUDA events on the launching stream; hqcgb_profile(0) clears and stops.
 * No counterpart in the reference (its only timing is wall clock prints,
 * test/test.py:71-78). */
int hqcgb_profile(int enable);

/* Launch count and summed device milliseconds of stage index `stage`
 * (0 <= stage < 13) since hqcgb_profile(1); `name` receives its label. */
int hqcgb_stage_stats(int stage, const char **name, long long *count, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* HQCGB_H */
