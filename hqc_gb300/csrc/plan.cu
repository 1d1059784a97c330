// C ABI and host-side SCF driver of the hqcgb engine.
//
// hqcgb_plan_create replaces the factory-time part of make_solver
// (hqc/pbc/solver.py:61-231); hqcgb_scf replaces one call of the jitted
// hf_gamma / dft_gamma closure (solver.py:705-767, 839-899) including the
// DIIS / fixed-point loops of hqc/pbc/scf.py.  The loop control runs on the
// host; every array operation is a kernel on the caller's stream.
#include <atomic>
#include <map>
#include <mutex>
#include <thread>
#include <cstring>
#include <string>
#include <vector>
#include <cmath>
#include <cstdlib>
#include <algorithm>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {
static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};
void set_error(const std::string &m) { g_err = m; }

// Tuning knobs: launch parameters that change no result beyond rounding
// (K-chunk lengths, group sizes), set by the autotuner (hqc_gb300/tune.py)
// from measurements and read by the launchers.
static std::mutex g_tune_mu;
static std::map<std::string, long long> g_tune;
long long tune_get(const char *name, long long dflt) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(name);
  return it == g_tune.end() ? dflt : it->second;
}
void count_launch(long long k) { g_launches += k; }
static thread_local int g_gpu_share = 1;
int gpu_share() { return g_gpu_share; }
void set_gpu_share(int workers) { g_gpu_share = workers > 1 ? workers : 1; }
// GPU share of a batch worker for the scope of its loop (the caller's own
// thread runs worker 0 and gets its previous value back)
struct GpuShareScope {
  int prev;
  explicit GpuShareScope(int workers) : prev(gpu_share()) { set_gpu_share(workers); }
  ~GpuShareScope() { set_gpu_share(prev); }
};

static const char *kStageNames[ST_COUNT] = {"gto1d", "phi", "density", "quadrature", "fft", "xc",
                                            "jacobi", "gemm_small", "overlap", "force_grid",
                                            "exchange", "ewald", "other", "psi_density", "split"};
struct StageRec {
  int stage;
  cudaEvent_t a, b;
};
static std::atomic<bool> g_profile{false};
// Dynamic shared-memory limits already raised, per (device, kernel).  Batch
// workers launch from several host threads, so check-and-raise is one
// critical section and a limit is never lowered under a concurrent launch.
static std::mutex g_smem_mu;
static std::map<std::pair<int, const void *>, size_t> g_smem_set;

void ensure_dyn_smem(const void *func, size_t bytes) {
  int dev = 0;
  HQ_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_smem_mu);
  size_t &cur = g_smem_set[{dev, func}];
  if (bytes <= cur) return;
  HQ_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}

static std::mutex g_rec_mu;  // guards g_recs and g_event_pool (batch workers record too)
static std::vector<StageRec> g_recs;
static std::vector<cudaEvent_t> g_event_pool;
static thread_local int g_open[ST_COUNT];
static thread_local cudaEvent_t g_open_ev[ST_COUNT];

static cudaEvent_t take_event() {
  std::lock_guard<std::mutex> lock(g_rec_mu);
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// HQCGB_NVTX=1 also opens an NVTX range per stage scope (named as in
// kStageNames), for ncu --nvtx filters and timeline tools.
static bool nvtx_on() {
  static const bool v = [] {
    const char *e = std::getenv("HQCGB_NVTX");
    return e && e[0] == '1';
  }();
  return v;
}

void stage_mark(int stage, cudaStream_t st, bool begin) {
  if (nvtx_on()) {
    if (begin) nvtxRangePushA(kStageNames[stage]);
    else nvtxRangePop();
  }
  if (!g_profile) return;
  if (begin) {
    if (g_open[stage]++ > 0) return;  // nested scopes of one stage count once
    g_open_ev[stage] = take_event();
    cudaEventRecord(g_open_ev[stage], st);
  } else {
    if (--g_open[stage] > 0) return;
    cudaEvent_t b = take_event();
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> lock(g_rec_mu);
    g_recs.push_back({stage, g_open_ev[stage], b});
  }
}
}  // namespace hqcgb

using namespace hqcgb;

static constexpr double kMadelungSC = 0.22578495;  // solver.py:404
// Exact exchange skips orbitals with occupation <= 1e-14 (besides the caller's
// exx_occ_threshold): each adds f_i times a bounded matrix to K, below FP64
// rounding of the sum; with Fermi smearing most virtual orbitals are such.
static constexpr double kExxOccFloor = 1e-14;
// K blocks of 32 AOs the orbital-density kernel accumulates per TMEM slot
// before a compensated drain: 2 measured 14% faster than 1 on the H54
// shapes at a relative density bias of -2.9e-7 (the tensor core truncates).
static constexpr int kPsiDrain = 2;
static constexpr int kThinOcc = 64;  // occupied-block GEMMs up to this many orbitals

// HQCGB_TRACE=1 prints one line per SCF iteration (energy, error norm) to stderr.
static bool trace_on() {
  static const bool v = [] {
    const char *e = std::getenv("HQCGB_TRACE");
    return e && e[0] == '1';
  }();
  return v;
}

struct hqcgb_plan {
  hqcgb_params P{};
  std::vector<double> h_alpha, h_coef, h_lat1d, h_lattice;
  std::vector<int> h_l, h_cart;
  int n = 0, nb = 0, nao = 0, ng = 0, nprim = 0;
  long long N = 0;
  double L = 0, Omega = 0, dV = 0;
  bool gga = false, need_dphi = false, hf = false;
  std::vector<void *> allocs;

  // constant tables
  double *alpha = nullptr, *coef = nullptr, *lat1d = nullptr, *lattice = nullptr;
  int *ao_l = nullptr, *ao_cart = nullptr;
  double2 *tw = nullptr;
  double *coul = nullptr;
  // geometry
  double *xp = nullptr, *F1d = nullptr, *phi = nullptr, *dphi = nullptr;
  double2 *ph = nullptr;
  double *S = nullptr, *T = nullptr, *V = nullptr, *H = nullptr, *St = nullptr, *vorth = nullptr;
  // scf matrices
  double *F = nullptr, *F2e = nullptr, *K = nullptr, *Fp = nullptr, *C = nullptr, *c1 = nullptr,
         *w = nullptr, *occ = nullptr, *D = nullptr, *t1 = nullptr, *t2 = nullptr, *err = nullptr,
         *Fk = nullptr, *ek = nullptr, *Bm = nullptr, *dc = nullptr, *jtmp = nullptr,
         *jA = nullptr, *ws = nullptr, *mu = nullptr;
  int *jstat = nullptr, *ibad = nullptr;
  // grid
  double *rho = nullptr, *grho = nullptr, *vh = nullptr, *wq = nullptr, *vxc = nullptr,
         *u = nullptr, *vloc = nullptr, *veff = nullptr, *X = nullptr, *Z = nullptr,
         *DPsi = nullptr, *W = nullptr, *psi = nullptr;
  double2 *cbuf = nullptr;
  long long cbuf_batch = 0;
  double *qpart = nullptr, *xpart = nullptr, *fpart = nullptr, *gpart = nullptr, *vpart = nullptr;
  // mixed-precision grid data (row stride ld floats)
  bool mixed = false;
  long long ld = 0;
  float *dphiT32 = nullptr, *Yhl = nullptr;  // grid-major AO gradients; split Y^T
  double *ovq = nullptr;                     // lattice sums of the S/T Hermite products
  bool allow_warm = false;                   // warm eigen-refinement after the DIIS warm-up
  // mixed path: occupied block Y = C_occ sqrt(f) (n x nuse_dm) when few
  // orbitals are occupied, so that D = Y Y^T and S D F = (S Y)(F^T Y)^T run
  // as GEMMs with K = nuse_dm
  double *Yd = nullptr, *Y2 = nullptr, *xerr = nullptr;
  int nuse_dm = 0;
  double *c1_prev = nullptr;                 // eigenvectors of the previous F'
  bool have_prev = false;
  // mixed Kohn-Sham forces from the occupied orbitals on the grid
  bool orb_forces = false, keep_psi = false;
  float *psi32 = nullptr, *F1d32 = nullptr, *Y32 = nullptr;  // [4][64][N], F1d, [nao][64]
  int npsi_kept = 0, nuse_kept = 0;
  std::vector<double> hocc;                   // host copy of the occupations
  float *phi32 = nullptr, *dphi32 = nullptr, *phiT32 = nullptr, *D32 = nullptr, *w32 = nullptr,
        *u32 = nullptr;
  float *phihl = nullptr, *zhl = nullptr;  // TF32 hi/lo pieces of phi and of the quadrature operand
  double *tcq_part = nullptr, *tcd_part = nullptr;
  float2 *cbuf32 = nullptr;
  int *tc_err = nullptr;
  MixedEigWork mew{};
  // exact exchange in the occupied-pair form (exchange.cu); R = double on
  // the FP64 path, float on the mixed path
  bool exx_fused = false;
  ExxGeom exx{};
  int exx_g = 0;               // orbitals per Fock group (Q and T capacity)
  int exx_grad_g = 0;          // orbitals per gradient group (4 rows per AO)
  void *exx_T = nullptr;       // plane-transformed pairs
  void *exx_Q = nullptr;       // FP64 [nao][g 2N_h], or the TF32 pieces [2][nao][exx_ldq]
  long long exx_ldq = 0;
  void *exx_psi = nullptr;     // psi~_k = sqrt(f_k) psi_k, [nao][N] (R)
  bool exx_psi_ready = false;  // psi~ of the current density already written (mixed density pass)
  double *exx_part = nullptr;  // gradient dot products
  double *exx_tcpart = nullptr, *exx_Kt = nullptr;  // mixed: Gram partial tiles, group sum
  void *exx_wsq = nullptr;     // pair weights (depend on the box)
  int exx_kchunk = 0;
  int nuse_occ = 0;            // orbitals with occupation > 1e-14 (host copy of occ in hocc)
  double *scal = nullptr;  // device scalars
  double *hscal = nullptr; // pinned host mirror
  // last state
  bool have_state = false;
  std::vector<double> h_occ;

  template <class T>
  T *alloc(size_t count) {
    void *p = nullptr;
    if (count == 0) count = 1;
    HQ_CUDA(cudaMalloc(&p, count * sizeof(T)));
    allocs.push_back(p);
    return (T *)p;
  }
  // concurrent batch workers: sub-plans with their own workspaces and streams
  int lat1d_cap = 0, lattice_cap = 0;  // device capacity of the lattice arrays (entries)
  int concurrency = 1;
  std::vector<hqcgb_plan *> workers;
  std::vector<cudaStream_t> wstreams;

  ~hqcgb_plan() {
    for (hqcgb_plan *w : workers) delete w;
    for (cudaStream_t s : wstreams) cudaStreamDestroy(s);
    for (void *p : allocs) cudaFree(p);
    if (hscal) cudaFreeHost(hscal);
  }
};

// scal slots
enum { S_TRHD = 0, S_EXC = 1, S_VHRHO = 2, S_TRKD = 3, S_ERR2 = 4, S_SE = 5, S_KI = 6, S_VEP = 7,
       S_SFREE = 8, S_NSLOT = 16 };

static void upload(void *dst, const void *src, size_t bytes) {
  HQ_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
}

static double occ_shift(const hqcgb_plan *p) {
  const hqcgb_params &P = p->P;
  if (!P.smearing) return 0.0;
  double n = P.n_atoms, nmo = p->nao;
  if (P.smearing_method == HQCGB_SMEAR_FERMI) return -P.smearing_sigma * std::log(2 * nmo / n - 1);
  // erfinv(1 - n/nmo) by Newton on erf (host, once)
  double y = 1.0 - n / nmo, x = 0.0;
  for (int it = 0; it < 200; ++it) {
    double f = std::erf(x) - y;
    double d = 2.0 / std::sqrt(M_PI) * std::exp(-x * x);
    double dx = f / d;
    x -= dx;
    if (std::fabs(dx) < 1e-16 * (1 + std::fabs(x))) break;
  }
  return -P.smearing_sigma * x;
}

static void create(const hqcgb_params *in, hqcgb_plan *p) {
  const hqcgb_params &P = *in;
  HQ_REQUIRE(P.n_atoms >= 1, "n_atoms must be >= 1");
  HQ_REQUIRE(P.n_grid >= 3 && P.n_grid <= kMaxGrid, "n_grid out of range");
  HQ_REQUIRE(P.nao_atom >= 1 && P.n_prim >= 1, "empty basis");
  HQ_REQUIRE(P.L > 0, "L must be positive");
  HQ_REQUIRE(P.n_atoms * P.nao_atom <= kMaxNao, "too many AOs");
  HQ_REQUIRE(P.diis_space >= 1 && P.diis_space <= 32, "diis_space must be in [1, 32]");
  HQ_REQUIRE(P.max_cycle >= 0, "max_cycle must be >= 0");
  HQ_REQUIRE(!P.smearing || P.smearing_sigma > 0, "smearing_sigma must be > 0 with smearing");
  HQ_REQUIRE(P.n_atoms * P.nao_atom >= P.n_atoms / 2, "n_mo < n/2");
  HQ_REQUIRE(P.precision == HQCGB_PREC_FP64 || P.precision == HQCGB_PREC_MIXED, "bad precision");
  p->P = P;
  p->n = P.n_atoms;
  p->nb = P.nao_atom;
  p->nao = p->n * p->nb;
  p->ng = P.n_grid;
  p->nprim = P.n_prim;
  p->N = (long long)p->ng * p->ng * p->ng;
  p->L = P.L;
  p->Omega = P.L * P.L * P.L;
  p->dV = p->Omega / (double)p->N;
  p->hf = !P.dft;
  p->gga = P.dft && P.xc == HQCGB_XC_PBE;
  p->need_dphi = p->gga || P.want_forces;
  p->h_alpha.assign(P.alpha, P.alpha + P.n_prim);
  p->h_coef.assign(P.coef, P.coef + P.nao_atom * P.n_prim);
  p->h_l.assign(P.ao_l, P.ao_l + P.nao_atom);
  p->h_cart.assign(P.ao_cart, P.ao_cart + P.nao_atom);
  for (int k = 0; k < P.nao_atom; ++k) {
    HQ_REQUIRE(p->h_l[k] == 0 || p->h_l[k] == 1, "only s and p AOs are supported");
    HQ_REQUIRE(p->h_cart[k] >= 0 && p->h_cart[k] < 3, "bad cartesian index");
  }
  p->h_lat1d.assign(P.lat1d, P.lat1d + P.n_lat1d);
  p->h_lattice.assign(P.lattice, P.lattice + 3 * P.n_lattice);
  int n = p->n, nao = p->nao;
  long long N = p->N;
  size_t nn = (size_t)nao * nao;

  p->alpha = p->alloc<double>(P.n_prim);
  upload(p->alpha, P.alpha, sizeof(double) * P.n_prim);
  p->coef = p->alloc<double>(P.nao_atom * P.n_prim);
  upload(p->coef, P.coef, sizeof(double) * P.nao_atom * P.n_prim);
  p->ao_l = p->alloc<int>(P.nao_atom);
  upload(p->ao_l, P.ao_l, sizeof(int) * P.nao_atom);
  p->ao_cart = p->alloc<int>(P.nao_atom);
  upload(p->ao_cart, P.ao_cart, sizeof(int) * P.nao_atom);
  p->lat1d = p->alloc<double>(P.n_lat1d);
  upload(p->lat1d, P.lat1d, sizeof(double) * P.n_lat1d);
  p->lattice = p->alloc<double>(3 * P.n_lattice);
  upload(p->lattice, P.lattice, sizeof(double) * 3 * P.n_lattice);
  p->lat1d_cap = P.n_lat1d;
  p->lattice_cap = P.n_lattice;
  std::vector<double2> tw(p->ng);
  for (int k = 0; k < p->ng; ++k) {
    double a = -2.0 * M_PI * k / p->ng;
    tw[k] = make_double2(std::cos(a), std::sin(a));
  }
  p->tw = p->alloc<double2>(p->ng);
  upload(p->tw, tw.data(), sizeof(double2) * p->ng);
  p->coul = p->alloc<double>(N);
  launch_coulomb_table(p->ng, p->L, p->coul, 0);

  p->mixed = P.precision == HQCGB_PREC_MIXED;
  p->ld = (N + 63) / 64 * 64;
  p->xp = p->alloc<double>(3 * n);
  p->F1d = p->alloc<double>((size_t)n * 3 * p->ng * P.n_prim * 6);
  // the FP64 AO grid is kept by the FP64 path, and by the mixed path for the
  // parts it runs in FP64 (exact exchange, forces)
  p->orb_forces = p->mixed && !p->hf && P.want_forces && !P.smearing;
  const bool fp64_forces = P.want_forces && !p->orb_forces;
  bool fp64_grid = !p->mixed || p->hf || fp64_forces;
  if (fp64_grid) {
    p->phi = p->alloc<double>((size_t)nao * N);
    if (p->need_dphi) p->dphi = p->alloc<double>((size_t)3 * nao * N);
  }
  if (p->mixed) {
    p->phi32 = p->alloc<float>((size_t)nao * p->ld);
    if (p->gga) p->dphi32 = p->alloc<float>((size_t)3 * nao * p->ld);
    p->phiT32 = p->alloc<float>((size_t)N * tc_ldk(nao));
    if (p->gga) p->dphiT32 = p->alloc<float>((size_t)3 * N * tc_ldk(nao));
    p->Yhl = p->alloc<float>((size_t)2 * tc_psi_max(false) * tc_ldk(nao));
    p->hocc.resize(nao);
    p->D32 = p->alloc<float>((size_t)nao * tc_ldk(nao));
    HQ_CUDA(cudaMemset(p->D32, 0, sizeof(float) * nao * tc_ldk(nao)));
    p->phihl = p->alloc<float>((size_t)2 * nao * p->ld);
    p->zhl = p->alloc<float>((size_t)2 * nao * p->ld);
    p->w32 = p->alloc<float>(p->ld);
    p->u32 = p->alloc<float>(3 * p->ld);
    p->tcq_part = p->alloc<double>(tc_quad_partial_doubles(nao, N));
    p->tcd_part = p->alloc<double>(tc_density_partial_doubles(nao, p->ld, p->gga));
    p->cbuf32 = p->alloc<float2>(N);
    p->tc_err = p->alloc<int>(1);
    HQ_CUDA(cudaMemset(p->tc_err, 0, sizeof(int)));
    p->mew.A32 = p->alloc<float>(nn);
    p->mew.V32 = p->alloc<float>(nn);
    p->mew.w32 = p->alloc<float>(nao);
    p->mew.work32 = p->alloc<float>(nn);
    p->mew.f32scr = p->alloc<float>(eigh_f32_scratch_floats(nao));
    p->mew.T1 = p->alloc<double>(nn);
    p->mew.S = p->alloc<double>(nn);
    p->mew.G = p->alloc<double>(nn);
    p->mew.E = p->alloc<double>(nn);
    p->mew.status = p->alloc<int>(1);
    p->mew.emax = p->alloc<double>(16);
    p->mew.wbuf = p->alloc<double>(2 * nn);
    p->mew.iwork = p->alloc<int>(5 * (size_t)nao + 1);
    p->c1_prev = p->alloc<double>(nn);
    p->Yd = p->alloc<double>((size_t)nao * kThinOcc);
    p->Y2 = p->alloc<double>((size_t)nao * kThinOcc);
    p->xerr = p->alloc<double>(nn);
    p->F1d32 = p->alloc<float>((size_t)n * 3 * p->ng * P.n_prim * 6);
    if (p->orb_forces) {
      p->psi32 = p->alloc<float>((size_t)(p->gga ? 4 : 1) * tc_psi_max(false) * N);
      p->Y32 = p->alloc<float>((size_t)nao * tc_psi_max(false));
    }
  }
  p->ph = p->alloc<double2>((size_t)n * 3 * p->ng);
  p->ovq = p->alloc<double>(ovl_scratch_doubles(n, P.n_prim));
  for (double **m : {&p->S, &p->T, &p->V, &p->H, &p->St, &p->vorth, &p->F, &p->F2e, &p->K, &p->Fp,
                     &p->C, &p->c1, &p->D, &p->t1, &p->t2, &p->err, &p->jtmp, &p->jA})
    *m = p->alloc<double>(nn);
  p->w = p->alloc<double>(nao);
  p->ws = p->alloc<double>(nao);
  p->occ = p->alloc<double>(nao);
  p->mu = p->alloc<double>(1);
  p->Fk = p->alloc<double>((size_t)P.diis_space * nn);
  p->ek = p->alloc<double>((size_t)P.diis_space * nn);
  p->Bm = p->alloc<double>((size_t)P.diis_space * P.diis_space);
  p->dc = p->alloc<double>(P.diis_space);
  p->jstat = p->alloc<int>(1);
  p->ibad = p->alloc<int>(1);
  p->rho = p->alloc<double>(N);
  p->vh = p->alloc<double>(N);
  p->wq = p->alloc<double>(N);
  p->vxc = p->alloc<double>(N);
  p->vloc = p->alloc<double>(N);
  p->veff = p->alloc<double>(N);
  p->psi = p->alloc<double>(N);
  if (p->gga) {
    p->grho = p->alloc<double>(3 * N);
    p->u = p->alloc<double>(3 * N);
    if (!p->mixed || fp64_forces) p->Z = p->alloc<double>((size_t)nao * N);
  }
  if (fp64_forces || p->hf) {
    p->X = p->alloc<double>((size_t)nao * N);
    if (!p->Z) p->Z = p->alloc<double>((size_t)nao * N);
  }
  if (fp64_forces && p->gga) p->DPsi = p->alloc<double>((size_t)nao * N);
  long long qcols = N;
  p->exx_fused = p->hf && exx_fused_supported(p->ng, P.n_prim, !p->mixed);
  if (p->exx_fused) {
    // orbitals per group: T and Q within about 1.5 GB
    const long long L2 = exx_pair_len(p->ng);  // reals of one pair's half spectrum
    const size_t rb = p->mixed ? sizeof(float) : sizeof(double);
    const double per_orb = (double)nao * L2 * (rb + 8.0);
    p->exx_g = (int)std::max(1.0, std::min(16.0, std::floor(1.5e9 / per_orb)));
    // a tuned group size, within 1..16 and twice the memory budget
    const long long tg = tune_get("exx_group", 0);
    if (tg > 0) p->exx_g = (int)std::max(1.0, std::min({16.0, (double)tg, std::floor(3e9 / per_orb)}));
    p->exx_g = std::min(p->exx_g, nao);
    const int rows_cap = std::max(p->exx_g, 4) * nao;  // pair rows T holds
    p->exx_grad_g = rows_cap / (4 * nao);
    p->exx_T = p->alloc<char>((size_t)rows_cap * (L2 / 2) * 2 * rb);
    // psi~ rows: every orbital, and at least the orbital-density kernel's
    // padded width (a multiple of 16, up to 64), which writes them on the
    // mixed path
    const int psi_rows = std::max(nao, tc_psi_width(std::min(nao, tc_psi_max(false))));
    p->exx_psi = p->alloc<char>((size_t)psi_rows * N * rb);
    p->exx_part = p->alloc<double>((size_t)p->exx_grad_g * nao * p->ng * 3);
    void *wsq = p->alloc<char>((size_t)(L2 / 2) * rb);
    const long long gK = (long long)p->exx_g * L2;
    if (p->mixed) {
      p->exx_ldq = (gK + 31) / 32 * 32;
      p->exx_Q = p->alloc<float>((size_t)2 * nao * p->exx_ldq);
      const int ctas = (int)std::max<long long>(1, tune_get("exx_gram_ctas", 2 * 152));
      const int chunks = std::max(1, ctas / tc_quad_tiles(nao, true));
      p->exx_kchunk = (int)std::max<long long>(2048, (gK + chunks - 1) / chunks / 32 * 32 + 32);
      p->exx_tcpart = p->alloc<double>(tc_quad_partial_doubles(nao, gK, p->exx_kchunk));
      p->exx_Kt = p->alloc<double>(nn);
      launch_exx_weights<float>(p->ng, p->L, p->dV, (float *)wsq, 0);
    } else {
      p->exx_ldq = gK;
      p->exx_Q = p->alloc<double>((size_t)nao * gK);
      qcols = std::max(qcols, gK);
      launch_exx_weights<double>(p->ng, p->L, p->dV, (double *)wsq, 0);
    }
    p->exx = ExxGeom{p->ng, nao, p->nb, p->nprim, p->tw, p->coef, p->ao_l, p->ao_cart, wsq};
    p->exx_wsq = wsq;
  }
  // the per-AO pair potentials of the fallback exchange (grids beyond the
  // fused kernels' shared memory)
  p->cbuf_batch = (p->hf && !p->exx_fused) ? nao : 1;
  if (p->hf && !p->exx_fused) p->W = p->alloc<double>((size_t)nao * N);
  p->cbuf = p->alloc<double2>((size_t)p->cbuf_batch * N);
  if (!p->mixed || p->hf) p->qpart = p->alloc<double>((size_t)quad_chunks(qcols) * nn);
  p->xpart = p->alloc<double>((size_t)2 * xc_blocks(N));
  if (P.want_forces) {
    p->fpart = p->alloc<double>(std::max((size_t)nao * force_grid_blocks(N) * 3,
                                         (size_t)force_orb_blocks(N) * n * 3));
    p->gpart = p->alloc<double>((size_t)n * n * p->nb * p->nb * 3);
    p->vpart = p->alloc<double>((size_t)vloc_force_blocks(N) * n * 3);
  }
  p->scal = p->alloc<double>(S_NSLOT);
  HQ_CUDA(cudaMallocHost(&p->hscal, S_NSLOT * sizeof(double)));
  HQ_CUDA(cudaDeviceSynchronize());
}

// ---------------------------------------------------------------------------
struct Ctx {
  hqcgb_plan *p;
  cudaStream_t st;
};

static void sync_scalars(Ctx &c) {
  HQ_CUDA(cudaMemcpyAsync(c.p->hscal, c.p->scal, S_NSLOT * sizeof(double), cudaMemcpyDeviceToHost,
                          c.st));
  HQ_CUDA(cudaStreamSynchronize(c.st));
}

// Symmetric eigensolver: Householder + QL (eigh_fp64.cu); the Jacobi solver
// is kept as the fallback when a QL sweep limit is hit.
static void eigh(Ctx &c, const double *A, double *vecs, double *vals, bool wide = false,
                 bool loose = false) {
  hqcgb_plan *p = c.p;
  int n = p->nao;
  if (p->mixed) {
    // FP32 solve, then FP64 Ogita-Aishima refinement
    if (eigh_mixed(n, A, vecs, vals, p->mew, c.st, wide, loose)) {
      HQ_CUDA(cudaMemsetAsync(p->jstat, 0, sizeof(int), c.st));
      return;
    }
    if (trace_on()) fprintf(stderr, "eigh: mixed solve did not converge, FP64 solve\n");
  }
  HQ_CUDA(cudaMemcpyAsync(p->jA, A, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
  eigh_tql(n, 1, p->jA, vecs, vals, p->jtmp, p->jstat, c.st);
  int stt = 0;
  HQ_CUDA(cudaMemcpyAsync(&stt, p->jstat, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  HQ_CUDA(cudaStreamSynchronize(c.st));
  if (stt < 0) {
    HQ_CUDA(cudaMemcpyAsync(p->jA, A, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
    jacobi_eigh(n, 1, p->jA, vecs, vals, p->jtmp, p->jstat, c.st);
  }
}

// C, w from a Fock matrix: F' = v^T F v, eigh, C = v c'.  In the mixed path
// the solves inside the SCF loop stop at the loose refinement level (their
// eigenvectors only build the next density); the returned orbitals are
// refined to rounding level after the loop (refine_last).
static void diagonalize(Ctx &c, const double *Fm) {
  hqcgb_plan *p = c.p;
  int n = p->nao;
  gemm(false, false, n, n, n, 1.0, Fm, n, p->vorth, n, nullptr, 0.0, p->t1, n, c.st);
  gemm(true, false, n, n, n, 1.0, p->vorth, n, p->t1, n, nullptr, 0.0, p->Fp, n, c.st);
  if (p->mixed) {  // exact symmetry for the refinement (rounding of the two GEMMs)
    axpby(n, 0.5, p->Fp, 0.5, p->Fp, true, p->t1, c.st);
    HQ_CUDA(cudaMemcpyAsync(p->Fp, p->t1, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
  }
  // mixed: refine the previous iteration's eigenvectors when they are close
  bool done = p->mixed && p->have_prev && p->allow_warm &&
              eigh_mixed_warm(n, p->Fp, p->c1_prev, p->c1, p->w, p->mew, c.st, true);
  if (!done) eigh(c, p->Fp, p->c1, p->w, false, p->mixed);
  if (p->mixed) {
    HQ_CUDA(cudaMemcpyAsync(p->c1_prev, p->c1, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
    p->have_prev = true;
  }
  if (trace_on() && p->mixed) fprintf(stderr, "eigh: %s\n", done ? "warm start" : "full solve");
  gemm(false, false, n, n, n, 1.0, p->vorth, n, p->c1, n, nullptr, 0.0, p->C, n, c.st);
}

// Mixed path: the last solve of the loop (F' in Fp, its vectors in c1_prev)
// refined to rounding level, then C = v c'.
static void refine_last(Ctx &c) {
  hqcgb_plan *p = c.p;
  const int n = p->nao;
  if (!eigh_mixed_warm(n, p->Fp, p->c1_prev, p->c1, p->w, p->mew, c.st, false))
    eigh(c, p->Fp, p->c1, p->w);
  HQ_CUDA(cudaMemcpyAsync(p->c1_prev, p->c1, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
  gemm(false, false, n, n, n, 1.0, p->vorth, n, p->c1, n, nullptr, 0.0, p->C, n, c.st);
}

static void density_matrix(Ctx &c) {
  hqcgb_plan *p = c.p;
  const hqcgb_params &P = p->P;
  int n = p->nao;
  occupations(P.n_atoms, n, P.smearing, P.smearing_method, P.smearing_sigma, P.search_method,
              P.search_cycle, P.search_tol, occ_shift(p), p->w, p->occ, p->mu, c.st);
  p->nuse_dm = 0;
  p->exx_psi_ready = false;
  if (p->mixed || p->hf) {
    // The one host copy of the occupations per iteration: the mixed density
    // and the exchange of the Fock build that follows size their launches
    // from it.  Orbitals with a non-negligible occupation come first
    // (ascending energies).
    p->hocc.resize(n);
    HQ_CUDA(cudaMemcpyAsync(p->hocc.data(), p->occ, sizeof(double) * n, cudaMemcpyDeviceToHost, c.st));
    HQ_CUDA(cudaStreamSynchronize(c.st));
    int nuse = 0;
    for (int k = 0; k < n; ++k)
      if (p->hocc[k] > 1e-14) nuse = k + 1;
    p->nuse_occ = nuse;
    if (p->mixed && nuse >= 1 && nuse <= kThinOcc) {
      launch_occ_block(p->C, p->occ, n, nuse, p->Yd, c.st);
      gemm(false, true, n, n, nuse, 1.0, p->Yd, nuse, p->Yd, nuse, nullptr, 0.0, p->D, n, c.st);
      p->nuse_dm = nuse;
      return;
    }
  }
  gemm(false, true, n, n, n, 1.0, p->C, n, p->C, n, p->occ, 0.0, p->D, n, c.st);
}

static void poisson(Ctx &c, const double *src, double *dst, bool keep_spectrum = false) {
  hqcgb_plan *p = c.p;
  launch_real_to_complex(src, nullptr, p->N, 1, p->cbuf, c.st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, false, c.st);
  (void)keep_spectrum;
  launch_scale_complex(p->cbuf, p->coul, p->N, 1, c.st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, true, c.st);
  launch_complex_real(p->cbuf, p->N, 1.0, dst, c.st);
}

// Madelung G = 0 term of the exchange: K = Kpair + c_M S~ D S~
// (solver.py:404, 431: eris0 = unknown1 * 4 pi / L * S~ (x) S~).
static void exchange_madelung(Ctx &c) {
  hqcgb_plan *p = c.p;
  const int n = p->nao;
  HQ_CUDA(cudaMemcpyAsync(p->t1, p->K, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
  double cM = 4.0 * M_PI / p->L * kMadelungSC;
  gemm(false, false, n, n, n, 1.0, p->St, n, p->D, n, nullptr, 0.0, p->t2, n, c.st);
  gemm(false, false, n, n, n, 1.0, p->t2, n, p->St, n, nullptr, 0.0, p->K, n, c.st);
  axpby(n, 1.0, p->t1, cM, p->K, false, p->K, c.st);
}

// Orbitals the exchange runs over: the prefix of orbitals whose occupation
// exceeds max(exx_occ_threshold, 1e-14) (each skipped one adds f_i times a
// bounded matrix to K, below FP64 rounding of the sum).
static int exx_count(const hqcgb_plan *p) {
  const double thr = std::max(p->P.exx_occ_threshold, kExxOccFloor);
  int nuse = 0;
  for (int k = 0; k < p->nao; ++k)
    if (p->hocc[k] > thr) nuse = k + 1;
  return nuse;
}

// psi~_k = sqrt(f_k) psi_k on the grid for k < nuse, unless the mixed
// density pass already wrote them.
static void exx_orbitals(Ctx &c, int nuse) {
  hqcgb_plan *p = c.p;
  if (p->exx_psi_ready || nuse == 0) return;
  if (p->mixed)
    launch_psi_all<float>(p->C, p->occ, p->nao, p->nao, nuse, p->phi32, p->ld, p->N,
                          static_cast<float *>(p->exx_psi), c.st);
  else
    launch_psi_all<double>(p->C, p->occ, p->nao, p->nao, nuse, p->phi, p->N, p->N,
                           static_cast<double *>(p->exx_psi), c.st);
  p->exx_psi_ready = true;
}

// Exact exchange K (with the Madelung G=0 term), solver.py:430-431, 604-614,
// in the occupied-pair form of exchange.cu: per group of orbitals the pair
// planes, the column transforms that write Q, and K += Q Q^T.
static void exchange(Ctx &c) {
  hqcgb_plan *p = c.p;
  const int n = p->nao;
  const long long N = p->N;
  HQ_STAGE(ST_EXCHANGE, c.st);
  HQ_CUDA(cudaMemsetAsync(p->K, 0, sizeof(double) * n * n, c.st));
  const int nuse = exx_count(p);
  exx_orbitals(c, nuse);
  const long long L2 = exx_pair_len(p->ng);
  for (int j0 = 0; j0 < nuse; j0 += p->exx_g) {
    const int g = std::min(p->exx_g, nuse - j0);
    const long long NK = (long long)g * L2;
    if (p->mixed) {
      launch_exx_plane<float>(p->exx, p->F1d32, nullptr, 0, static_cast<float *>(p->exx_psi) + j0 * N, N, g,
                              p->exx_T, c.st);
      launch_exx_column_q<float>(p->exx, p->exx_T, g, p->exx_Q, p->exx_ldq, true, c.st);
      const float *Q = static_cast<const float *>(p->exx_Q);
      // drained every K = 32 stage: K is a Gram matrix of same-sign sums on
      // its diagonal, where the tensor core's truncating FP32 accumulation
      // would bias long accumulator chains
      launch_tc_quad_split(Q, Q, n, NK, p->exx_ldq, true, false, 1.0, p->exx_tcpart, p->exx_Kt, p->tc_err,
                           c.st, 1, p->exx_kchunk);
      axpby(n, 1.0, p->K, 1.0, p->exx_Kt, false, p->K, c.st);
    } else {
      launch_exx_plane<double>(p->exx, p->F1d, nullptr, 0, static_cast<double *>(p->exx_psi) + j0 * N, N, g,
                               p->exx_T, c.st);
      launch_exx_column_q<double>(p->exx, p->exx_T, g, p->exx_Q, NK, false, c.st);
      const double *Q = static_cast<const double *>(p->exx_Q);
      launch_quadrature(Q, Q, nullptr, n, NK, true, 1.0, true, p->qpart, p->K, c.st);
    }
  }
  exchange_madelung(c);
}

// Exact exchange on grids beyond the fused kernels' shared memory: per
// orbital, pair densities, a full complex 3D FFT Poisson solve and the
// real-space quadrature.  With Zacc != nullptr also accumulates the orbital
// force operand Z_p += f_j psi_j (D W_j)_p.
static void exchange_legacy(Ctx &c, double *Zacc) {
  hqcgb_plan *p = c.p;
  int n = p->nao;
  long long N = p->N;
  HQ_CUDA(cudaMemsetAsync(p->K, 0, sizeof(double) * n * n, c.st));
  for (int i = 0; i < n; ++i) {
    double f = p->hocc[i];
    if (!(f > std::max(p->P.exx_occ_threshold, kExxOccFloor))) continue;
    launch_psi(p->C, n, i, p->phi, N, p->psi, c.st);
    launch_real_to_complex(p->phi, p->psi, N, n, p->cbuf, c.st);
    launch_fft3d(p->cbuf, p->ng, n, p->tw, false, c.st);
    launch_scale_complex(p->cbuf, p->coul, N, n, c.st);
    launch_fft3d(p->cbuf, p->ng, n, p->tw, true, c.st);
    launch_complex_real(p->cbuf, (long long)n * N, 1.0, p->W, c.st);
    launch_quadrature(p->phi, p->W, p->psi, n, N, false, f * p->dV, true, p->qpart, p->K, c.st);
    if (Zacc) {
      launch_density(p->W, nullptr, p->D, n, N, p->vh /*scratch*/, nullptr, p->X, c.st);
      launch_axpy_grid((long long)n * N, N, f, p->psi, p->X, Zacc, c.st);
    }
  }
  axpby(n, 0.5, p->K, 0.5, p->K, true, p->t1, c.st);
  HQ_CUDA(cudaMemcpyAsync(p->K, p->t1, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, c.st));
  exchange_madelung(c);
}

// Exchange part of the nuclear gradient (exchange.cu, gradient mode) for the
// density of the last Fock build; X = D phi (FP64) on the grid.
static void exchange_gradient(Ctx &c, double *grad) {
  hqcgb_plan *p = c.p;
  const long long N = p->N;
  const int nuse = exx_count(p);
  exx_orbitals(c, nuse);
  for (int j0 = 0; j0 < nuse; j0 += p->exx_grad_g) {
    const int g = std::min(p->exx_grad_g, nuse - j0);
    if (p->mixed) {
      launch_exx_plane<float>(p->exx, p->F1d32, p->X, N, static_cast<float *>(p->exx_psi) + j0 * N, N, g,
                              p->exx_T, c.st);
      launch_exx_column_grad<float>(p->exx, p->exx_T, g, p->exx_part, grad, c.st);
    } else {
      launch_exx_plane<double>(p->exx, p->F1d, p->X, N, static_cast<double *>(p->exx_psi) + j0 * N, N, g,
                               p->exx_T, c.st);
      launch_exx_column_grad<double>(p->exx, p->exx_T, g, p->exx_part, grad, c.st);
    }
  }
}

// Two-electron part of the Fock matrix and the energy pieces for density D.
// Leaves F = H + F2e in p->F; scalars in p->scal.
static double fock(Ctx &c) {
  hqcgb_plan *p = c.p;
  const hqcgb_params &P = p->P;
  int n = p->nao;
  long long N = p->N;
  int kind = P.dft ? P.xc : -1;
  if (p->mixed) {
    // tensor-core density (3xTF32, FP32 accumulation, FP64 sums), FP32
    // Poisson, FP64 xc, tensor-core quadrature
    // orbitals with a non-negligible occupation (sorted by energy, so first;
    // counted from the host copy density_matrix made)
    const int nuse = p->nuse_occ;
    if (nuse <= tc_psi_max(p->gga)) {
      // rho = sum_k |psi_k|^2 from Y = C_occ sqrt(f) (n_use / n_ao of the work);
      // Hartree-Fock keeps psi~_k = sqrt(f_k) psi_k for the exchange
      float *psi_out = p->keep_psi ? p->psi32 : nullptr;
      if (p->exx_fused && !psi_out) psi_out = static_cast<float *>(p->exx_psi);
      launch_psi_operand(p->C, p->occ, n, n, nuse, tc_ldk(n), p->Yhl, c.st);
      launch_tc_psi_density(p->phiT32, p->dphiT32, p->Yhl, tc_psi_width(nuse), tc_ldk(n), N, p->rho,
                            p->gga ? p->grho : nullptr, p->tc_err, c.st, psi_out, kPsiDrain);
      p->exx_psi_ready = p->exx_fused && psi_out == p->exx_psi;
      if (p->keep_psi) {
        p->npsi_kept = tc_psi_width(nuse);
        p->nuse_kept = nuse;
      }
    } else {
      if (p->keep_psi) p->npsi_kept = 0;
      launch_to_f32(p->D, n, n, n, 1.0, p->D32, tc_ldk(n), c.st);
      launch_tc_density(p->phi32, p->phiT32, p->dphi32, p->D32, n, N, p->ld, p->tcd_part, p->rho,
                        p->gga ? p->grho : nullptr, p->tc_err, c.st);
    }
    launch_poisson_f32(p->rho, p->vh, p->cbuf32, p->coul, p->ng, p->tw, c.st);
    launch_xc_pointwise(kind, p->rho, p->gga ? p->grho : nullptr, p->vh, N, p->dV, p->wq, p->vxc,
                        p->gga ? p->u : nullptr, p->xpart, c.st, true);
    launch_sum_partials(p->xpart, xc_blocks(N), 2, 2, 1.0, p->scal + S_EXC, false, c.st);
    launch_to_f32(p->wq, N, N, 1, 1.0, p->w32, p->ld, c.st);
    if (p->gga) launch_to_f32(p->u, N, N, 3, 1.0, p->u32, p->ld, c.st);
    // Hartree-Fock: the Hartree potential alone is the weight, same-signed,
    // where the truncating accumulation of 4-stage drains would bias J by
    // ~1e-6; its grids are small, so it drains every stage
    launch_tc_quadrature(p->phi32, p->dphi32, p->phihl, p->w32, p->u32, (float)p->dV, n, N, p->ld,
                         p->gga, 1.0, p->tcq_part, p->F2e, p->tc_err, c.st, p->hf ? 1 : 4, p->zhl);
  } else {
  launch_density(p->phi, p->gga ? p->dphi : nullptr, p->D, n, N, p->rho, p->gga ? p->grho : nullptr,
                 nullptr, c.st);
  poisson(c, p->rho, p->vh);
  launch_xc_pointwise(kind, p->rho, p->gga ? p->grho : nullptr, p->vh, N, p->dV, p->wq, p->vxc,
                      p->gga ? p->u : nullptr, p->xpart, c.st);
  launch_sum_partials(p->xpart, xc_blocks(N), 2, 2, 1.0, p->scal + S_EXC, false, c.st);
  if (p->gga) {
    launch_gga_operand(p->phi, p->dphi, p->wq, p->u, n, N, p->dV, p->Z, c.st);
    launch_quadrature(p->Z, p->phi, nullptr, n, N, false, 1.0, false, p->qpart, p->t1, c.st);
    axpby(n, 1.0, p->t1, 1.0, p->t1, true, p->F2e, c.st);
  } else {
    launch_quadrature(p->phi, p->phi, p->wq, n, N, true, 1.0, false, p->qpart, p->F2e, c.st);
  }
  }
  if (p->hf) {
    if (p->exx_fused) exchange(c);
    else exchange_legacy(c, nullptr);
    dot((long long)n * n, p->K, p->D, 1.0, p->scal + S_TRKD, false, c.st);
    axpby(n, 1.0, p->F2e, -0.5, p->K, false, p->F2e, c.st);
  }
  axpby(n, 1.0, p->H, 1.0, p->F2e, false, p->F, c.st);
  dot((long long)n * n, p->H, p->D, 1.0, p->scal + S_TRHD, false, c.st);
  sync_scalars(c);
  const double *s = p->hscal;
  double E = s[S_TRHD] + 0.5 * p->dV * s[S_VHRHO];
  E += P.dft ? p->dV * s[S_EXC] : -0.25 * s[S_TRKD];
  return E;
}

static double err_vector(Ctx &c, double *e) {
  hqcgb_plan *p = c.p;
  int n = p->nao;
  const int k = p->nuse_dm;
  if (k > 0) {
    // S D F = (S Y)(F^T Y)^T for D = Y Y^T
    gemm(false, false, n, k, n, 1.0, p->S, n, p->Yd, k, nullptr, 0.0, p->Y2, k, c.st);
    gemm(true, false, n, k, n, 1.0, p->F, n, p->Yd, k, nullptr, 0.0, p->t1, k, c.st);
    gemm(false, true, n, n, k, 1.0, p->Y2, k, p->t1, k, nullptr, 0.0, p->xerr, n, c.st);
    antisym(n, p->xerr, e, c.st);
  } else {
    gemm(false, false, n, n, n, 1.0, p->S, n, p->D, n, nullptr, 0.0, p->t1, n, c.st);
    gemm(false, false, n, n, n, 1.0, p->t1, n, p->F, n, nullptr, 0.0, p->t2, n, c.st);
    antisym(n, p->t2, e, c.st);
  }
  dot((long long)n * n, e, e, 1.0, p->scal + S_ERR2, false, c.st);
  sync_scalars(c);
  return std::sqrt(p->hscal[S_ERR2]);
}

static void check_eig(Ctx &c) {
  int st = 0;
  HQ_CUDA(cudaMemcpyAsync(&st, c.p->jstat, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  HQ_CUDA(cudaStreamSynchronize(c.st));
  if (st < 0) throw Error{HQCGB_EIG_FAIL, "Jacobi eigensolver did not converge"};
}

static void geometry(Ctx &c, const double *xp_dev) {
  hqcgb_plan *p = c.p;
  const hqcgb_params &P = p->P;
  int n = p->nao;
  long long N = p->N;
  HQ_CUDA(cudaMemcpyAsync(p->xp, xp_dev, sizeof(double) * 3 * p->n, cudaMemcpyDeviceToDevice, c.st));
  launch_gto1d(p->xp, p->n, p->ng, p->L, p->alpha, p->nprim, p->lat1d, P.n_lat1d, p->F1d, c.st);
  if (p->phi)
    launch_phi(p->F1d, p->coef, p->ao_l, p->ao_cart, p->nb, p->nprim, n, p->ng, p->phi, p->dphi,
               c.st);
  if (p->mixed) {
    launch_to_float((long long)p->n * 3 * p->ng * P.n_prim * 6, p->F1d, p->F1d32, c.st);
    launch_phi32(p->F1d32, p->coef, p->ao_l, p->ao_cart, p->nb, p->nprim, n, p->ng, p->ld, p->phi32,
                 p->dphi32, c.st);
    // phi split once per geometry into the TF32 pieces the quadrature reads
    launch_split_operand(p->phi32, nullptr, nullptr, nullptr, n, N, p->ld, p->ld, 1.f, 0.f, p->phihl, c.st);
    launch_transpose_phi(p->phi32, n, N, p->ld, p->phiT32, c.st);
    if (p->gga)
      for (int d = 0; d < 3; ++d)
        launch_transpose_phi(p->dphi32 + (size_t)d * n * p->ld, n, N, p->ld,
                             p->dphiT32 + (size_t)d * N * tc_ldk(n), c.st);
  }
  launch_overlap_kinetic(p->xp, p->n, p->nb, p->nprim, p->alpha, p->coef, p->ao_l, p->ao_cart,
                         p->lattice, P.n_lattice, p->S, p->T, nullptr, nullptr, nullptr, nullptr,
                         p->ovq, c.st);
  launch_vloc_G(p->xp, p->n, p->ng, p->L, p->ph, p->cbuf, c.st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, true, c.st);
  launch_complex_real(p->cbuf, N, 1.0, p->vloc, c.st);
  if (p->mixed) {
    launch_to_f32(p->vloc, N, N, 1, p->dV, p->w32, p->ld, c.st);
    // one-off per geometry: drained every stage for the most accurate V
    launch_tc_quadrature(p->phi32, nullptr, p->phihl, p->w32, nullptr, (float)p->dV, n, N, p->ld, false,
                         1.0, p->tcq_part, p->V, p->tc_err, c.st, 1, p->zhl);
  } else {
    launch_quadrature(p->phi, p->phi, p->vloc, n, N, true, p->dV, false, p->qpart, p->V, c.st);
  }
  axpby(n, 1.0, p->T, 1.0, p->V, false, p->H, c.st);
  if (p->hf) launch_quadrature(p->phi, p->phi, nullptr, n, N, true, p->dV, false, p->qpart, p->St, c.st);
  // S^{-1/2} as U w^{-1/2} (solver.py:729-730)
  HQ_CUDA(cudaMemsetAsync(p->ibad, 0, sizeof(int), c.st));
  eigh(c, p->S, p->c1, p->ws, true);
  inv_sqrt_cols(n, p->c1, p->ws, p->vorth, p->ibad, c.st);
  int bad = 0;
  HQ_CUDA(cudaMemcpyAsync(&bad, p->ibad, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  HQ_CUDA(cudaStreamSynchronize(c.st));
  check_eig(c);
  if (bad) throw Error{HQCGB_NAN, "overlap matrix is not positive definite (coincident atoms?)"};
}

static int scf_one(hqcgb_plan *p, const double *xp_dev, const hqcgb_scf_out *out, cudaStream_t st) {
  Ctx c{p, st};
  const hqcgb_params &P = p->P;
  int n = p->nao;
  size_t nn = (size_t)n * n;
  p->have_state = false;
  p->have_prev = false;
  p->allow_warm = false;
  geometry(c, xp_dev);
  // Hcore guess (solver.py:739-745)
  diagonalize(c, p->H);
  density_matrix(c);
  double E0 = 0.0, E1 = 1.0;
  int loop = 0;
  bool stopped = false;  // the stopping test was met before max_cycle
  if (P.diis) {
    int sp = P.diis_space;
    fock(c);
    err_vector(c, p->err);
    for (int k = 0; k < sp; ++k) {
      HQ_CUDA(cudaMemcpyAsync(p->Fk + k * nn, p->F, nn * 8, cudaMemcpyDeviceToDevice, st));
      HQ_CUDA(cudaMemcpyAsync(p->ek + k * nn, p->err, nn * 8, cudaMemcpyDeviceToDevice, st));
    }
    int head = sp - 1;
    double enorm = 0.0;
    auto step = [&](const double *Fin) {
      diagonalize(c, Fin);
      density_matrix(c);
      double En = fock(c);
      head = (head + 1) % sp;
      HQ_CUDA(cudaMemcpyAsync(p->Fk + head * nn, p->F, nn * 8, cudaMemcpyDeviceToDevice, st));
      enorm = err_vector(c, p->ek + head * nn);
      E0 = E1;
      E1 = En;
      ++loop;
      if (trace_on()) fprintf(stderr, "scf %3d E=%.12f dE=%.3e err=%.3e\n", loop, E1, E1 - E0, enorm);
    };
    // the Fock matrix still moves a lot in the plain warm-up iterations:
    // eigenvectors of the previous one are too far for the warm refinement
    p->allow_warm = false;
    while (loop < P.diis_start_cycle + sp) step(p->Fk + head * nn);
    p->allow_warm = true;
    E0 = E1 - 1.0;
    // The mixed path's Fock build carries noise (3xTF32, FP32 accumulation):
    // its stopping tests are floored at that noise (|dE| 1e-6 Ha, commutator
    // 2e-5) so that tol below the floor cannot make the loop spin to max_cycle.
    const double etol = p->mixed ? std::max(P.tol, 2e-6) : P.tol;
    const double errtol = p->mixed ? std::max(10.0 * P.tol, 2e-5) : 10.0 * P.tol;
    auto diis_step = [&] {
      diis_extrapolate(sp, n, p->Fk, p->ek, head, P.diis_damp, p->Bm, p->dc, p->t1, st);
      HQ_CUDA(cudaMemcpyAsync(p->Fp, p->t1, nn * 8, cudaMemcpyDeviceToDevice, st));
      step(p->Fp);
      if (!std::isfinite(E1)) throw Error{HQCGB_NAN, "non-finite energy in the SCF"};
    };
    while ((std::fabs(E1 - E0) > etol || enorm > errtol) && loop < P.max_cycle) diis_step();
    stopped = loop < P.max_cycle;
    // Mixed Hartree-Fock or smeared run, stopped at the floor with the
    // commutator still above the requested 10 tol: a few more iterations
    // while it keeps falling by at least a fifth (the gradient's error is
    // first order in it; at the noise floor it stops falling and the polish
    // ends).  Kohn-Sham runs without smearing skip it: the floored stop
    // already leaves their forces well inside the bound (H54 PBE: 2.4e-7
    // Ha/Bohr), and the polish would only add iterations.
    if (p->mixed && (P.smearing || !P.dft) && loop < P.max_cycle && enorm > 10.0 * P.tol) {
      for (int extra = 0; extra < 6 && loop < P.max_cycle && enorm > 10.0 * P.tol; ++extra) {
        const double prev = enorm;
        diis_step();
        if (enorm > 0.8 * prev) break;
      }
    }
  } else {
    const double etol = p->mixed ? std::max(P.tol, 2e-6) : P.tol;
    while (std::fabs(E1 - E0) > etol && loop < P.max_cycle) {
      p->allow_warm = loop >= 3;
      double En = fock(c);
      diagonalize(c, p->F);
      density_matrix(c);
      E0 = E1;
      E1 = En;
      ++loop;
      if (!std::isfinite(E1)) throw Error{HQCGB_NAN, "non-finite energy in the SCF"};
    }
    stopped = loop != P.max_cycle;
  }
  check_eig(c);
  if (p->mixed) {
    int te = 0;
    HQ_CUDA(cudaMemcpyAsync(&te, p->tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (te) {
      HQ_CUDA(cudaMemsetAsync(p->tc_err, 0, sizeof(int), st));
      throw Error{HQCGB_CUDA_ERROR, "tensor-core pipeline wait limit hit (code " + std::to_string(te) + ")"};
    }
  }
  int converged = stopped ? 1 : 0;
  if (p->mixed) refine_last(c);
  // post-processing (solver.py:758-767 / 890-899); the mixed force path keeps
  // the orbitals on the grid from this last density pass
  density_matrix(c);
  p->keep_psi = p->orb_forces;
  fock(c);
  p->keep_psi = false;
  dot((long long)nn, p->T, p->D, 1.0, p->scal + S_KI, false, st);
  dot((long long)nn, p->V, p->D, 1.0, p->scal + S_VEP, false, st);
  entropy(n, p->occ, p->scal + S_SE, st);
  if (P.smearing) free_entropy(n, P.smearing_method, P.smearing_sigma, p->w, p->mu, p->occ, p->scal + S_SFREE, st);
  sync_scalars(c);
  const double *s = p->hscal;
  double Exc = P.dft ? p->dV * s[S_EXC] : -0.25 * s[S_TRKD];
  double Vee = 0.5 * p->dV * s[S_VHRHO] + Exc;
  double en[5] = {E1, s[S_KI], s[S_VEP], Vee, s[S_SE]};
  const double Efree = P.smearing ? E1 - P.smearing_sigma * s[S_SFREE] : E1;
  if (out) {
    if (out->mo_coeff) HQ_CUDA(cudaMemcpyAsync(out->mo_coeff, p->C, nn * 8, cudaMemcpyDeviceToDevice, st));
    if (out->dm) HQ_CUDA(cudaMemcpyAsync(out->dm, p->D, nn * 8, cudaMemcpyDeviceToDevice, st));
    if (out->bands) HQ_CUDA(cudaMemcpyAsync(out->bands, p->w, n * 8, cudaMemcpyDeviceToDevice, st));
    if (out->energies) HQ_CUDA(cudaMemcpyAsync(out->energies, en, sizeof(en), cudaMemcpyHostToDevice, st));
    if (out->converged) HQ_CUDA(cudaMemcpyAsync(out->converged, &converged, sizeof(int), cudaMemcpyHostToDevice, st));
    if (out->iterations) HQ_CUDA(cudaMemcpyAsync(out->iterations, &loop, sizeof(int), cudaMemcpyHostToDevice, st));
    if (out->free_energy)
      HQ_CUDA(cudaMemcpyAsync(out->free_energy, &Efree, sizeof(double), cudaMemcpyHostToDevice, st));
    HQ_CUDA(cudaStreamSynchronize(st));
  }
  p->have_state = true;
  return converged ? HQCGB_OK : HQCGB_NOT_CONVERGED;
}

// Mixed Kohn-Sham forces: the S/T terms as in the FP64 path (done by the
// caller), the structure-factor term and the effective potential from the
// final SCF density, and the grid term from the orbitals kept by the last
// density pass (forces_mixed.cu).
static void orbital_forces(Ctx &c, double *grad) {
  hqcgb_plan *p = c.p;
  const hqcgb_params &P = p->P;
  cudaStream_t st = c.st;
  long long N = p->N;
  if (p->npsi_kept == 0)
    throw Error{HQCGB_BAD_ARG, "mixed forces need at most 32 (GGA) / 64 occupied orbitals"};
  launch_real_to_complex(p->rho, nullptr, N, 1, p->cbuf, st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, false, st);
  launch_vloc_force(p->ph, p->cbuf, p->n, p->ng, p->L, p->vpart, st);
  launch_sum_partials(p->vpart, vloc_force_blocks(N), 3 * p->n, 3 * p->n, 1.0, grad, true, st);
  launch_scale_complex(p->cbuf, p->coul, N, 1, st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, true, st);
  launch_complex_real(p->cbuf, N, 1.0, p->vh, st);
  launch_xc_pointwise(P.xc, p->rho, p->gga ? p->grho : nullptr, p->vh, N, p->dV, p->wq, p->vxc,
                      p->gga ? p->u : nullptr, p->xpart, st);
  launch_add3(N, p->vloc, p->vh, p->vxc, p->veff, st);
  launch_force_operand(p->C, p->occ, p->nao, p->nuse_kept, p->npsi_kept, p->Y32, st);
  launch_force_grid_orb(p->F1d32, p->coef, p->ao_l, p->ao_cart, p->n, p->nb, p->nprim, p->ng,
                        p->veff, p->gga ? p->u : nullptr, p->psi32, p->Y32, p->npsi_kept, p->dV,
                        p->fpart, grad, st);
  HQ_CUDA(cudaStreamSynchronize(st));
}

static void forces(hqcgb_plan *p, double *grad, cudaStream_t st) {
  Ctx c{p, st};
  const hqcgb_params &P = p->P;
  HQ_REQUIRE(P.want_forces, "plan was created without want_forces");
  if (!p->have_state) throw Error{HQCGB_NO_STATE, "hqcgb_forces called before a successful SCF"};
  int n = p->nao;
  long long N = p->N;
  HQ_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * 3 * p->n, st));
  // energy-weighted density W = C diag(f eps) C^T  -> t2
  launch_add3(n, nullptr, nullptr, nullptr, p->psi, st);  // psi[0..n) scratch = 0
  launch_axpy_grid(n, n, 1.0, p->occ, p->w, p->psi, st);   // psi = f * eps
  gemm(false, true, n, n, n, 1.0, p->C, n, p->C, n, p->psi, 0.0, p->t2, n, st);
  launch_overlap_kinetic(p->xp, p->n, p->nb, p->nprim, p->alpha, p->coef, p->ao_l, p->ao_cart,
                         p->lattice, P.n_lattice, nullptr, nullptr, p->D, p->t2, p->gpart, grad,
                         p->ovq, st);
  if (p->orb_forces) {
    orbital_forces(c, grad);
    return;
  }
  // density, X = D phi, Hartree, structure-factor term
  launch_density(p->phi, p->gga ? p->dphi : nullptr, p->D, n, N, p->rho, p->gga ? p->grho : nullptr,
                 p->X, st);
  launch_real_to_complex(p->rho, nullptr, N, 1, p->cbuf, st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, false, st);
  launch_vloc_force(p->ph, p->cbuf, p->n, p->ng, p->L, p->vpart, st);
  launch_sum_partials(p->vpart, vloc_force_blocks(N), 3 * p->n, 3 * p->n, 1.0, grad, true, st);
  launch_scale_complex(p->cbuf, p->coul, N, 1, st);
  launch_fft3d(p->cbuf, p->ng, 1, p->tw, true, st);
  launch_complex_real(p->cbuf, N, 1.0, p->vh, st);
  const double *uu = nullptr;
  if (P.dft) {
    launch_xc_pointwise(P.xc, p->rho, p->gga ? p->grho : nullptr, p->vh, N, p->dV, p->wq, p->vxc,
                        p->gga ? p->u : nullptr, p->xpart, st);
    launch_add3(N, p->vloc, p->vh, p->vxc, p->veff, st);
    if (p->gga) {
      launch_gga_psi(p->dphi, p->u, n, N, p->Z, st);
      launch_density(p->Z, nullptr, p->D, n, N, p->wq /*scratch*/, nullptr, p->DPsi, st);
      uu = p->u;
    }
  } else {
    launch_add3(N, p->vloc, p->vh, nullptr, p->veff, st);
    HQ_CUDA(cudaMemsetAsync(p->Z, 0, sizeof(double) * n * N, st));
    // the fallback exchange accumulates its orbital term into Z (it reuses X,
    // recomputed below); the fused form adds it to grad after X = D phi
    if (!p->exx_fused) exchange_legacy(c, p->Z);
    // Madelung term c dV (D S~ D phi)_p  folded into Z with weight cM
    gemm(false, false, n, n, n, 1.0, p->D, n, p->St, n, nullptr, 0.0, p->t1, n, st);
    gemm(false, false, n, n, n, 1.0, p->t1, n, p->D, n, nullptr, 0.0, p->t2, n, st);
    launch_density(p->phi, nullptr, p->t2, n, N, p->wq, nullptr, p->X, st);
    double cM = 4.0 * M_PI / p->L * kMadelungSC;
    launch_axpy_grid((long long)n * N, N, cM, nullptr, p->X, p->Z, st);
    launch_density(p->phi, nullptr, p->D, n, N, p->rho, nullptr, p->X, st);
    if (p->exx_fused) exchange_gradient(c, grad);
  }
  launch_force_grid(p->F1d, p->coef, p->ao_l, p->ao_cart, p->nb, p->nprim, n, p->ng, p->veff, p->X,
                    uu, p->DPsi, p->hf ? p->Z : nullptr, p->dV, p->fpart, st);
  launch_force_grid_reduce(p->fpart, n, p->nb, force_grid_blocks(N), grad, st);
  HQ_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------------------
// Batches: configuration b runs SCF (+ forces) on one of `concurrency` plans
// -- the plan itself on the caller's stream and clones with their own
// workspaces and streams -- each driven by its own host thread, so that the
// single-SM stages of one configuration (eigensolver, small FP64 linear
// algebra, host-side loop control) overlap the grid kernels of the others.
// The reference batches with jax.vmap over the same jitted SCF
// (test/test.py:157).
// ---------------------------------------------------------------------------
static hqcgb_params params_of(const hqcgb_plan *p) {
  hqcgb_params q = p->P;
  q.alpha = p->h_alpha.data();
  q.coef = p->h_coef.data();
  q.ao_l = p->h_l.data();
  q.ao_cart = p->h_cart.data();
  q.lat1d = p->h_lat1d.data();
  q.lattice = p->h_lattice.data();
  return q;
}

static void ensure_workers(hqcgb_plan *p, int k) {
  while ((int)p->workers.size() < k) {
    hqcgb_params q = params_of(p);
    cudaStream_t s;
    HQ_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    hqcgb_plan *w = new hqcgb_plan();
    try {
      create(&q, w);
    } catch (...) {  // nothing of a failed clone outlives this call
      delete w;
      cudaStreamDestroy(s);
      throw;
    }
    p->workers.push_back(w);
    p->wstreams.push_back(s);
  }
}

static hqcgb_scf_out slice(const hqcgb_scf_out &o, int b, int nao) {
  size_t nn = (size_t)nao * nao;
  hqcgb_scf_out r = o;
  if (r.mo_coeff) r.mo_coeff += b * nn;
  if (r.dm) r.dm += b * nn;
  if (r.bands) r.bands += (size_t)b * nao;
  if (r.energies) r.energies += 5 * b;
  if (r.converged) r.converged += b;
  if (r.iterations) r.iterations += b;
  if (r.free_energy) r.free_energy += b;
  return r;
}

static int run_batch(hqcgb_plan *p, int n_cfg, const double *xp, const hqcgb_scf_out *out,
                     double *grad, cudaStream_t st) {
  const int nthreads = std::min(p->concurrency, n_cfg);
  if (nthreads <= 1) {
    int worst = HQCGB_OK;
    for (int b = 0; b < n_cfg; ++b) {
      try {
        hqcgb_scf_out o = slice(*out, b, p->nao);
        int s = scf_one(p, xp + (size_t)b * 3 * p->n, &o, st);
        if (grad) forces(p, grad + (size_t)b * 3 * p->n, st);
        worst = std::max(worst, s);
      } catch (const Error &e) {  // name the configuration, as the concurrent path does
        throw Error{e.status, "configuration " + std::to_string(b) + ": " + e.msg};
      }
    }
    return worst;
  }
  ensure_workers(p, nthreads - 1);
  int dev = 0;
  HQ_CUDA(cudaGetDevice(&dev));
  HQ_CUDA(cudaStreamSynchronize(st));  // inputs may still be in flight on the caller's stream
  std::atomic<int> next{0};
  std::vector<int> status(n_cfg, HQCGB_OK);
  std::vector<std::string> msg(n_cfg);
  auto work = [&](int t) {
    hqcgb_plan *q = t == 0 ? p : p->workers[t - 1];
    cudaStream_t qs = t == 0 ? st : p->wstreams[t - 1];
    cudaSetDevice(dev);
    GpuShareScope share(nthreads);
    for (int b = next++; b < n_cfg; b = next++) {
      try {
        hqcgb_scf_out o = slice(*out, b, p->nao);
        status[b] = scf_one(q, xp + (size_t)b * 3 * p->n, &o, qs);
        if (grad) forces(q, grad + (size_t)b * 3 * p->n, qs);
        HQ_CUDA(cudaStreamSynchronize(qs));
      } catch (const Error &e) {
        status[b] = e.status;
        msg[b] = e.msg;
      } catch (const std::exception &e) {
        status[b] = HQCGB_CUDA_ERROR;
        msg[b] = e.what();
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto &th : pool) th.join();
  int worst = HQCGB_OK;
  for (int b = 0; b < n_cfg; ++b) {
    if (status[b] > HQCGB_NOT_CONVERGED) {
      throw Error{status[b], "configuration " + std::to_string(b) + ": " + msg[b]};
    }
    worst = std::max(worst, status[b]);
  }
  return worst;
}

// ---------------------------------------------------------------------------
// Uneven batches: configurations of different atom counts, boxes and grids
// in one call.  The reference batches with jax.vmap over configurations of
// one shape (test/test.py:157,179), so uneven sizes need one vmapped call per
// shape there.  Here configurations are grouped into size classes (n_atoms,
// n_grid); each worker thread owns one workspace per size class, whose
// box-dependent tables are reset per configuration (set_box), and takes the
// next configuration from a queue ordered largest first.
// ---------------------------------------------------------------------------

// Lattices of a cubic box of side L (Bohr), in the order the Python factory
// builds them: the 1D translations of the grid GTO sums, tmax = 24 // L
// (hqc/pbc/gto.py:47-49; make_pbc_gto is called without rcut,
// hqc/pbc/solver.py:211,217), and the S/T sphere |t| <= rcut of the
// meshgrid of -tmax..tmax, tmax = rcut // L (solver.py:162-176).
static void box_lattices(double L, double rcut, std::vector<double> &lat1d, std::vector<double> &lattice) {
  lat1d.clear();
  const double t1 = std::floor(24.0 / L);
  for (double t = -t1; t <= t1; t += 1.0) lat1d.push_back(t * L);
  lattice.clear();
  const double tm = std::floor(rcut / L);
  std::vector<double> nt;
  for (double t = -tm; t <= tm; t += 1.0) nt.push_back(t);
  for (double yi : nt)
    for (double xj : nt)
      for (double zk : nt) {
        const double x = xj * L, y = yi * L, z = zk * L;
        if (x * x + y * y + z * z <= rcut * rcut) {
          lattice.push_back(x);
          lattice.push_back(y);
          lattice.push_back(z);
        }
      }
}

// Reset the box-dependent tables of a plan to side L (Bohr): lattices,
// Coulomb table, exchange pair weights, cell volume.  Stream-ordered on st.
static void set_box(hqcgb_plan *p, double L, double rcut, cudaStream_t st) {
  HQ_REQUIRE(L > 0, "L must be positive");
  box_lattices(L, rcut, p->h_lat1d, p->h_lattice);
  const int n1 = (int)p->h_lat1d.size(), n3 = (int)p->h_lattice.size() / 3;
  if (n1 > p->lat1d_cap) {
    p->lat1d = p->alloc<double>(n1);
    p->lat1d_cap = n1;
  }
  if (n3 > p->lattice_cap) {
    p->lattice = p->alloc<double>(3 * (size_t)n3);
    p->lattice_cap = n3;
  }
  HQ_CUDA(cudaMemcpyAsync(p->lat1d, p->h_lat1d.data(), sizeof(double) * n1, cudaMemcpyHostToDevice, st));
  HQ_CUDA(cudaMemcpyAsync(p->lattice, p->h_lattice.data(), sizeof(double) * 3 * n3, cudaMemcpyHostToDevice, st));
  p->P.n_lat1d = n1;
  p->P.n_lattice = n3;
  p->P.L = L;
  p->L = L;
  p->Omega = L * L * L;
  p->dV = p->Omega / (double)p->N;
  launch_coulomb_table(p->ng, p->L, p->coul, st);
  if (p->exx_fused) {
    if (p->mixed) launch_exx_weights<float>(p->ng, p->L, p->dV, static_cast<float *>(p->exx_wsq), st);
    else launch_exx_weights<double>(p->ng, p->L, p->dV, static_cast<double *>(p->exx_wsq), st);
  }
  // host copies must outlive the copies from pageable memory
  HQ_CUDA(cudaStreamSynchronize(st));
}

struct hqcgb_batch {
  hqcgb_params base{};
  std::vector<double> h_alpha, h_coef;
  std::vector<int> h_l, h_cart;
  double rcut = 24.0;
  int workers = 1;
  // per worker: size class (n_atoms, n_grid) -> workspace; its stream
  std::vector<std::map<std::pair<int, int>, hqcgb_plan *>> plans;
  std::vector<cudaStream_t> streams;
  ~hqcgb_batch() {
    for (auto &m : plans)
      for (auto &kv : m) delete kv.second;
    for (cudaStream_t s : streams) cudaStreamDestroy(s);
  }
};

static hqcgb_plan *batch_plan(hqcgb_batch *b, int t, int n_atoms, int n_grid, double L) {
  auto key = std::make_pair(n_atoms, n_grid);
  auto it = b->plans[t].find(key);
  if (it != b->plans[t].end()) return it->second;
  std::vector<double> l1, lat;
  box_lattices(L, b->rcut, l1, lat);
  hqcgb_params q = b->base;
  q.n_atoms = n_atoms;
  q.n_grid = n_grid;
  q.L = L;
  q.alpha = b->h_alpha.data();
  q.coef = b->h_coef.data();
  q.ao_l = b->h_l.data();
  q.ao_cart = b->h_cart.data();
  q.n_lat1d = (int)l1.size();
  q.lat1d = l1.data();
  q.n_lattice = (int)lat.size() / 3;
  q.lattice = lat.data();
  hqcgb_plan *p = new hqcgb_plan();
  try {
    create(&q, p);
  } catch (...) {
    delete p;
    throw;
  }
  b->plans[t][key] = p;
  return p;
}

static int run_uneven(hqcgb_batch *b, int n_cfg, const int *n_atoms, const int *n_grid, const double *L,
                      const double *xp, const hqcgb_scf_out *out, double *grad, cudaStream_t st) {
  std::vector<long long> xoff(n_cfg + 1, 0), aoff(n_cfg + 1, 0), moff(n_cfg + 1, 0);
  for (int c = 0; c < n_cfg; ++c) {
    HQ_REQUIRE(n_atoms[c] >= 1 && n_grid[c] >= 3 && L[c] > 0, "bad configuration size");
    const long long nao = (long long)n_atoms[c] * b->base.nao_atom;
    xoff[c + 1] = xoff[c] + 3LL * n_atoms[c];
    aoff[c + 1] = aoff[c] + nao;
    moff[c + 1] = moff[c] + nao * nao;
  }
  // largest configurations first (their workers finish last otherwise)
  std::vector<int> order(n_cfg);
  for (int c = 0; c < n_cfg; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return (long long)n_atoms[a] * n_grid[a] * n_grid[a] * n_grid[a] >
           (long long)n_atoms[c] * n_grid[c] * n_grid[c] * n_grid[c];
  });
  const int nthreads = std::max(1, std::min(b->workers, n_cfg));
  while ((int)b->plans.size() < nthreads) b->plans.emplace_back();
  while ((int)b->streams.size() < nthreads) {
    cudaStream_t s;
    HQ_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    b->streams.push_back(s);
  }
  int dev = 0;
  HQ_CUDA(cudaGetDevice(&dev));
  HQ_CUDA(cudaStreamSynchronize(st));  // inputs may still be in flight on the caller's stream
  std::atomic<int> next{0};
  std::vector<int> status(n_cfg, HQCGB_OK);
  std::vector<std::string> msg(n_cfg);
  auto work = [&](int t) {
    cudaStream_t qs = b->streams[t];
    cudaSetDevice(dev);
    GpuShareScope share(nthreads);
    for (int k = next++; k < n_cfg; k = next++) {
      const int c = order[k];
      try {
        hqcgb_plan *q = batch_plan(b, t, n_atoms[c], n_grid[c], L[c]);
        if (q->L != L[c]) set_box(q, L[c], b->rcut, qs);
        hqcgb_scf_out o{};
        if (out->mo_coeff) o.mo_coeff = out->mo_coeff + moff[c];
        if (out->dm) o.dm = out->dm + moff[c];
        if (out->bands) o.bands = out->bands + aoff[c];
        if (out->energies) o.energies = out->energies + 5LL * c;
        if (out->converged) o.converged = out->converged + c;
        if (out->iterations) o.iterations = out->iterations + c;
        if (out->free_energy) o.free_energy = out->free_energy + c;
        status[c] = scf_one(q, xp + xoff[c], &o, qs);
        if (grad) forces(q, grad + xoff[c], qs);
        HQ_CUDA(cudaStreamSynchronize(qs));
      } catch (const Error &e) {
        status[c] = e.status;
        msg[c] = e.msg;
      } catch (const std::exception &e) {
        status[c] = HQCGB_CUDA_ERROR;
        msg[c] = e.what();
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto &th : pool) th.join();
  int worst = HQCGB_OK;
  for (int c = 0; c < n_cfg; ++c) {
    if (status[c] > HQCGB_NOT_CONVERGED)
      throw Error{status[c], "configuration " + std::to_string(c) + ": " + msg[c]};
    worst = std::max(worst, status[c]);
  }
  return worst;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define HQ_GUARD(...)                                     \
  try {                                                   \
    __VA_ARGS__;                                          \
  } catch (const Error &e) {                              \
    set_error(e.msg);                                     \
    return e.status;                                      \
  } catch (const std::exception &e) {                     \
    set_error(e.what());                                  \
    return HQCGB_CUDA_ERROR;                              \
  }

extern "C" {

int hqcgb_plan_create(const hqcgb_params *params, hqcgb_plan **plan) {
  HQ_GUARD({
    HQ_REQUIRE(params && plan, "null argument");
    hqcgb_plan *p = new hqcgb_plan();
    try {
      create(params, p);
    } catch (...) {
      delete p;
      throw;
    }
    *plan = p;
    return HQCGB_OK;
  });
}

int hqcgb_plan_destroy(hqcgb_plan *plan) {
  HQ_GUARD({
    delete plan;
    return HQCGB_OK;
  });
}

int hqcgb_scf(hqcgb_plan *plan, const double *xp, const hqcgb_scf_out *out, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(plan && xp, "null argument");
    return scf_one(plan, xp, out, (cudaStream_t)stream);
  });
}

int hqcgb_scf_batch(hqcgb_plan *plan, int n_cfg, const double *xp, const hqcgb_scf_out *out,
                    void *stream) {
  return hqcgb_pes_batch(plan, n_cfg, xp, out, nullptr, stream);
}

int hqcgb_plan_set_concurrency(hqcgb_plan *plan, int workers) {
  HQ_GUARD({
    HQ_REQUIRE(plan && workers >= 1 && workers <= 64, "workers must be in [1, 64]");
    plan->concurrency = workers;
    return HQCGB_OK;
  });
}

int hqcgb_pes_batch(hqcgb_plan *plan, int n_cfg, const double *xp, const hqcgb_scf_out *out,
                    double *grad, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(plan && xp && out && n_cfg >= 0, "null argument");
    HQ_REQUIRE(!grad || plan->P.want_forces, "plan was created without want_forces");
    return run_batch(plan, n_cfg, xp, out, grad, (cudaStream_t)stream);
  });
}

long long hqcgb_exchange_rebuild(hqcgb_plan *plan, void *stream) {
  try {
    if (!plan || !plan->hf || !plan->have_state || !plan->exx_fused) return -1;
    Ctx c{plan, (cudaStream_t)stream};
    exchange(c);
    HQ_CUDA(cudaStreamSynchronize(c.st));
    return (long long)plan->nao * exx_count(plan);
  } catch (const Error &e) {
    set_error(e.msg);
    return -2;
  }
}

int hqcgb_batch_create(const hqcgb_params *base, double rcut, int workers, hqcgb_batch **batch) {
  HQ_GUARD({
    HQ_REQUIRE(base && batch, "null argument");
    HQ_REQUIRE(workers >= 1 && workers <= 64, "workers must be in [1, 64]");
    HQ_REQUIRE(rcut > 0, "rcut must be positive");
    HQ_REQUIRE(base->nao_atom >= 1 && base->n_prim >= 1 && base->alpha && base->coef && base->ao_l &&
                   base->ao_cart, "empty basis");
    hqcgb_batch *b = new hqcgb_batch();
    b->base = *base;
    b->h_alpha.assign(base->alpha, base->alpha + base->n_prim);
    b->h_coef.assign(base->coef, base->coef + base->nao_atom * base->n_prim);
    b->h_l.assign(base->ao_l, base->ao_l + base->nao_atom);
    b->h_cart.assign(base->ao_cart, base->ao_cart + base->nao_atom);
    b->rcut = rcut;
    b->workers = workers;
    *batch = b;
    return HQCGB_OK;
  });
}

int hqcgb_batch_destroy(hqcgb_batch *batch) {
  HQ_GUARD({
    delete batch;
    return HQCGB_OK;
  });
}

int hqcgb_batch_run(hqcgb_batch *batch, int n_cfg, const int *n_atoms, const int *n_grid, const double *L,
                    const double *xp, const hqcgb_scf_out *out, double *grad, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(batch && n_atoms && n_grid && L && xp && out && n_cfg >= 0, "null argument");
    HQ_REQUIRE(!grad || batch->base.want_forces, "batch was created without want_forces");
    return run_uneven(batch, n_cfg, n_atoms, n_grid, L, xp, out, grad, (cudaStream_t)stream);
  });
}

int hqcgb_forces(hqcgb_plan *plan, double *grad, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(plan && grad, "null argument");
    forces(plan, grad, (cudaStream_t)stream);
    return HQCGB_OK;
  });
}

int hqcgb_ewald(const double *xp, int n, double L, double rs, double kappa, int gmax,
                double *energy, double *grad, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(xp && energy && n >= 1 && L > 0 && rs > 0 && kappa > 0 && gmax >= 1, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    HQ_REQUIRE(gmax <= 200, "Gmax too large");
    StreamBuf work(sizeof(double) * ewald_work_doubles(n, gmax), st);
    launch_ewald(xp, n, L, rs, kappa, gmax, work.as<double>(), energy, grad, st);
    return HQCGB_OK;
  });
}

long long hqcgb_plan_query(hqcgb_plan *p, const char *name, void *dst, size_t bytes, void *stream) {
  try {
    if (!p || !name) return -1;
    size_t nn = (size_t)p->nao * p->nao * 8;
    size_t ng = (size_t)p->N * 8;
    const void *src = nullptr;
    size_t sz = 0;
    std::string k(name);
    if (k == "S") { src = p->S; sz = nn; }
    else if (k == "T") { src = p->T; sz = nn; }
    else if (k == "V") { src = p->V; sz = nn; }
    else if (k == "H") { src = p->H; sz = nn; }
    else if (k == "fock") { src = p->F; sz = nn; }
    else if (k == "J") { src = p->F2e; sz = nn; }
    else if (k == "K") { src = p->K; sz = nn; }
    else if (k == "D") { src = p->D; sz = nn; }
    else if (k == "St") { src = p->St; sz = nn; }
    else if (k == "Fp") { src = p->Fp; sz = nn; }
    else if (k == "vorth") { src = p->vorth; sz = nn; }
    else if (k == "phi") { src = p->phi; sz = ng * p->nao; }
    else if (k == "rho") { src = p->rho; sz = ng; }
    else if (k == "vh") { src = p->vh; sz = ng; }
    else if (k == "vloc") { src = p->vloc; sz = ng; }
    else return -2;
    if (!dst) return (long long)sz;
    if (bytes < sz) return -3;
    HQ_CUDA(cudaMemcpyAsync(dst, src, sz, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    HQ_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return (long long)sz;
  } catch (const Error &e) {
    set_error(e.msg);
    return -4;
  }
}

int hqcgb_eigh(int n, int batch, const double *A, double *w, double *V, void *stream) {
  HQ_GUARD({
    HQ_REQUIRE(A && w && V && n >= 1 && n <= kMaxNao && batch >= 1, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    size_t nn = (size_t)n * n * batch;
    StreamBuf wbuf(nn * sizeof(double), st), abuf(nn * sizeof(double), st), sbuf(batch * sizeof(int), st);
    double *work = wbuf.as<double>(), *Ac = abuf.as<double>();
    int *stat = sbuf.as<int>();
    HQ_CUDA(cudaMemcpyAsync(Ac, A, nn * sizeof(double), cudaMemcpyDeviceToDevice, st));
    eigh_tql(n, batch, Ac, V, w, work, stat, st);
    std::vector<int> hs(batch);
    HQ_CUDA(cudaMemcpyAsync(hs.data(), stat, batch * sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    int status = HQCGB_OK;
    for (int b = 0; b < batch; ++b) {
      if (hs[b] < 0) {
        HQ_CUDA(cudaMemcpyAsync(Ac + (size_t)b * n * n, A + (size_t)b * n * n,
                                (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        jacobi_eigh(n, 1, Ac + (size_t)b * n * n, V + (size_t)b * n * n, w + (size_t)b * n,
                    work, stat, st);
        int js = 0;
        HQ_CUDA(cudaMemcpyAsync(&js, stat, sizeof(int), cudaMemcpyDeviceToHost, st));
        HQ_CUDA(cudaStreamSynchronize(st));
        if (js < 0) status = HQCGB_EIG_FAIL;
      }
    }
    if (status != HQCGB_OK) throw Error{status, "eigensolver did not converge"};
    return HQCGB_OK;
  });
}

const char *hqcgb_last_error(void) { return g_err.c_str(); }

int hqcgb_tune_set(const char *name, long long value) {
  HQ_GUARD({
    HQ_REQUIRE(name, "null argument");
    const std::string k(name);
    static const char *known[] = {"quad_kchunk", "quad_groups", "exx_group", "exx_gram_ctas", "psi_ring"};
    bool ok = false;
    for (const char *q : known) ok = ok || k == q;
    HQ_REQUIRE(ok, "unknown tuning knob: " + k);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (value <= 0) g_tune.erase(k);
    else g_tune[k] = value;
    return HQCGB_OK;
  });
}

long long hqcgb_tune_get(const char *name) { return name ? tune_get(name, 0) : 0; }

int hqcgb_profile(int enable) {
  HQ_GUARD({
    HQ_CUDA(cudaDeviceSynchronize());
    for (auto &r : g_recs) {
      g_event_pool.push_back(r.a);
      g_event_pool.push_back(r.b);
    }
    g_recs.clear();
    for (int k = 0; k < ST_COUNT; ++k) g_open[k] = 0;
    g_profile = enable != 0;
    return HQCGB_OK;
  });
}

int hqcgb_stage_stats(int stage, const char **name, long long *count, double *ms) {
  HQ_GUARD({
    HQ_REQUIRE(stage >= 0 && stage < ST_COUNT, "stage out of range");
    HQ_CUDA(cudaDeviceSynchronize());
    long long c = 0;
    double t = 0;
    for (auto &r : g_recs) {
      if (r.stage != stage) continue;
      float f = 0;
      HQ_CUDA(cudaEventElapsedTime(&f, r.a, r.b));
      t += f;
      ++c;
    }
    if (name) *name = kStageNames[stage];
    if (count) *count = c;
    if (ms) *ms = t;
    return HQCGB_OK;
  });
}

long long hqcgb_launch_count(int reset) {
  long long v = g_launches.load();
  if (reset) g_launches = 0;
  return v;
}

}  // extern "C"
