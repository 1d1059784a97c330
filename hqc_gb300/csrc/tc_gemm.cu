// tcgen05 (5th-generation tensor core) grid contractions of the mixed path.
//
//   quadrature  M_pq = sum_g A_p(g) B_q(g)        A = phi * w (or the GGA
//               operand), B = phi; K = grid split over CTAs, FP64 partial
//               tiles reduced in FP64 (hqc/pbc/solver.py:693: Vxc, J, Vep);
//   density     X = D phi (M = AO, N = grid, K = AO) with the fused epilogue
//               rho(g) = sum_p phi_p(g) X_p(g) (+ grad rho for GGA)
//               (hqc/pbc/solver.py:690).
//
// Precision.  Products: 3xTF32 -- each fp32 operand x is split into
// hi = rna_tf32(x) and lo = x - hi and the MMA accumulates hi*hi + hi*lo +
// lo*hi (kind::tf32, M = 128, N = 128, K = 8 per instruction).  Sums: the
// tensor core accumulates in FP32 in TMEM only over a short K sub-chunk
// (`drain` stages of K = 32); the epilogue threads then drain the sub-chunk
// into register-resident compensated sums (Knuth's TwoSum in FP32, about 46
// significant bits) while the MMA fills the other TMEM buffer.  Long sums
// across CTAs are reduced in FP64.
//
// Kernels and their CTA layouts (each lists its own below):
//   k_tc_density      288 threads: warps 0-3 copy fp32 tiles with cp.async and
//                     split them hi/lo in shared memory, warps 4-7 drain TMEM,
//                     warp 8 allocates TMEM and issues the MMAs;
//   k_tc_psi_density  persistent; one warp issues TMA bulk tensor loads into
//                     a 4-stage ring, four warps split the A box in place,
//                     four drain, one issues the MMAs;
//   k_tc_quad_tma /   TMA loads of operands split once by the pass that forms
//   k_tc_quad_persist them (k_split_operand), one MMA thread, four or eight
//                     drain warps; FP64 partial tiles per K chunk (tile-list
//                     form) or per K slice of a persistent CTA group.
// Shared memory holds every operand in the UMMA canonical K-major
// 128-byte-swizzled layout.  Every mbarrier wait has a time limit: on expiry
// the kernel records an error code in *err, stops issuing work, waits
// (bounded) for its MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace hqcgb {
namespace tc {

constexpr int kProducers = 128;          // warps 0-3: loads + TF32 split
constexpr int kDrainers = 128;           // warps 4-7: TMEM drains + epilogue
constexpr int kThreads = kProducers + kDrainers + 32;  // + MMA warp 8
constexpr int kStageK = 32;              // fp32 elements per row per stage (128 bytes)
constexpr int kM = 128, kN = 128;
constexpr size_t kTile = 16384;          // 128 rows x 128 bytes
constexpr int kMaxSplit = 2;             // pieces per operand (hi, lo)
constexpr size_t kStageBytes = 2 * kMaxSplit * kTile;  // A pieces, then B pieces
constexpr uint64_t kWaitNs = 4000000000ull;  // 4 s

__device__ inline uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ inline void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ inline void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ inline bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ inline uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: gives up after kWaitNs of wall time (no stage of these
// kernels takes more than milliseconds), records `code` and returns false.
__device__ inline bool mbar_wait(uint64_t *bar, unsigned parity, int *err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) break;
  }
  if (err) atomicCAS(err, 0, code);
  return false;
}

__device__ inline uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Split fp32 x into two TF32 pieces, each rounded to nearest: x ~ hi + lo.
__device__ __forceinline__ void split2(float x, float &hi, float &lo) {
  hi = __uint_as_float(tf32_rna(x));
  lo = __uint_as_float(tf32_rna(x - hi));
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ inline uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                 // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;       // SBO
  d |= (uint64_t)1 << 46;                 // version
  d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
  return d;
}

// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ inline void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ inline void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(smem_u32(bar)) : "memory");
}

__device__ inline void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ inline void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ inline void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ inline void tmem_alloc(uint32_t *dst_smem, int ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               ::"r"(smem_u32(dst_smem)), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ inline void tmem_dealloc(uint32_t taddr, int ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns
__device__ inline void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
      " [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline void tmem_st16(uint32_t taddr, const float *v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
      ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15]))
      : "memory");
}

__device__ inline void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ inline void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 16 columns without the wait (several loads in flight, then one wait)
__device__ inline void tmem_ld16_nowait(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
      " [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// byte offset of the 16-byte chunk `c` of row `r` in a K-major SW128 tile
__device__ inline uint32_t swz(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }

// Store the hi/lo pieces of 4 K-consecutive elements of row r (K chunk c);
// the hi piece goes to `tiles`, the lo piece to `tiles + kTile`.
__device__ __forceinline__ void store_split4(char *tiles, int r, int c, float4 v) {
  float4 h, l;
  split2(v.x, h.x, l.x);
  split2(v.y, h.y, l.y);
  split2(v.z, h.z, l.z);
  split2(v.w, h.w, l.w);
  uint32_t off = swz(r, c);
  *reinterpret_cast<float4 *>(tiles + off) = h;
  *reinterpret_cast<float4 *>(tiles + kTile + off) = l;
}

// MMAs of one stage (K = 32 -> 4 instructions of K = 8 per product pair):
// lo*hi + hi*lo + hi*hi (small products first).  A 3-piece split (6
// products) was measured to give no gain: the FP32 accumulation in TMEM, not
// the operand representation, limits the accuracy, and the short drains
// address that.
__device__ __forceinline__ void issue_stage(uint32_t tmem_d, uint32_t base, uint32_t idesc,
                                            bool first) {
  const uint32_t Ah = base, Al = base + kTile, Bh = base + kMaxSplit * kTile,
                 Bl = base + kMaxSplit * kTile + kTile;
#pragma unroll
  for (int ks = 0; ks < kStageK / 8; ++ks) {
    uint32_t off = ks * 32;  // 8 tf32 = 32 bytes along K
    mma_tf32(tmem_d, sdesc(Al + off), sdesc(Bh + off), idesc, (first && ks == 0) ? 0 : 1);
    mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bl + off), idesc, 1);
    mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bh + off), idesc, 1);
  }
}

// Compensated accumulation (TwoSum): (s, c) += v
__device__ inline void two_sum_add(float &s, float &c, float v) {
  float t = s + v;
  float z = t - s;
  c += (s - (t - z)) + (v - z);
  s = t;
}

// Compensated dot-product step in FP32 (Ogita-Rump-Oishi Dot2): (s, c) +=
// x y, the product split exactly by an FMA and added by TwoSum, so the sum
// (double)s + (double)c keeps about twice FP32's precision.  Used for the
// per-point sums of the orbital density: GB300 runs FP64 at 1/64 of the FP32
// rate, and FP64 accumulation there made the epilogue the kernel's limit.
__device__ __forceinline__ void dot2_add(float &s, float &c, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float e = fmaf(x, y, -p);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
  s = t;
}

// Shared skeleton: `fill(stage_index, smem_stage_base)` is executed by the
// 256 worker threads; after every `drain` stages the workers add the TMEM
// sub-chunk sum into (s[64], c[64]) -- their row (lane) and column half.
constexpr int kRing = 3;
struct Pipe {
  uint64_t full_bar[kRing], empty_bar[kRing], acc_full[2], acc_empty[2];
  uint32_t tmem_base;
};

// TMEM columns: [0,128) and [128,256) the two MMA accumulators, [256,384)
// the compensated sums S, [384,512) their carries C.
constexpr uint32_t kColS = 2 * kN, kColC = 3 * kN, kTmemCols = 4 * kN;

// Drain the accumulator of sub-chunk j into (S, C): S, C += A_j (TwoSum).
// Drainer warp w (4..7) owns TMEM lanes 32(w%4)..+31 and all 128 columns;
// per round of 32 columns six TMEM loads are in flight before one wait.
__device__ __forceinline__ bool drain_sub(Pipe &P, int j, int *err, int code) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  const int b = j & 1, use = j >> 1;
  bool got = mbar_wait(&P.acc_full[b], use & 1, err, code);
  tc_fence_after();
  if (got) {
#pragma unroll 1
    for (int col = 0; col < kN; col += 32) {
      uint32_t va[32], sa[32], ca[32];
      tmem_ld16_nowait(P.tmem_base + lane_off + b * kN + col, va);
      tmem_ld16_nowait(P.tmem_base + lane_off + b * kN + col + 16, va + 16);
      if (j > 0) {
        tmem_ld16_nowait(P.tmem_base + lane_off + kColS + col, sa);
        tmem_ld16_nowait(P.tmem_base + lane_off + kColS + col + 16, sa + 16);
        tmem_ld16_nowait(P.tmem_base + lane_off + kColC + col, ca);
        tmem_ld16_nowait(P.tmem_base + lane_off + kColC + col + 16, ca + 16);
      }
      tmem_wait_ld();
      float sv[32], cv[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        float v = __uint_as_float(va[i]);
        if (j == 0) {
          sv[i] = v;
          cv[i] = 0.f;
        } else {
          sv[i] = __uint_as_float(sa[i]);
          cv[i] = __uint_as_float(ca[i]);
          two_sum_add(sv[i], cv[i], v);
        }
      }
      tmem_st16(P.tmem_base + lane_off + kColS + col, sv);
      tmem_st16(P.tmem_base + lane_off + kColS + col + 16, sv + 16);
      tmem_st16(P.tmem_base + lane_off + kColC + col, cv);
      tmem_st16(P.tmem_base + lane_off + kColC + col + 16, cv + 16);
    }
    tmem_wait_st();
  }
  tc_fence_before();
  mbar_arrive(&P.acc_empty[b]);
  return got;
}

// Read back (S + C) of 16 columns (starting at col) of this drainer's row.
__device__ __forceinline__ void read_sum16(const Pipe &P, int col, double *out) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  uint32_t sv[16], cv[16];
  tmem_ld16_nowait(P.tmem_base + lane_off + kColS + col, sv);
  tmem_ld16_nowait(P.tmem_base + lane_off + kColC + col, cv);
  tmem_wait_ld();
#pragma unroll
  for (int i = 0; i < 16; ++i) out[i] = (double)__uint_as_float(sv[i]) + (double)__uint_as_float(cv[i]);
}

__device__ inline void cp_async16(uint32_t saddr, const void *g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ inline void cp_async_zero16(uint32_t saddr, const void *g) {
  // src-size 0: fills the 16 bytes with zeros without reading global memory
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, 0;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Generic K-major operand description: element (row, k) at
// ptr[row * ld + (k / 32) * kstride + k % 32] -- row-major with ld = row
// stride and kstride = 32, or K-blocked ([k / 32][row][32]) with ld = 32 and
// kstride = rows x 32; rows >= rows_valid and k >= k_end read as zero.  Every
// row start and every 4-element chunk is 16-byte aligned.
struct Operand {
  const float *ptr;
  long long ld;
  int rows_valid;
  long long kstride;
};

constexpr int kStages = 3;  // smem ring depth; copies run 2 stages ahead

// Producer/MMA/drain pipeline over `nstages` K-stages of 32 starting at k_begin.
// Producer thread t copies (cp.async) and later splits, in place, the 16-byte
// chunks t + 128 j (j = 0..7) of the A and B tiles -- all in K chunk t % 8 --
// and the matching 4 weights w[k..k+3] (into its own smem slot).
__device__ __forceinline__ bool run_pipe(Pipe &P, char *sm, float4 *wslot, const Operand &A,
                                         int a_row0, const Operand &B, int b_row0, const float *w,
                                         long long k_begin, long long k_end, int nstages, int drain,
                                         int ns, int *err, int code0) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nsub = (nstages + drain - 1) / drain;
  bool ok = true;
  if (warp < 4) {
    const int cch = tid & 7;
    // the 8 A rows and 8 B rows this thread copies never change
    const float *arow[8], *brow[8];
    uint32_t avalid = 0, bvalid = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int r = (tid >> 3) + 16 * j;
      int ra = a_row0 + r, rb = b_row0 + r;
      arow[j] = A.ptr + (long long)(ra < A.rows_valid ? ra : 0) * A.ld + cch * 4;
      brow[j] = B.ptr + (long long)(rb < B.rows_valid ? rb : 0) * B.ld + cch * 4;
      avalid |= (ra < A.rows_valid ? 1u : 0u) << j;
      bvalid |= (rb < B.rows_valid ? 1u : 0u) << j;
    }
    const uint32_t sbase = smem_u32(sm);
    auto issue = [&](int st) {  // async copies of stage st into buffer st % kStages
      const int buf = st % kStages;
      const uint32_t base = sbase + buf * (uint32_t)kStageBytes;
      long long kk = k_begin + (long long)st * kStageK;  // chunk start (without cch*4)
      long long k = kk + cch * 4;
      bool kin = k < k_end;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        int r = (tid >> 3) + 16 * j;
        uint32_t off = swz(r, cch);
        const float *ga = arow[j] + (kin ? (kk / kStageK) * A.kstride : 0);
        const float *gb = brow[j] + (kin ? (kk / kStageK) * B.kstride : 0);
        if (kin && ((avalid >> j) & 1u)) cp_async16(base + off, ga);
        else cp_async_zero16(base + off, arow[j]);
        if (kin && ((bvalid >> j) & 1u)) cp_async16(base + kMaxSplit * kTile + off, gb);
        else cp_async_zero16(base + kMaxSplit * kTile + off, brow[j]);
      }
      if (w) {
        uint32_t ws = smem_u32(&wslot[buf * kProducers + tid]);
        if (kin) cp_async16(ws, w + k);
        else cp_async_zero16(ws, w);
      }
      cp_async_commit();
    };
    auto split_stage = [&](int st) {  // in place: raw fp32 in piece 0 -> pieces
      const int buf = st % kStages;
      char *base = sm + buf * kStageBytes;
      float4 wv = w ? wslot[buf * kProducers + tid] : make_float4(1.f, 1.f, 1.f, 1.f);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        int r = (tid >> 3) + 16 * j;
        uint32_t off = swz(r, cch);
        float4 av = *reinterpret_cast<float4 *>(base + off);
        av.x *= wv.x; av.y *= wv.y; av.z *= wv.z; av.w *= wv.w;
        float4 bv = *reinterpret_cast<float4 *>(base + kMaxSplit * kTile + off);
        store_split4(base, r, cch, av);
        store_split4(base + kMaxSplit * kTile, r, cch, bv);
      }
    };
    for (int st = 0; st < 2 && st < nstages; ++st) issue(st);
    for (int stage = 0; stage < nstages; ++stage) {
      // stage `stage` landed once at most one newer group is pending
      if (stage + 1 < nstages) cp_async_wait<1>();
      else cp_async_wait<0>();
      if (ok) split_stage(stage);
      fence_proxy_async();
      mbar_arrive(&P.full_bar[stage % kStages]);
      int nx = stage + 2;  // refill the buffer of stage - 1 once the MMA released it
      if (nx < nstages) {
        int use = nx / kStages;
        if (ok && use > 0 && !mbar_wait(&P.empty_bar[nx % kStages], (use - 1) & 1, err, code0 + 1))
          ok = false;
        issue(nx);
      }
    }
  } else if (warp < 8) {
    for (int j = 0; j < nsub; ++j) ok = drain_sub(P, j, err, code0 + 3) && ok;
  } else if (lane == 0) {
    const uint32_t idesc = idesc_tf32(kM, kN);
    int stage = 0;
    for (int j = 0; j < nsub; ++j) {
      int ab = j & 1, ause = j >> 1;
      if (ok && ause > 0 && !mbar_wait(&P.acc_empty[ab], (ause - 1) & 1, err, code0 + 4)) ok = false;
      tc_fence_after();
      uint32_t tmem_d = P.tmem_base + (uint32_t)(ab * kN);
      int s_end = min(nstages, (j + 1) * drain);
      bool first = true;
      for (; stage < s_end; ++stage) {
        int b = stage % kStages, use = stage / kStages;
        if (ok && !mbar_wait(&P.full_bar[b], use & 1, err, code0 + 2)) ok = false;
        tc_fence_after();
        if (ok) issue_stage(tmem_d, smem_u32(sm + b * kStageBytes), idesc, first);
        first = false;
        mma_commit(&P.empty_bar[b]);
      }
      mma_commit(&P.acc_full[ab]);
    }
  }
  return ok;
}

__device__ inline void pipe_init(Pipe &P) {
  if (threadIdx.x == 0) {
    for (int b = 0; b < kStages; ++b) {
      mbar_init(&P.full_bar[b], kProducers);
      mbar_init(&P.empty_bar[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&P.acc_full[b], 1);
      mbar_init(&P.acc_empty[b], kDrainers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 8) tmem_alloc(&P.tmem_base, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

__device__ inline void pipe_finish(Pipe &P) {
  tc_fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 8) {
    tc_fence_after();
    tmem_dealloc(P.tmem_base, kTmemCols);
  }
}

// FP64 partial tiles of the quadrature: P[chunk][tile_m][tile_n][128][128].
constexpr size_t kWslotBytes = kStages * kProducers * sizeof(float4);

// The corner kernel's partial tiles summed in a fixed order: CTA (p, q) adds
// P[k][last][last][p][q] over k < nparts (256 threads, a shared-memory tree)
// into P[0][last][last][p][q].
__global__ void __launch_bounds__(256) k_quad_corner_sum(double *__restrict__ P, int nparts, int mtiles,
                                                         int ntiles, int last) {
  __shared__ double red[256];
  const int p = blockIdx.x >> 4, q = blockIdx.x & 15, t = threadIdx.x;
  const long long tsz = (long long)kM * kN, stride = (long long)mtiles * ntiles * tsz;
  double *e = P + ((long long)last * ntiles + last) * tsz + (long long)p * kN + q;
  double v = 0;
  for (int k = t; k < nparts; k += 256) v += e[k * stride];
  red[t] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (t < h) red[t] += red[t + h];
    __syncthreads();
  }
  if (t == 0) e[0] = red[0];
}

// P[0][tile] = sum_k P[k][tile] in place, one thread per element of the
// computed tiles (upper triangle when sym): coalesced reads of every partial
// tile, four loads in flight per thread.  The tile (corner, corner), when
// corner >= 0, sums ncorner partial tiles.
__global__ void k_tc_quad_sum_parts(double *__restrict__ P, int nchunk, int mtiles, int ntiles, int sym,
                                    int corner, int ncorner) {
  const long long tsz = (long long)kM * kN;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)mtiles * ntiles * tsz) return;
  const int tile = (int)(idx / tsz), tm = tile / ntiles, tn = tile % ntiles;
  if (sym && tn < tm) return;
  const int nk = (tm == corner && tn == corner) ? ncorner : nchunk;
  const long long stride = (long long)mtiles * ntiles * tsz;
  double *src = P + idx;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  int k = 0;
  for (; k + 4 <= nk; k += 4) {
    s0 += src[(k + 0) * stride];
    s1 += src[(k + 1) * stride];
    s2 += src[(k + 2) * stride];
    s3 += src[(k + 3) * stride];
  }
  for (; k < nk; ++k) s0 += src[k * stride];
  src[0] = (s0 + s1) + (s2 + s3);
}

// M[p][q] = scale * sum_chunks P  (+ mirror for sym; + transpose-add for GGA);
// the tile (corner, corner), when corner >= 0, sums ncorner partial tiles
__global__ void k_tc_quad_reduce(const double *__restrict__ P, int nchunk, int mtiles, int ntiles,
                                 int nao, int sym, int add_transpose, double scale,
                                 double *__restrict__ M, int corner, int ncorner) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nao * nao) return;
  int p = idx / nao, q = idx % nao;
  auto get = [&](int pp, int qq) {
    if (sym && (qq / kN) < (pp / kM)) { int t = pp; pp = qq; qq = t; }
    int tm = pp / kM, tn = qq / kN, r = pp % kM, cc = qq % kN;
    const int nk = (tm == corner && tn == corner) ? ncorner : nchunk;
    const long long stride = (long long)mtiles * ntiles * kM * kN;
    const double *src = P + (((long long)tm * ntiles + tn) * kM + r) * kN + cc;
    // four independent partial sums keep four loads in flight
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int k = 0;
    for (; k + 4 <= nk; k += 4) {
      s0 += src[(k + 0) * stride];
      s1 += src[(k + 1) * stride];
      s2 += src[(k + 2) * stride];
      s3 += src[(k + 3) * stride];
    }
    for (; k < nk; ++k) s0 += src[k * stride];
    return (s0 + s1) + (s2 + s3);
  };
  // sym: the (p, q) and (q, p) elements of a diagonal tile round differently
  // (the weight multiplies one operand before its TF32 split), so both are
  // averaged -- the result is exactly symmetric, as every Fock piece must be
  // before the orthogonalisation amplifies any asymmetry by 1/s_min(S).
  double v = (sym && !add_transpose) ? 0.5 * (get(p, q) + get(q, p)) : get(p, q);
  if (add_transpose) v += get(q, p);
  M[idx] = scale * v;
}

// ---------------------------------------------------------------------------
// Density: X = D phi on tiles (128 AOs) x (128 grid points), K = AO, from the
// K-major operands D[p][q] (row stride ldk) and phiT (the grid-major copy,
// K-blocked: phiT[q / 32][g][q % 32]).  Epilogue: part[mt][g] = sum_{p in tile} phi_p(g) X_p(g)
// and, for GGA, part_g[c][mt][g] = 2 sum_p dphi_c,p(g) X_p(g) (FP64).
// ---------------------------------------------------------------------------
struct DensArgs {
  Operand D, phiT;
  const float *phi, *dphi;  // AO-major (row stride ld) for the epilogue
  int nao, kpad, drain, ns;
  long long N, ld;
  double *part, *part_g;
  int *err;
};

constexpr int kProdLd = kN + 1;
constexpr size_t kProdBytes = 2 * (size_t)kM * kProdLd * sizeof(float);
constexpr size_t kDensSmem =
    (kProdBytes > kStages * kStageBytes ? kProdBytes : kStages * kStageBytes) + kWslotBytes + 1024;

__global__ void __launch_bounds__(kThreads, 1) k_tc_density(DensArgs a) {
  extern __shared__ __align__(1024) char smraw[];
  char *sm = (char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ Pipe P;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int mt = blockIdx.x;
  const long long g0 = (long long)blockIdx.y * kN;
  const int mtiles = gridDim.x;
  pipe_init(P);
  const int nstages = a.kpad / kStageK;
  const int p0 = mt * kM;
  float4 *wslot = reinterpret_cast<float4 *>(
      sm + (kProdBytes > kStages * kStageBytes ? kProdBytes : kStages * kStageBytes));
  bool ok = run_pipe(P, sm, wslot, a.D, p0, a.phiT, (int)g0, nullptr, 0, a.nao, nstages, a.drain,
                     a.ns, a.err, 10);

  // epilogue: products with phi (and grad phi), column sums over the 128 AO rows
  __syncthreads();  // all MMAs consumed and drained: the stage smem is free
  float *prod = reinterpret_cast<float *>(sm);   // [128][129] sums
  float *prodc = prod + kM * kProdLd;             // [128][129] compensations
  int ncomp = a.part_g ? 4 : 1;
  for (int comp = 0; comp < ncomp; ++comp) {
    if (warp >= 4 && warp < 8) {
      int row = (warp & 3) * 32 + (tid & 31), p = p0 + row;
      const float *src = (comp == 0) ? a.phi + (long long)p * a.ld
                                     : a.dphi + ((long long)(comp - 1) * a.nao + p) * a.ld;
#pragma unroll 1
      for (int c0 = 0; c0 < kN; c0 += 16) {
        double x[16];
        read_sum16(P, c0, x);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          int col = c0 + i;
          long long g = g0 + col;
          float f = (ok && p < a.nao && g < a.N) ? src[g] : 0.f;
          // X * f as an unevaluated pair (hi, lo) of floats
          float xs = (float)x[i];
          float xc = (float)(x[i] - (double)xs);
          float hi = xs * f;
          float lo = fmaf(xs, f, -hi) + xc * f;
          prod[row * kProdLd + col] = hi;
          prodc[row * kProdLd + col] = lo;
        }
      }
    }
    __syncthreads();
    if (tid < kN) {
      long long g = g0 + tid;
      float ss = 0.f, cc = 0.f;
      for (int r = 0; r < kM; ++r) {
        two_sum_add(ss, cc, prod[r * kProdLd + tid]);
        cc += prodc[r * kProdLd + tid];
      }
      if (ok && g < a.N) {
        double v = (double)ss + (double)cc;
        if (comp == 0) a.part[(long long)mt * a.ld + g] = v;
        else a.part_g[((long long)(comp - 1) * mtiles + mt) * a.ld + g] = 2.0 * v;
      }
    }
    __syncthreads();
  }
  pipe_finish(P);
}

// rho[g] = sum_mt part[mt][g], grho similarly
__global__ void k_tc_density_reduce(const double *__restrict__ part, const double *__restrict__ part_g,
                                    int mtiles, long long N, long long ld, double *__restrict__ rho,
                                    double *__restrict__ grho) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  double s = 0;
  for (int m = 0; m < mtiles; ++m) s += part[(long long)m * ld + g];
  rho[g] = s;
  if (grho) {
    for (int c = 0; c < 3; ++c) {
      double t = 0;
      for (int m = 0; m < mtiles; ++m) t += part_g[((long long)c * mtiles + m) * ld + g];
      grho[(long long)c * N + g] = t;
    }
  }
}

// Grid-major copy of phi in K-blocks of 32 AOs: phiT[q / 32][g][q % 32] =
// phi[q][g] for g < N, q < nao; zero for q in [nao, ldk).  A 128-point x
// 32-AO box of it is one contiguous 16 KB run of memory, so the tensor-core
// kernels' TMA loads stream whole DRAM pages instead of 128 rows of 128 bytes
// spread over the row stride.
__global__ void k_transpose_phi(const float *__restrict__ phi, int nao, long long N, long long ld,
                                float *__restrict__ phiT) {
  __shared__ float t[32][33];
  long long g0 = (long long)blockIdx.x * 32;
  int q0 = blockIdx.y * 32;
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 rows per pass
  for (int r = ty; r < 32; r += 8) {
    int q = q0 + r;
    long long g = g0 + tx;
    t[r][tx] = (q < nao && g < N) ? phi[(long long)q * ld + g] : 0.f;
  }
  __syncthreads();
  // K-blocked: AO block blockIdx.y, grid point g, AO q0 + tx (128 contiguous bytes per g)
  for (int r = ty; r < 32; r += 8) {
    long long g = g0 + r;
    if (g < N) phiT[((long long)blockIdx.y * N + g) * 32 + tx] = t[tx][r];
  }
}

// ---------------------------------------------------------------------------
// Orbital density: psi_k(g) = sum_p phi_p(g) Y_pk with Y = C_occ sqrt(f)
// (npsi <= kPsiMaxN columns, zero-padded), rho(g) = sum_k psi_k(g)^2 and,
// for GGA, grad rho = 2 sum_k psi_k grad psi_k.  This is the density
// sum_pq D_pq phi_p phi_q of D = C diag(f) C^T (hqc/pbc/solver.py:566-577,
// 690) at npsi / n_ao of the GEMM work.
//
// Tiles: M = 128 grid points (A = rows of the grid-major, K-blocked phiT /
// dphiT: [component][AO block][g][32]), N = npsi (B = the TF32 hi/lo pieces
// of Y^T, pre-split in global memory), K = AO in stages of 32.  Persistent CTAs loop over grid tiles;
// stage s of a CTA is (tile, component, K block).
//
// Accuracy.  The tensor core's FP32 accumulation truncates, so sums of many
// MMAs drift low (about half an ulp per instruction).  Every group of DR
// K blocks therefore accumulates in its own TMEM slot -- the large hi*hi
// products and the 2^-11 smaller cross products in separate accumulators --
// and the epilogue warps drain each group into compensated (TwoSum) FP32
// sums held in registers for the current component; psi = S + C is rounded
// to FP32 once (unbiased) and rho, grad rho are summed as compensated FP32
// dot products (dot2_add), rounded to FP64 at the end.
// Loads: bulk tensor copies (TMA) issued by one thread into a 4-stage ring.
// TMEM: a ring of up to 8 accumulator slots of 2 npsi columns.
// ---------------------------------------------------------------------------
constexpr int kPsiMaxN = 64;
constexpr int kPsiPW = 4;                       // splitter warps (in-place TF32 split)
constexpr int kPsiProducers = kPsiPW * 32;
constexpr int kPsiRowsPerThread = kM * 8 / kPsiProducers;  // A rows per splitter thread
constexpr int kPsiMmaWarp = kPsiPW + 4;         // after the 4 drain warps
constexpr int kPsiTmaWarp = kPsiMmaWarp + 1;    // one thread issues the bulk tensor loads
constexpr int kPsiThreads = kPsiProducers + kDrainers + 64;
constexpr int kPsiRing = 4;
constexpr size_t kPsiAPieces = 2 * kTile;                       // A hi, A lo
constexpr size_t kPsiBPiece = (size_t)kPsiMaxN * 128;           // one B piece
constexpr size_t kPsiStageBytes = kPsiAPieces + 2 * kPsiBPiece;  // 48 KB
constexpr size_t kPsiSmem = kPsiRing * kPsiStageBytes + 1024;

struct PsiArgs {
  const float *phiT;   // [N][ldk]
  const float *dphiT;  // [3][N][ldk] (GGA) or null
  const float *Yhl;    // [2][npsi][ldk]: TF32 hi and lo pieces of Y^T
  long long N;
  int ldk, npsi, ncomp;
  double *rho, *grho;  // [N], [3][N]
  float *psi_out;      // [ncomp][npsi][N] psi_k and grad psi_k (fp32), or null
  int drain;           // K blocks per drained accumulation (1 = every 32 AOs)
  int *err;
};

// TMEM accumulator-slot ring depth for npsi (2 npsi columns per slot).
__host__ __device__ inline int psi_ring(int npsi, int ncomp) {
  (void)ncomp;
  int ra = 512 / (2 * npsi);
  return ra > 8 ? 8 : ra;
}

struct PsiPipe {
  uint64_t loaded[kPsiRing], full[kPsiRing], empty[kPsiRing], acc_full[8], acc_empty[8];
  uint32_t tmem_base;
};

// TMA: bulk tensor copy of one box of a 2D tensor map into shared memory,
// completion counted in bytes on an mbarrier.
__device__ inline void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// TMA: one box of a 3D tensor map (the K-blocked operand layouts: x = the 32
// elements of a K block, y = row, z = K block).
__device__ inline void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                   uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ inline void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

template <int NPSI>
__global__ void __launch_bounds__(kPsiThreads, 1)
    k_tc_psi_density(PsiArgs a, const __grid_constant__ CUtensorMap tmA,
                     const __grid_constant__ CUtensorMap tmD, const __grid_constant__ CUtensorMap tmY) {
  extern __shared__ __align__(1024) char smraw[];
  char *sm = (char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ PsiPipe P;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkb = a.ldk / kStageK;
  const long long ntiles = (a.N + kM - 1) / kM;
  const long long my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int per_tile = a.ncomp * nkb;
  const long long S = my_tiles * per_tile;
  const int RA = psi_ring(NPSI, a.ncomp);
  const int DR = a.drain;  // K blocks of 32 accumulated per TMEM slot before a drain
  const int ncols = RA * 2 * NPSI;
  int tcols = 32;
  while (tcols < ncols) tcols <<= 1;

  if (tid == 0) {
    for (int b = 0; b < kPsiRing; ++b) {
      mbar_init(&P.loaded[b], 1);
      mbar_init(&P.full[b], kPsiProducers);
      mbar_init(&P.empty[b], 1);
    }
    for (int b = 0; b < 8; ++b) {
      mbar_init(&P.acc_full[b], 1);
      mbar_init(&P.acc_empty[b], kDrainers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kPsiMmaWarp) tmem_alloc(&P.tmem_base, tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  bool ok = true;
  if (warp == kPsiTmaWarp) {
    // loads: stage s of this CTA is (tile, component, K block); the A box
    // (128 grid points x 32 AOs, raw fp32) lands in the stage's high-piece
    // slot in the 128-byte-swizzled K-major layout, the two pieces of Y^T in
    // the B slots.  Rows past the grid read as zero (OOB fill).
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)kTile + 2u * NPSI * 128u;
      for (long long st = 0; st < S; ++st) {
        const int slot = (int)(st % kPsiRing);
        const long long use = st / kPsiRing;
        if (ok && use > 0 && !mbar_wait(&P.empty[slot], (unsigned)((use - 1) & 1), a.err, 25))
          ok = false;
        if (!ok) break;
        const long long t = st / per_tile;
        const int r = (int)(st % per_tile), comp = r / nkb, kb = r % nkb;
        const int g0 = (int)((blockIdx.x + t * gridDim.x) * (long long)kM);
        const uint32_t base = smem_u32(sm + slot * kPsiStageBytes);
        mbar_expect_tx(&P.loaded[slot], bytes);
        if (comp == 0) tma_load_3d(base, &tmA, 0, g0, kb, &P.loaded[slot]);
        else tma_load_3d(base, &tmD, 0, g0, (comp - 1) * nkb + kb, &P.loaded[slot]);
        tma_load_2d(base + (uint32_t)kPsiAPieces, &tmY, kb * kStageK, 0, &P.loaded[slot]);
        tma_load_2d(base + (uint32_t)kPsiAPieces + (uint32_t)NPSI * 128u, &tmY, kb * kStageK, NPSI,
                    &P.loaded[slot]);
      }
    }
  } else if (warp < kPsiPW) {
    // splitters: raw fp32 -> TF32 hi (in place) and lo pieces of the A box
    const int cch = tid & 7;
    for (long long st = 0; st < S; ++st) {
      const int slot = (int)(st % kPsiRing);
      if (ok && !mbar_wait(&P.loaded[slot], (unsigned)((st / kPsiRing) & 1), a.err, 21)) ok = false;
      if (ok) {
        char *base = sm + slot * kPsiStageBytes;
#pragma unroll
        for (int j = 0; j < kPsiRowsPerThread; ++j) {
          int row = (tid >> 3) + (kPsiProducers / 8) * j;
          uint32_t off = swz(row, cch);
          float4 v = *reinterpret_cast<float4 *>(base + off);
          store_split4(base, row, cch, v);
        }
      }
      fence_proxy_async();
      mbar_arrive(&P.full[slot]);
    }
  } else if (warp < kPsiPW + 4) {
    // drains and epilogue: thread = grid point (TMEM lane).  Group G of this
    // CTA is (tile, component, K blocks [g0, g0 + DR)) and lives in slot
    // G % RA.  The compensated sums of the current component stay in
    // registers; psi (the value component) is kept for the gradient products.
    const int row = (warp & 3) * 32 + lane;
    const uint32_t tbase = P.tmem_base + ((uint32_t)((warp & 3) * 32) << 16);
    long long G = 0;
    for (long long t = 0; t < my_tiles; ++t) {
      const long long g = (blockIdx.x + t * gridDim.x) * (long long)kM + row;
      float p0[NPSI];
      float rs = 0.f, rc = 0.f, gs[3] = {0.f, 0.f, 0.f}, gc[3] = {0.f, 0.f, 0.f};
      for (int comp = 0; comp < a.ncomp; ++comp) {
        float sv[NPSI], cv[NPSI];
        for (int g0 = 0; g0 < nkb; g0 += DR, ++G) {
          const int b = (int)(G % RA);
          const long long use = G / RA;
          bool got = ok && mbar_wait(&P.acc_full[b], (unsigned)(use & 1), a.err, 23);
          if (!got) ok = false;
          tc_fence_after();
          if (got) {
            const uint32_t slot = tbase + (uint32_t)(b * 2 * NPSI);
#pragma unroll
            for (int c0 = 0; c0 < NPSI; c0 += 16) {
              uint32_t vb[16], vs[16];
              tmem_ld16_nowait(slot + c0, vb);
              tmem_ld16_nowait(slot + NPSI + c0, vs);
              tmem_wait_ld();
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                const float big = __uint_as_float(vb[i]), small = __uint_as_float(vs[i]);
                if (g0 == 0) {
                  sv[c0 + i] = big;
                  cv[c0 + i] = small;
                } else {
                  two_sum_add(sv[c0 + i], cv[c0 + i], big);
                  cv[c0 + i] += small;
                }
              }
            }
          }
          tc_fence_before();
          mbar_arrive(&P.acc_empty[b]);
        }
        // component complete: value = S + C (FP32, rounded once)
        if (ok) {
          float cs = 0.f, cc = 0.f;  // this component's compensated sum over the orbitals
#pragma unroll
          for (int k = 0; k < NPSI; ++k) {
            const float v = sv[k] + cv[k];
            if (comp == 0) p0[k] = v;
            dot2_add(cs, cc, comp == 0 ? v : p0[k], v);
            if (a.psi_out && g < a.N) a.psi_out[(long long)(comp * NPSI + k) * a.N + g] = v;
          }
          if (comp == 0) {
            rs = cs;
            rc = cc;
          } else if (comp == 1) {
            gs[0] = cs;
            gc[0] = cc;
          } else if (comp == 2) {
            gs[1] = cs;
            gc[1] = cc;
          } else {
            gs[2] = cs;
            gc[2] = cc;
          }
        }
      }
      if (ok && g < a.N) {
        a.rho[g] = (double)rs + (double)rc;
        if (a.ncomp > 1)
#pragma unroll
          for (int c = 0; c < 3; ++c) a.grho[(long long)c * a.N + g] = 2.0 * ((double)gs[c] + (double)gc[c]);
      }
    }
  } else if (lane == 0) {
    const uint32_t idesc = idesc_tf32(kM, NPSI), idesc2 = idesc_tf32(kM, 2 * NPSI);
    long long st = 0, G = 0;
    for (long long t = 0; t < my_tiles; ++t) {
      for (int comp = 0; comp < a.ncomp; ++comp) {
        for (int g0 = 0; g0 < nkb; g0 += DR, ++G) {
          const int b = (int)(G % RA);
          const long long ause = G / RA;
          if (ok && ause > 0 && !mbar_wait(&P.acc_empty[b], (unsigned)((ause - 1) & 1), a.err, 24))
            ok = false;
          tc_fence_after();
          const uint32_t dbig = P.tmem_base + (uint32_t)(b * 2 * NPSI), dsmall = dbig + NPSI;
          const int g1 = min(g0 + DR, nkb);
          for (int kb = g0; kb < g1; ++kb, ++st) {
            const int slot = (int)(st % kPsiRing);
            if (ok && !mbar_wait(&P.full[slot], (unsigned)((st / kPsiRing) & 1), a.err, 22)) ok = false;
            tc_fence_after();
            if (ok) {
              const uint32_t base = smem_u32(sm + slot * kPsiStageBytes);
              const uint32_t Ah = base, Al = base + kTile;
              const uint32_t Bh = base + (uint32_t)kPsiAPieces, Bl = Bh + (uint32_t)NPSI * 128u;
              // descriptors advance by 32 bytes (2 units of 16) per K step of 8.
              // Y^T's lo rows follow its hi rows, so one MMA of N = 2 npsi
              // gives hi*hi (into the big slot) and hi*lo (into the small slot
              // right after it); lo*hi adds into the small slot.
              const uint64_t dAh = sdesc(Ah), dAl = sdesc(Al), dBh = sdesc(Bh);
              (void)Bl;
#pragma unroll
              for (int ks = 0; ks < kStageK / 8; ++ks) {
                const uint64_t o = 2u * (uint32_t)ks;
                const int acc = (kb > g0 || ks > 0) ? 1 : 0;
                mma_tf32(dbig, dAh + o, dBh + o, idesc2, acc);
                mma_tf32(dsmall, dAl + o, dBh + o, idesc, 1);
              }
            }
            mma_commit(&P.empty[slot]);
          }
          mma_commit(&P.acc_full[b]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kPsiMmaWarp) {
    tc_fence_after();
    tmem_dealloc(P.tmem_base, tcols);
  }
}

// ---------------------------------------------------------------------------
// Orbital density, resident-Y form (npsi <= 32): the same contraction and
// epilogue as k_tc_psi_density with the pipeline rearranged so that more
// bytes are in flight per SM.
//  * Y^T (both TF32 pieces, every K block) is loaded once per CTA and stays
//    in shared memory (npsi x ldk x 8 B, 72 KB at npsi = 32, 288 AOs).
//  * The TMA ring holds only raw fp32 A boxes (16 KB each, kPsrRing deep);
//    the splitter warps copy a box into one of two split buffers as TF32
//    hi/lo pieces and release the ring slot at once, so a slot is busy for
//    the load latency plus one read rather than until its MMAs complete.
//  * The MMA reads A from the split buffer and B from the resident Y.
// ---------------------------------------------------------------------------
constexpr int kPsrMaxN = 32;
constexpr int kPsrRing = 5;                                          // raw A boxes in flight
__host__ __device__ constexpr size_t psr_y_bytes(int npsi, int ldk) {
  return (size_t)(ldk / kStageK) * 2 * npsi * 128;
}
constexpr size_t kPsrYMax = psr_y_bytes(kPsrMaxN, 288);               // 72 KB: up to 288 AOs
constexpr size_t kPsrSmem = kPsrYMax + kPsrRing * kTile + 2 * 2 * kTile + 1024;

struct PsrPipe {
  uint64_t raw_full[kPsrRing], raw_empty[kPsrRing], sp_full[2], sp_empty[2], y_full;
  uint64_t acc_full[8], acc_empty[8];
  uint32_t tmem_base;
};

template <int NPSI>
__global__ void __launch_bounds__(kPsiThreads, 1)
    k_tc_psi_density_r(PsiArgs a, const __grid_constant__ CUtensorMap tmA,
                       const __grid_constant__ CUtensorMap tmD, const __grid_constant__ CUtensorMap tmY) {
  extern __shared__ __align__(1024) char smraw[];
  char *sm = (char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  char *ysm = sm;                                    // [kb][hi | lo][NPSI rows x 128 B]
  char *raw = sm + kPsrYMax;                         // [kPsrRing][16 KB]
  char *spl = raw + kPsrRing * kTile;                // [2][hi 16 KB | lo 16 KB]
  __shared__ PsrPipe P;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkb = a.ldk / kStageK;
  const long long ntiles = (a.N + kM - 1) / kM;
  const long long my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int per_tile = a.ncomp * nkb;
  const long long S = my_tiles * per_tile;
  const int RA = psi_ring(NPSI, a.ncomp);
  const int DR = a.drain;
  const int ncols = RA * 2 * NPSI;
  int tcols = 32;
  while (tcols < ncols) tcols <<= 1;
  constexpr uint32_t kYPiece = (uint32_t)NPSI * 128u;

  if (tid == 0) {
    for (int b = 0; b < kPsrRing; ++b) {
      mbar_init(&P.raw_full[b], 1);
      mbar_init(&P.raw_empty[b], kPsiProducers);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&P.sp_full[b], kPsiProducers);
      mbar_init(&P.sp_empty[b], 1);
    }
    mbar_init(&P.y_full, 1);
    for (int b = 0; b < 8; ++b) {
      mbar_init(&P.acc_full[b], 1);
      mbar_init(&P.acc_empty[b], kDrainers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kPsiMmaWarp) tmem_alloc(&P.tmem_base, tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  bool ok = true;
  if (warp == kPsiTmaWarp) {
    if (lane == 0) {
      // the whole Y^T once, then the raw A boxes of stage (tile, component, K block)
      mbar_expect_tx(&P.y_full, (uint32_t)nkb * 2u * kYPiece);
      for (int kb = 0; kb < nkb; ++kb) {
        const uint32_t yb = smem_u32(ysm) + (uint32_t)kb * 2u * kYPiece;
        tma_load_2d(yb, &tmY, kb * kStageK, 0, &P.y_full);
        tma_load_2d(yb + kYPiece, &tmY, kb * kStageK, NPSI, &P.y_full);
      }
      for (long long st = 0; st < S; ++st) {
        const int slot = (int)(st % kPsrRing);
        const long long use = st / kPsrRing;
        if (ok && use > 0 && !mbar_wait(&P.raw_empty[slot], (unsigned)((use - 1) & 1), a.err, 55))
          ok = false;
        if (!ok) break;
        const long long t = st / per_tile;
        const int r = (int)(st % per_tile), comp = r / nkb, kb = r % nkb;
        const int g0 = (int)((blockIdx.x + t * gridDim.x) * (long long)kM);
        const uint32_t dst = smem_u32(raw + slot * kTile);
        mbar_expect_tx(&P.raw_full[slot], (uint32_t)kTile);
        if (comp == 0) tma_load_3d(dst, &tmA, 0, g0, kb, &P.raw_full[slot]);
        else tma_load_3d(dst, &tmD, 0, g0, (comp - 1) * nkb + kb, &P.raw_full[slot]);
      }
    }
  } else if (warp < kPsiPW) {
    // splitters: raw box -> TF32 hi / lo pieces in the split buffer st % 2
    const int cch = tid & 7;
    for (long long st = 0; st < S; ++st) {
      const int slot = (int)(st % kPsrRing), sb = (int)(st & 1);
      if (ok && !mbar_wait(&P.raw_full[slot], (unsigned)((st / kPsrRing) & 1), a.err, 51)) ok = false;
      if (ok && st >= 2 && !mbar_wait(&P.sp_empty[sb], (unsigned)(((st >> 1) - 1) & 1), a.err, 52)) ok = false;
      if (ok) {
        const char *src = raw + slot * kTile;
        char *dst = spl + sb * 2 * kTile;
        float4 v[kPsiRowsPerThread];
#pragma unroll
        for (int j = 0; j < kPsiRowsPerThread; ++j) {
          const int row = (tid >> 3) + (kPsiProducers / 8) * j;
          v[j] = *reinterpret_cast<const float4 *>(src + swz(row, cch));
        }
        mbar_arrive(&P.raw_empty[slot]);  // the box is in registers: the slot can be refilled
#pragma unroll
        for (int j = 0; j < kPsiRowsPerThread; ++j) {
          const int row = (tid >> 3) + (kPsiProducers / 8) * j;
          store_split4(dst, row, cch, v[j]);
        }
      } else {
        mbar_arrive(&P.raw_empty[slot]);
      }
      fence_proxy_async();
      mbar_arrive(&P.sp_full[sb]);
    }
  } else if (warp < kPsiPW + 4) {
    // drains and epilogue, as in k_tc_psi_density
    const int row = (warp & 3) * 32 + lane;
    const uint32_t tbase = P.tmem_base + ((uint32_t)((warp & 3) * 32) << 16);
    long long G = 0;
    for (long long t = 0; t < my_tiles; ++t) {
      const long long g = (blockIdx.x + t * gridDim.x) * (long long)kM + row;
      float p0[NPSI];
      float rs = 0.f, rc = 0.f, gs[3] = {0.f, 0.f, 0.f}, gc[3] = {0.f, 0.f, 0.f};
      for (int comp = 0; comp < a.ncomp; ++comp) {
        float sv[NPSI], cv[NPSI];
        for (int g0 = 0; g0 < nkb; g0 += DR, ++G) {
          const int b = (int)(G % RA);
          const long long use = G / RA;
          bool got = ok && mbar_wait(&P.acc_full[b], (unsigned)(use & 1), a.err, 53);
          if (!got) ok = false;
          tc_fence_after();
          if (got) {
            const uint32_t slot = tbase + (uint32_t)(b * 2 * NPSI);
#pragma unroll
            for (int c0 = 0; c0 < NPSI; c0 += 16) {
              uint32_t vb[16], vs[16];
              tmem_ld16_nowait(slot + c0, vb);
              tmem_ld16_nowait(slot + NPSI + c0, vs);
              tmem_wait_ld();
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                const float big = __uint_as_float(vb[i]), small = __uint_as_float(vs[i]);
                if (g0 == 0) {
                  sv[c0 + i] = big;
                  cv[c0 + i] = small;
                } else {
                  two_sum_add(sv[c0 + i], cv[c0 + i], big);
                  cv[c0 + i] += small;
                }
              }
            }
          }
          tc_fence_before();
          mbar_arrive(&P.acc_empty[b]);
        }
        if (ok) {
          float cs = 0.f, cc = 0.f;  // this component's compensated sum over the orbitals
#pragma unroll
          for (int k = 0; k < NPSI; ++k) {
            const float v = sv[k] + cv[k];
            if (comp == 0) p0[k] = v;
            dot2_add(cs, cc, comp == 0 ? v : p0[k], v);
            if (a.psi_out && g < a.N) a.psi_out[(long long)(comp * NPSI + k) * a.N + g] = v;
          }
          if (comp == 0) {
            rs = cs;
            rc = cc;
          } else if (comp == 1) {
            gs[0] = cs;
            gc[0] = cc;
          } else if (comp == 2) {
            gs[1] = cs;
            gc[1] = cc;
          } else {
            gs[2] = cs;
            gc[2] = cc;
          }
        }
      }
      if (ok && g < a.N) {
        a.rho[g] = (double)rs + (double)rc;
        if (a.ncomp > 1)
#pragma unroll
          for (int c = 0; c < 3; ++c) a.grho[(long long)c * a.N + g] = 2.0 * ((double)gs[c] + (double)gc[c]);
      }
    }
  } else if (lane == 0) {
    const uint32_t idesc = idesc_tf32(kM, NPSI), idesc2 = idesc_tf32(kM, 2 * NPSI);
    if (!mbar_wait(&P.y_full, 0u, a.err, 56)) ok = false;
    long long st = 0, G = 0;
    for (long long t = 0; t < my_tiles; ++t) {
      for (int comp = 0; comp < a.ncomp; ++comp) {
        for (int g0 = 0; g0 < nkb; g0 += DR, ++G) {
          const int b = (int)(G % RA);
          const long long ause = G / RA;
          if (ok && ause > 0 && !mbar_wait(&P.acc_empty[b], (unsigned)((ause - 1) & 1), a.err, 54))
            ok = false;
          tc_fence_after();
          const uint32_t dbig = P.tmem_base + (uint32_t)(b * 2 * NPSI), dsmall = dbig + NPSI;
          const int g1 = min(g0 + DR, nkb);
          for (int kb = g0; kb < g1; ++kb, ++st) {
            const int sb = (int)(st & 1);
            if (ok && !mbar_wait(&P.sp_full[sb], (unsigned)((st >> 1) & 1), a.err, 57)) ok = false;
            tc_fence_after();
            if (ok) {
              const uint32_t Ah = smem_u32(spl + sb * 2 * kTile), Al = Ah + (uint32_t)kTile;
              const uint32_t Bh = smem_u32(ysm) + (uint32_t)kb * 2u * kYPiece, Bl = Bh + kYPiece;
              // descriptors advance by 32 bytes (2 units of 16) per K step of 8.
              // Y^T's lo rows follow its hi rows, so one MMA of N = 2 npsi
              // gives hi*hi (into the big slot) and hi*lo (into the small slot
              // right after it); lo*hi adds into the small slot.
              const uint64_t dAh = sdesc(Ah), dAl = sdesc(Al), dBh = sdesc(Bh);
              (void)Bl;
#pragma unroll
              for (int ks = 0; ks < kStageK / 8; ++ks) {
                const uint64_t o = 2u * (uint32_t)ks;
                const int acc = (kb > g0 || ks > 0) ? 1 : 0;
                mma_tf32(dbig, dAh + o, dBh + o, idesc2, acc);
                mma_tf32(dsmall, dAl + o, dBh + o, idesc, 1);
              }
            }
            mma_commit(&P.sp_empty[sb]);
          }
          mma_commit(&P.acc_full[b]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kPsiMmaWarp) {
    tc_fence_after();
    tmem_dealloc(P.tmem_base, tcols);
  }
}

// ---------------------------------------------------------------------------
// Quadrature on pre-split operands: M_pq = sum_g A_p(g) B_q(g) with A and B
// given as TF32 hi/lo arrays [nao][ld] (A = w phi or the GGA operand, split
// by the pass that forms it; B = phi, split once per geometry).  Grid: (tile,
// K chunk); one warp issues TMA bulk tensor loads of the four pieces into a
// 3-stage ring, one thread issues the MMAs (lo*hi + hi*lo + hi*hi into one
// accumulator), four warps drain the two ping-pong TMEM accumulators every
// `drain` stages into TMEM-resident TwoSum sums (S, C) and write the FP64
// partial tile.  Tiles are 128 x 128; the last, partial AO block (nao % 128
// rows) runs as an N = 16..112 MMA: as the B side directly, or -- for tiles
// whose A side is that block (non-symmetric case) -- by swapping the roles of
// A and B and storing the transposed result.
// ---------------------------------------------------------------------------
constexpr int kQtDrainWarps = 4;
constexpr int kQtMmaWarp = kQtDrainWarps;
constexpr int kQtTmaWarp = kQtMmaWarp + 1;
constexpr int kQtThreads = (kQtTmaWarp + 1) * 32;
constexpr int kQtRing = 3;
constexpr size_t kQtStageBytes = 4 * kTile;  // A hi, A lo, B hi, B lo (B pieces may be narrower)
constexpr size_t kQtSmem = kQtRing * kQtStageBytes + 1024;

struct QtTile {
  int arow, brow;  // first AO row of the A-side and B-side operand blocks
  int nb;          // MMA N (B rows): 128, or the partial block rounded up to 16
  int swap;        // A side reads the B arrays (and vice versa); store transposed
  int mt, nt;      // destination tile of the partial sums
};

constexpr int kQtMaxTiles = 12;  // tiles per k_tc_quad_tma launch (kernel parameter space)

struct QtArgs {
  QtTile tiles[kQtMaxTiles];
  int ntile;
  int blocked;  // operands K-blocked ([K / 32][row][32], 3D maps) rather than row-major
  long long N;
  int kchunk, drain, mtiles, ntiles;
  double *partial;
  int *err;
};

struct QtPipe {
  uint64_t full[kQtRing], empty[kQtRing], acc_full[2], acc_empty[2];
  uint32_t tmem_base;
};

__global__ void __launch_bounds__(kQtThreads, 1)
    k_tc_quad_tma(QtArgs a, const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                  const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl,
                  const __grid_constant__ CUtensorMap mAh16, const __grid_constant__ CUtensorMap mAl16,
                  const __grid_constant__ CUtensorMap mBh16, const __grid_constant__ CUtensorMap mBl16) {
  extern __shared__ __align__(1024) char smraw[];
  char *sm = (char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ QtPipe P;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const QtTile T = a.tiles[blockIdx.x];
  const int chunk = blockIdx.y;
  const long long k0 = (long long)chunk * a.kchunk;
  const long long k1 = min(k0 + (long long)a.kchunk, a.N);
  const int nstages = (int)((k1 - k0 + kStageK - 1) / kStageK);
  const int nsub = (nstages + a.drain - 1) / a.drain;
  const int nb = T.nb;
  if (tid == 0) {
    for (int b = 0; b < kQtRing; ++b) {
      mbar_init(&P.full[b], 1);
      mbar_init(&P.empty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&P.acc_full[b], 1);
      mbar_init(&P.acc_empty[b], kQtDrainWarps * 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kQtMmaWarp) tmem_alloc(&P.tmem_base, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  bool ok = true;
  if (warp == kQtTmaWarp) {
    if (lane == 0) {
      // the A side always has 128 rows; the B side nb rows (box 16 for narrow blocks)
      const CUtensorMap *ah = T.swap ? &mBh : &mAh, *al = T.swap ? &mBl : &mAl;
      const CUtensorMap *bh, *bl;
      if (nb == kN) {
        bh = T.swap ? &mAh : &mBh;
        bl = T.swap ? &mAl : &mBl;
      } else {
        bh = T.swap ? &mAh16 : &mBh16;
        bl = T.swap ? &mAl16 : &mBl16;
      }
      const int bbox = nb == kN ? kN : 16;
      const int nbox = nb / bbox;
      const uint32_t bytes = 2u * (uint32_t)kTile + 2u * (uint32_t)nb * 128u;
      for (int st = 0; st < nstages; ++st) {
        const int slot = st % kQtRing, use = st / kQtRing;
        if (ok && use > 0 && !mbar_wait(&P.empty[slot], (unsigned)((use - 1) & 1), a.err, 31)) ok = false;
        if (!ok) break;
        const int x = (int)(k0 + (long long)st * kStageK);
        const uint32_t base = smem_u32(sm + slot * kQtStageBytes);
        mbar_expect_tx(&P.full[slot], bytes);
        auto load = [&](uint32_t dst, const CUtensorMap *m, int row) {
          if (a.blocked) tma_load_3d(dst, m, 0, row, x / kStageK, &P.full[slot]);
          else tma_load_2d(dst, m, x, row, &P.full[slot]);
        };
        load(base, ah, T.arow);
        load(base + (uint32_t)kTile, al, T.arow);
        for (int q = 0; q < nbox; ++q) {
          const uint32_t off = (uint32_t)(q * bbox * 128);
          load(base + 2u * (uint32_t)kTile + off, bh, T.brow + q * bbox);
          load(base + 3u * (uint32_t)kTile + off, bl, T.brow + q * bbox);
        }
      }
    }
  } else if (warp == kQtMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(kM, nb);
      int stage = 0;
      for (int j = 0; j < nsub; ++j) {
        const int ab = j & 1, ause = j >> 1;
        if (ok && ause > 0 && !mbar_wait(&P.acc_empty[ab], (unsigned)((ause - 1) & 1), a.err, 34)) ok = false;
        tc_fence_after();
        const uint32_t tmem_d = P.tmem_base + (uint32_t)(ab * kN);
        const int s_end = min(nstages, (j + 1) * a.drain);
        bool first = true;
        for (; stage < s_end; ++stage) {
          const int slot = stage % kQtRing, use = stage / kQtRing;
          if (ok && !mbar_wait(&P.full[slot], (unsigned)(use & 1), a.err, 32)) ok = false;
          tc_fence_after();
          if (ok) {
            const uint32_t base = smem_u32(sm + slot * kQtStageBytes);
            const uint32_t Ah = base, Al = base + (uint32_t)kTile, Bh = base + 2u * (uint32_t)kTile,
                           Bl = base + 3u * (uint32_t)kTile;
            const uint64_t dAh = sdesc(Ah), dAl = sdesc(Al), dBh = sdesc(Bh), dBl = sdesc(Bl);
#pragma unroll
            for (int ks = 0; ks < kStageK / 8; ++ks) {
              const uint64_t o = 2u * (uint32_t)ks;
              mma_tf32(tmem_d, dAl + o, dBh + o, idesc, (first && ks == 0) ? 0 : 1);
              mma_tf32(tmem_d, dAh + o, dBl + o, idesc, 1);
              mma_tf32(tmem_d, dAh + o, dBh + o, idesc, 1);
            }
          }
          first = false;
          mma_commit(&P.empty[slot]);
        }
        mma_commit(&P.acc_full[ab]);
      }
    }
  } else {
    // drains: thread = TMEM lane (output row); nb columns
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    for (int j = 0; j < nsub; ++j) {
      const int b = j & 1, use = j >> 1;
      const bool got = ok && mbar_wait(&P.acc_full[b], (unsigned)(use & 1), a.err, 33);
      if (!got) ok = false;
      tc_fence_after();
      if (got) {
#pragma unroll 1
        for (int col = 0; col < nb; col += 16) {
          uint32_t va[16], sa[16], ca[16];
          tmem_ld16_nowait(P.tmem_base + lane_off + b * kN + col, va);
          if (j > 0) {
            tmem_ld16_nowait(P.tmem_base + lane_off + kColS + col, sa);
            tmem_ld16_nowait(P.tmem_base + lane_off + kColC + col, ca);
          }
          tmem_wait_ld();
          float sv[16], cv[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float v = __uint_as_float(va[i]);
            if (j == 0) {
              sv[i] = v;
              cv[i] = 0.f;
            } else {
              sv[i] = __uint_as_float(sa[i]);
              cv[i] = __uint_as_float(ca[i]);
              two_sum_add(sv[i], cv[i], v);
            }
          }
          tmem_st16(P.tmem_base + lane_off + kColS + col, sv);
          tmem_st16(P.tmem_base + lane_off + kColC + col, cv);
        }
        tmem_wait_st();
      }
      tc_fence_before();
      mbar_arrive(&P.acc_empty[b]);
    }
    // FP64 partial tile: P[chunk][mt][nt][row][col]
    const int row = warp * 32 + lane;
    double *tile = a.partial + (((long long)chunk * a.mtiles + T.mt) * a.ntiles + T.nt) * (kM * kN);
#pragma unroll 1
    for (int c0 = 0; c0 < nb; c0 += 16) {
      uint32_t sr[16], cr[16];
      tmem_ld16_nowait(P.tmem_base + lane_off + kColS + c0, sr);
      tmem_ld16_nowait(P.tmem_base + lane_off + kColC + c0, cr);
      tmem_wait_ld();
      double v[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = (double)__uint_as_float(sr[i]) + (double)__uint_as_float(cr[i]);
      if (ok) {
        if (!T.swap) {
#pragma unroll
          for (int i = 0; i < 16; ++i) tile[(long long)row * kN + c0 + i] = v[i];
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) tile[(long long)(c0 + i) * kN + row] = v[i];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kQtMmaWarp) {
    tc_fence_after();
    tmem_dealloc(P.tmem_base, kTmemCols);
  }
}

// ---------------------------------------------------------------------------
// Persistent quadrature for n_ao = 128 nfull + last with last <= 16 (e.g.
// 270 = 2 x 128 + 14) or no partial block: grid (tiles, groups).  The CTAs
// of group g share one contiguous K slice (1/groups of the grid points) and
// each computes one full 128 x 128 destination tile over all of it, so the
// CTAs of a group stream the same 128-row blocks at about the same pace.  The
// compensated sums stay in TMEM / registers over the whole slice; one FP64
// partial tile per CTA is written at the end and the reduce adds the groups.
// Operands are K-blocked ([K / 32][row][32]): every TMA box is one
// contiguous run of memory.
//
// The products with the partial block (at most 16 AOs) ride in the main MMA
// as its columns 128..143 (N = 144), the 16-row box stored right after the
// 128-row B block in shared memory:
//   tile (m, m), not swapped:  A = A block m, B = [B block m; narrow B]
//                              -> tiles (m, m) and (m, last);
//   swapped tile (m, n):       A = B block n, B = [A block m; narrow A]
//                              -> (m, n)^T and (last, n)^T, stored transposed;
// other tiles run with N = 128.  The (last, last) corner is computed apart
// (k_quad_corner).  TMEM (512 columns): two accumulator slots of 128 + 32
// columns, the main tile's TwoSum sums S (128 columns) and the narrow
// columns' sums and carries (16 each); the carries C of the main tile live in
// the registers of eight drain warps (two per TMEM lane group, 64 main
// columns each).
// ---------------------------------------------------------------------------
constexpr int kQpDrainWarps = 8;
constexpr int kQpMmaWarp = kQpDrainWarps;
constexpr int kQpTmaWarp = kQpMmaWarp + 1;
constexpr int kQpThreads = (kQpTmaWarp + 1) * 32;
constexpr uint32_t kQpSlot = kN + 32;           // 128 main + 16 narrow accumulator columns (+16 unused)
constexpr uint32_t kQpColS = 2 * kQpSlot;       // main-tile sums S (128 columns)
constexpr uint32_t kQpColXS = kQpColS + kN;     // narrow sums S (16)
constexpr uint32_t kQpColXC = kQpColXS + 16;    // narrow carries C (16)
constexpr int kQpTmemCols = 512;
constexpr uint32_t kQpNarrow = 16 * 128;        // one 16-row piece of a narrow box
// Stage layout: A hi | A lo | B hi + narrow hi | B lo + narrow lo.
constexpr uint32_t kQpOffBh = 2 * kTile, kQpOffBl = 3 * kTile + kQpNarrow;
constexpr size_t kQpStageBytes = 4 * kTile + 2 * kQpNarrow;
constexpr size_t kQpSmem = kQtRing * kQpStageBytes + 1024;
constexpr int kQpMaxFull = 6;  // full AO blocks handled by the persistent form
constexpr int kQpMaxTiles = kQpMaxFull * kQpMaxFull;

struct QpTile {
  int mt, nt;  // the full destination tile
  int swap;    // computed transposed: A side from the B operand, B side from the A operand
  int nb;      // MMA N: 128, or 144 with the narrow box
};

struct QpArgs {
  QpTile tiles[kQpMaxTiles];
  int ntile, groups;
  int blocked;  // operands K-blocked ([K / 32][row][32], 3D maps) rather than row-major
  int xrow;     // first AO row of the narrow block
  long long N;
  int drain, mtiles, ntiles;
  double *partial;  // [parts][mtiles][ntiles][128][128]
  int *err;
};

// Layout invariants of the tensor-core kernels, checked at compile time:
// dynamic shared memory within the 227 KB a CTA may use, TMEM columns within
// the 512 of an SM, kernel parameters (tile lists + eight tensor maps) within
// the classic 4 KB parameter space.
constexpr size_t kMaxDynSmem = 227 * 1024;
static_assert(kDensSmem <= kMaxDynSmem && kPsiSmem <= kMaxDynSmem && kQtSmem <= kMaxDynSmem &&
                  kQpSmem <= kMaxDynSmem,
              "dynamic shared memory above 227 KB");
static_assert(kTmemCols <= 512 && kQpColXC + 16 <= (uint32_t)kQpTmemCols && kQpTmemCols <= 512,
              "TMEM column layout");
static_assert(sizeof(QtArgs) + 8 * sizeof(CUtensorMap) <= 4096 &&
                  sizeof(QpArgs) + 8 * sizeof(CUtensorMap) <= 4096,
              "kernel parameters above 4 KB");
static_assert(kPsiRowsPerThread * kPsiProducers == kM * 8, "splitter rows per thread");
static_assert(kPsrSmem <= kMaxDynSmem, "resident-Y orbital density above 227 KB");
static_assert(kQpOffBh % 1024 == 0 && kQpOffBl % 1024 == 0 && kQpStageBytes % 1024 == 0,
              "operand pieces must start on 1024-byte boundaries (128-byte swizzle atoms)");

__global__ void __launch_bounds__(kQpThreads, 1)
    k_tc_quad_persist(QpArgs a, const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                      const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl,
                      const __grid_constant__ CUtensorMap mAh16, const __grid_constant__ CUtensorMap mAl16,
                      const __grid_constant__ CUtensorMap mBh16, const __grid_constant__ CUtensorMap mBl16) {
  extern __shared__ __align__(1024) char smraw[];
  char *sm = (char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ QtPipe P;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const QpTile T = a.tiles[blockIdx.x];
  const int g = blockIdx.y;
  const bool wide = T.nb > kN;  // the narrow box rides as MMA columns 128..143
  // this group's K slice: stages [s0, s0 + nstages) of 32 points
  const long long NS = (a.N + kStageK - 1) / kStageK;
  const long long s0 = NS * g / a.groups;
  const int nstages = (int)(NS * (g + 1) / a.groups - s0);
  const int nsub = (nstages + a.drain - 1) / a.drain;
  if (tid == 0) {
    for (int b = 0; b < kQtRing; ++b) {
      mbar_init(&P.full[b], 1);
      mbar_init(&P.empty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&P.acc_full[b], 1);
      mbar_init(&P.acc_empty[b], kQpDrainWarps * 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kQpMmaWarp) tmem_alloc(&P.tmem_base, kQpTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  bool ok = true;
  if (warp == kQpTmaWarp) {
    if (lane == 0) {
      // A side: 128 rows of the A operand (or of the B operand when swapped);
      // B side: 128 rows of the other operand, then its narrow box
      const CUtensorMap *ah = T.swap ? &mBh : &mAh, *al = T.swap ? &mBl : &mAl;
      const CUtensorMap *bh = T.swap ? &mAh : &mBh, *bl = T.swap ? &mAl : &mBl;
      const CUtensorMap *xh = T.swap ? &mAh16 : &mBh16, *xl = T.swap ? &mAl16 : &mBl16;
      const int arow = (T.swap ? T.nt : T.mt) * kM, brow = (T.swap ? T.mt : T.nt) * kN;
      const uint32_t bytes = 4u * (uint32_t)kTile + (wide ? 2u * kQpNarrow : 0u);
      for (int st = 0; st < nstages; ++st) {
        const int slot = st % kQtRing, use = st / kQtRing;
        if (ok && use > 0 && !mbar_wait(&P.empty[slot], (unsigned)((use - 1) & 1), a.err, 41)) ok = false;
        if (!ok) break;
        const int x = (int)((s0 + st) * kStageK);
        const uint32_t base = smem_u32(sm + slot * kQpStageBytes);
        mbar_expect_tx(&P.full[slot], bytes);
        auto load = [&](uint32_t dst, const CUtensorMap *m, int row) {
          if (a.blocked) tma_load_3d(dst, m, 0, row, (int)(s0 + st), &P.full[slot]);
          else tma_load_2d(dst, m, x, row, &P.full[slot]);
        };
        load(base, ah, arow);
        load(base + (uint32_t)kTile, al, arow);
        load(base + kQpOffBh, bh, brow);
        load(base + kQpOffBl, bl, brow);
        if (wide) {
          load(base + kQpOffBh + (uint32_t)kTile, xh, a.xrow);
          load(base + kQpOffBl + (uint32_t)kTile, xl, a.xrow);
        }
      }
    }
  } else if (warp == kQpMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(kM, T.nb);
      int stage = 0;
      for (int j = 0; j < nsub; ++j) {
        const int ab = j & 1, ause = j >> 1;
        if (ok && ause > 0 && !mbar_wait(&P.acc_empty[ab], (unsigned)((ause - 1) & 1), a.err, 44)) ok = false;
        tc_fence_after();
        const uint32_t tmem_d = P.tmem_base + (uint32_t)ab * kQpSlot;
        const int s_end = min(nstages, (j + 1) * a.drain);
        bool first = true;
        for (; stage < s_end; ++stage) {
          const int slot = stage % kQtRing, use = stage / kQtRing;
          if (ok && !mbar_wait(&P.full[slot], (unsigned)(use & 1), a.err, 42)) ok = false;
          tc_fence_after();
          if (ok) {
            // descriptors: offsets in 16-byte units from the stage base (every
            // piece starts on a 1024-byte boundary, so no carry leaves the
            // 14-bit address field); K steps of 8 advance by 2 units
            const uint64_t d0 = sdesc(smem_u32(sm + slot * kQpStageBytes));
            const uint64_t dAh = d0, dAl = d0 + (kTile >> 4), dBh = d0 + (kQpOffBh >> 4),
                           dBl = d0 + (kQpOffBl >> 4);
#pragma unroll
            for (int ks = 0; ks < kStageK / 8; ++ks) {
              const uint64_t o = 2u * (uint32_t)ks;
              const int acc = (first && ks == 0) ? 0 : 1;
              mma_tf32(tmem_d, dAl + o, dBh + o, idesc, acc);
              mma_tf32(tmem_d, dAh + o, dBl + o, idesc, 1);
              mma_tf32(tmem_d, dAh + o, dBh + o, idesc, 1);
            }
          }
          first = false;
          mma_commit(&P.empty[slot]);
        }
        mma_commit(&P.acc_full[ab]);
      }
    }
  } else {
    // drains: warp w owns TMEM lanes 32 (w % 4) .. and main columns 64 (w / 4) .. + 63;
    // the warps of half 0 also own the 16 narrow columns
    const int h = warp >> 2;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    const int c0 = h * 64;
    const bool has_x = wide && h == 0;
    float cm[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) cm[i] = 0.f;
    for (int j = 0; j < nsub; ++j) {
      const int b = j & 1, use = j >> 1;
      const bool got = ok && mbar_wait(&P.acc_full[b], (unsigned)(use & 1), a.err, 43);
      if (!got) ok = false;
      tc_fence_after();
      if (got) {
        const uint32_t slot = P.tmem_base + lane_off + (uint32_t)b * kQpSlot;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t va[16], sa[16];
          tmem_ld16_nowait(slot + c0 + q * 16, va);
          if (j > 0) tmem_ld16_nowait(P.tmem_base + lane_off + kQpColS + c0 + q * 16, sa);
          tmem_wait_ld();
          float sv[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float v = __uint_as_float(va[i]);
            if (j == 0) {
              sv[i] = v;
            } else {
              sv[i] = __uint_as_float(sa[i]);
              two_sum_add(sv[i], cm[q * 16 + i], v);
            }
          }
          tmem_st16(P.tmem_base + lane_off + kQpColS + c0 + q * 16, sv);
        }
        if (has_x) {
          const uint32_t xsa = P.tmem_base + lane_off + kQpColXS, xca = P.tmem_base + lane_off + kQpColXC;
          uint32_t va[16], sa[16], ca[16];
          tmem_ld16_nowait(slot + kN, va);
          if (j > 0) {
            tmem_ld16_nowait(xsa, sa);
            tmem_ld16_nowait(xca, ca);
          }
          tmem_wait_ld();
          float sv[16], cv[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float v = __uint_as_float(va[i]);
            if (j == 0) {
              sv[i] = v;
              cv[i] = 0.f;
            } else {
              sv[i] = __uint_as_float(sa[i]);
              cv[i] = __uint_as_float(ca[i]);
              two_sum_add(sv[i], cv[i], v);
            }
          }
          tmem_st16(xsa, sv);
          tmem_st16(xca, cv);
        }
        tmem_wait_st();
      }
      tc_fence_before();
      mbar_arrive(&P.acc_empty[b]);
    }
    const int row = (warp & 3) * 32 + lane;
    const long long tsz = (long long)kM * kN;
    double *tile = a.partial + (((long long)g * a.mtiles + T.mt) * a.ntiles + T.nt) * tsz;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t sr[16];
      tmem_ld16_nowait(P.tmem_base + lane_off + kQpColS + c0 + q * 16, sr);
      tmem_wait_ld();
      if (ok) {
        if (!T.swap) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            tile[(long long)row * kN + c0 + q * 16 + i] = (double)__uint_as_float(sr[i]) + (double)cm[q * 16 + i];
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            tile[(long long)(c0 + q * 16 + i) * kN + row] = (double)__uint_as_float(sr[i]) + (double)cm[q * 16 + i];
        }
      }
    }
    if (has_x) {
      uint32_t sr[16], cr[16];
      tmem_ld16_nowait(P.tmem_base + lane_off + kQpColXS, sr);
      tmem_ld16_nowait(P.tmem_base + lane_off + kQpColXC, cr);
      tmem_wait_ld();
      if (ok) {
        const int last = a.xrow / kM;
        if (!T.swap) {  // tile (mt, last): rows of the A block, narrow columns
          double *xt = a.partial + (((long long)g * a.mtiles + T.mt) * a.ntiles + last) * tsz;
#pragma unroll
          for (int i = 0; i < 16; ++i)
            xt[(long long)row * kN + i] = (double)__uint_as_float(sr[i]) + (double)__uint_as_float(cr[i]);
        } else {  // tile (last, nt): narrow rows, columns of the B block
          double *xt = a.partial + (((long long)g * a.mtiles + last) * a.ntiles + T.nt) * tsz;
#pragma unroll
          for (int i = 0; i < 16; ++i)
            xt[(long long)i * kN + row] = (double)__uint_as_float(sr[i]) + (double)__uint_as_float(cr[i]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kQpMmaWarp) {
    tc_fence_after();
    tmem_dealloc(P.tmem_base, kQpTmemCols);
  }
}

// The (last, last) corner of the quadrature for a partial block of at most
// 16 AOs, on the CUDA cores: C[p][q] = sum_g A_p(g) B_q(g) over K-blocked
// hi/lo pieces (x = hi + lo in FP32), a 32-term FMA chain per K block added
// into compensated (TwoSum) FP32 sums.  CTA c sums K blocks
// [c nkb / gridDim.x, (c + 1) nkb / gridDim.x), kCornerKB of them per pass
// (each thread keeps eight 16-byte loads of the next pass in flight while
// the current one computes), and writes
// its FP64 partial tile P[part0 + c][last][last]; thread (p, q) =
// (tid / 16, tid % 16).
constexpr int kCornerKB = 4;
__global__ void __launch_bounds__(256) k_quad_corner(const float *__restrict__ Ahl, const float *__restrict__ Bhl,
                                                     int nao, long long nkb, int xrow, int nrow, double *partial,
                                                     int part0, int mtiles, int ntiles) {
  __shared__ float sa[16][kCornerKB * 32 + 4], sb[16][kCornerKB * 32 + 4];
  const int tid = threadIdx.x, p = tid >> 4, q = tid & 15;
  const long long piece = nkb * nao * 32;  // floats per piece (hi, then lo)
  const long long kb0 = nkb * blockIdx.x / gridDim.x, kb1 = nkb * (blockIdx.x + 1) / gridDim.x;
  float s = 0.f, c = 0.f;
  // kCornerKB K blocks x 16 rows x 8 float4 per operand and piece: 2 per
  // thread; the next pass is loaded into registers while this one computes
  float4 ra[2][2], rb[2][2];  // [slot h][hi, lo]
  auto fetch = [&](long long kb) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = tid + 256 * h, kl = i >> 7, r = (i >> 3) & 15, e = (i & 7) * 4;
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      ra[h][0] = ra[h][1] = rb[h][0] = rb[h][1] = z;
      if (r < nrow && kb + kl < kb1) {
        const long long o = ((kb + kl) * nao + xrow + r) * 32 + e;
        ra[h][0] = *reinterpret_cast<const float4 *>(Ahl + o);
        ra[h][1] = *reinterpret_cast<const float4 *>(Ahl + piece + o);
        rb[h][0] = *reinterpret_cast<const float4 *>(Bhl + o);
        rb[h][1] = *reinterpret_cast<const float4 *>(Bhl + piece + o);
      }
    }
  };
  if (kb0 < kb1) fetch(kb0);
  for (long long kb = kb0; kb < kb1; kb += kCornerKB) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = tid + 256 * h, kl = i >> 7, r = (i >> 3) & 15, e = (i & 7) * 4;
      float *da = &sa[r][kl * 32 + e], *db = &sb[r][kl * 32 + e];
      da[0] = ra[h][0].x + ra[h][1].x;
      da[1] = ra[h][0].y + ra[h][1].y;
      da[2] = ra[h][0].z + ra[h][1].z;
      da[3] = ra[h][0].w + ra[h][1].w;
      db[0] = rb[h][0].x + rb[h][1].x;
      db[1] = rb[h][0].y + rb[h][1].y;
      db[2] = rb[h][0].z + rb[h][1].z;
      db[3] = rb[h][0].w + rb[h][1].w;
    }
    __syncthreads();
    if (kb + kCornerKB < kb1) fetch(kb + kCornerKB);
#pragma unroll
    for (int kl = 0; kl < kCornerKB; ++kl) {
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < 32; ++k) t = fmaf(sa[p][kl * 32 + k], sb[q][kl * 32 + k], t);
      two_sum_add(s, c, t);
    }
    __syncthreads();
  }
  const int last = xrow / kM;
  double *tile = partial + (((long long)(part0 + blockIdx.x) * mtiles + last) * ntiles + last) * ((long long)kM * kN);
  tile[(long long)p * kN + q] = (double)s + (double)c;
}

// hi/lo TF32 pieces of Z = a w phi + b u . grad phi (u, dphi optional; w
// optional, = 1): inputs with row stride ldi; outputs K-blocked,
// [ldo / 32][nao][32] per piece, with zeros in [N, ldo), so that the
// quadrature's 128-row x 32-point TMA boxes are contiguous 16 KB runs.
// Grid (column blocks of 1024, rows); 4 columns per thread (ldi a multiple of
// 4, ldo of 32, 16-byte aligned rows).
__global__ void __launch_bounds__(256)
    k_split_operand(const float *__restrict__ phi, const float *__restrict__ dphi,
                    const float *__restrict__ w, const float *__restrict__ u, int nao, long long N,
                    long long ldi, long long ldo, float a, float b, float *__restrict__ hi,
                    float *__restrict__ lo) {
  const int p = blockIdx.y;
  const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (g >= ldo) return;
  const long long j = (long long)p * ldi + g, NN = (long long)nao * ldi;
  float z[4] = {0.f, 0.f, 0.f, 0.f};
  if (g + 3 < N) {
    const float4 f = *reinterpret_cast<const float4 *>(phi + j);
    float4 wv = w ? *reinterpret_cast<const float4 *>(w + g) : make_float4(1.f, 1.f, 1.f, 1.f);
    z[0] = a * wv.x * f.x;
    z[1] = a * wv.y * f.y;
    z[2] = a * wv.z * f.z;
    z[3] = a * wv.w * f.w;
    if (u) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float4 uv = *reinterpret_cast<const float4 *>(u + d * ldi + g);
        const float4 dv = *reinterpret_cast<const float4 *>(dphi + d * NN + j);
        z[0] += b * uv.x * dv.x;
        z[1] += b * uv.y * dv.y;
        z[2] += b * uv.z * dv.z;
        z[3] += b * uv.w * dv.w;
      }
    }
  } else {
    for (int e = 0; e < 4; ++e) {
      if (g + e >= N) break;
      float v = (w ? a * w[g + e] : a) * phi[j + e];
      if (u)
        for (int d = 0; d < 3; ++d) v += b * u[d * ldi + g + e] * dphi[d * NN + j + e];
      z[e] = v;
    }
  }
  float4 h, l;
  split2(z[0], h.x, l.x);
  split2(z[1], h.y, l.y);
  split2(z[2], h.z, l.z);
  split2(z[3], h.w, l.w);
  const long long o = ((g >> 5) * nao + p) * 32 + (g & 31);
  *reinterpret_cast<float4 *>(hi + o) = h;
  *reinterpret_cast<float4 *>(lo + o) = l;
}

// Yhl[0][k][p], Yhl[1][k][p]: TF32 hi/lo pieces of C[p][k] sqrt(occ[k]) for
// k < nuse, zero for k in [nuse, npsi) and p in [nao, ldk).
__global__ void k_psi_operand(const double *__restrict__ C, const double *__restrict__ occ, int nao,
                              int nmo, int nuse, int npsi, int ldk, float *__restrict__ Yhl) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npsi * ldk) return;
  int k = idx / ldk, pp = idx % ldk;
  float x = 0.f;
  if (k < nuse && pp < nao) x = (float)(C[(long long)pp * nmo + k] * sqrt(fmax(occ[k], 0.0)));
  float hi, lo;
  split2(x, hi, lo);
  Yhl[idx] = hi;
  Yhl[(long long)npsi * ldk + idx] = lo;
}

}  // namespace tc

namespace tc {
// 2D row-major fp32 tensor [rows][ld] as a TMA map with boxes of 32 x box_rows
// and 128-byte swizzle (the UMMA K-major canonical layout of a 32-element
// K block); out-of-range rows read as zero.  The driver's encoder is looked
// up at run time (no link-time dependency on the driver library).
CUtensorMap tensor_map_2d_ext(const float *base, long long ld, long long cols, long long rows,
                              int box_rows);
// K-blocked fp32 operand [nkb][rows][32] as a 3D TMA map (x: the 32
// elements of a K block, y: row, z: K block) with boxes of 32 x box_rows x 1
// -- one contiguous run of box_rows x 128 bytes -- and 128-byte swizzle;
// rows past `rows` read as zero.
CUtensorMap tensor_map_3d_kblk(const float *base, long long rows, long long nkb, int box_rows);
CUtensorMap tensor_map_2d(const float *base, long long ld, long long rows, int box_rows) {
  return tensor_map_2d_ext(base, ld, ld, rows, box_rows);
}
// as tensor_map_2d with the valid row length `cols` <= ld: columns past it read as zero
CUtensorMap tensor_map_2d_ext(const float *base, long long ld, long long cols, long long rows,
                              int box_rows) {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {  // thread-safe one-time lookup
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    HQ_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    HQ_REQUIRE(fn && q == cudaDriverEntryPointSuccess, "cuTensorMapEncodeTiled unavailable");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  HQ_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base must be 16-byte aligned");
  HQ_REQUIRE(ld % 32 == 0, "TMA row stride must be a multiple of 32 floats");
  CUtensorMap m;
  HQ_REQUIRE(cols >= 1 && cols <= ld, "TMA row length out of range");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)kStageK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides,
                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cuTensorMapEncodeTiled failed"};
  return m;
}
CUtensorMap tensor_map_3d_kblk(const float *base, long long rows, long long nkb, int box_rows) {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    HQ_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    HQ_REQUIRE(fn && q == cudaDriverEntryPointSuccess, "cuTensorMapEncodeTiled unavailable");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  HQ_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base must be 16-byte aligned");
  HQ_REQUIRE(rows >= 1 && nkb >= 1 && rows < (1LL << 31) && nkb < (1LL << 31), "TMA extents out of range");
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)kStageK, (cuuint64_t)rows, (cuuint64_t)nkb};
  cuuint64_t strides[2] = {(cuuint64_t)kStageK * sizeof(float), (cuuint64_t)rows * kStageK * sizeof(float)};
  cuuint32_t box[3] = {(cuuint32_t)kStageK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides,
                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error{HQCGB_CUDA_ERROR, "cuTensorMapEncodeTiled (3D) failed"};
  return m;
}
}  // namespace tc

// ---------------------------------------------------------------------------
int tc_psi_max(bool gga) { return gga ? 32 : tc::kPsiMaxN; }
int tc_psi_width(int nuse) { return ceil_div(nuse, 16) * 16; }

void launch_psi_operand(const double *C, const double *occ, int nao, int nmo, int nuse, int ldk,
                        float *Yhl, cudaStream_t st) {
  int npsi = tc_psi_width(nuse);
  tc::k_psi_operand<<<ceil_div(npsi * ldk, 256), 256, 0, st>>>(C, occ, nao, nmo, nuse, npsi, ldk, Yhl);
  HQ_LAUNCH_CHECK();
}

// rho (and grad rho) from the grid-major AO values and the pre-split Y^T.
void launch_tc_psi_density(const float *phiT, const float *dphiT, const float *Yhl, int npsi, int ldk,
                           long long N, double *rho, double *grho, int *err, cudaStream_t st,
                           float *psi_out, int psi_drain) {
  HQ_REQUIRE(psi_drain >= 1, "drain interval must be >= 1");
  HQ_STAGE(ST_PSI, st);
  HQ_REQUIRE(npsi >= 16 && npsi <= tc::kPsiMaxN && npsi % 16 == 0, "orbital count out of range");
  HQ_REQUIRE(tc::psi_ring(npsi, grho ? 4 : 1) > 0, "orbital count too large for the TMEM layout");
  HQ_REQUIRE(ldk % tc::kStageK == 0, "AO stride must be a multiple of 32");
  static const int nsm = [] {
    int dev = 0, v = 0;
    HQ_CUDA(cudaGetDevice(&dev));
    HQ_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v;
  }();
  ensure_dyn_smem((const void *)tc::k_tc_psi_density<16>, tc::kPsiSmem);
  ensure_dyn_smem((const void *)tc::k_tc_psi_density<32>, tc::kPsiSmem);
  ensure_dyn_smem((const void *)tc::k_tc_psi_density<48>, tc::kPsiSmem);
  ensure_dyn_smem((const void *)tc::k_tc_psi_density<64>, tc::kPsiSmem);
  tc::PsiArgs a;
  a.phiT = phiT; a.dphiT = grho ? dphiT : nullptr; a.Yhl = Yhl; a.N = N; a.ldk = ldk;
  a.npsi = npsi; a.ncomp = grho ? 4 : 1; a.rho = rho; a.grho = grho; a.err = err;
  a.psi_out = psi_out;
  a.drain = psi_drain;
  HQ_REQUIRE(!grho || dphiT, "GGA density needs the gradient operand");
  HQ_REQUIRE(N <= (1LL << 29), "grid too large for 32-bit TMA row coordinates");
  // boxes of 32 fp32 (128 B, the swizzle span) x rows; row strides ldk * 4 B
  // phiT / dphiT are K-blocked ([component][AO block][g][32]): 3D maps whose
  // 128-point x 32-AO boxes are contiguous
  CUtensorMap tmA = tc::tensor_map_3d_kblk(phiT, N, ldk / tc::kStageK, tc::kM);
  CUtensorMap tmD = tc::tensor_map_3d_kblk(grho ? dphiT : phiT, N, (grho ? 3 : 1) * (ldk / tc::kStageK), tc::kM);
  CUtensorMap tmY = tc::tensor_map_2d(Yhl, ldk, 2LL * npsi, npsi);
  long long ntiles = ceil_div(N, tc::kM);
  int grid = (int)std::min<long long>(ntiles, nsm);
  // resident-Y form when Y^T fits its shared-memory region (knob
  // "psi_ring" = 1 selects the ring form for comparison)
  const bool resident = npsi <= tc::kPsrMaxN && tc::psr_y_bytes(npsi, ldk) <= tc::kPsrYMax &&
                        tune_get("psi_ring", 0) == 0;
  if (resident) {
    ensure_dyn_smem((const void *)tc::k_tc_psi_density_r<16>, tc::kPsrSmem);
    ensure_dyn_smem((const void *)tc::k_tc_psi_density_r<32>, tc::kPsrSmem);
    if (npsi == 16) tc::k_tc_psi_density_r<16><<<grid, tc::kPsiThreads, tc::kPsrSmem, st>>>(a, tmA, tmD, tmY);
    else tc::k_tc_psi_density_r<32><<<grid, tc::kPsiThreads, tc::kPsrSmem, st>>>(a, tmA, tmD, tmY);
    HQ_LAUNCH_CHECK();
    return;
  }
  switch (npsi) {
    case 16: tc::k_tc_psi_density<16><<<grid, tc::kPsiThreads, tc::kPsiSmem, st>>>(a, tmA, tmD, tmY); break;
    case 32: tc::k_tc_psi_density<32><<<grid, tc::kPsiThreads, tc::kPsiSmem, st>>>(a, tmA, tmD, tmY); break;
    case 48: tc::k_tc_psi_density<48><<<grid, tc::kPsiThreads, tc::kPsiSmem, st>>>(a, tmA, tmD, tmY); break;
    default: tc::k_tc_psi_density<64><<<grid, tc::kPsiThreads, tc::kPsiSmem, st>>>(a, tmA, tmD, tmY); break;
  }
  HQ_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
int tc_quad_chunk() { return 2048; }

size_t tc_quad_partial_doubles(int nao, long long N, int kchunk) {
  int mt = ceil_div(nao, tc::kM), nt = ceil_div(nao, tc::kN);
  long long chunks = ceil_div(N, kchunk > 0 ? kchunk : tc_quad_chunk());
  return (size_t)chunks * mt * nt * tc::kM * tc::kN;
}

int tc_quad_tiles(int nao, bool sym) {
  const int nb = ceil_div(nao, tc::kM);
  return sym ? nb * (nb + 1) / 2 : nb * nb;
}

// Tile plan of the quadrature for nao AOs in 128-row blocks: which CTA writes
// which 128 x 128 destination tile (mt, nt) of the partial sums.
//  * persistent form (K-blocked operands; 1..6 full blocks and a last block
//    of at most 16 rows, or none): k_tc_quad_persist runs the full tiles; the
//    products with the partial block ride as MMA columns 128..143:
//      (m, last) on tile (m, m);
//      non-symmetric: (last, n) on tile ((n + 1) % nfull, n), computed
//      transposed (its A side from the B operand);
//    the (last, last) corner runs in k_quad_corner.  One full block and a
//    partial one, non-symmetric, would need tile (0, 0) both ways: tile-list
//    form;
//  * tile-list form otherwise: every tile of the upper triangle (sym) or of
//    the whole square through k_tc_quad_tma, at most kQtMaxTiles per launch.
// A tile whose A-side block is the narrow one is computed transposed
// (swap = 1: A side from the B arrays), so the narrow block is always the
// MMA's N side, rounded up to a multiple of 16 rows.
struct QuadTilePlan {
  int nblk = 0, nb_last = 0;
  bool persist = false;
  bool corner = false;            // persistent form with a partial block: k_quad_corner
  tc::QpArgs f{};                 // persistent form: the full tiles
  std::vector<tc::QtArgs> lists;  // k_tc_quad_tma launches, tile lists only
};

static bool plan_persist(int nao, bool sym, tc::QpArgs &f) {
  const int nblk = ceil_div(nao, tc::kM);
  const int last = nao - tc::kM * (nblk - 1);
  const bool narrow = last < tc::kM;
  const int nfull = narrow ? nblk - 1 : nblk;
  if ((narrow && last > 16) || nfull < 1 || nfull > tc::kQpMaxFull) return false;
  if (narrow && !sym && nfull == 1) return false;
  f = tc::QpArgs{};
  f.xrow = nfull * tc::kM;
  for (int mt = 0; mt < nfull; ++mt)
    for (int nt = 0; nt < nfull; ++nt) {
      if (sym && nt < mt) continue;
      tc::QpTile &t = f.tiles[f.ntile++];
      t.mt = mt;
      t.nt = nt;
      t.swap = 0;
      t.nb = tc::kN;
      if (!narrow) continue;
      if (mt == nt) {
        t.nb = tc::kN + 16;  // (m, last)
      } else if (!sym && mt == (nt + 1) % nfull) {
        t.swap = 1;          // (m, n)^T and (last, n)^T
        t.nb = tc::kN + 16;
      }
    }
  return true;
}

static QuadTilePlan plan_quad_tiles(int nao, bool sym, bool allow_persist = true) {
  QuadTilePlan p;
  p.nblk = ceil_div(nao, tc::kM);
  const int last = nao - tc::kM * (p.nblk - 1);
  const bool narrow = last < tc::kM;
  p.nb_last = ceil_div(last, 16) * 16;
  if (allow_persist && plan_persist(nao, sym, p.f)) {
    p.persist = true;
    p.corner = narrow;
    return p;
  }
  auto push = [&p](const tc::QtTile &t) {
    if (p.lists.empty() || p.lists.back().ntile == tc::kQtMaxTiles) p.lists.push_back(tc::QtArgs{});
    tc::QtArgs &a = p.lists.back();
    a.tiles[a.ntile++] = t;
  };
  for (int mt = 0; mt < p.nblk; ++mt)
    for (int nt = 0; nt < p.nblk; ++nt) {
      if (sym && nt < mt) continue;
      const bool nm = narrow && mt == p.nblk - 1, nn = narrow && nt == p.nblk - 1;
      tc::QtTile t;
      t.mt = mt;
      t.nt = nt;
      if (nm && !nn) {  // narrow A block: compute the transposed tile
        t.arow = nt * tc::kM;
        t.brow = mt * tc::kM;
        t.nb = p.nb_last;
        t.swap = 1;
      } else {
        t.arow = mt * tc::kM;
        t.brow = nt * tc::kN;
        t.nb = nn ? p.nb_last : tc::kN;
        t.swap = 0;
      }
      push(t);
    }
  return p;
}

// K slices (CTA groups) of the persistent quadrature: one CTA per SM for
// the whole launch (the autotuner's "quad_groups" when set); half of that
// inside a concurrent batch, whose other configurations' kernels need SMs
// too (measured on the H54 batch of 16: 9.56 evals/s at 19 groups against
// 9.10 at 38); at most one slice per 64 stages and at most the chunk count
// the partial buffer holds.
static int quad_groups(int ntile, long long N) {
  int dev = 0, sms = 0;
  HQ_CUDA(cudaGetDevice(&dev));
  HQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  long long g = std::max(1, sms / std::max(1, ntile));
  const long long t = tune_get("quad_groups", 0);
  if (t > 0) g = t;
  if (gpu_share() > 1) g = std::max(1LL, g / 2);
  g = std::min<long long>(g, std::max<long long>(1, ceil_div(N, (long long)tc::kStageK * 64)));
  g = std::min<long long>(g, ceil_div(N, (long long)tc_quad_chunk()));
  return (int)std::max<long long>(1, g);
}

// M = scale * sum_g A_p(g) B_q(g) (+ its transpose when add_transpose) from the
// pre-split pieces Ahl, Bhl [2][nao][ld] (hi rows, then lo rows); sym: M is
// symmetric (only tiles nt >= mt are computed; the reduce mirrors them).
void launch_tc_quad_split(const float *Ahl, const float *Bhl, int nao, long long N, long long ld,
                          bool sym, bool add_transpose, double scale, double *partial, double *M,
                          int *err, cudaStream_t st, int drain, int kchunk, bool blocked) {
  HQ_STAGE(ST_QUAD, st);
  HQ_REQUIRE(drain >= 1, "drain must be >= 1");
  if (kchunk <= 0) kchunk = tc_quad_chunk();
  HQ_REQUIRE(kchunk % tc::kStageK == 0, "K chunk must be a multiple of 32");
  HQ_REQUIRE(ld % 32 == 0 && ld >= N, "pre-split operands need a row stride that is a multiple of 32");
  HQ_REQUIRE(N <= (1LL << 31) - 64, "grid too large for 32-bit TMA coordinates");
  const QuadTilePlan plan = plan_quad_tiles(nao, sym, blocked);  // the persistent form reads K-blocked pieces
  const int nblk = plan.nblk;
  const long long rows = nao;
  const float *Ah = Ahl, *Al = Ahl + (size_t)nao * ld, *Bh = Bhl, *Bl = Bhl + (size_t)nao * ld;
  // row-major pieces: 2D maps whose columns past N read as zero; K-blocked
  // pieces ([ld / 32][nao][32], zero-padded past N): 3D maps
  auto map = [&](const float *b, int box) {
    return blocked ? tc::tensor_map_3d_kblk(b, rows, ld / tc::kStageK, box)
                   : tc::tensor_map_2d_ext(b, ld, N, rows, box);
  };
  CUtensorMap mAh = map(Ah, tc::kM), mAl = map(Al, tc::kM), mBh = map(Bh, tc::kN), mBl = map(Bl, tc::kN);
  CUtensorMap mAh16 = map(Ah, 16), mAl16 = map(Al, 16), mBh16 = map(Bh, 16), mBl16 = map(Bl, 16);
  int nparts = 0;    // partial tiles per destination tile
  int ncorner = -1;  // of the (last, last) tile, when k_quad_corner computes it
  if (plan.persist) {
    ensure_dyn_smem((const void *)tc::k_tc_quad_persist, tc::kQpSmem);
    tc::QpArgs f = plan.f;
    f.blocked = blocked ? 1 : 0;
    f.groups = quad_groups(f.ntile, N);
    f.N = N;
    f.drain = drain;
    f.mtiles = nblk;
    f.ntiles = nblk;
    f.partial = partial;
    f.err = err;
    nparts = f.groups;
    tc::k_tc_quad_persist<<<dim3(f.ntile, f.groups), tc::kQpThreads, tc::kQpSmem, st>>>(
        f, mAh, mAl, mBh, mBl, mAh16, mAl16, mBh16, mBl16);
    HQ_LAUNCH_CHECK();
    if (plan.corner) {
      // two CTAs per SM, within the partial tiles the buffer holds
      int dev = 0, sms = 0;
      HQ_CUDA(cudaGetDevice(&dev));
      HQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      const long long nkb = ld / tc::kStageK;
      ncorner = (int)std::max<long long>(
          1, std::min<long long>({2LL * sms, nkb, ceil_div(N, (long long)tc_quad_chunk())}));
      tc::k_quad_corner<<<ncorner, 256, 0, st>>>(Ahl, Bhl, nao, nkb, f.xrow, nao - f.xrow, partial, 0, nblk, nblk);
      HQ_LAUNCH_CHECK();
      tc::k_quad_corner_sum<<<256, 256, 0, st>>>(partial, ncorner, nblk, nblk, nblk - 1);
      HQ_LAUNCH_CHECK();
      ncorner = 1;  // the corner's sum now sits in part 0
    }
  } else {
    ensure_dyn_smem((const void *)tc::k_tc_quad_tma, tc::kQtSmem);
    nparts = (int)ceil_div(N, (long long)kchunk);
    for (tc::QtArgs a : plan.lists) {
      a.blocked = blocked ? 1 : 0;
      a.N = N;
      a.kchunk = kchunk;
      a.drain = drain;
      a.mtiles = nblk;
      a.ntiles = nblk;
      a.partial = partial;
      a.err = err;
      tc::k_tc_quad_tma<<<dim3(a.ntile, nparts), tc::kQtThreads, tc::kQtSmem, st>>>(
          a, mAh, mAl, mBh, mBl, mAh16, mAl16, mBh16, mBl16);
      HQ_LAUNCH_CHECK();
    }
  }
  // sum the partial tiles in place (coalesced), then assemble M from the sums
  tc::k_tc_quad_sum_parts<<<ceil_div((long long)nblk * nblk * tc::kM * tc::kN, 256), 256, 0, st>>>(
      partial, nparts, nblk, nblk, sym ? 1 : 0, ncorner >= 0 ? nblk - 1 : -1, ncorner);
  HQ_LAUNCH_CHECK();
  tc::k_tc_quad_reduce<<<ceil_div((long long)nao * nao, 256), 256, 0, st>>>(
      partial, 1, nblk, nblk, nao, sym ? 1 : 0, add_transpose ? 1 : 0, scale, M, -1, 0);
  HQ_LAUNCH_CHECK();
}

// hi/lo pieces of a w phi + b u . grad phi into out [2][nao][ldo]
void launch_split_operand(const float *phi, const float *dphi, const float *w, const float *u, int nao,
                          long long N, long long ldi, long long ldo, float a, float b, float *out,
                          cudaStream_t st) {
  HQ_STAGE(ST_SPLIT, st);
  HQ_REQUIRE(ldi % 4 == 0 && ldo % 32 == 0 && ldo >= N && ldi >= N, "split operand: bad row strides");
  dim3 grid(ceil_div(ldo, 1024), nao);
  tc::k_split_operand<<<grid, 256, 0, st>>>(phi, dphi, w, u, nao, N, ldi, ldo, a, b, out,
                                             out + (size_t)nao * ldo);
  HQ_LAUNCH_CHECK();
}

// Quadrature of the Fock build from the pre-split phi (phihl [2][nao][ld]):
// LDA  M = (w phi) phi^T (symmetric);  GGA  M = Z phi^T + phi Z^T with
// Z = 0.5 w phi + dV u . grad phi.  zhl [2][nao][ld] receives the split operand.
void launch_tc_quadrature(const float *phi, const float *dphi, const float *phihl, const float *w,
                          const float *u, float dV, int nao, long long N, long long ld, bool gga,
                          double scale, double *partial, double *M, int *err, cudaStream_t st, int drain,
                          float *zhl) {
  HQ_REQUIRE(zhl && phihl, "quadrature needs the split operand buffers");
  // K chunk: a tuned multiple of the default (the partial tiles are sized
  // for the default, so longer chunks always fit)
  long long kc = tune_get("quad_kchunk", tc_quad_chunk());
  if (kc < tc_quad_chunk() || kc % tc_quad_chunk() != 0 || kc > (1 << 20)) kc = tc_quad_chunk();
  if (!gga) {
    launch_split_operand(phi, nullptr, w, nullptr, nao, N, ld, ld, 1.f, 0.f, zhl, st);
    launch_tc_quad_split(zhl, phihl, nao, N, ld, true, false, scale, partial, M, err, st, drain, (int)kc, true);
    return;
  }
  HQ_REQUIRE(dphi && u, "GGA quadrature needs dphi and u");
  launch_split_operand(phi, dphi, w, u, nao, N, ld, ld, 0.5f, dV, zhl, st);
  launch_tc_quad_split(zhl, phihl, nao, N, ld, false, true, scale, partial, M, err, st, drain, (int)kc, true);
}

size_t tc_density_partial_doubles(int nao, long long ld, bool gga) {
  int mt = ceil_div(nao, tc::kM);
  return (size_t)mt * ld * (gga ? 4 : 1);
}

int tc_ldk(int nao) { return ceil_div(nao, 32) * 32; }

void launch_transpose_phi(const float *phi, int nao, long long N, long long ld, float *phiT,
                          cudaStream_t st) {
  int ldk = tc_ldk(nao);
  dim3 grid(ceil_div(N, 32), ceil_div(ldk, 32));
  tc::k_transpose_phi<<<grid, 256, 0, st>>>(phi, nao, N, ld, phiT);
  HQ_LAUNCH_CHECK();
}

// D32: [nao][ldk] (zero columns beyond nao); phiT: [N][ldk] grid-major copy.
void launch_tc_density(const float *phi, const float *phiT, const float *dphi, const float *D32,
                       int nao, long long N, long long ld, double *part, double *rho, double *grho,
                       int *err, cudaStream_t st, int nsplit, int drain) {
  HQ_STAGE(ST_DENSITY, st);
  HQ_REQUIRE(ld % 4 == 0, "row stride must be a multiple of 4 floats");
  HQ_REQUIRE(nsplit == 2, "nsplit must be 2 (3xTF32)");
  HQ_REQUIRE(drain >= 1, "drain must be >= 1");
  ensure_dyn_smem((const void *)tc::k_tc_density, tc::kDensSmem);
  int mt = ceil_div(nao, tc::kM);
  int ldk = tc_ldk(nao);
  tc::DensArgs a;
  a.D = tc::Operand{D32, ldk, nao, tc::kStageK};
  a.phiT = tc::Operand{phiT, tc::kStageK, (int)N, N * tc::kStageK};
  a.phi = phi; a.dphi = grho ? dphi : nullptr; a.nao = nao;
  a.kpad = ldk; a.drain = drain; a.ns = nsplit; a.N = N; a.ld = ld; a.part = part;
  a.part_g = grho ? part + (size_t)mt * ld : nullptr; a.err = err;
  dim3 grid(mt, ceil_div(N, tc::kN));
  tc::k_tc_density<<<grid, tc::kThreads, tc::kDensSmem, st>>>(a);
  HQ_LAUNCH_CHECK();
  tc::k_tc_density_reduce<<<ceil_div(N, 256), 256, 0, st>>>(part, a.part_g, mt, N, ld, rho, grho);
  HQ_LAUNCH_CHECK();
}

}  // namespace hqcgb

// ---------------------------------------------------------------------------
// C ABI: the two tensor-core contractions as library calls (tests and tools).
// ---------------------------------------------------------------------------
// C ABI: the GGA Fock quadrature of the mixed path, M = Z phi^T + phi Z^T with
// Z = 0.5 w phi + dV u . grad phi (hqc/pbc/solver.py:680-694 with the PBE
// gradient term); phi [nao][ld], dphi [3][nao][ld], w [ld], u [3][ld] fp32
// (device), ld % 32 == 0.  Splits phi and Z into TF32 pieces, then runs the
// tensor-core quadrature (non-symmetric tile set).
extern "C" int hqcgb_tc_quadrature_gga(int nao, long long N, long long ld, const float *phi,
                                       const float *dphi, const float *w, const float *u, float dV,
                                       int drain, double *M, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(nao >= 1 && N >= 1 && ld >= N && ld % 32 == 0 && phi && dphi && w && u && M, "bad argument");
    StreamBuf part_buf(tc_quad_partial_doubles(nao, N) * sizeof(double), st),
        hl_buf(4 * (size_t)nao * ld * sizeof(float), st), err_buf(sizeof(int), st);
    double *part = part_buf.as<double>();
    float *hl = hl_buf.as<float>();
    int *err = err_buf.as<int>();
    HQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    float *phl = hl, *zhl = hl + 2 * (size_t)nao * ld;
    launch_split_operand(phi, nullptr, nullptr, nullptr, nao, N, ld, ld, 1.f, 0.f, phl, st);
    launch_tc_quadrature(phi, dphi, phl, w, u, dV, nao, N, ld, true, 1.0, part, M, err, st, drain, zhl);
    int h = 0;
    HQ_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (h) throw Error{HQCGB_CUDA_ERROR, "tensor-core pipeline wait limit hit"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

extern "C" int hqcgb_tc_quadrature(int nao, long long N, long long ld, const float *phi,
                                   const float *w, int nsplit, int drain, double *M, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(nao >= 1 && N >= 1 && ld >= N && ld % 4 == 0 && phi && w && M, "bad argument");
    HQ_REQUIRE(nsplit == 2, "nsplit must be 2 (3xTF32)");
    const long long ldo = (N + 31) / 32 * 32;
    StreamBuf part_buf(tc_quad_partial_doubles(nao, N) * sizeof(double), st),
        hl_buf(4 * (size_t)nao * ldo * sizeof(float), st), err_buf(sizeof(int), st);
    double *part = part_buf.as<double>();
    float *hl = hl_buf.as<float>();
    int *err = err_buf.as<int>();
    HQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    float *phl = hl, *zhl = hl + 2 * (size_t)nao * ldo;
    launch_split_operand(phi, nullptr, nullptr, nullptr, nao, N, ld, ldo, 1.f, 0.f, phl, st);
    launch_split_operand(phi, nullptr, w, nullptr, nao, N, ld, ldo, 1.f, 0.f, zhl, st);
    launch_tc_quad_split(zhl, phl, nao, N, ldo, true, false, 1.0, part, M, err, st, drain, 0, true);
    int h = 0;
    HQ_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (h) throw Error{HQCGB_CUDA_ERROR, "tensor-core pipeline wait limit hit"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

extern "C" int hqcgb_tc_density(int nao, long long N, long long ld, const float *phi,
                                const float *D, int nsplit, int drain, double *rho, void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(nao >= 1 && N >= 1 && ld >= N && ld % 4 == 0 && phi && D && rho, "bad argument");
    int ldk = tc_ldk(nao);
    StreamBuf part_buf(tc_density_partial_doubles(nao, ld, false) * sizeof(double), st),
        phiT_buf((size_t)N * ldk * sizeof(float), st), D32_buf((size_t)nao * ldk * sizeof(float), st),
        err_buf(sizeof(int), st);
    double *part = part_buf.as<double>();
    float *phiT = phiT_buf.as<float>(), *D32 = D32_buf.as<float>();
    int *err = err_buf.as<int>();
    HQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    HQ_CUDA(cudaMemsetAsync(D32, 0, (size_t)nao * ldk * sizeof(float), st));
    HQ_CUDA(cudaMemcpy2DAsync(D32, ldk * sizeof(float), D, nao * sizeof(float), nao * sizeof(float),
                              nao, cudaMemcpyDeviceToDevice, st));
    launch_transpose_phi(phi, nao, N, ld, phiT, st);
    launch_tc_density(phi, phiT, nullptr, D32, nao, N, ld, part, rho, nullptr, err, st, nsplit, drain);
    int h = 0;
    HQ_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (h) throw Error{HQCGB_CUDA_ERROR, "tensor-core pipeline wait limit hit"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

// rho (and grad rho when dphi and grho are given) = sum_k occ_k |sum_p C_pk phi_p|^2
// over the first nuse orbitals; C is [nao][nmo] row-major (FP64), phi and
// dphi are AO-major fp32 with row stride ld.
extern "C" int hqcgb_tc_orbital_density(int nao, long long N, long long ld, const float *phi,
                                        const float *dphi, const double *C, const double *occ,
                                        int nmo, int nuse, int drain, double *rho, double *grho,
                                        void *stream) {
  using namespace hqcgb;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    HQ_REQUIRE(nao >= 1 && N >= 1 && ld >= N && ld % 4 == 0 && phi && C && occ && rho,
               "bad argument");
    HQ_REQUIRE(nuse >= 1 && nuse <= nmo && nuse <= tc_psi_max(dphi != nullptr), "orbital count out of range");
    HQ_REQUIRE((dphi == nullptr) == (grho == nullptr), "dphi and grho go together");
    int ldk = tc_ldk(nao);
    int ncomp = dphi ? 4 : 1;
    StreamBuf phiT_buf((size_t)ncomp * N * ldk * sizeof(float), st),
        Yhl_buf((size_t)2 * tc_psi_max(false) * ldk * sizeof(float), st), err_buf(sizeof(int), st);
    float *phiT = phiT_buf.as<float>(), *Yhl = Yhl_buf.as<float>();
    int *err = err_buf.as<int>();
    HQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    launch_transpose_phi(phi, nao, N, ld, phiT, st);
    if (dphi)
      for (int d = 0; d < 3; ++d)
        launch_transpose_phi(dphi + (size_t)d * nao * ld, nao, N, ld, phiT + (size_t)(d + 1) * N * ldk,
                             st);
    launch_psi_operand(C, occ, nao, nmo, nuse, ldk, Yhl, st);
    launch_tc_psi_density(phiT, dphi ? phiT + (size_t)N * ldk : nullptr, Yhl, tc_psi_width(nuse), ldk,
                          N, rho, grho, err, st, nullptr, drain);
    int h = 0;
    HQ_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (h) throw Error{HQCGB_CUDA_ERROR, "tensor-core pipeline wait limit hit"};
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}

// C ABI (host only, no device work): the quadrature's tile plan for nao AOs
// (sym: upper-triangle tiles only).  One row of 7 ints per computed product,
// {kind, mt, nt, arow, brow, nb, swap}: kind 0 a full tile of the
// persistent kernel, 1 a narrow product (the MMA columns 128..143 of a
// persistent CTA, or the corner of k_quad_corner), 2 a tile of the tile-list
// kernel; (mt, nt) the destination tile, arow / brow the first AO
// row of the MMA's A / B side (swap = 1: A side from the B operand, stored
// transposed), nb the MMA N.  count = rows (at most cap are written);
// launches = tensor-core quadrature kernel launches before the reduce (the
// CUDA-core corner kernel not counted).
extern "C" int hqcgb_tc_quad_tiles(int nao, int sym, int cap, int *tiles, int *count, int *launches) {
  using namespace hqcgb;
  try {
    HQ_REQUIRE(nao >= 1 && nao <= kMaxNao && cap >= 0 && (cap == 0 || tiles) && count && launches,
               "bad argument");
    const QuadTilePlan p = plan_quad_tiles(nao, sym != 0);
    int k = 0;
    auto row = [&](int kind, int mt, int nt, int arow, int brow, int nb, int swap) {
      if (k < cap) {
        int *r = tiles + 7 * (size_t)k;
        r[0] = kind; r[1] = mt; r[2] = nt; r[3] = arow; r[4] = brow; r[5] = nb; r[6] = swap;
      }
      ++k;
    };
    if (p.persist) {
      for (int t = 0; t < p.f.ntile; ++t)
        row(0, p.f.tiles[t].mt, p.f.tiles[t].nt, p.f.tiles[t].mt * tc::kM, p.f.tiles[t].nt * tc::kN, tc::kN, 0);
      const int last = p.f.xrow / tc::kM;
      for (int t = 0; t < p.f.ntile; ++t) {
        const tc::QpTile &q = p.f.tiles[t];
        if (q.nb == tc::kN) continue;
        // the narrow columns of a wide CTA: (mt, last), or (last, nt) transposed
        if (!q.swap) row(1, q.mt, last, q.mt * tc::kM, p.f.xrow, 16, 0);
        else row(1, last, q.nt, q.nt * tc::kN, p.f.xrow, 16, 1);
      }
      if (p.corner) row(1, last, last, p.f.xrow, p.f.xrow, 16, 0);  // k_quad_corner
    }
    for (const tc::QtArgs &a : p.lists)
      for (int t = 0; t < a.ntile; ++t) {
        const tc::QtTile &q = a.tiles[t];
        row(2, q.mt, q.nt, q.arow, q.brow, q.nb, q.swap);
      }
    *count = k;
    *launches = (p.persist ? 1 : 0) + (int)p.lists.size();
    return HQCGB_OK;
  } catch (const Error &e) {
    set_error(e.msg);
    return e.status;
  }
}
