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

// Generic K-major operand description: element (row, k) at ptr[row * ld + k];
// rows >= rows_valid and k >= k_end read as zero.  Every row start and every
// 4-element chunk is 16-byte aligned (ld % 4 == 0, k offsets multiples of 4).
struct Operand {
  const float *ptr;
  long long ld;
  int rows_valid;
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
        const float *ga = arow[j] + (kin ? kk : 0);
        const float *gb = brow[j] + (kin ? kk : 0);
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

// M[p][q] = scale * sum_chunks P  (+ mirror for sym; + transpose-add for GGA)
__global__ void k_tc_quad_reduce(const double *__restrict__ P, int nchunk, int mtiles, int ntiles,
                                 int nao, int sym, int add_transpose, double scale,
                                 double *__restrict__ M) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nao * nao) return;
  int p = idx / nao, q = idx % nao;
  auto get = [&](int pp, int qq) {
    if (sym && (qq / kN) < (pp / kM)) { int t = pp; pp = qq; qq = t; }
    int tm = pp / kM, tn = qq / kN, r = pp % kM, cc = qq % kN;
    double s = 0;
    for (int k = 0; k < nchunk; ++k)
      s += P[((((long long)k * mtiles + tm) * ntiles + tn) * kM + r) * kN + cc];
    return s;
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
// K-major operands D[p][q] (row stride ldk) and phiT[g][q] (grid-major copy,
// row stride ldk).  Epilogue: part[mt][g] = sum_{p in tile} phi_p(g) X_p(g)
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

// phiT[g][q] (row stride ldk) = phi[q][g] for g < N, q < nao; zero for q in [nao, ldk)
__global__ void k_transpose_phi(const float *__restrict__ phi, int nao, long long N, long long ld,
                                float *__restrict__ phiT, int ldk) {
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
  for (int r = ty; r < 32; r += 8) {
    long long g = g0 + r;
    int q = q0 + tx;
    if (g < N && q < ldk) phiT[g * ldk + q] = t[tx][r];
  }
}

// ---------------------------------------------------------------------------
// Orbital density: psi_k(g) = sum_p phi_p(g) Y_pk with Y = C_occ sqrt(f)
// (npsi <= kPsiMaxN columns, zero-padded), rho(g) = sum_k psi_k(g)^2 and,
// for GGA, grad rho = 2 sum_k psi_k grad psi_k.  This is the density
// sum_pq D_pq phi_p phi_q of D = C diag(f) C^T (hqc/pbc/solver.py:566-577,
// 690) at npsi / n_ao of the GEMM work.
//
// Tiles: M = 128 grid points (A = rows of the grid-major phiT / dphiT,
// K-major), N = npsi (B = the TF32 hi/lo pieces of Y^T, pre-split in global
// memory), K = AO in stages of 32.  Persistent CTAs loop over grid tiles;
// stage s of a CTA is (tile, component, K block).
//
// Accuracy.  The tensor core's FP32 accumulation truncates, so sums of many
// MMAs drift low (about half an ulp per instruction).  Every group of DR
// K blocks therefore accumulates in its own TMEM slot -- the large hi*hi
// products and the 2^-11 smaller cross products in separate accumulators --
// and the epilogue warps drain each group into compensated (TwoSum) FP32
// sums held in registers for the current component; psi = S + C is rounded
// to FP32 once (unbiased) and rho, grad rho are summed in FP64.
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
        if (comp == 0) tma_load_2d(base, &tmA, kb * kStageK, g0, &P.loaded[slot]);
        else tma_load_2d(base, &tmD, kb * kStageK, (int)((comp - 1) * a.N) + g0, &P.loaded[slot]);
        tma_load_2d(base + (uint32_t)kPsiAPieces, &tmY, kb * kStageK, 0, &P.loaded[slot]);
        tma_load_2d(base + (uint32_t)(kPsiAPieces + kPsiBPiece), &tmY, kb * kStageK, NPSI,
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
      double rho = 0, gr[3] = {0, 0, 0};
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
#pragma unroll
          for (int k = 0; k < NPSI; ++k) {
            const float v = sv[k] + cv[k];
            if (comp == 0) {
              p0[k] = v;
              rho += (double)v * (double)v;
            } else {
              gr[comp - 1] += (double)p0[k] * (double)v;
            }
            if (a.psi_out && g < a.N) a.psi_out[(long long)(comp * NPSI + k) * a.N + g] = v;
          }
        }
      }
      if (ok && g < a.N) {
        a.rho[g] = rho;
        if (a.ncomp > 1)
          for (int c = 0; c < 3; ++c) a.grho[(long long)c * a.N + g] = 2.0 * gr[c];
      }
    }
  } else if (lane == 0) {
    const uint32_t idesc = idesc_tf32(kM, NPSI);
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
              const uint32_t Bh = base + (uint32_t)kPsiAPieces, Bl = Bh + (uint32_t)kPsiBPiece;
#pragma unroll
              for (int ks = 0; ks < kStageK / 8; ++ks) {
                const uint32_t off = ks * 32;
                const int acc = (kb > g0 || ks > 0) ? 1 : 0;
                mma_tf32(dsmall, sdesc(Al + off), sdesc(Bh + off), idesc, acc);
                mma_tf32(dsmall, sdesc(Ah + off), sdesc(Bl + off), idesc, 1);
                mma_tf32(dbig, sdesc(Ah + off), sdesc(Bh + off), idesc, acc);
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
        tma_load_2d(base, ah, x, T.arow, &P.full[slot]);
        tma_load_2d(base + (uint32_t)kTile, al, x, T.arow, &P.full[slot]);
        for (int q = 0; q < nbox; ++q) {
          const uint32_t off = (uint32_t)(q * bbox * 128);
          tma_load_2d(base + 2u * (uint32_t)kTile + off, bh, x, T.brow + q * bbox, &P.full[slot]);
          tma_load_2d(base + 3u * (uint32_t)kTile + off, bl, x, T.brow + q * bbox, &P.full[slot]);
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
#pragma unroll
            for (int ks = 0; ks < kStageK / 8; ++ks) {
              const uint32_t off = ks * 32;
              mma_tf32(tmem_d, sdesc(Al + off), sdesc(Bh + off), idesc, (first && ks == 0) ? 0 : 1);
              mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bl + off), idesc, 1);
              mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bh + off), idesc, 1);
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
// each computes one full 128 x 128 destination tile over all of it.  The
// CTAs of a group stream the same 128-row blocks at about the same pace, so
// a block that one of them brings in from DRAM is still in L2 when the others
// ask for it.  The compensated sums stay in TMEM / registers over the whole
// slice; one FP64 partial tile per CTA is written at the end and the reduce
// adds the groups.
//
// The products with the partial block (at most 16 AOs, MMA N = 16) ride
// along, at most two per CTA, spread over the tiles of a group so that each
// CTA does about the same work:
//   kind 0  tile (m, last)    = A block m x narrow B box;
//   kind 1  tile (last, n)    = (B block n x narrow A box)^T, stored transposed;
//   kind 2  tile (last, last) = narrow A box x narrow B box.  The MMA reads a
//           128-row A window that starts at the narrow A box; its rows past
//           16 are other operand data of the same stage, and the TMEM lanes
//           they produce are never read.
// TMEM (512 columns): two slots of 128 + 16 + 16 accumulator columns, the
// main tile's TwoSum sums S (128 columns) and the narrow products' sums and
// carries (2 x 16 each); the carries C of the main tile live in the
// registers of eight drain warps (two per TMEM lane group, 64 main columns
// each).
// ---------------------------------------------------------------------------
constexpr int kQpDrainWarps = 8;
constexpr int kQpMmaWarp = kQpDrainWarps;
constexpr int kQpTmaWarp = kQpMmaWarp + 1;
constexpr int kQpThreads = (kQpTmaWarp + 1) * 32;
constexpr uint32_t kQpSlot = kN + 32;           // main + two narrow accumulators
constexpr uint32_t kQpColS = 2 * kQpSlot;       // main-tile sums S (128 columns)
constexpr uint32_t kQpColXS = kQpColS + kN;     // narrow sums S (2 x 16)
constexpr uint32_t kQpColXC = kQpColXS + 32;    // narrow carries C (2 x 16), ends at 512
constexpr int kQpTmemCols = 512;
constexpr uint32_t kQpNarrow = 16 * 128;        // one 16-row piece of a narrow box
// Stage layout: narrow A hi, lo | narrow B hi, lo | A hi | A lo | B hi | B lo.
// The narrow pieces come first so that the 16 KB window of a kind-2 product
// (from either narrow A piece) ends inside the stage.
constexpr uint32_t kQpOffNA = 0, kQpOffNB = 2 * kQpNarrow, kQpOffMain = 4 * kQpNarrow;
constexpr size_t kQpStageBytes = 4 * kQpNarrow + 4 * kTile;
constexpr size_t kQpSmem = kQtRing * kQpStageBytes + 1024;
constexpr int kQpMaxFull = 6;  // full AO blocks handled by the persistent form
constexpr int kQpMaxTiles = kQpMaxFull * kQpMaxFull;

struct QpTile {
  int mt, nt;          // the full destination tile
  int nx;              // narrow products carried (0..2)
  int kind[2];         // 0, 1 or 2 (above)
  int xmt[2], xnt[2];  // their destination tiles
  int loadA, loadB;    // narrow A / B boxes loaded with every stage
};

struct QpArgs {
  QpTile tiles[kQpMaxTiles];
  int ntile, groups;
  int xrow;  // first AO row of the narrow block
  long long N;
  int drain, mtiles, ntiles;
  double *partial;  // [groups][mtiles][ntiles][128][128]
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
static_assert(kTmemCols <= 512 && kQpColXC + 32 == (uint32_t)kQpTmemCols && kQpTmemCols <= 512,
              "TMEM column layout");
static_assert(sizeof(QtArgs) + 8 * sizeof(CUtensorMap) <= 4096 &&
                  sizeof(QpArgs) + 8 * sizeof(CUtensorMap) <= 4096,
              "kernel parameters above 4 KB");
static_assert(kPsiRowsPerThread * kPsiProducers == kM * 8, "splitter rows per thread");
static_assert(kQpOffNA + kQpNarrow + kTile <= kQpStageBytes, "kind-2 window leaves the stage");

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
      const uint32_t bytes = 4u * (uint32_t)kTile + (uint32_t)(T.loadA + T.loadB) * 2u * kQpNarrow;
      for (int st = 0; st < nstages; ++st) {
        const int slot = st % kQtRing, use = st / kQtRing;
        if (ok && use > 0 && !mbar_wait(&P.empty[slot], (unsigned)((use - 1) & 1), a.err, 41)) ok = false;
        if (!ok) break;
        const int x = (int)((s0 + st) * kStageK);
        const uint32_t base = smem_u32(sm + slot * kQpStageBytes), mb = base + kQpOffMain;
        mbar_expect_tx(&P.full[slot], bytes);
        tma_load_2d(mb, &mAh, x, T.mt * kM, &P.full[slot]);
        tma_load_2d(mb + (uint32_t)kTile, &mAl, x, T.mt * kM, &P.full[slot]);
        tma_load_2d(mb + 2u * (uint32_t)kTile, &mBh, x, T.nt * kN, &P.full[slot]);
        tma_load_2d(mb + 3u * (uint32_t)kTile, &mBl, x, T.nt * kN, &P.full[slot]);
        if (T.loadA) {
          tma_load_2d(base + kQpOffNA, &mAh16, x, a.xrow, &P.full[slot]);
          tma_load_2d(base + kQpOffNA + kQpNarrow, &mAl16, x, a.xrow, &P.full[slot]);
        }
        if (T.loadB) {
          tma_load_2d(base + kQpOffNB, &mBh16, x, a.xrow, &P.full[slot]);
          tma_load_2d(base + kQpOffNB + kQpNarrow, &mBl16, x, a.xrow, &P.full[slot]);
        }
      }
    }
  } else if (warp == kQpMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(kM, kN), idesc16 = idesc_tf32(kM, 16);
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
            const uint32_t base = smem_u32(sm + slot * kQpStageBytes), mb = base + kQpOffMain;
            const uint32_t Ah = mb, Al = mb + (uint32_t)kTile, Bh = mb + 2u * (uint32_t)kTile,
                           Bl = mb + 3u * (uint32_t)kTile;
            const uint32_t nAh = base + kQpOffNA, nAl = nAh + kQpNarrow, nBh = base + kQpOffNB,
                           nBl = nBh + kQpNarrow;
#pragma unroll
            for (int ks = 0; ks < kStageK / 8; ++ks) {
              const uint32_t off = ks * 32;
              const int acc = (first && ks == 0) ? 0 : 1;
              mma_tf32(tmem_d, sdesc(Al + off), sdesc(Bh + off), idesc, acc);
              mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bl + off), idesc, 1);
              mma_tf32(tmem_d, sdesc(Ah + off), sdesc(Bh + off), idesc, 1);
              for (int e = 0; e < T.nx; ++e) {
                const int kind = T.kind[e];
                // the 128-row side and the 16-row narrow box of this product
                const uint32_t Wh = kind == 0 ? Ah : (kind == 1 ? Bh : nAh);
                const uint32_t Wl = kind == 0 ? Al : (kind == 1 ? Bl : nAl);
                const uint32_t Nh = kind == 1 ? nAh : nBh, Nl = kind == 1 ? nAl : nBl;
                const uint32_t dx = tmem_d + (uint32_t)kN + (uint32_t)e * 16u;
                mma_tf32(dx, sdesc(Wl + off), sdesc(Nh + off), idesc16, acc);
                mma_tf32(dx, sdesc(Wh + off), sdesc(Nl + off), idesc16, 1);
                mma_tf32(dx, sdesc(Wh + off), sdesc(Nh + off), idesc16, 1);
              }
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
    // the warps of half h also own narrow product h (16 columns)
    const int h = warp >> 2;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    const int c0 = h * 64;
    const bool has_x = h < T.nx;
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
          const uint32_t xsa = P.tmem_base + lane_off + kQpColXS + (uint32_t)h * 16u,
                         xca = P.tmem_base + lane_off + kQpColXC + (uint32_t)h * 16u;
          uint32_t va[16], sa[16], ca[16];
          tmem_ld16_nowait(slot + kN + (uint32_t)h * 16u, va);
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
      if (ok)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          tile[(long long)row * kN + c0 + q * 16 + i] = (double)__uint_as_float(sr[i]) + (double)cm[q * 16 + i];
    }
    if (has_x) {
      uint32_t sr[16], cr[16];
      tmem_ld16_nowait(P.tmem_base + lane_off + kQpColXS + (uint32_t)h * 16u, sr);
      tmem_ld16_nowait(P.tmem_base + lane_off + kQpColXC + (uint32_t)h * 16u, cr);
      tmem_wait_ld();
      const int kind = T.kind[h];
      if (ok && (kind != 2 || row < 16)) {
        double *xt = a.partial + (((long long)g * a.mtiles + T.xmt[h]) * a.ntiles + T.xnt[h]) * tsz;
        if (kind != 1) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            xt[(long long)row * kN + i] = (double)__uint_as_float(sr[i]) + (double)__uint_as_float(cr[i]);
        } else {
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

// hi/lo TF32 pieces of Z = a w phi + b u . grad phi (u, dphi optional; w
// optional, = 1): inputs with row stride ldi, outputs [nao][ldo] with zeros
// in [N, ldo).  Grid (column blocks of 1024, rows); 4 columns per thread
// (ldi, ldo multiples of 4, 16-byte aligned rows).
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
  *reinterpret_cast<float4 *>(hi + (long long)p * ldo + g) = h;
  *reinterpret_cast<float4 *>(lo + (long long)p * ldo + g) = l;
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
  CUtensorMap tmA = tc::tensor_map_2d(phiT, ldk, N, tc::kM);
  CUtensorMap tmD = tc::tensor_map_2d(grho ? dphiT : phiT, ldk, grho ? 3 * N : N, tc::kM);
  CUtensorMap tmY = tc::tensor_map_2d(Yhl, ldk, 2LL * npsi, npsi);
  long long ntiles = ceil_div(N, tc::kM);
  int grid = (int)std::min<long long>(ntiles, nsm);
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
//  * persistent form (1..6 full blocks and a last block of at most 16 rows,
//    or none): k_tc_quad_persist runs the full tiles; the narrow products
//    (kind 0 (m, last), kind 1 (last, n) transposed, kind 2 the corner) are
//    spread over them, at most two per CTA:
//      non-symmetric: (m, last) on (m, m); (last, n) on ((n + 1) % nfull, n);
//      symmetric:     (m, last) on (m, m + 1) (or (m, m) for the last block);
//      the corner on the first tile carrying the fewest;
//    a shape where some CTA would carry three takes the tile-list form;
//  * tile-list form otherwise: every tile of the upper triangle (sym) or of
//    the whole square through k_tc_quad_tma, at most kQtMaxTiles per launch.
// A tile whose A-side block is the narrow one is computed transposed
// (swap = 1: A side from the B arrays), so the narrow block is always the
// MMA's N side, rounded up to a multiple of 16 rows.
struct QuadTilePlan {
  int nblk = 0, nb_last = 0;
  bool persist = false;
  tc::QpArgs f{};                 // persistent form: the full tiles and the narrow products they carry
  std::vector<tc::QtArgs> lists;  // k_tc_quad_tma launches, tile lists only
};

static bool plan_persist(int nao, bool sym, tc::QpArgs &f) {
  const int nblk = ceil_div(nao, tc::kM);
  const int last = nao - tc::kM * (nblk - 1);
  const bool narrow = last < tc::kM;
  const int nfull = narrow ? nblk - 1 : nblk;
  if ((narrow && last > 16) || nfull < 1 || nfull > tc::kQpMaxFull) return false;
  f = tc::QpArgs{};
  f.xrow = nfull * tc::kM;
  for (int mt = 0; mt < nfull; ++mt)
    for (int nt = 0; nt < nfull; ++nt) {
      if (sym && nt < mt) continue;
      tc::QpTile &t = f.tiles[f.ntile++];
      t.mt = mt;
      t.nt = nt;
    }
  if (!narrow) return true;
  auto find = [&f](int mt, int nt) {
    for (int i = 0; i < f.ntile; ++i)
      if (f.tiles[i].mt == mt && f.tiles[i].nt == nt) return i;
    return -1;
  };
  bool fits = true;
  auto add = [&](int i, int kind, int xmt, int xnt) {
    if (i < 0 || f.tiles[i].nx >= 2) {
      fits = false;
      return;
    }
    tc::QpTile &t = f.tiles[i];
    t.kind[t.nx] = kind;
    t.xmt[t.nx] = xmt;
    t.xnt[t.nx] = xnt;
    ++t.nx;
    if (kind != 0) t.loadA = 1;
    if (kind != 1) t.loadB = 1;
  };
  for (int m = 0; m < nfull && fits; ++m)
    add(sym && m + 1 < nfull ? find(m, m + 1) : find(m, m), 0, m, nfull);
  if (!sym)
    for (int n = 0; n < nfull && fits; ++n) add(find(nfull > 1 ? (n + 1) % nfull : n, n), 1, nfull, n);
  if (fits) {
    int best = 0;
    for (int i = 1; i < f.ntile; ++i)
      if (f.tiles[i].nx < f.tiles[best].nx) best = i;
    add(best, 2, nfull, nfull);
  }
  return fits;
}

static QuadTilePlan plan_quad_tiles(int nao, bool sym) {
  QuadTilePlan p;
  p.nblk = ceil_div(nao, tc::kM);
  const int last = nao - tc::kM * (p.nblk - 1);
  const bool narrow = last < tc::kM;
  p.nb_last = ceil_div(last, 16) * 16;
  if (plan_persist(nao, sym, p.f)) {
    p.persist = true;
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
// the whole launch (the autotuner's "quad_groups" when set), at most one
// slice per 64 stages and at most the chunk count the partial buffer holds.
static int quad_groups(int ntile, long long N) {
  int dev = 0, sms = 0;
  HQ_CUDA(cudaGetDevice(&dev));
  HQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  long long g = std::max(1, sms / std::max(1, ntile));
  const long long t = tune_get("quad_groups", 0);
  if (t > 0) g = t;
  g = std::min<long long>(g, std::max<long long>(1, ceil_div(N, (long long)tc::kStageK * 64)));
  g = std::min<long long>(g, ceil_div(N, (long long)tc_quad_chunk()));
  return (int)std::max<long long>(1, g);
}

// M = scale * sum_g A_p(g) B_q(g) (+ its transpose when add_transpose) from the
// pre-split pieces Ahl, Bhl [2][nao][ld] (hi rows, then lo rows); sym: M is
// symmetric (only tiles nt >= mt are computed; the reduce mirrors them).
void launch_tc_quad_split(const float *Ahl, const float *Bhl, int nao, long long N, long long ld,
                          bool sym, bool add_transpose, double scale, double *partial, double *M,
                          int *err, cudaStream_t st, int drain, int kchunk) {
  HQ_STAGE(ST_QUAD, st);
  HQ_REQUIRE(drain >= 1, "drain must be >= 1");
  if (kchunk <= 0) kchunk = tc_quad_chunk();
  HQ_REQUIRE(kchunk % tc::kStageK == 0, "K chunk must be a multiple of 32");
  HQ_REQUIRE(ld % 32 == 0 && ld >= N, "pre-split operands need a row stride that is a multiple of 32");
  HQ_REQUIRE(N <= (1LL << 31) - 64, "grid too large for 32-bit TMA coordinates");
  const QuadTilePlan plan = plan_quad_tiles(nao, sym);
  const int nblk = plan.nblk;
  const long long rows = nao;
  const float *Ah = Ahl, *Al = Ahl + (size_t)nao * ld, *Bh = Bhl, *Bl = Bhl + (size_t)nao * ld;
  CUtensorMap mAh = tc::tensor_map_2d_ext(Ah, ld, N, rows, tc::kM);
  CUtensorMap mAl = tc::tensor_map_2d_ext(Al, ld, N, rows, tc::kM);
  CUtensorMap mBh = tc::tensor_map_2d_ext(Bh, ld, N, rows, tc::kN);
  CUtensorMap mBl = tc::tensor_map_2d_ext(Bl, ld, N, rows, tc::kN);
  CUtensorMap mAh16 = tc::tensor_map_2d_ext(Ah, ld, N, rows, 16);
  CUtensorMap mAl16 = tc::tensor_map_2d_ext(Al, ld, N, rows, 16);
  CUtensorMap mBh16 = tc::tensor_map_2d_ext(Bh, ld, N, rows, 16);
  CUtensorMap mBl16 = tc::tensor_map_2d_ext(Bl, ld, N, rows, 16);
  int nparts = 0;  // partial tiles per destination tile
  if (plan.persist) {
    ensure_dyn_smem((const void *)tc::k_tc_quad_persist, tc::kQpSmem);
    tc::QpArgs f = plan.f;
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
  } else {
    ensure_dyn_smem((const void *)tc::k_tc_quad_tma, tc::kQtSmem);
    nparts = (int)ceil_div(N, (long long)kchunk);
    for (tc::QtArgs a : plan.lists) {
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
  tc::k_tc_quad_reduce<<<ceil_div((long long)nao * nao, 256), 256, 0, st>>>(
      partial, nparts, nblk, nblk, nao, sym ? 1 : 0, add_transpose ? 1 : 0, scale, M);
  HQ_LAUNCH_CHECK();
}

// hi/lo pieces of a w phi + b u . grad phi into out [2][nao][ldo]
void launch_split_operand(const float *phi, const float *dphi, const float *w, const float *u, int nao,
                          long long N, long long ldi, long long ldo, float a, float b, float *out,
                          cudaStream_t st) {
  HQ_STAGE(ST_SPLIT, st);
  HQ_REQUIRE(ldi % 4 == 0 && ldo % 4 == 0 && ldo >= N && ldi >= N, "split operand: bad row strides");
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
    launch_tc_quad_split(zhl, phihl, nao, N, ld, true, false, scale, partial, M, err, st, drain, (int)kc);
    return;
  }
  HQ_REQUIRE(dphi && u, "GGA quadrature needs dphi and u");
  launch_split_operand(phi, dphi, w, u, nao, N, ld, ld, 0.5f, dV, zhl, st);
  launch_tc_quad_split(zhl, phihl, nao, N, ld, false, true, scale, partial, M, err, st, drain, (int)kc);
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
  tc::k_transpose_phi<<<grid, 256, 0, st>>>(phi, nao, N, ld, phiT, ldk);
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
  a.D = tc::Operand{D32, ldk, nao};
  a.phiT = tc::Operand{phiT, ldk, (int)N};
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
    launch_tc_quad_split(zhl, phl, nao, N, ldo, true, false, 1.0, part, M, err, st, drain);
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
// persistent kernel, 1 a narrow product carried by one of its CTAs, 2 a tile
// of the tile-list kernel; (mt, nt) the destination tile, arow / brow the first AO
// row of the MMA's A / B side (swap = 1: A side from the B operand, stored
// transposed), nb the MMA N.  count = rows (at most cap are written);
// launches = quadrature kernel launches before the reduce.
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
      for (int t = 0; t < p.f.ntile; ++t) {
        const tc::QpTile &q = p.f.tiles[t];
        for (int x = 0; x < q.nx; ++x) {
          // the MMA's 128-row side: A block (kind 0), B block (kind 1, transposed), narrow A box (kind 2)
          const int arow = q.kind[x] == 0 ? q.mt * tc::kM : (q.kind[x] == 1 ? q.nt * tc::kN : p.f.xrow);
          row(1, q.xmt[x], q.xnt[x], arow, p.f.xrow, 16, q.kind[x] == 1 ? 1 : 0);
        }
      }
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
