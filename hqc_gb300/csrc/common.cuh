// Shared helpers of the hqcgb engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <cstdio>
#include <cmath>

#include "../../include/hqcgb.h"

namespace hqcgb {

void set_error(const std::string &msg);
// Run-time tuning knobs (hqcgb_tune_set): the value set for `name`, or dflt.
long long tune_get(const char *name, long long dflt);
void count_launch(long long k = 1);
// How many batch workers of this host thread's batch share the GPU (1 outside
// a concurrent batch): kernels that hold one CTA per SM for their whole run
// (the persistent quadrature) take a correspondingly smaller grid.
int gpu_share();
void set_gpu_share(int workers);
// Raise the dynamic shared-memory limit of kernel `func` on the current
// device to at least `bytes` (never lowers it); callable from concurrent
// host threads.
void ensure_dyn_smem(const void *func, size_t bytes);

// Per-stage device timing (CUDA events on the launching stream), enabled by
// hqcgb_profile(1).  Stage names are listed in plan.cu (kStageNames).
enum Stage { ST_GTO = 0, ST_PHI, ST_DENSITY, ST_QUAD, ST_FFT, ST_XC, ST_JACOBI, ST_GEMM_SMALL,
             ST_OVERLAP, ST_FORCE_GRID, ST_EXCHANGE, ST_EWALD, ST_OTHER, ST_PSI, ST_SPLIT, ST_COUNT };
void stage_mark(int stage, cudaStream_t st, bool begin);
struct StageScope {
  int s;
  cudaStream_t st;
  StageScope(int s_, cudaStream_t st_) : s(s_), st(st_) { stage_mark(s, st, true); }
  ~StageScope() { stage_mark(s, st, false); }
};
#define HQ_STAGE(stage, stream) ::hqcgb::StageScope _hq_scope_##__LINE__(stage, stream)

struct Error {
  int status;
  std::string msg;
};

#define HQ_CUDA(call)                                                               \
  do {                                                                              \
    cudaError_t _e = (call);                                                        \
    if (_e != cudaSuccess)                                                          \
      throw ::hqcgb::Error{HQCGB_CUDA_ERROR, std::string(#call) + ": " +            \
                                                cudaGetErrorString(_e)};            \
  } while (0)

#define HQ_LAUNCH_CHECK()                                                           \
  do {                                                                              \
    ::hqcgb::count_launch();                                                        \
    cudaError_t _e = cudaGetLastError();                                            \
    if (_e != cudaSuccess)                                                          \
      throw ::hqcgb::Error{HQCGB_CUDA_ERROR,                                        \
                           std::string("launch in ") + __func__ + ": " +             \
                               cudaGetErrorString(_e)};                             \
  } while (0)

#define HQ_REQUIRE(cond, msg)                                                       \
  do {                                                                              \
    if (!(cond)) throw ::hqcgb::Error{HQCGB_BAD_ARG, msg};                          \
  } while (0)

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Stream-ordered scratch memory, released (stream-ordered) when the scope
// ends -- also when a call in between throws.
class StreamBuf {
 public:
  StreamBuf(size_t bytes, cudaStream_t st) : st_(st) { HQ_CUDA(cudaMallocAsync(&p_, bytes, st_)); }
  ~StreamBuf() {
    if (p_) cudaFreeAsync(p_, st_);
  }
  StreamBuf(const StreamBuf &) = delete;
  StreamBuf &operator=(const StreamBuf &) = delete;
  template <typename T>
  T *as(size_t byte_offset = 0) const {
    return reinterpret_cast<T *>(static_cast<char *>(p_) + byte_offset);
  }

 private:
  void *p_ = nullptr;
  cudaStream_t st_;
};

constexpr int kMaxGrid = 255;        // points per axis handled by the direct DFT passes
constexpr int kMaxNao = 1024;        // AOs per configuration

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
template <typename T>
__device__ inline T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block, returned to every thread. blockDim.x multiple of 32;
// every thread of the block must call it.
template <typename T>
__device__ inline T block_sum(T v, T *sh /* >= 32 */) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = v;
  __syncthreads();
  v = sh[0];
  __syncthreads();
  return v;
}

// Maximum over the block, returned to every thread (same contract).
template <typename T>
__device__ inline T block_max(T v, T *sh /* >= 32 */) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
    v = (lane < nw) ? sh[lane] : sh[0];
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[0] = v;
  }
  __syncthreads();
  v = sh[0];
  __syncthreads();
  return v;
}

}  // namespace hqcgb
