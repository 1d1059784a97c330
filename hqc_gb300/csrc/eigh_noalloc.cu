// hqcgb_eigh_noalloc: the FP64 symmetric eigensolver without any allocation.
//
// hqcgb_eigh allocates its scratch (a working copy of the matrix and the
// eigensolver's n x n work array) with cudaMallocAsync on every call.  Some
// callers cannot allocate device memory: code running inside a framework that
// owns all device memory (for instance an XLA custom call executing inside a
// jitted program, which must take every buffer from the framework's
// allocator), or latency-critical loops that must not risk the implicit
// synchronisation or failure of an allocation.  This entry point keeps its
// scratch in a file-scope __device__ array instead, so it never calls
// cudaMalloc / cudaFree or any allocating routine.  The caller still passes
// the input matrix and the output buffers.
//
// Limits and sharing:
//  * n <= HQCGB_EIGH_NOALLOC_MAX_N (320); larger n is rejected with
//    HQCGB_BAD_ARG before any device work.  The array holds
//    2 * 320 * 320 doubles + 64 doubles (about 1.6 MB); every GPU that loads
//    this library keeps it until the process exits.
//  * Every call on a device uses the same array and leaves the last call's
//    contents in it.  Calls whose device work overlaps (concurrent streams,
//    host threads) race on it and must be serialised by the caller.
//  * The first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before starting any stream capture.
//  * The call blocks the host: it synchronises the caller's stream to read
//    the solver's status word (once, and twice more on the Jacobi fallback).
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int kMaxN = HQCGB_EIGH_NOALLOC_MAX_N;
constexpr size_t kScratchDoubles = 2 * (size_t)kMaxN * kMaxN + 64;

// Device-side scratch.  In host code this name is only a stand-in for the
// symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_eigh_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};

double *scratch_on_current_device() {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    throw hqcgb::Error{HQCGB_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e)};
  if (dev < 0 || dev >= kMaxDevices)
    throw hqcgb::Error{HQCGB_BAD_ARG, "device index beyond the supported range"};
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_eigh_scratch);
    if (e != cudaSuccess || !p)
      throw hqcgb::Error{HQCGB_CUDA_ERROR,
                         std::string("cudaGetSymbolAddress(eigensolver scratch): ") +
                             cudaGetErrorString(e)};
    g_addr[dev] = static_cast<double *>(p);
  }
  return g_addr[dev];
}

int run(int n, const double *A, double *w, double *V, cudaStream_t st) {
  using namespace hqcgb;
  if (!A || !w || !V) throw Error{HQCGB_BAD_ARG, "null argument"};
  if (n < 1 || n > kMaxN)
    throw Error{HQCGB_BAD_ARG, "hqcgb_eigh_noalloc: n = " + std::to_string(n) +
                                   " outside 1.." + std::to_string(kMaxN)};
  double *s = scratch_on_current_device();
  double *Ac = s;                                         // working copy of A
  double *work = s + (size_t)kMaxN * kMaxN;               // n x n eigenvector work
  int *status = reinterpret_cast<int *>(s + 2 * (size_t)kMaxN * kMaxN);
  // The kernels overwrite everything they read except the status word,
  // which is cleared here so a stale value from an earlier call is never read.
  HQ_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
  HQ_CUDA(cudaMemcpyAsync(Ac, A, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  eigh_tql(n, 1, Ac, V, w, work, status, st);
  int hs = 0;
  HQ_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HQ_CUDA(cudaStreamSynchronize(st));
  if (hs < 0) {  // QL sweep limit: same Jacobi fallback as hqcgb_eigh
    HQ_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
    HQ_CUDA(cudaMemcpyAsync(Ac, A, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    jacobi_eigh(n, 1, Ac, V, w, work, status, st);
    HQ_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    HQ_CUDA(cudaStreamSynchronize(st));
    if (hs < 0) throw Error{HQCGB_EIG_FAIL, "eigensolver did not converge"};
  }
  return HQCGB_OK;
}

}  // namespace

extern "C" int hqcgb_eigh_noalloc(int n, const double *A, double *w, double *V, void *stream) {
  try {
    return run(n, A, w, V, (cudaStream_t)stream);
  } catch (const hqcgb::Error &e) {
    hqcgb::set_error(e.msg);
    return e.status;
  } catch (const std::exception &e) {
    hqcgb::set_error(e.what());
    return HQCGB_CUDA_ERROR;
  }
}
