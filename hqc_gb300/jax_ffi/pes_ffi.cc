// XLA FFI handler of the engine's energy + force evaluation, for JAX callers
// (jax.ffi.ffi_call).  The reference jits its closures (hqc/pbc/solver.py:
// 975-976, hqc/pbc/pes.py:152-153); this handler puts one call of the
// engine's batched PES into a jitted JAX program, on the stream XLA provides,
// writing into buffers XLA owns.
//
// Built only where jaxlib is installed (its headers give xla/ffi/api/ffi.h;
// see build.py in this folder) and linked against libhqcgb.so.
//
// Inputs:  xp_rs  [B, n, 3] f64 positions in rs units (the reference's xp),
//          xp_bohr [B, n, 3] f64 the same positions in Bohr.
// Attrs:   plan (int64, an hqcgb_plan* made with want_forces = 1), L_rs, rs,
//          kappa (f64), gmax (int64) -- make_pes's Ewald parameters.
// Results: energies [B, 5] (E, Ki, Vep, Vee in Hartree, Se), free [B]
//          (E - sigma S, Hartree), grad [B, n, 3] (d free / dR, Hartree/Bohr),
//          vpp [B] (Rydberg), vpp_grad [B, n, 3] (Rydberg per rs unit),
//          converged [B] int32.
//
// HqcgbPesKpt is the single-k-point form (pes_kpt, hqc/pbc/pes.py:88-98):
// one more input, kpts [B, 3] f64 in 1/Bohr, and `plan` an hqcgb_kplan*
// made with want_forces = 1; the same results.
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hqcgb.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

static ffi::Error EwaldAll(cudaStream_t stream, const double *xp_rs, int64_t B, int64_t n, double L_rs,
                           double rs, double kappa, int64_t gmax, double *vpp, double *vpp_grad) {
  for (int64_t b = 0; b < B; ++b) {
    const int st = hqcgb_ewald(xp_rs + b * n * 3, static_cast<int>(n), L_rs, rs, kappa, static_cast<int>(gmax),
                               vpp + b, vpp_grad + b * n * 3, stream);
    if (st != HQCGB_OK) {
      return ffi::Error(ffi::ErrorCode::kInternal, std::string("hqcgb_ewald: ") + hqcgb_last_error());
    }
  }
  return ffi::Error::Success();
}

static ffi::Error PesImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> xp_rs, ffi::Buffer<ffi::F64> xp_bohr,
                          ffi::ResultBuffer<ffi::F64> energies, ffi::ResultBuffer<ffi::F64> free_energy,
                          ffi::ResultBuffer<ffi::F64> grad, ffi::ResultBuffer<ffi::F64> vpp,
                          ffi::ResultBuffer<ffi::F64> vpp_grad, ffi::ResultBuffer<ffi::S32> converged,
                          int64_t plan, double L_rs, double rs, double kappa, int64_t gmax) {
  const auto dims = xp_rs.dimensions();
  if (dims.size() < 2 || dims.back() != 3) {
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "xp must have shape [..., n, 3]");
  }
  const int64_t n = dims[dims.size() - 2];
  int64_t B = 1;
  for (size_t d = 0; d + 2 < dims.size(); ++d) B *= dims[d];
  hqcgb_scf_out out{};
  out.energies = energies->typed_data();
  out.free_energy = free_energy->typed_data();
  out.converged = converged->typed_data();
  auto *p = reinterpret_cast<hqcgb_plan *>(plan);
  const int st =
      hqcgb_pes_batch(p, static_cast<int>(B), xp_bohr.typed_data(), &out, grad->typed_data(), stream);
  if (st > HQCGB_NOT_CONVERGED) {
    return ffi::Error(ffi::ErrorCode::kInternal, std::string("hqcgb_pes_batch: ") + hqcgb_last_error());
  }
  return EwaldAll(stream, xp_rs.typed_data(), B, n, L_rs, rs, kappa, gmax, vpp->typed_data(),
                  vpp_grad->typed_data());
}

static ffi::Error PesKptImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> xp_rs, ffi::Buffer<ffi::F64> xp_bohr,
                             ffi::Buffer<ffi::F64> kpts, ffi::ResultBuffer<ffi::F64> energies,
                             ffi::ResultBuffer<ffi::F64> free_energy, ffi::ResultBuffer<ffi::F64> grad,
                             ffi::ResultBuffer<ffi::F64> vpp, ffi::ResultBuffer<ffi::F64> vpp_grad,
                             ffi::ResultBuffer<ffi::S32> converged, int64_t plan, double L_rs, double rs,
                             double kappa, int64_t gmax) {
  const auto dims = xp_rs.dimensions();
  if (dims.size() < 2 || dims.back() != 3) {
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "xp must have shape [..., n, 3]");
  }
  const int64_t n = dims[dims.size() - 2];
  int64_t B = 1;
  for (size_t d = 0; d + 2 < dims.size(); ++d) B *= dims[d];
  if (static_cast<int64_t>(kpts.element_count()) != 3 * B) {
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "kpts must have shape [..., 3] matching xp");
  }
  // the engine takes the k-points on the host
  std::vector<double> k(3 * B);
  if (cudaMemcpyAsync(k.data(), kpts.typed_data(), sizeof(double) * 3 * B, cudaMemcpyDeviceToHost, stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess) {
    return ffi::Error(ffi::ErrorCode::kInternal, "copying the k-points to the host failed");
  }
  hqcgb_scf_out out{};
  out.energies = energies->typed_data();
  out.free_energy = free_energy->typed_data();
  out.converged = converged->typed_data();
  auto *p = reinterpret_cast<hqcgb_kplan *>(plan);
  const int st = hqcgb_pes_kpt_batch(p, static_cast<int>(B), xp_bohr.typed_data(), k.data(), &out,
                                     grad->typed_data(), stream);
  if (st > HQCGB_NOT_CONVERGED) {
    return ffi::Error(ffi::ErrorCode::kInternal, std::string("hqcgb_pes_kpt_batch: ") + hqcgb_last_error());
  }
  return EwaldAll(stream, xp_rs.typed_data(), B, n, L_rs, rs, kappa, gmax, vpp->typed_data(),
                  vpp_grad->typed_data());
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(HqcgbPesKpt, PesKptImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Attr<int64_t>("plan")
                                  .Attr<double>("L_rs")
                                  .Attr<double>("rs")
                                  .Attr<double>("kappa")
                                  .Attr<int64_t>("gmax"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(HqcgbPes, PesImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Attr<int64_t>("plan")
                                  .Attr<double>("L_rs")
                                  .Attr<double>("rs")
                                  .Attr<double>("kappa")
                                  .Attr<int64_t>("gmax"));
