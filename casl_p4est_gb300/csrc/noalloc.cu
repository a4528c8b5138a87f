// FP64 reinitialisation whose work vectors live in a fixed, file-scope device array instead of
// memory allocated by the call (lsg_reinitialize_device_noalloc in include/lsgpu.h).
//
// The allocating path (LevelSet::reinit_fp64) allocates phi_0, phi_np1, two second-derivative
// sets, the subcell distances and the status word per node on its first call and keeps them for
// the object's lifetime. This variant carves the same vectors out of g_reinit_scratch and runs the
// same kernels in the same order, so its results are identical to the allocating path's.
//
// Set-up: every call looks up the array's address on the level set's device (which the C ABI makes
// current for the call) with cudaGetSymbolAddress and checks the result. The lookup is cheap once the
// module is loaded and is never stale, even after the device's primary context was reset and made again.
// The first call on a device also loads this file's device code: make it before any stream capture.
// Nothing in the scratch must start at zero: every vector is written before it is read (status for
// every node; subcell distances only for the nodes whose status says they are read).
// There is one array per device: calls that overlap on the same device (other streams, other
// threads, other level-set objects) race on it and must be serialised by the caller.
#include <stdexcept>
#include <string>

#include "../../include/lsgpu.h"
#include "devbuf.hpp"
#include "kernels.h"

namespace lsg {

namespace {

static __device__ __align__(256) unsigned char g_reinit_scratch[LSG_NOALLOC_SCRATCH_BYTES];

// the array's device address on the current device (host code cannot use the symbol itself)
unsigned char* scratch_address() {
  void* p = nullptr;
  cuda_check(cudaGetSymbolAddress(&p, g_reinit_scratch), "cudaGetSymbolAddress(static reinitialisation scratch)");
  return static_cast<unsigned char*>(p);
}

constexpr size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// Carves consecutive 256-byte-aligned sub-arrays off the front of the scratch.
struct Carver {
  unsigned char* base;
  size_t used = 0;
  template <typename T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += round256(count * sizeof(T));
    return p;
  }
};

template <int D>
struct ReinitScratch {
  double *phi0, *phi1, *dd0, *ddc, *snear;
  uint16_t* status;
  size_t bytes;
  ReinitScratch(unsigned char* base, int64_t N) {
    Carver c{base};
    phi0 = c.take<double>((size_t)N);
    phi1 = c.take<double>((size_t)N);
    dd0 = c.take<double>((size_t)D * N);
    ddc = c.take<double>((size_t)D * N);
    snear = c.take<double>((size_t)2 * D * N);
    status = c.take<uint16_t>((size_t)N);
    bytes = c.used;
  }
};

}  // namespace

// reinitialize_within_range_of_phi_0 (src/my_p4est_level_set.cpp:290-557), FP64, the kernel
// sequence of LevelSet::reinit_fp64 over the static scratch. hi/lo are the widened phi_0 limits.
template <int D>
void reinit_fp64_static(const DTab64<D>& T, double zdt, double* phi, int os, int ot, double hi, double lo, int iters,
                        cudaStream_t stream) {
  const int64_t N = T.N;
  const size_t need = ReinitScratch<D>(nullptr, N).bytes;
  if (need > (size_t)LSG_NOALLOC_SCRATCH_BYTES)
    throw std::invalid_argument("lsg_reinitialize_device_noalloc: " + std::to_string(N) + " nodes in " + std::to_string(D) +
                                "D need " + std::to_string(need) + " bytes of scratch; the static scratch holds " +
                                std::to_string((size_t)LSG_NOALLOC_SCRATCH_BYTES) +
                                " bytes (LSG_NOALLOC_SCRATCH_BYTES); use lsg_reinitialize_device for this grid");
  const ReinitScratch<D> S(scratch_address(), N);
  if (N == 0) return;
  cuda_check(cudaMemcpyAsync(S.phi0, phi, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi_0");
  launch_dd64<D>(T, S.phi0, S.dd0, stream);
  launch_reinit_prep64<D>(T, S.phi0, S.dd0, zdt, lo, hi, os, S.status, S.snear, stream);
  for (int it = 0; it < iters; ++it) {
    launch_dd64<D>(T, phi, S.ddc, stream);
    launch_reinit_stage64<D>(T, os, S.status, S.snear, S.phi0, phi, S.ddc, S.phi1, nullptr, stream);
    if (ot > 1) {
      launch_dd64<D>(T, S.phi1, S.ddc, stream);
      launch_reinit_stage64<D>(T, os, S.status, S.snear, S.phi0, S.phi1, S.ddc, phi, phi, stream);
    } else {
      cuda_check(cudaMemcpyAsync(phi, S.phi1, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy phi_np1");
    }
  }
  cuda_check(cudaGetLastError(), "reinitialize (fp64, static scratch)");
}

template void reinit_fp64_static<2>(const DTab64<2>&, double, double*, int, int, double, double, int, cudaStream_t);
template void reinit_fp64_static<3>(const DTab64<3>&, double, double*, int, int, double, double, int, cudaStream_t);

}  // namespace lsg
