// Owning device buffer and CUDA error checking for the host drivers.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

namespace lsg {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
// device memory exhausted (reported as LSG_ENOMEM)
struct CudaOutOfMemory : CudaError {
  using CudaError::CudaError;
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    const cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();  // not a sticky error: clear it so that later calls proceed
      p = nullptr;
      throw CudaOutOfMemory("cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes: out of device memory");
    }
    cuda_check(e, "cudaMalloc");
    n = count;
  }
  // grow-only allocation for work buffers whose size varies between calls
  void ensure(size_t count) {
    if (count > n) alloc(count);
  }
  void upload(const std::vector<T>& v, cudaStream_t s) {
    alloc(v.size());
    if (!v.empty()) cuda_check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
  size_t bytes() const { return n * sizeof(T); }
};

}  // namespace lsg
