// Owning device buffer and CUDA error checking for the host drivers.
#pragma once
#include <cuda_runtime.h>

#include <stdint.h>

#include <map>
#include <mutex>
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
// a bounded device-side wait gave up (reported as LSG_ETIMEOUT)
struct DeviceTimeout : CudaError {
  using CudaError::CudaError;
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Makes `dev` the current device for its lifetime and restores the caller's device afterwards.
class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    cuda_check(cudaGetDevice(&prev_), "cudaGetDevice");
    if (dev != prev_) {
      cuda_check(cudaSetDevice(dev), "cudaSetDevice");
      switched_ = true;
    }
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = 0;
  bool switched_ = false;
};

inline int current_device() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  return dev;
}

// Device memory cache behind every DevBuf. A released block is kept for reuse instead of going back
// to the driver (cudaMalloc and cudaFree cost tens of microseconds each, and cudaFree waits for the
// whole device); a level set built for every new grid otherwise pays that for each of its tables.
// Reuse keeps cudaFree's guarantee: a block released since its device's last synchronisation is handed
// out again only after a cudaDeviceSynchronize of that device, so no kernel still in flight can see it
// change owner. The synchronisation count is kept per device: synchronising one GPU says nothing about
// the kernels in flight on another.
// Blocks are grouped by size class (eight classes per power of two, at most 12.5% unused).
class DeviceCache {
 public:
  static DeviceCache& get() {
    static DeviceCache* c = new DeviceCache();  // never destroyed: the driver frees everything at exit
    return *c;
  }
  static size_t size_class(size_t bytes) {
    if (bytes <= 4096) return 4096;
    int e = 63 - __builtin_clzll((unsigned long long)(bytes - 1));  // 2^e < bytes <= 2^(e+1)
    const size_t step = (size_t)1 << (e - 3);
    return (bytes + step - 1) / step * step;
  }
  // a block of size_class(bytes) on the current device; nullptr when the device is out of memory
  void* take(size_t bytes, int& dev) {
    const size_t cls = size_class(bytes);
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    {
      std::lock_guard<std::mutex> g(mu_);
      auto it = free_.find(Key{dev, cls});
      if (it != free_.end() && !it->second.empty()) {
        Block b = it->second.back();
        it->second.pop_back();
        cached_ -= cls;
        if (b.epoch == epoch_[dev]) {  // released since this device's last synchronisation
          cuda_check(cudaDeviceSynchronize(), "device synchronisation before reuse");
          ++epoch_[dev];
        }
        return b.p;
      }
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, cls);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();  // not a sticky error: clear it so that later calls proceed
      trim();
      e = cudaMalloc(&p, cls);
      if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return nullptr;
      }
    }
    cuda_check(e, "cudaMalloc");
    return p;
  }
  void give(void* p, size_t bytes, int dev) {
    const size_t cls = size_class(bytes);
    {
      std::lock_guard<std::mutex> g(mu_);
      if (cls <= kMaxBlock && cached_ + cls <= kMaxCached) {
        free_[Key{dev, cls}].push_back(Block{p, epoch_[dev]});
        cached_ += cls;
        return;
      }
    }
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != dev) {
      cudaSetDevice(dev);
      cudaFree(p);
      cudaSetDevice(cur);
    } else {
      cudaFree(p);
    }
  }
  // return every cached block to the driver (each device synchronised before its blocks are freed)
  void trim() {
    std::lock_guard<std::mutex> g(mu_);
    if (cached_ == 0) return;
    int cur = 0;
    cudaGetDevice(&cur);
    int synced = -1;
    for (auto& kv : free_) {  // ordered by device
      if (kv.second.empty()) continue;
      const int dev = kv.first.dev;
      if (dev != synced) {
        cudaSetDevice(dev);
        cudaDeviceSynchronize();
        ++epoch_[dev];
        synced = dev;
      }
      for (const Block& b : kv.second) cudaFree(b.p);
    }
    cudaSetDevice(cur);
    free_.clear();
    cached_ = 0;
  }
  size_t cached_bytes() {
    std::lock_guard<std::mutex> g(mu_);
    return cached_;
  }

 private:
  static constexpr size_t kMaxBlock = (size_t)4 << 30;    // larger blocks go straight back
  static constexpr size_t kMaxCached = (size_t)16 << 30;  // total kept
  struct Key {
    int dev;
    size_t cls;
    bool operator<(const Key& o) const { return dev != o.dev ? dev < o.dev : cls < o.cls; }
  };
  struct Block {
    void* p;
    uint64_t epoch;  // its device's synchronisation count at release
  };
  std::mutex mu_;
  std::map<Key, std::vector<Block>> free_;
  size_t cached_ = 0;
  std::map<int, uint64_t> epoch_;  // synchronisations per device
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int dev = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) DeviceCache::get().give(p, n * sizeof(T), dev);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    p = static_cast<T*>(DeviceCache::get().take(count * sizeof(T), dev));
    if (!p) throw CudaOutOfMemory("cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes: out of device memory");
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
