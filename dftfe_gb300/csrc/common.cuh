// Shared helpers for the CheFSI CUDA library: status handling, device buffers, launch
// geometry. One process drives one GB300 (152 SMs); grid sizes are multiples of the SM count
// where a kernel is grid-stride.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/chefsi.h"

namespace chefsi {

struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define CHEFSI_CUDA(call)                                                                 \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess)                                                                \
      throw ::chefsi::Error(CHEFSI_ERR_CUDA, std::string(#call " failed: ") +             \
                                                 cudaGetErrorString(_e) + " at " +        \
                                                 __FILE__ + ":" + std::to_string(__LINE__)); \
  } while (0)

// every kernel launch of the library is followed by CHEFSI_CHECK_LAUNCH, which also counts it
void count_launch();
#define CHEFSI_CHECK_LAUNCH()      \
  do {                             \
    ::chefsi::count_launch();      \
    CHEFSI_CUDA(cudaGetLastError()); \
  } while (0)

#define CHEFSI_REQUIRE(cond, msg)                                   \
  do {                                                              \
    if (!(cond)) throw ::chefsi::Error(CHEFSI_ERR_INVALID, (msg)); \
  } while (0)

// Host-side fault injection for tests (the failure is made on the host, never on the GPU):
// CHEFSI_FAULT_INJECT = "alloc" (device allocations fail), "not_spd" (the overlap handed to
// the Cholesky gets a negative diagonal), "nan" (operator inputs are treated as non-finite).
bool fault_injected(const char* what);

// Device allocation that honours the "alloc" fault hook.
void* dmalloc(size_t bytes);
void dfree(void* p);

template <typename T>
struct DeviceBuffer {
  T* ptr = nullptr;
  size_t n = 0;
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t count) { reset(count); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() { release(); }
  void reset(size_t count) {
    release();
    if (count) ptr = static_cast<T*>(dmalloc(count * sizeof(T)));
    n = count;
  }
  // grow-only reuse (workspace semantics)
  T* ensure(size_t count) {
    if (count > n) reset(count);
    return ptr;
  }
  void release() {
    if (ptr) dfree(ptr);
    ptr = nullptr;
    n = 0;
  }
};

constexpr int kNumSMs = 152;

inline int grid_for(int64_t n, int threads, int max_blocks = kNumSMs * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace chefsi
