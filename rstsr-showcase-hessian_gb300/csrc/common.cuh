// Shared helpers of libcphf: status handling, device buffers, launch accounting.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/cphf.h"

namespace cphf {

// Exception carrying a cphf_status; converted to a return code at the C ABI.
struct Error : std::runtime_error {
  cphf_status status;
  Error(cphf_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

inline void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    throw Error(CPHF_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
  }
  throw Error(CPHF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CPHF_CUDA(call) ::cphf::check_cuda((call), #call)

// Mirrors check_shape! (src/util/panic_handling.rs:36-58): a shape mismatch is an error.
#define CPHF_CHECK_SHAPE(cond, msg)                                   \
  do {                                                                \
    if (!(cond)) throw ::cphf::Error(CPHF_ERR_SHAPE, std::string(msg)); \
  } while (0)

#define CPHF_CHECK_ARG(cond, msg)                                   \
  do {                                                              \
    if (!(cond)) throw ::cphf::Error(CPHF_ERR_ARG, std::string(msg)); \
  } while (0)

// Bumped whenever a device buffer is (re)allocated or released, or a cached launch plan is
// rebuilt: a captured CUDA graph bakes in pointers and plan contents and is replayed only
// while the generation it was captured at is current.
extern std::atomic<int64_t> g_state_generation;
inline void bump_generation() { g_state_generation.fetch_add(1, std::memory_order_relaxed); }
inline int64_t state_generation() { return g_state_generation.load(std::memory_order_relaxed); }

// Owning device allocation; byte size tracked for cphf_ctx_device_bytes.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int64_t* counter = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      if (counter) *counter -= (int64_t)bytes;
      bump_generation();
    }
    p = nullptr;
    bytes = 0;
  }
  // Grow to at least n bytes (contents are not preserved when growing).
  void ensure(size_t n, int64_t* cnt) {
    if (n <= bytes && p) return;
    release();
    counter = cnt;
    if (n == 0) return;
    CPHF_CUDA(cudaMalloc(&p, n));
    bump_generation();
    bytes = n;
    if (counter) *counter += (int64_t)n;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Launch accounting: every kernel launch of the library goes through CPHF_LAUNCHED.
extern thread_local int64_t* g_launch_counter;
inline void count_launch(int64_t n = 1) {
  if (g_launch_counter) *g_launch_counter += n;
}

inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace cphf
