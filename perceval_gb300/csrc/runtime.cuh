// Host-side runtime shared by the ABI entry points: per-thread error text, CUDA
// status checks and a per-device workspace cache.
#pragma once
#include <cstdarg>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/pcvl_gb300.h"

namespace pcvl {

void set_error(const char* fmt, ...);

// Returns PCVL_ERR_CUDA (with the call's text in the error message) when `expr`
// does not return cudaSuccess.
#define PCVL_CUDA(expr)                                                               \
  do {                                                                                \
    cudaError_t _e = (expr);                                                          \
    if (_e != cudaSuccess) {                                                          \
      ::pcvl::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, \
                        __LINE__);                                                    \
      return PCVL_ERR_CUDA;                                                           \
    }                                                                                 \
  } while (0)

#define PCVL_CHECK(cond, ...)        \
  do {                               \
    if (!(cond)) {                   \
      ::pcvl::set_error(__VA_ARGS__); \
      return PCVL_ERR_ARG;           \
    }                                \
  } while (0)

#define PCVL_TRY(expr)          \
  do {                          \
    int _s = (expr);            \
    if (_s != PCVL_OK) return _s; \
  } while (0)

// Scratch of one call, stream-ordered: taken from the library's memory pool of the
// current device on `stream` and handed back on the same stream after the work queued
// by the call (ScratchGuard does both), so calls on different streams or host threads
// never share scratch.  The pool keeps freed memory for reuse (release threshold at
// the maximum) until pcvl_release_workspace() trims it.
int scratch_alloc(size_t bytes, cudaStream_t stream, void** ptr);

class ScratchGuard {
 public:
  explicit ScratchGuard(cudaStream_t s) : s_(s) {}
  ScratchGuard(const ScratchGuard&) = delete;
  ScratchGuard& operator=(const ScratchGuard&) = delete;
  int alloc(size_t bytes, void** ptr) {
    const int rc = scratch_alloc(bytes, s_, &p_);
    *ptr = p_;
    return rc;
  }
  ~ScratchGuard() {
    if (p_) cudaFreeAsync(p_, s_);
  }

 private:
  cudaStream_t s_;
  void* p_ = nullptr;
};

// Copies `bytes` of host memory to device memory on `stream` through a pinned
// staging buffer (kept per device); the host buffer may be reused on return.
int stage_h2d(const void* src, size_t bytes, void* dst_d, cudaStream_t stream);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

inline int num_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace pcvl
