// Error reporting, version and workspace cache of the C ABI.
#include <cstring>
#include <mutex>

#include "runtime.cuh"

namespace pcvl {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

namespace {
constexpr int kMaxDevices = 64;
struct Buf {
  void* ptr = nullptr;
  size_t bytes = 0;
};
Buf g_ws[kMaxDevices][WS_SLOTS];
std::mutex g_ws_mu;
}  // namespace

int workspace(int slot, size_t bytes, void** ptr) {
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < kMaxDevices && slot >= 0 && slot < WS_SLOTS, "bad workspace slot");
  std::lock_guard<std::mutex> lock(g_ws_mu);
  Buf& b = g_ws[dev][slot];
  if (b.bytes < bytes) {
    if (b.ptr) {
      // the old buffer may still be read by work queued on any stream
      PCVL_CUDA(cudaDeviceSynchronize());
      PCVL_CUDA(cudaFree(b.ptr));
      b.ptr = nullptr;
      b.bytes = 0;
    }
    size_t want = bytes < 4096 ? 4096 : bytes;
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
      b.ptr = nullptr;
      set_error("workspace allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
      return PCVL_ERR_MEMORY;
    }
    b.bytes = want;
  }
  *ptr = b.ptr;
  return PCVL_OK;
}

namespace {
struct Staging {
  void* host = nullptr;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
  bool pending = false;
};
Staging g_stage[kMaxDevices];
std::mutex g_stage_mu;
}  // namespace

int stage_h2d(const void* src, size_t bytes, void* dst_d, cudaStream_t stream) {
  if (bytes == 0) return PCVL_OK;
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < kMaxDevices, "device index out of range");
  std::lock_guard<std::mutex> lock(g_stage_mu);
  Staging& st = g_stage[dev];
  if (!st.done) PCVL_CUDA(cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming));
  // the previous copy out of the staging buffer must finish before it is rewritten
  if (st.pending) PCVL_CUDA(cudaEventSynchronize(st.done));
  st.pending = false;
  if (st.bytes < bytes) {
    if (st.host) PCVL_CUDA(cudaFreeHost(st.host));
    st.host = nullptr;
    st.bytes = 0;
    size_t want = bytes < 65536 ? 65536 : bytes;
    cudaError_t e = cudaMallocHost(&st.host, want);
    if (e != cudaSuccess) {
      st.host = nullptr;
      set_error("pinned staging allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
      return PCVL_ERR_MEMORY;
    }
    st.bytes = want;
  }
  memcpy(st.host, src, bytes);
  PCVL_CUDA(cudaMemcpyAsync(dst_d, st.host, bytes, cudaMemcpyHostToDevice, stream));
  PCVL_CUDA(cudaEventRecord(st.done, stream));
  st.pending = true;
  return PCVL_OK;
}

}  // namespace pcvl

extern "C" const char* pcvl_version(void) { return "pcvl_gb300 0.1.0 sm_103a"; }

extern "C" int pcvl_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PCVL_ERR_ARG;
  strncpy(buf, pcvl::g_err, len - 1);
  buf[len - 1] = '\0';
  return PCVL_OK;
}

extern "C" int pcvl_release_workspace(void) {
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(pcvl::g_ws_mu);
  PCVL_CUDA(cudaDeviceSynchronize());
  for (int s = 0; s < pcvl::WS_SLOTS; ++s) {
    auto& b = pcvl::g_ws[dev][s];
    if (b.ptr) PCVL_CUDA(cudaFree(b.ptr));
    b.ptr = nullptr;
    b.bytes = 0;
  }
  return PCVL_OK;
}
