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
cudaMemPool_t g_pool[kMaxDevices] = {};
std::mutex g_pool_mu;

int device_pool(int dev, cudaMemPool_t* pool) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    PCVL_CUDA(cudaMemPoolCreate(&p, &props));
    uint64_t keep = ~0ull;  // freed blocks stay in the pool for the next call
    PCVL_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pool[dev] = p;
  }
  *pool = g_pool[dev];
  return PCVL_OK;
}
}  // namespace

int scratch_alloc(size_t bytes, cudaStream_t stream, void** ptr) {
  *ptr = nullptr;
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < kMaxDevices, "device index %d out of range", dev);
  cudaMemPool_t pool = nullptr;
  PCVL_TRY(device_pool(dev, &pool));
  const size_t want = bytes < 4096 ? 4096 : bytes;
  cudaError_t e = cudaMallocFromPoolAsync(ptr, want, pool, stream);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    set_error("scratch allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PCVL_ERR_MEMORY : PCVL_ERR_CUDA;
  }
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

extern "C" const char* pcvl_version(void) { return "pcvl_gb300 0.3.0 sm_103a"; }

extern "C" int pcvl_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PCVL_ERR_ARG;
  strncpy(buf, pcvl::g_err, len - 1);
  buf[len - 1] = '\0';
  return PCVL_OK;
}

extern "C" int pcvl_release_workspace(void) {
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < pcvl::kMaxDevices, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(pcvl::g_pool_mu);
  PCVL_CUDA(cudaDeviceSynchronize());
  if (pcvl::g_pool[dev]) PCVL_CUDA(cudaMemPoolTrimTo(pcvl::g_pool[dev], 0));
  return PCVL_OK;
}
