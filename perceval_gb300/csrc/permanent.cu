// Batched permanents: host planner, preparation and reduction kernels, C ABI.
//
// Replaces xq.permanent_cx (perceval/backends/_naive.py:70-71).
//
// Flow of pcvl_permanent_batch:
//  1. perm_prepare: every row i of every matrix is scaled by an exact power of two
//     2^{e_i} so that its l1 norm lies in [2^{c-1}, 2^c), c = min(20, 120 / n); then
//     every |row sum| <= 2^c and every row-sum product stays inside the FP32 range.
//     The scaled matrix is stored as float-float pairs; sum_i e_i is kept.
//  2. one perm_bin_kernel<n> launch per distinct size n, each CTA handling a chunk
//     of Gray-code hi patterns of one matrix and writing one FP64 partial.
//  3. perm_reduce: per matrix, Neumaier-compensated FP64 sum of its partials, times
//     2^{1-n} (Glynn) or (-1)^n (Ryser), times 2^{-sum e_i}.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "permanent_kernel.cuh"
#include "runtime.cuh"

namespace pcvl {

struct PermDesc {
  int64_t base;   // first partial of the matrix
  int32_t items;  // number of partials
  int32_t n;
};

__global__ void perm_prepare(const double2* __restrict__ src, const int64_t* __restrict__ offs,
                             const int32_t* __restrict__ sizes, int32_t count, cdd* __restrict__ dst,
                             int32_t* __restrict__ exps) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= count) return;
  const int n = sizes[warp];
  const int64_t off = offs[warp];
  if (n == 0) {
    if (lane == 0) exps[warp] = 0;
    return;
  }
  const int c = min(20, 120 / n);
  int esum = 0;
  for (int i = lane; i < n; i += 32) {
    double l1 = 0.0;
    for (int j = 0; j < n; ++j) {
      const double2 v = src[off + (int64_t)i * n + j];
      l1 += hypot(v.x, v.y);
    }
    int e = 0;
    if (l1 > 0.0 && isfinite(l1)) {
      int x;
      frexp(l1, &x);
      e = c - x;
    }
    esum += e;
    for (int j = 0; j < n; ++j) {
      const double2 v = src[off + (int64_t)i * n + j];
      dst[off + (int64_t)i * n + j] = cdd_from(ldexp(v.x, e), ldexp(v.y, e));
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) esum += __shfl_down_sync(0xffffffffu, esum, d);
  if (lane == 0) exps[warp] = esum;
}

__device__ __forceinline__ void neumaier_add(double& s, double& comp, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x))
    comp += (s - t) + x;
  else
    comp += (x - t) + s;
  s = t;
}

__global__ void perm_reduce(const double2* __restrict__ partials, const PermDesc* __restrict__ descs,
                            const int32_t* __restrict__ exps, int32_t count, int32_t ryser,
                            double2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const PermDesc d = descs[i];
  if (d.n == 0) {
    out[i] = make_double2(1.0, 0.0);
    return;
  }
  double sr = 0, cr = 0, si = 0, ci = 0;
  for (int k = 0; k < d.items; ++k) {
    const double2 p = partials[d.base + k];
    neumaier_add(sr, cr, p.x);
    neumaier_add(si, ci, p.y);
  }
  double re = sr + cr, im = si + ci;
  int sh = -exps[i];
  if (!ryser) sh -= d.n - 1;
  re = ldexp(re, sh);
  im = ldexp(im, sh);
  if (ryser && (d.n & 1)) {
    re = -re;
    im = -im;
  }
  out[i] = make_double2(re, im);
}

static int launch_bin(int n, const PermBinArgs& a) {
  if (n <= 12) return launch_perm_bin_1_12(n, a);
  if (n <= 20) return launch_perm_bin_13_20(n, a);
  if (n <= 26) return launch_perm_bin_21_26(n, a);
  if (n <= 32) return launch_perm_bin_27_32(n, a);
  if (n <= 36) return launch_perm_bin_33_36(n, a);
  return launch_perm_bin_37_40(n, a);
}

// Chooses lo bits, patterns per thread and CTAs per matrix for one size bin.
struct BinPlan {
  int n = 0;
  int L = 0, Hbits = 0;
  int64_t P = 1, items_per_mat = 1;
  std::vector<int32_t> mids;
};

static void plan_bin(BinPlan& b, int ryser, int sms) {
  const int F = ryser ? b.n : b.n - 1;  // free bits
  b.L = std::min(7, std::max(0, F - 7));
  b.Hbits = F - b.L;
  const int64_t nhi = int64_t(1) << b.Hbits;
  const int64_t total_hi = nhi * (int64_t)b.mids.size();
  // aim for >= 8 CTAs per SM over the bin, never fewer patterns than one per thread
  int64_t P = total_hi / ((int64_t)kPermThreads * 8 * sms);
  P = std::max<int64_t>(1, std::min<int64_t>(P, std::max<int64_t>(1, nhi / kPermThreads)));
  b.P = P;
  b.items_per_mat = (nhi + kPermThreads * P - 1) / (kPermThreads * P);
}

}  // namespace pcvl

using namespace pcvl;

extern "C" int pcvl_permanent_batch(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                                    int32_t count, double* out_d, int32_t method, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  PCVL_CHECK(count >= 0, "count must be >= 0 (got %d)", count);
  if (count == 0) return PCVL_OK;
  PCVL_CHECK(mats_d && offsets_h && sizes_h && out_d, "null pointer argument");
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  const int ryser = method;

  int64_t total_elems = 0;
  std::vector<BinPlan> bins(kPermMaxN + 1);
  for (int i = 0; i < count; ++i) {
    const int n = sizes_h[i];
    PCVL_CHECK(n >= 0 && n <= kPermMaxN, "matrix %d: size %d outside [0, %d]", i, n, kPermMaxN);
    PCVL_CHECK(offsets_h[i] >= 0, "matrix %d: negative offset", i);
    total_elems = std::max<int64_t>(total_elems, offsets_h[i] + (int64_t)n * n);
    if (n > 0) bins[n].mids.push_back(i);
  }
  const int sms = num_sms();

  std::vector<PermDesc> descs(count);
  int64_t total_items = 0;
  for (int n = 1; n <= kPermMaxN; ++n) {
    BinPlan& b = bins[n];
    if (b.mids.empty()) continue;
    b.n = n;
    plan_bin(b, ryser, sms);
    for (size_t k = 0; k < b.mids.size(); ++k) {
      descs[b.mids[k]] = {total_items + (int64_t)k * b.items_per_mat, (int32_t)b.items_per_mat, n};
    }
    total_items += (int64_t)b.mids.size() * b.items_per_mat;
  }
  for (int i = 0; i < count; ++i)
    if (sizes_h[i] == 0) descs[i] = {0, 0, 0};

  // workspace: [prepared cdd][exps][offs][sizes][mids][descs][partials]
  size_t o_prep = 0;
  size_t o_exps = align_up(o_prep + (size_t)total_elems * sizeof(cdd), 256);
  size_t o_offs = align_up(o_exps + (size_t)count * 4, 256);
  size_t o_size = align_up(o_offs + (size_t)count * 8, 256);
  size_t o_mids = align_up(o_size + (size_t)count * 4, 256);
  size_t o_desc = align_up(o_mids + (size_t)count * 4, 256);
  size_t o_part = align_up(o_desc + (size_t)count * sizeof(PermDesc), 256);
  size_t total = align_up(o_part + (size_t)std::max<int64_t>(total_items, 1) * sizeof(double2), 256);
  void* ws = nullptr;
  PCVL_TRY(workspace(WS_PERM, total, &ws));
  unsigned char* base = (unsigned char*)ws;

  // one host blob for the small arrays -> one staged copy
  std::vector<unsigned char> blob(o_part - o_offs);
  memcpy(blob.data(), offsets_h, (size_t)count * 8);
  memcpy(blob.data() + (o_size - o_offs), sizes_h, (size_t)count * 4);
  int64_t mid_pos = 0;
  std::vector<int32_t> mids_all(count);
  for (int n = 1; n <= kPermMaxN; ++n)
    for (int32_t id : bins[n].mids) mids_all[mid_pos++] = id;
  memcpy(blob.data() + (o_mids - o_offs), mids_all.data(), (size_t)mid_pos * 4);
  memcpy(blob.data() + (o_desc - o_offs), descs.data(), (size_t)count * sizeof(PermDesc));
  PCVL_TRY(stage_h2d(blob.data(), blob.size(), base + o_offs, stream));

  cdd* prep = (cdd*)(base + o_prep);
  int32_t* exps_d = (int32_t*)(base + o_exps);
  const int64_t* offs_d = (const int64_t*)(base + o_offs);
  const int32_t* sizes_d = (const int32_t*)(base + o_size);
  int32_t* mids_d = (int32_t*)(base + o_mids);
  const PermDesc* descs_d = (const PermDesc*)(base + o_desc);
  double2* parts = (double2*)(base + o_part);

  {
    const int threads = 256;
    const int blocks = (int)(((int64_t)count * 32 + threads - 1) / threads);
    perm_prepare<<<blocks, threads, 0, stream>>>((const double2*)mats_d, offs_d, sizes_d, count, prep, exps_d);
    PCVL_CUDA(cudaGetLastError());
  }

  int64_t mid_off = 0;
  for (int n = 1; n <= kPermMaxN; ++n) {
    BinPlan& b = bins[n];
    if (b.mids.empty()) continue;
    PermBinArgs a;
    a.A = prep;
    a.offs = offs_d;
    a.mids = mids_d + mid_off;
    a.nmat = (int32_t)b.mids.size();
    a.L = b.L;
    a.Hbits = b.Hbits;
    a.P = b.P;
    a.items_per_mat = b.items_per_mat;
    a.ryser = ryser;
    a.partials = parts + descs[b.mids[0]].base;
    a.stream = stream;
    const int rc = launch_bin(n, a);
    if (rc != 0) {
      set_error("permanent kernel launch for n=%d failed: %s", n, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
    mid_off += (int64_t)b.mids.size();
  }

  perm_reduce<<<(count + 127) / 128, 128, 0, stream>>>(parts, descs_d, exps_d, count, ryser, (double2*)out_d);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

// ------------------------------------------------------------------ allocation-free variant
// pcvl_permanent_batch_noalloc: the same computation as pcvl_permanent_batch for callers
// that may not allocate device memory.  Its scratch (prepared matrices, descriptors, CTA
// partials) is one file-scope device array of fixed size, present on every device that
// loads the library until the process exits; descriptors travel from a static host buffer.
namespace pcvl {
namespace noalloc {

constexpr int64_t kMaxElems = int64_t(3) << 20;  // matrix elements per call (48 MiB as float-float)
constexpr int32_t kMaxCount = 16384;             // matrices per call
constexpr int64_t kMaxItems = int64_t(1) << 17;  // CTA partial sums per call (2 MiB)

constexpr size_t kPrep = 0;
constexpr size_t kExps = kPrep + (size_t)kMaxElems * sizeof(cdd);
constexpr size_t kOffs = kExps + (size_t)kMaxCount * 4;
constexpr size_t kSize = kOffs + (size_t)kMaxCount * 8;
constexpr size_t kMids = kSize + (size_t)kMaxCount * 4;
constexpr size_t kDesc = kMids + (size_t)kMaxCount * 4;
constexpr size_t kPart = kDesc + (size_t)kMaxCount * sizeof(PermDesc);
constexpr size_t kBytes = kPart + (size_t)kMaxItems * sizeof(double2);
static_assert(kExps % 256 == 0 && kOffs % 256 == 0 && kSize % 256 == 0 && kMids % 256 == 0 &&
                  kDesc % 256 == 0 && kPart % 256 == 0,
              "scratch regions stay 256-byte aligned");

constexpr int kMaxDevices = 64;
void* g_dev_ptr[kMaxDevices] = {};
unsigned char g_host_blob[kPart - kOffs];  // offsets, sizes, mids, descriptors of one call
std::mutex g_mu;

}  // namespace noalloc

// The scratch itself.  Host code must not use this name as an address: it only
// names a host-side stand-in, so kernels receive the address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_perm_scratch[noalloc::kBytes];

// Per-device set-up, once, with that device current: the device address of the scratch.
static int noalloc_scratch(unsigned char** ptr) {
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < noalloc::kMaxDevices, "device index %d out of range", dev);
  if (!noalloc::g_dev_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_perm_scratch);
    if (e != cudaSuccess || !p) {
      set_error("cudaGetSymbolAddress of the permanent scratch failed: %s", cudaGetErrorString(e));
      return PCVL_ERR_CUDA;
    }
    noalloc::g_dev_ptr[dev] = p;
  }
  *ptr = (unsigned char*)noalloc::g_dev_ptr[dev];
  return PCVL_OK;
}

}  // namespace pcvl

extern "C" int pcvl_permanent_batch_noalloc(const double* mats_d, const int64_t* offsets_h,
                                            const int32_t* sizes_h, int32_t count, double* out_d,
                                            int32_t method, void* stream_) {
  using namespace pcvl::noalloc;
  cudaStream_t stream = (cudaStream_t)stream_;
  PCVL_CHECK(count >= 0, "count must be >= 0 (got %d)", count);
  if (count == 0) return PCVL_OK;
  PCVL_CHECK(mats_d && offsets_h && sizes_h && out_d, "null pointer argument");
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK(count <= kMaxCount, "allocation-free permanents: %d matrices exceed the maximum of %d per call",
             count, kMaxCount);
  const int ryser = method;

  // size bins without heap memory: counts per size, then matrix ids grouped by size
  int32_t bin_count[kPermMaxN + 1] = {0};
  int64_t total_elems = 0;
  for (int i = 0; i < count; ++i) {
    const int n = sizes_h[i];
    PCVL_CHECK(n >= 0 && n <= kPermMaxN, "matrix %d: size %d outside [0, %d]", i, n, kPermMaxN);
    PCVL_CHECK(offsets_h[i] >= 0, "matrix %d: negative offset", i);
    total_elems = std::max<int64_t>(total_elems, offsets_h[i] + (int64_t)n * n);
    ++bin_count[n];
  }
  PCVL_CHECK(total_elems <= kMaxElems,
             "allocation-free permanents: the matrices span %lld elements, more than the maximum of %lld per call",
             (long long)total_elems, (long long)kMaxElems);

  const int sms = num_sms();
  int L[kPermMaxN + 1], Hb[kPermMaxN + 1];
  int64_t P[kPermMaxN + 1], ipm[kPermMaxN + 1], item_base[kPermMaxN + 1], mid_base[kPermMaxN + 1];
  int64_t total_items = 0, mids_so_far = 0;
  for (int n = 1; n <= kPermMaxN; ++n) {
    mid_base[n] = mids_so_far;
    item_base[n] = total_items;
    if (bin_count[n] == 0) continue;
    const int F = ryser ? n : n - 1;
    L[n] = std::min(7, std::max(0, F - 7));
    Hb[n] = F - L[n];
    const int64_t nhi = int64_t(1) << Hb[n];
    int64_t p = nhi * bin_count[n] / ((int64_t)kPermThreads * 8 * sms);
    p = std::max<int64_t>(1, std::min<int64_t>(p, std::max<int64_t>(1, nhi / kPermThreads)));
    P[n] = p;
    ipm[n] = (nhi + kPermThreads * p - 1) / (kPermThreads * p);
    total_items += bin_count[n] * ipm[n];
    mids_so_far += bin_count[n];
  }
  PCVL_CHECK(total_items <= kMaxItems,
             "allocation-free permanents: the batch needs %lld partial sums, more than the maximum of %lld per call",
             (long long)total_items, (long long)kMaxItems);

  std::lock_guard<std::mutex> lock(g_mu);
  unsigned char* scratch = nullptr;
  PCVL_TRY(noalloc_scratch(&scratch));

  // descriptors into the static host buffer (same layout as the device region [kOffs, kPart))
  int64_t* h_offs = (int64_t*)(g_host_blob + (kOffs - kOffs));
  int32_t* h_size = (int32_t*)(g_host_blob + (kSize - kOffs));
  int32_t* h_mids = (int32_t*)(g_host_blob + (kMids - kOffs));
  PermDesc* h_desc = (PermDesc*)(g_host_blob + (kDesc - kOffs));
  int64_t fill[kPermMaxN + 1];
  for (int n = 0; n <= kPermMaxN; ++n) fill[n] = 0;
  for (int i = 0; i < count; ++i) {
    const int n = sizes_h[i];
    h_offs[i] = offsets_h[i];
    h_size[i] = n;
    if (n == 0) {
      h_desc[i] = {0, 0, 0};
      continue;
    }
    const int64_t k = fill[n]++;
    h_mids[mid_base[n] + k] = i;
    h_desc[i] = {item_base[n] + k * ipm[n], (int32_t)ipm[n], n};
  }
  // pageable source: the call returns once the bytes are staged, so the buffer is reusable
  PCVL_CUDA(cudaMemcpyAsync(scratch + kOffs, g_host_blob, kPart - kOffs, cudaMemcpyHostToDevice, stream));

  cdd* prep = (cdd*)(scratch + kPrep);
  int32_t* exps_d = (int32_t*)(scratch + kExps);
  const int64_t* offs_d = (const int64_t*)(scratch + kOffs);
  const int32_t* sizes_d = (const int32_t*)(scratch + kSize);
  int32_t* mids_d = (int32_t*)(scratch + kMids);
  const PermDesc* descs_d = (const PermDesc*)(scratch + kDesc);
  double2* parts = (double2*)(scratch + kPart);
  {
    const int threads = 256;
    const int blocks = (int)(((int64_t)count * 32 + threads - 1) / threads);
    perm_prepare<<<blocks, threads, 0, stream>>>((const double2*)mats_d, offs_d, sizes_d, count, prep, exps_d);
    PCVL_CUDA(cudaGetLastError());
  }
  for (int n = 1; n <= kPermMaxN; ++n) {
    if (bin_count[n] == 0) continue;
    PermBinArgs a;
    a.A = prep;
    a.offs = offs_d;
    a.mids = mids_d + mid_base[n];
    a.nmat = bin_count[n];
    a.L = L[n];
    a.Hbits = Hb[n];
    a.P = P[n];
    a.items_per_mat = ipm[n];
    a.ryser = ryser;
    a.partials = parts + item_base[n];
    a.stream = stream;
    const int rc = launch_bin(n, a);
    if (rc != 0) {
      set_error("permanent kernel launch for n=%d failed: %s", n, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
  }
  perm_reduce<<<(count + 127) / 128, 128, 0, stream>>>(parts, descs_d, exps_d, count, ryser, (double2*)out_d);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}
