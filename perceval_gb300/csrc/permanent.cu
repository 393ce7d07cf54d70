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
