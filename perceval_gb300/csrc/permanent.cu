// Batched permanents: host planner, preparation and reduction kernels, C ABI.
//
// Replaces xq.permanent_cx (perceval/backends/_naive.py:70-71).
//
// Flow of pcvl_permanent_batch:
//  1. perm_prepare: every row i of every matrix is scaled by an exact power of two
//     2^{e_i} so that its l1 norm lies in [2^{c-1}, 2^c), c = min(20, 120 / n); then
//     every |row sum| <= 2^c and every row-sum product stays inside the FP32 range
//     (and far inside the FP64 range).  The scaled matrix is stored as 64-bit fixed
//     point (FP64), double2 (FP64 with FP64 row sums) or float-float pairs; sum_i e_i
//     is kept.
//  2. one bin launch per distinct size n (perm_bin_fx<n>, perm_bin_f64<n> or
//     perm_bin_kernel<n>), each CTA handling a chunk of hi sign patterns of one matrix
//     and writing one FP64 partial.
//  3. perm_reduce: per matrix, Neumaier-compensated FP64 sum of its partials, times
//     2^{1-n} (Glynn) or (-1)^n (Ryser), times 2^{-sum e_i}.
#include <algorithm>
#include <type_traits>
#include <atomic>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "permanent_kernel.cuh"
#include "runtime.cuh"

namespace pcvl {

struct PermDesc {
  int64_t base;   // first partial of the matrix
  int32_t items;  // number of partials
  int32_t n;
};

__device__ __forceinline__ void store_prepared(cdd* dst, double re, double im, int) { *dst = cdd_from(re, im); }
__device__ __forceinline__ void store_prepared(double2* dst, double re, double im, int) {
  *dst = make_double2(re, im);
}
// fixed point with F fraction bits (the exact-row-sum FP64 kernel): |value| < 2^c, F = 62 - c
__device__ __forceinline__ void store_prepared(longlong2* dst, double re, double im, int F) {
  *dst = make_longlong2(__double2ll_rn(ldexp(re, F)), __double2ll_rn(ldexp(im, F)));
}

template <typename E>
__global__ void perm_prepare(const double2* __restrict__ src, const int64_t* __restrict__ offs,
                             const int32_t* __restrict__ sizes, int32_t count, E* __restrict__ dst,
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
    // Fixed point (the FP64 default): |every row sum| <= l1 must stay below 2^62 in the
    // block-floating products, so l1 is nudged up by far more than its rounding error and
    // the elements' roundings (a row whose l1 lies within 2^-40 below a power of two is
    // scaled one binade lower).
    if constexpr (std::is_same<E, longlong2>::value) l1 *= 1.0 + 0x1p-40;
    int e = 0;
    if (l1 > 0.0 && isfinite(l1)) {
      int x;
      frexp(l1, &x);
      e = c - x;
    }
    esum += e;
    for (int j = 0; j < n; ++j) {
      const double2 v = src[off + (int64_t)i * n + j];
      store_prepared(&dst[off + (int64_t)i * n + j], ldexp(v.x, e), ldexp(v.y, e), 62 - c);
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

static int launch_bin(int n, const PermBinArgs& a, PermNode* node = nullptr) {
  if (n <= 12) return launch_perm_bin_1_12(n, a, node);
  if (n <= 20) return launch_perm_bin_13_20(n, a, node);
  if (n <= 26) return launch_perm_bin_21_26(n, a, node);
  if (n <= 32) return launch_perm_bin_27_32(n, a, node);
  if (n <= 36) return launch_perm_bin_33_36(n, a, node);
  return launch_perm_bin_37_40(n, a, node);
}

// Tuning table: per arithmetic (0 float-float, 1 FP64, 2 FP64 with FP64 row sums), method
// and size, the lo bits and the target CTAs per SM of a bin, packed as (L + 1) | ctas << 8
// (0 in a field: the built-in choice).  Written by pcvl_perm_set_tuning (the autotuner),
// read without locks by every launch.
static std::atomic<uint32_t> g_tune[3][2][kPermMaxN + 1];

static int prec_slot(int prec) { return prec == kPrecFP64 ? 1 : prec == kPrecFP64Dadd ? 2 : 0; }

// prepare kernel of an arithmetic (prepared elements: fixed-point longlong2 for FP64,
// double2 for FP64 with FP64 row sums, cdd for float-float)
static void* prepare_func(int prec) {
  if (prec == kPrecFP64) return reinterpret_cast<void*>(perm_prepare<longlong2>);
  if (prec == kPrecFP64Dadd) return reinterpret_cast<void*>(perm_prepare<double2>);
  return reinterpret_cast<void*>(perm_prepare<cdd>);
}

static void launch_prepare(int prec, unsigned blocks, cudaStream_t stream, const double2* src, const int64_t* offs,
                           const int32_t* sizes, int32_t count, void* prep, int32_t* exps) {
  if (prec == kPrecFP64)
    perm_prepare<longlong2><<<blocks, 256, 0, stream>>>(src, offs, sizes, count, (longlong2*)prep, exps);
  else if (prec == kPrecFP64Dadd)
    perm_prepare<double2><<<blocks, 256, 0, stream>>>(src, offs, sizes, count, (double2*)prep, exps);
  else
    perm_prepare<cdd><<<blocks, 256, 0, stream>>>(src, offs, sizes, count, (cdd*)prep, exps);
}

constexpr int kDefaultCtasPerSm = 8;
constexpr size_t kMaxPermSmem = 227 * 1024;

static int default_lo_bits(int F) { return std::min(7, std::max(0, F - 7)); }

// Launch shape of one size bin: lo bits, hi bits, patterns per thread, CTAs per matrix.
struct BinShape {
  int L, Hbits;
  int64_t P, items_per_mat;
};

static BinShape bin_shape(int n, int ryser, int prec, int64_t nmat, int sms) {
  const uint32_t t = g_tune[prec_slot(prec)][ryser][n].load(std::memory_order_relaxed);
  const int F = ryser ? n : n - 1;  // free bits
  const int tl = (int)(t & 0xffu) - 1;
  const int tc = (int)((t >> 8) & 0xffu);
  BinShape s;
  s.L = tl >= 0 ? std::min(tl, F) : default_lo_bits(F);
  s.Hbits = F - s.L;
  const int ctas = tc > 0 ? tc : kDefaultCtasPerSm;
  const int64_t nhi = int64_t(1) << s.Hbits;
  // aim for >= ctas CTAs per SM over the bin, never fewer patterns than one per thread
  int64_t P = nhi * nmat / ((int64_t)kPermThreads * ctas * sms);
  const int64_t units = std::max<int64_t>(1, nhi / kPermThreads);  // patterns per thread of one whole matrix
  P = std::max<int64_t>(1, std::min<int64_t>(P, units));
  // Equal CTAs: split each matrix into `items` near-equal parts; then add parts until the
  // CTAs spread over the SMs within 3% (every SM ends with the same count, or the
  // busiest SM has at most 3% more work than the average).  Without this, 471 matrices
  // of 64 units with P = 49 ran as one 49-unit and one 15-unit CTA per matrix and the
  // bin reached 0.7 of its rate.
  // Each pass lowers P below the smallest P of the current part count, so the count
  // grows by at least one per pass; the loop ends by the time nmat * items reaches
  // about 33 CTAs per SM.
  for (;;) {
    const int64_t items = (units + P - 1) / P;
    P = (units + items - 1) / items;
    const int64_t c = nmat * items, per_sm = (c + sms - 1) / sms;
    if (P == 1 || 100 * c >= 97 * per_sm * sms) break;
    --P;
  }
  s.P = P;
  s.items_per_mat = (nhi + kPermThreads * P - 1) / (kPermThreads * P);
  return s;
}

struct BinPlan {
  int n = 0;
  int L = 0, Hbits = 0;
  int64_t P = 1, items_per_mat = 1;
  std::vector<int32_t> mids;
};

static void plan_bin(BinPlan& b, int ryser, int prec, int sms) {
  const BinShape s = bin_shape(b.n, ryser, prec, (int64_t)b.mids.size(), sms);
  b.L = s.L;
  b.Hbits = s.Hbits;
  b.P = s.P;
  b.items_per_mat = s.items_per_mat;
}

// Device layout of one batch: [prepared elements][exps][offs][sizes][mids][descs][partials];
// the small arrays travel as one host blob covering [offs, partials).
struct BatchLayout {
  std::vector<BinPlan> bins;  // indexed by n; empty bins have no mids
  std::vector<PermDesc> descs;
  int64_t total_elems = 0, total_items = 0;
  size_t o_prep = 0, o_exps = 0, o_offs = 0, o_size = 0, o_mids = 0, o_desc = 0, o_part = 0, total = 0;
  std::vector<unsigned char> blob;
};

// The prepare kernel writes each scaled matrix over the caller's offsets, so two
// matrices may share elements only as identical entries (same offset and size).  One
// linear pass accepts the usual packed, ascending layout; otherwise `order` (count
// entries of scratch) is sorted by offset.
static int check_no_overlap(const int64_t* offs, const int32_t* sizes, int32_t count, int32_t* order) {
  bool sorted = true;
  int64_t end = 0;
  for (int i = 0; i < count && sorted; ++i) {
    if (sizes[i] == 0) continue;
    if (offs[i] < end) sorted = false;
    end = offs[i] + (int64_t)sizes[i] * sizes[i];
  }
  if (sorted) return PCVL_OK;
  int32_t k = 0;
  for (int i = 0; i < count; ++i)
    if (sizes[i] > 0) order[k++] = i;
  std::sort(order, order + k, [&](int32_t a, int32_t b) {
    return offs[a] != offs[b] ? offs[a] < offs[b] : sizes[a] < sizes[b];
  });
  for (int32_t q = 1; q < k; ++q) {
    const int32_t a = order[q - 1], b = order[q];
    if (offs[a] == offs[b] && sizes[a] == sizes[b]) continue;
    PCVL_CHECK(offs[b] >= offs[a] + (int64_t)sizes[a] * sizes[a],
               "matrices %d and %d overlap in mats (offsets %lld and %lld): matrices may share elements only as "
               "identical entries (same offset and size)",
               a, b, (long long)offs[a], (long long)offs[b]);
  }
  return PCVL_OK;
}

static int make_layout(const int64_t* offsets_h, const int32_t* sizes_h, int32_t count, int ryser, int prec,
                       BatchLayout& L) {
  L.bins.assign(kPermMaxN + 1, BinPlan());
  for (int i = 0; i < count; ++i) {
    const int n = sizes_h[i];
    PCVL_CHECK(n >= 0 && n <= kPermMaxN, "matrix %d: size %d outside [0, %d]", i, n, kPermMaxN);
    PCVL_CHECK(offsets_h[i] >= 0, "matrix %d: negative offset", i);
    L.total_elems = std::max<int64_t>(L.total_elems, offsets_h[i] + (int64_t)n * n);
    if (n > 0) L.bins[n].mids.push_back(i);
  }
  {
    std::vector<int32_t> order(count);
    PCVL_TRY(check_no_overlap(offsets_h, sizes_h, count, order.data()));
  }
  const int sms = num_sms();
  L.descs.assign(count, PermDesc{0, 0, 0});
  for (int n = 1; n <= kPermMaxN; ++n) {
    BinPlan& b = L.bins[n];
    if (b.mids.empty()) continue;
    b.n = n;
    plan_bin(b, ryser, prec, sms);
    for (size_t k = 0; k < b.mids.size(); ++k)
      L.descs[b.mids[k]] = {L.total_items + (int64_t)k * b.items_per_mat, (int32_t)b.items_per_mat, n};
    L.total_items += (int64_t)b.mids.size() * b.items_per_mat;
  }
  L.o_prep = 0;
  L.o_exps = align_up(L.o_prep + (size_t)L.total_elems * sizeof(double2), 256);
  L.o_offs = align_up(L.o_exps + (size_t)count * 4, 256);
  L.o_size = align_up(L.o_offs + (size_t)count * 8, 256);
  L.o_mids = align_up(L.o_size + (size_t)count * 4, 256);
  L.o_desc = align_up(L.o_mids + (size_t)count * 4, 256);
  L.o_part = align_up(L.o_desc + (size_t)count * sizeof(PermDesc), 256);
  L.total = align_up(L.o_part + (size_t)std::max<int64_t>(L.total_items, 1) * sizeof(double2), 256);
  L.blob.assign(L.o_part - L.o_offs, 0);
  memcpy(L.blob.data(), offsets_h, (size_t)count * 8);
  memcpy(L.blob.data() + (L.o_size - L.o_offs), sizes_h, (size_t)count * 4);
  std::vector<int32_t> mids_all;
  mids_all.reserve(count);
  for (int n = 1; n <= kPermMaxN; ++n)
    for (int32_t id : L.bins[n].mids) mids_all.push_back(id);
  if (!mids_all.empty()) memcpy(L.blob.data() + (L.o_mids - L.o_offs), mids_all.data(), mids_all.size() * 4);
  memcpy(L.blob.data() + (L.o_desc - L.o_offs), L.descs.data(), (size_t)count * sizeof(PermDesc));
  return PCVL_OK;
}

// Bin kernel arguments of a layout placed at device address base.
static PermBinArgs bin_args(const BatchLayout& L, unsigned char* base, int n, int64_t mid_off, int ryser, int prec,
                            cudaStream_t stream) {
  const BinPlan& b = L.bins[n];
  PermBinArgs a;
  a.A = base + L.o_prep;
  a.offs = (const int64_t*)(base + L.o_offs);
  a.mids = (const int32_t*)(base + L.o_mids) + mid_off;
  a.nmat = (int32_t)b.mids.size();
  a.L = b.L;
  a.Hbits = b.Hbits;
  a.P = b.P;
  a.items_per_mat = b.items_per_mat;
  a.ryser = ryser;
  a.prec = prec;
  a.partials = (double2*)(base + L.o_part) + L.descs[b.mids[0]].base;
  a.stream = stream;
  return a;
}

}  // namespace pcvl

using namespace pcvl;

#define PCVL_CHECK_PERM_PREC(p)                                                                           \
  PCVL_CHECK((p) == PCVL_PREC_FP64 || (p) == PCVL_PREC_FP64_DADD || (p) == PCVL_PREC_FLOAT_FLOAT,          \
             "precision must be %d (FP64), %d (FP64 with FP64 row sums) or %d (float-float), got %d",       \
             PCVL_PREC_FP64, PCVL_PREC_FP64_DADD, PCVL_PREC_FLOAT_FLOAT, (p))

extern "C" int pcvl_permanent_batch(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                                    int32_t count, double* out_d, int32_t method, int32_t precision, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  PCVL_CHECK(count >= 0, "count must be >= 0 (got %d)", count);
  if (count == 0) return PCVL_OK;
  PCVL_CHECK(mats_d && offsets_h && sizes_h && out_d, "null pointer argument");
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK_PERM_PREC(precision);
  const int ryser = method;
  BatchLayout L;
  PCVL_TRY(make_layout(offsets_h, sizes_h, count, ryser, precision, L));
  ScratchGuard scratch(stream);
  void* ws = nullptr;
  PCVL_TRY(scratch.alloc(L.total, &ws));
  unsigned char* base = (unsigned char*)ws;
  PCVL_TRY(stage_h2d(L.blob.data(), L.blob.size(), base + L.o_offs, stream));

  int32_t* exps_d = (int32_t*)(base + L.o_exps);
  const int64_t* offs_d = (const int64_t*)(base + L.o_offs);
  const int32_t* sizes_d = (const int32_t*)(base + L.o_size);
  const PermDesc* descs_d = (const PermDesc*)(base + L.o_desc);
  double2* parts = (double2*)(base + L.o_part);
  {
    const unsigned blocks = (unsigned)(((int64_t)count * 32 + 255) / 256);
    launch_prepare(precision, blocks, stream, (const double2*)mats_d, offs_d, sizes_d, count, base + L.o_prep, exps_d);
    PCVL_CUDA(cudaGetLastError());
  }
  int64_t mid_off = 0;
  for (int n = 1; n <= kPermMaxN; ++n) {
    if (L.bins[n].mids.empty()) continue;
    const PermBinArgs a = bin_args(L, base, n, mid_off, ryser, precision, stream);
    const int rc = launch_bin(n, a);
    if (rc != 0) {
      set_error("permanent kernel launch for n=%d failed: %s", n, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
    mid_off += (int64_t)L.bins[n].mids.size();
  }
  perm_reduce<<<(count + 127) / 128, 128, 0, stream>>>(parts, descs_d, exps_d, count, ryser, (double2*)out_d);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

// ------------------------------------------------------------------ tuning
extern "C" int pcvl_perm_set_tuning(int32_t method, int32_t precision, int32_t n, int32_t lo_bits,
                                    int32_t ctas_per_sm) {
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK_PERM_PREC(precision);
  PCVL_CHECK(n >= 1 && n <= kPermMaxN, "n=%d outside [1, %d]", n, kPermMaxN);
  PCVL_CHECK(lo_bits >= -1 && lo_bits <= 12, "lo_bits=%d outside [-1, 12]", lo_bits);
  PCVL_CHECK(ctas_per_sm >= 0 && ctas_per_sm <= 64, "ctas_per_sm=%d outside [0, 64]", ctas_per_sm);
  if (lo_bits >= 0) {
    const int F = method ? n : n - 1;
    const int l = std::min(lo_bits, F);
    const size_t smem = (size_t)(n * n + (1 << l) * n) * sizeof(double2);
    PCVL_CHECK(smem <= kMaxPermSmem, "n=%d with %d lo bits needs %zu bytes of shared memory (max %zu)", n, l, smem,
               kMaxPermSmem);
  }
  g_tune[prec_slot(precision)][method][n].store((uint32_t)(lo_bits + 1) | ((uint32_t)ctas_per_sm << 8),
                                                std::memory_order_relaxed);
  return PCVL_OK;
}

extern "C" int pcvl_perm_get_tuning(int32_t method, int32_t precision, int32_t n, int32_t* lo_bits,
                                    int32_t* ctas_per_sm) {
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK_PERM_PREC(precision);
  PCVL_CHECK(n >= 1 && n <= kPermMaxN, "n=%d outside [1, %d]", n, kPermMaxN);
  PCVL_CHECK(lo_bits && ctas_per_sm, "null pointer argument");
  const uint32_t t = g_tune[prec_slot(precision)][method][n].load(std::memory_order_relaxed);
  const int F = method ? n : n - 1;
  const int tl = (int)(t & 0xffu) - 1;
  const int tc = (int)((t >> 8) & 0xffu);
  *lo_bits = tl >= 0 ? std::min(tl, F) : default_lo_bits(F);
  *ctas_per_sm = tc > 0 ? tc : kDefaultCtasPerSm;
  return PCVL_OK;
}

// ------------------------------------------------------------------ plans (CUDA graphs)
// A plan fixes the sizes and offsets of a batch.  Its device buffers hold the prepared
// matrices, descriptors and partials; the launch sequence is one CUDA graph: prepare,
// then every size bin as an independent branch (bins run concurrently), then reduce.
// Executing again only updates the input and output pointers of the first and last
// nodes and relaunches the graph.
struct pcvl_perm_plan {
  int device = 0, count = 0, ryser = 0, prec = 0;
  size_t bytes = 0;
  unsigned char* dev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t prep_node = nullptr, red_node = nullptr;
  unsigned prep_blocks = 0, red_blocks = 0;
  // arguments of the prepare and reduce kernels (src and out change per call)
  const double2* src = nullptr;
  const int64_t* offs_d = nullptr;
  const int32_t* sizes_d = nullptr;
  void* prep = nullptr;
  int32_t* exps_d = nullptr;
  double2* parts = nullptr;
  const PermDesc* descs_d = nullptr;
  double2* out = nullptr;
};

namespace {

void destroy_perm_plan(pcvl_perm_plan* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->dev) cudaFree(p->dev);
  delete p;
}

cudaKernelNodeParams prep_params(pcvl_perm_plan* p, void** args) {
  args[0] = &p->src;
  args[1] = &p->offs_d;
  args[2] = &p->sizes_d;
  args[3] = &p->count;
  args[4] = &p->prep;
  args[5] = &p->exps_d;
  cudaKernelNodeParams kp{};
  kp.func = prepare_func(p->prec);
  kp.gridDim = dim3(p->prep_blocks);
  kp.blockDim = dim3(256);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  return kp;
}

cudaKernelNodeParams red_params(pcvl_perm_plan* p, void** args) {
  args[0] = &p->parts;
  args[1] = &p->descs_d;
  args[2] = &p->exps_d;
  args[3] = &p->count;
  args[4] = &p->ryser;
  args[5] = &p->out;
  cudaKernelNodeParams kp{};
  kp.func = reinterpret_cast<void*>(perm_reduce);
  kp.gridDim = dim3(p->red_blocks);
  kp.blockDim = dim3(128);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  return kp;
}

}  // namespace

extern "C" int pcvl_perm_plan_create(pcvl_perm_plan** plan, const int64_t* offsets_h, const int32_t* sizes_h,
                                     int32_t count, int32_t method, int32_t precision) {
  PCVL_CHECK(plan, "null plan pointer");
  *plan = nullptr;
  PCVL_CHECK(offsets_h && sizes_h, "null pointer argument");
  PCVL_CHECK(count >= 1, "a plan needs at least one matrix (got %d)", count);
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK_PERM_PREC(precision);
  BatchLayout L;
  PCVL_TRY(make_layout(offsets_h, sizes_h, count, method, precision, L));
  pcvl_perm_plan* p = new (std::nothrow) pcvl_perm_plan();
  PCVL_CHECK(p, "out of host memory");
  p->count = count;
  p->ryser = method;
  p->prec = precision;
  p->bytes = L.total;
  cudaError_t e = cudaGetDevice(&p->device);
  if (e == cudaSuccess) e = cudaMalloc(&p->dev, L.total);
  if (e != cudaSuccess) {
    destroy_perm_plan(p);
    set_error("permanent plan: device allocation of %zu bytes failed: %s", L.total, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PCVL_ERR_MEMORY : PCVL_ERR_CUDA;
  }
  e = cudaMemcpy(p->dev + L.o_offs, L.blob.data(), L.blob.size(), cudaMemcpyHostToDevice);
  p->offs_d = (const int64_t*)(p->dev + L.o_offs);
  p->sizes_d = (const int32_t*)(p->dev + L.o_size);
  p->prep = p->dev + L.o_prep;
  p->exps_d = (int32_t*)(p->dev + L.o_exps);
  p->parts = (double2*)(p->dev + L.o_part);
  p->descs_d = (const PermDesc*)(p->dev + L.o_desc);
  p->prep_blocks = (unsigned)(((int64_t)count * 32 + 255) / 256);
  p->red_blocks = (unsigned)((count + 127) / 128);
  if (e == cudaSuccess) e = cudaGraphCreate(&p->graph, 0);
  void* pargs[6];
  void* rargs[6];
  if (e == cudaSuccess) {
    const cudaKernelNodeParams kp = prep_params(p, pargs);
    e = cudaGraphAddKernelNode(&p->prep_node, p->graph, nullptr, 0, &kp);
  }
  std::vector<cudaGraphNode_t> bin_nodes;
  int64_t mid_off = 0;
  for (int n = 1; n <= kPermMaxN && e == cudaSuccess; ++n) {
    if (L.bins[n].mids.empty()) continue;
    PermBinArgs a = bin_args(L, p->dev, n, mid_off, method, precision, nullptr);
    PermNode nd{};
    const int rc = launch_bin(n, a, &nd);
    if (rc != 0) {
      e = (cudaError_t)rc;
      break;
    }
    void* args[1] = {&a};
    cudaKernelNodeParams kp{};
    kp.func = nd.func;
    kp.gridDim = dim3(nd.grid);
    kp.blockDim = dim3(kPermThreads);
    kp.sharedMemBytes = (unsigned)nd.smem;
    kp.kernelParams = args;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddKernelNode(&node, p->graph, &p->prep_node, 1, &kp);
    bin_nodes.push_back(node);
    mid_off += (int64_t)L.bins[n].mids.size();
  }
  if (e == cudaSuccess) {
    const cudaKernelNodeParams kp = red_params(p, rargs);
    if (bin_nodes.empty())
      e = cudaGraphAddKernelNode(&p->red_node, p->graph, &p->prep_node, 1, &kp);
    else
      e = cudaGraphAddKernelNode(&p->red_node, p->graph, bin_nodes.data(), bin_nodes.size(), &kp);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  if (e != cudaSuccess) {
    destroy_perm_plan(p);
    set_error("permanent plan: graph construction failed: %s", cudaGetErrorString(e));
    return PCVL_ERR_CUDA;
  }
  *plan = p;
  return PCVL_OK;
}

extern "C" int pcvl_perm_plan_execute(pcvl_perm_plan* p, const double* mats_d, double* out_d, void* stream_) {
  PCVL_CHECK(p && mats_d && out_d, "null pointer argument");
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev == p->device, "the plan belongs to device %d, the current device is %d", p->device, dev);
  void* args[6];
  if ((const double2*)mats_d != p->src) {
    p->src = (const double2*)mats_d;
    const cudaKernelNodeParams kp = prep_params(p, args);
    PCVL_CUDA(cudaGraphExecKernelNodeSetParams(p->exec, p->prep_node, &kp));
  }
  if ((double2*)out_d != p->out) {
    p->out = (double2*)out_d;
    const cudaKernelNodeParams kp = red_params(p, args);
    PCVL_CUDA(cudaGraphExecKernelNodeSetParams(p->exec, p->red_node, &kp));
  }
  PCVL_CUDA(cudaGraphLaunch(p->exec, (cudaStream_t)stream_));
  return PCVL_OK;
}

extern "C" int pcvl_perm_plan_bytes(const pcvl_perm_plan* p, int64_t* bytes) {
  PCVL_CHECK(p && bytes, "null pointer argument");
  *bytes = (int64_t)p->bytes;
  return PCVL_OK;
}

extern "C" int pcvl_perm_plan_destroy(pcvl_perm_plan* p) {
  destroy_perm_plan(p);
  return PCVL_OK;
}

// ------------------------------------------------------------------ allocation-free variant
// pcvl_permanent_batch_noalloc: the same computation as pcvl_permanent_batch for callers
// that may not allocate device memory.  Its scratch (prepared matrices, descriptors, CTA
// partials) is one file-scope device array of fixed size, present on every device that
// loads the library until the process exits; descriptors travel from a static host buffer.
namespace pcvl {
namespace noalloc {

constexpr size_t align_up_c(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int64_t kMaxElems = int64_t(3) << 20;  // matrix elements per call (48 MiB prepared, 16 B each)
constexpr int32_t kMaxCount = 16384;             // matrices per call
constexpr int64_t kMaxItems = int64_t(1) << 17;  // CTA partial sums per call (2 MiB)

constexpr size_t kPrep = 0;
constexpr size_t kExps = kPrep + (size_t)kMaxElems * sizeof(double2);
constexpr size_t kOffs = kExps + (size_t)kMaxCount * 4;
// offsets, sizes, matrix ids by size and descriptors of one call, packed by count
constexpr size_t kDescBytes = 3 * 256 + (size_t)kMaxCount * (8 + 4 + 4 + sizeof(PermDesc));
constexpr size_t kPart = align_up_c(kOffs + kDescBytes, 256);
constexpr size_t kBytes = kPart + (size_t)kMaxItems * sizeof(double2);
static_assert(kExps % 256 == 0 && kOffs % 256 == 0 && kPart % 256 == 0, "scratch regions stay 256-byte aligned");

constexpr int kMaxDevices = 64;
void* g_dev_ptr[kMaxDevices] = {};
unsigned char g_host_blob[kDescBytes];  // offsets, sizes, mids, descriptors of one call
int32_t g_order[kMaxCount];               // matrix order of the overlap check
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
                                            int32_t method, int32_t precision, void* stream_) {
  using namespace pcvl::noalloc;
  cudaStream_t stream = (cudaStream_t)stream_;
  PCVL_CHECK(count >= 0, "count must be >= 0 (got %d)", count);
  if (count == 0) return PCVL_OK;
  PCVL_CHECK(mats_d && offsets_h && sizes_h && out_d, "null pointer argument");
  PCVL_CHECK(method == 0 || method == 1, "method must be 0 (Glynn) or 1 (Ryser), got %d", method);
  PCVL_CHECK_PERM_PREC(precision);
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
    const BinShape sh = bin_shape(n, ryser, precision, bin_count[n], sms);
    L[n] = sh.L;
    Hb[n] = sh.Hbits;
    P[n] = sh.P;
    ipm[n] = sh.items_per_mat;
    total_items += bin_count[n] * ipm[n];
    mids_so_far += bin_count[n];
  }
  PCVL_CHECK(total_items <= kMaxItems,
             "allocation-free permanents: the batch needs %lld partial sums, more than the maximum of %lld per call",
             (long long)total_items, (long long)kMaxItems);

  std::lock_guard<std::mutex> lock(g_mu);
  PCVL_TRY(check_no_overlap(offsets_h, sizes_h, count, g_order));
  unsigned char* scratch = nullptr;
  PCVL_TRY(noalloc_scratch(&scratch));

  // descriptors of this call packed at the start of the static host buffer: offsets,
  // sizes, matrix ids by size, descriptors (each region 256-byte aligned, sized by count),
  // so one copy of about 24 bytes per matrix travels, not the whole descriptor region
  const size_t r_size = align_up((size_t)count * 8, 256);
  const size_t r_mids = r_size + align_up((size_t)count * 4, 256);
  const size_t r_desc = r_mids + align_up((size_t)count * 4, 256);
  const size_t r_end = r_desc + (size_t)count * sizeof(PermDesc);
  int64_t* h_offs = (int64_t*)g_host_blob;
  int32_t* h_size = (int32_t*)(g_host_blob + r_size);
  int32_t* h_mids = (int32_t*)(g_host_blob + r_mids);
  PermDesc* h_desc = (PermDesc*)(g_host_blob + r_desc);
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
  PCVL_CUDA(cudaMemcpyAsync(scratch + kOffs, g_host_blob, r_end, cudaMemcpyHostToDevice, stream));

  int32_t* exps_d = (int32_t*)(scratch + kExps);
  const int64_t* offs_d = (const int64_t*)(scratch + kOffs);
  const int32_t* sizes_d = (const int32_t*)(scratch + kOffs + r_size);
  int32_t* mids_d = (int32_t*)(scratch + kOffs + r_mids);
  const PermDesc* descs_d = (const PermDesc*)(scratch + kOffs + r_desc);
  double2* parts = (double2*)(scratch + kPart);
  {
    const unsigned blocks = (unsigned)(((int64_t)count * 32 + 255) / 256);
    launch_prepare(precision, blocks, stream, (const double2*)mats_d, offs_d, sizes_d, count, scratch + kPrep,
                   exps_d);
    PCVL_CUDA(cudaGetLastError());
  }
  for (int n = 1; n <= kPermMaxN; ++n) {
    if (bin_count[n] == 0) continue;
    PermBinArgs a;
    a.A = scratch + kPrep;
    a.offs = offs_d;
    a.mids = mids_d + mid_base[n];
    a.nmat = bin_count[n];
    a.L = L[n];
    a.Hbits = Hb[n];
    a.P = P[n];
    a.items_per_mat = ipm[n];
    a.ryser = ryser;
    a.prec = precision;
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
