// SLAP: every output amplitude of one input state by a depth-first walk over the outputs,
// each walker holding one dense table of 2^n photon-subset values.
//
// Replaces xq.SLAP for circuits without feed-forward (perceval/backends/_slap.py:38-80:
// set_unitary, all_prob_ampli, all_prob, prob_distribution).  The reference documents
// the algorithm only as iterating over a lattice of intermediary results of 2^n complex
// values, with less memory than SLOS and faster than SLOS when m >> n
// (docs/source/backends.rst:145-157); its code is closed.  This file's own algorithm
// with that profile:
//
// An output state of n photons is the sorted list a_1 <= ... <= a_n of its photons'
// output modes; ascending lexicographic order of the lists is the descending
// lexicographic order of the occupation vectors, the reference's output order.  With the
// input photons p = 0..n-1 in input modes c_p (each mode repeated by its count), define
// for a prefix a_1..a_k and a set S of k photons
//     F_k[S] = sum over bijections b: {1..k} -> S of prod_e U[a_e, c_b(e)]
// so that F_n[all] = Perm(U[a, c]), and the amplitude is F_n[all] / sqrt(prod s! prod t!)
// (the Naive amplitude, perceval/backends/_naive.py:46-71).  Adding element a:
//     F_{k+1}[S] = sum_{p in S} F_k[S \ {p}] U[a, c_p]         (|S| = k + 1).
// Along one root-to-leaf path level k uses the subsets of popcount k, so a single dense
// array F[0 .. 2^n - 1] holds the whole path: moving to a sibling at depth k rewrites
// level k + 1 only.  Outputs sharing a prefix are contiguous in output order, so a
// walker writes its outputs in order.
//
// Work units: the prefixes of k0 elements (k0-multisets of [m] in order, i.e. the
// k0-photon states), taken by warps from an atomic counter, so the first units, which
// have the largest subtrees, start first.  A warp rebuilds F for its prefix (k0 steps),
// walks the levels k0 + 1 .. n - 1 depth-first with the subsets of each level split over
// its lanes, and at the last level writes the m - a_{n-1} leaves of a node at once, one
// per lane: F_n = sum_p F_{n-1}[all \ {p}] U[a_n, c_p].  Arithmetic: float-float complex
// with exact accumulation of the high products, as in SLOS.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {
namespace {

constexpr int kSlapMaxN = 12;
constexpr int kSlapMaxM = 4096;
constexpr uint64_t kSlapMaxOutputs = 1ull << 36;
constexpr int kSlapSmemBudget = 64 * 1024;  // subset tables per CTA

// Cn(M, x) = C(M + x - 1, x) for M = 0..m, x = 0..n+1 by Pascal's rule, saturating
std::vector<uint64_t> cn_table(int m, int n) {
  const int cs = n + 2;
  std::vector<uint64_t> cn((size_t)(m + 1) * cs, 0);
  for (int M = 0; M <= m; ++M)
    for (int x = 0; x < cs; ++x) {
      uint64_t v;
      if (x == 0)
        v = 1;
      else if (M == 0)
        v = 0;
      else {
        const uint64_t p = cn[(size_t)(M - 1) * cs + x], q = cn[(size_t)M * cs + x - 1];
        v = p > ~0ull - q ? ~0ull : p + q;
      }
      cn[(size_t)M * cs + x] = v;
    }
  return cn;
}

struct SlapArgs {
  int m, n, k0;
  uint64_t units;                    // prefixes of k0 elements
  const cdd* uc;                     // uc[a * n + p] = U[a, c_p]
  const uint16_t* masks;             // subsets ordered by popcount; level k at moff[k] .. moff[k+1]
  const uint32_t* moff;
  const uint64_t* cn;                // cn[M * cs + x] = C(M + x - 1, x)
  int cs;
  dd inv_t;                          // 1 / prod t! (probabilities) or 1 / sqrt(prod t!) (amplitudes)
  const dd* invf;                    // invf[k] = 1 / k! or 1 / sqrt(k!), k = 0..n+1
  int mode;                          // 0: probabilities, 1: amplitudes
  double* out_p;
  double2* out_a;
  unsigned long long* next;          // unit counter
};

__device__ __forceinline__ uint64_t slap_cn(const SlapArgs& a, int M, int x) {
  return x < 0 ? 0ull : __ldg(&a.cn[M * a.cs + x]);
}

// level k + 1 of F for a new element (output mode) e
__device__ __forceinline__ void slap_level(const SlapArgs& a, cdd* F, int k, int e, int lane) {
  const uint32_t b = __ldg(&a.moff[k + 1]), t = __ldg(&a.moff[k + 2]);  // the masks of level k + 1
  const cdd* ue = a.uc + (size_t)e * a.n;
  for (uint32_t i = b + lane; i < t; i += 32) {
    const uint32_t M = __ldg(&a.masks[i]);
    cacc acc = cacc_zero();
    for (uint32_t r = M; r; r &= r - 1) {
      const int p = __ffs(r) - 1;
      cacc_fma(acc, F[M ^ (1u << p)], ue[p]);
    }
    F[M] = cacc_finish(acc);
  }
  __syncwarp();
}

__device__ __forceinline__ void slap_store(const SlapArgs& a, uint64_t o, const cdd& c, const dd& f) {
  if (a.mode == 0) {
    const dd c2 = dd_add(dd_mul(c.re, c.re), dd_mul(c.im, c.im));
    a.out_p[o] = dd_to_double_fast(dd_mul(c2, f));
  } else {
    a.out_a[o] = make_double2(dd_to_double_fast(dd_mul(c.re, f)), dd_to_double_fast(dd_mul(c.im, f)));
  }
}

// The outputs of the node elem[0..n-2] (F valid up to level n - 1): (..., y) for
// y = elem[n-2] .. m-1, one per lane, at positions pos ..  (units that fix n - 1 elements)
__device__ void slap_leaves(const SlapArgs& a, const cdd* F, const int* elem, uint64_t pos, int lane) {
  const int n = a.n, m = a.m;
  dd base = a.inv_t;
  int run = 0;
  for (int e = 0; e < n - 1; ++e) {
    if (e > 0 && elem[e] == elem[e - 1]) {
      ++run;
    } else {
      if (run > 0) base = dd_mul(base, a.invf[run]);
      run = 1;
    }
  }
  const int lo = elem[n - 2];
  const dd f0 = dd_mul(base, a.invf[run]), f1 = dd_mul(base, a.invf[run + 1]);
  const uint32_t full = (1u << n) - 1u;
  for (int y = lo + lane; y < m; y += 32) {
    const cdd* uy = a.uc + (size_t)y * n;
    cacc acc = cacc_zero();
    for (int p = 0; p < n; ++p) cacc_fma(acc, F[full ^ (1u << p)], uy[p]);
    slap_store(a, pos + (uint64_t)(y - lo), cacc_finish(acc), y == lo ? f1 : f0);
  }
}

// The last two levels of the node elem[0..n-3] (F valid up to level n - 2; n >= 2): for the
// siblings x = v0 .. m-1 (v0 = elem[n-3], or 0 for n = 2), in chunks of 32,
//   level n-1: Fs[x][p] = F_{n-1}(x)[all \ {p}] = sum_{q != p} F[all \ {p, q}] U[x, c_q]
// with the lanes over (x, p) pairs, then every output (..., x, y), y >= x:
//   F_n = sum_p Fs[x][p] U[y, c_p],
// with the lanes over the chunk's outputs in order (rows x, columns y: a contiguous range
// of the output order).  Normalisation 1 / (prod s! prod t!) (its square root for
// amplitudes) from float-float tables on the FP32 pipe: the prefix's closed runs give
// base, its last run (length r0, value v0) is closed by x > v0 or extended by x = v0, and
// y = x adds one more to the run of x.  Returns the position after the node's outputs.
__device__ uint64_t slap_batch(const SlapArgs& a, const cdd* F, cdd* Fs, const int* elem, uint64_t pos, int lane) {
  const int n = a.n, m = a.m;
  dd base = a.inv_t;
  int run = 0;
  for (int e = 0; e < n - 2; ++e) {
    if (e > 0 && elem[e] == elem[e - 1]) {
      ++run;
    } else {
      if (run > 0) base = dd_mul(base, a.invf[run]);
      run = 1;
    }
  }
  const int v0 = n >= 3 ? elem[n - 3] : 0;
  const dd A0 = run > 0 ? dd_mul(base, a.invf[run]) : base;
  const dd A1 = dd_mul(base, a.invf[run + 1]), A2 = dd_mul(base, a.invf[run + 2]);
  const dd A0y = dd_mul(A0, a.invf[2]);
  const uint32_t full = (1u << n) - 1u;
  for (int x0 = v0; x0 < m; x0 += 32) {
    const int nx = min(32, m - x0);
    for (int t = lane; t < nx * n; t += 32) {
      const int xi = t / n, p = t - xi * n;
      const uint32_t M = full ^ (1u << p);
      const cdd* ux = a.uc + (size_t)(x0 + xi) * n;
      cacc acc = cacc_zero();
      for (uint32_t r = M; r; r &= r - 1) {
        const int q = __ffs(r) - 1;
        cacc_fma(acc, F[M ^ (1u << q)], ux[q]);
      }
      Fs[t] = cacc_finish(acc);
    }
    __syncwarp();
    // rows xi = 0 .. nx-1 hold y = x0 + xi .. m-1 (lengths m - x0 - xi)
    const uint64_t total = (uint64_t)nx * (m - x0) - (uint64_t)nx * (nx - 1) / 2;
    uint64_t t = lane;
    int xi = 0, y = x0 + lane;
    while (xi < nx && y >= m) {
      const int over = y - m;
      ++xi;
      y = x0 + xi + over;
    }
    while (xi < nx) {
      const int x = x0 + xi;
      const cdd* uy = a.uc + (size_t)y * n;
      const cdd* fx = Fs + xi * n;
      cacc acc = cacc_zero();
      for (int p = 0; p < n; ++p) cacc_fma(acc, fx[p], uy[p]);
      const dd f = (n >= 3 && x == v0) ? (y == x ? A2 : A1) : (y == x ? A0y : A0);
      slap_store(a, pos + t, cacc_finish(acc), f);
      t += 32;
      y += 32;
      while (xi < nx && y >= m) {
        const int over = y - m;
        ++xi;
        y = x0 + xi + over;
      }
    }
    __syncwarp();  // Fs is rewritten by the next chunk
    pos += total;
  }
  return pos;
}

// Sorted mode list el[0..k-1] of rank r among the k-element lists on modes lo..m-1.  The
// lists with first element below i number Cn(m - lo, k) - Cn(m - i, k), so the first
// element is the largest i with that count <= r (binary search), and so on.
__device__ __forceinline__ void slap_unrank(const SlapArgs& a, uint64_t r, int k, int* el) {
  int lo = 0;
  for (int e = 0; e < k; ++e) {
    const int kk = k - e;
    const uint64_t tot = slap_cn(a, a.m - lo, kk);
    int L = lo, R = a.m - 1;
    while (L < R) {
      const int mid = (L + R + 1) >> 1;
      if (tot - slap_cn(a, a.m - mid, kk) <= r)
        L = mid;
      else
        R = mid - 1;
    }
    r -= tot - slap_cn(a, a.m - L, kk);
    el[e] = L;
    lo = L;
  }
}

constexpr int kSlapChunk = 16;  // consecutive units per grab: they share most of their prefix

__global__ void __launch_bounds__(256) slap_walk(SlapArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = a.n, m = a.m, k0 = a.k0;
  cdd* F = reinterpret_cast<cdd*>(smem_raw) + ((size_t)w << n);
  cdd* Fs = reinterpret_cast<cdd*>(smem_raw) + ((size_t)blockDim.x / 32 << n) + (size_t)w * 32 * n;
  int elem[kSlapMaxN], pre[kSlapMaxN];
  while (true) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.next, 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    const uint64_t u0 = (uint64_t)c * kSlapChunk;
    if (u0 >= a.units) break;
    const uint64_t u1 = min(a.units, u0 + kSlapChunk);
    for (uint64_t u = u0; u < u1; ++u) {
      // the prefix (k0 elements); F levels 0..d stay valid when the first change is at d
      slap_unrank(a, u, k0, pre);
      int d = 0;
      if (u != u0)
        while (d < k0 && pre[d] == elem[d]) ++d;
      else if (lane == 0)
        F[0] = cdd_one();
      for (int e = 0; e < k0; ++e) elem[e] = pre[e];
      __syncwarp();
      for (int k = d; k < k0; ++k) slap_level(a, F, k, elem[k], lane);
      // first output: the prefix followed by n - k0 copies of its last element; in list
      // order, rank = sum_j [Cn(m - a_{j-1}, n - j + 1) - Cn(m - a_j, n - j + 1)], a_0 = 0
      uint64_t pos = 0;
      {
        int prev = 0;
        for (int j = 0; j < n; ++j) {
          const int aj = j < k0 ? elem[j] : (k0 > 0 ? elem[k0 - 1] : 0);
          pos += slap_cn(a, m - prev, n - j) - slap_cn(a, m - aj, n - j);
          prev = aj;
        }
      }
      if (n == 1) {  // every output is one element: U[x, c_0] / sqrt(prod t!)
        for (int x = lane; x < m; x += 32) slap_store(a, pos + x, cdd{a.uc[x].re, a.uc[x].im}, a.inv_t);
        continue;
      }
      if (k0 == n - 1) {  // the prefix fixes level n - 1: its outputs only
        slap_leaves(a, F, elem, pos, lane);
        __syncwarp();  // the next unit rewrites level n - 1
        continue;
      }
      if (k0 == n - 2) {
        slap_batch(a, F, Fs, elem, pos, lane);
        continue;
      }
      int k = k0;
      elem[k] = k > 0 ? elem[k - 1] : 0;
      while (true) {
        slap_level(a, F, k, elem[k], lane);
        if (k + 1 == n - 2) {
          pos = slap_batch(a, F, Fs, elem, pos, lane);
          while (true) {
            if (++elem[k] < m) break;
            if (--k < k0) break;
          }
          if (k < k0) break;
        } else {
          ++k;
          elem[k] = elem[k - 1];
        }
      }
      __syncwarp();
    }
  }
}

// uc[a * n + p] = U[a, c_p] as float-float
__global__ void slap_convert(const double2* __restrict__ u, int m, int n, const int32_t* __restrict__ cols,
                             cdd* __restrict__ uc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * n) return;
  const int x = i / n, p = i - x * n;
  const double2 v = u[(size_t)x * m + cols[p]];
  uc[i] = cdd_from(v.x, v.y);
}


int slap_run(const double* u_d, int32_t m, const int32_t* input_state_h, int32_t mode, double* out_d,
             cudaStream_t s) {
  PCVL_CHECK(u_d && input_state_h && out_d, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= kSlapMaxM, "m=%d outside [1, %d]", m, kSlapMaxM);
  PCVL_CHECK(mode == 0 || mode == 1, "mode must be 0 (probabilities) or 1 (amplitudes)");
  std::vector<int32_t> cols;
  double tfact = 1.0;
  for (int i = 0; i < m; ++i) {
    PCVL_CHECK(input_state_h[i] >= 0, "negative photon count in mode %d", i);
    for (int v = 1; v <= input_state_h[i]; ++v) {
      cols.push_back(i);
      tfact *= v;
    }
    PCVL_CHECK((int)cols.size() <= kSlapMaxN, "more than %d photons", kSlapMaxN);
  }
  const int n = (int)cols.size();
  // Cn(M, x) = C(M + x - 1, x), M = 0..m, x = 0..n+1 (Pascal, saturating)
  const int cs = n + 2;
  const std::vector<uint64_t> cn = cn_table(m, n);
  const uint64_t count = cn[(size_t)m * cs + n];
  PCVL_CHECK(count <= kSlapMaxOutputs, "%llu outputs exceed the supported 2^36", (unsigned long long)count);
  if (n == 0) {  // one output, the vacuum, with amplitude 1
    const double one[2] = {1.0, 0.0};
    PCVL_CUDA(cudaMemcpyAsync(out_d, one, mode == 0 ? sizeof(double) : 2 * sizeof(double), cudaMemcpyHostToDevice, s));
    return PCVL_OK;
  }
  // subsets grouped by popcount: level k at moff[k] .. moff[k + 1]
  std::vector<uint16_t> masks;
  std::vector<uint32_t> moff(n + 2, 0);
  for (int k = 0; k <= n; ++k) {
    moff[k] = (uint32_t)masks.size();
    for (uint32_t M = 0; M < (1u << n); ++M)
      if (__builtin_popcount(M) == k) masks.push_back((uint16_t)M);
  }
  moff[n + 1] = (uint32_t)masks.size();
  const int warp_bytes = (int)(sizeof(cdd) * ((1 << n) + 32 * n));  // subset table + sibling level
  const int W = std::max(1, std::min(8, kSlapSmemBudget / warp_bytes));
  const size_t smem = (size_t)W * warp_bytes;
  PCVL_CUDA(cudaFuncSetAttribute(slap_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PCVL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, slap_walk, W * 32, smem));
  per_sm = std::max(per_sm, 1);
  // Work units: prefixes of k0 elements.  A node of level n - 1 has about m / n outputs.
  // From m >= 16 n on they keep at least half the lanes busy: units fix n - 1 elements and
  // write their outputs (k0 = n - 1).  Below that the walk ends with the sibling batches of
  // level n - 2 (k0 <= n - 2): the smallest k0 giving every resident warp eight chunks (the
  // first units have the largest subtrees), or n - 2.  (Measured: m = 1024, n = 3 and
  // m = 256, n = 4 run 2-60x faster on the first form; m = 64, n = 6, m = 32, n = 8 and
  // m = 24, n = 10 run 3-6x faster on the second.)
  const uint64_t warps = (uint64_t)num_sms() * per_sm * W;
  int k0 = n - 1;
  if (n >= 2 && m < 16 * n) {
    k0 = n - 2;
    for (int k = 0; k < n - 2; ++k)
      if (cn[(size_t)m * cs + k] >= warps * 8 * kSlapChunk) {
        k0 = k;
        break;
      }
  }
  // 1 / k! (probabilities) or 1 / sqrt(k!) (amplitudes), k = 0..n+1, as float-float
  std::vector<dd> invf(n + 2);
  {
    double f = 1.0;
    for (int k = 0; k <= n + 1; ++k) {
      if (k > 1) f *= k;
      invf[k] = dd_from_double(mode == 0 ? 1.0 / f : 1.0 / std::sqrt(f));
    }
  }
  // one staged upload: cols | cn | moff | masks | invf | counter
  const size_t o_cols = 0, o_cn = align_up(cols.size() * 4, 16);
  const size_t o_moff = o_cn + align_up(cn.size() * 8, 16);
  const size_t o_masks = o_moff + align_up(moff.size() * 4, 16);
  const size_t o_invf = o_masks + align_up(masks.size() * 2, 16);
  const size_t o_next = o_invf + align_up(invf.size() * sizeof(dd), 16);
  const size_t o_uc = o_next + 16;
  const size_t total = o_uc + (size_t)m * n * sizeof(cdd);
  std::vector<unsigned char> host(o_uc, 0);
  std::memcpy(host.data() + o_cols, cols.data(), cols.size() * 4);
  std::memcpy(host.data() + o_cn, cn.data(), cn.size() * 8);
  std::memcpy(host.data() + o_moff, moff.data(), moff.size() * 4);
  std::memcpy(host.data() + o_masks, masks.data(), masks.size() * 2);
  std::memcpy(host.data() + o_invf, invf.data(), invf.size() * sizeof(dd));
  ScratchGuard scratch(s);
  void* ws = nullptr;
  PCVL_TRY(scratch.alloc(total, &ws));
  unsigned char* base = static_cast<unsigned char*>(ws);
  PCVL_TRY(stage_h2d(host.data(), o_uc, base, s));
  slap_convert<<<(m * n + 255) / 256, 256, 0, s>>>((const double2*)u_d, m, n, (const int32_t*)(base + o_cols),
                                                   (cdd*)(base + o_uc));
  PCVL_CUDA(cudaGetLastError());
  SlapArgs a{};
  a.m = m;
  a.n = n;
  a.k0 = k0;
  a.units = cn[(size_t)m * cs + k0];
  a.uc = (const cdd*)(base + o_uc);
  a.masks = (const uint16_t*)(base + o_masks);
  a.moff = (const uint32_t*)(base + o_moff);
  a.cn = (const uint64_t*)(base + o_cn);
  a.cs = cs;
  a.inv_t = dd_from_double(mode == 0 ? 1.0 / tfact : 1.0 / std::sqrt(tfact));
  a.invf = (const dd*)(base + o_invf);
  a.mode = mode;
  a.out_p = out_d;
  a.out_a = (double2*)out_d;
  a.next = (unsigned long long*)(base + o_next);
  const uint64_t blocks_needed = ((a.units + kSlapChunk - 1) / kSlapChunk + W - 1) / W;
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)num_sms() * per_sm));
  slap_walk<<<grid, W * 32, smem, s>>>(a);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

// ---------------------------------------------------------------- mask selection
// The outputs a mask keeps (xq.FSArray(m, n, mask)): n-photon states that can still be
// completed to an accepted state of N = mask_n photons.  For one mask string: v_i <= d_i
// on fixed modes, and sum over constrained modes of max(d_i - v_i, 0) <= N - n.  Strings
// combine by OR.  One thread per rank: the state is unranked mode by mode while each
// string's conditions are checked; once every photon is placed, the empty remaining
// modes add the suffix sum of their digits to the missing count.
struct MaskSel {
  int m, n, N, nmask, cs;
  const int8_t* digits;    // [nmask][m], -1: any count
  const uint8_t* atl;      // [m]: digit is a lower bound
  const int32_t* sufmiss;  // [nmask][m + 1]: sum of the digits >= 0 over modes i..m-1
  const uint64_t* cn;
};

__device__ __forceinline__ uint64_t sel_cn(const MaskSel& s, int M, int x) {
  return x < 0 ? 0ull : __ldg(&s.cn[M * s.cs + x]);
}

__device__ __forceinline__ bool sel_apply(const MaskSel& s, int d, int i, int v, int& miss) {
  if (d < 0) return true;
  if (s.atl[i]) {
    if (v < d) miss += d - v;
    return true;
  }
  if (v > d) return false;
  miss += d - v;
  return true;
}

__device__ bool fock_accepted(const MaskSel& s, uint64_t r0) {
  const int m = s.m;
  for (int q = 0; q < s.nmask; ++q) {
    const int8_t* dg = s.digits + (size_t)q * m;
    uint64_t r = r0;
    int rem = s.n, miss = 0, i = 0;
    bool ok = true;
    for (; i < m - 1 && rem > 0; ++i) {
      int x = 0;
      while (x < rem && r >= sel_cn(s, m - i, x)) ++x;
      r -= sel_cn(s, m - i, x - 1);
      ok = sel_apply(s, dg[i], i, rem - x, miss);
      rem = x;
      if (!ok) break;
    }
    if (!ok) continue;
    if (i == m - 1) {  // the last mode holds what is left
      if (!sel_apply(s, dg[m - 1], m - 1, rem, miss)) continue;
      i = m;
    }
    miss += __ldg(&s.sufmiss[(size_t)q * (m + 1) + i]);
    if (miss <= s.N - s.n) return true;
  }
  return false;
}

// Count pass (out == nullptr): accepted ranks per 256-rank block to bsum.  Write pass:
// the accepted ranks in order from boff[block].
__global__ void __launch_bounds__(256) fock_mask_pass(MaskSel s, uint64_t count, const uint64_t* __restrict__ boff,
                                                     uint32_t* __restrict__ bsum, uint64_t* __restrict__ out) {
  __shared__ uint32_t wsum[8];
  const uint64_t r = (uint64_t)blockIdx.x * 256 + threadIdx.x;
  const bool acc = r < count && fock_accepted(s, r);
  const unsigned bal = __ballot_sync(0xffffffffu, acc);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wsum[w] = __popc(bal);
  __syncthreads();
  uint32_t base = 0, total = 0;
  for (int q = 0; q < 8; ++q) {
    if (q < w) base += wsum[q];
    total += wsum[q];
  }
  if (out == nullptr) {
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
    return;
  }
  if (acc) out[boff[blockIdx.x] + base + __popc(bal & ((1u << lane) - 1u))] = r;
}


int mask_ranks(int32_t m, int32_t n, int32_t n_masks, const int8_t* digits_h, const uint8_t* at_least_h,
               int32_t mask_n, uint64_t* ranks_d, int64_t capacity, int64_t* kept) {
  PCVL_CHECK(digits_h && kept, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= kSlapMaxM, "m=%d outside [1, %d]", m, kSlapMaxM);
  PCVL_CHECK(n >= 0 && n <= 64, "n=%d outside [0, 64]", n);
  PCVL_CHECK(n_masks >= 1 && n_masks <= 64, "n_masks=%d outside [1, 64]", n_masks);
  PCVL_CHECK(mask_n >= 0, "mask photon count %d is negative", mask_n);
  const int cs = n + 2;
  const std::vector<uint64_t> cn = cn_table(m, n);
  const uint64_t count = cn[(size_t)m * cs + n];
  PCVL_CHECK(count <= kSlapMaxOutputs, "%llu states exceed the supported 2^36", (unsigned long long)count);
  std::vector<int32_t> suf((size_t)n_masks * (m + 1), 0);
  for (int q = 0; q < n_masks; ++q)
    for (int i = m - 1; i >= 0; --i) {
      const int d = digits_h[(size_t)q * m + i];
      PCVL_CHECK(d >= -1, "mask digit %d at mode %d: digits are counts >= 0, or -1 for any", d, i);
      suf[(size_t)q * (m + 1) + i] = suf[(size_t)q * (m + 1) + i + 1] + (d > 0 ? d : 0);
    }
  std::vector<uint8_t> atl(m, 0);
  if (at_least_h)
    for (int i = 0; i < m; ++i) atl[i] = at_least_h[i] ? 1 : 0;
  // one buffer: cn | digits | atl | sufmiss | bsum | boff
  const uint64_t nb = std::max<uint64_t>(1, (count + 255) / 256);
  const size_t o_dg = align_up(cn.size() * 8, 16), o_atl = o_dg + align_up((size_t)n_masks * m, 16);
  const size_t o_suf = o_atl + align_up(m, 16), o_bsum = o_suf + align_up(suf.size() * 4, 16);
  const size_t o_boff = o_bsum + align_up(nb * 4, 16), total = o_boff + nb * 8;
  ScratchGuard scratch(nullptr);
  void* ws = nullptr;
  PCVL_TRY(scratch.alloc(total, &ws));
  unsigned char* base = static_cast<unsigned char*>(ws);
  PCVL_CUDA(cudaMemcpy(base, cn.data(), cn.size() * 8, cudaMemcpyHostToDevice));
  PCVL_CUDA(cudaMemcpy(base + o_dg, digits_h, (size_t)n_masks * m, cudaMemcpyHostToDevice));
  PCVL_CUDA(cudaMemcpy(base + o_atl, atl.data(), m, cudaMemcpyHostToDevice));
  PCVL_CUDA(cudaMemcpy(base + o_suf, suf.data(), suf.size() * 4, cudaMemcpyHostToDevice));
  MaskSel s{m, n, mask_n, n_masks, cs, (const int8_t*)(base + o_dg), (const uint8_t*)(base + o_atl),
            (const int32_t*)(base + o_suf), (const uint64_t*)base};
  fock_mask_pass<<<(unsigned)nb, 256>>>(s, count, nullptr, (uint32_t*)(base + o_bsum), nullptr);
  PCVL_CUDA(cudaGetLastError());
  std::vector<uint32_t> bsum(nb);
  PCVL_CUDA(cudaMemcpy(bsum.data(), base + o_bsum, nb * 4, cudaMemcpyDeviceToHost));
  std::vector<uint64_t> boff(nb);
  uint64_t acc = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    boff[b] = acc;
    acc += bsum[b];
  }
  *kept = (int64_t)acc;
  if (!ranks_d) return PCVL_OK;
  PCVL_CHECK(capacity >= (int64_t)acc, "ranks buffer holds %lld entries, %llu are needed", (long long)capacity,
             (unsigned long long)acc);
  PCVL_CUDA(cudaMemcpy(base + o_boff, boff.data(), nb * 8, cudaMemcpyHostToDevice));
  fock_mask_pass<<<(unsigned)nb, 256>>>(s, count, (const uint64_t*)(base + o_boff), nullptr, ranks_d);
  PCVL_CUDA(cudaGetLastError());
  PCVL_CUDA(cudaDeviceSynchronize());
  return PCVL_OK;
}

}  // namespace
}  // namespace pcvl

extern "C" int pcvl_fock_mask_ranks(int32_t m, int32_t n, int32_t n_masks, const int8_t* digits_h,
                                    const uint8_t* at_least_h, int32_t mask_n, uint64_t* ranks_d, int64_t capacity,
                                    int64_t* kept) {
  return pcvl::mask_ranks(m, n, n_masks, digits_h, at_least_h, mask_n, ranks_d, capacity, kept);
}

extern "C" int pcvl_slap_output_count(int32_t m, const int32_t* input_state_h, int64_t* count) {
  PCVL_CHECK(input_state_h && count, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= pcvl::kSlapMaxM, "m=%d outside [1, %d]", m, pcvl::kSlapMaxM);
  int n = 0;
  for (int i = 0; i < m; ++i) {
    PCVL_CHECK(input_state_h[i] >= 0, "negative photon count in mode %d", i);
    n += input_state_h[i];
  }
  PCVL_CHECK(n <= pcvl::kSlapMaxN, "more than %d photons", pcvl::kSlapMaxN);
  *count = (int64_t)pcvl::cn_table(m, n)[(size_t)m * (n + 2) + n];
  return PCVL_OK;
}

extern "C" int pcvl_slap_probabilities(const double* u_d, int32_t m, const int32_t* input_state_h, double* probs_d,
                                       void* stream) {
  return pcvl::slap_run(u_d, m, input_state_h, 0, probs_d, (cudaStream_t)stream);
}

extern "C" int pcvl_slap_amplitudes(const double* u_d, int32_t m, const int32_t* input_state_h, double* amps_d,
                                    void* stream) {
  return pcvl::slap_run(u_d, m, input_state_h, 1, amps_d, (cudaStream_t)stream);
}
