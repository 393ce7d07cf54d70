// Exact boson sampling, Clifford & Clifford (SODA 2018) "algorithm B".
//
// Replaces xq.Clifford2017 (perceval/backends/_clifford2017.py:36-57).  For input
// occupation t (n photons) let cols be the input modes repeated t_i times.  One
// sample:
//   1. shuffle cols uniformly (Fisher-Yates; draw for position q uses Philox counter
//      (sample, 0xffffffff, q)): photon l enters through column cols[l];
//   2. for k = 1..n, with rows r_0..r_{k-2} drawn so far and B = U[rows, cols[0..k-1]]
//      ((k-1) x k), compute all k sub-permanents
//          sub_l = Per(B without column l)
//      (Glynn over the k-1 row signs, all l at once through leave-one-out products of
//      the column sums), weigh every output mode i by
//          w_i = |sum_l U[i, cols[l]] sub_l|^2
//      (Laplace expansion of the k x k permanent along the new row), and draw r_{k-1}
//      with probability w_i / sum w (uniform from Philox counter (sample, k, 0); the
//      first i whose running sum exceeds u * sum w, summed in index order);
//   3. the sample is the histogram of the rows.
// Common factors of the sub-permanents (the Glynn 2^{2-k}, power-of-two column scales)
// cancel in the normalisation and are dropped.
//
// GPU organisation: a wavefront over photons.  Up to kWave samples are in flight and,
// for every photon k, two kernels run over all of them:
//   cc_sub_kernel   the k sub-permanents of every sample.  The 2^{k-2} sign patterns are
//                   split into lo bits (a shared-memory table of column-sum parts) and
//                   hi bits spread over lane groups and CTAs.  Four lanes share one
//                   pattern and each owns K/4 columns: its suffix products and the
//                   accumulators of its columns stay in registers, and the products of
//                   the other lanes' columns come from a two-step shuffle butterfly.
//                   One partial sum per (sample, chunk of hi patterns) goes to memory.
//   cc_draw_kernel  one CTA per sample: adds the chunk partials, undoes the column
//                   scaling, forms w_i in FP64 for every mode, and a block scan over
//                   the modes locates the draw.
// The sub-permanents run in one of three arithmetic policies: float-float (ArDD, the
// default), FP64 precision on the integer pipes (ArFX) or FP32 (ArF32).
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "blockfloat.cuh"
#include "runtime.cuh"

namespace pcvl {

__device__ __forceinline__ float shx(float v, int mask) { return __shfl_xor_sync(0xffffffffu, v, mask); }

// ------------------------------------------------------------ arithmetic policies
struct ArDD {  // float-float (FP64-class): lazy products and sums in the pattern loop,
               // exact two_sum accumulation of the high parts
  using C = cdd;
  static constexpr bool kFixed = false;
  static __device__ __forceinline__ C fix(C a, int) { return a; }
  struct Acc {
    float rh, rl, ih, il;
  };
  static __device__ __forceinline__ C zero() { return cdd_zero(); }
  static __device__ __forceinline__ C one() { return cdd_one(); }
  static __device__ __forceinline__ C add(C a, C b) { return cdd_add_lazy(a, b); }
  static __device__ __forceinline__ C add_n(C a, C b) { return cdd_add(a, b); }
  static __device__ __forceinline__ C sub_n(C a, C b) { return cdd_sub(a, b); }
  static __device__ __forceinline__ C mul(C a, C b) { return cdd_mul_lazy(a, b); }
  static __device__ __forceinline__ C neg(C a) { return cdd_neg(a); }
  static __device__ __forceinline__ C twice(C a) { return cdd_ldexp(a, 1); }
  static __device__ __forceinline__ C from(double2 v) { return cdd_from(v.x, v.y); }
  static __device__ __forceinline__ C scale(C a, int e) { return cdd_ldexp(a, e); }
  static __device__ __forceinline__ float mag(C a) { return fabsf(a.re.hi) + fabsf(a.im.hi); }
  static __device__ __forceinline__ C shfl(C v, int mask) {
    return {{shx(v.re.hi, mask), shx(v.re.lo, mask)}, {shx(v.im.hi, mask), shx(v.im.lo, mask)}};
  }
  static __device__ __forceinline__ Acc acc_zero() { return {0.f, 0.f, 0.f, 0.f}; }
  static __device__ __forceinline__ void acc_add(Acc& a, C x) {
    const dd r = two_sum(a.rh, x.re.hi);
    const dd i = two_sum(a.ih, x.im.hi);
    a.rh = r.hi;
    a.rl += r.lo + x.re.lo;
    a.ih = i.hi;
    a.il += i.lo + x.im.lo;
  }
  static __device__ __forceinline__ void acc_fold(Acc& a) {
    const dd r = two_sum(a.rh, a.rl);
    const dd i = two_sum(a.ih, a.il);
    a = {r.hi, r.lo, i.hi, i.lo};
  }
  static __device__ __forceinline__ Acc acc_merge(Acc a, Acc b) {
    const dd r = dd_add({a.rh, a.rl}, {b.rh, b.rl});
    const dd i = dd_add({a.ih, a.il}, {b.ih, b.il});
    return {r.hi, r.lo, i.hi, i.lo};
  }
  static __device__ __forceinline__ Acc acc_shfl(Acc v, int mask) {
    return {shx(v.rh, mask), shx(v.rl, mask), shx(v.ih, mask), shx(v.il, mask)};
  }
  static __device__ __forceinline__ double2 acc_value(Acc a) {
    return make_double2((double)a.rh + (double)a.rl, (double)a.ih + (double)a.il);
  }
};

struct ArF32 {  // FP32 with Kahan-compensated accumulation
  using C = float2;
  static constexpr bool kFixed = false;
  static __device__ __forceinline__ C fix(C a, int) { return a; }
  struct Acc {
    float sr, cr, si, ci;  // sums and compensations
  };
  static __device__ __forceinline__ C zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ C one() { return make_float2(1.f, 0.f); }
  static __device__ __forceinline__ C add(C a, C b) { return make_float2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ C add_n(C a, C b) { return add(a, b); }
  static __device__ __forceinline__ C sub_n(C a, C b) { return make_float2(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ C mul(C a, C b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
  }
  static __device__ __forceinline__ C neg(C a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ C twice(C a) { return make_float2(2.f * a.x, 2.f * a.y); }
  static __device__ __forceinline__ C from(double2 v) { return make_float2((float)v.x, (float)v.y); }
  static __device__ __forceinline__ C scale(C a, int e) { return make_float2(ldexpf(a.x, e), ldexpf(a.y, e)); }
  static __device__ __forceinline__ float mag(C a) { return fabsf(a.x) + fabsf(a.y); }
  static __device__ __forceinline__ C shfl(C v, int mask) { return make_float2(shx(v.x, mask), shx(v.y, mask)); }
  static __device__ __forceinline__ Acc acc_zero() { return {0.f, 0.f, 0.f, 0.f}; }
  static __device__ __forceinline__ void kahan(float& s, float& c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  static __device__ __forceinline__ void acc_add(Acc& a, C x) {
    kahan(a.sr, a.cr, x.x);
    kahan(a.si, a.ci, x.y);
  }
  static __device__ __forceinline__ void acc_fold(Acc&) {}
  static __device__ __forceinline__ Acc acc_merge(Acc a, Acc b) {
    kahan(a.sr, a.cr, b.sr);
    kahan(a.sr, a.cr, -b.cr);
    kahan(a.si, a.ci, b.si);
    kahan(a.si, a.ci, -b.ci);
    return a;
  }
  static __device__ __forceinline__ Acc acc_shfl(Acc v, int mask) {
    return {shx(v.sr, mask), shx(v.cr, mask), shx(v.si, mask), shx(v.ci, mask)};
  }
  static __device__ __forceinline__ double2 acc_value(Acc a) {
    return make_double2((double)a.sr - (double)a.cr, (double)a.si - (double)a.ci);
  }
};

// FP64 precision on two pipes (the sampler's FP64 mode): every element of the (k-1) x k
// matrix is turned, after its column's power-of-two scaling, into 64-bit fixed point
// (value x 2^F, F = 62 - c0, with c0 the bound on the scaled column l1 norms), so the lo
// table, the hi parts and the column sums of every sign pattern are exact integer sums;
// each column sum is then normalised to 64-bit block floating point and every product of
// the leave-one-out products is a block-floating product on the integer pipes (62
// significant bits); the terms are converted to FP64 once and summed in FP64.  The fixed
// point keeps every element to 2^-F of its column's l1 norm, the normwise accuracy of an
// FP64 column sum.
struct ArFX {
  using C = BFC;
  static constexpr bool kFixed = true;
  struct Acc {
    double r, i;
  };
  static __device__ __forceinline__ C zero() { return {0, 0, 0}; }
  static __device__ __forceinline__ C one() { return {1ll << 61, 0, -61}; }
  // fixed-point sums (equal exponents), in two's-complement arithmetic
  static __device__ __forceinline__ C add_n(C a, C b) {
    return {(long long)((unsigned long long)a.re + (unsigned long long)b.re),
            (long long)((unsigned long long)a.im + (unsigned long long)b.im), a.e};
  }
  static __device__ __forceinline__ C sub_n(C a, C b) {
    return {(long long)((unsigned long long)a.re - (unsigned long long)b.re),
            (long long)((unsigned long long)a.im - (unsigned long long)b.im), a.e};
  }
  static __device__ __forceinline__ C twice(C a) {
    return {(long long)((unsigned long long)a.re << 1), (long long)((unsigned long long)a.im << 1), a.e};
  }
  // a column sum of one sign pattern: exact, then normalised for the products
  static __device__ __forceinline__ C add(C a, C b) {
    const C s = add_n(a, b);
    return bf_norm(s.re, s.im, s.e);
  }
  static __device__ __forceinline__ C mul(C a, C b) { return bf_mul(a, b); }
  static __device__ __forceinline__ C neg(C a) {
    return {(long long)(0ull - (unsigned long long)a.re), (long long)(0ull - (unsigned long long)a.im), a.e};
  }
  // an element of U: both parts on the exponent of the larger (rounded to 62 bits below it)
  static __device__ __forceinline__ C from(double2 v) {
    const double mx = fmax(fabs(v.x), fabs(v.y));
    if (mx == 0.0) return {0, 0, 0};
    int e0;
    frexp(mx, &e0);  // mx in [2^(e0-1), 2^e0)
    return {__double2ll_rn(ldexp(v.x, 61 - e0)), __double2ll_rn(ldexp(v.y, 61 - e0)), e0 - 61};
  }
  static __device__ __forceinline__ C scale(C a, int e) { return {a.re, a.im, a.e + e}; }
  static __device__ __forceinline__ float mag(C a) {
    return ldexpf((float)llabs(a.re) + (float)llabs(a.im), a.e);
  }
  // the element as fixed point with F fraction bits (|value| < 2^(62 - F) after scaling)
  static __device__ __forceinline__ C fix(C a, int F) {
    const int sh = a.e + F;
    if (sh >= 0) return {(long long)((unsigned long long)a.re << sh), (long long)((unsigned long long)a.im << sh), -F};
    if (sh <= -63) return {0, 0, -F};
    return {a.re >> -sh, a.im >> -sh, -F};
  }
  static __device__ __forceinline__ C shfl(C v, int mask) {
    return {__shfl_xor_sync(0xffffffffu, v.re, mask), __shfl_xor_sync(0xffffffffu, v.im, mask),
            __shfl_xor_sync(0xffffffffu, v.e, mask)};
  }
  static __device__ __forceinline__ Acc acc_zero() { return {0.0, 0.0}; }
  static __device__ __forceinline__ void acc_add(Acc& a, C x) {
    a.r += bf_to_f64(x.re, x.e);
    a.i += bf_to_f64(x.im, x.e);
  }
  static __device__ __forceinline__ void acc_fold(Acc&) {}
  static __device__ __forceinline__ Acc acc_merge(Acc a, Acc b) { return {a.r + b.r, a.i + b.i}; }
  static __device__ __forceinline__ double shd(double v, int mask) { return __shfl_xor_sync(0xffffffffu, v, mask); }
  static __device__ __forceinline__ Acc acc_shfl(Acc v, int mask) { return {shd(v.r, mask), shd(v.i, mask)}; }
  static __device__ __forceinline__ double2 acc_value(Acc a) { return make_double2(a.r, a.i); }
};

constexpr int kCCThreads = 128;
constexpr int kMaxPhotons = 32;

template <class Ar>
__global__ void cc_convert(const double2* __restrict__ u, int m, typename Ar::C* __restrict__ uc) {
  const int tot = m * m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) uc[i] = Ar::from(u[i]);
}

// ------------------------------------------------------------ sub-permanents
struct CCSubArgs {
  const void* uc;         // U converted to Ar::C, row-major m x m
  int m, k, L, Hb, chunks;
  int64_t nsamp;          // samples in the wavefront
  const int32_t* cols;    // [nsamp][32] shuffled input columns
  const int32_t* rows;    // [nsamp][32] rows drawn so far
  int32_t* cexp;          // [nsamp][32] column exponents (written by chunk 0)
  double2* partials;      // [nsamp][chunks][K]
};

// K padded columns (K / 4 per lane), TW warps per sample team (1: four samples per
// CTA, lo table of <= 16 patterns; 4: the CTA works on one sample, 64 lo patterns).
template <class Ar, int K, int TW>
struct SubCfg {
  static constexpr int Q = K / 4;
  static constexpr int TEAMS = 4 / TW;
  static constexpr int LMAX = TW == 1 ? 4 : 6;
  static constexpr size_t c_elems = (size_t)K * K + (size_t)(1 << LMAX) * K;
  static constexpr size_t team_bytes = c_elems * sizeof(typename Ar::C) + (size_t)TW * K * sizeof(typename Ar::Acc);
  static constexpr size_t smem = TEAMS * team_bytes;
};

template <int TW>
__device__ __forceinline__ void team_sync() {
  if constexpr (TW == 1)
    __syncwarp();
  else
    __syncthreads();
}

template <class Ar, int K, int TW>
__global__ void __launch_bounds__(kCCThreads) cc_sub_kernel(CCSubArgs a) {
  using C = typename Ar::C;
  using Acc = typename Ar::Acc;
  using Cfg = SubCfg<Ar, K, TW>;
  constexpr int Q = Cfg::Q;
  constexpr int NT = 32 * TW;  // threads per team
  constexpr int NG = 8 * TW;   // lane groups per team
  extern __shared__ __align__(16) unsigned char smem[];
  const int team = threadIdx.x / NT;
  const int tt = threadIdx.x - team * NT;
  unsigned char* tb = smem + team * Cfg::team_bytes;
  C* Bs = reinterpret_cast<C*>(tb);                                   // K x K (rows 0..k-2)
  C* Ts = Bs + K * K;                                                 // (1 << L) x K
  Acc* red = reinterpret_cast<Acc*>(tb + Cfg::c_elems * sizeof(C));  // TW x K

  const int64_t tg = (int64_t)blockIdx.x * Cfg::TEAMS + team;
  const int64_t s = tg / a.chunks;
  if (s >= a.nsamp) return;  // the whole team leaves (a warp for TW = 1, the CTA for TW = 4)
  const int chunk = (int)(tg - s * a.chunks);
  const int m = a.m, k = a.k, d = k - 1, L = a.L, Hb = a.Hb;
  const int32_t* rows = a.rows + s * kMaxPhotons;
  const int32_t* cols = a.cols + s * kMaxPhotons;
  const C* U = reinterpret_cast<const C*>(a.uc);

  // B (padding columns: S_c = 1 for every pattern, so they drop out of the products)
  for (int e = tt; e < d * K; e += NT) {
    const int r = e / K, c = e - r * K;
    Bs[e] = c < k ? U[(size_t)rows[r] * m + cols[c]] : (r == 0 ? Ar::one() : Ar::zero());
  }
  team_sync<TW>();
  // Scale column c by 2^e_c so that its l1 norm lies in [2^(c0-1), 2^c0) with
  // (k - 1) c0 + (k - 2) <= 120: every product of k - 1 column sums and every sum of
  // the 2^(k-2) terms stays inside the FP32 range.  Exact; the draw undoes it.
  if (tt < k) {
    float l1 = 0.f;
    for (int r = 0; r < d; ++r) l1 += Ar::mag(Bs[r * K + tt]);
    const int c0 = min(4, (120 - (k - 2)) / (k - 1));
    // fixed point: every column sum must stay below 2^62, so the FP32 l1 (a few ulps of
    // rounding) is nudged up before the binade is taken
    if (Ar::kFixed) l1 *= 1.f + 0x1p-16f;
    int ex = 0;
    if (l1 > 0.f) frexpf(l1, &ex);
    const int e = l1 > 0.f ? c0 - ex : 0;
    if (chunk == 0) a.cexp[s * kMaxPhotons + tt] = e;
    for (int r = 0; r < d; ++r) Bs[r * K + tt] = Ar::scale(Bs[r * K + tt], e);
  }
  team_sync<TW>();
  if constexpr (Ar::kFixed) {  // every element (padding included) into fixed point
    const int F = 62 - min(4, (120 - (k - 2)) / (k - 1));
    for (int e = tt; e < d * K; e += NT) Bs[e] = Ar::fix(Bs[e], F);
    team_sync<TW>();
  }
  // lo table over rows 1..L: T[b][c] = sum_l (bit l of b ? -1 : +1) B[1 + l][c]
  for (int c = tt; c < K; c += NT) {
    C t0 = Ar::zero();
    for (int l = 0; l < L; ++l) t0 = Ar::add_n(t0, Bs[(1 + l) * K + c]);
    Ts[c] = t0;
  }
  team_sync<TW>();
  for (int l = 0; l < L; ++l) {
    const int half = 1 << l;
    for (int e = tt; e < half * K; e += NT) {
      const int b = e / K, c = e - b * K;
      Ts[(b + half) * K + c] = Ar::sub_n(Ts[b * K + c], Ar::twice(Bs[(1 + l) * K + c]));
    }
    team_sync<TW>();
  }

  // lane group grp (4 lanes, lane g owns columns 4j + g) takes hi patterns
  // h0 + grp, h0 + grp + NG, ... of this chunk; every lane runs the same rounds so the
  // shuffles see the full warp
  const int lane = threadIdx.x & 31, g = lane & 3, grp = tt >> 2;
  const uint64_t nhi = 1ull << Hb;
  const uint64_t per = (nhi + (uint64_t)a.chunks - 1) / (uint64_t)a.chunks;
  const uint64_t h0 = (uint64_t)chunk * per;
  const uint64_t h1 = min(nhi, h0 + per);
  const int nlo = 1 << L;
  Acc acc[Q];
#pragma unroll
  for (int j = 0; j < Q; ++j) acc[j] = Ar::acc_zero();

  for (uint64_t base = h0; base < h1; base += NG) {
    const uint64_t h = base + grp;
    const bool active = h < h1;  // uniform within the lane group
    C Hq[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const int c = 4 * j + g;
      C v = Bs[c];  // row 0, sign +1
      for (int t = 0; t < Hb; ++t) {
        const C x = Bs[(1 + L + t) * K + c];
        v = ((h >> t) & 1ull) ? Ar::sub_n(v, x) : Ar::add_n(v, x);
      }
      Hq[j] = v;
    }
    const int hs = __popcll(h) & 1;
    for (int b = 0; b < nlo; ++b) {
      const C* Tr = Ts + b * K + g;
      C S[Q], sq[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) S[j] = Ar::add(Hq[j], Tr[4 * j]);
      sq[Q - 1] = S[Q - 1];
#pragma unroll
      for (int j = Q - 2; j >= 0; --j) sq[j] = Ar::mul(S[j], sq[j + 1]);
      // product of the other three lanes' columns
      const C x1 = Ar::shfl(sq[0], 1);
      const C x2 = Ar::shfl(Ar::mul(sq[0], x1), 2);
      C pre = Ar::mul(x1, x2);
      const bool neg = ((__popc(b) & 1) ^ hs) != 0;
      if (active) {
#pragma unroll
        for (int j = 0; j < Q; ++j) {
          const C term = j + 1 < Q ? Ar::mul(pre, sq[j + 1]) : pre;
          Ar::acc_add(acc[j], neg ? Ar::neg(term) : term);
          if (j + 1 < Q) pre = Ar::mul(pre, S[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) Ar::acc_fold(acc[j]);
  }

  // lanes with the same g hold the same columns: reduce over the warp's 8 groups
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    Acc v = acc[j];
    v = Ar::acc_merge(v, Ar::acc_shfl(v, 4));
    v = Ar::acc_merge(v, Ar::acc_shfl(v, 8));
    v = Ar::acc_merge(v, Ar::acc_shfl(v, 16));
    acc[j] = v;
  }
  double2* out = a.partials + ((size_t)s * a.chunks + chunk) * K;
  if constexpr (TW == 1) {
    if (lane < 4) {
#pragma unroll
      for (int j = 0; j < Q; ++j) out[4 * j + g] = Ar::acc_value(acc[j]);
    }
  } else {
    const int w = tt >> 5;
    if (lane < 4) {
#pragma unroll
      for (int j = 0; j < Q; ++j) red[w * K + 4 * j + g] = acc[j];
    }
    __syncthreads();
    if (tt < K) {
      Acc v = red[tt];
      for (int w2 = 1; w2 < TW; ++w2) v = Ar::acc_merge(v, red[w2 * K + tt]);
      out[tt] = Ar::acc_value(v);
    }
  }
}

// ------------------------------------------------------------ draw
struct CCDrawArgs {
  const double2* u;  // U, row-major m x m (FP64)
  int m, n, k, K, chunks;
  int64_t nsamp, s0;  // wavefront size and index of its first sample in the call
  uint64_t first;
  uint32_t k0, k1;
  const int32_t* cols0;      // input columns of every input state: [state][kMaxPhotons], ascending
  const int64_t* state_off;  // first sample (call-relative) of every input state; nstates + 1 entries
  int32_t nstates;
  int32_t* cols;
  int32_t* rows;
  const int32_t* cexp;
  const double2* partials;
  int32_t* out;  // count x m
};

constexpr int kDrawThreads = 128;

__global__ void __launch_bounds__(kDrawThreads) cc_draw_kernel(CCDrawArgs a) {
  __shared__ double2 sub[kMaxPhotons];
  __shared__ int sx[kMaxPhotons];
  __shared__ int cl[kMaxPhotons];
  __shared__ double wtot[kDrawThreads / 32];
  __shared__ double tgt;
  __shared__ int pick, lastpos;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int m = a.m, k = a.k;
  const int per = (m + kDrawThreads - 1) / kDrawThreads;
  const int i0 = min(m, tid * per), i1 = min(m, i0 + per);

  for (int64_t sl = blockIdx.x; sl < a.nsamp; sl += gridDim.x) {
    const uint64_t sid = a.first + (uint64_t)(a.s0 + sl);
    const uint32_t s_lo = (uint32_t)sid, s_hi = (uint32_t)(sid >> 32);
    int32_t* cols = a.cols + sl * kMaxPhotons;
    int32_t* rows = a.rows + sl * kMaxPhotons;
    if (k == 1) {
      if (tid == 0) {
        // the input state of this sample: the last state starting at or before it
        const int64_t g = a.s0 + sl;
        int lo = 0, hi = a.nstates - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (a.state_off[mid] <= g)
            lo = mid;
          else
            hi = mid - 1;
        }
        const int32_t* c0 = a.cols0 + (size_t)lo * kMaxPhotons;
        for (int l = 0; l < a.n; ++l) cols[l] = c0[l];
        for (int q = a.n - 1; q >= 1; --q) {
          const u4 r = philox4x32_10({s_lo, s_hi, 0xffffffffu, (uint32_t)q}, a.k0, a.k1);
          const int j = (int)mulhi32(r.x, (uint32_t)(q + 1));
          const int t = cols[q];
          cols[q] = cols[j];
          cols[j] = t;
        }
        sub[0] = make_double2(1.0, 0.0);
      }
    } else if (tid < k) {
      double2 v = make_double2(0.0, 0.0);
      const double2* p = a.partials + (size_t)sl * a.chunks * a.K + tid;
      for (int c = 0; c < a.chunks; ++c) {
        v.x += p[(size_t)c * a.K].x;
        v.y += p[(size_t)c * a.K].y;
      }
      sub[tid] = v;
      const double mg = fabs(v.x) + fabs(v.y);
      sx[tid] = mg > 0.0 ? ilogb(mg) + a.cexp[sl * kMaxPhotons + tid] : INT_MIN;
    }
    if (tid == 0) {
      pick = INT_MAX;
      lastpos = -1;
    }
    __syncthreads();
    if (tid < k) {
      cl[tid] = cols[tid];
      if (k > 1) {
        // true sub_l is proportional to sub_l 2^{e_l}; bring the largest near 1
        int emax = INT_MIN;
        for (int l = 0; l < k; ++l) emax = max(emax, sx[l]);
        const double2 v = sub[tid];
        const int e = a.cexp[sl * kMaxPhotons + tid] - emax;
        sub[tid] = sx[tid] == INT_MIN ? make_double2(0.0, 0.0) : make_double2(ldexp(v.x, e), ldexp(v.y, e));
      }
    }
    __syncthreads();
    auto weight = [&](int i) {
      const double2* ur = a.u + (size_t)i * m;
      double zr = 0.0, zi = 0.0;
      for (int l = 0; l < k; ++l) {
        const double2 x = ur[cl[l]], y = sub[l];
        zr = fma(x.x, y.x, fma(-x.y, y.y, zr));
        zi = fma(x.x, y.y, fma(x.y, y.x, zi));
      }
      return zr * zr + zi * zi;
    };
    double loc = 0.0;
    int lp = -1;
    for (int i = i0; i < i1; ++i) {
      const double w = weight(i);
      loc += w;
      if (w > 0.0) lp = i;
    }
    double incl = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) wtot[wid] = incl;
    if (lp >= 0) atomicMax(&lastpos, lp);
    __syncthreads();
    double base = incl - loc, W = 0.0;
    for (int w2 = 0; w2 < kDrawThreads / 32; ++w2) {
      if (w2 < wid) base += wtot[w2];
      W += wtot[w2];
    }
    if (tid == 0) {
      const u4 r = philox4x32_10({s_lo, s_hi, (uint32_t)k, 0u}, a.k0, a.k1);
      tgt = u01_from(r.x, r.y) * W;
    }
    __syncthreads();
    const double target = tgt;
    if (i0 < i1 && base + loc > target) {
      double run = base;
      for (int i = i0; i < i1; ++i) {
        run += weight(i);
        if (run > target) {
          atomicMin(&pick, i);
          break;
        }
      }
    }
    __syncthreads();
    if (tid == 0) rows[k - 1] = pick != INT_MAX ? pick : (lastpos >= 0 ? lastpos : 0);
    if (k == a.n) {
      __syncthreads();
      int32_t* o = a.out + (size_t)(a.s0 + sl) * m;
      for (int i = tid; i < m; i += kDrawThreads) o[i] = 0;
      __syncthreads();
      if (tid == 0)
        for (int q = 0; q < a.n; ++q) o[rows[q]] += 1;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ host side
struct StepPlan {
  int K, TW, L, Hb, chunks;
};

static StepPlan plan_step(int k, int64_t nsamp, int target_ctas) {
  StepPlan p{};
  const int F = k - 2;
  p.K = k <= 8 ? 8 : k <= 12 ? 12 : (k + 3) / 4 * 4;
  p.TW = k <= 12 ? 1 : 4;
  p.L = std::min(p.TW == 1 ? 4 : 6, F);
  p.Hb = F - p.L;
  p.chunks = 1;
  if (p.TW == 4) {
    const int64_t max_chunks = std::max<int64_t>(1, (1ll << p.Hb) / 32);
    const int64_t want = (target_ctas + nsamp - 1) / nsamp;
    p.chunks = (int)std::min<int64_t>(max_chunks, std::max<int64_t>(1, want));
  }
  return p;
}

template <class Ar, int K, int TW>
static int launch_sub(const CCSubArgs& a, cudaStream_t s) {
  using Cfg = SubCfg<Ar, K, TW>;
  const size_t smem = Cfg::smem;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(cc_sub_kernel<Ar, K, TW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  const int64_t teams = a.nsamp * a.chunks;
  const int64_t grid = (teams + Cfg::TEAMS - 1) / Cfg::TEAMS;
  cc_sub_kernel<Ar, K, TW><<<(unsigned)grid, kCCThreads, smem, s>>>(a);
  return (int)cudaGetLastError();
}

template <class Ar>
static int sub_dispatch(const StepPlan& p, const CCSubArgs& a, cudaStream_t s) {
  switch (p.K) {
    case 8: return launch_sub<Ar, 8, 1>(a, s);
    case 12: return launch_sub<Ar, 12, 1>(a, s);
    case 16: return launch_sub<Ar, 16, 4>(a, s);
    case 20: return launch_sub<Ar, 20, 4>(a, s);
    case 24: return launch_sub<Ar, 24, 4>(a, s);
    case 28: return launch_sub<Ar, 28, 4>(a, s);
    case 32: return launch_sub<Ar, 32, 4>(a, s);
    default: return (int)cudaErrorInvalidValue;
  }
}

constexpr int64_t kWave = 32768;  // samples in flight

}  // namespace pcvl

using namespace pcvl;

// Samples of nstates input states of one photon count: state b's counts[b] samples
// occupy rows off_b .. off_b + counts[b] - 1 of out_counts_d (off_b = counts of the states
// before it) and use the Philox counters of samples first_sample + off_b + j.
static int cc2017_run(const double* u_d, int32_t m, int32_t nstates, const int32_t* input_states_h,
                      const int64_t* counts_h, uint64_t seed, uint64_t first_sample, int32_t precision,
                      int32_t* out_counts_d, cudaStream_t s) {
  PCVL_CHECK(u_d && input_states_h && counts_h && out_counts_d, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= 2048, "m=%d outside [1, 2048]", m);
  PCVL_CHECK(nstates >= 1 && nstates <= (1 << 20), "nstates=%d outside [1, 2^20]", nstates);
  PCVL_CHECK(precision == kPrecFloatFloat || precision == kPrecFP32 || precision == kPrecFP64,
             "precision must be %d (float-float), %d (FP32) or %d (FP64), got %d", (int)kPrecFloatFloat,
             (int)kPrecFP32, (int)kPrecFP64, precision);
  std::vector<int32_t> cols((size_t)nstates * kMaxPhotons, 0);
  std::vector<int64_t> state_off(nstates + 1, 0);
  int n = -1;
  for (int b = 0; b < nstates; ++b) {
    PCVL_CHECK(counts_h[b] >= 0, "count of input state %d is negative", b);
    int nb = 0;
    for (int i = 0; i < m; ++i) {
      const int32_t v = input_states_h[(size_t)b * m + i];
      PCVL_CHECK(v >= 0, "negative photon count in input state %d", b);
      for (int t = 0; t < v; ++t) {
        PCVL_CHECK(nb < kMaxPhotons, "input state %d has more than %d photons", b, kMaxPhotons);
        cols[(size_t)b * kMaxPhotons + nb++] = i;
      }
    }
    PCVL_CHECK(n < 0 || nb == n, "input state %d has %d photons, state 0 has %d: one call samples one photon count",
               b, nb, n);
    n = nb;
    state_off[b + 1] = state_off[b] + counts_h[b];
  }
  const int64_t count = state_off[nstates];
  if (count == 0) return PCVL_OK;
  if (n == 0) {
    PCVL_CUDA(cudaMemsetAsync(out_counts_d, 0, (size_t)count * m * sizeof(int32_t), s));
    return PCVL_OK;
  }
  // wavefronts of equal size
  const int64_t waves = (count + kWave - 1) / kWave;
  const int64_t W = (count + waves - 1) / waves;
  const int target_ctas = 8 * num_sms();
  int max_chunks = 1;
  for (int k = 2; k <= n; ++k) max_chunks = std::max(max_chunks, plan_step(k, std::min(W, count), target_ctas).chunks);
  // also the last (possibly shorter) wavefront
  const int64_t last = count - (waves - 1) * W;
  for (int k = 2; k <= n; ++k) max_chunks = std::max(max_chunks, plan_step(k, last, target_ctas).chunks);

  const size_t csz = precision == kPrecFloatFloat ? sizeof(cdd) : precision == kPrecFP64 ? sizeof(BFC)
                                                                                          : sizeof(float2);
  const size_t o_cols0 = align_up((size_t)m * m * csz, 256);
  const size_t o_soff = o_cols0 + align_up(cols.size() * sizeof(int32_t), 256);
  const size_t o_cols = o_soff + align_up(state_off.size() * sizeof(int64_t), 256);
  const size_t st_bytes = align_up((size_t)W * kMaxPhotons * sizeof(int32_t), 256);
  const size_t o_rows = o_cols + st_bytes;
  const size_t o_cexp = o_rows + st_bytes;
  const size_t o_part = o_cexp + st_bytes;
  const size_t total = o_part + (size_t)W * max_chunks * kMaxPhotons * sizeof(double2);
  ScratchGuard scratch(s);
  void* ws = nullptr;
  PCVL_TRY(scratch.alloc(total, &ws));
  unsigned char* base = (unsigned char*)ws;
  {
    // one staged upload: the columns of every state, then the state offsets
    std::vector<unsigned char> up(o_cols - o_cols0, 0);
    std::memcpy(up.data(), cols.data(), cols.size() * sizeof(int32_t));
    std::memcpy(up.data() + (o_soff - o_cols0), state_off.data(), state_off.size() * sizeof(int64_t));
    PCVL_TRY(stage_h2d(up.data(), up.size(), base + o_cols0, s));
  }
  const int cgrid = std::max(1, std::min(1024, (m * m + 255) / 256));
  if (precision == kPrecFloatFloat)
    cc_convert<ArDD><<<cgrid, 256, 0, s>>>((const double2*)u_d, m, (cdd*)base);
  else if (precision == kPrecFP64)
    cc_convert<ArFX><<<cgrid, 256, 0, s>>>((const double2*)u_d, m, (BFC*)base);
  else
    cc_convert<ArF32><<<cgrid, 256, 0, s>>>((const double2*)u_d, m, (float2*)base);
  PCVL_CUDA(cudaGetLastError());

  CCSubArgs sa{};
  sa.uc = base;
  sa.m = m;
  sa.cols = (const int32_t*)(base + o_cols);
  sa.rows = (const int32_t*)(base + o_rows);
  sa.cexp = (int32_t*)(base + o_cexp);
  sa.partials = (double2*)(base + o_part);
  CCDrawArgs da{};
  da.u = (const double2*)u_d;
  da.m = m;
  da.n = n;
  da.first = first_sample;
  da.k0 = (uint32_t)seed;
  da.k1 = (uint32_t)(seed >> 32);
  da.cols0 = (const int32_t*)(base + o_cols0);
  da.state_off = (const int64_t*)(base + o_soff);
  da.nstates = nstates;
  da.cols = (int32_t*)(base + o_cols);
  da.rows = (int32_t*)(base + o_rows);
  da.cexp = (const int32_t*)(base + o_cexp);
  da.partials = (const double2*)(base + o_part);
  da.out = out_counts_d;
  const int draw_grid_cap = 16 * num_sms();

  for (int64_t s0 = 0; s0 < count; s0 += W) {
    const int64_t nw = std::min(W, count - s0);
    da.s0 = s0;
    da.nsamp = nw;
    sa.nsamp = nw;
    for (int k = 1; k <= n; ++k) {
      da.k = k;
      da.K = 1;
      da.chunks = 1;
      if (k >= 2) {
        const StepPlan p = plan_step(k, nw, target_ctas);
        sa.k = k;
        sa.L = p.L;
        sa.Hb = p.Hb;
        sa.chunks = p.chunks;
        const int rc = precision == kPrecFloatFloat ? sub_dispatch<ArDD>(p, sa, s)
                       : precision == kPrecFP64     ? sub_dispatch<ArFX>(p, sa, s)
                                                    : sub_dispatch<ArF32>(p, sa, s);
        if (rc != 0) {
          set_error("CC2017 sub-permanent launch failed: %s", cudaGetErrorString((cudaError_t)rc));
          return PCVL_ERR_CUDA;
        }
        da.K = p.K;
        da.chunks = p.chunks;
      }
      cc_draw_kernel<<<(unsigned)std::min<int64_t>(nw, draw_grid_cap), kDrawThreads, 0, s>>>(da);
      PCVL_CUDA(cudaGetLastError());
    }
  }
  return PCVL_OK;
}

extern "C" int pcvl_cc2017_sample(const double* u_d, int32_t m, const int32_t* input_state_h, int64_t count,
                                  uint64_t seed, uint64_t first_sample, int32_t precision, int32_t* out_counts_d,
                                  void* stream_) {
  PCVL_CHECK(count >= 0, "count must be >= 0");
  return cc2017_run(u_d, m, 1, input_state_h, &count, seed, first_sample, precision, out_counts_d,
                    (cudaStream_t)stream_);
}

extern "C" int pcvl_cc2017_sample_multi(const double* u_d, int32_t m, int32_t nstates, const int32_t* input_states_h,
                                        const int64_t* counts_h, uint64_t seed, uint64_t first_sample,
                                        int32_t precision, int32_t* out_counts_d, void* stream_) {
  return cc2017_run(u_d, m, nstates, input_states_h, counts_h, seed, first_sample, precision, out_counts_d,
                    (cudaStream_t)stream_);
}
