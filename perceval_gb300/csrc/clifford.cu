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
//      (Glynn over the k-1 row signs, all l at once through prefix/suffix products of
//      the column sums), weigh every output mode i by
//          w_i = |sum_l U[i, cols[l]] sub_l|^2
//      (Laplace expansion of the k x k permanent along the new row), and draw r_{k-1}
//      with probability w_i / sum w (uniform from Philox counter (sample, k, 0); the
//      first i whose running sum exceeds u * sum w, summed in index order);
//   3. the sample is the histogram of the rows.
// The common factor 2^{2-k} of the Glynn sums and a power-of-two scaling of U cancel
// in the normalisation and are dropped.
//
// One CTA per sample (grid-stride).  Step k splits the 2^{k-2} sign patterns into
// lo bits (a shared table of column-sum parts, as in the permanent kernel) and hi
// bits spread over the threads; each thread keeps its k accumulators in shared memory.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {

// ------------------------------------------------------------ arithmetic policies
struct ArDD {  // float-float (FP64-class); products and sums stay unnormalised in the
               // Glynn loop (bounded low parts, see cdd_mul_lazy), accumulators exact
  using C = cdd;
  using Acc = cdd;
  static __device__ __forceinline__ C zero() { return cdd_zero(); }
  static __device__ __forceinline__ C one() { return cdd_one(); }
  static __device__ __forceinline__ C add(C a, C b) { return cdd_add_lazy(a, b); }
  static __device__ __forceinline__ C sub(C a, C b) { return cdd_sub(a, b); }
  static __device__ __forceinline__ C mul(C a, C b) { return cdd_mul_lazy(a, b); }
  static __device__ __forceinline__ C neg(C a) { return cdd_neg(a); }
  static __device__ __forceinline__ C twice(C a) { return cdd_ldexp(a, 1); }
  static __device__ __forceinline__ C from(double2 v) { return cdd_from(v.x, v.y); }
  static __device__ __forceinline__ Acc acc_zero() { return cdd_zero(); }
  static __device__ __forceinline__ void acc_add(Acc& a, C x) { a = cdd_add(a, x); }
  static __device__ __forceinline__ Acc acc_merge(Acc a, Acc b) { return cdd_add(a, b); }
  static __device__ __forceinline__ C acc_value(Acc a) { return a; }
  static __device__ __forceinline__ double norm2(C a) {
    const dd r = dd_add(dd_mul(a.re, a.re), dd_mul(a.im, a.im));
    return dd_to_double(r);
  }
  static __device__ __forceinline__ C scale(C a, int e) { return cdd_ldexp(a, e); }
  static __device__ __forceinline__ float mag(C a) { return fabsf(a.re.hi) + fabsf(a.im.hi); }
};

struct f4 {
  float sr, cr, si, ci;  // Kahan-compensated complex: sum and compensation
};
struct ArF32 {  // FP32 with compensated accumulation
  using C = float2;
  using Acc = f4;
  static __device__ __forceinline__ C zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ C one() { return make_float2(1.f, 0.f); }
  static __device__ __forceinline__ C add(C a, C b) { return make_float2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ C sub(C a, C b) { return make_float2(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ C mul(C a, C b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
  }
  static __device__ __forceinline__ C neg(C a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ C twice(C a) { return make_float2(2.f * a.x, 2.f * a.y); }
  static __device__ __forceinline__ C from(double2 v) { return make_float2((float)v.x, (float)v.y); }
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
  static __device__ __forceinline__ Acc acc_merge(Acc a, Acc b) {
    kahan(a.sr, a.cr, b.sr);
    kahan(a.sr, a.cr, -b.cr);
    kahan(a.si, a.ci, b.si);
    kahan(a.si, a.ci, -b.ci);
    return a;
  }
  static __device__ __forceinline__ C acc_value(Acc a) { return make_float2(a.sr - a.cr, a.si - a.ci); }
  static __device__ __forceinline__ double norm2(C a) {
    return (double)a.x * (double)a.x + (double)a.y * (double)a.y;
  }
  static __device__ __forceinline__ C scale(C a, int e) { return make_float2(ldexpf(a.x, e), ldexpf(a.y, e)); }
  static __device__ __forceinline__ float mag(C a) { return fabsf(a.x) + fabsf(a.y); }
};

struct CCArgs {
  const void* uc;        // converted, scaled U (Ar::C), row-major m x m
  int m, n;
  const int32_t* cols0;  // input columns (n entries, ascending)
  int64_t count;
  uint32_t k0, k1;       // Philox key (seed)
  uint64_t first;
  int32_t* out;          // count x m
};

constexpr int kCCThreads = 128;

template <class Ar>
__global__ void cc_convert(const double2* __restrict__ u, int m, double scale, typename Ar::C* __restrict__ uc) {
  const int tot = m * m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) {
    double2 v = u[i];
    v.x *= scale;
    v.y *= scale;
    uc[i] = Ar::from(v);
  }
}

template <class Ar, int KMAX>
__global__ void __launch_bounds__(kCCThreads) cc2017_kernel(CCArgs a) {
  using C = typename Ar::C;
  using Acc = typename Ar::Acc;
  extern __shared__ __align__(16) unsigned char smem[];
  const int m = a.m, n = a.n, tid = threadIdx.x;
  constexpr int LMAX = 6;
  // shared layout
  C* Bm = reinterpret_cast<C*>(smem);                        // KMAX x KMAX
  C* Tb = Bm + KMAX * KMAX;                                  // (1 << LMAX) x KMAX
  C* sub = Tb + (1 << LMAX) * KMAX;                          // KMAX
  Acc* accs = reinterpret_cast<Acc*>(sub + KMAX);            // KMAX x threads
  double* w = reinterpret_cast<double*>(accs + KMAX * kCCThreads);  // m
  int* cols = reinterpret_cast<int*>(w + m);                 // KMAX
  int* rows = cols + KMAX;                                   // KMAX
  int* cexp = rows + KMAX;                                   // KMAX column exponents
  int* sexp = cexp + KMAX;                                   // KMAX sub-permanent exponents
  const C* U = reinterpret_cast<const C*>(a.uc);

  for (int64_t s = blockIdx.x; s < a.count; s += gridDim.x) {
    const uint64_t sid = a.first + (uint64_t)s;
    const uint32_t s_lo = (uint32_t)sid, s_hi = (uint32_t)(sid >> 32);
    if (tid == 0) {
      for (int l = 0; l < n; ++l) cols[l] = a.cols0[l];
      for (int q = n - 1; q >= 1; --q) {
        const u4 r = philox4x32_10({s_lo, s_hi, 0xffffffffu, (uint32_t)q}, a.k0, a.k1);
        const int j = (int)mulhi32(r.x, (uint32_t)(q + 1));
        const int t = cols[q];
        cols[q] = cols[j];
        cols[j] = t;
      }
    }
    __syncthreads();

    for (int k = 1; k <= n; ++k) {
      const int d = k - 1;  // rows chosen so far
      if (k == 1) {
        if (tid == 0) sub[0] = Ar::one();
        __syncthreads();
      } else {
        for (int e = tid; e < d * k; e += blockDim.x) {
          const int r = e / k, c = e - r * k;
          Bm[r * KMAX + c] = U[(size_t)rows[r] * m + cols[c]];
        }
        const int F = d - 1;  // free sign bits (row 0 fixed to +1)
        const int L = min(LMAX, max(0, F - 7));
        const int Hb = F - L;
        __syncthreads();
        // Scale column c by 2^e_c so that its l1 norm lies in [2^(c0-1), 2^c0) with
        // (k - 1) c0 + (k - 2) <= 120: every product of k - 1 column sums times the
        // 2^(k-2) terms of the sum stays inside the FP32 range (a global scaling of U
        // does not: aligned columns reach 1e56 at n = 30).  Exact (powers of two);
        // undone below through the sub-permanent exponents.
        if (tid < k) {
          float l1 = 0.f;
          for (int r = 0; r < d; ++r) l1 += Ar::mag(Bm[r * KMAX + tid]);
          const int c0 = min(4, (120 - (k - 2)) / (k - 1));
          int ex = 0;
          if (l1 > 0.f) frexpf(l1, &ex);
          const int e = l1 > 0.f ? c0 - ex : 0;
          cexp[tid] = e;
          for (int r = 0; r < d; ++r) Bm[r * KMAX + tid] = Ar::scale(Bm[r * KMAX + tid], e);
        }
        __syncthreads();
        // lo table over rows 1..L
        for (int c = tid; c < k; c += blockDim.x) {
          C t0 = Ar::zero();
          for (int l = 0; l < L; ++l) t0 = Ar::add(t0, Bm[(1 + l) * KMAX + c]);
          Tb[c] = t0;
        }
        __syncthreads();
        for (int l = 0; l < L; ++l) {
          const int half = 1 << l;
          for (int e = tid; e < half * k; e += blockDim.x) {
            const int b = e / k, c = e - b * k;
            Tb[(b + half) * KMAX + c] = Ar::sub(Tb[b * KMAX + c], Ar::twice(Bm[(1 + l) * KMAX + c]));
          }
          __syncthreads();
        }
        for (int l = 0; l < k; ++l) accs[l * kCCThreads + tid] = Ar::acc_zero();
        const uint64_t nhi = 1ull << Hb;
        for (uint64_t h = tid; h < nhi; h += blockDim.x) {
          C H[KMAX];
#pragma unroll
          for (int c = 0; c < KMAX; ++c) {
            if (c < k) {
              C v = Bm[c];  // row 0, sign +1
              for (int t = 0; t < Hb; ++t) {
                const C x = Bm[(1 + L + t) * KMAX + c];
                v = ((h >> t) & 1ull) ? Ar::sub(v, x) : Ar::add(v, x);
              }
              H[c] = v;
            }
          }
          const int hsign = __popcll(h) & 1;
          for (int b = 0; b < (1 << L); ++b) {
            const C* Tr = Tb + b * KMAX;
            C suf[KMAX + 1];
            suf[KMAX] = Ar::one();
#pragma unroll
            for (int c = KMAX - 1; c >= 0; --c) suf[c] = (c < k) ? Ar::mul(Ar::add(H[c], Tr[c]), suf[c + 1]) : suf[c + 1];
            const bool neg = (__popc(b) & 1) ^ hsign;
            C pre = Ar::one();
#pragma unroll
            for (int l = 0; l < KMAX; ++l) {
              if (l < k) {
                C term = Ar::mul(pre, suf[l + 1]);
                if (neg) term = Ar::neg(term);
                Acc acc = accs[l * kCCThreads + tid];
                Ar::acc_add(acc, term);
                accs[l * kCCThreads + tid] = acc;
                pre = Ar::mul(pre, Ar::add(H[l], Tr[l]));
              }
            }
          }
        }
        __syncthreads();
        for (int l = tid; l < k; l += blockDim.x) {
          Acc tot = accs[l * kCCThreads];
          for (int t = 1; t < kCCThreads; ++t) tot = Ar::acc_merge(tot, accs[l * kCCThreads + t]);
          sub[l] = Ar::acc_value(tot);
          // true sub_l is proportional to sub_l * 2^{e_l} (the scales of the other
          // columns are common to all l); record its binary exponent
          const float mg = Ar::mag(sub[l]);
          int ex = 0;
          if (mg > 0.f) frexpf(mg, &ex);
          sexp[l] = mg > 0.f ? ex + cexp[l] : INT_MIN;
        }
        __syncthreads();
        if (tid < k) {
          int emax = INT_MIN;
          for (int l = 0; l < k; ++l) emax = max(emax, sexp[l]);
          // largest |sub_l| near 1: the weights below cannot overflow
          sub[tid] = sexp[tid] == INT_MIN ? Ar::zero() : Ar::scale(sub[tid], cexp[tid] - emax);
        }
        __syncthreads();
      }
      // weights of every output mode for the next photon
      for (int i = tid; i < m; i += blockDim.x) {
        C z = Ar::zero();
        for (int l = 0; l < k; ++l) z = Ar::add(z, Ar::mul(U[(size_t)i * m + cols[l]], sub[l]));
        w[i] = Ar::norm2(z);
      }
      __syncthreads();
      if (tid == 0) {
        double W = 0.0;
        for (int i = 0; i < m; ++i) W += w[i];
        const u4 r = philox4x32_10({s_lo, s_hi, (uint32_t)k, 0u}, a.k0, a.k1);
        const double target = u01_from(r.x, r.y) * W;
        double run = 0.0;
        int pick = -1, last_pos = 0;
        for (int i = 0; i < m; ++i) {
          if (w[i] > 0.0) last_pos = i;
          run += w[i];
          if (run > target) {
            pick = i;
            break;
          }
        }
        rows[k - 1] = pick >= 0 ? pick : last_pos;
      }
      __syncthreads();
    }
    int32_t* o = a.out + (size_t)s * m;
    for (int i = tid; i < m; i += blockDim.x) o[i] = 0;
    __syncthreads();
    if (tid == 0)
      for (int k = 0; k < n; ++k) o[rows[k]] += 1;
    __syncthreads();
  }
}

template <class Ar, int KMAX>
static size_t cc_smem(int m) {
  using C = typename Ar::C;
  size_t b = sizeof(C) * (KMAX * KMAX + (1 << 6) * KMAX + KMAX);
  b += sizeof(typename Ar::Acc) * KMAX * kCCThreads;
  b += sizeof(double) * m + sizeof(int) * 4 * KMAX;
  return b;
}

template <class Ar, int KMAX>
static int cc_launch(const CCArgs& a, cudaStream_t s) {
  const size_t smem = cc_smem<Ar, KMAX>(a.m);
  cudaError_t e = cudaFuncSetAttribute(cc2017_kernel<Ar, KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cc2017_kernel<Ar, KMAX>, kCCThreads, smem);
  if (e != cudaSuccess) return (int)e;
  const int64_t grid = std::min<int64_t>(a.count, (int64_t)num_sms() * std::max(1, per_sm));
  cc2017_kernel<Ar, KMAX><<<(unsigned)grid, kCCThreads, smem, s>>>(a);
  return (int)cudaGetLastError();
}

template <class Ar>
static int cc_dispatch(const CCArgs& a, cudaStream_t s) {
  if (a.n <= 8) return cc_launch<Ar, 8>(a, s);
  if (a.n <= 16) return cc_launch<Ar, 16>(a, s);
  if (a.n <= 24) return cc_launch<Ar, 24>(a, s);
  return cc_launch<Ar, 32>(a, s);
}

}  // namespace pcvl

using namespace pcvl;

extern "C" int pcvl_cc2017_sample(const double* u_d, int32_t m, const int32_t* input_state_h, int64_t count,
                                  uint64_t seed, uint64_t first_sample, int32_t precision, int32_t* out_counts_d,
                                  void* stream_) {
  cudaStream_t s = (cudaStream_t)stream_;
  PCVL_CHECK(u_d && input_state_h && out_counts_d, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= 2048, "m=%d outside [1, 2048]", m);
  PCVL_CHECK(count >= 0, "count must be >= 0");
  PCVL_CHECK(precision == 0 || precision == 1, "precision must be 0 (float-float) or 1 (FP32)");
  std::vector<int32_t> cols;
  for (int i = 0; i < m; ++i) {
    PCVL_CHECK(input_state_h[i] >= 0, "negative photon count in input state");
    for (int v = 0; v < input_state_h[i]; ++v) cols.push_back(i);
  }
  const int n = (int)cols.size();
  PCVL_CHECK(n <= 32, "n=%d photons exceeds 32", n);
  if (count == 0) return PCVL_OK;
  if (n == 0) {
    PCVL_CUDA(cudaMemsetAsync(out_counts_d, 0, (size_t)count * m * sizeof(int32_t), s));
    return PCVL_OK;
  }
  const size_t csz = precision == 0 ? sizeof(cdd) : sizeof(float2);
  const size_t o_cols = align_up((size_t)m * m * csz, 256);
  void* ws = nullptr;
  PCVL_TRY(workspace(WS_CC2017, o_cols + 256, &ws));
  unsigned char* base = (unsigned char*)ws;
  PCVL_TRY(stage_h2d(cols.data(), cols.size() * sizeof(int32_t), base + o_cols, s));
  // |U_ij| ~ m^{-1/2} for Haar unitaries: scale by 2^round(log2 sqrt m) (exact), which
  // keeps the column-sum products near 1 and cancels in the normalisation
  const double scale = std::ldexp(1.0, (int)std::lround(0.5 * std::log2((double)m)));
  const int cgrid = std::max(1, std::min(1024, (m * m + 255) / 256));
  if (precision == 0)
    cc_convert<ArDD><<<cgrid, 256, 0, s>>>((const double2*)u_d, m, scale, (cdd*)base);
  else
    cc_convert<ArF32><<<cgrid, 256, 0, s>>>((const double2*)u_d, m, scale, (float2*)base);
  PCVL_CUDA(cudaGetLastError());
  CCArgs a{};
  a.uc = base;
  a.m = m;
  a.n = n;
  a.cols0 = (const int32_t*)(base + o_cols);
  a.count = count;
  a.k0 = (uint32_t)seed;
  a.k1 = (uint32_t)(seed >> 32);
  a.first = first_sample;
  a.out = out_counts_d;
  const int rc = precision == 0 ? cc_dispatch<ArDD>(a, s) : cc_dispatch<ArF32>(a, s);
  if (rc != 0) {
    set_error("CC2017 kernel launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return PCVL_ERR_CUDA;
  }
  return PCVL_OK;
}
