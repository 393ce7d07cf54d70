// Glynn / Ryser permanent kernel, one instantiation per matrix size N.
//
// Work split.  The n - 1 free Glynn signs (all n Ryser subset bits) are split into
// L "lo" bits enumerated by every thread's inner loop and H "hi" bits that select
// the thread's pattern.  With the outer sum r_i(hi, lo) = H_i(hi) + T_i(lo), each
// step costs n complex adds (the row sums are rebuilt from two exact-ish parts, so
// no Gray-code drift accumulates) and n - 1 complex multiplies in a balanced tree.
// The table T (2^L x n, in shared memory) is read with warp-broadcast loads.
//
//   Glynn (Glynn 2010):  perm(A) = 2^{1-n} sum_{d in {+-1}^n, d_0 = 1} (prod_k d_k)
//                                   prod_i sum_j d_j a_ij
//   Ryser (Ryser 1963):  perm(A) = (-1)^n sum_{S subset [n]} (-1)^{|S|} prod_i sum_{j in S} a_ij
//
// Bit layout.  Glynn: lo bit l is the sign of column 1 + l, hi bit t the sign of
// column 1 + L + t (bit set = -1).  Ryser: lo bit l includes column l, hi bit t
// column L + t.  Term sign = (-1)^(popc(lo) + popc(hi)) in both.
//
// Work item = (matrix of the bin, chunk of threads * P consecutive hi patterns);
// each CTA writes one FP64 partial sum; pcvl_perm_reduce adds the partials of a
// matrix with compensation and applies the 2^{1-n} (or (-1)^n) and row-scaling
// factors.
//
// Three arithmetics share this layout (16 bytes per prepared element in each):
//  * FP64 precision (perm_bin_fx, the default): exact fixed-point row sums on the
//    integer pipe; each sign vector's product split between an FP64 DMUL/DFMA tree and
//    a 64-bit block-floating tree on the integer pipes (blockfloat.cuh), the two halves
//    meeting in the signed accumulation; each hi pattern's lo sweep added to a
//    Neumaier-compensated FP64 sum.  The hi patterns of a thread are walked in
//    Gray-code order, so consecutive patterns differ in one column.
//  * FP64 with FP64 row sums (perm_bin_f64): the same with the row sums and their
//    Gray-code updates in DADD / DFMA (H rebuilt exactly every 32 patterns).
//  * float-float (perm_bin_kernel): every value an unevaluated pair of FP32 numbers on
//    the FP32 pipe (~48 significant bits), several times faster on GB300, opt-in.
#pragma once
#include "common.cuh"
#include "blockfloat.cuh"

namespace pcvl {

struct PermBinArgs {
  const void* A;          // prepared (scaled) matrices: cdd (float-float) or double2 (FP64)
  const int64_t* offs;    // element offset of each matrix in A (global matrix index)
  const int32_t* mids;    // matrix ids of this bin
  int32_t nmat;           // matrices in the bin
  int32_t L;              // lo bits
  int32_t Hbits;          // hi bits
  int64_t P;              // hi patterns per thread per item
  int64_t items_per_mat;  // CTAs per matrix
  int32_t ryser;          // 0 Glynn, 1 Ryser
  int32_t prec;           // kPrecFP64 (exact row sums), kPrecFP64Dadd or kPrecFloatFloat
  double2* partials;      // one per item, bin-local indexing
  cudaStream_t stream;
};

constexpr int kPermThreads = 128;

// prod_i (H_i + T_i) over rows [LO, HI) as a balanced tree.  Glynn uses the lazy
// float-float operations; Ryser, whose alternating subset sum cancels far more, keeps
// every intermediate normalised.
template <int LO, int HI, bool LAZY>
struct RowProd {
  static __device__ __forceinline__ cdd run(const cdd* H, const cdd* Tb) {
    if constexpr (HI - LO == 1) {
      return LAZY ? cdd_add_lazy(H[LO], Tb[LO]) : cdd_add(H[LO], Tb[LO]);
    } else {
      constexpr int MID = (LO + HI) / 2;
      const cdd a = RowProd<LO, MID, LAZY>::run(H, Tb);
      const cdd b = RowProd<MID, HI, LAZY>::run(H, Tb);
      return LAZY ? cdd_mul_lazy(a, b) : cdd_mul(a, b);
    }
  }
};

// signed sum over the lo patterns of one hi pattern
template <int N, bool LAZY>
__device__ __forceinline__ void lo_sweep(const cdd* H, const cdd* T, int nsteps, int hsign, float& arh, float& arl,
                                         float& aih, float& ail) {
  for (int b = 0; b < nsteps; ++b) {
    cdd prod = RowProd<0, N, LAZY>::run(H, T + b * N);
    if ((__popc(b) & 1) ^ hsign) prod = cdd_neg(prod);
    const dd r = two_sum(arh, prod.re.hi);
    const dd i = two_sum(aih, prod.im.hi);
    arh = r.hi;
    arl += r.lo + prod.re.lo;
    aih = i.hi;
    ail += i.lo + prod.im.lo;
  }
}

__device__ __forceinline__ cdd shfl_down_cdd(cdd v, int d) {
  cdd r;
  r.re.hi = __shfl_down_sync(0xffffffffu, v.re.hi, d);
  r.re.lo = __shfl_down_sync(0xffffffffu, v.re.lo, d);
  r.im.hi = __shfl_down_sync(0xffffffffu, v.im.hi, d);
  r.im.lo = __shfl_down_sync(0xffffffffu, v.im.lo, d);
  return r;
}

template <int N>
__global__ void __launch_bounds__(kPermThreads) perm_bin_kernel(PermBinArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cdd* As = reinterpret_cast<cdd*>(smem_raw);  // N x N
  cdd* T = As + N * N;                         // (1 << L) x N
  __shared__ cdd red[kPermThreads / 32];

  const int64_t item = blockIdx.x;
  const int64_t mat_local = item / a.items_per_mat;
  const int64_t chunk = item - mat_local * a.items_per_mat;
  const int mid = a.mids[mat_local];
  const cdd* A = static_cast<const cdd*>(a.A) + a.offs[mid];
  const int L = a.L;
  const int ryser = a.ryser;
  const int tid = threadIdx.x;

  for (int e = tid; e < N * N; e += blockDim.x) As[e] = A[e];
  __syncthreads();

  // table: T[b][i] = lo part of row sum i for lo pattern b, built level by level
  const int lo_col0 = ryser ? 0 : 1;
  for (int i = tid; i < N; i += blockDim.x) {
    cdd t0 = cdd_zero();
    if (!ryser)
      for (int l = 0; l < L; ++l) t0 = cdd_add(t0, As[i * N + lo_col0 + l]);
    T[i] = t0;
  }
  __syncthreads();
  for (int l = 0; l < L; ++l) {
    const int half = 1 << l;
    for (int e = tid; e < half * N; e += blockDim.x) {
      const int b = e / N, i = e - b * N;
      cdd d = As[i * N + lo_col0 + l];
      if (!ryser) d = cdd_ldexp(cdd_neg(d), 1);
      T[(b + half) * N + i] = cdd_add(T[b * N + i], d);
    }
    __syncthreads();
  }

  const uint64_t nhi = 1ull << a.Hbits;
  const uint64_t h0 = (uint64_t)chunk * (uint64_t)(kPermThreads * a.P) + (uint64_t)tid * a.P;
  const int hi_col0 = ryser ? L : 1 + L;
  const int nsteps = 1 << L;
  // signed sum of the products: high parts through two_sum, the rest in float
  float arh = 0.f, arl = 0.f, aih = 0.f, ail = 0.f;

  for (int64_t p = 0; p < a.P; ++p) {
    const uint64_t h = h0 + p;
    if (h >= nhi) break;
    cdd H[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      cdd v = ryser ? cdd_zero() : As[i * N];
      for (int t = 0; t < a.Hbits; ++t) {
        const cdd x = As[i * N + hi_col0 + t];
        const bool bit = (h >> t) & 1ull;
        if (ryser) {
          if (bit) v = cdd_add(v, x);
        } else {
          v = cdd_add(v, bit ? cdd_neg(x) : x);
        }
      }
      H[i] = v;
    }
    const int hsign = __popcll(h) & 1;
    if (ryser)
      lo_sweep<N, false>(H, T, nsteps, hsign, arh, arl, aih, ail);
    else
      lo_sweep<N, true>(H, T, nsteps, hsign, arh, arl, aih, ail);
    // fold the low parts in every hi pattern so they stay small
    const dd r = two_sum(arh, arl);
    const dd i = two_sum(aih, ail);
    arh = r.hi;
    arl = r.lo;
    aih = i.hi;
    ail = i.lo;
  }
  cdd acc = {{arh, arl}, {aih, ail}};

  // block reduction (df64), one FP64 partial per CTA
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc = cdd_add(acc, shfl_down_cdd(acc, d));
  if ((tid & 31) == 0) red[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    cdd s = red[0];
    for (int w = 1; w < kPermThreads / 32; ++w) s = cdd_add(s, red[w]);
    a.partials[item] = make_double2(dd_to_double(s.re), dd_to_double(s.im));
  }
}


// ------------------------------------------------------------------ FP64 arithmetic
__device__ __forceinline__ double2 cmul64(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// x with its sign bit XORed with s (0 or 0x80000000): one integer op on the high word
__device__ __forceinline__ double flip64(double x, uint32_t s) {
  return __hiloint2double(__double2hiint(x) ^ (int)s, __double2loint(x));
}
// Neumaier-compensated accumulation s + c += x
__device__ __forceinline__ void comp_add(double& s, double& c, double x) {
  const double t = s + x;
  c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
  s = t;
}

// prod_{i in [LO, HI)} (H_i + T_i) in FP64 as a balanced tree
template <int LO, int HI>
struct RowProd64 {
  static __device__ __forceinline__ double2 run(const double2* H, const double2* Tb) {
    if constexpr (HI - LO == 1) {
      const double2 t = Tb[LO];
      return make_double2(H[LO].x + t.x, H[LO].y + t.y);
    } else {
      constexpr int MID = (LO + HI) / 2;
      const double2 x = RowProd64<LO, MID>::run(H, Tb);
      const double2 y = RowProd64<MID, HI>::run(H, Tb);
      return cmul64(x, y);
    }
  }
};

// signed sum over the lo patterns of one hi pattern: the last product of the tree is
// fused into the accumulation (four DFMA), its sign applied to one factor's sign bits
template <int N>
__device__ __forceinline__ void lo_sweep64(const double2* H, const double2* T, int nsteps, uint32_t hsign,
                                           double& sr, double& si) {
  for (int b = 0; b < nsteps; ++b) {
    const double2* Tb = T + b * N;
    const uint32_t s = (((uint32_t)__popc(b) ^ hsign) & 1u) << 31;
    if constexpr (N == 1) {
      sr += flip64(H[0].x + Tb[0].x, s);
      si += flip64(H[0].y + Tb[0].y, s);
    } else {
      constexpr int MID = N / 2;
      double2 x = RowProd64<0, MID>::run(H, Tb);
      const double2 y = RowProd64<MID, N>::run(H, Tb);
      x.x = flip64(x.x, s);
      x.y = flip64(x.y, s);
      sr = fma(x.x, y.x, sr);
      sr = fma(-x.y, y.y, sr);
      si = fma(x.x, y.y, si);
      si = fma(x.y, y.x, si);
    }
  }
}

// Hi pattern g of row i: Glynn a_i0 + sum_t (bit t ? -1 : +1) a_{i, 1 + L + t};
// Ryser sum over set bits of a_{i, L + t}
template <int N>
__device__ __forceinline__ double2 hi_row64(const double2* As, int i, uint64_t g, int Hbits, int hi_col0,
                                            int ryser) {
  double2 v = ryser ? make_double2(0.0, 0.0) : As[i * N];
  for (int t = 0; t < Hbits; ++t) {
    const double2 x = As[i * N + hi_col0 + t];
    const bool bit = (g >> t) & 1ull;
    if (ryser) {
      if (bit) {
        v.x += x.x;
        v.y += x.y;
      }
    } else {
      v.x += bit ? -x.x : x.x;
      v.y += bit ? -x.y : x.y;
    }
  }
  return v;
}

template <int N>
__global__ void __launch_bounds__(kPermThreads) perm_bin_f64(PermBinArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* As = reinterpret_cast<double2*>(smem_raw);  // N x N
  double2* T = As + N * N;                             // (1 << L) x N
  __shared__ double red[4][kPermThreads / 32];

  const int64_t item = blockIdx.x;
  const int64_t mat_local = item / a.items_per_mat;
  const int64_t chunk = item - mat_local * a.items_per_mat;
  const int mid = a.mids[mat_local];
  const double2* A = static_cast<const double2*>(a.A) + a.offs[mid];
  const int L = a.L;
  const int ryser = a.ryser;
  const int tid = threadIdx.x;

  for (int e = tid; e < N * N; e += blockDim.x) As[e] = A[e];
  __syncthreads();

  // table: T[b][i] = lo part of row sum i for lo pattern b, built level by level
  const int lo_col0 = ryser ? 0 : 1;
  for (int i = tid; i < N; i += blockDim.x) {
    double2 t0 = make_double2(0.0, 0.0);
    if (!ryser)
      for (int l = 0; l < L; ++l) {
        t0.x += As[i * N + lo_col0 + l].x;
        t0.y += As[i * N + lo_col0 + l].y;
      }
    T[i] = t0;
  }
  __syncthreads();
  for (int l = 0; l < L; ++l) {
    const int half = 1 << l;
    for (int e = tid; e < half * N; e += blockDim.x) {
      const int b = e / N, i = e - b * N;
      const double2 d = As[i * N + lo_col0 + l];
      const double c = ryser ? 1.0 : -2.0;
      T[(b + half) * N + i] = make_double2(fma(c, d.x, T[b * N + i].x), fma(c, d.y, T[b * N + i].y));
    }
    __syncthreads();
  }

  const uint64_t nhi = 1ull << a.Hbits;
  const uint64_t h0 = (uint64_t)chunk * (uint64_t)(kPermThreads * a.P) + (uint64_t)tid * a.P;
  const int hi_col0 = ryser ? L : 1 + L;
  const int nsteps = 1 << L;
  double Sr = 0.0, Cr = 0.0, Si = 0.0, Ci = 0.0;
  double2 H[N];
  for (int64_t p = 0; p < a.P; ++p) {
    const uint64_t h = h0 + p;
    if (h >= nhi) break;
    const uint64_t g = h ^ (h >> 1);  // Gray code: g(h) and g(h - 1) differ in bit ctz(h)
    if ((p & 31) == 0) {
#pragma unroll
      for (int i = 0; i < N; ++i) H[i] = hi_row64<N>(As, i, g, a.Hbits, hi_col0, ryser);
    } else {
      const int t = __ffsll((long long)h) - 1;
      const bool set = (g >> t) & 1ull;
      const double c = ryser ? (set ? 1.0 : -1.0) : (set ? -2.0 : 2.0);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const double2 x = As[i * N + hi_col0 + t];
        H[i].x = fma(c, x.x, H[i].x);
        H[i].y = fma(c, x.y, H[i].y);
      }
    }
    double sr = 0.0, si = 0.0;
    lo_sweep64<N>(H, T, nsteps, (uint32_t)(__popcll(g) & 1), sr, si);
    comp_add(Sr, Cr, sr);
    comp_add(Si, Ci, si);
  }

  // block reduction of the compensated pairs, one FP64 partial per CTA
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const double or_ = __shfl_down_sync(0xffffffffu, Sr, d), oc = __shfl_down_sync(0xffffffffu, Cr, d);
    const double oi = __shfl_down_sync(0xffffffffu, Si, d), od = __shfl_down_sync(0xffffffffu, Ci, d);
    Cr += oc;
    comp_add(Sr, Cr, or_);
    Ci += od;
    comp_add(Si, Ci, oi);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = Sr;
    red[1][tid >> 5] = Cr;
    red[2][tid >> 5] = Si;
    red[3][tid >> 5] = Ci;
  }
  __syncthreads();
  if (tid == 0) {
    double sr = red[0][0], cr = red[1][0], si = red[2][0], ci = red[3][0];
    for (int w = 1; w < kPermThreads / 32; ++w) {
      cr += red[1][w];
      comp_add(sr, cr, red[0][w]);
      ci += red[3][w];
      comp_add(si, ci, red[2][w]);
    }
    a.partials[item] = make_double2(sr + cr, si + ci);
  }
}

// ------------------------------------------------------------------ exact row sums
// The FP64 default (perm_bin_fx) keeps every row sum exact: the prepared matrix holds
// each scaled element as a 64-bit fixed-point integer (value 2^F x element, F = 62 - c,
// so every row sum, |r| < 2^c, stays below 2^62), the lo table, the hi parts and their
// Gray-code updates are integer additions on the integer pipe.  The product of a sign
// vector's row sums splits in two (fx_int_rows below): the first rows are converted to
// FP64 once by the hardware's round-to-nearest-even conversion (RowProdCV, unscaled) and
// multiplied by the FP64 tree above; the others are multiplied in 64-bit block floating
// point on the integer pipes (62 significant bits) and converted once.  The two halves
// meet in the compensated FP64 accumulation, so the row sums carry no rounding and every
// product at most an FP64 one.  Per sign vector the FP64 pipe issues 4 (n - KI)
// multiplies and n - KI conversions instead of the 6n - 4 instructions of FP64 row sums.
// With KI = 0 (every product in FP64, the configuration measured as the baseline of the
// split) the rows go through fx_to_f64 and RowProdFX instead.
template <int N>
struct FixedPoint {
  static constexpr int c = 20 < 120 / N ? 20 : 120 / N;  // row l1 norms in [2^(c-1), 2^c)
  static constexpr int F = 62 - c;                        // fixed-point fraction bits
};

// x 2^-F as a double, rounded to nearest even, from the binary64 format's definition
// (sign, 11-bit biased exponent, 52 stored mantissa bits) with integer operations only.
__device__ __forceinline__ double fx_to_f64(long long x, int F) {
  const unsigned long long ux = (unsigned long long)x;
  const unsigned long long sgn = ux & 0x8000000000000000ull;
  const unsigned long long ax = x < 0 ? 0ull - ux : ux;
  const int lz = __clzll((long long)ax);                 // 64 when ax == 0
  const unsigned long long mn = ax << (lz & 63);         // leading one at bit 63
  unsigned long long mant = mn >> 11;                    // 53 bits, leading one at bit 52
  const unsigned int rem = (unsigned int)mn & 0x7ffu;    // the 11 bits rounded away
  mant += (rem + (unsigned int)(mant & 1ull) + 0x3ffu) >> 11;  // up when rem > half, or = half and odd
  const unsigned long long e = (unsigned long long)(1023 + 63 - F - lz);
  const unsigned long long bits = sgn | ((e << 52) + mant - (1ull << 52));  // a carry out of mant bumps e
  return ax == 0 ? 0.0 : __longlong_as_double((long long)bits);
}

template <int LO, int HI, int F>
struct RowProdFX {
  static __device__ __forceinline__ double2 run(const longlong2* H, const longlong2* Tb) {
    if constexpr (HI - LO == 1) {
      const longlong2 t = Tb[LO];
      return make_double2(fx_to_f64(H[LO].x + t.x, F), fx_to_f64(H[LO].y + t.y, F));
    } else {
      constexpr int MID = (LO + HI) / 2;
      const double2 x = RowProdFX<LO, MID, F>::run(H, Tb);
      const double2 y = RowProdFX<MID, HI, F>::run(H, Tb);
      return cmul64(x, y);
    }
  }
};

// The FP64 rows of the split product, unscaled: each exact row sum (an integer, value x
// 2^F) is converted by the hardware's round-to-nearest-even int64 -> FP64 conversion, and
// the common factor 2^(-F (n - KI)) is applied once to the CTA's partial sums (a power of
// two: no rounding).  At most 14 rows of magnitude below 2^62 keep the product below 2^868.
template <int LO, int HI>
struct RowProdCV {
  static __device__ __forceinline__ double2 run(const longlong2* H, const longlong2* Tb) {
    if constexpr (HI - LO == 1) {
      const longlong2 t = Tb[LO];
      return make_double2(__ll2double_rn(H[LO].x + t.x), __ll2double_rn(H[LO].y + t.y));
    } else {
      constexpr int MID = (LO + HI) / 2;
      return cmul64(RowProdCV<LO, MID>::run(H, Tb), RowProdCV<MID, HI>::run(H, Tb));
    }
  }
};

template <int LO, int HI, int F>
struct RowProdBF {
  static __device__ __forceinline__ BFC run(const longlong2* H, const longlong2* Tb) {
    if constexpr (HI - LO == 1) {
      const longlong2 t = Tb[LO];
      return bf_norm(H[LO].x + t.x, H[LO].y + t.y, -F);
    } else {
      constexpr int MID = (LO + HI) / 2;
      return bf_mul(RowProdBF<LO, MID, F>::run(H, Tb), RowProdBF<MID, HI, F>::run(H, Tb));
    }
  }
};

// Rows whose product goes to the integer pipes in the FP64 kernel: rows [0, N - KI) are
// multiplied in FP64 (4 DFMA per complex product; GB300's FP64 pipe retires 2 per SM per
// clock), rows [N - KI, N) in 64-bit block floating point on the integer pipes (a product
// measured at 2.3x the FP64 product's rate), and the two partial products meet in the
// FP64 multiply-add that accumulates the sign vector's term, so both pipes work at once.
// Measured on the 8192-matrix batch (FP64 perms/s, built-in launch shapes), with the FP64
// rows converted by integer operations on their bits: KI = 0: 6710, N/4: 8262, N/3: 8828,
// N/2: 9411, 3N/5: 9665, 2N/3: 9798, 3N/4: 9181, N - 1: 7666 (the integer pipes then bound
// it); with the hardware conversion of RowProdCV, which takes that work off the integer
// pipes: 2N/3: 10917, 3N/4: 10742, 4N/5: 10827.
// Per size, the best of a second sweep over the FP64 rows d = N - KI in 4..8 (TFLOP/s of the
// size's bin in the batch, built-in launch shapes): n = 16: d = 5 (1.66 against 1.52 at 2N/3),
// 20: 6 (1.94 / 1.85), 22: 5 (1.90 / 1.79), 23: 7 (1.94 / 1.85); at 18, 21 and 24, 2N/3 was
// best or level.  The rates move irregularly with d (n = 22: 1.90, 1.61, 1.70, 1.79 for
// d = 5..8), the same in both sweeps, with how the two product trees split the rows.  Among
// single large permanents (d in {6, 8, 11, 13} against 2N/3): n = 26: d = 8 (1.88 against
// 1.82), 28: 6 (1.74 / 1.65), 34: 8 (1.52 / 1.47); at 30 and 32, 2N/3 was best.
template <int N>
__host__ __device__ constexpr int fx_int_rows() {
  return N == 16 ? 11 : N == 20 ? 14 : N == 22 ? 17 : N == 23 ? 16 : N == 26 ? 18 : N == 28 ? 22 : N == 34 ? 26
         : N >= 2 ? (2 * N) / 3 : 0;
}

template <int N>
__device__ __forceinline__ void lo_sweep_fx(const longlong2* H, const longlong2* T, int nsteps, uint32_t hsign,
                                            double& sr, double& si) {
  constexpr int F = FixedPoint<N>::F;
  constexpr int KI = fx_int_rows<N>();
  static_assert(KI >= 0 && KI < N, "at least one row of the product stays in FP64");
  static_assert(KI == 0 || 62 * (N - KI) + FixedPoint<N>::c * KI < 1000,
                "unscaled terms stay inside the FP64 range");
  for (int b = 0; b < nsteps; ++b) {
    const longlong2* Tb = T + b * N;
    const uint32_t s = (((uint32_t)__popc(b) ^ hsign) & 1u) << 31;
    if constexpr (KI > 0 && N > 1) {
      double2 x = RowProdCV<0, N - KI>::run(H, Tb);
      const BFC z = RowProdBF<N - KI, N, F>::run(H, Tb);
      const double2 y = make_double2(bf_to_f64(z.re, z.e), bf_to_f64(z.im, z.e));
      x.x = flip64(x.x, s);
      x.y = flip64(x.y, s);
      sr = fma(x.x, y.x, sr);
      sr = fma(-x.y, y.y, sr);
      si = fma(x.x, y.y, si);
      si = fma(x.y, y.x, si);
    } else if constexpr (N == 1) {
      sr += flip64(fx_to_f64(H[0].x + Tb[0].x, F), s);
      si += flip64(fx_to_f64(H[0].y + Tb[0].y, F), s);
    } else {
      constexpr int MID = N / 2;
      double2 x = RowProdFX<0, MID, F>::run(H, Tb);
      const double2 y = RowProdFX<MID, N, F>::run(H, Tb);
      x.x = flip64(x.x, s);
      x.y = flip64(x.y, s);
      sr = fma(x.x, y.x, sr);
      sr = fma(-x.y, y.y, sr);
      si = fma(x.x, y.y, si);
      si = fma(x.y, y.x, si);
    }
  }
}

template <int N>
__global__ void __launch_bounds__(kPermThreads) perm_bin_fx(PermBinArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  longlong2* As = reinterpret_cast<longlong2*>(smem_raw);  // N x N fixed-point elements
  longlong2* T = As + N * N;                               // (1 << L) x N
  __shared__ double red[4][kPermThreads / 32];

  const int64_t item = blockIdx.x;
  const int64_t mat_local = item / a.items_per_mat;
  const int64_t chunk = item - mat_local * a.items_per_mat;
  const int mid = a.mids[mat_local];
  const longlong2* A = static_cast<const longlong2*>(a.A) + a.offs[mid];
  const int L = a.L;
  const int ryser = a.ryser;
  const int tid = threadIdx.x;

  for (int e = tid; e < N * N; e += blockDim.x) As[e] = A[e];
  __syncthreads();

  const int lo_col0 = ryser ? 0 : 1;
  for (int i = tid; i < N; i += blockDim.x) {
    longlong2 t0 = make_longlong2(0, 0);
    if (!ryser)
      for (int l = 0; l < L; ++l) {
        t0.x += As[i * N + lo_col0 + l].x;
        t0.y += As[i * N + lo_col0 + l].y;
      }
    T[i] = t0;
  }
  __syncthreads();
  for (int l = 0; l < L; ++l) {
    const int half = 1 << l;
    for (int e = tid; e < half * N; e += blockDim.x) {
      const int b = e / N, i = e - b * N;
      const longlong2 d = As[i * N + lo_col0 + l];
      const longlong2 t = T[b * N + i];
      T[(b + half) * N + i] = ryser ? make_longlong2(t.x + d.x, t.y + d.y) : make_longlong2(t.x - 2 * d.x, t.y - 2 * d.y);
    }
    __syncthreads();
  }

  const uint64_t nhi = 1ull << a.Hbits;
  const uint64_t h0 = (uint64_t)chunk * (uint64_t)(kPermThreads * a.P) + (uint64_t)tid * a.P;
  const int hi_col0 = ryser ? L : 1 + L;
  const int nsteps = 1 << L;
  double Sr = 0.0, Cr = 0.0, Si = 0.0, Ci = 0.0;
  longlong2 H[N];
  for (int64_t p = 0; p < a.P; ++p) {
    const uint64_t h = h0 + p;
    if (h >= nhi) break;
    const uint64_t g = h ^ (h >> 1);  // Gray code: g(h) and g(h - 1) differ in bit ctz(h)
    if (p == 0) {                     // integer updates are exact: one build per thread
#pragma unroll
      for (int i = 0; i < N; ++i) {
        longlong2 v = ryser ? make_longlong2(0, 0) : As[i * N];
        for (int t = 0; t < a.Hbits; ++t) {
          const longlong2 x = As[i * N + hi_col0 + t];
          const bool bit = (g >> t) & 1ull;
          if (ryser) {
            if (bit) {
              v.x += x.x;
              v.y += x.y;
            }
          } else {
            v.x += bit ? -x.x : x.x;
            v.y += bit ? -x.y : x.y;
          }
        }
        H[i] = v;
      }
    } else {
      const int t = __ffsll((long long)h) - 1;
      const bool set = (g >> t) & 1ull;
      const long long c = ryser ? (set ? 1 : -1) : (set ? -2 : 2);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const longlong2 x = As[i * N + hi_col0 + t];
        H[i].x += c * x.x;
        H[i].y += c * x.y;
      }
    }
    double sr = 0.0, si = 0.0;
    lo_sweep_fx<N>(H, T, nsteps, (uint32_t)(__popcll(g) & 1), sr, si);
    comp_add(Sr, Cr, sr);
    comp_add(Si, Ci, si);
  }

#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const double or_ = __shfl_down_sync(0xffffffffu, Sr, d), oc = __shfl_down_sync(0xffffffffu, Cr, d);
    const double oi = __shfl_down_sync(0xffffffffu, Si, d), od = __shfl_down_sync(0xffffffffu, Ci, d);
    Cr += oc;
    comp_add(Sr, Cr, or_);
    Ci += od;
    comp_add(Si, Ci, oi);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = Sr;
    red[1][tid >> 5] = Cr;
    red[2][tid >> 5] = Si;
    red[3][tid >> 5] = Ci;
  }
  __syncthreads();
  if (tid == 0) {
    double sr = red[0][0], cr = red[1][0], si = red[2][0], ci = red[3][0];
    for (int w = 1; w < kPermThreads / 32; ++w) {
      cr += red[1][w];
      comp_add(sr, cr, red[0][w]);
      ci += red[3][w];
      comp_add(si, ci, red[2][w]);
    }
    // the FP64 rows of the split product were multiplied unscaled
    constexpr int KI = fx_int_rows<N>();
    const double sc = KI > 0 && N > 1 ? ldexp(1.0, -FixedPoint<N>::F * (N - KI)) : 1.0;
    a.partials[item] = make_double2((sr + cr) * sc, (si + ci) * sc);
  }
}

// Launch shape of one bin, for callers that build a CUDA graph node instead of launching.
struct PermNode {
  void* func;
  unsigned grid;
  size_t smem;
};

// Launches the bin on a.stream, or (node != nullptr) only fills in its launch shape.
template <int N>
int launch_perm_bin_n(const PermBinArgs& a, PermNode* node) {
  static_assert(sizeof(cdd) == sizeof(double2), "both arithmetics use 16-byte elements");
  const size_t smem = (size_t)(N * N + (1 << a.L) * N) * sizeof(double2);
  void (*kern)(PermBinArgs) = a.prec == kPrecFP64       ? perm_bin_fx<N>
                              : a.prec == kPrecFP64Dadd ? perm_bin_f64<N>
                                                        : perm_bin_kernel<N>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  const int64_t items = (int64_t)a.nmat * a.items_per_mat;
  if (node) {
    node->func = reinterpret_cast<void*>(kern);
    node->grid = (unsigned)items;
    node->smem = smem;
    return 0;
  }
  kern<<<(unsigned)items, kPermThreads, smem, a.stream>>>(a);
  return (int)cudaGetLastError();
}

// Dispatch over the sizes instantiated in one translation unit.
template <int LO, int HI>
int launch_perm_bin_range(int n, const PermBinArgs& a, PermNode* node) {
  if constexpr (LO > HI) {
    return -1;
  } else {
    if (n == LO) return launch_perm_bin_n<LO>(a, node);
    return launch_perm_bin_range<LO + 1, HI>(n, a, node);
  }
}

int launch_perm_bin_1_12(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_13_20(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_21_26(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_27_32(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_33_36(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_37_40(int n, const PermBinArgs& a, PermNode* node);

constexpr int kPermMaxN = 40;

}  // namespace pcvl
