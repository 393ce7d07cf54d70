// Shared device/host helpers for the linear-optics kernels.
//
// Arithmetic: GB300 issues FP64 at 1/73 of its FP32 rate (measured: 505 G FP64 FMA/s
// against 36.8 T FP32 FMA/s).  The kernels compute in native FP64 by default (the
// reference's arithmetic) and offer, opt-in, FP64-class precision as float-float pairs
// ("df64": value = hi + lo, |lo| <= ulp(hi)/2 when normalised) built from error-free
// transformations on the FP32 pipe:
//   two_sum   (Knuth 1969):  s = fl(a+b), e = (a+b) - s exactly;
//   two_prod  (FMA form):    p = fl(a*b), e = fma(a, b, -p) exactly;
//   fast_two_sum (Dekker 1971) when |a| >= |b|.
// The pair carries ~48 significant bits (relative error ~2^-47 per operation).
#pragma once
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>

#define PCVL_HD __host__ __device__ __forceinline__

namespace pcvl {

// Arithmetic of the permanent, SLOS and sampler kernels (the ABI's PCVL_PREC_* codes).
enum Precision : int { kPrecFloatFloat = 0, kPrecFP32 = 1, kPrecFP64 = 2, kPrecFP64Dadd = 3 };

// ------------------------------------------------------------------ df64 scalars
struct dd {
  float hi, lo;
};

PCVL_HD dd two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
PCVL_HD dd fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
PCVL_HD dd two_prod(float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  return {p, e};
}
PCVL_HD dd dd_from_double(double x) {
  float hi = (float)x;
  float lo = (float)(x - (double)hi);
  return {hi, lo};
}
PCVL_HD double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }
PCVL_HD dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
// normalised sum (two_sum on the high parts, fold the low parts, renormalise)
PCVL_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  float e = s.lo + (a.lo + b.lo);
  return two_sum(s.hi, e);
}
PCVL_HD dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
PCVL_HD dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  float e = fmaf(a.hi, b.lo, p.lo);
  e = fmaf(a.lo, b.hi, e);
  return two_sum(p.hi, e);
}
PCVL_HD dd dd_mul_f(dd a, float b) {
  dd p = two_prod(a.hi, b);
  float e = fmaf(a.lo, b, p.lo);
  return two_sum(p.hi, e);
}
// exact scaling by a power of two
PCVL_HD dd dd_ldexp(dd a, int e) { return {ldexpf(a.hi, e), ldexpf(a.lo, e)}; }

// ------------------------------------------------------------------ df64 complex
struct cdd {
  dd re, im;
};

#ifdef __CUDACC__
// 16-byte read-only load of a float-float complex (address must be 16-byte aligned)
__device__ __forceinline__ cdd ld_cdd(const cdd* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return {{v.x, v.y}, {v.z, v.w}};
}
// double from a float by exponent re-bias on the integer pipe (GB300 issues FP64 at a
// small fraction of its FP32 rate); zero, subnormals, infinities and NaN take the
// conversion instruction
__device__ __forceinline__ double f2d_int(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const uint64_t bits = ((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                        ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}
// hi + lo as a double: two integer-pipe conversions and one FP64 add
__device__ __forceinline__ double dd_to_double_fast(dd a) { return f2d_int(a.hi) + f2d_int(a.lo); }
#endif
PCVL_HD cdd cdd_zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
PCVL_HD cdd cdd_one() { return {{1.f, 0.f}, {0.f, 0.f}}; }
PCVL_HD cdd cdd_from(double re, double im) { return {dd_from_double(re), dd_from_double(im)}; }
PCVL_HD cdd cdd_add(cdd a, cdd b) { return {dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
PCVL_HD cdd cdd_sub(cdd a, cdd b) { return {dd_sub(a.re, b.re), dd_sub(a.im, b.im)}; }
PCVL_HD cdd cdd_neg(cdd a) { return {dd_neg(a.re), dd_neg(a.im)}; }
PCVL_HD cdd cdd_conj(cdd a) { return {a.re, dd_neg(a.im)}; }
PCVL_HD cdd cdd_ldexp(cdd a, int e) { return {dd_ldexp(a.re, e), dd_ldexp(a.im, e)}; }

// (x.re + i x.im)(y.re + i y.im); the two high products of each part are summed
// with two_sum so cancellation between them stays exact.
PCVL_HD cdd cdd_mul(cdd x, cdd y) {
  dd p1 = two_prod(x.re.hi, y.re.hi);
  dd p2 = two_prod(x.im.hi, y.im.hi);
  dd s = two_sum(p1.hi, -p2.hi);
  float t = s.lo + (p1.lo - p2.lo);
  t = fmaf(x.re.hi, y.re.lo, t);
  t = fmaf(x.re.lo, y.re.hi, t);
  t = fmaf(-x.im.hi, y.im.lo, t);
  t = fmaf(-x.im.lo, y.im.hi, t);
  dd re = two_sum(s.hi, t);

  dd q1 = two_prod(x.re.hi, y.im.hi);
  dd q2 = two_prod(x.im.hi, y.re.hi);
  dd u = two_sum(q1.hi, q2.hi);
  float v = u.lo + (q1.lo + q2.lo);
  v = fmaf(x.re.hi, y.im.lo, v);
  v = fmaf(x.re.lo, y.im.hi, v);
  v = fmaf(x.im.hi, y.re.lo, v);
  v = fmaf(x.im.lo, y.re.hi, v);
  dd im = two_sum(u.hi, v);
  return {re, im};
}

// Lazy variants for chains of operations.  The result pair (hi, lo) is exact up to the
// FP32 roundings of the low-order terms but not renormalised: |lo| stays below about
// 2^-20 of the operands' magnitude, so feeding it to cdd_mul_lazy (whose cross terms
// multiply lo by hi in FP32) costs at most ~2^-46 of the product's magnitude.
PCVL_HD cdd cdd_add_lazy(cdd a, cdd b) {
  const dd r = two_sum(a.re.hi, b.re.hi);
  const dd i = two_sum(a.im.hi, b.im.hi);
  return {{r.hi, r.lo + (a.re.lo + b.re.lo)}, {i.hi, i.lo + (a.im.lo + b.im.lo)}};
}
PCVL_HD cdd cdd_mul_lazy(cdd x, cdd y) {
  const dd p1 = two_prod(x.re.hi, y.re.hi);
  const dd p2 = two_prod(x.im.hi, y.im.hi);
  const dd s = two_sum(p1.hi, -p2.hi);
  float t = s.lo + (p1.lo - p2.lo);
  t = fmaf(x.re.hi, y.re.lo, t);
  t = fmaf(x.re.lo, y.re.hi, t);
  t = fmaf(-x.im.hi, y.im.lo, t);
  t = fmaf(-x.im.lo, y.im.hi, t);
  const dd q1 = two_prod(x.re.hi, y.im.hi);
  const dd q2 = two_prod(x.im.hi, y.re.hi);
  const dd u = two_sum(q1.hi, q2.hi);
  float v = u.lo + (q1.lo + q2.lo);
  v = fmaf(x.re.hi, y.im.lo, v);
  v = fmaf(x.re.lo, y.im.hi, v);
  v = fmaf(x.im.hi, y.re.lo, v);
  v = fmaf(x.im.lo, y.re.hi, v);
  return {{s.hi, t}, {u.hi, v}};
}
PCVL_HD cdd cdd_norm(cdd a) { return {two_sum(a.re.hi, a.re.lo), two_sum(a.im.hi, a.im.lo)}; }

// Lazy complex accumulator for sums of products: the high parts accumulate through
// two_sum (exact), everything of lower order goes to a plain float accumulator.
// One finish() renormalises.
struct cacc {
  float rh, rl, ih, il;
};
PCVL_HD cacc cacc_zero() { return {0.f, 0.f, 0.f, 0.f}; }
PCVL_HD void cacc_fma(cacc& a, cdd x, cdd y) {
  dd p1 = two_prod(x.re.hi, y.re.hi);
  dd p2 = two_prod(x.im.hi, y.im.hi);
  dd s1 = two_sum(a.rh, p1.hi);
  dd s2 = two_sum(s1.hi, -p2.hi);
  float t = a.rl + (s1.lo + s2.lo) + (p1.lo - p2.lo);
  t = fmaf(x.re.hi, y.re.lo, t);
  t = fmaf(x.re.lo, y.re.hi, t);
  t = fmaf(-x.im.hi, y.im.lo, t);
  t = fmaf(-x.im.lo, y.im.hi, t);
  a.rh = s2.hi;
  a.rl = t;

  dd q1 = two_prod(x.re.hi, y.im.hi);
  dd q2 = two_prod(x.im.hi, y.re.hi);
  dd u1 = two_sum(a.ih, q1.hi);
  dd u2 = two_sum(u1.hi, q2.hi);
  float v = a.il + (u1.lo + u2.lo) + (q1.lo + q2.lo);
  v = fmaf(x.re.hi, y.im.lo, v);
  v = fmaf(x.re.lo, y.im.hi, v);
  v = fmaf(x.im.hi, y.re.lo, v);
  v = fmaf(x.im.lo, y.re.hi, v);
  a.ih = u2.hi;
  a.il = v;
}
PCVL_HD cdd cacc_finish(const cacc& a) { return {two_sum(a.rh, a.rl), two_sum(a.ih, a.il)}; }


// ------------------------------------------------------------------ Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
// as easy as 1, 2, 3" (SC 2011): ten rounds of two 32x32->64 multiplies with the
// paper's multipliers and Weyl key increments.
struct u4 {
  uint32_t x, y, z, w;
};
PCVL_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}
PCVL_HD u4 philox4x32_10(u4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = mulhi32(M1, c.z), lo1 = M1 * c.z;
    c = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}
// 53-bit uniform double in [0, 1) from two 32-bit words
PCVL_HD double u01_from(uint32_t a, uint32_t b) {
  uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)v * (1.0 / 9007199254740992.0);
}

// ------------------------------------------------------------------ combinatorics
// Number of k-photon states on M modes: C(M + k - 1, k); exact in 64 bits for the
// sizes this library accepts (checked on the host).
PCVL_HD uint64_t fock_count(int M, int k) {
  if (k < 0) return 0;
  if (M <= 0) return k == 0 ? 1 : 0;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(M - 1 + i) / (uint64_t)i;
  return r;
}

}  // namespace pcvl
