// 64-bit block floating point for complex products on the integer pipes (GB300's FP64 pipe
// retires 2 DFMA per SM per clock; these products run beside it).
#pragma once

#include <cstdint>

namespace pcvl {

// 64-bit block floating point on the integer pipes: the complex value (re + i im) 2^e with
// |re|, |im| < 2^62 and, after bf_norm, the larger magnitude's leading one at bit 61.  A
// product takes the high 64 bits of the four 128-bit products (__mul64hi) and shifts back:
// 62 significant bits, truncated once per product (relative error below 2^-59, under the
// 2^-53 of an FP64 product).  Exact row sums enter with e = -F.
struct BFC {
  long long re, im;
  int e;
};

__device__ __forceinline__ BFC bf_norm(long long re, long long im, int e) {
  const unsigned long long ar = re < 0 ? 0ull - (unsigned long long)re : (unsigned long long)re;
  const unsigned long long ai = im < 0 ? 0ull - (unsigned long long)im : (unsigned long long)im;
  const int sh = __clzll((long long)(ar | ai)) - 2;  // >= 0 below 2^62; 62 for zero
  BFC z;
  z.re = (long long)((unsigned long long)re << sh);
  z.im = (long long)((unsigned long long)im << sh);
  z.e = e - sh;
  return z;
}

__device__ __forceinline__ BFC bf_mul(const BFC& a, const BFC& b) {
  const long long rr = __mul64hi(a.re, b.re), ii = __mul64hi(a.im, b.im);
  const long long ri = __mul64hi(a.re, b.im), ir = __mul64hi(a.im, b.re);
  return bf_norm(rr - ii, ri + ir, a.e + b.e + 64);  // |rr|, |ii| <= 2^60: no overflow
}

// x 2^e as a double, rounded to nearest even (x from bf_norm / bf_mul: |x| < 2^62).  A
// product of many small fixed-point sums can fall below the normal FP64 range (a sum is at
// least 2^-F when not zero, and 26 of them at n = 40 reach 2^-1534); such a term is flushed
// to zero, beside the terms whose FP64 roundings are larger by hundreds of binades.
__device__ __forceinline__ double bf_to_f64(long long x, int e) {
  const unsigned long long ux = (unsigned long long)x;
  const unsigned long long sgn = ux & 0x8000000000000000ull;
  const unsigned long long ax = x < 0 ? 0ull - ux : ux;
  const int lz = __clzll((long long)ax);
  const int be = 1023 + 63 + e - lz;  // biased exponent of the leading one
  if (ax == 0 || be <= 0) return 0.0;
  const unsigned long long mn = ax << (lz & 63);
  unsigned long long mant = mn >> 11;
  const unsigned int rem = (unsigned int)mn & 0x7ffu;
  mant += (rem + (unsigned int)(mant & 1ull) + 0x3ffu) >> 11;
  const unsigned long long bits = sgn | (((unsigned long long)be << 52) + mant - (1ull << 52));
  return __longlong_as_double((long long)bits);
}

}  // namespace pcvl
