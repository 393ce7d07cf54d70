// Arithmetic policies of the SLOS kernels: every kernel is written once against a
// policy P and instantiated for both arithmetics.
//
//  * Arith64 (the default, the reference's arithmetic: complex128 coefficients in
//    perceval/backends/_slos.py:44,99): values double2, multiply-adds by DFMA (four per
//    complex multiply-add), normalisation factors double.
//  * ArithFF (opt-in): values float-float complex pairs (cdd, ~48 significant bits) on
//    the FP32 pipe, multiply-adds through cacc_fma (exact two_sum of the high products),
//    factors dd.
//
// Both store a complex value in 16 bytes and a factor in 8, so layers, unitary columns
// and factor tables have one layout for both.
#pragma once
#include "common.cuh"

namespace pcvl {

struct ArithFF {
  using V = cdd;
  using Acc = cacc;
  using F = dd;
  PCVL_HD static V zero() { return cdd_zero(); }
  PCVL_HD static V one() { return cdd_one(); }
  PCVL_HD static V from(double re, double im) { return cdd_from(re, im); }
  PCVL_HD static V conj(V a) { return cdd_conj(a); }
  PCVL_HD static V add(V a, V b) { return cdd_add(a, b); }
  PCVL_HD static Acc acc_zero() { return cacc_zero(); }
  PCVL_HD static void fma(Acc& a, V x, V y) { cacc_fma(a, x, y); }
  PCVL_HD static V finish(const Acc& a) { return cacc_finish(a); }
  PCVL_HD static double re(V a) { return dd_to_double(a.re); }
  PCVL_HD static double im(V a) { return dd_to_double(a.im); }
  // normalisation factors
  PCVL_HD static F f_from(double x) { return dd_from_double(x); }
  PCVL_HD static F f_mul(F a, F b) { return dd_mul(a, b); }
  PCVL_HD static F f_mul_int(F a, int k) { return dd_mul_f(a, (float)k); }
#ifdef __CUDACC__
  __device__ static V ld(const V* p) { return ld_cdd(p); }
  __device__ static V shfl_down(V v, int d) {
    V r;
    r.re.hi = __shfl_down_sync(0xffffffffu, v.re.hi, d);
    r.re.lo = __shfl_down_sync(0xffffffffu, v.re.lo, d);
    r.im.hi = __shfl_down_sync(0xffffffffu, v.im.hi, d);
    r.im.lo = __shfl_down_sync(0xffffffffu, v.im.lo, d);
    return r;
  }
  __device__ static V shfl_xor(V v, int d) {
    V r;
    r.re.hi = __shfl_xor_sync(0xffffffffu, v.re.hi, d);
    r.re.lo = __shfl_xor_sync(0xffffffffu, v.re.lo, d);
    r.im.hi = __shfl_xor_sync(0xffffffffu, v.im.hi, d);
    r.im.lo = __shfl_xor_sync(0xffffffffu, v.im.lo, d);
    return r;
  }
  __device__ static F f_shfl(F f, int src) {
    return {__shfl_sync(0xffffffffu, f.hi, src), __shfl_sync(0xffffffffu, f.lo, src)};
  }
  // a factor as two 32-bit words (shared-memory slots)
  __device__ static void f_pack(F f, uint32_t* w) {
    w[0] = __float_as_uint(f.hi);
    w[1] = __float_as_uint(f.lo);
  }
  __device__ static F f_unpack(const uint32_t* w) { return {__uint_as_float(w[0]), __uint_as_float(w[1])}; }
  // |c|^2 F, c sqrt(F), 2 w F c
  __device__ static double prob(V c, F f) {
    const dd c2 = dd_add(dd_mul(c.re, c.re), dd_mul(c.im, c.im));
    return dd_to_double_fast(dd_mul(c2, f));
  }
  __device__ static double2 amp(V c, F f) {
    const double sF = sqrt(dd_to_double_fast(f));
    return make_double2(dd_to_double_fast(c.re) * sF, dd_to_double_fast(c.im) * sF);
  }
  __device__ static V seed(V c, double w, F f) {
    const dd f2 = dd_mul(dd_from_double(2.0 * w), f);
    return {dd_mul(c.re, f2), dd_mul(c.im, f2)};
  }
#endif
};

struct Arith64 {
  using V = double2;
  using Acc = double2;
  using F = double;
  PCVL_HD static V zero() { return make_double2(0.0, 0.0); }
  PCVL_HD static V one() { return make_double2(1.0, 0.0); }
  PCVL_HD static V from(double re, double im) { return make_double2(re, im); }
  PCVL_HD static V conj(V a) { return make_double2(a.x, -a.y); }
  PCVL_HD static V add(V a, V b) { return make_double2(a.x + b.x, a.y + b.y); }
  PCVL_HD static Acc acc_zero() { return make_double2(0.0, 0.0); }
  PCVL_HD static void fma(Acc& a, V x, V y) {
    a.x = ::fma(x.x, y.x, a.x);
    a.x = ::fma(-x.y, y.y, a.x);
    a.y = ::fma(x.x, y.y, a.y);
    a.y = ::fma(x.y, y.x, a.y);
  }
  PCVL_HD static V finish(const Acc& a) { return a; }
  PCVL_HD static double re(V a) { return a.x; }
  PCVL_HD static double im(V a) { return a.y; }
  PCVL_HD static F f_from(double x) { return x; }
  PCVL_HD static F f_mul(F a, F b) { return a * b; }
  PCVL_HD static F f_mul_int(F a, int k) { return a * (double)k; }
#ifdef __CUDACC__
  __device__ static V ld(const V* p) { return __ldg(p); }
  __device__ static V shfl_down(V v, int d) {
    return make_double2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
  }
  __device__ static V shfl_xor(V v, int d) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, d), __shfl_xor_sync(0xffffffffu, v.y, d));
  }
  __device__ static F f_shfl(F f, int src) { return __shfl_sync(0xffffffffu, f, src); }
  __device__ static void f_pack(F f, uint32_t* w) {
    w[0] = (uint32_t)__double2loint(f);
    w[1] = (uint32_t)__double2hiint(f);
  }
  __device__ static F f_unpack(const uint32_t* w) { return __hiloint2double((int)w[1], (int)w[0]); }
  __device__ static double prob(V c, F f) { return ::fma(c.x, c.x, c.y * c.y) * f; }
  __device__ static double2 amp(V c, F f) {
    const double sF = sqrt(f);
    return make_double2(c.x * sF, c.y * sF);
  }
  __device__ static V seed(V c, double w, F f) {
    const double f2 = 2.0 * w * f;
    return make_double2(c.x * f2, c.y * f2);
  }
#endif
};

static_assert(sizeof(ArithFF::V) == sizeof(Arith64::V) && sizeof(ArithFF::F) == sizeof(Arith64::F),
              "both arithmetics share the layouts of values and factors");

}  // namespace pcvl
