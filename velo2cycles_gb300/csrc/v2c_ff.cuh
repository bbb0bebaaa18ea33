// v2c_ff.cuh -- float-float ("double-single") arithmetic on FP32 units.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  GB300 issues FP32 FMAs at 64x its FP64 rate,
// so a float-float evaluation with a few dozen FP32 operations per step is
// several times cheaper than the FP64 one it replaces.
//
// Error-free transforms (Knuth's two-sum, Dekker's fast two-sum, the FMA
// two-product) and the add/mul/div/sqrt built on them follow the published
// double-double algorithms of Hida, Li and Bailey ("Library for
// double-double and quad-double arithmetic", 2007), restated for float
// pairs.  The intrinsics __fadd_rn/__fsub_rn/__fmul_rn keep the compiler from
// contracting or reordering the transforms.
//
// exp: table-driven range reduction to |r| <= ln2/128 and a short Taylor
// series (details at ff_exp).  log: a = m 2^e, then one Newton
// step for y = log m from the FP32 logf, y <- y + m e^-y - 1, which doubles
// the number of correct bits, plus e ln 2.  Relative errors, checked against FP64 in the
// tests: ~1e-14 for exp and log over the ranges used here.
//
// Range: ff_exp returns 0 below e^-87 and loses the low word's bits below
// about e^-70 (the low word goes subnormal), so callers form only values
// above ~1e-30 where the full precision matters.
#pragma once
#include <math.h>

namespace v2c {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_f(float h) { return ff{h, 0.f}; }

__device__ __forceinline__ ff ff_from_double(double d) {
  const float h = __double2float_rn(d);
  return ff{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ float two_sum(float a, float b, float &e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}
__device__ __forceinline__ float fast_two_sum(float a, float b, float &e) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
  return s;
}
__device__ __forceinline__ float two_prod(float a, float b, float &e) {
  const float p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
  return p;
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s2, t2;
  float s1 = two_sum(a.hi, b.hi, s2);
  const float t1 = two_sum(a.lo, b.lo, t2);
  s2 = __fadd_rn(s2, t1);
  s1 = fast_two_sum(s1, s2, s2);
  s2 = __fadd_rn(s2, t2);
  s1 = fast_two_sum(s1, s2, s2);
  return ff{s1, s2};
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  float e;
  const float s = two_sum(a.hi, b, e);
  e = __fadd_rn(e, a.lo);
  float l;
  const float h = fast_two_sum(s, e, l);
  return ff{h, l};
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float e;
  const float p = two_prod(a.hi, b.hi, e);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float l;
  const float h = fast_two_sum(p, e, l);
  return ff{h, l};
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  float e;
  const float p = two_prod(a.hi, b, e);
  e = __fmaf_rn(a.lo, b, e);
  float l;
  const float h = fast_two_sum(p, e, l);
  return ff{h, l};
}
// exact scaling by a power of two s (no overflow/underflow in the uses here)
__device__ __forceinline__ ff ff_scale(ff a, float s) {
  return ff{__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)};
}
// 2^k for -126 <= k <= 127, built from the exponent bits
__device__ __forceinline__ float pow2i(int k) { return __int_as_float((k + 127) << 23); }
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  ff r = ff_sub(a, ff_mul_f(b, q1));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  r = ff_sub(r, ff_mul_f(b, q2));
  const float q3 = __fdiv_rn(r.hi, b.hi);
  float l;
  const float h = fast_two_sum(q1, q2, l);
  return ff_add_f(ff{h, l}, q3);
}
// a / b from the approximate reciprocal of b.hi and one correction: the
// first quotient carries ~2 ulps, the remainder a - b q1 is formed exactly,
// and its quotient (a term ~1e-7 of the result) may carry the same relative
// error, so the pair is good to ~2^-44 -- for quotients rounded to FP32 at
// the end, or used to that accuracy.  b.hi a normal, finite nonzero float.
__device__ __forceinline__ ff ff_div_fast(ff a, ff b) {
  const float rb = __fdividef(1.f, b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  const ff r = ff_sub(a, ff_mul_f(b, q1));
  const float q2 = __fmul_rn(r.hi, rb);
  float l;
  const float h = fast_two_sum(q1, q2, l);
  return ff{h, l};
}
// a = m 4^e with m in [0.25, 1): sqrt a = sqrt(m) 2^e, one Newton step on
// the FP32 square root, so the low words stay normal for any normal a.hi
__device__ __forceinline__ ff ff_sqrt(ff a) {
  if (!(a.hi > 0.f)) return ff_f(0.f);
  int e;
  (void)frexpf(a.hi, &e);
  const int h = e >> 1;  // a = m 2^(2h), m in [0.25, 1)
  const ff m = ff_scale(ff_scale(a, pow2i(-h)), pow2i(-h));
  const float y = __fsqrt_rn(m.hi);
  float err;
  const float yy = two_prod(y, y, err);
  const ff r = ff_sub(m, ff{yy, err});
  const float c = __fdiv_rn(r.hi, __fmul_rn(2.f, y));
  float l;
  const float hh = fast_two_sum(y, c, l);
  return ff_scale(ff{hh, l}, pow2i(h));
}

// the float nearest to a float pair
__device__ __forceinline__ float ff_round(ff a) { return __fadd_rn(a.hi, a.lo); }
// b - c of two floats, exactly, as a float pair
__device__ __forceinline__ ff ff_diff(float b, float c) {
  ff r;
  r.hi = two_sum(b, -c, r.lo);
  return r;
}

// ln 2 as a float pair
__device__ __forceinline__ ff ff_ln2() { return ff{0.693147182464599609375f, -1.9046542e-09f}; }

// 2^(j/64), j = 0..63, as float pairs (hi = the float nearest to 2^(j/64),
// lo = the float nearest to the remainder)
__device__ const float2 k_ff_exp2_64[64] = {
    {1.000000000e+00f, 0.000000000e+00f}, {1.010889292e+00f, -5.711605411e-09f},
    {1.021897197e+00f, -4.811559862e-08f}, {1.033024907e+00f, -2.809089317e-08f},
    {1.044273734e+00f, 4.833470157e-08f}, {1.055645227e+00f, -4.907169426e-08f},
    {1.067140460e+00f, -5.933751979e-08f}, {1.078760743e+00f, 5.461594554e-08f},
    {1.090507746e+00f, -1.307753994e-08f}, {1.102382541e+00f, 4.260501996e-08f},
    {1.114386797e+00f, -5.435540018e-08f}, {1.126521587e+00f, 3.123641434e-08f},
    {1.138788581e+00f, 5.386222313e-08f}, {1.151189208e+00f, 2.192228266e-08f},
    {1.163724899e+00f, -4.051441493e-08f}, {1.176396966e+00f, 2.566975077e-08f},
    {1.189207077e+00f, 3.797635273e-08f}, {1.202156782e+00f, -5.069756526e-08f},
    {1.215247393e+00f, -3.267394888e-08f}, {1.228480577e+00f, -4.136200360e-08f},
    {1.241857767e+00f, 4.496838102e-08f}, {1.255380750e+00f, 7.322237483e-09f},
    {1.269050956e+00f, 1.419333318e-09f}, {1.282870054e+00f, -3.816621685e-08f},
    {1.296839595e+00f, -4.018999533e-08f}, {1.310961246e+00f, -3.496571566e-08f},
    {1.325236678e+00f, -3.496373324e-08f}, {1.339667559e+00f, -3.461673970e-08f},
    {1.354255557e+00f, -1.012334927e-08f}, {1.369002461e+00f, -3.845881835e-08f},
    {1.383909941e+00f, -5.875577358e-08f}, {1.398979664e+00f, 8.689434061e-09f},
    {1.414213538e+00f, 2.420323497e-08f}, {1.429613352e+00f, -1.342992917e-08f},
    {1.445180774e+00f, 3.324199938e-08f}, {1.460917830e+00f, -3.628657552e-08f},
    {1.476826191e+00f, -4.500898854e-08f}, {1.492907763e+00f, -3.423620143e-08f},
    {1.509164453e+00f, -2.495937323e-08f}, {1.525598168e+00f, -1.762856883e-08f},
    {1.542210817e+00f, 8.070904833e-09f}, {1.559004426e+00f, -2.576466507e-08f},
    {1.575980902e+00f, -5.661025426e-08f}, {1.593142152e+00f, -4.903136785e-10f},
    {1.610490322e+00f, 9.836217174e-09f}, {1.628027439e+00f, -1.726008314e-08f},
    {1.645755529e+00f, -5.124972091e-08f}, {1.663676620e+00f, -3.920298752e-08f},
    {1.681792855e+00f, -2.475532668e-08f}, {1.700106382e+00f, -2.865147231e-08f},
    {1.718619347e+00f, -4.849617596e-08f}, {1.737333894e+00f, -5.850223417e-08f},
    {1.756252170e+00f, -9.235770371e-09f}, {1.775376439e+00f, 5.343197884e-08f},
    {1.794709086e+00f, -1.141504491e-08f}, {1.814252138e+00f, 3.736258236e-08f},
    {1.834008098e+00f, -1.123927795e-08f}, {1.853979111e+00f, 1.436561181e-08f},
    {1.874167681e+00f, -4.663005626e-08f}, {1.894575953e+00f, 2.810338451e-08f},
    {1.915206552e+00f, 9.845328108e-09f}, {1.936061740e+00f, 5.357072297e-08f},
    {1.957144141e+00f, -1.702180441e-08f}, {1.978456020e+00f, 6.032726318e-09f},
};

// exp: n = round(64 a / ln 2) = 64 k + j, r = a - n ln2/64 with ln2/64 split
// in three floats (the first with 9 significant bits, so n*c1 is exact for
// |n| < 2^15), |r| <= ln2/128; expm1(r) by its Taylor series (r^2/2 and
// r^3/6 in float-float, the r^4 and r^5 terms in float; the first omitted
// term is below 4e-17), then e^a = 2^k 2^(j/64) (1 + expm1(r)).
// Out of line (as ff_log): the per-marker viscosity calls them several
// times, and inlined copies of their ~50 instructions each made the marker
// physics kernel wait on instruction fetch.
static __device__ __noinline__ ff ff_exp(ff a) {
  if (a.hi < -87.0f) return ff_f(0.f);
  if (a.hi > 88.0f) return ff_f(INFINITY);
  const float nf = rintf(__fmul_rn(a.hi, 0x1.715476p+6f));  // 64/ln 2
  const int n = (int)nf;
  const float c1 = 0x1.63p-7f, c2 = -0x1.bd0106p-19f, c3 = 0x1.cf79acp-46f;
  ff r = ff_add_f(a, -__fmul_rn(nf, c1));  // n*c1 exact
  float e;
  const float p2 = two_prod(nf, c2, e);
  r = ff_sub(r, ff{p2, e});
  r = ff_add_f(r, -__fmul_rn(nf, c3));
  const ff s2 = ff_mul(r, r);
  const ff s3 = ff_mul(s2, r);
  const float rh = r.hi;
  const float tail = rh * rh * rh * rh * (1.f / 24.f + rh * (1.f / 120.f));
  ff p = ff_add(r, ff_scale(s2, 0.5f));
  p = ff_add(p, ff_mul(s3, ff{1.666666716e-01f, -4.967053879e-09f}));
  p = ff_add_f(p, tail);
  const float2 t = __ldg(&k_ff_exp2_64[n & 63]);
  const ff T{t.x, t.y};
  return ff_scale(ff_add(T, ff_mul(T, p)), pow2i(n >> 6));
}

// a = m 2^e with m in [0.5, 1); log a = log m + e ln 2, so that e^-log m
// stays in (1, 2] whatever the size of a (a.hi a positive normal float)
static __device__ __noinline__ ff ff_log(ff a) {
  int e;
  (void)frexpf(a.hi, &e);
  const int e1 = e >> 1, e2 = e - e1;
  const ff m = ff_scale(ff_scale(a, pow2i(-e1)), pow2i(-e2));
  const float y = logf(m.hi);
  const ff z = ff_exp(ff_f(-y));
  const ff t = ff_add_f(ff_mul(m, z), -1.f);
  return ff_add(ff_add_f(t, y), ff_mul_f(ff_ln2(), (float)e));
}

}  // namespace v2c
