// Double-float arithmetic (a value is hi + lo, two FP32 words, ~48-bit significand) for the
// Nose-Hoover thermostat chain.
//
// Why: the chain update is a serial dependency of ~80 operations that every MD step waits for
// (src/md.cpp:401-406, 457-460).  On GB300 one dependent FP64 operation takes on the order of
// 150-300 cycles, which made the chain cost ~11 us per step; the same chain in double-float runs
// on the FP32 pipe with ~4-cycle latencies.  The chain state is kept as double-float in memory
// too (the host reads hi + lo); the arithmetic error is ~2^-46 relative per operation (the
// reference's double is 2^-53), far below the FP32 force error that drives the dynamics.
//
// Algorithms: TwoSum (Knuth), FastTwoSum (Dekker), TwoProduct via fused multiply-add, and the
// double-float add/multiply built from them (Dekker 1971; Hida, Li & Bailey, "Library for
// double-double and quad-double arithmetic", 2000).  exp by Taylor series with a single-precision
// tail for the small terms, and argument halving with repeated squaring beyond |x| = 1/8.
#pragma once
#include <cmath>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace souffle {

// Error-free transformations need each sum and product rounded on its own: on the device the
// _rn intrinsics are never contracted into fused multiply-adds (host builds that compile this
// header pass -ffp-contract=off).
#ifdef __CUDA_ARCH__
#define DF_ADD(a, b) __fadd_rn(a, b)
#define DF_SUB(a, b) __fsub_rn(a, b)
#define DF_MUL(a, b) __fmul_rn(a, b)
#else
#define DF_ADD(a, b) ((a) + (b))
#define DF_SUB(a, b) ((a) - (b))
#define DF_MUL(a, b) ((a) * (b))
#endif

struct dfloat {
  float hi, lo;
};

__host__ __device__ inline dfloat df_quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = DF_ADD(a, b);
  return {s, DF_SUB(b, DF_SUB(s, a))};
}

__host__ __device__ inline dfloat df_two_sum(float a, float b) {
  const float s = DF_ADD(a, b);
  const float bb = DF_SUB(s, a);
  return {s, DF_ADD(DF_SUB(a, DF_SUB(s, bb)), DF_SUB(b, bb))};
}

__host__ __device__ inline dfloat df_from(double a) {
  const float h = (float)a;
  return {h, (float)(a - (double)h)};
}

__host__ __device__ inline double df_to(dfloat a) { return (double)a.hi + (double)a.lo; }

__host__ __device__ inline dfloat df_add(dfloat a, dfloat b) {
  dfloat s = df_two_sum(a.hi, b.hi);
  const dfloat t = df_two_sum(a.lo, b.lo);
  s.lo = DF_ADD(s.lo, t.hi);
  s = df_quick_two_sum(s.hi, s.lo);
  s.lo = DF_ADD(s.lo, t.lo);
  return df_quick_two_sum(s.hi, s.lo);
}

__host__ __device__ inline dfloat df_neg(dfloat a) { return {-a.hi, -a.lo}; }

__host__ __device__ inline dfloat df_mul(dfloat a, dfloat b) {
  const float p = DF_MUL(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_quick_two_sum(p, e);
}

// e^x - 1 for |x| <= 1/8 as x S(x), S = 1 + x/2 + x^2/6 + x^3/24 + x^4/120 + x^5 T(x), where the
// tail T = 1/720 + x/5040 + ... is small enough (|x^5 T| < 5e-8) to be evaluated in FP32.
// S = a + x^2 (b + x^2 c) with a = 1 + x/2, b = 1/6 + x/24, c = 1/120 + x T (Estrin's scheme:
// a, b, c and x^2 are independent, so the dependent chain is half of Horner's).
__host__ __device__ inline dfloat df_expm1_small(dfloat x) {
  const float xf = x.hi;
  const float t = fmaf(xf, fmaf(xf, fmaf(xf, fmaf(xf, 1.0f / 3628800.0f, 1.0f / 362880.0f), 1.0f / 40320.0f),
                                1.0f / 5040.0f), 1.0f / 720.0f);
  // 1/6, 1/24, 1/120 as double-float pairs (head = the FP32 rounding, tail = the remainder)
  const dfloat c6 = {1.666666716e-01f, -4.967053879e-09f};
  const dfloat c24 = {4.166666791e-02f, -1.241763470e-09f};
  const dfloat c120 = {8.333333768e-03f, -4.346172033e-10f};
  const dfloat x2 = df_mul(x, x);
  const dfloat a = df_add(dfloat{1.0f, 0.0f}, dfloat{0.5f * x.hi, 0.5f * x.lo});
  const dfloat b = df_add(c6, df_mul(x, c24));
  const dfloat c = df_add(c120, dfloat{DF_MUL(xf, t), 0.0f});
  const dfloat S = df_add(a, df_mul(x2, df_add(b, df_mul(x2, c))));
  return df_mul(x, S);
}

// e^x: for |x| <= 1/8 from the series; beyond, e^x = (e^{x/2^s})^(2^s) with the smallest s
// that brings |x|/2^s under 1/8 (each squaring doubles the relative error, so s <= 10 keeps it
// near 2^-36 for |x| up to 128; larger |x| falls back to FP64 exp).  Results below ~1e-26
// (x < -60) lose precision as the low word turns subnormal.
__host__ __device__ inline dfloat df_exp(dfloat x) {
  const float ax = fabsf(x.hi);
  if (!(ax <= 128.0f)) return df_from(exp(df_to(x)));
  int s = 0;
  float m = ax;
  while (m > 0.125f) {
    m *= 0.5f;
    s++;
  }
  const float scale = ldexpf(1.0f, -s);
  const dfloat xs = {x.hi * scale, x.lo * scale};  // exact: a power of two
  dfloat e = df_add(df_expm1_small(xs), dfloat{1.0f, 0.0f});
  for (int k = 0; k < s; k++) e = df_mul(e, e);
  return e;
}

// e^x - 1 without cancellation: the series for |x| <= 1/8, beyond which |e^x - 1| > 0.11.
__host__ __device__ inline dfloat df_expm1(dfloat x) {
  if (fabsf(x.hi) <= 0.125f) return df_expm1_small(x);
  return df_add(df_exp(x), dfloat{-1.0f, 0.0f});
}

__host__ __device__ inline unsigned int df_f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned int u;
  __builtin_memcpy(&u, &x, 4);
  return u;
#endif
}

// Integer part of a float exactly as int64 (for |x| < 2^63), fraction returned in frac.
// Below 2^23 a float may carry fraction bits and fits int32; above, it is an integer whose value
// is its 24-bit significand shifted by its exponent, read from the bits (no 64-bit conversion).
__host__ __device__ inline long long df_f32_int_part(float x, float& frac) {
  if (fabsf(x) < 8388608.0f) {
    const float t = truncf(x);
    frac = x - t;
    return (long long)(int)t;
  }
  frac = 0.0f;
  const unsigned int b = df_f32_bits(x);
  const int e = (int)((b >> 23) & 0xffu) - 150;  // x = significand * 2^e, 0 <= e <= 39 here
  if (e > 39) return 0;                          // out of range or not finite: callers check
  const long long m = (long long)((b & 0x7fffffu) | 0x800000u) << e;
  return (b >> 31) ? -m : m;
}

// round(v * scale) to nearest (ties to even) as int64, for a power-of-two scale and
// |v scale| < 2^63 - 2^40, using FP32 and integer operations only: the integer parts of hi and
// lo are exact; their fractions (each in (-1, 1)) are summed exactly as s + e (TwoSum), and the
// fraction d = s - floor(s) is compared with 1/2 (d is exact near 1/2, and |e| is below the
// spacing of s there, so e only matters when d is exactly 1/2; an exact tie goes to even).
__host__ __device__ inline long long df_to_fixed(dfloat v, float scale) {
  float fa, fb;
  const long long ia = df_f32_int_part(v.hi * scale, fa);
  const long long ib = df_f32_int_part(v.lo * scale, fb);
  const dfloat f = df_two_sum(fa, fb);
  const float fl = floorf(f.hi);
  const float d = f.hi - fl;
  const long long base = ia + ib + (long long)(int)fl;
  long long up;
  if (d != 0.5f) up = d > 0.5f ? 1 : 0;
  else up = f.lo > 0.0f ? 1 : (f.lo < 0.0f ? 0 : (base & 1));
  return base + up;
}

// k * scale as a double-float for any int64 k and power-of-two scale: k is cut into 24-, 20- and
// 20-bit pieces, each exact in FP32, and summed exactly (TwoSum) then rounded to ~48 bits.
__host__ __device__ inline dfloat df_from_fixed(long long k, float scale) {
  const float c2 = (float)(int)(k >> 40) * 1099511627776.0f;        // 2^40
  const float c1 = (float)(int)((k >> 20) & 0xfffff) * 1048576.0f;  // 2^20
  const float c0 = (float)(int)(k & 0xfffff);
  const dfloat s = df_add(df_two_sum(c2, c1), dfloat{c0, 0.0f});
  return {s.hi * scale, s.lo * scale};
}

}  // namespace souffle
