// Double-float arithmetic on the FP32 pipe and table-driven exponentials.
//
// On GB300 the FP32 pipe issues ~67x more operations per clock than the FP64
// pipe (measured: 3.4e13 FFMA/s vs 5.0e11 DFMA/s), so FP64-accurate work that
// does not need FP64's exponent range is done here in double-float form: a value
// is an unevaluated sum hi + lo of two floats (about 48 significant bits).
// Error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the
// FMA-based TwoProduct. Exponentials use Tang's table-driven method (Tang 1989,
// ACM TOMS 15:144): 2^y = 2^n * 2^(j/64) * 2^r with |r| <= 1/128 and a short
// Taylor polynomial for 2^r.
//
// Every operation is written with round-to-nearest intrinsics, which the
// compiler never contracts or reassociates. With BGB_HOST_EMULATION the same
// code compiles on the host (used to check the routines' accuracy on a CPU).
#pragma once

#include <cstdint>

#ifdef BGB_HOST_EMULATION
#include <cmath>
#include <cstring>
#define BGB_HD inline
#define BGB_FADD(a, b) ((float)((a) + (b)))
#define BGB_FSUB(a, b) ((float)((a) - (b)))
#define BGB_FMUL(a, b) ((float)((a) * (b)))
#define BGB_FMA(a, b, c) std::fmaf((a), (b), (c))
#define BGB_FDIV(a, b) ((float)((a) / (b)))
#define BGB_RINTF(x) std::rintf(x)
#define BGB_FMINF(a, b) std::fmin((a), (b))
#define BGB_FMAXF(a, b) std::fmax((a), (b))
#define BGB_RCP_APPROX(x) (1.0f / (x))
#define BGB_DMA(a, b, c) std::fma((a), (b), (c))
static inline float bgb_int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline long long bgb_double_as_ll(double d) { long long i; std::memcpy(&i, &d, 8); return i; }
static inline double bgb_ll_as_double(long long i) { double d; std::memcpy(&d, &i, 8); return d; }
static inline unsigned bgb_float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline int bgb_clz(unsigned x) { return __builtin_clz(x); }
#else
#define BGB_HD __device__ __forceinline__
#define BGB_FADD(a, b) __fadd_rn((a), (b))
#define BGB_FSUB(a, b) __fsub_rn((a), (b))
#define BGB_FMUL(a, b) __fmul_rn((a), (b))
#define BGB_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define BGB_FDIV(a, b) __fdiv_rn((a), (b))
#define BGB_RINTF(x) rintf(x)
#define BGB_FMINF(a, b) fminf((a), (b))
#define BGB_FMAXF(a, b) fmaxf((a), (b))
#define BGB_RCP_APPROX(x) bgb_rcp_approx(x)
// float reciprocal, relative error within 2^-23 (PTX rcp.approx; normal inputs)
__device__ __forceinline__ float bgb_rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
#define BGB_DMA(a, b, c) __fma_rn((a), (b), (c))
#define bgb_int_as_float(i) __int_as_float(i)
#define bgb_double_as_ll(d) __double_as_longlong(d)
#define bgb_ll_as_double(i) __longlong_as_double(i)
#define bgb_float_as_uint(f) __float_as_uint(f)
#define bgb_clz(x) __clz((int)(x))
#endif

#include "dfconst.h"

namespace bgb {

struct df2 {
  float hi, lo;
};

BGB_HD df2 df_make(float hi) { return {hi, 0.0f}; }

// float -> double by moving the sign, exponent (rebiased by 1023 - 127) and mantissa into
// place with integer operations (exact for normal numbers and zero, which is all a
// conversion does): keeps the conversion off the FP64 pipe, where an F2F would issue.
// Subnormals, infinities and NaN take the ordinary conversion.
BGB_HD double f2d_bits(float f) {
  const unsigned u = bgb_float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e - 1u < 254u)
    return bgb_ll_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) |
                                        ((unsigned long long)(u & 0x7fffffu) << 29)));
  if ((u & 0x7fffffffu) == 0u) return bgb_ll_as_double((long long)sign);
  return (double)f;
}

// int -> double with integer operations (exact; |k| < 2^31).
BGB_HD double i2d_bits(int k) {
  if (k == 0) return 0.0;
  const unsigned long long sign = k < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned a = k < 0 ? 0u - (unsigned)k : (unsigned)k;
  const int msb = 31 - bgb_clz(a);
  const unsigned long long mant = ((unsigned long long)a << (52 - msb)) & 0xfffffffffffffull;
  return bgb_ll_as_double((long long)(sign | ((unsigned long long)(1023 + msb) << 52) | mant));
}

// Split an FP64 value into a double-float (exact for |x| in the float range).
BGB_HD df2 df_from_double(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

// The same split with integer operations for |x| in [2^-60, 2^101): hi = x truncated to
// 24 significand bits, lo = the remaining 29 bits as a float (one int -> float conversion,
// rounding them to 24 bits), so hi + lo is within 2^-48 |x| of x and |lo| < 2^-23 |hi|;
// no FP64-pipe instruction. Zero and values outside that range take df_from_double.
BGB_HD df2 df_from_double_bits(double x) {
  const long long b = bgb_double_as_ll(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 1023 - 60 || e >= 1023 + 101) return df_from_double(x);
  const unsigned sign = (unsigned)((unsigned long long)b >> 32) & 0x80000000u;
  const float hi = bgb_int_as_float((int)(sign | ((unsigned)(e - 896) << 23) | (unsigned)((b >> 29) & 0x7fffff)));
  // the remaining bits times 2^(e - 1075) (a normal float power for e in range)
  const float r = BGB_FMUL((float)(unsigned)(b & 0x1fffffff), bgb_int_as_float((e - 948) << 23));
  return {hi, sign ? -r : r};
}

// hi + lo in FP64: the two conversions on the integer pipe, one FP64 add.
BGB_HD double df_to_double(df2 a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

// TwoSum: s + e == a + b exactly.
BGB_HD df2 two_sum(float a, float b) {
  const float s = BGB_FADD(a, b);
  const float bb = BGB_FSUB(s, a);
  const float e = BGB_FADD(BGB_FSUB(a, BGB_FSUB(s, bb)), BGB_FSUB(b, bb));
  return {s, e};
}

// Fast2Sum for |a| >= |b|.
BGB_HD df2 fast_two_sum(float a, float b) {
  const float s = BGB_FADD(a, b);
  return {s, BGB_FSUB(b, BGB_FSUB(s, a))};
}

BGB_HD df2 df_add(df2 a, df2 b) {
  const df2 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, BGB_FADD(s.lo, BGB_FADD(a.lo, b.lo)));
}

BGB_HD df2 df_neg(df2 a) { return {-a.hi, -a.lo}; }

BGB_HD df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }

BGB_HD df2 df_mul(df2 a, df2 b) {
  const float p = BGB_FMUL(a.hi, b.hi);
  float e = BGB_FMA(a.hi, b.hi, -p);
  e = BGB_FMA(a.hi, b.lo, e);
  e = BGB_FMA(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

BGB_HD df2 df_mul_f(df2 a, float b) {
  const float p = BGB_FMUL(a.hi, b);
  float e = BGB_FMA(a.hi, b, -p);
  e = BGB_FMA(a.lo, b, e);
  return fast_two_sum(p, e);
}

// a * b + c (products and sum as double-floats).
BGB_HD df2 df_fma(df2 a, df2 b, df2 c) {
  const float p = BGB_FMUL(a.hi, b.hi);
  float e = BGB_FMA(a.hi, b.hi, -p);
  e = BGB_FMA(a.hi, b.lo, e);
  e = BGB_FMA(a.lo, b.hi, e);
  const df2 s = two_sum(c.hi, p);
  return fast_two_sum(s.hi, BGB_FADD(s.lo, BGB_FADD(e, c.lo)));
}

// 1 / b for a double-float b whose hi part is a normal float: an approximate float
// reciprocal r0 (relative error within 2^-23) refined by one Newton step with its square
// term, r = r0 (1 + e + e^2), e = 1 - b r0 formed with FMA; relative error ~2^-45.
BGB_HD df2 df_recip(df2 b) {
  const float r0 = BGB_RCP_APPROX(b.hi);
  const float e = BGB_FMA(-b.lo, r0, BGB_FMA(-b.hi, r0, 1.0f));
  return fast_two_sum(r0, BGB_FMUL(r0, BGB_FMA(e, e, e)));
}

// a / b with three correction steps (quotient digits q1 + q2 + q3).
BGB_HD df2 df_div(df2 a, df2 b) {
  const float q1 = BGB_FDIV(a.hi, b.hi);
  df2 r = df_sub(a, df_mul_f(b, q1));
  const float q2 = BGB_FDIV(r.hi, b.hi);
  r = df_sub(r, df_mul_f(b, q2));
  const float q3 = BGB_FDIV(r.hi, b.hi);
  return df_add(fast_two_sum(q1, q2), df_make(q3));
}

// a + (b - a) * w, the reference's linear interpolation step.
BGB_HD df2 df_lerp(df2 a, df2 b, df2 w) { return df_add(a, df_mul(df_sub(b, a), w)); }

// 2^y for a double-float y, returned as a double-float mantissa m (1/sqrt2 <= m < 2)
// and an integer exponent: 2^y = m * 2^n. Relative error ~1e-14. y.hi is clamped to
// [-16000, 16000] (the callers' 2^n is 0 or infinite well inside that; NaN propagates).
// tab_hi / tab_lo: 2^(j/64), j = -32..32 (index j + 32).
// k = round(64 y.hi) by the float shifter 1.5 * 2^23 (n = floor((k + 32) / 64) and j = k - 64 n
// in [-32, 31]); r = y - k/64 exactly as a double-float (|r| <= 1/128 + |y.lo|), t = r ln2,
// 2^r = 1 + t + t^2/2 + t^3 (1/6 + t/24 + t^2/120) with t^2 as an exact float product plus
// its error and the cubic tail in float (|t| <= 5.5e-3: tail error below 1e-15 relative),
// m = T_j (1 + s) as one double-float FMA.
BGB_HD df2 df_exp2(df2 y, int& n, const float* tab_hi, const float* tab_lo) {
  const float yc = BGB_FMINF(BGB_FMAXF(y.hi, -16000.0f), 16000.0f);
  const float yh = y.hi != y.hi ? y.hi : yc;
  const float tf = BGB_FMA(yh, 64.0f, 12582912.0f);
  const int k = (int)bgb_float_as_uint(tf) - 0x4B400000;
  const float kf = BGB_FSUB(tf, 12582912.0f);
  n = (k + 32) >> 6;  // arithmetic shift: floor
  const int j = k - (n << 6);
  const df2 r = two_sum(BGB_FMA(-kf, 0.015625f, yh), y.lo);  // yh - k/64 is exact
  const df2 t = df_mul(r, df2{kLn2Hi, kLn2Lo});
  const float th = t.hi;
  const float sq = BGB_FMUL(th, th);
  const float sq_lo = BGB_FMA(2.0f * th, t.lo, BGB_FMA(th, th, -sq));  // t^2 = sq + sq_lo
  const float tail = BGB_FMUL(BGB_FMUL(sq, th),
                              BGB_FMA(th, BGB_FMA(th, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f));
  const df2 s1 = two_sum(th, BGB_FMUL(sq, 0.5f));  // t.hi + t^2/2 (hi part), exact
  const df2 s = fast_two_sum(s1.hi, BGB_FADD(BGB_FADD(s1.lo, t.lo), BGB_FMA(sq_lo, 0.5f, tail)));
  const df2 T = {tab_hi[j + 32], tab_lo[j + 32]};
  return df_fma(T, s, T);
}

// 2^(float exponent) as a float, for n in [-126, 127]; 0 below.
BGB_HD float pow2f(int n) { return n < -126 ? 0.0f : bgb_int_as_float((n + 127) << 23); }

// Multiply a double-float by 2^n (exact unless it under/overflows the float range).
BGB_HD df2 df_ldexp(df2 a, int n) {
  if (n >= -126) {
    const float s = pow2f(n);
    return {BGB_FMUL(a.hi, s), BGB_FMUL(a.lo, s)};
  }
  // two steps for the lowest exponents (flushes below the float range)
  const float s1 = pow2f(-126), s2 = pow2f(n + 126);
  return {BGB_FMUL(BGB_FMUL(a.hi, s1), s2), BGB_FMUL(BGB_FMUL(a.lo, s1), s2)};
}

// 2^n as a double for n in [-1022, 1023]; 0 below.
BGB_HD double pow2d(int n) { return n < -1022 ? 0.0 : bgb_ll_as_double((long long)(n + 1023) << 52); }

// exp(x) in FP64 by Tang's method with a 2048-entry table (tab: 2^(j/2048), j = 0..2047):
// x = k ln2/2048 + r (Cody-Waite with a two-part ln2/2048 and FMA), |r| <= ln2/4096, so the
// degree-3 Taylor polynomial r + r^2/2 + r^3/6 suffices
// (remainder r^4/24 < 3.5e-17): 8 FP64 operations.
// Valid for x in [-700, 700]; about 1 ulp.
BGB_HD double exp_tang2048(double x, const double* tab) {
  const double shifter = 6755399441055744.0;  // 1.5 * 2^52
  const double t = BGB_DMA(x, k2048OverLn2, shifter);
  const int k = (int)(bgb_double_as_ll(t) & 0xffffffff);
  const double kd = i2d_bits(k);  // == t - shifter, formed on the integer pipe
  double r = BGB_DMA(-kd, kLn2Over2048Hi, x);
  r = BGB_DMA(-kd, kLn2Over2048Lo, r);
  double p = BGB_DMA(r, 1.0 / 6.0, 0.5);
  p = BGB_DMA(r * r, p, r);
  const int j = k & 2047;
  const int m = k >> 11;  // floor(k / 2048)
  const double T = tab[j];
  const double scaled = bgb_ll_as_double(bgb_double_as_ll(T) + ((long long)m << 52));
  return BGB_DMA(scaled, p, scaled);
}

// A float approximation of a double d >= 0 from its bits (truncated mantissa, relative
// error below 2^-23; 0 below the float normal range), formed on the integer pipe.
BGB_HD float d2f_trunc(double d) {
  const long long b = bgb_double_as_ll(d);
  if (((b >> 52) & 0x7ff) < 897) return 0.0f;
  return bgb_int_as_float((int)((b >> 29) - (896LL << 23)));
}

constexpr float k2048OverLn2F = (float)k2048OverLn2;

// exp_tang2048 with the table index chosen in FP32: k = round(xf 2048 / ln2) by the float
// shifter 1.5 * 2^23 (|xf| < 1400), xf a float estimate of x with relative error below
// 2^-23. k then differs from round(x 2048 / ln2) by at most 2^-23 |x| 2048 / ln2 + 1/2 in
// index units (0.25 at |x| = 700, 0.014 at |x| = 40), so |r| <= 0.75 ln2/2048 and the
// degree-3 polynomial's remainder r^4/24 stays below 1.7e-16 (2.7e-20 for |x| <= 40):
// one FP64 operation fewer than exp_tang2048. Valid for x in [-700, 700].
BGB_HD double exp_tang2048_f(double x, float xf, const double* tab) {
  const float tf = BGB_FMA(xf, k2048OverLn2F, 12582912.0f);
  const int k = (int)bgb_float_as_uint(tf) - 0x4B400000;
  const double kd = i2d_bits(k);
  double r = BGB_DMA(-kd, kLn2Over2048Hi, x);
  r = BGB_DMA(-kd, kLn2Over2048Lo, r);
  double p = BGB_DMA(r, 1.0 / 6.0, 0.5);
  p = BGB_DMA(r * r, p, r);
  const int j = k & 2047;
  const int m = k >> 11;  // floor(k / 2048)
  const double T = tab[j];
  const double scaled = bgb_ll_as_double(bgb_double_as_ll(T) + ((long long)m << 52));
  return BGB_DMA(scaled, p, scaled);
}

// exp(-d) in FP64 for a double-float d with 0 <= d.hi <= 700, by Tang's method with the
// table tab = 2^(j/2048): k = round(d 2048/ln2) is chosen in FP32 from d.hi (as in
// exp_tang2048_f, |r| <= 0.75 ln2/2048), the reduced argument r = k ln2/2048 - d is formed as
// a double-float from an error-free product and sum (ln2/2048 as the float pair
// kLn2Over2048FHi + kLn2Over2048FLo) whose low part is rounded once, q = e^r - 1 =
// r + r^2/2 + r^3/6 in double-float, and exp(-d) = 2^(-k/2048) (1 + q) with 2^(-k/2048) an
// FP64 table value times 2^m: one conversion add and one FMA on the FP64 pipe. The rounding
// of r's low part costs up to ~1e-14 d relative (~2^-47 d; d itself, a double-float product
// of the layer depth, carries about as much); the polynomial's remainder is below r^4/24.
// exp_neg_df_fp32 is the FP32 part (returns tf, the rounded index with its float shifter,
// and q = qh + ql); exp_neg_df_finish the integer and FP64 part.
BGB_HD void exp_neg_df_fp32(df2 d, float& tf, float& qh, float& ql) {
  tf = BGB_FMA(d.hi, k2048OverLn2F, 12582912.0f);
  const float kf = BGB_FSUB(tf, 12582912.0f);
  const float p = BGB_FMUL(kf, kLn2Over2048FHi);
  const float pe = BGB_FMA(kf, kLn2Over2048FHi, -p);  // k Ch = p + pe exactly
  const df2 s = two_sum(p, -d.hi);
  // the low parts (pe, d.lo ~ 2^-24 d) can reach a few percent of s.hi: renormalise
  const df2 r = two_sum(s.hi, BGB_FADD(s.lo, BGB_FADD(pe, BGB_FMA(kf, kLn2Over2048FLo, -d.lo))));
  const float rh = r.hi, rl = r.lo;
  const float sq = BGB_FMUL(rh, rh);
  const float sq_lo = BGB_FMA(BGB_FMUL(2.0f, rh), rl, BGB_FMA(rh, rh, -sq));  // r^2 = sq + sq_lo
  const float t3 = BGB_FMUL(BGB_FMUL(sq, rh), 1.0f / 6.0f);
  const df2 q1 = fast_two_sum(rh, BGB_FMUL(sq, 0.5f));
  qh = q1.hi;
  ql = BGB_FADD(q1.lo, BGB_FADD(rl, BGB_FMA(sq_lo, 0.5f, t3)));
}

BGB_HD double exp_neg_df_finish(float tf, float qh, float ql, const double* tab) {
  const int K = 0x4B400000 - (int)bgb_float_as_uint(tf);  // -k
  const int j = K & 2047;
  const int m = K >> 11;  // floor(K / 2048)
  const double T = tab[j];
  const double S = bgb_ll_as_double(bgb_double_as_ll(T) + ((long long)m << 52));
  const double q = f2d_bits(qh) + f2d_bits(ql);
  return BGB_DMA(S, q, S);
}

BGB_HD double exp_neg_df(df2 d, const double* tab) {
  float tf, qh, ql;
  exp_neg_df_fp32(d, tf, qh, ql);
  return exp_neg_df_finish(tf, qh, ql, tab);
}

}  // namespace bgb
