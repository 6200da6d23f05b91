// Two independent double-floats per thread with paired FP32 arithmetic.
//
// Blackwell issues FADD2 / FMUL2 / FFMA2 (__fadd2_rn, __fmul2_rn, __ffma2_rn): one
// instruction performs the same FP32 operation on the two halves of a register pair, each
// rounded exactly as the scalar __fadd_rn / __fmul_rn / __fmaf_rn would round it. A kernel
// that carries two wavenumbers per thread therefore runs the double-float arithmetic of
// dfloat.cuh for both in one instruction stream: element e of every dfx result is bit for
// bit the dfloat.cuh result for element e's inputs, with half the FP32 issue slots. (On this
// GPU the FP32 pipe is rarely full; the issue slot is what the double-float kernels run out of.)
//
// Integer parts (exponent and table-index extraction) and table lookups stay per element.
#pragma once

#include "dfloat.cuh"

namespace bgb {

struct dfx {
  float2 hi, lo;  // element 0 in .x, element 1 in .y
};

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as one paired FMA: b * (-1) + a, rounded once (exactly the scalar a - b)
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ dfx dfx_make(df2 a, df2 b) { return {make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
__device__ __forceinline__ df2 dfx_get(const dfx& a, int e) {
  return e ? df2{a.hi.y, a.lo.y} : df2{a.hi.x, a.lo.x};
}
__device__ __forceinline__ dfx dfx_bcast(df2 a) { return {f2(a.hi), f2(a.lo)}; }

// TwoSum per element (dfloat.cuh two_sum)
__device__ __forceinline__ dfx two_sum_x(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  const float2 bb = f2sub(s, a);
  const float2 e = f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
  return {s, e};
}

// Fast2Sum per element (|a| >= |b|)
__device__ __forceinline__ dfx fast_two_sum_x(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  return {s, f2sub(b, f2sub(s, a))};
}

__device__ __forceinline__ dfx dfx_add(dfx a, dfx b) {
  const dfx s = two_sum_x(a.hi, b.hi);
  return fast_two_sum_x(s.hi, f2add(s.lo, f2add(a.lo, b.lo)));
}

__device__ __forceinline__ dfx dfx_neg(dfx a) { return {f2neg(a.hi), f2neg(a.lo)}; }

__device__ __forceinline__ dfx dfx_sub(dfx a, dfx b) { return dfx_add(a, dfx_neg(b)); }

__device__ __forceinline__ dfx dfx_mul(dfx a, dfx b) {
  const float2 p = f2mul(a.hi, b.hi);
  float2 e = f2fma(a.hi, b.hi, f2neg(p));
  e = f2fma(a.hi, b.lo, e);
  e = f2fma(a.lo, b.hi, e);
  return fast_two_sum_x(p, e);
}

__device__ __forceinline__ dfx dfx_mul_f(dfx a, float2 b) {
  const float2 p = f2mul(a.hi, b);
  float2 e = f2fma(a.hi, b, f2neg(p));
  e = f2fma(a.lo, b, e);
  return fast_two_sum_x(p, e);
}

__device__ __forceinline__ dfx dfx_fma(dfx a, dfx b, dfx c) {
  const float2 p = f2mul(a.hi, b.hi);
  float2 e = f2fma(a.hi, b.hi, f2neg(p));
  e = f2fma(a.hi, b.lo, e);
  e = f2fma(a.lo, b.hi, e);
  const dfx s = two_sum_x(c.hi, p);
  return fast_two_sum_x(s.hi, f2add(s.lo, f2add(e, c.lo)));
}

// 1 / b per element (dfloat.cuh df_recip)
__device__ __forceinline__ dfx dfx_recip(dfx b) {
  const float2 r0 = make_float2(bgb_rcp_approx(b.hi.x), bgb_rcp_approx(b.hi.y));
  const float2 e = f2fma(f2neg(b.lo), r0, f2fma(f2neg(b.hi), r0, f2(1.0f)));
  return fast_two_sum_x(r0, f2mul(r0, f2fma(e, e, e)));
}

// 2^y per element (dfloat.cuh df_exp2): mantissa m and exponents n.x, n.y with 2^y = m 2^n.
__device__ __forceinline__ dfx dfx_exp2(dfx y, int2& n, const float* tab_hi, const float* tab_lo) {
  float2 yh;
  {
    const float c0 = fminf(fmaxf(y.hi.x, -16000.0f), 16000.0f), c1 = fminf(fmaxf(y.hi.y, -16000.0f), 16000.0f);
    yh = make_float2(y.hi.x != y.hi.x ? y.hi.x : c0, y.hi.y != y.hi.y ? y.hi.y : c1);
  }
  const float2 tf = f2fma(yh, f2(64.0f), f2(12582912.0f));
  const int k0 = (int)__float_as_uint(tf.x) - 0x4B400000, k1 = (int)__float_as_uint(tf.y) - 0x4B400000;
  const float2 kf = f2add(tf, f2(-12582912.0f));
  n.x = (k0 + 32) >> 6;
  n.y = (k1 + 32) >> 6;
  const int j0 = k0 - (n.x << 6), j1 = k1 - (n.y << 6);
  const dfx r = two_sum_x(f2fma(f2neg(kf), f2(0.015625f), yh), y.lo);  // yh - k/64 is exact
  const dfx t = dfx_mul(r, dfx_bcast(df2{kLn2Hi, kLn2Lo}));
  const float2 th = t.hi;
  const float2 sq = f2mul(th, th);
  const float2 sq_lo = f2fma(f2mul(f2(2.0f), th), t.lo, f2fma(th, th, f2neg(sq)));
  const float2 tail = f2mul(f2mul(sq, th), f2fma(th, f2fma(th, f2(1.0f / 120.0f), f2(1.0f / 24.0f)), f2(1.0f / 6.0f)));
  const dfx s1 = two_sum_x(th, f2mul(sq, f2(0.5f)));
  const dfx s = fast_two_sum_x(s1.hi, f2add(f2add(s1.lo, t.lo), f2fma(sq_lo, f2(0.5f), tail)));
  const dfx T = {make_float2(tab_hi[j0 + 32], tab_hi[j1 + 32]), make_float2(tab_lo[j0 + 32], tab_lo[j1 + 32])};
  return dfx_fma(T, s, T);
}

// m 2^n per element for n >= -126 on both (dfloat.cuh df_ldexp's first branch).
__device__ __forceinline__ dfx dfx_ldexp_normal(dfx m, int2 n) {
  const float2 s = make_float2(pow2f(n.x), pow2f(n.y));
  return {f2mul(m.hi, s), f2mul(m.lo, s)};
}

// df_ldexp for any n <= 127 per element: the two-step scaling of its second branch, with
// the second factor 1 (an exact multiplication) for an element in the first branch's range.
__device__ __forceinline__ dfx dfx_ldexp(dfx m, int2 n) {
  const bool w0 = n.x >= -126, w1 = n.y >= -126;
  const float2 s1 = make_float2(pow2f(w0 ? n.x : -126), pow2f(w1 ? n.y : -126));
  const float2 s2 = make_float2(w0 ? 1.0f : pow2f(n.x + 126), w1 ? 1.0f : pow2f(n.y + 126));
  return {f2mul(f2mul(m.hi, s1), s2), f2mul(f2mul(m.lo, s1), s2)};
}

// element e of a where c_e holds, of b elsewhere
__device__ __forceinline__ dfx dfx_select(bool c0, bool c1, dfx a, dfx b) {
  return {make_float2(c0 ? a.hi.x : b.hi.x, c1 ? a.hi.y : b.hi.y),
          make_float2(c0 ? a.lo.x : b.lo.x, c1 ? a.lo.y : b.lo.y)};
}

// element e replaced by the double-float v
__device__ __forceinline__ void dfx_set(dfx& a, int e, df2 v) {
  if (e) {
    a.hi.y = v.hi;
    a.lo.y = v.lo;
  } else {
    a.hi.x = v.hi;
    a.lo.x = v.lo;
  }
}

}  // namespace bgb
