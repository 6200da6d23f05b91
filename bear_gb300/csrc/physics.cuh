// Per-wavenumber physics helpers shared by the radiative-transfer kernels,
// written on top of dfloat.cuh (host-compilable for accuracy checks).
#pragma once

#include "dfloat.cuh"

namespace bgb {

// Exponential tables staged in shared memory (divergent indices).
struct ExpTables {
  float hi[65];
  float lo[65];
};

// Planck function B_nu(T) = 2 h c^2 nu^3 / (exp(h nu c / k T) - 1)
// (aux::planckFunctionWavenumber, src/additional/aux_functions.cpp:272-278),
// evaluated as c1 u / (1 - u) with u = 2^(-(h nu c / k) log2(e) / T) in
// double-float arithmetic. c1 = 2 h c^2 nu^3 and c2l = (h nu c / k) log2(e) as
// double-floats, invT = 1/T as a double-float. Returns FP64.
BGB_HD double planck_df(df2 c1, df2 c2l, df2 invT, const float* tab_hi, const float* tab_lo) {
  const df2 y = df_neg(df_mul(c2l, invT));
  int n;
  const df2 m = df_exp2(y, n, tab_hi, tab_lo);  // u = m 2^n, n <= 0
  if (n < -60) return df_to_double(df_mul(c1, m)) * pow2d(n);  // 1 - u == 1 at this precision
  const df2 u = df_ldexp(m, n);
  const df2 d = df_sub(df_make(1.0f), u);
  return df_to_double(df_mul(df_mul(c1, u), df_recip(d)));
}

// The Planck function of planck_df kept as a double-float for the emission recurrence,
// which forms (B - B') / tau in double-float. tiny: u = exp(-h nu c / k T) < 2^-60, where
// the double-float can leave the float range; then d holds B in FP64 (as planck_df returns
// it) and the recurrence takes its FP64 path for the layers next to this level.
struct PlanckD {
  df2 v;
  double d;
  bool tiny;
};

BGB_HD PlanckD planck_dd(df2 c1, df2 c2l, df2 invT, const float* tab_hi, const float* tab_lo) {
  const df2 y = df_neg(df_mul(c2l, invT));
  int n;
  const df2 m = df_exp2(y, n, tab_hi, tab_lo);  // u = m 2^n, n <= 0
  PlanckD r;
  if (n < -60) {
    r.v = df2{0.0f, 0.0f};
    r.d = df_to_double(df_mul(c1, m)) * pow2d(n);  // 1 - u == 1 at this precision
    r.tiny = true;
    return r;
  }
  const df2 u = df_ldexp(m, n);
  const df2 d = df_sub(df_make(1.0f), u);
  r.v = df_mul(df_mul(c1, u), df_recip(d));
  r.d = 0.0;
  r.tiny = false;
  return r;
}

// B in FP64 (the value planck_df returns).
BGB_HD double planck_value(const PlanckD& b) { return b.tiny ? b.d : df_to_double(b.v); }

// The same Planck function returned as a double-float (values below the float
// range flush to zero); used by the adjoint, whose arithmetic is double-float.
BGB_HD df2 planck_df2(df2 c1, df2 c2l, df2 invT, const float* tab_hi, const float* tab_lo) {
  const df2 y = df_neg(df_mul(c2l, invT));
  int n;
  const df2 m = df_exp2(y, n, tab_hi, tab_lo);
  if (n < -60) return df_ldexp(df_mul(c1, m), n);
  const df2 u = df_ldexp(m, n);
  const df2 d = df_sub(df_make(1.0f), u);
  return df_mul(df_mul(c1, u), df_recip(d));
}

// exp(-d) for a double-float d >= 0 (0 for d > 700 and below the float range).
BGB_HD df2 df_exp_neg(df2 d, const float* tab_hi, const float* tab_lo) {
  if (d.hi > 700.0f) return df2{0.0f, 0.0f};
  int n;
  const df2 m = df_exp2(df_neg(df_mul(d, df2{kLog2eHi, kLog2eLo})), n, tab_hi, tab_lo);
  return df_ldexp(m, n);
}

// 10^x * n as a double for a double-float log10 cross section x and log2(n):
// 2^(x log2(10) + log2(n)).
BGB_HD double pow10_times_n(df2 x, df2 lg2n, const float* tab_hi, const float* tab_lo, df2& acc, double& wide) {
  const df2 y = df_add(df_mul(x, df2{kLog2_10Hi, kLog2_10Lo}), lg2n);
  int n;
  const df2 m = df_exp2(y, n, tab_hi, tab_lo);
  if (n > -100 && n < 100) {
    acc = df_add(acc, df_ldexp(m, n));
  } else {
    wide += df_to_double(m) * pow2d(n);  // outside the float exponent range: FP64 accumulator
  }
  return 0.0;
}

}  // namespace bgb
