// Two-wavenumber versions of the emission helpers in rt_common.cuh and physics.cuh.
//
// A thread of emission_kernel_x2 carries the wavenumbers k0 (element 0) and k1
// (element 1). Every double-float step below is the rt_common.cuh / physics.cuh step,
// issued once for both elements with paired FP32 instructions (dfloat2x.cuh), so each
// element's result is bit for bit the single-wavenumber result; branches that can differ
// between the elements (terms outside the float exponent range, the Planck function's
// small-u regime, layers outside the comfortable float range) fall back to the scalar code
// for that element.
#pragma once

#include "dfloat2x.cuh"
#include "rt_common.cuh"

namespace bgb {

struct KappaX {
  dfx v;
  double wide0, wide1;
};

// level_kappa_df_cb for wavenumbers k0 and k1: the sum over table species of 2^y n with
// y = lo + (hi - lo) wT + log2 n (level-table values, log2 units). The level-table reads
// of GRP species are issued before their arithmetic (the order of the sum is unchanged).
// term(s, t, wide0, wide1, lo, hi) receives each species' term of both wavenumbers (zero
// for an element whose term lies outside the float range, flagged wide, and for a species
// of zero number density).
template <int GRP = 1, class F>
__device__ __forceinline__ KappaX level_kappa_x_cb(const float2* __restrict__ ltab, size_t N,
                                                   const LevelSpeciesDF* __restrict__ f, int S, int k0, int k1,
                                                   const ExpTables& et, F&& term) {
  KappaX r;
  r.wide0 = r.wide1 = 0.0;
  float2 acc_hi = f2(0.0f), acc_lo = f2(0.0f);
  const dfx zero = {f2(0.0f), f2(0.0f)};
  for (int s0 = 0; s0 < S; s0 += GRP) {
    float4 fb[GRP];
    float2 a0[GRP], a1[GRP], b0[GRP], b1[GRP];
#pragma unroll
    for (int g = 0; g < GRP; ++g) {
      if (s0 + g >= S) break;
      const int4 rw = __ldg(reinterpret_cast<const int4*>(f + s0 + g));
      fb[g] = __ldg(reinterpret_cast<const float4*>(f + s0 + g) + 1);  // wT, log2 n
      if (fb[g].z != kNoSpecies) {
        const float2* r0 = ltab + (size_t)rw.x * N;
        const float2* r1 = ltab + (size_t)rw.y * N;
        a0[g] = __ldg(r0 + k0);
        a1[g] = __ldg(r0 + k1);
        b0[g] = __ldg(r1 + k0);
        b1[g] = __ldg(r1 + k1);
      }
    }
#pragma unroll
    for (int g = 0; g < GRP; ++g) {
      const int s = s0 + g;
      if (s >= S) break;
      if (fb[g].z == kNoSpecies) {  // zero number density: the species adds nothing
        term(s, zero, false, false, zero, zero);
        continue;
      }
      const dfx lo = {make_float2(a0[g].x, a1[g].x), make_float2(a0[g].y, a1[g].y)};
      const dfx hi = {make_float2(b0[g].x, b1[g].x), make_float2(b0[g].y, b1[g].y)};
      const dfx y =
          dfx_fma(dfx_sub(hi, lo), dfx_bcast(df2{fb[g].x, fb[g].y}), dfx_add(lo, dfx_bcast(df2{fb[g].z, fb[g].w})));
      int2 n;
      const dfx m = dfx_exp2(y, n, et.hi, et.lo);
      const bool nar0 = n.x > -100 && n.x < 100, nar1 = n.y > -100 && n.y < 100;
      if (nar0 && nar1) {
        const dfx t = dfx_ldexp_normal(m, n);
        const dfx a = two_sum_x(acc_hi, t.hi);
        acc_hi = a.hi;
        acc_lo = f2add(acc_lo, f2add(a.lo, t.lo));
        term(s, t, false, false, lo, hi);
      } else {
        // one or both terms outside the float exponent range: the scalar steps per element
        dfx tt = zero;
        if (nar0) {
          const df2 t = df_ldexp(dfx_get(m, 0), n.x);
          const df2 a = two_sum(acc_hi.x, t.hi);
          acc_hi.x = a.hi;
          acc_lo.x = BGB_FADD(acc_lo.x, BGB_FADD(a.lo, t.lo));
          dfx_set(tt, 0, t);
        } else {
          r.wide0 += df_to_double(dfx_get(m, 0)) * pow2d(n.x);
        }
        if (nar1) {
          const df2 t = df_ldexp(dfx_get(m, 1), n.y);
          const df2 a = two_sum(acc_hi.y, t.hi);
          acc_hi.y = a.hi;
          acc_lo.y = BGB_FADD(acc_lo.y, BGB_FADD(a.lo, t.lo));
          dfx_set(tt, 1, t);
        } else {
          r.wide1 += df_to_double(dfx_get(m, 1)) * pow2d(n.y);
        }
        term(s, tt, !nar0, !nar1, lo, hi);
      }
    }
  }
  r.v = fast_two_sum_x(acc_hi, acc_lo);
  return r;
}

template <int GRP = 1>
__device__ __forceinline__ KappaX level_kappa_x(const float2* __restrict__ ltab, size_t N,
                                                const LevelSpeciesDF* __restrict__ f, int S, int k0, int k1,
                                                const ExpTables& et) {
  return level_kappa_x_cb<GRP>(ltab, N, f, S, k0, k1, et,
                               [](int, const dfx&, bool, bool, const dfx&, const dfx&) {});
}

// df_exp_neg (physics.cuh) for two double-floats
__device__ __forceinline__ dfx dfx_exp_neg(dfx d, const float* tab_hi, const float* tab_lo) {
  int2 n;
  const dfx m = dfx_exp2(dfx_neg(dfx_mul(d, dfx_bcast(df2{kLog2eHi, kLog2eLo}))), n, tab_hi, tab_lo);
  const dfx z = {f2(0.0f), f2(0.0f)};
  return dfx_select(d.hi.x > 700.0f, d.hi.y > 700.0f, z, dfx_ldexp(m, n));
}

// planck_dd (physics.cuh) for two wavenumbers.
struct PlanckX {
  dfx v;
  double d0, d1;
  bool tiny0, tiny1;
};

__device__ __forceinline__ PlanckD planck_get(const PlanckX& b, int e) {
  PlanckD r;
  r.v = dfx_get(b.v, e);
  r.d = e ? b.d1 : b.d0;
  r.tiny = e ? b.tiny1 : b.tiny0;
  return r;
}

__device__ __forceinline__ PlanckX planck_x(dfx c1, dfx c2l, df2 invT, const ExpTables& et) {
  const dfx y = dfx_neg(dfx_mul(c2l, dfx_bcast(invT)));
  int2 n;
  const dfx m = dfx_exp2(y, n, et.hi, et.lo);  // u = m 2^n, n <= 0
  PlanckX r;
  if (n.x >= -60 && n.y >= -60) {
    const dfx u = dfx_ldexp_normal(m, n);
    const dfx d = dfx_sub(dfx_bcast(df_make(1.0f)), u);
    r.v = dfx_mul(dfx_mul(c1, u), dfx_recip(d));
    r.d0 = r.d1 = 0.0;
    r.tiny0 = r.tiny1 = false;
    return r;
  }
  // the scalar steps per element
  PlanckD b[2];
  for (int e = 0; e < 2; ++e) {
    const df2 me = dfx_get(m, e), c1e = dfx_get(c1, e);
    const int ne = e ? n.y : n.x;
    if (ne < -60) {
      b[e].v = df2{0.0f, 0.0f};
      b[e].d = df_to_double(df_mul(c1e, me)) * pow2d(ne);
      b[e].tiny = true;
    } else {
      const df2 u = df_ldexp(me, ne);
      const df2 d = df_sub(df_make(1.0f), u);
      b[e].v = df_mul(df_mul(c1e, u), df_recip(d));
      b[e].d = 0.0;
      b[e].tiny = false;
    }
  }
  r.v = dfx_make(b[0].v, b[1].v);
  r.d0 = b[0].d;
  r.d1 = b[1].d;
  r.tiny0 = b[0].tiny;
  r.tiny1 = b[1].tiny;
  return r;
}

// exp_neg_df_fp32 (dfloat.cuh) for two double-floats.
__device__ __forceinline__ void exp_neg_x_fp32(dfx d, float2& tf, float2& qh, float2& ql) {
  tf = f2fma(d.hi, f2(k2048OverLn2F), f2(12582912.0f));
  const float2 kf = f2add(tf, f2(-12582912.0f));
  const float2 p = f2mul(kf, f2(kLn2Over2048FHi));
  const float2 pe = f2fma(kf, f2(kLn2Over2048FHi), f2neg(p));
  const dfx s = two_sum_x(p, f2neg(d.hi));
  const dfx r = two_sum_x(s.hi, f2add(s.lo, f2add(pe, f2fma(kf, f2(kLn2Over2048FLo), f2neg(d.lo)))));
  const float2 rh = r.hi, rl = r.lo;
  const float2 sq = f2mul(rh, rh);
  const float2 sq_lo = f2fma(f2mul(f2(2.0f), rh), rl, f2fma(rh, rh, f2neg(sq)));
  const float2 t3 = f2mul(f2mul(sq, rh), f2(1.0f / 6.0f));
  const dfx q1 = fast_two_sum_x(rh, f2mul(sq, f2(0.5f)));
  qh = q1.hi;
  ql = f2add(q1.lo, f2add(rl, f2fma(sq_lo, f2(0.5f), t3)));
}

// emission_layer (rt_common.cuh) for two wavenumbers: K1[e], K2[e] of element e; with OUT,
// tk0 / tk1 receive the stored layer depth and half opacity sum of each element.
template <bool OUT = false>
__device__ __forceinline__ void emission_layer_x(const LevelInfo* __restrict__ lv, int l, const KappaX& kap,
                                                 const KappaX& kap_prev, const PlanckX& B, const PlanckX& Bp,
                                                 double (&K1)[2], double (&K2)[2], const double* tab2048,
                                                 float4* tk0 = nullptr, float4* tk1 = nullptr) {
  const float4 g = __ldg(reinterpret_cast<const float4*>(&lv[l - 1].dzh_hi));  // dzh, cloud
  const dfx ks = dfx_add(kap.v, kap_prev.v);
  const dfx t = dfx_add(dfx_mul(dfx_bcast(df2{g.x, g.y}), ks), dfx_bcast(df2{g.z, g.w}));
  const bool nar0 = ((__double_as_longlong(kap.wide0) | __double_as_longlong(kap_prev.wide0)) << 1) == 0 &&
                    t.hi.x > 1e-30f && t.hi.x < 1e30f;
  const bool nar1 = ((__double_as_longlong(kap.wide1) | __double_as_longlong(kap_prev.wide1)) << 1) == 0 &&
                    t.hi.y > 1e-30f && t.hi.y < 1e30f;
  if (nar0 && nar1 && !(B.tiny0 | B.tiny1 | Bp.tiny0 | Bp.tiny1)) {
    if (OUT) {
      const dfx ksh = dfx_mul_f(ks, f2(0.5f));
      *tk0 = make_float4(t.hi.x, t.lo.x, ksh.hi.x, ksh.lo.x);
      *tk1 = make_float4(t.hi.y, t.lo.y, ksh.hi.y, ksh.lo.y);
    }
    const dfx ux = dfx_mul(dfx_sub(B.v, Bp.v), dfx_recip(t));
    const double u0 = df_to_double(dfx_get(ux, 0)), u1 = df_to_double(dfx_get(ux, 1));
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const dfx d =
          dfx_mul(t, dfx_bcast(i == 0 ? df2{kInvMuF[0][0], kInvMuF[0][1]} : df2{kInvMuF[1][0], kInvMuF[1][1]}));
      float2 tf, qh, ql;
      exp_neg_x_fp32(d, tf, qh, ql);
      const double a0 = d.hi.x > 700.0f ? 0.0 : exp_neg_df_finish(tf.x, qh.x, ql.x, tab2048);
      const double a1 = d.hi.y > 700.0f ? 0.0 : exp_neg_df_finish(tf.y, qh.y, ql.y, tab2048);
      double(&K)[2] = i == 0 ? K1 : K2;
      K[0] = fma(a0, K[0], fma(a0, u0, -u0));
      K[1] = fma(a1, K[1], fma(a1, u1, -u1));
    }
    return;
  }
  // the scalar steps per element
  for (int e = 0; e < 2; ++e) {
    Kappa kc, kp;
    kc.v = dfx_get(kap.v, e);
    kc.wide = e ? kap.wide1 : kap.wide0;
    kp.v = dfx_get(kap_prev.v, e);
    kp.wide = e ? kap_prev.wide1 : kap_prev.wide0;
    emission_layer<false, OUT>(lv, l, kc, kp, planck_get(B, e), planck_get(Bp, e), K1[e], K2[e], tab2048, 1.0,
                               df2{1.0f, 0.0f}, OUT ? (e ? tk1 : tk0) : nullptr);
  }
}

}  // namespace bgb
