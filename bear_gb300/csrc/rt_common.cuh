// Per-wavenumber device helpers shared by the forward kernels (engine.cu) and
// the adjoint kernels (adjoint.cu): level opacity assembly, the layer optical
// depth of the emission recurrence and the short-characteristics layer update.
// The adjoint recomputes level opacities with exactly these functions, so the
// optical depths it differentiates are bit-identical to the forward pass.
#pragma once

#include "model.h"
#include "physics.cuh"

namespace bgb {

// Gauss nodes of ShortCharacteristics (src/radiative_transfer/short_characteristics.h:62-63)
static __device__ __constant__ double kMu[2] = {0.211324865405187, 0.788675134594813};
static __device__ __constant__ double kInvMu[2] = {1.0 / 0.211324865405187, 1.0 / 0.788675134594813};

// 700.0 as the bit pattern of a double: for non-negative x, x > 700 <=>
// bits(x) > bits(700) (an integer comparison, off the FP64 pipe).
constexpr long long kBits700 = 0x4085E00000000000LL;

__device__ __forceinline__ void load_exp_tables(ExpTables& t) {
  for (int i = threadIdx.x; i < 65; i += blockDim.x) {
    t.hi[i] = kExp2TabHi[i];
    t.lo[i] = kExp2TabLo[i];
  }
}

// Level opacity as a double-float plus an FP64 part for terms outside the float
// exponent range (zero almost always).
struct Kappa {
  df2 v;
  double wide;
};

// Sum over table species of 10^(bilinear log-p / T interpolation) * n at one
// level and one wavenumber (OpacitySpecies::calcAbsorptionCrossSections
// src/transport_coeff/opacity_species.cpp:277-345 and calcTransportCoefficients
// :400-455), double-float arithmetic. The log-p step of the interpolation depends
// only on the fixed pressure grid and is read from the level table ltab (log2
// units), so one evaluation does the temperature step:
// y = lo + (hi - lo) wT + log2(n), term = 2^y. term(s, t, t_wide, is_wide, lo, hi)
// is called for every species with its term (t as a double-float, or t_wide in
// FP64 when outside the float range; zero for a skipped species) and the level
// table values at the lower and upper temperature nodes (log2 units).
// GRP: species handled per group; a group's table reads are issued together before its
// arithmetic (the accumulation order is unchanged), which hides memory latency where
// registers allow.
template <int GRP = 1, class F>
__device__ __forceinline__ Kappa level_kappa_df_cb(const float2* __restrict__ ltab, size_t N,
                                                   const LevelSpeciesDF* __restrict__ f, int S, int k,
                                                   const ExpTables& et, F&& term) {
  Kappa r = {{0.0f, 0.0f}, 0.0};
  // the sum as an unnormalised pair: exact two-sum into hi, low parts added into lo,
  // renormalised once at the end
  float acc_hi = 0.0f, acc_lo = 0.0f;
  for (int s0 = 0; s0 < S; s0 += GRP) {
    int4 rw[GRP];
    float4 fb[GRP];
    float2 t0[GRP], t1[GRP];
#pragma unroll
    for (int g = 0; g < GRP; ++g) {
      if (s0 + g >= S) break;
      rw[g] = __ldg(reinterpret_cast<const int4*>(f + s0 + g));
      fb[g] = __ldg(reinterpret_cast<const float4*>(f + s0 + g) + 1);  // wT, log2 n
      if (fb[g].z != kNoSpecies) {
        t0[g] = __ldg(ltab + (size_t)rw[g].x * N + k);
        t1[g] = __ldg(ltab + (size_t)rw[g].y * N + k);
      }
    }
#pragma unroll
    for (int g = 0; g < GRP; ++g) {
      const int s = s0 + g;
      if (s >= S) break;
      if (fb[g].z == kNoSpecies) {  // zero number density: the species adds nothing
        term(s, df2{0.0f, 0.0f}, 0.0, false, df2{0.0f, 0.0f}, df2{0.0f, 0.0f});
        continue;
      }
      const df2 lo = {t0[g].x, t0[g].y}, hi = {t1[g].x, t1[g].y};
      // lo + (hi - lo) wT + log2 n
      const df2 y = df_fma(df_sub(hi, lo), df2{fb[g].x, fb[g].y}, df_add(lo, df2{fb[g].z, fb[g].w}));
      int n;
      const df2 m = df_exp2(y, n, et.hi, et.lo);
      if (n > -100 && n < 100) {
        const df2 t = df_ldexp(m, n);
        const df2 a = two_sum(acc_hi, t.hi);
        acc_hi = a.hi;
        acc_lo = BGB_FADD(acc_lo, BGB_FADD(a.lo, t.lo));
        term(s, t, 0.0, false, lo, hi);
      } else {
        const double w = df_to_double(m) * pow2d(n);
        r.wide += w;
        term(s, df2{0.0f, 0.0f}, w, true, lo, hi);
      }
    }
  }
  r.v = fast_two_sum(acc_hi, acc_lo);
  return r;
}

struct NoTerm {
  __device__ __forceinline__ void operator()(int, df2, double, bool, df2, df2) const {}
};

template <int GRP = 1>
__device__ __forceinline__ Kappa level_kappa_df(const float2* __restrict__ ltab, size_t N,
                                                const LevelSpeciesDF* __restrict__ f, int S, int k,
                                                const ExpTables& et) {
  return level_kappa_df_cb<GRP>(ltab, N, f, S, k, et, NoTerm{});
}

// The same sum in FP64 with the CUDA math library (validation path);
// term(s, t, lo, hi) receives each species' term 10^x n.
template <class F>
__device__ __forceinline__ double level_absorption_fp64_cb(const double* __restrict__ tab, size_t N,
                                                           const LevelSpecies* __restrict__ d, int S, int k,
                                                           F&& term) {
  double kap = 0.0;
  for (int s = 0; s < S; ++s) {
    const int4 r = __ldg(reinterpret_cast<const int4*>(d + s));
    const double2 w = __ldg(reinterpret_cast<const double2*>(&d[s].wp_lo));
    const double2 t = __ldg(reinterpret_cast<const double2*>(&d[s].wT));
    const double v0 = __ldg(tab + (size_t)r.x * N + k);
    const double v1 = __ldg(tab + (size_t)r.y * N + k);
    const double v2 = __ldg(tab + (size_t)r.z * N + k);
    const double v3 = __ldg(tab + (size_t)r.w * N + k);
    const double lo = v0 + (v1 - v0) * w.x;
    const double hi = v2 + (v3 - v2) * w.y;
    const double x = lo + (hi - lo) * t.x;
    const double term_s = exp10(x) * t.y;
    kap += term_s;
    term(s, term_s, lo, hi);
  }
  return kap;
}

struct NoTerm64 {
  __device__ __forceinline__ void operator()(int, double, double, double) const {}
};

__device__ __forceinline__ double level_absorption_fp64(const double* __restrict__ tab, size_t N,
                                                        const LevelSpecies* __restrict__ d, int S, int k) {
  return level_absorption_fp64_cb(tab, N, d, S, k, NoTerm64{});
}

// Wavelength factor of the non-grey clouds at wavenumber k (1 for grey):
// power law wl^a / wl_ref^a (PowerLawCloudModel::opticalProperties
// src/cloud_model/power_law_cloud_model.cpp:113-119), KH non-grey
// Q_ref / (q0 x^-a0 + x^0.2) with x = 2 pi r / wl (KHCloudModel::opticalProperties
// src/cloud_model/kh_cloud_model.cpp:115-132), FP64.
__device__ __forceinline__ double cloud_shape(const DeviceModel& dm, const EvalInfo& e, int k) {
  const double wl = __ldg(&dm.wl[k]);
  if (dm.cloud_kind == 1) return pow(wl, e.cs[0]) / e.cs[3];
  const double x = e.cs[2] / wl;
  return e.cs[3] / (e.cs[0] * pow(x, -e.cs[1]) + pow(x, 0.2));
}

// Derivatives of cloud_shape along the cloud's shape parameters, FP64: power law
// d/d a of (wl / wl_ref)^a; KH d/d q0, d/d a0, d/d r of Q_ref / Q with
// Q = q0 x^-a0 + x^0.2, x = 2 pi r / wl (Q_ref at the reference wavelength).
__device__ __forceinline__ void cloud_shape_tangent(const DeviceModel& dm, const EvalInfo& e, int k, double d[3]) {
  const double wl = __ldg(&dm.wl[k]);
  const double wl_ref = dm.cfg->cloud_ref_wl;
  d[0] = d[1] = d[2] = 0.0;
  if (dm.cloud_kind == 1) {
    d[0] = pow(wl, e.cs[0]) / e.cs[3] * (log(wl) - log(wl_ref));
    return;
  }
  const double q0 = e.cs[0], a0 = e.cs[1], tpr = e.cs[2];
  const double x = tpr / wl, xr = tpr / wl_ref;
  const double xa = pow(x, -a0), xra = pow(xr, -a0);
  const double Q = q0 * xa + pow(x, 0.2), Qr = e.cs[3];
  const double f = Qr / Q;
  // dQ/dr = dQ/dx dx/dr with dQ/dx = (-a0 q0 x^-a0 + 0.2 x^0.2) / x and dx/dr = x / r
  const double r = tpr / (2.0 * kPi);
  const double dQ_dr = (-a0 * q0 * xa + 0.2 * pow(x, 0.2)) / r;
  const double dQr_dr = (-a0 * q0 * xra + 0.2 * pow(xr, 0.2)) / r;
  d[0] = f * (xra / Qr - xa / Q);                                  // q0
  d[1] = f * (-q0 * xra * log(xr) / Qr + q0 * xa * log(x) / Q);    // a0
  d[2] = f * (dQr_dr / Qr - dQ_dr / Q);                            // r
}

// 1/mu_i of the Gauss angles as double-floats.
constexpr float kInvMuF[2][2] = {{(float)(1.0 / 0.211324865405187),
                                  (float)(1.0 / 0.211324865405187 - (double)(float)(1.0 / 0.211324865405187))},
                                 {(float)(1.0 / 0.788675134594813),
                                  (float)(1.0 / 0.788675134594813 - (double)(float)(1.0 / 0.788675134594813))}};

// One layer of the two-angle short-characteristics recurrence
// (ShortCharacteristics::calcSpectrum src/radiative_transfer/short_characteristics.cpp:85-115):
// delta = tau/mu, a = exp(-delta), I <- I a + (1 + (a-1)/delta) B_top + (-a - (a-1)/delta) B_bottom.
// All FP64 with the CUDA math library (the validation path).
__device__ __forceinline__ void sc_layer(double tau, double B, double B_prev, double& I1, double& I2) {
  if (tau == 0) return;  // the reference skips exactly transparent layers only
  const double rtau = 1.0 / tau;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double d = tau * kInvMu[i];
    const double a = exp(-d);
    const double q = (a - 1.0) * (kMu[i] * rtau);
    double& I = i == 0 ? I1 : I2;
    I = I * a;
    I += (1.0 + q) * B + (-a - q) * B_prev;
  }
}

// The FP64 form of emission_layer below (the CUDA-free table exponential exp_tang2048):
// layers with an opacity term outside the float range or a depth outside the comfortable
// float range, layers next to a level whose Planck function is below the float range, and
// exactly transparent layers (tau == 0, which the reference skips: I stays, so K_i moves by
// (B' - B) / mu_i). tau_df: tau as the double-float path formed it (when `narrow`).
template <bool SHAPE, bool OUT>
__device__ __noinline__ void emission_layer_fp64(const LevelInfo* __restrict__ lv, int l, const Kappa& kap,
                                                 const Kappa& kap_prev, bool narrow, df2 tau_df, df2 ks,
                                                 double B, double Bp, double& K1, double& K2,
                                                 const double* tab2048, double csh, float4* tk) {
  double tau;
  if (narrow) {
    tau = df_to_double(tau_df);
    if (OUT) {
      const df2 ksh = df_mul_f(ks, 0.5f);
      *tk = make_float4(tau_df.hi, tau_df.lo, ksh.hi, ksh.lo);
    }
  } else {
    const double ks64 = (df_to_double(kap.v) + kap.wide) + (df_to_double(kap_prev.v) + kap_prev.wide);
    tau = __ldg(&lv[l - 1].dz) * ks64 / 2. + (SHAPE ? __ldg(&lv[l - 1].cloud) * csh : __ldg(&lv[l - 1].cloud));
    if (OUT) {
      const df2 td = df_from_double(fmin(tau, 1e37)), kd = df_from_double(fmin(0.5 * ks64, 1e37));
      *tk = make_float4(td.hi, td.lo, kd.hi, kd.lo);
    }
  }
  if (tau == 0) {  // the reference skips exactly transparent layers only
    const double dB = Bp - B;
    K1 += dB * kInvMu[0];
    K2 += dB * kInvMu[1];
    return;
  }
  const double u = (B - Bp) * (1.0 / tau);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double d = tau * kInvMu[i];
    const double a = __double_as_longlong(d) > kBits700 ? 0.0 : exp_tang2048(-d, tab2048);
    double& K = i == 0 ? K1 : K2;
    K = fma(a, K, fma(a, u, -u));
  }
}

// One emission layer (between levels l-1 and l) of the two-angle short-characteristics
// recurrence, carried as K_i = (I_i - B) / mu_i, B the Planck function of the level just
// passed:
//   K_i <- a_i K_i + (a_i - 1) u,   u = (B - B') / tau,   a_i = exp(-tau / mu_i),
// which is ShortCharacteristics::calcSpectrum's update I <- I a + (1 + q) B + (-a - q) B'
// with q = (a - 1) / delta (src/radiative_transfer/short_characteristics.cpp:85-115) with B
// subtracted and divided by mu_i. tau = dz (kappa_l + kappa_{l-1}) / 2 + cloud, 1 / tau, u
// and the angles' depths tau / mu_i are double-floats, a_i comes from exp_neg_df, and
// (a_i - 1) u is one FMA (a_i u - u, rounded once; a_i == 1 leaves K_i unchanged, as the
// reference leaves I - B): nine FP64 operations per layer (u's conversion; per angle the
// conversion add and FMA of exp_neg_df and two FMAs). Other layers take emission_layer_fp64.
// SHAPE: the cloud depth is scaled by the non-grey cloud factor (csh, FP64, and its
// double-float split csd). OUT (gradient pass): tk receives tau and (k_l + k_{l-1}) / 2 as
// double-floats (FP64 values clamped to 1e37), which the adjoint sweep reads back.
template <bool SHAPE = false, bool OUT = false>
__device__ __forceinline__ void emission_layer(const LevelInfo* __restrict__ lv, int l, const Kappa& kap,
                                               const Kappa& kap_prev, const PlanckD& B, const PlanckD& Bp,
                                               double& K1, double& K2, const double* tab2048, double csh = 1.0,
                                               df2 csd = df2{1.0f, 0.0f}, float4* tk = nullptr) {
  const float4 g = __ldg(reinterpret_cast<const float4*>(&lv[l - 1].dzh_hi));  // dzh, cloud
  const df2 cl = SHAPE ? df_mul(df2{g.z, g.w}, csd) : df2{g.z, g.w};
  const df2 ks = df_add(kap.v, kap_prev.v);
  const df2 t = df_add(df_mul(df2{g.x, g.y}, ks), cl);
  // both wide parts zero (+-0), tested on the bits to stay off the FP64 pipe
  const bool narrow = ((__double_as_longlong(kap.wide) | __double_as_longlong(kap_prev.wide)) << 1) == 0 &&
                      t.hi > 1e-30f && t.hi < 1e30f;
  if (!narrow || B.tiny || Bp.tiny) {
    emission_layer_fp64<SHAPE, OUT>(lv, l, kap, kap_prev, narrow, t, ks, planck_value(B), planck_value(Bp), K1,
                                    K2, tab2048, csh, tk);
    return;
  }
  if (OUT) {
    const df2 ksh = df_mul_f(ks, 0.5f);
    *tk = make_float4(t.hi, t.lo, ksh.hi, ksh.lo);
  }
  const double u = df_to_double(df_mul(df_sub(B.v, Bp.v), df_recip(t)));
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const df2 d = df_mul(t, i == 0 ? df2{kInvMuF[0][0], kInvMuF[0][1]} : df2{kInvMuF[1][0], kInvMuF[1][1]});
    const double a = d.hi > 700.0f ? 0.0 : exp_neg_df(d, tab2048);
    double& K = i == 0 ? K1 : K2;
    K = fma(a, K, fma(a, u, -u));
  }
}

}  // namespace bgb
