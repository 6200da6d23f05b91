// GB300 kernels of the likelihood engine and their host-side launch code.
//
// Data layout in HBM
//   tables      rows x N log10 cross sections, wavenumber contiguous (one row per
//               (species, T, p) table point, sampled on the model grid), stored
//               twice: as double-floats (float2, the default path) and as FP64
//               (the validation path)
//   LevelSpecies(+DF) B x L x S, LevelInfo B x L, EvalInfo B: per-evaluation
//               atmosphere and stencils written by atmosphere_kernel
//   spectrum    B x N native units (per cm^-1 flux or ppm transit depth)
//   W           banded observation operator, one contiguous row per bin
//
// Kernels (per batch):
//   atmosphere_kernel  (atmosphere.cu)  one block per evaluation
//   emission_kernel    opacity + short-characteristics RT fused per wavenumber;
//                      the per-level opacities are never materialised
//   transmission_*     geometry per evaluation, then opacity + tangent-ray
//                      optical depths + effective height per wavenumber
//   obs_loglike_kernel banded W . F per bin with warp-shuffle reductions and the
//                      Gaussian log-likelihood reduced per evaluation
// Grids put the evaluation index on blockIdx.x and the wavenumber tile on
// blockIdx.y, so the blocks resident at any time share one wavenumber tile of
// the tables in L2.
//
// Arithmetic. This GPU issues ~67x more FP32 than FP64 operations per clock.
// The default kernels therefore assemble opacities in double-float arithmetic
// on the FP32 pipe (interpolation, 10^x via Tang's table method, accumulation;
// ~1e-12 relative) and evaluate the Planck function the same way; the
// short-characteristics recurrence and the tangent-ray sums stay FP64 with a
// table-driven FP64 exponential. The *_fp64 kernels do every step in FP64 with
// the CUDA math library and serve as the validation path (precision mode 1).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "../../include/bear_gb300.h"
#include "model.h"
#include "physics.cuh"
#include "rt_common.cuh"
#include "rt_pair.cuh"
#include "star.cuh"

namespace bgb {

__global__ void atmosphere_kernel(DeviceModel dm, const double* __restrict__ params, int P,
                                  LevelInfo* __restrict__ lev, LevelSpecies* __restrict__ ls,
                                  LevelSpeciesDF* __restrict__ lsdf, double* __restrict__ ray_n,
                                  EvalInfo* __restrict__ ev, float2* __restrict__ dwT);

// Dynamic shared memory the transmission kernels opt into (the per-block maximum of
// 227 KB less room for their static tables).
constexpr size_t kTransmissionDynSmem = 220 * 1024;

// Fused opacity assembly + short characteristics, one thread per wavenumber.
// Writes the flux in W m^-2 cm times the radius-distance scaling. With STORE the
// two Gauss-angle intensities after every level are also written to
// istore[b][l][angle][k] (the adjoint pass reads them back top-down), and, when
// layer_store is given, each layer's optical depth and half opacity sum as
// double-floats to layer_store[b][l][k] (layer l between levels l-1 and l).
//
// EXT (models with the H- continuum or a non-grey cloud): the H- continuum (rows R_ray
// .. R-1 of the linear-term table, coefficients in ray_n) has its level coefficients
// staged in dynamic shared memory as double-floats (L x kHmTerms float2) and added to
// the level absorption; a non-grey cloud scales the cloud depths by its wavelength factor.
template <bool STORE, bool EXT = false>
__global__ void __launch_bounds__(256, 6) emission_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                       const LevelSpecies* __restrict__ ls,
                                                       const LevelSpeciesDF* __restrict__ lsdf,
                                                       const double* __restrict__ ray_n,
                                                       const EvalInfo* __restrict__ ev,
                                                       double* __restrict__ spectrum, double* __restrict__ istore,
                                                       float4* __restrict__ layer_store = nullptr) {
  __shared__ ExpTables et;
  __shared__ double tab2048[2048];
  extern __shared__ float2 hm_s[];  // [L][kHmTerms] when the H- continuum is on
  load_exp_tables(et);
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) tab2048[i] = kExp2TabD2048[i];
  const bool hm = EXT && dm.R > dm.R_ray;
  if (hm)
    for (int i = threadIdx.x; i < dm.L * kHmTerms; i += blockDim.x) {
      const int l = i / kHmTerms, c = i - l * kHmTerms;
      const df2 d = df_from_double(__ldg(&ray_n[((size_t)blockIdx.x * dm.L + l) * dm.R + dm.R_ray + c]));
      hm_s[i] = make_float2(d.hi, d.lo);
    }
  __syncthreads();
  const int b = blockIdx.x;
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= dm.N) return;
  const int L = dm.L, S = dm.S;
  const size_t N = dm.N;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpeciesDF* sf = lsdf + (size_t)b * L * S;
  double* Is = STORE ? istore + (size_t)b * L * 2 * N + k : nullptr;
  const float2 c1f = __ldg(dm.planck_c1_df + k), c2f = __ldg(dm.planck_c2l_df + k);
  const df2 c1 = {c1f.x, c1f.y}, c2l = {c2f.x, c2f.y};
  auto planck = [&](int l) {
    const float2 it = __ldg(reinterpret_cast<const float2*>(&lv[l].invT_hi));
    return planck_dd(c1, c2l, df2{it.x, it.y}, et.hi, et.lo);
  };
  auto kappa = [&](int l) {
    Kappa kp = level_kappa_df(dm.ltab, N, sf + (size_t)l * S, S, k, et);
    if (hm) {
      df2 x = kp.v;
      for (int c = 0; c < kHmTerms; ++c) {
        const float2 r = __ldg(&dm.rayleigh_df[(size_t)(dm.R_ray + c) * N + k]);
        const float2 q = hm_s[l * kHmTerms + c];
        x = df_fma(df2{r.x, r.y}, df2{q.x, q.y}, x);
      }
      kp.v = x;
    }
    return kp;
  };
  const double csh = (EXT && dm.cloud_kind) ? cloud_shape(dm, ev[b], k) : 1.0;
  const df2 csd = df_from_double(csh);
  Kappa kap_prev = kappa(0);
  PlanckD B_prev = planck(0);
  double K1 = 0.0, K2 = 0.0;  // (I - B) / mu: the bottom boundary is I = B
  if (STORE) {
    const double B0 = planck_value(B_prev);
    Is[0] = B0;
    Is[N] = B0;
  }
  for (int l = 1; l < L; ++l) {
    const Kappa kap = kappa(l);
    const PlanckD B = planck(l);
    if (STORE) {
      float4 tk;
      emission_layer<EXT, true>(lv, l, kap, kap_prev, B, B_prev, K1, K2, tab2048, csh, csd, &tk);
      layer_store[((size_t)b * L + l) * N + k] = tk;
      const double Bd = planck_value(B);
      Is[(size_t)l * 2 * N] = fma(kMu[0], K1, Bd);
      Is[(size_t)l * 2 * N + N] = fma(kMu[1], K2, Bd);
    } else {
      emission_layer<EXT>(lv, l, kap, kap_prev, B, B_prev, K1, K2, tab2048, csh, csd);
    }
    kap_prev = kap;
    B_prev = B;
  }
  const double Bt = planck_value(B_prev);
  const double I1 = fma(kMu[0], K1, Bt), I2 = fma(kMu[1], K2, Bt);
  const double flux = 2.0 * kPi * (I1 * kMu[0] * 0.5 + I2 * kMu[1] * 0.5) * 1e-3;
  spectrum[(size_t)b * N + k] = flux * __ldg(&ev[b].scaling);
}

// The same fused kernel with two wavenumbers per thread, k0 = 2 x (thread index) and
// k0 + 1: the double-float opacity assembly, Planck function and layer recurrence of both
// are issued as paired FP32 instructions (rt_pair.cuh), the FP64 steps run per
// wavenumber. Each wavenumber's result is bit for bit emission_kernel<STORE>'s (with N odd,
// the last thread's second element repeats k0 and is not written). Used for batches; models
// with the H- continuum or a non-grey cloud use emission_kernel<false, true>.
// Launch bound: at most 128 threads per block and 8 resident blocks, which caps the kernel
// at 64 registers (a few bytes spill): the kernel waits mostly on level-table reads from L2,
// and 32 resident warps per SM hide them better than 24 at the 83 registers it would take
// (measured 17.9 against 19.9 ms for the 512-evaluation batch).
constexpr int kPairThreads = 128;
template <bool STORE>
__global__ void __launch_bounds__(kPairThreads, 8) emission_kernel_x2(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                          const LevelSpeciesDF* __restrict__ lsdf,
                                                          const EvalInfo* __restrict__ ev,
                                                          double* __restrict__ spectrum, double* __restrict__ istore,
                                                          float4* __restrict__ layer_store = nullptr) {
  __shared__ ExpTables et;
  __shared__ double tab2048[2048];
  load_exp_tables(et);
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) tab2048[i] = kExp2TabD2048[i];
  __syncthreads();
  const int b = blockIdx.x;
  const int k0 = 2 * (blockIdx.y * blockDim.x + threadIdx.x);
  if (k0 >= dm.N) return;
  const bool two = k0 + 1 < dm.N;
  const int k1 = two ? k0 + 1 : k0;
  const int L = dm.L, S = dm.S;
  const size_t N = dm.N;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpeciesDF* sf = lsdf + (size_t)b * L * S;
  dfx c1, c2l;
  {
    const float2 a0 = __ldg(dm.planck_c1_df + k0), a1 = __ldg(dm.planck_c1_df + k1);
    const float2 b0 = __ldg(dm.planck_c2l_df + k0), b1 = __ldg(dm.planck_c2l_df + k1);
    c1 = {make_float2(a0.x, a1.x), make_float2(a0.y, a1.y)};
    c2l = {make_float2(b0.x, b1.x), make_float2(b0.y, b1.y)};
  }
  auto inv_t = [&](int l) {
    const float2 it = __ldg(reinterpret_cast<const float2*>(&lv[l].invT_hi));
    return df2{it.x, it.y};
  };
  KappaX kap_prev = level_kappa_x(dm.ltab, N, sf, S, k0, k1, et);
  PlanckX Bp = planck_x(c1, c2l, inv_t(0), et);
  double K1[2] = {0.0, 0.0}, K2[2] = {0.0, 0.0};  // (I - B) / mu: the bottom boundary is I = B
  double* Is0 = STORE ? istore + (size_t)b * L * 2 * N + k0 : nullptr;
  double* Is1 = STORE ? istore + (size_t)b * L * 2 * N + k1 : nullptr;
  if (STORE) {
    const double B0 = planck_value(planck_get(Bp, 0)), B1 = planck_value(planck_get(Bp, 1));
    Is0[0] = B0;
    Is0[N] = B0;
    if (two) {
      Is1[0] = B1;
      Is1[N] = B1;
    }
  }
  for (int l = 1; l < L; ++l) {
    const KappaX kap = level_kappa_x(dm.ltab, N, sf + (size_t)l * S, S, k0, k1, et);
    const PlanckX B = planck_x(c1, c2l, inv_t(l), et);
    if (STORE) {
      float4 tk0, tk1;
      emission_layer_x<true>(lv, l, kap, kap_prev, B, Bp, K1, K2, tab2048, &tk0, &tk1);
      layer_store[((size_t)b * L + l) * N + k0] = tk0;
      const double B0 = planck_value(planck_get(B, 0));
      Is0[(size_t)l * 2 * N] = fma(kMu[0], K1[0], B0);
      Is0[(size_t)l * 2 * N + N] = fma(kMu[1], K2[0], B0);
      if (two) {
        layer_store[((size_t)b * L + l) * N + k1] = tk1;
        const double B1 = planck_value(planck_get(B, 1));
        Is1[(size_t)l * 2 * N] = fma(kMu[0], K1[1], B1);
        Is1[(size_t)l * 2 * N + N] = fma(kMu[1], K2[1], B1);
      }
    } else {
      emission_layer_x(lv, l, kap, kap_prev, B, Bp, K1, K2, tab2048);
    }
    kap_prev = kap;
    Bp = B;
  }
  const double scaling = __ldg(&ev[b].scaling);
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    if (e == 1 && !two) break;
    const double Bt = planck_value(planck_get(Bp, e));
    const double I1 = fma(kMu[0], K1[e], Bt), I2 = fma(kMu[1], K2[e], Bt);
    const double flux = 2.0 * kPi * (I1 * kMu[0] * 0.5 + I2 * kMu[1] * 0.5) * 1e-3;
    spectrum[(size_t)b * N + (e ? k1 : k0)] = flux * scaling;
  }
}

// Validation path: every step in FP64 with the CUDA math library.
template <bool STORE>
__global__ void __launch_bounds__(256) emission_kernel_fp64(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                            const LevelSpecies* __restrict__ ls,
                                                            const double* __restrict__ ray_n,
                                                            const EvalInfo* __restrict__ ev,
                                                            double* __restrict__ spectrum,
                                                            double* __restrict__ istore) {
  const int b = blockIdx.x;
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= dm.N) return;
  const int L = dm.L, S = dm.S;
  const size_t N = dm.N;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpecies* sp = ls + (size_t)b * L * S;
  double* Is = STORE ? istore + (size_t)b * L * 2 * N + k : nullptr;
  const double c1 = dm.planck_c1[k], c2 = dm.planck_c2[k];
  auto kappa = [&](int l) {
    double kp = level_absorption_fp64(dm.table64, N, sp + (size_t)l * S, S, k);
    const double* rn = ray_n + ((size_t)b * L + l) * dm.R;
    for (int r = dm.R_ray; r < dm.R; ++r) kp += __ldg(&dm.rayleigh[(size_t)r * N + k]) * __ldg(&rn[r]);
    return kp;
  };
  const double csh = dm.cloud_kind ? cloud_shape(dm, ev[b], k) : 1.0;
  double kap_prev = kappa(0);
  double B_prev = c1 / (exp(c2 * __ldg(&lv[0].invT)) - 1.0);
  double I1 = B_prev, I2 = B_prev;
  if (STORE) {
    Is[0] = I1;
    Is[N] = I2;
  }
  for (int l = 1; l < L; ++l) {
    const double kap = kappa(l);
    const double B = c1 / (exp(c2 * __ldg(&lv[l].invT)) - 1.0);
    const double tau = __ldg(&lv[l - 1].dz) * (kap + kap_prev) / 2. + __ldg(&lv[l - 1].cloud) * csh;
    sc_layer(tau, B, B_prev, I1, I2);
    if (STORE) {
      Is[(size_t)l * 2 * N] = I1;
      Is[(size_t)l * 2 * N + N] = I2;
    }
    kap_prev = kap;
    B_prev = B;
  }
  const double flux = 2.0 * kPi * (I1 * kMu[0] * 0.5 + I2 * kMu[1] * 0.5) * 1e-3;
  spectrum[(size_t)b * N + k] = flux * __ldg(&ev[b].scaling);
}

// ------------------------------------------------------------------ transmission
// Tangent-ray path lengths of every evaluation: geom[b][t][i] for t <= i < L-1 is
// sqrt((R+z_{i+1})^2 - (R+z_t)^2) - sqrt((R+z_i)^2 - (R+z_t)^2)
// (TransmissionModel::distanceToTangentCenter src/forward_model/transmission/
// transmission_spectrum.cpp:145-154). Squares are rounded separately so the
// tangent level gives exactly zero. Computed in FP64; stored as FP64 (precision
// mode 1) or as double-floats (DF, the default tangent sums). Also the effective-height
// weights rw_t = (R + z_t)((z_{t+1} - z_t) + (z_t - z_{t-1})), t < L-1, into
// rays[b][L + t] (the layout of the annuli geometry with one ray per level).
template <bool DF>
__global__ void transmission_geometry_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                             const EvalInfo* __restrict__ ev, double* __restrict__ geom,
                                             double* __restrict__ rays) {
  const int b = blockIdx.x;
  const int L = dm.L;
  const LevelInfo* lv = lev + (size_t)b * L;
  const double R = ev[b].radius;
  if (blockIdx.y == 0)
    for (int t = threadIdx.x; t < L - 1; t += blockDim.x) {
      const double zt = lv[t].z;
      rays[(size_t)b * 2 * L + L + t] = (R + zt) * ((lv[t + 1].z - zt) + (t >= 1 ? zt - lv[t - 1].z : 0.0));
    }
  // grid: evaluations x blocks of elements
  for (int idx = blockIdx.y * blockDim.x + threadIdx.x; idx < L * L; idx += gridDim.y * blockDim.x) {
    const int t = idx / L, i = idx % L;
    double v = 0.0;
    if (i >= t && i < L - 1) {
      const double bt = R + lv[t].z;
      const double a1 = R + lv[i + 1].z;
      const double a0 = R + lv[i].z;
      const double bb = __dmul_rn(bt, bt);
      v = sqrt(__dsub_rn(__dmul_rn(a1, a1), bb)) - sqrt(__dsub_rn(__dmul_rn(a0, a0), bb));
    }
    if (DF) {
      const df2 d = df_from_double(v);
      reinterpret_cast<float2*>(geom)[(size_t)b * L * L + idx] = make_float2(d.hi, d.lo);
    } else {
      geom[(size_t)b * L * L + idx] = v;
    }
  }
}

// Transit depth (TransmissionModel::calcTransmissionSpectrum ... tangentOpticalDepth
// src/forward_model/transmission/transmission_spectrum.cpp:32-141). A block covers
// VPB wavenumbers with TPN = 4 threads each (lane = wavenumber, so table reads stay
// coalesced; VPB is the tuned launch shape and does not change any sum's order).
// The TPN threads of a wavenumber split the levels' opacities, then share the
// staged extinction column chi[L][VPB] and split the tangent levels. With DF the
// extinction column and the tangent optical depths are double-floats on the FP32
// pipe (the reference's tau > 10 cut-off tested on the double-float value), and so are
// exp(-tau) and 1 - T (relative error ~1e-14); the effective-height (annulus) sum is
// FP64 in both modes. The effective height is summed per level,
// sum_t rw_t (1 - T_t), rw_t = (R + z_t)(dz_{t-1} + dz_t) (from the geometry
// kernel), which regroups the reference's
// trapezoid sum. Dynamic shared memory: chi [L][VPB] (8 B each), then with DF the
// evaluation's Rayleigh number densities [L][R] as double-floats.
// With STORE (double-float path, gradient pass) the kernel also writes, per
// (evaluation, level, wavenumber), the pair sums c, the ray transmissions T_t, the
// last index inside the cut-off and the sum of c_i dG[t][i]/dz_t over each ray (taps.tr_*;
// dG/dz_t from taps.tr_geo, computed before this kernel).
constexpr int kTPN = 4;
// The effective-height sum sum_t rw_t (1 - T_t) is formed as kHeightGroups partial sums,
// group g holding the rays t = L - 2 - g - kHeightGroups m in descending order, added in
// group order; every transmission kernel with one tangent level per ray keeps this order,
// whatever its threads per wavenumber (4: two groups per thread; 8: one), so all of them
// give the same bits.
constexpr int kHeightGroups = 8;

__global__ void tr_geometry_adjoint_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                           const EvalInfo* __restrict__ ev, const float2* __restrict__ geom,
                                           float2* __restrict__ geo);
__global__ void tr_geometry_adjoint_annuli_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                  const EvalInfo* __restrict__ ev, const float2* __restrict__ geom,
                                                  const double* __restrict__ rays, float2* __restrict__ geo);

// Extinction abs + scat + cloud of every level of wavenumber k into the staged column
// chi[l][VPB] (double-floats with DF, FP64 otherwise); thread j of the wavenumber's TPN
// takes every TPN-th level. rn_s: the Rayleigh / continuum coefficients as double-floats (DF).
template <bool DF, int VPB, int TPN = kTPN>
__device__ __forceinline__ void tr_extinction(const DeviceModel& dm, const LevelInfo* __restrict__ lv,
                                              const LevelSpecies* __restrict__ sp,
                                              const LevelSpeciesDF* __restrict__ sf,
                                              const double* __restrict__ ray_n, int b, int k, int v, int j,
                                              const ExpTables& et, const float2* rn_s, double csh,
                                              double* chi_s) {
  float2* chi_f = reinterpret_cast<float2*>(chi_s);
  const int L = dm.L, S = dm.S, R = dm.R;
  const size_t N = dm.N;
  for (int l = j; l < L; l += TPN) {
    if (DF) {
      const Kappa kp = level_kappa_df<4>(dm.ltab, N, sf + (size_t)l * S, S, k, et);
      df2 x = kp.v;
      if ((__double_as_longlong(kp.wide) << 1) != 0) x = df_add(x, df_from_double(kp.wide));
      for (int r = 0; r < R; ++r) {
        const float2 sr = __ldg(&dm.rayleigh_df[(size_t)r * N + k]);
        const float2 nr = rn_s[l * R + r];
        x = df_fma(df2{sr.x, sr.y}, df2{nr.x, nr.y}, x);
      }
      const float2 cl = __ldg(reinterpret_cast<const float2*>(&lv[l].cloud_hi));
      x = dm.cloud_kind ? df_fma(df2{cl.x, cl.y}, df_from_double(csh), x) : df_add(x, df2{cl.x, cl.y});
      chi_f[l * VPB + v] = make_float2(x.hi, x.lo);
    } else {
      const double a = level_absorption_fp64(dm.table64, N, sp + (size_t)l * S, S, k);
      double sc = 0.0;
      for (int r = 0; r < R; ++r)
        sc += __ldg(&dm.rayleigh[(size_t)r * N + k]) * __ldg(&ray_n[((size_t)b * L + l) * R + r]);
      chi_s[l * VPB + v] = a + sc + __ldg(&lv[l].cloud) * csh;
    }
  }
}

// The same double-float extinction for the gradient's forward pass when it stores the
// opacity terms: each table species' term into taps.tr_ts and the temperature-slope sum
// sum_s term_s (hi_s - lo_s) d wT_s / dT into taps.tr_dk (NaN where a term lies outside
// the float range), in the order the transmission adjoint would recompute them.
template <int VPB>
__device__ __forceinline__ void tr_extinction_terms(const DeviceModel& dm, const LevelInfo* __restrict__ lv,
                                                    const LevelSpeciesDF* __restrict__ sf, int b, int k, int v,
                                                    int j, const ExpTables& et, const float2* rn_s, double csh,
                                                    double* chi_s, const ForwardTaps& taps) {
  float2* chi_f = reinterpret_cast<float2*>(chi_s);
  const int L = dm.L, S = dm.S, R = dm.R;
  const size_t N = dm.N;
  for (int l = j; l < L; l += kTPN) {
    const float2* dwl = taps.dwT + ((size_t)b * L + l) * S;
    float2* tso = taps.tr_ts + ((size_t)b * L + l) * S * N + k;
    df2 dk = {0.0f, 0.0f};
    bool wide = false;
    const Kappa kp = level_kappa_df_cb<4>(dm.ltab, N, sf + (size_t)l * S, S, k, et,
                                          [&](int s, df2 t, double, bool is_wide, df2 lo, df2 hi) {
                                            tso[(size_t)s * N] = make_float2(t.hi, t.lo);
                                            const float2 d = __ldg(dwl + s);
                                            if (d.x != 0.0f && !is_wide)
                                              dk = df_add(dk, df_mul(t, df_mul(df_sub(hi, lo), df2{d.x, d.y})));
                                            wide = wide || is_wide;
                                          });
    taps.tr_dk[((size_t)b * L + l) * N + k] = wide ? make_float2(__int_as_float(0x7fc00000), 0.0f)
                                                   : make_float2(dk.hi, dk.lo);
    df2 x = kp.v;
    if ((__double_as_longlong(kp.wide) << 1) != 0) x = df_add(x, df_from_double(kp.wide));
    for (int r = 0; r < R; ++r) {
      const float2 sr = __ldg(&dm.rayleigh_df[(size_t)r * N + k]);
      const float2 nr = rn_s[l * R + r];
      x = df_fma(df2{sr.x, sr.y}, df2{nr.x, nr.y}, x);
    }
    const float2 cl = __ldg(reinterpret_cast<const float2*>(&lv[l].cloud_hi));
    x = dm.cloud_kind ? df_fma(df2{cl.x, cl.y}, df_from_double(csh), x) : df_add(x, df2{cl.x, cl.y});
    chi_f[l * VPB + v] = make_float2(x.hi, x.lo);
  }
}

template <bool DF, int VPB, bool STORE = false>
__global__ void __launch_bounds__(kTPN * VPB) transmission_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                           const LevelSpecies* __restrict__ ls,
                                                           const LevelSpeciesDF* __restrict__ lsdf,
                                                           const double* __restrict__ ray_n,
                                                           const EvalInfo* __restrict__ ev,
                                                           const double* __restrict__ geom,
                                                           const double* __restrict__ rays,
                                                           double* __restrict__ spectrum, ForwardTaps taps) {
  constexpr int TPN = kTPN;
  extern __shared__ double chi_s[];  // [L][VPB]
  float2* chi_f = reinterpret_cast<float2*>(chi_s);
  __shared__ ExpTables et;
  const int v = threadIdx.x % VPB, j = threadIdx.x / VPB;
  const int b = blockIdx.x;
  const int k = blockIdx.y * VPB + v;
  const int L = dm.L, S = dm.S, R = dm.R;
  const size_t N = dm.N;
  const bool active = k < dm.N;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpecies* sp = ls + (size_t)b * L * S;
  const LevelSpeciesDF* sf = lsdf + (size_t)b * L * S;
  float2* rn_s = chi_f + (size_t)L * VPB;  // [L][R] (DF only)
  // non-grey cloud: the extinction of every level scaled by the wavelength factor
  const double csh = (dm.cloud_kind && active) ? cloud_shape(dm, ev[b], k) : 1.0;
  if (DF) {
    load_exp_tables(et);
    for (int idx = threadIdx.x; idx < L * R; idx += blockDim.x) {
      const df2 d = df_from_double(__ldg(&ray_n[(size_t)b * L * R + idx]));
      rn_s[idx] = make_float2(d.hi, d.lo);
    }
  }
  __syncthreads();
  // extinction abs + scat + cloud of every level (the TPN threads take every TPN-th level)
  if (active) {
    if (STORE && DF && taps.tr_ts) tr_extinction_terms<VPB>(dm, lv, sf, b, k, v, j, et, rn_s, csh, chi_s, taps);
    else tr_extinction<DF, VPB>(dm, lv, sp, sf, ray_n, b, k, v, j, et, rn_s, csh, chi_s);
  }
  __syncthreads();
  // neighbour sums chi_i + chi_{i+1}, the bracket of every trapezoid term
  if (active && j == 0) {
    for (int i = 0; i < L - 1; ++i) {
      if (DF) {
        const float2 c0 = chi_f[i * VPB + v], c1 = chi_f[(i + 1) * VPB + v];
        const df2 s2 = df_add(df2{c0.x, c0.y}, df2{c1.x, c1.y});
        chi_f[i * VPB + v] = make_float2(s2.hi, s2.lo);
      } else {
        chi_s[i * VPB + v] += chi_s[(i + 1) * VPB + v];
      }
    }
  }
  __syncthreads();
  double h = 0.0, h_other = 0.0;  // height groups j and j + TPN
  const double Rp = ev[b].radius;
  const double* rw = rays + (size_t)b * 2 * L + L;  // effective-height weights
  const size_t col = (size_t)b * L * N + k;  // [b][level][k] of level 0 (gradient pass stores)
  if (STORE && active)
    for (int i = j; i < L - 1; i += TPN) taps.tr_c[col + (size_t)i * N] = chi_f[i * VPB + v];
  if (active) {
    for (int t = L - 2 - j; t >= 0; t -= TPN) {
      double tau = 0.0;
      df2 tsd = {0.0f, 0.0f};  // the tangent sum as a double-float (DF)
      df2 qs = {0.0f, 0.0f};
      int last = L - 2;
      if (DF && STORE) {
        const float2* Gt = reinterpret_cast<const float2*>(geom) + (size_t)b * L * L + (size_t)t * L;
        const float2* Qt = taps.tr_geo + (size_t)b * 3 * L * L + (size_t)L * L + (size_t)t * L;
        const float ch = dm.tau_cut_hi, cl = dm.tau_cut_lo;
        df2 ts = {0.0f, 0.0f};
        bool cut = false;
        // one segment of the two ray sums; true at the cut-off (tau > cut-off)
        auto seg = [&](float2 g, float2 c, float2 q) {
          const df2 cc = {c.x, c.y};
          ts = df_fma(df2{g.x, g.y}, cc, ts);
          qs = df_fma(df2{q.x, q.y}, cc, qs);
          return ts.hi > ch || (ts.hi == ch && ts.lo > cl);
        };
        int i = t;
        // two segments per step with their loads issued together (same sums, same break)
        for (; i + 1 < L - 1 && !cut; i += 2) {
          const float2 g0 = __ldg(&Gt[i]), g1 = __ldg(&Gt[i + 1]);
          const float2 q0 = __ldg(&Qt[i]), q1 = __ldg(&Qt[i + 1]);
          const float2 c0 = chi_f[i * VPB + v], c1 = chi_f[(i + 1) * VPB + v];
          if (seg(g0, c0, q0)) {
            last = i;
            cut = true;
          } else if (seg(g1, c1, q1)) {
            last = i + 1;
            cut = true;
          }
        }
        if (i < L - 1 && !cut && seg(__ldg(&Gt[i]), chi_f[i * VPB + v], __ldg(&Qt[i]))) last = i;
        tsd = ts;
      } else if (DF) {
        const float2* Gt = reinterpret_cast<const float2*>(geom) + (size_t)b * L * L + (size_t)t * L;
        df2 ts = {0.0f, 0.0f};
        const float ch = dm.tau_cut_hi, cl = dm.tau_cut_lo;
        auto over = [ch, cl](df2 x) { return x.hi > ch || (x.hi == ch && x.lo > cl); };  // tau > cut-off
        int i = t;
        bool cut = false;
        // four terms per iteration with their loads issued together (same sum, same break)
        for (; i + 3 < L - 1 && !cut; i += 4) {
          float2 g[4], c[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            g[u] = __ldg(&Gt[i + u]);
            c[u] = chi_f[(i + u) * VPB + v];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            ts = df_fma(df2{g[u].x, g[u].y}, df2{c[u].x, c[u].y}, ts);
            if (over(ts)) {
              cut = true;
              break;
            }
          }
        }
        for (; i < L - 1 && !cut; ++i) {
          const float2 g = __ldg(&Gt[i]);
          const float2 c = chi_f[i * VPB + v];
          ts = df_fma(df2{g.x, g.y}, df2{c.x, c.y}, ts);
          cut = over(ts);
        }
        tsd = ts;
      } else {
        const double* Gt = geom + (size_t)b * L * L + (size_t)t * L;
        tau = 0.0;
        for (int i = t; i < L - 1; ++i) {
          tau = fma(__ldg(&Gt[i]), chi_s[i * VPB + v], tau);
          if (__double_as_longlong(tau) > dm.tau_cut_bits) break;  // tau > cut-off (tau >= 0)
        }
      }
      // 1 - T: with DF, T = exp(-tau) and 1 - T in double-float (relative error ~1e-14),
      // so the ray costs one conversion add and one FMA on the FP64 pipe
      double omt;
      if (DF) {
        const df2 T = df_exp_neg(tsd, et.hi, et.lo);
        if (STORE) {
          const size_t at = col + (size_t)t * N;
          taps.tr_T[at] = make_float2(T.hi, T.lo);
          taps.tr_qs[at] = make_float2(qs.hi, qs.lo);
          taps.tr_I[at] = (short)last;
        }
        omt = df_to_double(df_sub(df_make(1.0f), T));
      } else {
        omt = 1. - exp(-tau);
      }
      h = fma(__ldg(&rw[t]), omt, h);
      // the next ray (t - TPN) belongs to the other height group of this thread
      const double x = h;
      h = h_other;
      h_other = x;
    }
  }
  // after an even number of rays h holds group j again, after an odd number group j + TPN;
  // the group sums [kHeightGroups][VPB] take the place of the extinction column
  const bool odd = j <= L - 2 && (((L - 2 - j) / TPN) & 1) == 0;
  double* h_part = chi_s;
  __syncthreads();
  h_part[j * VPB + v] = odd ? h_other : h;
  h_part[(j + TPN) * VPB + v] = odd ? h : h_other;
  __syncthreads();
  if (active && j == 0) {
    double hs = 0.0;
#pragma unroll
    for (int q = 0; q < kHeightGroups; ++q) hs += h_part[q * VPB + v];
    hs = sqrt(hs + Rp * Rp) - Rp;
    const double rp = hs + Rp;
    const double Rs = ev[b].star_radius;
    spectrum[(size_t)b * N + k] = rp * rp / Rs / Rs * 1e6;
  }
}

// transmission_kernel's double-float forward path with two wavenumbers per thread group:
// a block covers VP pairs (k, k + VP), 2 VP wavenumbers, with TPN threads per pair (4 or 8).
// Every double-float step is that kernel's step issued once for both wavenumbers with
// paired FP32 instructions (dfloat2x.cuh), and the effective-height sums run in the same
// groups and order (kHeightGroups), so each transit depth is bit for bit
// transmission_kernel's. A tangent sum runs paired until either wavenumber passes the
// cut-off; the other one finishes alone. The level-table reads of GRP species are issued
// together. Dynamic shared memory: the extinction column chi[L][VP] as paired
// double-floats (hi0, hi1, lo0, lo1), then the evaluation's Rayleigh number densities [L][R]
// as double-floats; after the tangent sums the kHeightGroups partial sums take its place.
// Measured on 64 evaluations of 100 levels x 33976 points (10 tables, 2 Rayleigh species):
// <16, 8, 8, 2> (63 registers, 7 blocks = 28 warps per SM) 14.76 ms, against 16.28 ms for
// transmission_kernel at 64 wavenumbers per block; 4 threads per pair (16 warps per SM) took
// 19.8 ms, and issuing the next species' table reads ahead of the current arithmetic
// 15.5-16.9 ms. About two thirds of the time is the extinction column.
// With STORE (the gradient's forward pass) it also writes transmission_kernel<STORE>'s
// stores: the opacity terms and temperature-slope sums, the pair sums c, and per ray T_t,
// the cut-off index and the ray sum of c dG/dz_t.
template <int VP, int TPN, int MINB, int GRP, bool STORE = false>
__global__ void __launch_bounds__(TPN * VP, MINB) transmission_kernel_x2(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                                  const LevelSpeciesDF* __restrict__ lsdf,
                                                                  const double* __restrict__ ray_n,
                                                                  const EvalInfo* __restrict__ ev,
                                                                  const double* __restrict__ geom,
                                                                  const double* __restrict__ rays,
                                                                  double* __restrict__ spectrum, ForwardTaps taps) {
  static_assert(TPN == 4 || TPN == 8, "4 or 8 threads per pair");
  constexpr int NG = kHeightGroups / TPN;  // height groups per thread
  extern __shared__ float4 chi_x[];  // [L][VP]
  __shared__ ExpTables et;
  const int v = threadIdx.x % VP, j = threadIdx.x / VP;
  const int b = blockIdx.x;
  const int ka = blockIdx.y * 2 * VP + v, kb = ka + VP;
  const int L = dm.L, S = dm.S, R = dm.R;
  const size_t N = dm.N;
  const bool act0 = ka < dm.N, act1 = kb < dm.N;  // act1 implies act0
  const int k0 = act0 ? ka : dm.N - 1, k1 = act1 ? kb : dm.N - 1;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpeciesDF* sf = lsdf + (size_t)b * L * S;
  float2* rn_s = reinterpret_cast<float2*>(chi_x + (size_t)L * VP);  // [L][R]
  // non-grey cloud: the extinction of every level scaled by the wavelength factor
  double csh0 = 1.0, csh1 = 1.0;
  if (dm.cloud_kind && act0) {
    csh0 = cloud_shape(dm, ev[b], k0);
    csh1 = cloud_shape(dm, ev[b], k1);
  }
  load_exp_tables(et);
  for (int idx = threadIdx.x; idx < L * R; idx += blockDim.x) {
    const df2 d = df_from_double(__ldg(&ray_n[(size_t)b * L * R + idx]));
    rn_s[idx] = make_float2(d.hi, d.lo);
  }
  __syncthreads();
  // extinction abs + scat + cloud of every level (the TPN threads take every TPN-th level)
  if (act0) {
    const dfx zero = {f2(0.0f), f2(0.0f)};
    for (int l = j; l < L; l += TPN) {
      KappaX kp;
      if (STORE && taps.tr_ts) {
        // each species' term and the temperature-slope sum sum_s term_s (hi_s - lo_s) dwT_s/dT
        // (tr_extinction_terms per element)
        const float2* dwl = taps.dwT + ((size_t)b * L + l) * S;
        float2* tso = taps.tr_ts + ((size_t)b * L + l) * S * N;
        dfx dk = zero;
        bool wide0 = false, wide1 = false;
        kp = level_kappa_x_cb<GRP>(dm.ltab, N, sf + (size_t)l * S, S, k0, k1, et,
                                   [&](int s, const dfx& t, bool w0, bool w1, const dfx& lo, const dfx& hi) {
                                     tso[(size_t)s * N + k0] = make_float2(t.hi.x, t.lo.x);
                                     if (act1) tso[(size_t)s * N + k1] = make_float2(t.hi.y, t.lo.y);
                                     const float2 d = __ldg(dwl + s);
                                     if (d.x != 0.0f) {
                                       if (!w0 && !w1) {
                                         dk = dfx_add(dk, dfx_mul(t, dfx_mul(dfx_sub(hi, lo), dfx_bcast(df2{d.x, d.y}))));
                                       } else {
#pragma unroll
                                         for (int e = 0; e < 2; ++e) {
                                           if (e ? w1 : w0) continue;
                                           dfx_set(dk, e, df_add(dfx_get(dk, e),
                                                                 df_mul(dfx_get(t, e),
                                                                        df_mul(df_sub(dfx_get(hi, e), dfx_get(lo, e)),
                                                                               df2{d.x, d.y}))));
                                         }
                                       }
                                     }
                                     wide0 = wide0 || w0;
                                     wide1 = wide1 || w1;
                                   });
        const float2 nan2 = make_float2(__int_as_float(0x7fc00000), 0.0f);
        float2* dko = taps.tr_dk + ((size_t)b * L + l) * N;
        dko[k0] = wide0 ? nan2 : make_float2(dk.hi.x, dk.lo.x);
        if (act1) dko[k1] = wide1 ? nan2 : make_float2(dk.hi.y, dk.lo.y);
      } else {
        kp = level_kappa_x<GRP>(dm.ltab, N, sf + (size_t)l * S, S, k0, k1, et);
      }
      dfx x = kp.v;
      if ((__double_as_longlong(kp.wide0) << 1) != 0) dfx_set(x, 0, df_add(dfx_get(x, 0), df_from_double(kp.wide0)));
      if ((__double_as_longlong(kp.wide1) << 1) != 0) dfx_set(x, 1, df_add(dfx_get(x, 1), df_from_double(kp.wide1)));
      for (int r = 0; r < R; ++r) {
        const float2 s0 = __ldg(&dm.rayleigh_df[(size_t)r * N + k0]), s1 = __ldg(&dm.rayleigh_df[(size_t)r * N + k1]);
        const float2 nr = rn_s[l * R + r];
        x = dfx_fma(dfx{make_float2(s0.x, s1.x), make_float2(s0.y, s1.y)}, dfx_bcast(df2{nr.x, nr.y}), x);
      }
      const float2 cl = __ldg(reinterpret_cast<const float2*>(&lv[l].cloud_hi));
      x = dm.cloud_kind ? dfx_fma(dfx_bcast(df2{cl.x, cl.y}), dfx_make(df_from_double(csh0), df_from_double(csh1)), x)
                        : dfx_add(x, dfx_bcast(df2{cl.x, cl.y}));
      chi_x[l * VP + v] = make_float4(x.hi.x, x.hi.y, x.lo.x, x.lo.y);
    }
  }
  // neighbour sums chi_i + chi_{i+1}, the bracket of every trapezoid term: thread j takes a
  // run of levels and reads the value after its run before any thread writes
  const int run = (L - 1 + TPN - 1) / TPN;
  const int i0 = j * run, i1 = min(i0 + run, L - 1);
  __syncthreads();
  float4 after = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (act0 && i0 < i1) after = chi_x[i1 * VP + v];
  __syncthreads();
  if (act0 && i0 < i1) {
    float4 cur = chi_x[i0 * VP + v];
    for (int i = i0; i < i1; ++i) {
      const float4 nx = i + 1 < i1 ? chi_x[(i + 1) * VP + v] : after;
      const dfx s2 = dfx_add(dfx{make_float2(cur.x, cur.y), make_float2(cur.z, cur.w)},
                             dfx{make_float2(nx.x, nx.y), make_float2(nx.z, nx.w)});
      chi_x[i * VP + v] = make_float4(s2.hi.x, s2.hi.y, s2.lo.x, s2.lo.y);
      if (STORE) {
        taps.tr_c[((size_t)b * L + i) * N + k0] = make_float2(s2.hi.x, s2.lo.x);
        if (act1) taps.tr_c[((size_t)b * L + i) * N + k1] = make_float2(s2.hi.y, s2.lo.y);
      }
      cur = nx;
    }
  }
  __syncthreads();
  double h0 = 0.0, h1 = 0.0, h0o = 0.0, h1o = 0.0;  // groups j (and j + TPN when NG = 2)
  const double* rw = rays + (size_t)b * 2 * L + L;  // effective-height weights
  if (act0) {
    const float ch = dm.tau_cut_hi, cl = dm.tau_cut_lo;
    for (int t = L - 2 - j; t >= 0; t -= TPN) {
      const float2* Gt = reinterpret_cast<const float2*>(geom) + (size_t)b * L * L + (size_t)t * L;
      // STORE: the ray sum of c dG/dz_t (Q) beside the optical depth
      const float2* Qt = STORE ? taps.tr_geo + (size_t)b * 3 * L * L + (size_t)L * L + (size_t)t * L : nullptr;
      dfx ts = {f2(0.0f), f2(0.0f)}, qs = ts;
      bool cut0 = false, cut1 = false;
      int last0 = L - 2, last1 = L - 2;  // the last index inside the cut-off
      int i = t;
      for (; i < L - 1; ++i) {
        const float2 g = __ldg(&Gt[i]);
        const float4 c = chi_x[i * VP + v];
        const dfx cc = {make_float2(c.x, c.y), make_float2(c.z, c.w)};
        ts = dfx_fma(dfx_bcast(df2{g.x, g.y}), cc, ts);
        if (STORE) {
          const float2 q = __ldg(&Qt[i]);
          qs = dfx_fma(dfx_bcast(df2{q.x, q.y}), cc, qs);
        }
        if (ts.hi.x >= ch || ts.hi.y >= ch) {  // tau > cut-off needs hi >= the cut-off's hi
          cut0 = ts.hi.x > ch || (ts.hi.x == ch && ts.lo.x > cl);
          cut1 = ts.hi.y > ch || (ts.hi.y == ch && ts.lo.y > cl);
          if (cut0 || cut1) {
            if (cut0) last0 = i;
            if (cut1) last1 = i;
            ++i;
            break;
          }
        }
      }
      if (cut0 != cut1) {
        // one wavenumber is past the cut-off: the other one's remaining terms alone
        const int e = cut0 ? 1 : 0;
        df2 te = dfx_get(ts, e), qe = dfx_get(qs, e);
        for (; i < L - 1; ++i) {
          const float2 g = __ldg(&Gt[i]);
          const float4 c = chi_x[i * VP + v];
          const df2 ce = e ? df2{c.y, c.w} : df2{c.x, c.z};
          te = df_fma(df2{g.x, g.y}, ce, te);
          if (STORE) {
            const float2 q = __ldg(&Qt[i]);
            qe = df_fma(df2{q.x, q.y}, ce, qe);
          }
          if (te.hi > ch || (te.hi == ch && te.lo > cl)) {
            (e ? last1 : last0) = i;
            break;
          }
        }
        dfx_set(ts, e, te);
        dfx_set(qs, e, qe);
      }
      const dfx T = dfx_exp_neg(ts, et.hi, et.lo);
      if (STORE) {
        const size_t at = ((size_t)b * L + t) * N;
        taps.tr_T[at + k0] = make_float2(T.hi.x, T.lo.x);
        taps.tr_qs[at + k0] = make_float2(qs.hi.x, qs.lo.x);
        taps.tr_I[at + k0] = (short)last0;
        if (act1) {
          taps.tr_T[at + k1] = make_float2(T.hi.y, T.lo.y);
          taps.tr_qs[at + k1] = make_float2(qs.hi.y, qs.lo.y);
          taps.tr_I[at + k1] = (short)last1;
        }
      }
      // 1 - T with T = exp(-tau) in double-float
      const dfx omt = dfx_sub(dfx_bcast(df_make(1.0f)), T);
      const double w = __ldg(&rw[t]);
      h0 = fma(w, df_to_double(dfx_get(omt, 0)), h0);
      h1 = fma(w, df_to_double(dfx_get(omt, 1)), h1);
      if (NG == 2) {  // the next ray belongs to the thread's other group
        double x = h0;
        h0 = h0o;
        h0o = x;
        x = h1;
        h1 = h1o;
        h1o = x;
      }
    }
  }
  // the group sums [kHeightGroups][2][VP] take the place of the extinction column
  double* h_part = reinterpret_cast<double*>(chi_x);
  __syncthreads();
  if (NG == 2) {
    // after an odd number of rays the other group's sums are current
    const bool odd = j <= L - 2 && (((L - 2 - j) / TPN) & 1) == 0;
    h_part[(2 * j) * VP + v] = odd ? h0o : h0;
    h_part[(2 * j + 1) * VP + v] = odd ? h1o : h1;
    h_part[(2 * (j + TPN)) * VP + v] = odd ? h0 : h0o;
    h_part[(2 * (j + TPN) + 1) * VP + v] = odd ? h1 : h1o;
  } else {
    h_part[(2 * j) * VP + v] = h0;
    h_part[(2 * j + 1) * VP + v] = h1;
  }
  __syncthreads();
  if (j == 0) {
    const double Rp = ev[b].radius, Rs = ev[b].star_radius;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      if (!(e ? act1 : act0)) continue;
      double hs = 0.0;
#pragma unroll
      for (int q = 0; q < kHeightGroups; ++q) hs += h_part[(2 * q + e) * VP + v];
      hs = sqrt(hs + Rp * Rp) - Rp;
      const double rp = hs + Rp;
      spectrum[(size_t)b * N + (e ? k1 : k0)] = rp * rp / Rs / Rs * 1e6;
    }
  }
}

// ------------------------------------------------------------------ transmission with annuli
// Transit depth with A = dm.annuli impact parameters per layer (not in the reference, whose
// rays touch the levels only; A = 1 is that formula and uses transmission_kernel): in layer t
// the rays' altitudes are zb = z_t + (z_{t+1} - z_t) j / A, j = 0..A-1, plus the top level. A
// ray's first, partial segment (from its tangent point to level t+1) takes the extinction
// interpolated linearly in altitude, chi_t + (chi_{t+1} - chi_t) j / A; the other segments,
// the tau > cut-off rule and the effective-height trapezoid (over the finer grid of impact
// parameters) are those of transmission_kernel. The double-float path forms exp(-tau) and
// 1 - T in double-float (relative error ~1e-14) and adds rw_k (1 - T_k) into h in FP64, so
// a ray costs one FP64 FMA and one conversion add on the FP64 pipe.
//
// Geometry per evaluation: geom[b][t][i][j], the path length through level pair (i, i+1)
// of ray k = t A + j of layer t (i == t: the partial segment; the A rays of a layer are
// contiguous for each i), and rays[b] = {zb[K+1], rw[K+1]}, K = (L-1) A: the altitudes
// and rw_k = (R + zb_k) ((zb_{k+1} - zb_k) + (zb_k - zb_{k-1})), so that the effective
// height is h = sum_k rw_k (1 - T_k).
template <bool DF>
__global__ void transmission_annuli_geometry_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                    const EvalInfo* __restrict__ ev, double* __restrict__ geom,
                                                    double* __restrict__ rays) {
  // one thread per ray kr (grid: evaluations x ray blocks); kr == K is the top level
  const int b = blockIdx.x;
  const int L = dm.L, A = dm.annuli, K = (L - 1) * A;
  const int kr = blockIdx.y * blockDim.x + threadIdx.x;
  if (kr > K) return;
  const LevelInfo* lv = lev + (size_t)b * L;
  const double R = ev[b].radius;
  auto zb_of = [&](int q) {
    if (q >= K) return lv[L - 1].z;
    const int t = q / A, jj = q - t * A;
    const double z0 = lv[t].z, z1 = lv[t + 1].z;
    return __dadd_rn(z0, __ddiv_rn(__dmul_rn(__dsub_rn(z1, z0), (double)jj), (double)A));
  };
  const double z = zb_of(kr);
  const double wz = (kr < K ? zb_of(kr + 1) - z : 0.0) + (kr >= 1 ? z - zb_of(kr - 1) : 0.0);
  double* zb = rays + (size_t)b * 2 * (K + 1);
  zb[kr] = z;
  zb[K + 1 + kr] = (R + z) * wz;
  if (kr == K) return;
  // path lengths through level pairs (i, i+1), i = t..L-2: s_{i+1} - s_i with
  // s_i = sqrt((R + z_i)^2 - b^2), each root taken once; the partial segment is s_{t+1}
  const int t = kr / A, jj = kr - t * A;
  const double bt = R + z;
  const double bb = __dmul_rn(bt, bt);
  double s_prev = 0.0;
  for (int i = t; i < L - 1; ++i) {
    const double a1 = R + lv[i + 1].z;
    const double s_next = sqrt(__dsub_rn(__dmul_rn(a1, a1), bb));
    const double v = s_next - s_prev;
    s_prev = s_next;
    const size_t at = (((size_t)b * (L - 1) + t) * L + i) * A + jj;  // [b][t][i][j]
    if (DF) {
      const df2 d = df_from_double(v);
      reinterpret_cast<float2*>(geom)[at] = make_float2(d.hi, d.lo);
    } else {
      geom[at] = v;
    }
  }
}

// Dynamic shared memory: the extinction pair sums [L][VPB], their differences
// chi_{i+1} - chi_i [L][VPB] (double-floats with DF, FP64 otherwise), then (DF) the
// Rayleigh / continuum coefficients [L][R].
constexpr int kMaxAnnuli = 64;  // transmission_annuli upper bound

// dynamic shared memory of transmission_annuli_kernel (32 wavenumbers per block)
inline size_t annuli_dyn_smem(int L, int R, bool df) {
  return 2 * (size_t)L * 32 * sizeof(double) + (df ? (size_t)L * R * sizeof(float2) : 0);
}

// With STORE (double-float path, the gradient's forward pass) the kernel also writes, per
// (evaluation, level, wavenumber), the pair sums c_i and differences d_i = chi_{i+1} - chi_i,
// and per (evaluation, ray, wavenumber) the ray transmission, the last segment inside the
// cut-off and the ray sum of the extinction times dG/db (b = R + zb the impact radius; dG/db
// from taps.tr_geo, computed before this kernel).
template <bool DF, int VPB, int TPN, int RG, bool STORE = false>
__global__ void __launch_bounds__(TPN * VPB, 4) transmission_annuli_kernel(
    DeviceModel dm, const LevelInfo* __restrict__ lev, const LevelSpecies* __restrict__ ls,
    const LevelSpeciesDF* __restrict__ lsdf, const double* __restrict__ ray_n, const EvalInfo* __restrict__ ev,
    const double* __restrict__ geom, const double* __restrict__ rays, double* __restrict__ spectrum,
    ForwardTaps taps) {
  extern __shared__ double chi_s[];
  const int L = dm.L, S = dm.S, R = dm.R, A = dm.annuli, K = (L - 1) * A;
  float2* chi_f = reinterpret_cast<float2*>(chi_s);
  double* dif_s = chi_s + (size_t)L * VPB;
  float2* dif_f = reinterpret_cast<float2*>(dif_s);
  float2* rn_s = reinterpret_cast<float2*>(dif_s + (size_t)L * VPB);
  __shared__ ExpTables et;
  __shared__ double h_part[TPN][VPB];
  __shared__ float2 wj_s[kMaxAnnuli];  // j / A as double-floats
  const int v = threadIdx.x % VPB, j = threadIdx.x / VPB;
  const int b = blockIdx.x;
  const int k = blockIdx.y * VPB + v;
  const size_t N = dm.N;
  const bool active = k < dm.N;
  const LevelInfo* lv = lev + (size_t)b * L;
  const LevelSpecies* sp = ls + (size_t)b * L * S;
  const LevelSpeciesDF* sf = lsdf + (size_t)b * L * S;
  const double csh = (dm.cloud_kind && active) ? cloud_shape(dm, ev[b], k) : 1.0;
  if (DF) {
    load_exp_tables(et);
    for (int q = threadIdx.x; q < A; q += blockDim.x) {
      const df2 d = df_from_double((double)q / A);
      wj_s[q] = make_float2(d.hi, d.lo);
    }
    for (int idx = threadIdx.x; idx < L * R; idx += blockDim.x) {
      const df2 d = df_from_double(__ldg(&ray_n[(size_t)b * L * R + idx]));
      rn_s[idx] = make_float2(d.hi, d.lo);
    }
  }
  __syncthreads();
  if (active) tr_extinction<DF, VPB, TPN>(dm, lv, sp, sf, ray_n, b, k, v, j, et, rn_s, csh, chi_s);
  __syncthreads();
  // pair sums chi_i + chi_{i+1} (in place) and differences chi_{i+1} - chi_i
  if (active && j == 0) {
    for (int i = 0; i < L - 1; ++i) {
      if (DF) {
        const float2 c0 = chi_f[i * VPB + v], c1 = chi_f[(i + 1) * VPB + v];
        const df2 x0 = {c0.x, c0.y}, x1 = {c1.x, c1.y};
        const df2 s2 = df_add(x0, x1), d2 = df_sub(x1, x0);
        chi_f[i * VPB + v] = make_float2(s2.hi, s2.lo);
        dif_f[i * VPB + v] = make_float2(d2.hi, d2.lo);
        if (STORE) {
          const size_t at = ((size_t)b * L + i) * N + k;
          taps.tr_c[at] = make_float2(s2.hi, s2.lo);
          taps.tr_d[at] = make_float2(d2.hi, d2.lo);
        }
      } else {
        const double c0 = chi_s[i * VPB + v], c1 = chi_s[(i + 1) * VPB + v];
        chi_s[i * VPB + v] = c0 + c1;
        dif_s[i * VPB + v] = c1 - c0;
      }
    }
  }
  __syncthreads();
  const double Rp = ev[b].radius;
  const double* rw = rays + (size_t)b * 2 * (K + 1) + (K + 1);
  double h = 0.0;
  if (active) {
    // each thread takes every TPN-th layer and walks its A rays in groups of at most RG:
    // per level pair, the group's path lengths (contiguous, the same for the warp's
    // wavenumbers) are loaded together; every ray keeps its own sum, in level order, and
    // stops at its own cut-off
    const int ng = (A + RG - 1) / RG, gs = (A + ng - 1) / ng;
    for (int t = L - 2 - j; t >= 0; t -= TPN) {
      for (int a0 = 0; a0 < A; a0 += gs) {
        const int na = min(gs, A - a0);
        if (DF) {
          const float2* Gt = reinterpret_cast<const float2*>(geom) + ((size_t)b * (L - 1) + t) * L * A + a0;
          const float ch = dm.tau_cut_hi, cl = dm.tau_cut_lo;
          auto over = [ch, cl](df2 x) { return x.hi > ch || (x.hi == ch && x.lo > cl); };  // tau > cut-off
          const float2 c0 = chi_f[t * VPB + v], d0 = dif_f[t * VPB + v];
          df2 ts[RG], qs[RG];
          int last[RG];
          unsigned live = 0;
          // STORE: dG/db of the group's rays, in the layout of the path lengths
          const float2* Qt =
              STORE ? taps.tr_geo + (size_t)b * 3 * L * K + (size_t)2 * L * K + (size_t)t * L * A + a0 : nullptr;
#pragma unroll
          for (int u = 0; u < RG; ++u) {
            ts[u] = df2{0.0f, 0.0f};
            qs[u] = df2{0.0f, 0.0f};
            last[u] = L - 2;
            if (u < na) {
              const float2 g = __ldg(&Gt[(size_t)t * A + u]), w = wj_s[a0 + u];
              const df2 seg = df_add(df2{c0.x, c0.y}, df_mul(df2{w.x, w.y}, df2{d0.x, d0.y}));
              ts[u] = df_mul(df2{g.x, g.y}, seg);
              if (STORE) {
                const float2 q = __ldg(&Qt[(size_t)t * A + u]);
                qs[u] = df_mul(df2{q.x, q.y}, seg);
              }
              if (!over(ts[u])) live |= 1u << u;
              else last[u] = t;
            }
          }
          for (int i = t + 1; i < L - 1 && live; ++i) {
            const float2 c = chi_f[i * VPB + v];
            float2 g[RG], q[RG];
#pragma unroll
            for (int u = 0; u < RG; ++u)
              if (u < na) {
                g[u] = __ldg(&Gt[(size_t)i * A + u]);
                if (STORE) q[u] = __ldg(&Qt[(size_t)i * A + u]);
              }
            // branch-free over the group (a finished ray's sum is kept, not advanced), so
            // that the group's independent sums overlap
#pragma unroll
            for (int u = 0; u < RG; ++u)
              if (u < na) {
                const df2 n = df_fma(df2{g[u].x, g[u].y}, df2{c.x, c.y}, ts[u]);
                const bool l = (live >> u) & 1u;
                ts[u].hi = l ? n.hi : ts[u].hi;
                ts[u].lo = l ? n.lo : ts[u].lo;
                if (STORE) {
                  const df2 nq = df_fma(df2{q[u].x, q[u].y}, df2{c.x, c.y}, qs[u]);
                  qs[u].hi = l ? nq.hi : qs[u].hi;
                  qs[u].lo = l ? nq.lo : qs[u].lo;
                  if (l && over(n)) last[u] = i;
                }
                live &= ~((unsigned)(l && over(n)) << u);
              }
          }
          // T = exp(-tau) and 1 - T in double-float; one FP64 FMA per ray into h
#pragma unroll
          for (int u = 0; u < RG; ++u)
            if (u < na) {
              const df2 T = df_exp_neg(ts[u], et.hi, et.lo);
              if (STORE) {
                const size_t at = ((size_t)b * K + t * A + a0 + u) * N + k;
                taps.tr_T[at] = make_float2(T.hi, T.lo);
                taps.tr_qs[at] = make_float2(qs[u].hi, qs[u].lo);
                taps.tr_I[at] = (short)last[u];
              }
              h = fma(__ldg(&rw[t * A + a0 + u]), df_to_double(df_sub(df_make(1.0f), T)), h);
            }
        } else {
          const double* Gt = geom + ((size_t)b * (L - 1) + t) * L * A;
          for (int u = 0; u < na; ++u) {
            const int jj = a0 + u;
            double tau = __ldg(&Gt[(size_t)t * A + jj]) * (chi_s[t * VPB + v] + (double)jj / A * dif_s[t * VPB + v]);
            for (int i = t + 1; i < L - 1 && !(__double_as_longlong(tau) > dm.tau_cut_bits); ++i)
              tau = fma(__ldg(&Gt[(size_t)i * A + jj]), chi_s[i * VPB + v], tau);
            h = fma(__ldg(&rw[t * A + jj]), 1. - exp(-tau), h);
          }
        }
      }
    }
  }
  h_part[j][v] = h;
  __syncthreads();
  if (active && j == 0) {
    double hs = 0.0;
#pragma unroll
    for (int q = 0; q < TPN; ++q) hs += h_part[q][v];
    hs = sqrt(hs + Rp * Rp) - Rp;
    const double rp = hs + Rp;
    const double Rs = ev[b].star_radius;
    spectrum[(size_t)b * N + k] = rp * rp / Rs / Rs * 1e6;
  }
}

// ------------------------------------------------------------------ observation + likelihood
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Observation operator and Gaussian log-likelihood, one block per evaluation
// (Observation::processModelSpectrum src/observations/observations.cpp:290-304,
// ForwardModel::applyObservationModifier src/forward_model/forward_model.cpp:161-180,
// Retrieval::logLikelihood src/retrieval/retrieval.cpp:314-369).
//
// Secondary eclipse (OccultationModel::calcModelGPU src/forward_model/secondary_eclipse/
// secondary_eclipse.cpp:262-335, OccultationDevice src/CUDA_kernels/secondary_eclipse_kernels.cu:35-51):
// each row is binned planet flux / binned stellar flux x (R_p / R_s)^2 x 1e6 before the shift.
// The blackbody star is binned here from its point values (double-float, or FP64 when fp64
// is set); file and grid stars use their precomputed binned rows (the grid's eight corners
// interpolated per evaluation).
__global__ void obs_loglike_kernel(DeviceModel dm, const double* __restrict__ spectrum,
                                   const double* __restrict__ params, int P,
                                   const EvalInfo* __restrict__ ev, double* __restrict__ obs,
                                   double* __restrict__ loglike, uint8_t* __restrict__ neglect_out, int fp64) {
  const int b = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double* F = spectrum + (size_t)b * dm.N;
  const double infl = ev[b].inflation;
  const int star = dm.star_model;
  __shared__ ExpTables et;
  __shared__ StarCell cell;
  double teff = 0.0;
  df2 invT = {0.0f, 0.0f};
  if (star == 1) {
    load_exp_tables(et);
    teff = params[(size_t)b * P + 2];
    const double it = 1.0 / teff;
    invT.hi = (float)it;
    invT.lo = (float)(it - (double)invT.hi);
  } else if (star == 3 && threadIdx.x == 0) {
    cell = star_grid_cell(dm, params + (size_t)b * P + 2);
  }
  if (star) __syncthreads();
  double acc = 0.0;
  for (int r = warp; r < dm.M; r += nw) {
    const int k0 = __ldg(&dm.row_k0[r]), len = __ldg(&dm.row_len[r]);
    const double* w = dm.W + __ldg(&dm.row_off[r]);
    double s = 0.0, ss = 0.0;
    for (int j = lane; j < len; j += 32) s += __ldg(&w[j]) * F[k0 + j];
    if (star == 1)
      for (int j = lane; j < len; j += 32)
        ss += __ldg(&w[j]) * (fp64 ? star_blackbody_fp64(dm, k0 + j, teff) : star_blackbody_df(dm, k0 + j, invT, et));
    s = warp_sum(s);
    if (star == 1) ss = warp_sum(ss);
    if (lane == 0) {
      if (star) {
        if (star == 2) ss = __ldg(&dm.star_bin[r]);
        else if (star == 3) {
          double v[8];
          for (int i = 0; i < 8; ++i) v[i] = __ldg(&dm.star_bin[(size_t)cell.c[i] * dm.M + r]);
          ss = star_trilinear(v, cell.w);
        }
        const double rr = ev[b].radius;
        s = s / ss * rr * rr * 1e6;
      }
      const int mp = __ldg(&dm.obs_mod_param[__ldg(&dm.row_obs[r])]);
      if (mp >= 0) {
        const double shift = params[(size_t)b * P + mp];
        if (shift != 0) s += shift;
      }
      if (obs) obs[(size_t)b * dm.M + r] = s;
      const double es = __ldg(&dm.row_err2[r]) + infl;
      const double d = __ldg(&dm.row_data[r]) - s;
      const double lt = (infl == 0.0) ? __ldg(&dm.row_logterm[r]) : -0.5 * log(es * 2.0 * kPi);
      acc += (lt - 0.5 * d * d / es) * __ldg(&dm.row_weight[r]);
    }
  }
  __shared__ double red[32];
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    double v = lane < nw ? red[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) {
      const int ng = ev[b].neglect;
      if (loglike) loglike[b] = ng ? -1e30 : v;
      if (neglect_out) neglect_out[b] = (uint8_t)ng;
    }
  }
}

// High-resolution output of the plain path (RadiativeTransfer::changeSpectrumUnits
// src/radiative_transfer/radiative_transfer.h:58-60 for emission; transit depth as is;
// for the secondary eclipse planet / star x (R_p / R_s)^2 x 1e6,
// src/forward_model/secondary_eclipse/secondary_eclipse.cpp:326-332). Evaluation 0.
__global__ void spectrum_output_kernel(DeviceModel dm, const double* __restrict__ spectrum,
                                       int emission, const double* __restrict__ params,
                                       const EvalInfo* __restrict__ ev, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= dm.N) return;
  const double f = spectrum[k];
  if (dm.star_model) {
    double st;
    if (dm.star_model == 1) st = star_blackbody_fp64(dm, k, params[2]);
    else if (dm.star_model == 2) st = dm.star_hr[k];
    else {
      const StarCell c = star_grid_cell(dm, params + 2);
      double v[8];
      for (int i = 0; i < 8; ++i) v[i] = dm.star_hr[(size_t)c.c[i] * dm.N + k];
      st = star_trilinear(v, c.w);
    }
    const double rr = ev[0].radius;
    out[k] = f / st * rr * rr * 1e6;
    return;
  }
  out[k] = emission ? f / dm.wl[k] / dm.wl[k] * 10000.0 : f;
}

// Level table (set-up): for every pressure-bracket entry (species, temperature
// node, level) the log-p interpolation of the two table rows at that level,
// x = t0 + (t1 - t0) w in FP64 as the reference does per evaluation
// (OpacitySpecies::calcAbsorptionCrossSections src/transport_coeff/opacity_species.cpp:308-338),
// converted to log2 units with a two-part log2(10) and stored as a double-float.
constexpr double kLog2_10 = 3.321928094887362348, kLog2_10Tail = 1.661617516973592e-16;

__global__ void level_table_kernel(const double* __restrict__ table64, const int* __restrict__ row0,
                                   const int* __restrict__ row1, const double* __restrict__ w, long long n_lrows,
                                   size_t N, float2* __restrict__ ltab) {
  const size_t total = (size_t)n_lrows * N;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t r = idx / N, k = idx - r * N;
    const double t0 = table64[(size_t)__ldg(&row0[r]) * N + k];
    const double t1 = table64[(size_t)__ldg(&row1[r]) * N + k];
    const double x = t0 + (t1 - t0) * __ldg(&w[r]);
    const double p = x * kLog2_10;
    const double err = fma(x, kLog2_10, -p) + x * kLog2_10Tail;
    const float hi = (float)p;
    ltab[idx] = make_float2(hi, (float)((p - (double)hi) + err));
  }
}

// ------------------------------------------------------------------ host side
template <typename T>
static T* dev_upload(Model& m, const std::vector<T>& v) {
  T* p = nullptr;
  const size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
  BGB_CUDA(cudaMalloc(&p, bytes));
  if (!v.empty()) BGB_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  m.allocations.push_back(p);
  m.device_bytes += bytes;
  return p;
}

static float2 split_df(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// ------------------------------------------------------------------ shared opacity tables
struct TableSet {
  int device = 0;
  size_t bytes = 0;
  std::vector<void*> ptrs;
  double* table64 = nullptr;
  float2* ltab = nullptr;
  double* table_T = nullptr;
  int* pb_row0 = nullptr;
  int* pb_row1 = nullptr;
  double* pb_w = nullptr;
  ~TableSet() {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    for (void* p : ptrs) cudaFree(p);
    cudaSetDevice(prev);
  }
  template <typename T>
  T* upload(const std::vector<T>& v) {
    T* p = nullptr;
    const size_t n = std::max<size_t>(v.size(), 1) * sizeof(T);
    BGB_CUDA(cudaMalloc(&p, n));
    ptrs.push_back(p);
    bytes += n;
    if (!v.empty()) BGB_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
  }
};

namespace {

std::mutex g_tables_mutex;
std::map<std::string, std::weak_ptr<TableSet>> g_tables;

void fnv1a(uint64_t& h, const void* data, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
}

// Identity of a table set: device, table directory and species, spectral grid,
// pressure grid and table shapes.
std::string table_key(const Model& m) {
  uint64_t h = 1469598103934665603ull;
  fnv1a(h, m.xsec_path.data(), m.xsec_path.size());
  for (const auto& c : m.opac_cfg) {
    fnv1a(h, c.first.data(), c.first.size());
    fnv1a(h, "|", 1);
    fnv1a(h, c.second.data(), c.second.size());
    fnv1a(h, ";", 1);
  }
  fnv1a(h, m.nu.data(), m.nu.size() * sizeof(double));
  fnv1a(h, m.p.data(), m.p.size() * sizeof(double));
  fnv1a(h, m.table_T.data(), m.table_T.size() * sizeof(double));
  fnv1a(h, m.pb_row0.data(), m.pb_row0.size() * sizeof(int));
  fnv1a(h, m.pb_row1.data(), m.pb_row1.size() * sizeof(int));
  fnv1a(h, m.pb_w.data(), m.pb_w.size() * sizeof(double));
  return std::to_string(m.device) + ":" + std::to_string(m.n_rows) + ":" + std::to_string(m.N) + ":" +
         std::to_string(h);
}

}  // namespace

// Finds or builds the device tables of the model (FP64 table, level table, brackets).
static void attach_tables(Model& m) {
  const std::string key = table_key(m);
  std::lock_guard<std::mutex> lock(g_tables_mutex);
  auto it = g_tables.find(key);
  if (it != g_tables.end()) {
    if (auto ts = it->second.lock()) {
      m.tables = ts;
      m.tables_shared = true;
      return;
    }
  }
  auto ts = std::make_shared<TableSet>();
  ts->device = m.device;
  const size_t N = m.N;
  ts->table64 = ts->upload(m.table_host);
  ts->table_T = ts->upload(m.table_T);
  ts->pb_row0 = ts->upload(m.pb_row0);
  ts->pb_row1 = ts->upload(m.pb_row1);
  ts->pb_w = ts->upload(m.pb_w);
  // level table: the parameter-independent log-p step of every stencil, built once on the device
  const size_t bytes = std::max<size_t>((size_t)m.n_lrows * N, 1) * sizeof(float2);
  BGB_CUDA(cudaMalloc(&ts->ltab, bytes));
  ts->ptrs.push_back(ts->ltab);
  ts->bytes += bytes;
  if (m.n_lrows > 0) {
    level_table_kernel<<<1184, 256>>>(ts->table64, ts->pb_row0, ts->pb_row1, ts->pb_w, m.n_lrows, N, ts->ltab);
    BGB_CUDA(cudaGetLastError());
    BGB_CUDA(cudaDeviceSynchronize());
  }
  g_tables[key] = ts;
  m.tables = ts;
  m.tables_shared = false;
}

size_t table_bytes(const Model& m) { return m.tables ? m.tables->bytes : 0; }

void set_tau_cutoff(Model& m, double tau) {
  long long bits;
  std::memcpy(&bits, &tau, sizeof bits);
  m.dm.tau_cut_bits = bits;
  const float hi = (float)tau;
  m.dm.tau_cut_hi = hi;
  m.dm.tau_cut_lo = std::isinf(tau) ? 0.0f : (float)(tau - (double)hi);
}

void upload_model(Model& m) {
  BGB_CUDA(cudaSetDevice(m.device));
  const size_t N = m.N;
  DeviceModel& dm = m.dm;
  dm.L = m.L;
  dm.S = m.acfg.S;
  dm.R = m.acfg.R;
  dm.N = (int)N;
  dm.M = m.M;
  dm.P = m.acfg.nparam_total;
  dm.nobs = (int)m.obs.size();
  set_tau_cutoff(m, 10.0);  // TransmissionModel::tangentOpticalDepth src/forward_model/transmission/transmission_spectrum.cpp:136-137
  // (h nu c / k) log2(e) with log2(e) as a two-part constant
  const double log2e_hi = 1.4426950408889634, log2e_lo = 2.0355273740931033e-17;
  std::vector<double> c1(N), c2(N);
  std::vector<float2> c1df(N), c2ldf(N);
  for (size_t k = 0; k < N; ++k) {
    const double nu = m.nu[k];
    c1[k] = 2. * kPlanckH * kLightC * kLightC * nu * nu * nu;
    c2[k] = kPlanckH * nu * kLightC / kBoltzmann;
    c1df[k] = split_df(c1[k]);
    const double p = c2[k] * log2e_hi;
    const double perr = std::fma(c2[k], log2e_hi, -p) + c2[k] * log2e_lo;
    const float hi = (float)p;
    c2ldf[k] = make_float2(hi, (float)((p - (double)hi) + perr));
  }
  dm.nu = dev_upload(m, m.nu);
  dm.wl = dev_upload(m, m.wl);
  dm.planck_c1 = dev_upload(m, c1);
  dm.planck_c2 = dev_upload(m, c2);
  dm.planck_c1_df = dev_upload(m, c1df);
  dm.planck_c2l_df = dev_upload(m, c2ldf);
  dm.pressure = dev_upload(m, m.p);
  dm.log10p = dev_upload(m, m.log10p);
  m.n_lrows = (long long)m.pb_row0.size();
  attach_tables(m);
  std::vector<double>().swap(m.table_host);
  const TableSet& ts = *m.tables;
  m.d_table64 = ts.table64;
  dm.table64 = ts.table64;
  dm.ltab = ts.ltab;
  dm.table_T = ts.table_T;
  dm.pb_row0 = ts.pb_row0;
  dm.pb_row1 = ts.pb_row1;
  dm.pb_w = ts.pb_w;
  m.device_bytes += ts.bytes;
  std::vector<double> ray;
  for (int r : m.rayleigh_species) ray.insert(ray.end(), m.opac[r].rayleigh.begin(), m.opac[r].rayleigh.end());
  ray.insert(ray.end(), m.hm_rows.begin(), m.hm_rows.end());  // H- continuum rows follow the Rayleigh rows
  dm.R_ray = m.acfg.R_ray;
  dm.annuli = m.transmission ? m.annuli : 1;
  dm.cloud_kind = m.acfg.cloud_kind;
  dm.rayleigh = dev_upload(m, ray);
  {
    // two zero entries past the last row: whole 16-byte units of the last row can be
    // bulk-copied when the row length is odd
    std::vector<float2> rdf(ray.size() + 2, make_float2(0.0f, 0.0f));
    for (size_t i = 0; i < ray.size(); ++i) rdf[i] = split_df(ray[i]);
    dm.rayleigh_df = dev_upload(m, rdf);
  }
  // observation operator rows in internal order, observations concatenated
  std::vector<int> k0, len, robs, rout, modp;
  std::vector<long long> off;
  std::vector<double> data, err2, wgt, logt;
  int pidx = m.nparam_general + m.nparam_chem + m.nparam_temp + m.nparam_cloud;
  for (size_t o = 0; o < m.obs.size(); ++o) {
    const ObservationSetup& ob = m.obs[o];
    modp.push_back(ob.nb_modifier ? pidx : -1);
    pidx += ob.nb_modifier;
    for (int j = 0; j < ob.n; ++j) {
      k0.push_back(ob.row_k0[j]);
      len.push_back(ob.row_len[j]);
      off.push_back(ob.row_off[j]);
      robs.push_back((int)o);
      rout.push_back(ob.out_offset + (ob.ascending ? ob.n - 1 - j : j));
      data.push_back(ob.data[j]);
      const double es = ob.error[j] * ob.error[j];
      err2.push_back(es);
      wgt.push_back(ob.weight[j]);
      logt.push_back(-0.5 * std::log(es * 2.0 * kPi));
    }
  }
  dm.row_k0 = dev_upload(m, k0);
  dm.row_len = dev_upload(m, len);
  dm.row_off = dev_upload(m, off);
  dm.W = dev_upload(m, m.W);
  dm.row_obs = dev_upload(m, robs);
  dm.row_out = dev_upload(m, rout);
  dm.row_data = dev_upload(m, data);
  dm.row_err2 = dev_upload(m, err2);
  dm.row_weight = dev_upload(m, wgt);
  dm.row_logterm = dev_upload(m, logt);
  dm.obs_mod_param = dev_upload(m, modp);
  dm.star_model = m.occultation ? m.star_model : 0;
  for (int a = 0; a < 3; ++a) dm.star_n[a] = m.star_n[a];
  dm.star_axes = m.star_axes.empty() ? nullptr : dev_upload(m, m.star_axes);
  dm.star_hr = m.star_hr.empty() ? nullptr : dev_upload(m, m.star_hr);
  dm.star_bin = m.star_bin.empty() ? nullptr : dev_upload(m, m.star_bin);
  {
    // first row of each observation, and the operator transposed (rows reading
    // each wavenumber, in ascending row order) for the adjoint
    std::vector<int> start(m.obs.size() + 1, 0);
    for (size_t o = 0; o < m.obs.size(); ++o) start[o + 1] = start[o] + m.obs[o].n;
    dm.obs_row_start = dev_upload(m, start);
    std::vector<int> cptr(N + 1, 0);
    for (size_t r = 0; r < k0.size(); ++r)
      for (int j = 0; j < len[r]; ++j) ++cptr[(size_t)k0[r] + j + 1];
    for (size_t k = 0; k < N; ++k) cptr[k + 1] += cptr[k];
    std::vector<int> crow((size_t)cptr[N]), fill(cptr.begin(), cptr.end() - 1);
    std::vector<double> cw((size_t)cptr[N]);
    for (size_t r = 0; r < k0.size(); ++r)
      for (int j = 0; j < len[r]; ++j) {
        const int at = fill[(size_t)k0[r] + j]++;
        crow[at] = (int)r;
        cw[at] = m.W[(size_t)off[r] + j];
      }
    dm.col_ptr = dev_upload(m, cptr);
    dm.col_row = dev_upload(m, crow);
    dm.col_w = dev_upload(m, cw);
  }
  std::vector<AtmosphereConfig> cfg{m.acfg};
  m.d_cfg = dev_upload(m, cfg);
  dm.cfg = m.d_cfg;
  BGB_CUDA(cudaMallocHost(&m.h_pinned, 64 * 1024));
  m.h_pinned_bytes = 64 * 1024;
  // the transmission kernels stage L x blockDim doubles of extinction in shared memory
  if (m.transmission) {
    const int sm = (int)kTransmissionDynSmem;
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<true, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<false, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<false, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<true, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<false, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<true, 32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel<true, 64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 8, 8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<32, 8, 3, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 8, 8, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 8, 7, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 4, 16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 8, 8, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_kernel_x2<16, 8, 6, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_annuli_kernel<true, 32, 4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_annuli_kernel<true, 32, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_annuli_kernel<true, 32, 8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_annuli_kernel<false, 32, 4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    BGB_CUDA(cudaFuncSetAttribute(transmission_annuli_kernel<true, 32, 4, 4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  }
}

static void free_workspace(Workspace& w) {
  cudaFree(w.params);
  cudaFree(w.lev);
  cudaFree(w.ls);
  cudaFree(w.lsdf);
  cudaFree(w.ray_n);
  cudaFree(w.ev);
  cudaFree(w.spectrum);
  cudaFree(w.obs);
  cudaFree(w.loglike);
  cudaFree(w.geom);
  cudaFree(w.rays);
  w = Workspace{};
}

void ensure_workspace(Model& m, int batch) {
  if (batch <= m.ws.capacity) return;
  BGB_CUDA(cudaSetDevice(m.device));
  BGB_CUDA(cudaDeviceSynchronize());
  free_workspace(m.ws);
  Workspace& w = m.ws;
  const size_t B = batch, L = m.L, S = std::max(m.acfg.S, 1), N = m.N, M = std::max(m.M, 1);
  const size_t P = std::max(m.acfg.nparam_total, 1);
  const size_t R = std::max(m.acfg.R, 1);
  BGB_CUDA(cudaMalloc(&w.params, B * P * sizeof(double)));
  BGB_CUDA(cudaMalloc(&w.lev, B * L * sizeof(LevelInfo)));
  BGB_CUDA(cudaMalloc(&w.ls, B * L * S * sizeof(LevelSpecies)));
  BGB_CUDA(cudaMalloc(&w.lsdf, B * L * S * sizeof(LevelSpeciesDF)));
  BGB_CUDA(cudaMalloc(&w.ray_n, B * L * R * sizeof(double)));
  BGB_CUDA(cudaMalloc(&w.ev, B * sizeof(EvalInfo)));
  BGB_CUDA(cudaMalloc(&w.spectrum, B * N * sizeof(double)));
  BGB_CUDA(cudaMalloc(&w.obs, B * M * sizeof(double)));
  BGB_CUDA(cudaMalloc(&w.loglike, B * sizeof(double)));
  if (m.transmission) {
    const size_t K = transmission_rays(m);
    BGB_CUDA(cudaMalloc(&w.geom, B * std::max(K, L) * L * sizeof(double)));
    BGB_CUDA(cudaMalloc(&w.rays, B * 2 * (K + 1) * sizeof(double)));
  }
  w.capacity = batch;
  ++m.ws_generation;
}

// Kernel sequence of one batch on the given work buffers.
// taps (optional, gradient pass): receives d wT / dT of every stencil and the
// intensities after every level.
static void launch_stages(Model& m, const double* params_dev, int batch, const Workspace& w, cudaStream_t st,
                          bool profile, uint8_t* neglect_dev, double* loglike_dev,
                          const ForwardTaps* taps = nullptr) {
  const DeviceModel& dm = m.dm;
  const int L = m.L;
  const int atm_threads = ((L + 31) / 32) * 32;
  if (profile) BGB_CUDA(cudaEventRecord(m.ev[0], st));
  atmosphere_kernel<<<batch, atm_threads, 4 * L * sizeof(double), st>>>(dm, params_dev, dm.P, w.lev, w.ls,
                                                                        w.lsdf, w.ray_n, w.ev,
                                                                        taps ? taps->dwT : nullptr);
  BGB_CUDA(cudaGetLastError());
  if (profile) BGB_CUDA(cudaEventRecord(m.ev[1], st));
  // launch shape: explicit setting, else the autotuned one for batches, else the default
  const int rt = m.rt_threads > 0 ? m.rt_threads : (batch > 1 ? m.tuned_rt : 0);
  if (!m.transmission) {
    const int TB = rt > 0 ? rt : (batch == 1 ? 64 : 128);
    dim3 grid(batch, (dm.N + TB - 1) / TB);
    // batches: two wavenumbers per thread (the single evaluation of the plain path keeps one
    // per thread, which puts twice as many threads on its one spectrum)
    const bool pair = batch >= 2;
    const int TB2 = std::min(TB, kPairThreads);  // launch bound of the two-wavenumber kernel
    const dim3 grid2(batch, (dm.N + 2 * TB2 - 1) / (2 * TB2));
    const size_t hm_smem = m.hm ? (size_t)L * kHmTerms * sizeof(float2) : 0;
    if (taps && m.precision == 1)
      emission_kernel_fp64<true><<<grid, TB, 0, st>>>(dm, w.lev, w.ls, w.ray_n, w.ev, w.spectrum, taps->istore);
    else if (taps && (m.acfg.cloud_kind || m.hm))  // non-grey cloud or H- continuum
      emission_kernel<true, true><<<grid, TB, hm_smem, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.spectrum,
                                                            taps->istore, taps->em_layer);
    else if (taps && pair)
      emission_kernel_x2<true><<<grid2, TB2, 0, st>>>(dm, w.lev, w.lsdf, w.ev, w.spectrum, taps->istore,
                                                     taps->em_layer);
    else if (taps)
      emission_kernel<true><<<grid, TB, 0, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.spectrum,
                                                taps->istore, taps->em_layer);
    else if (m.precision == 1)
      emission_kernel_fp64<false><<<grid, TB, 0, st>>>(dm, w.lev, w.ls, w.ray_n, w.ev, w.spectrum, nullptr);
    else if (m.hm || m.acfg.cloud_kind)
      emission_kernel<false, true><<<grid, TB, hm_smem, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev,
                                                             w.spectrum, nullptr);
    else if (pair)
      emission_kernel_x2<false><<<grid2, TB2, 0, st>>>(dm, w.lev, w.lsdf, w.ev, w.spectrum, nullptr);
    else
      emission_kernel<false><<<grid, TB, 0, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.spectrum, nullptr);
  } else if (m.annuli > 1) {
    // A impact parameters per layer: 32 wavenumbers per block, extinction sums and
    // differences staged; the launch shape selects threads per wavenumber x rays summed
    // together: 16 -> 4 x 4, 32 (default) -> 8 x 4, 64 -> 8 x 8 (FP64 path: 4 threads)
    const bool df = m.precision != 1;
    const size_t sm = annuli_dyn_smem(L, dm.R, df);
    if (sm > kTransmissionDynSmem) throw Error(BEAR_ERR_UNSUPPORTED, "too many levels for the transmission kernel");
    const dim3 grid(batch, (dm.N + 31) / 32);
    const int K = transmission_rays(m);
    const dim3 ggrid(batch, (K + 1 + 127) / 128);  // one thread per ray + the top level
    auto go = [&](auto kernel, int tpn) {
      kernel<<<grid, tpn * 32, sm, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.geom, w.rays, w.spectrum,
                                         ForwardTaps{});
    };
    if (taps) {
      // gradient pass: the double-float kernel storing the ray data (4 threads per wavenumber,
      // 4 rays per group)
      if (!df) throw Error(BEAR_ERR_UNSUPPORTED, "the transmission gradient runs in precision mode 0");
      transmission_annuli_geometry_kernel<true><<<ggrid, 128, 0, st>>>(dm, w.lev, w.ev, w.geom, w.rays);
      BGB_CUDA(cudaGetLastError());
      tr_geometry_adjoint_annuli_kernel<<<dim3(batch, (unsigned)std::min<size_t>(((size_t)K * L + 255) / 256, 65535)),
                                          256, 0, st>>>(
          dm, w.lev, w.ev, reinterpret_cast<const float2*>(w.geom), w.rays, taps->tr_geo);
      BGB_CUDA(cudaGetLastError());
      transmission_annuli_kernel<true, 32, 4, 4, true><<<grid, 4 * 32, sm, st>>>(
          dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.geom, w.rays, w.spectrum, *taps);
    } else if (df) {
      transmission_annuli_geometry_kernel<true><<<ggrid, 128, 0, st>>>(dm, w.lev, w.ev, w.geom, w.rays);
      BGB_CUDA(cudaGetLastError());
      if (rt == 16) go(transmission_annuli_kernel<true, 32, 4, 4>, 4);
      else if (rt == 64) go(transmission_annuli_kernel<true, 32, 8, 8>, 8);
      else go(transmission_annuli_kernel<true, 32, 8, 4>, 8);
    } else {
      transmission_annuli_geometry_kernel<false><<<ggrid, 128, 0, st>>>(dm, w.lev, w.ev, w.geom, w.rays);
      BGB_CUDA(cudaGetLastError());
      go(transmission_annuli_kernel<false, 32, 4, 1>, 4);
    }
  } else {
    const dim3 ggrid(batch, (L * L + 255) / 256);
    if (m.precision == 1) transmission_geometry_kernel<false><<<ggrid, 256, 0, st>>>(dm, w.lev, w.ev, w.geom, w.rays);
    else transmission_geometry_kernel<true><<<ggrid, 256, 0, st>>>(dm, w.lev, w.ev, w.geom, w.rays);
    // the launch shape: 16, 32 or 64 wavenumbers per block with 4 threads each; paired
    // wavenumbers: 160 (the double-float default; 32 wavenumbers per block, 8 threads per pair,
    // table reads of two species issued together), 176 (one species per group), 208 (four),
    // 224 (4 threads per pair: twice the levels per thread), 192 (64 wavenumbers per block).
    // The FP64 path takes 32 for the paired shapes.
    const int vpb = (rt == 16 || rt == 64) ? rt : 32;
    dim3 grid(batch, (dm.N + vpb - 1) / vpb);
    const bool df = m.precision != 1;
    const int pairs = (rt == 16 || rt == 32 || rt == 64) ? 0 : (rt == 192 ? 32 : 16);
    const int tpn_x = rt == 224 ? 4 : 8;  // threads per pair (levels per thread: L / tpn_x)
    // extinction column and Rayleigh densities, at least the height-group sums that reuse them
    const size_t sm = std::max((size_t)L * vpb * sizeof(double) + (df ? (size_t)L * dm.R * sizeof(float2) : 0),
                               (size_t)kHeightGroups * vpb * sizeof(double));
    if (sm > kTransmissionDynSmem) throw Error(BEAR_ERR_UNSUPPORTED, "too many levels for the transmission kernel");
    const ForwardTaps none{};
    auto go = [&](auto kernel) {
      kernel<<<grid, kTPN * vpb, sm, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev, w.geom, w.rays, w.spectrum, none);
    };
    if (taps) {
      // gradient pass: double-float kernel storing the ray data
      if (!df) throw Error(BEAR_ERR_UNSUPPORTED, "the transmission gradient runs in precision mode 0");
      tr_geometry_adjoint_kernel<<<dim3(batch, (L * L + 255) / 256), 256, 0, st>>>(
          dm, w.lev, w.ev, reinterpret_cast<const float2*>(w.geom), taps->tr_geo);
      BGB_CUDA(cudaGetLastError());
      if (pairs) {
        // the paired kernel, 32 wavenumbers per block, whatever the paired shape
        const size_t smx = std::max((size_t)L * 16 * sizeof(float4) + (size_t)L * dm.R * sizeof(float2),
                                    (size_t)kHeightGroups * 2 * 16 * sizeof(double));
        if (smx > kTransmissionDynSmem) throw Error(BEAR_ERR_UNSUPPORTED, "too many levels for the transmission kernel");
        const dim3 gx(batch, (dm.N + 31) / 32);
        if (rt == 192)
          transmission_kernel_x2<16, 8, 6, 2, true><<<gx, 128, smx, st>>>(dm, w.lev, w.lsdf, w.ray_n, w.ev, w.geom,
                                                                          w.rays, w.spectrum, *taps);
        else
          transmission_kernel_x2<16, 8, 8, 2, true><<<gx, 128, smx, st>>>(dm, w.lev, w.lsdf, w.ray_n, w.ev, w.geom,
                                                                          w.rays, w.spectrum, *taps);
        BGB_CUDA(cudaGetLastError());
        if (profile) BGB_CUDA(cudaEventRecord(m.ev[2], st));
        const int OTx = m.obs_threads > 0 ? m.obs_threads : 256;
        obs_loglike_kernel<<<batch, OTx, 0, st>>>(dm, w.spectrum, params_dev, dm.P, w.ev, w.obs, loglike_dev,
                                                 neglect_dev, m.precision == 1);
        BGB_CUDA(cudaGetLastError());
        if (profile) BGB_CUDA(cudaEventRecord(m.ev[3], st));
        return;
      }
      // the tuned wavenumbers per block when it is 64, else 32
      const int sv = vpb == 64 ? 64 : 32;
      const dim3 gs(batch, (dm.N + sv - 1) / sv);
      const size_t sms = std::max((size_t)L * sv * sizeof(double) + (size_t)L * dm.R * sizeof(float2),
                                  (size_t)kHeightGroups * sv * sizeof(double));
      if (sv == 64)
        transmission_kernel<true, 64, true><<<gs, kTPN * 64, sms, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev,
                                                                        w.geom, w.rays, w.spectrum, *taps);
      else
        transmission_kernel<true, 32, true><<<gs, kTPN * 32, sms, st>>>(dm, w.lev, w.ls, w.lsdf, w.ray_n, w.ev,
                                                                        w.geom, w.rays, w.spectrum, *taps);
    } else if (df && pairs) {
      const size_t smx = std::max((size_t)L * pairs * sizeof(float4) + (size_t)L * dm.R * sizeof(float2),
                                  (size_t)kHeightGroups * 2 * pairs * sizeof(double));
      if (smx > kTransmissionDynSmem) throw Error(BEAR_ERR_UNSUPPORTED, "too many levels for the transmission kernel");
      const dim3 gx(batch, (dm.N + 2 * pairs - 1) / (2 * pairs));
      auto gox = [&](auto kernel, int tpn) {
        kernel<<<gx, tpn * pairs, smx, st>>>(dm, w.lev, w.lsdf, w.ray_n, w.ev, w.geom, w.rays, w.spectrum, none);
      };
      if (pairs == 32) gox(transmission_kernel_x2<32, 8, 3, 2>, 8);
      else if (rt == 176) gox(transmission_kernel_x2<16, 8, 8, 1>, 8);   // one species per table-read group
      else if (rt == 208) gox(transmission_kernel_x2<16, 8, 7, 4>, 8);   // four species per group
      else if (rt == 224) gox(transmission_kernel_x2<16, 4, 16, 2>, tpn_x);  // 4 threads per pair
      else gox(transmission_kernel_x2<16, 8, 8, 2>, 8);
    } else if (vpb == 16) df ? go(transmission_kernel<true, 16>) : go(transmission_kernel<false, 16>);
    else if (vpb == 64) df ? go(transmission_kernel<true, 64>) : go(transmission_kernel<false, 64>);
    else df ? go(transmission_kernel<true, 32>) : go(transmission_kernel<false, 32>);
  }
  BGB_CUDA(cudaGetLastError());
  if (profile) BGB_CUDA(cudaEventRecord(m.ev[2], st));
  const int OT = m.obs_threads > 0 ? m.obs_threads : 256;
  obs_loglike_kernel<<<batch, OT, 0, st>>>(dm, w.spectrum, params_dev, dm.P, w.ev, w.obs, loglike_dev,
                                          neglect_dev, m.precision == 1);
  BGB_CUDA(cudaGetLastError());
  if (profile) BGB_CUDA(cudaEventRecord(m.ev[3], st));
}

void launch_forward(Model& m, const double* params_dev, int batch, cudaStream_t st,
                    bool want_loglike, uint8_t* neglect_dev, double* loglike_dev) {
  ensure_workspace(m, batch);
  if (m.profiling)
    for (auto& e : m.ev)
      if (!e) BGB_CUDA(cudaEventCreate(&e));
  launch_stages(m, params_dev, batch, m.ws, st, m.profiling, neglect_dev,
                want_loglike ? (loglike_dev ? loglike_dev : m.ws.loglike) : nullptr);
  if (m.profiling) m.ev_recorded = true;
}

// One evaluation with caller-supplied work buffers (used by the allocation-free
// entry point): the kernels and launch shapes of the plain path, no workspace
// growth, no profiling events.
void launch_forward_into(Model& m, const double* params_dev, const Workspace& w, cudaStream_t st,
                         uint8_t* neglect_dev, double* loglike_dev) {
  launch_stages(m, params_dev, 1, w, st, false, neglect_dev, loglike_dev);
}

// Forward pass of the gradient: the plain kernel sequence on the model's
// workspace with the adjoint's taps.
void launch_forward_taps(Model& m, const double* params_dev, int batch, cudaStream_t st, uint8_t* neglect_dev,
                         double* loglike_dev, const ForwardTaps& taps) {
  launch_stages(m, params_dev, batch, m.ws, st, false, neglect_dev, loglike_dev, &taps);
}

void stage_times(Model& m, float* ms3) {
  if (!m.ev_recorded) throw Error(BEAR_ERR_STATE, "no profiled evaluation recorded");
  BGB_CUDA(cudaEventSynchronize(m.ev[3]));
  for (int i = 0; i < 3; ++i) BGB_CUDA(cudaEventElapsedTime(&ms3[i], m.ev[i], m.ev[i + 1]));
}

// Distinct table rows the last batch's stencils read: rows of the level table
// (2 per species and level, double-float path) or of the FP64 table (4 per
// species and level, precision mode 1).
long long stencil_rows(Model& m, int batch) {
  if (batch < 1 || batch > m.ws.capacity) throw Error(BEAR_ERR_SIZE, "batch exceeds the workspace");
  const size_t n = (size_t)batch * m.L * std::max(m.acfg.S, 1);
  BGB_CUDA(cudaDeviceSynchronize());
  long long count = 0;
  if (m.precision == 0) {
    std::vector<LevelSpeciesDF> h(n);
    BGB_CUDA(cudaMemcpy(h.data(), m.ws.lsdf, n * sizeof(LevelSpeciesDF), cudaMemcpyDeviceToHost));
    std::vector<char> seen((size_t)m.n_lrows, 0);
    for (const auto& e : h) {
      if (e.lg2n_hi == kNoSpecies) continue;
      for (int r : e.lrow)
        if (r >= 0 && r < m.n_lrows && !seen[r]) {
          seen[r] = 1;
          ++count;
        }
    }
  } else {
    std::vector<LevelSpecies> h(n);
    BGB_CUDA(cudaMemcpy(h.data(), m.ws.ls, n * sizeof(LevelSpecies), cudaMemcpyDeviceToHost));
    std::vector<char> seen((size_t)m.n_rows, 0);
    for (const auto& e : h)
      for (int r : e.row)
        if (r >= 0 && r < m.n_rows && !seen[r]) {
          seen[r] = 1;
          ++count;
        }
  }
  return count;
}

void launch_spectrum_output(Model& m, double* out_dev, cudaStream_t st) {
  spectrum_output_kernel<<<(m.dm.N + 255) / 256, 256, 0, st>>>(m.dm, m.ws.spectrum, m.transmission ? 0 : 1,
                                                              m.ws.params, m.ws.ev, out_dev);
  BGB_CUDA(cudaGetLastError());
}

void release_model(Model& m) {
  cudaSetDevice(m.device);
  cudaDeviceSynchronize();
  free_workspace(m.ws);
  free_grad_workspace(m);
  m.tables.reset();
  for (void* p : m.allocations) cudaFree(p);
  m.allocations.clear();
  for (auto& e : m.ev)
    if (e) cudaEventDestroy(e);
  if (m.h_pinned) cudaFreeHost(m.h_pinned);
  m.h_pinned = nullptr;
}

}  // namespace bgb
