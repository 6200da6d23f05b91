// Adjoint (reverse-mode) gradient of the log-likelihood with respect to the
// physical parameters, emission models.
//
// Kernel chain for one chunk of evaluations:
//   atmosphere_kernel + emission_kernel<STORE> + obs_loglike_kernel
//       the forward pass, also writing d wT / dT of every table stencil and the
//       two Gauss-angle intensities after every level (B x L x 2 x N FP64)
//   obs_adjoint_kernel         d log L / d binned model, the shift and error-
//                              inflation parameters, sum_k dlogL/dF_k F_k
//   emission_adjoint_kernel    per wavenumber: the seed W^T dlogL/dbin, then the
//                              short-characteristics recurrence run backwards from
//                              the top with every level opacity recomputed (never
//                              stored); per-level sinks (log number densities,
//                              temperature, layer thickness, cloud optical depth)
//                              reduced per block into partial sums
//   atmosphere_adjoint_kernel  per evaluation: the partial sums reduced in a fixed
//                              order, then mapped onto the parameters through the
//                              tangents of the level physics (temperature profile,
//                              chemistry, hydrostatic layer thickness, grey cloud,
//                              radius-distance scaling)
// Every reduction runs in a fixed order, so the gradient is bit-reproducible.
//
// Derivative conventions at the model's non-smooth points: discrete decisions
// are held fixed -- opacity-table brackets (the gradient of the bilinear
// interpolation on the current cell; zero temperature slope when T is clamped
// to the table's end), the grey cloud's integer layer indices (so d/d cloud-top
// pressure and d/d cloud-bottom factor are 0), exactly transparent layers
// (tau == 0 contributes nothing). A model neglected by the forward pass (50 K
// temperature clamp, negative background abundance) has log L = -1e30 and a
// zero gradient.
//
// Arithmetic: in precision mode 0 the adjoint runs in double-float on the FP32
// pipe (about 48 significant bits, ample for a gradient): the level opacities
// are recomputed with the forward's own double-float routines, the layer adjoint
// uses a double-float exponential and Taylor series for thin layers, and the
// per-level sinks are reduced as double-floats. Precision mode 1 does every step
// in FP64 with the CUDA math library and serves as the reference gradient.

#include <algorithm>
#include <cmath>
#include <string>

#include "../../include/bear_gb300.h"
#include "adjoint_common.cuh"
#include "level_physics.cuh"
#include "model.h"
#include "rt_common.cuh"
#include "rt_pair.cuh"
#include "star.cuh"

namespace bgb {

// ------------------------------------------------------------------ likelihood adjoint
// log L = sum_r w_r (-0.5 log(2 pi e_r) - 0.5 (d_r - s_r)^2 / e_r), e_r = sigma_r^2 + 10^b
// (Retrieval::logLikelihood src/retrieval/retrieval.cpp:314-369): writes
// gS_r = d log L / d s_r, the shift (src/forward_model/forward_model.cpp:161-180) and
// error-inflation derivatives into the gradient row (zeroing the rest), and per
// evaluation the seed normaliser 2^-e, its inverse and sum_r gS_r (s_r - shift_r).
//
// Secondary eclipse: s_r = p_r / q_r (R_p/R_s)^2 1e6 + shift with p_r the binned planet
// flux and q_r the binned stellar flux. gS_r then receives d log L / d p_r =
// d log L / d s_r (R_p/R_s)^2 1e6 / q_r (the seed of the emission adjoint), and the
// gradient row d/d(R_p/R_s) = sum_r d log L / d s_r 2 (s_r - shift_r) / (R_p/R_s) and
// d/d(stellar parameters) = -sum_r d log L / d s_r (s_r - shift_r) / q_r dq_r/d theta
// (blackbody: q_r and dq_r/dT_eff in FP64 from the row's points; grid: the trilinear
// weights' derivatives, zero where a parameter is clamped or on a node).
__global__ void __launch_bounds__(256) obs_adjoint_kernel(DeviceModel dm, const double* __restrict__ params, int P,
                                                          const EvalInfo* __restrict__ ev,
                                                          const double* __restrict__ obs, double* __restrict__ gS,
                                                          double* __restrict__ seed, double* __restrict__ grad,
                                                          int transmission) {
  __shared__ double red[7][256];
  __shared__ StarCell cell;
  const int b = blockIdx.x, tid = threadIdx.x;
  const int M = dm.M;
  const bool neg = ev[b].neglect != 0;
  const double infl = ev[b].inflation;
  const double* par = params + (size_t)b * P;
  for (int j = tid; j < P; j += blockDim.x) grad[(size_t)b * P + j] = 0.0;
  auto row_grad = [&](int r, double& s_out, double& d_out, double& es_out) {
    const double s = obs[(size_t)b * M + r];
    const double es = __ldg(&dm.row_err2[r]) + infl;
    const double d = __ldg(&dm.row_data[r]) - s;
    s_out = s;
    d_out = d;
    es_out = es;
    return neg ? 0.0 : __ldg(&dm.row_weight[r]) * d / es;
  };
  const int star = dm.star_model;
  if (star == 3 && tid == 0) cell = star_grid_cell(dm, par + 2);
  __syncthreads();
  const double rr = ev[b].radius;
  double sgs = 0.0, sinf = 0.0, gmax = 0.0, grr = 0.0, gst[3] = {0.0, 0.0, 0.0};
  for (int r = tid; r < M; r += blockDim.x) {
    double s, d, es;
    const double g = row_grad(r, s, d, es);
    const int mp = __ldg(&dm.obs_mod_param[__ldg(&dm.row_obs[r])]);
    double pre = s;
    if (mp >= 0) {
      const double sh = par[mp];
      if (sh != 0) pre = s - sh;
    }
    sinf += __ldg(&dm.row_weight[r]) * 0.5 * (d * d / es - 1.0) / es;
    if (star) {
      double q = 0.0, dq[3] = {0.0, 0.0, 0.0};
      if (star == 1) {
        const int k0 = __ldg(&dm.row_k0[r]), len = __ldg(&dm.row_len[r]);
        const double* w = dm.W + __ldg(&dm.row_off[r]);
        const double teff = par[2];
        for (int j = 0; j < len; ++j) {
          const double wj = __ldg(&w[j]);
          q = fma(wj, star_blackbody_fp64(dm, k0 + j, teff), q);
          dq[0] = fma(wj, star_blackbody_dT(dm, k0 + j, teff), dq[0]);
        }
      } else if (star == 2) {
        q = __ldg(&dm.star_bin[r]);
      } else {
        double v[8], dv[3];
        for (int i = 0; i < 8; ++i) v[i] = __ldg(&dm.star_bin[(size_t)cell.c[i] * M + r]);
        q = star_trilinear(v, cell.w);
        star_trilinear_dw(v, cell.w, dv);
        for (int a = 0; a < 3; ++a) dq[a] = dv[a] * cell.dw[a];
      }
      const double gp = g * rr * rr * 1e6 / q;
      gS[(size_t)b * M + r] = gp;
      gmax = fmax(gmax, fabs(gp));
      grr = fma(g, 2.0 * pre / rr, grr);
      for (int a = 0; a < 3; ++a) gst[a] = fma(-g * pre / q, dq[a], gst[a]);
    } else {
      gS[(size_t)b * M + r] = g;
      sgs = fma(g, pre, sgs);
      gmax = fmax(gmax, fabs(g));
    }
  }
  red[0][tid] = sgs;
  red[1][tid] = sinf;
  red[2][tid] = gmax;
  red[3][tid] = grr;
  for (int a = 0; a < 3; ++a) red[4 + a][tid] = gst[a];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (tid < h) {
      red[0][tid] += red[0][tid + h];
      red[1][tid] += red[1][tid + h];
      red[2][tid] = fmax(red[2][tid], red[2][tid + h]);
      for (int a = 3; a < 7; ++a) red[a][tid] += red[a][tid + h];
    }
    __syncthreads();
  }
  const double tot_gs = red[0][0], tot_inf = red[1][0], tot_max = red[2][0];
  if (tid == 0 && star && !neg) {
    grad[(size_t)b * P + 1] += red[3][0];
    const int nst = star == 1 ? 1 : star == 3 ? 3 : 0;
    for (int a = 0; a < nst; ++a) grad[(size_t)b * P + 2 + a] += red[4 + a][0];
  }
  __syncthreads();
  // observation shifts: d log L / d shift_o = sum of gS over the observation's rows
  for (int o = 0; o < dm.nobs; ++o) {
    const int mp = __ldg(&dm.obs_mod_param[o]);
    if (mp < 0) continue;
    double acc = 0.0;
    for (int r = __ldg(&dm.obs_row_start[o]) + tid; r < __ldg(&dm.obs_row_start[o + 1]); r += blockDim.x) {
      double s, d, es;
      acc += row_grad(r, s, d, es);
    }
    red[0][tid] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if (tid < h) red[0][tid] += red[0][tid + h];
      __syncthreads();
    }
    if (tid == 0 && !neg) grad[(size_t)b * P + mp] += red[0][0];
    __syncthreads();
  }
  if (tid == 0) {
    if (!neg && infl != 0.0) grad[(size_t)b * P + P - 1] += tot_inf * infl * kLn10;
    // normalise the seed of the spectral adjoint to O(1) so the double-float sinks
    // stay well inside the float range
    // emission: dF/dI scale; transmission: d depth / dh times R_p^2 (so g_tau ~ wz / R_p)
    const double unit = transmission ? 1e6 / (ev[b].star_radius * ev[b].star_radius) * ev[b].radius * ev[b].radius
                                     : ev[b].scaling * kPi * 1e-3;
    const double mx = tot_max * unit;
    double nrm = 1.0, inv = 1.0;
    if (mx > 0.0 && isfinite(mx)) {
      const int e = ilogb(mx);
      nrm = ldexp(1.0, -e);
      inv = ldexp(1.0, e);
    }
    seed[b * 3 + 0] = nrm;
    seed[b * 3 + 1] = inv;
    seed[b * 3 + 2] = tot_gs;
  }
}

// ------------------------------------------------------------------ spectral adjoint (emission)
struct AdjointArgs {
  const LevelInfo* lev;
  const LevelSpecies* ls;
  const LevelSpeciesDF* lsdf;
  const EvalInfo* ev;
  const float2* dwT;
  const double* istore;
  const double* gS;
  const double* seed;
  double* partial;
  int V;
};

// Adjoint of one short-characteristics layer in FP64 (forward: sc_layer):
// I = a (I' - B') + B + q (B - B'), a = exp(-delta), q = (a - 1) / delta,
// delta = tau / mu. Given lam = d log L / d I it accumulates d/dB, d/dB', d/dtau and
// replaces lam by d log L / d I'.
__device__ __forceinline__ void sc_layer_adjoint_fp64(double tau, double B, double Bp, double Ip1, double Ip2,
                                                      double& lam1, double& lam2, double& gB, double& gBp,
                                                      double& gtau) {
  const double dB = B - Bp;
  const double rtau = 1.0 / tau;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double d = tau * kInvMu[i];
    const double a = exp(-d);
    const double rd = kMu[i] * rtau;  // 1 / delta
    const double q = (a - 1.0) * rd;
    double& lam = i == 0 ? lam1 : lam2;
    const double Ip = i == 0 ? Ip1 : Ip2;
    gB = fma(lam, 1.0 + q, gB);
    gBp = fma(lam, -a - q, gBp);
    // dq/ddelta = -(a + q) / delta; Taylor series 1/2 - d/3 + d^2/8 - d^3/30 + d^4/144 below 1e-2
    const double dq = d < 1e-2 ? fma(d, fma(d, fma(d, fma(d, 1.0 / 144.0, -1.0 / 30.0), 0.125), -1.0 / 3.0), 0.5)
                               : -(a + q) * rd;
    const double gd = fma(-a * lam, Ip - Bp, dq * lam * dB);
    gtau = fma(gd, kInvMu[i], gtau);
    lam *= a;
  }
}

// Gauss nodes and their reciprocals as double-floats
constexpr double kMu0 = 0.211324865405187, kMu1 = 0.788675134594813;
constexpr float kMuHi0 = (float)kMu0, kMuLo0 = (float)(kMu0 - (double)kMuHi0);
constexpr float kMuHi1 = (float)kMu1, kMuLo1 = (float)(kMu1 - (double)kMuHi1);
constexpr float kInvMuHi0 = (float)(1.0 / kMu0), kInvMuLo0 = (float)(1.0 / kMu0 - (double)kInvMuHi0);
constexpr float kInvMuHi1 = (float)(1.0 / kMu1), kInvMuLo1 = (float)(1.0 / kMu1 - (double)kInvMuHi1);
constexpr float kThirdHi = (float)(1.0 / 3.0), kThirdLo = (float)(1.0 / 3.0 - (double)kThirdHi);
constexpr float kSixthHi = (float)(1.0 / 6.0), kSixthLo = (float)(1.0 / 6.0 - (double)kSixthHi);

// The same layer adjoint in double-float arithmetic (precision mode 0), from the
// layer's optical depth t and its reciprocal rt as double-floats. Below delta = 1e-2
// 1 + q, -a - q and dq/ddelta come from their Taylor series (no cancellation):
// 1 + q = d (1/2 - d/6 + d^2/24 - d^3/120 + d^4/720), dq/dd = 1/2 - d/3 + d^2/8 - d^3/30
// + d^4/144, -a - q = d dq/dd.
__device__ __forceinline__ void sc_layer_adjoint_df(df2 t, df2 rt, df2 B, df2 Bp, df2 Ip1, df2 Ip2, df2& lam1,
                                                    df2& lam2, df2& gB, df2& gBp, df2& gtau, const ExpTables& et) {
  const df2 dB = df_sub(B, Bp);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const df2 invmu = i == 0 ? df2{kInvMuHi0, kInvMuLo0} : df2{kInvMuHi1, kInvMuLo1};
    const df2 mu = i == 0 ? df2{kMuHi0, kMuLo0} : df2{kMuHi1, kMuLo1};
    const df2 d = df_mul(t, invmu);
    const df2 a = df_exp_neg(d, et.hi, et.lo);
    df2 s1, nq, dq;
    if (d.hi < 1e-2f) {
      const float df_ = d.hi;
      const float p1 = BGB_FMA(-df_, BGB_FMA(-df_, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f);
      df2 P = df_sub(df2{kSixthHi, kSixthLo}, df_mul_f(d, p1));
      P = df_sub(df_make(0.5f), df_mul(d, P));
      s1 = df_mul(d, P);
      const float p2 = BGB_FMA(-df_, BGB_FMA(-df_, 1.0f / 144.0f, 1.0f / 30.0f), 0.125f);
      df2 Q = df_sub(df2{kThirdHi, kThirdLo}, df_mul_f(d, p2));
      dq = df_sub(df_make(0.5f), df_mul(d, Q));
      nq = df_mul(d, dq);
    } else {
      const df2 rd = df_mul(rt, mu);  // 1 / delta
      const df2 q = df_mul(df_sub(a, df_make(1.0f)), rd);
      s1 = df_add(df_make(1.0f), q);
      nq = df_neg(df_add(a, q));
      dq = df_mul(nq, rd);
    }
    df2& lam = i == 0 ? lam1 : lam2;
    const df2 Ip = i == 0 ? Ip1 : Ip2;
    gB = df_add(gB, df_mul(lam, s1));
    gBp = df_add(gBp, df_mul(lam, nq));
    const df2 gd = df_sub(df_mul(dq, df_mul(lam, dB)), df_mul(a, df_mul(lam, df_sub(Ip, Bp))));
    gtau = df_add(gtau, df_mul(gd, invmu));
    lam = df_mul(lam, a);
  }
}

// ------------------------------------------------------------------ two wavenumbers per thread
// The double-float steps above for two wavenumbers with paired FP32 instructions
// (dfloat2x.cuh): element e of every result is bit for bit the single-wavenumber result for
// element e's inputs.

// planck_df2 (physics.cuh) per element, c1 and c2l per element, 1/T shared
__device__ __forceinline__ dfx planck_dfx(dfx c1, dfx c2l, df2 invT, const ExpTables& et) {
  const dfx y = dfx_neg(dfx_mul(c2l, dfx_bcast(invT)));
  int2 n;
  const dfx m = dfx_exp2(y, n, et.hi, et.lo);
  if (n.x >= -60 && n.y >= -60) {
    const dfx u = dfx_ldexp_normal(m, n);
    const dfx d = dfx_sub(dfx_bcast(df_make(1.0f)), u);
    return dfx_mul(dfx_mul(c1, u), dfx_recip(d));
  }
  dfx r;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const df2 me = dfx_get(m, e), c1e = dfx_get(c1, e);
    const int ne = e ? n.y : n.x;
    df2 v;
    if (ne < -60) {
      v = df_ldexp(df_mul(c1e, me), ne);
    } else {
      const df2 u = df_ldexp(me, ne);
      v = df_mul(df_mul(c1e, u), df_recip(df_sub(df_make(1.0f), u)));
    }
    dfx_set(r, e, v);
  }
  return r;
}

// sc_layer_adjoint_df per element, both elements with a nonzero layer depth; rt is the
// reciprocal depth where t.hi > 1e-30 and zero elsewhere. Where the elements fall on
// different sides of delta = 1e-2, both branches are formed and each element keeps its own.
__device__ __forceinline__ void sc_layer_adjoint_x(dfx t, dfx rt, dfx B, dfx Bp, dfx Ip1, dfx Ip2, dfx& lam1,
                                                   dfx& lam2, dfx& gB, dfx& gBp, dfx& gtau, const ExpTables& et) {
  const dfx dB = dfx_sub(B, Bp);
  const dfx one = dfx_bcast(df_make(1.0f)), half = dfx_bcast(df_make(0.5f));
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const dfx invmu = dfx_bcast(i == 0 ? df2{kInvMuHi0, kInvMuLo0} : df2{kInvMuHi1, kInvMuLo1});
    const dfx mu = dfx_bcast(i == 0 ? df2{kMuHi0, kMuLo0} : df2{kMuHi1, kMuLo1});
    const dfx d = dfx_mul(t, invmu);
    const dfx a = dfx_exp_neg(d, et.hi, et.lo);
    const bool sm0 = d.hi.x < 1e-2f, sm1 = d.hi.y < 1e-2f;
    const dfx z = {f2(0.0f), f2(0.0f)};
    dfx s1 = z, nq = z, dq = z;
    if (sm0 || sm1) {
      const float2 dh = f2neg(d.hi);
      const float2 p1 = f2fma(dh, f2fma(dh, f2(1.0f / 720.0f), f2(1.0f / 120.0f)), f2(1.0f / 24.0f));
      dfx P = dfx_sub(dfx_bcast(df2{kSixthHi, kSixthLo}), dfx_mul_f(d, p1));
      P = dfx_sub(half, dfx_mul(d, P));
      s1 = dfx_mul(d, P);
      const float2 p2 = f2fma(dh, f2fma(dh, f2(1.0f / 144.0f), f2(1.0f / 30.0f)), f2(0.125f));
      const dfx Q = dfx_sub(dfx_bcast(df2{kThirdHi, kThirdLo}), dfx_mul_f(d, p2));
      dq = dfx_sub(half, dfx_mul(d, Q));
      nq = dfx_mul(d, dq);
    }
    if (!(sm0 && sm1)) {
      const dfx rd = dfx_mul(rt, mu);  // 1 / delta
      const dfx q = dfx_mul(dfx_sub(a, one), rd);
      const dfx s1n = dfx_add(one, q);
      const dfx nqn = dfx_neg(dfx_add(a, q));
      const dfx dqn = dfx_mul(nqn, rd);
      s1 = dfx_select(sm0, sm1, s1, s1n);
      nq = dfx_select(sm0, sm1, nq, nqn);
      dq = dfx_select(sm0, sm1, dq, dqn);
    }
    dfx& lam = i == 0 ? lam1 : lam2;
    const dfx Ip = i == 0 ? Ip1 : Ip2;
    gB = dfx_add(gB, dfx_mul(lam, s1));
    gBp = dfx_add(gBp, dfx_mul(lam, nq));
    const dfx gd = dfx_sub(dfx_mul(dq, dfx_mul(lam, dB)), dfx_mul(a, dfx_mul(lam, dfx_sub(Ip, Bp))));
    gtau = dfx_add(gtau, dfx_mul(gd, invmu));
    lam = dfx_mul(lam, a);
  }
}

// One thread per wavenumber (kAdjThreads per block), grid (evaluations, tiles).
// Dynamic shared memory: per-species opacity terms of two levels,
// float2 [2][S][kAdjThreads] then double [2][S][kAdjThreads].
// partial[b][l][v][tile]: v = 0..S-1 d log L / d ln n_s, S temperature, S+1 lev.dz,
// S+2 lev.cloud (all times the evaluation's seed normaliser).
// Six blocks per SM in the double-float path (80 registers): the sweep is bound by
// the latency of the table reads, so occupancy beats the few spilled registers.
template <bool DF, int VP>
__global__ void __launch_bounds__(kAdjThreads, DF ? 6 : 4) emission_adjoint_kernel(DeviceModel dm, AdjointArgs a) {
  typedef AccType<DF> AT;
  typedef typename AT::type A;
  constexpr int NW = kAdjThreads / 32;
  constexpr int G = 32 / VP;
  __shared__ ExpTables et;
  __shared__ double red[NW][VP];
  extern __shared__ __align__(16) unsigned char adj_smem[];
  const int S = dm.S, L = dm.L;
  float2* tdf = reinterpret_cast<float2*>(adj_smem);
  double* twd = reinterpret_cast<double*>(adj_smem + (size_t)2 * S * kAdjThreads * sizeof(float2));
  if (DF) load_exp_tables(et);
  __syncthreads();
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int kk = blockIdx.y * kAdjThreads + tid;
  const bool active = kk < dm.N;
  const int k = active ? kk : dm.N - 1;  // idle lanes repeat the last wavenumber with a zero seed
  const size_t N = dm.N;
  const LevelInfo* lv = a.lev + (size_t)b * L;
  const LevelSpecies* sp = a.ls + (size_t)b * L * S;
  const LevelSpeciesDF* sf = a.lsdf + (size_t)b * L * S;
  const float2* dw = a.dwT + (size_t)b * L * S;
  const double* Is = a.istore + (size_t)b * L * 2 * N + k;

  // seed: d log L / dF_k = sum_r W_rk gS_r, F = scaling 2 pi 1e-3 (mu1 I1 + mu2 I2) / 2
  double gF = 0.0;
  {
    const double* g = a.gS + (size_t)b * dm.M;
    const int e1 = __ldg(&dm.col_ptr[k + 1]);
    for (int e = __ldg(&dm.col_ptr[k]); e < e1; ++e) gF = fma(__ldg(&dm.col_w[e]), g[__ldg(&dm.col_row[e])], gF);
  }
  const double sd = active ? gF * a.seed[b * 3] * __ldg(&a.ev[b].scaling) * (kPi * 1e-3) : 0.0;

  // level opacity; per-species terms into buffer q; d kappa / dT (double-float part
  // and an FP64 part for terms outside the float range)
  auto kappa_terms = [&](int l, int q, df2& dk_out, double& dkw_out, bool& wide) -> Kappa {
    float2* td = tdf + (size_t)q * S * kAdjThreads + tid;
    double* tw = twd + (size_t)q * S * kAdjThreads + tid;
    const float2* dwl = dw + (size_t)l * S;
    Kappa kp;
    if (DF) {
      df2 dk = {0.0f, 0.0f};
      double dkw = 0.0;
      bool wd = false;
      kp = level_kappa_df_cb(dm.ltab, N, sf + (size_t)l * S, S, k, et,
                             [&](int s, df2 t, double t_w, bool is_wide, df2 lo, df2 hi) {
                               const float2 d = __ldg(dwl + s);
                               td[(size_t)s * kAdjThreads] = make_float2(t.hi, t.lo);
                               tw[(size_t)s * kAdjThreads] = t_w;
                               if (d.x != 0.0f) {
                                 const df2 slope = df_mul(df_sub(hi, lo), df2{d.x, d.y});
                                 if (is_wide) dkw += t_w * df_to_double(slope);
                                 else dk = df_add(dk, df_mul(t, slope));
                               }
                               wd = wd || is_wide;
                             });
      // level-table values are log2 cross sections: d(2^y)/dy = 2^y ln 2
      dk_out = df_mul(dk, df2{kLn2Hi, kLn2Lo});
      dkw_out = dkw * 0.693147180559945309;
      wide = wd;
    } else {
      double dk = 0.0;
      kp.v = df2{0.0f, 0.0f};
      kp.wide = level_absorption_fp64_cb(dm.table64, N, sp + (size_t)l * S, S, k,
                                         [&](int s, double t, double lo, double hi) {
                                           const float2 d = __ldg(dwl + s);
                                           tw[(size_t)s * kAdjThreads] = t;
                                           dk += t * (hi - lo) * ((double)d.x + (double)d.y);
                                         });
      dk_out = df2{0.0f, 0.0f};
      dkw_out = dk * kLn10;
      wide = true;
    }
    return kp;
  };
  // reduce one level's sinks over the block and write the block's partial sums;
  // gK, gT, gdz, gcl as double-floats (mode 0) or in the .wide-style FP64 arguments (mode 1)
  auto emit = [&](int l, int q, df2 gK, double gK64, A gT, A gdz, A gcl, bool wide) {
    const float2* td = tdf + (size_t)q * S * kAdjThreads + tid;
    const double* tw = twd + (size_t)q * S * kAdjThreads + tid;
    A v[VP];
#pragma unroll
    for (int j = 0; j < VP; ++j) {
      A x = AT::zero();
      if (j < S) {
        if constexpr (DF) {
          const float2 t = td[(size_t)j * kAdjThreads];
          x = df_mul(gK, df2{t.x, t.y});
          if (wide) x = df_add(x, df_from_double(df_to_double(gK) * tw[(size_t)j * kAdjThreads]));
        } else {
          x = gK64 * tw[(size_t)j * kAdjThreads];
        }
      } else if (j == S) {
        x = gT;
      } else if (j == S + 1) {
        x = gdz;
      } else if (j == S + 2) {
        x = gcl;
      }
      v[j] = x;
    }
    const A r = warp_reduce_scatter<VP>(v, lane);
    if (lane % G == 0) red[warp][lane / G] = acc_to_double(r);
    __syncthreads();
    if (tid < a.V) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < NW; ++w) s += red[w][tid];
      a.partial[(((size_t)b * L + l) * a.V + tid) * gridDim.y + blockIdx.y] = s;
    }
    __syncthreads();
  };

  int q = 0;
  if constexpr (DF) {
    // ---------------- double-float recurrence (precision mode 0)
    const float2 c1f = __ldg(dm.planck_c1_df + k), c2f = __ldg(dm.planck_c2l_df + k);
    const df2 c1 = {c1f.x, c1f.y}, c2l = {c2f.x, c2f.y};
    const df2 c2 = df_mul(c2l, df2{kLn2Hi, kLn2Lo});  // h nu c / k
    const df2 rc1 = df_div(df_make(1.0f), c1);
    auto invT = [&](int l) {
      const float2 it = __ldg(reinterpret_cast<const float2*>(&lv[l].invT_hi));
      return df2{it.x, it.y};
    };
    // dB/dT = B (1 + B / c1) x / T with x = c2 / T
    auto dplanck = [&](int l, df2 B) {
      const df2 it = invT(l);
      return df_mul(df_mul(B, df_add(df_make(1.0f), df_mul(B, rc1))), df_mul(df_mul(c2, it), it));
    };
    df2 lam1 = df_from_double(sd * kMu[0]), lam2 = df_from_double(sd * kMu[1]);
    df2 dk_l;
    double dkw_l;
    bool wide_l;
    Kappa kap_l = kappa_terms(L - 1, q, dk_l, dkw_l, wide_l);
    df2 B_l = planck_df2(c1, c2l, invT(L - 1), et.hi, et.lo);
    const df2 z = {0.0f, 0.0f};
    df2 gB_l = z, gK_l = z, gdz_l = z, gcl_l = z;
    for (int l = L - 1; l >= 1; --l) {
      df2 dk_m;
      double dkw_m;
      bool wide_m;
      const Kappa kap_m = kappa_terms(l - 1, q ^ 1, dk_m, dkw_m, wide_m);
      const df2 B_m = planck_df2(c1, c2l, invT(l - 1), et.hi, et.lo);
      // layer optical depth as in the forward pass (emission_layer_tau_df)
      const float4 g = __ldg(reinterpret_cast<const float4*>(&lv[l - 1].dzh_hi));  // dzh, cloud
      const df2 dzh = {g.x, g.y};
      const bool narrow = kap_l.wide == 0.0 && kap_m.wide == 0.0;
      df2 t = df_add(df_mul(dzh, df_add(kap_l.v, kap_m.v)), df2{g.z, g.w});
      bool opaque_layer = t.hi != 0.0f;
      if (!narrow || !(t.hi > 1e-30f && t.hi < 1e30f)) {
        const double ks = (df_to_double(kap_l.v) + kap_l.wide) + (df_to_double(kap_m.v) + kap_m.wide);
        const double tau = __ldg(&lv[l - 1].dz) * ks / 2. + __ldg(&lv[l - 1].cloud);
        opaque_layer = tau != 0.0;
        t = df_from_double(fmin(tau, 1e37));
      }
      df2 gB_m = z, gtau = z;
      if (opaque_layer) {
        const df2 rt = t.hi > 1e-30f ? df_recip(t) : z;  // only used above delta = 1e-2
        const df2 Ip1 = df_from_double_bits(Is[(size_t)(l - 1) * 2 * N]);
        const df2 Ip2 = df_from_double_bits(Is[(size_t)(l - 1) * 2 * N + N]);
        sc_layer_adjoint_df(t, rt, B_l, B_m, Ip1, Ip2, lam1, lam2, gB_l, gB_m, gtau, et);
      }
      gK_l = df_add(gK_l, df_mul(gtau, dzh));
      df2 gT = df_add(df_mul(gK_l, dk_l), df_mul(gB_l, dplanck(l, B_l)));
      if (wide_l) gT = df_add(gT, df_from_double(df_to_double(gK_l) * dkw_l));
      emit(l, q, gK_l, 0.0, gT, gdz_l, gcl_l, wide_l);
      // layer l's own sinks belong to lev[l-1] (its dz and cloud)
      if (narrow) {
        gdz_l = df_mul(gtau, df_mul_f(df_add(kap_l.v, kap_m.v), 0.5f));
      } else {
        const double ks = (df_to_double(kap_l.v) + kap_l.wide) + (df_to_double(kap_m.v) + kap_m.wide);
        gdz_l = df_from_double(df_to_double(gtau) * 0.5 * ks);
      }
      gcl_l = gtau;
      gK_l = df_mul(gtau, dzh);
      gB_l = gB_m;
      B_l = B_m;
      kap_l = kap_m;
      dk_l = dk_m;
      dkw_l = dkw_m;
      wide_l = wide_m;
      q ^= 1;
    }
    gB_l = df_add(gB_l, df_add(lam1, lam2));  // both angles start from I = B at the bottom level
    df2 gT = df_add(df_mul(gK_l, dk_l), df_mul(gB_l, dplanck(0, B_l)));
    if (wide_l) gT = df_add(gT, df_from_double(df_to_double(gK_l) * dkw_l));
    emit(0, q, gK_l, 0.0, gT, gdz_l, gcl_l, wide_l);
  } else {
    // ---------------- FP64 recurrence with the CUDA math library (precision mode 1)
    const double c1d = __ldg(dm.planck_c1 + k), c2d = __ldg(dm.planck_c2 + k);
    const double rc1 = 1.0 / c1d;
    auto planck = [&](int l) { return c1d / (exp(c2d * __ldg(&lv[l].invT)) - 1.0); };
    auto dplanck = [&](int l, double B) {
      const double it = __ldg(&lv[l].invT);
      return B * fma(B, rc1, 1.0) * (c2d * it) * it;
    };
    double lam1 = sd * kMu[0], lam2 = sd * kMu[1];
    df2 unused = {0.0f, 0.0f};
    double dk_l;
    bool wide_l;
    Kappa kap_l = kappa_terms(L - 1, q, unused, dk_l, wide_l);
    double B_l = planck(L - 1);
    double gB_l = 0.0, gK_l = 0.0, gdz_l = 0.0, gcl_l = 0.0;
    for (int l = L - 1; l >= 1; --l) {
      double dk_m;
      bool wide_m;
      const Kappa kap_m = kappa_terms(l - 1, q ^ 1, unused, dk_m, wide_m);
      const double B_m = planck(l - 1);
      const double tau = __ldg(&lv[l - 1].dz) * (kap_l.wide + kap_m.wide) / 2. + __ldg(&lv[l - 1].cloud);
      double gB_m = 0.0, gtau = 0.0;
      if (tau != 0.0) {
        const double Ip1 = Is[(size_t)(l - 1) * 2 * N], Ip2 = Is[(size_t)(l - 1) * 2 * N + N];
        sc_layer_adjoint_fp64(tau, B_l, B_m, Ip1, Ip2, lam1, lam2, gB_l, gB_m, gtau);
      }
      const double dzh = 0.5 * __ldg(&lv[l - 1].dz);
      gK_l = fma(gtau, dzh, gK_l);
      emit(l, q, unused, gK_l, fma(gK_l, dk_l, gB_l * dplanck(l, B_l)), gdz_l, gcl_l, wide_l);
      gdz_l = gtau * 0.5 * (kap_l.wide + kap_m.wide);
      gcl_l = gtau;
      gK_l = gtau * dzh;
      gB_l = gB_m;
      B_l = B_m;
      kap_l = kap_m;
      dk_l = dk_m;
      wide_l = wide_m;
      q ^= 1;
    }
    gB_l += lam1 + lam2;
    emit(0, q, unused, gK_l, fma(gK_l, dk_l, gB_l * dplanck(0, B_l)), gdz_l, gcl_l, wide_l);
  }
}

// ------------------------------------------------------------------ split adjoint (precision mode 0)
// The default gradient splits the emission adjoint in two kernels so that the
// opacity recomputation and the per-level reductions run with full occupancy:
//
// emission_adjoint_sweep_kernel   one thread per (evaluation, two wavenumbers): the reverse
//     short-characteristics recurrence from the forward's stored intensities, layer
//     optical depths and half opacity sums (so no opacities are recomputed here), the
//     Planck function recomputed per level; writes d log L / d kappa of every level and
//     reduces the level sinks that need no opacity: temperature through B_nu, layer
//     thickness and cloud depth (values S, S+1, S+2 of the partial sums).
// emission_adjoint_sinks_kernel   one block per (evaluation, level, 1024 wavenumbers), eight
//     wavenumbers per thread: recomputes the species terms of the level opacity and their
//     temperature slope, accumulates d log L / d ln n_s and the opacity part of
//     d log L / dT in registers over the eight wavenumbers, then one warp reduce-scatter and
//     one block reduction (values 0 .. S).
// The two write disjoint tile slots of the (zeroed) partial sums, which
// atmosphere_adjoint_kernel reduces as before.
struct SweepArgs {
  const LevelInfo* lev;
  const EvalInfo* ev;
  const double* istore;
  const float4* layer;  // forward's layer optical depth and half opacity sum
  const double* gS;
  const double* seed;
  float2* gK;           // out: d log L / d kappa per (evaluation, level, wavenumber)
  double* partial;
  int V, tiles_total;
};

// Two wavenumbers per thread: ka = tile 2 kAdjThreads + tid (element 0) and ka + kAdjThreads
// (element 1), each with its own seed; an element past the grid repeats the last
// wavenumber with a zero seed. The recurrence of each element is the single-wavenumber
// double-float recurrence bit for bit; the block sums of the level sinks add the thread's
// two elements first.
// Five blocks per SM (96 registers, a few spilled): 55.7 ms for the gradient of 512
// evaluations of 80 levels x 10257 points, against 56.7 ms at 128 registers and 58.7 ms
// unbounded (152 registers, three blocks per SM).
// CLOUD (power-law and KH clouds): the layer's cloud depth is cloud_l f_k with the
// wavelength factor f_k of the evaluation's cloud parameters, so the cloud sink of level l
// is sum_k g_tau f_k, and value S + 3 + c of level 0 receives
// sum_k (sum_l g_tau cloud_l) df_k/dtheta_c for the NC shape parameters theta_c.
template <bool CLOUD>
__global__ void __launch_bounds__(kAdjThreads, 5) emission_adjoint_sweep_kernel(DeviceModel dm, SweepArgs a) {
  constexpr int NW = kAdjThreads / 32;
  __shared__ ExpTables et;
  __shared__ double red[NW][4];
  load_exp_tables(et);
  __syncthreads();
  const int L = dm.L;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t N = dm.N;
  const LevelInfo* lv = a.lev + (size_t)b * L;
  const double* Is[2];
  const float4* lay[2];
  float2* gKo[2];
  bool act[2];
  double sd[2];
  dfx c1, c2l, c2, rc1;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const int kk = blockIdx.y * 2 * kAdjThreads + e * kAdjThreads + tid;
    act[e] = kk < dm.N;
    const int k = act[e] ? kk : dm.N - 1;
    Is[e] = a.istore + (size_t)b * L * 2 * N + k;
    lay[e] = a.layer + (size_t)b * L * N + k;
    gKo[e] = a.gK + (size_t)b * L * N + k;
    // seed: d log L / dF_k = sum_r W_rk gS_r, F = scaling 2 pi 1e-3 (mu1 I1 + mu2 I2) / 2
    double gF = 0.0;
    const double* g = a.gS + (size_t)b * dm.M;
    const int e1 = __ldg(&dm.col_ptr[k + 1]);
    for (int j = __ldg(&dm.col_ptr[k]); j < e1; ++j) gF = fma(__ldg(&dm.col_w[j]), g[__ldg(&dm.col_row[j])], gF);
    sd[e] = act[e] ? gF * a.seed[b * 3] * __ldg(&a.ev[b].scaling) * (kPi * 1e-3) : 0.0;
    const float2 c1f = __ldg(dm.planck_c1_df + k), c2f = __ldg(dm.planck_c2l_df + k);
    const df2 c1e = {c1f.x, c1f.y}, c2le = {c2f.x, c2f.y};
    dfx_set(c1, e, c1e);
    dfx_set(c2l, e, c2le);
    dfx_set(c2, e, df_mul(c2le, df2{kLn2Hi, kLn2Lo}));  // h nu c / k
    dfx_set(rc1, e, df_div(df_make(1.0f), c1e));
  }
  auto invT = [&](int l) {
    const float2 it = __ldg(reinterpret_cast<const float2*>(&lv[l].invT_hi));
    return df2{it.x, it.y};
  };
  const dfx one = dfx_bcast(df_make(1.0f));
  // dB/dT = B (1 + B / c1) x / T with x = c2 / T
  auto dplanck = [&](int l, dfx B) {
    const dfx it = dfx_bcast(invT(l));
    return dfx_mul(dfx_mul(B, dfx_add(one, dfx_mul(B, rc1))), dfx_mul(dfx_mul(c2, it), it));
  };
  // the three opacity-free sinks of level l, the thread's two elements added, reduced over the block
  auto emit3 = [&](int l, dfx gBT, dfx gdz, dfx gcl) {
    df2 v[4] = {df_add(dfx_get(gBT, 0), dfx_get(gBT, 1)), df_add(dfx_get(gdz, 0), dfx_get(gdz, 1)),
                df_add(dfx_get(gcl, 0), dfx_get(gcl, 1)), df2{0.0f, 0.0f}};
    const df2 r = warp_reduce_scatter<4>(v, lane);
    if ((lane & 7) == 0) red[warp][lane >> 3] = df_to_double(r);
    __syncthreads();
    if (tid < 3) {
      double sum = 0.0;
#pragma unroll
      for (int w = 0; w < NW; ++w) sum += red[w][tid];
      a.partial[(((size_t)b * L + l) * a.V + dm.S + tid) * a.tiles_total + blockIdx.y] = sum;
    }
    __syncthreads();
  };

  const df2 z = {0.0f, 0.0f};
  const dfx zx = dfx_bcast(z);
  // non-grey cloud: the wavelength factors as the forward pass forms them, and the
  // per-wavenumber sum of g_tau cloud_l over the layers
  dfx csx = zx, wc = zx;
  if (CLOUD) {
    const int k0 = min((int)(blockIdx.y * 2 * kAdjThreads + tid), dm.N - 1);
    const int k1 = min((int)(blockIdx.y * 2 * kAdjThreads + kAdjThreads + tid), dm.N - 1);
    csx = dfx_make(df_from_double(cloud_shape(dm, a.ev[b], k0)), df_from_double(cloud_shape(dm, a.ev[b], k1)));
  }
  dfx lam1 = dfx_make(df_from_double(sd[0] * kMu[0]), df_from_double(sd[1] * kMu[0]));
  dfx lam2 = dfx_make(df_from_double(sd[0] * kMu[1]), df_from_double(sd[1] * kMu[1]));
  dfx B_l = planck_dfx(c1, c2l, invT(L - 1), et);
  dfx gB_l = zx, gK_l = zx, gdz_l = zx, gcl_l = zx;
  for (int l = L - 1; l >= 1; --l) {
    const dfx B_m = planck_dfx(c1, c2l, invT(l - 1), et);
    const float4 ta = lay[0][(size_t)l * N], tb = lay[1][(size_t)l * N];
    const dfx t = {make_float2(ta.x, tb.x), make_float2(ta.y, tb.y)};
    const dfx ksh = {make_float2(ta.z, tb.z), make_float2(ta.w, tb.w)};
    const float4 gz = __ldg(reinterpret_cast<const float4*>(&lv[l - 1].dzh_hi));  // dzh, cloud
    const dfx dzh = dfx_bcast(df2{gz.x, gz.y});
    dfx gB_m = zx, gtau = zx;
    const bool nz0 = t.hi.x != 0.0f, nz1 = t.hi.y != 0.0f;
    if (nz0 || nz1) {
      const size_t ip = (size_t)(l - 1) * 2 * N;
      const dfx Ip1 = dfx_make(df_from_double_bits(Is[0][ip]), df_from_double_bits(Is[1][ip]));
      const dfx Ip2 = dfx_make(df_from_double_bits(Is[0][ip + N]), df_from_double_bits(Is[1][ip + N]));
      if (nz0 && nz1) {
        // the reciprocal depth is only used above delta = 1e-2
        const dfx rt = dfx_select(t.hi.x > 1e-30f, t.hi.y > 1e-30f, dfx_recip(t), zx);
        sc_layer_adjoint_x(t, rt, B_l, B_m, Ip1, Ip2, lam1, lam2, gB_l, gB_m, gtau, et);
      } else {
        // one element's layer has zero depth (its sweep passes the layer unchanged): the
        // single-wavenumber steps for the other
        const int e = nz0 ? 0 : 1;
        const df2 te = dfx_get(t, e);
        const df2 rt = te.hi > 1e-30f ? df_recip(te) : z;
        df2 l1 = dfx_get(lam1, e), l2 = dfx_get(lam2, e), gb = dfx_get(gB_l, e), gbm = z, gt = z;
        sc_layer_adjoint_df(te, rt, dfx_get(B_l, e), dfx_get(B_m, e), dfx_get(Ip1, e), dfx_get(Ip2, e), l1, l2, gb,
                            gbm, gt, et);
        dfx_set(lam1, e, l1);
        dfx_set(lam2, e, l2);
        dfx_set(gB_l, e, gb);
        dfx_set(gB_m, e, gbm);
        dfx_set(gtau, e, gt);
      }
    }
    gK_l = dfx_add(gK_l, dfx_mul(gtau, dzh));
    if (act[0]) gKo[0][(size_t)l * N] = make_float2(gK_l.hi.x, gK_l.lo.x);
    if (act[1]) gKo[1][(size_t)l * N] = make_float2(gK_l.hi.y, gK_l.lo.y);
    emit3(l, dfx_mul(gB_l, dplanck(l, B_l)), gdz_l, gcl_l);
    // layer l's own sinks belong to lev[l-1] (its dz and cloud)
    gdz_l = dfx_mul(gtau, ksh);
    gcl_l = CLOUD ? dfx_mul(gtau, csx) : gtau;
    if (CLOUD && gz.z != 0.0f) wc = dfx_fma(gtau, dfx_bcast(df2{gz.z, gz.w}), wc);
    gK_l = dfx_mul(gtau, dzh);
    gB_l = gB_m;
    B_l = B_m;
  }
  gB_l = dfx_add(gB_l, dfx_add(lam1, lam2));  // both angles start from I = B at the bottom level
  if (act[0]) gKo[0][0] = make_float2(gK_l.hi.x, gK_l.lo.x);
  if (act[1]) gKo[1][0] = make_float2(gK_l.hi.y, gK_l.lo.y);
  emit3(0, dfx_mul(gB_l, dplanck(0, B_l)), gdz_l, gcl_l);
  if (CLOUD) {
    // sum_k w_k df_k/dtheta_c over the block, into value S + 3 + c of level 0
    const int nc = dm.cloud_kind == 1 ? 1 : 3;
    double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      if (!act[e]) continue;
      const int k = blockIdx.y * 2 * kAdjThreads + e * kAdjThreads + tid;
      double d[3];
      cloud_shape_tangent(dm, a.ev[b], k, d);
      const double w = df_to_double(dfx_get(wc, e));
      for (int c = 0; c < nc; ++c) v[c] = fma(w, d[c], v[c]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = warp_sum_d(v[c]);
    if (lane == 0)
      for (int c = 0; c < 3; ++c) red[warp][c] = v[c];
    __syncthreads();
    if (tid < nc) {
      double sum = 0.0;
#pragma unroll
      for (int w = 0; w < NW; ++w) sum += red[w][tid];
      a.partial[(((size_t)b * L + 0) * a.V + dm.S + 3 + tid) * a.tiles_total + blockIdx.y] = sum;
    }
  }
}

struct SinkArgs {
  const LevelSpeciesDF* lsdf;
  const float2* dwT;
  const float2* gK;
  double* partial;
  int V, tiles_total, tile0;  // this kernel's slots start at tile0
  int hm_v0;                  // H- continuum: the value of its first coefficient (0: none)
};

constexpr int kSinkKPT = 8;  // wavenumbers per thread of the sink kernel (55.3 ms gradient batch at B = 512, 56.4 with 4)
constexpr int kSinkGrp = 2;  // species whose table reads the sink kernel issues together

template <int VP>
__global__ void __launch_bounds__(kAdjThreads) emission_adjoint_sinks_kernel(DeviceModel dm, SinkArgs a) {
  constexpr int NW = kAdjThreads / 32;
  constexpr int G = 32 / VP;
  __shared__ ExpTables et;
  __shared__ double red[NW][VP];
  load_exp_tables(et);
  __syncthreads();
  const int S = dm.S, L = dm.L;
  const int b = blockIdx.x, l = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t N = dm.N;
  const LevelSpeciesDF* sf = a.lsdf + ((size_t)b * L + l) * S;
  const float2* dwl = a.dwT + ((size_t)b * L + l) * S;
  const float2* gKl = a.gK + ((size_t)b * L + l) * N;
  const df2 z = {0.0f, 0.0f};
  df2 acc[VP];
#pragma unroll
  for (int j = 0; j < VP; ++j) acc[j] = z;
  // the thread's wavenumbers in pairs (j, j + 1) = (ka, ka + kAdjThreads): the species terms
  // and slopes of both are formed with paired FP32 instructions (dfloat2x.cuh, per element bit
  // for bit the single-wavenumber arithmetic), and each accumulator receives the pair's
  // contributions in wavenumber order, as one wavenumber per step would add them
#pragma unroll 1
  for (int j = 0; j < kSinkKPT; j += 2) {
    const int ka = (blockIdx.z * kSinkKPT + j) * kAdjThreads + tid;
    if (ka >= dm.N) break;
    const bool hb = ka + kAdjThreads < dm.N;
    const int kb = hb ? ka + kAdjThreads : ka;
    const float2 gka = gKl[ka];
    const float2 gkb = hb ? gKl[kb] : make_float2(0.0f, 0.0f);
    const bool use_a = gka.x != 0.0f, use_b = gkb.x != 0.0f;  // zero seeds add nothing
    if (!use_a && !use_b) continue;
    const df2 gKa = {gka.x, gka.y}, gKb = {gkb.x, gkb.y};
    double gK64a = 0.0, gK64b = 0.0;
    dfx dk = {f2(0.0f), f2(0.0f)};
    double dkwa = 0.0, dkwb = 0.0;
    // species in groups of kSinkGrp: a group's table reads are issued before its arithmetic
#pragma unroll
    for (int s0 = 0; s0 < VP - 1; s0 += kSinkGrp) {
      if (s0 >= S) break;
      float2 t0a[kSinkGrp], t0b[kSinkGrp], t1a[kSinkGrp], t1b[kSinkGrp];
#pragma unroll
      for (int g = 0; g < kSinkGrp; ++g) {
        const int s = s0 + g;
        if (s >= S || s >= VP - 1) break;
        const int4 rw = __ldg(reinterpret_cast<const int4*>(sf + s));
        const float2* r0 = dm.ltab + (size_t)rw.x * N;
        const float2* r1 = dm.ltab + (size_t)rw.y * N;
        t0a[g] = __ldg(r0 + ka);
        t0b[g] = __ldg(r0 + kb);
        t1a[g] = __ldg(r1 + ka);
        t1b[g] = __ldg(r1 + kb);
      }
#pragma unroll
      for (int g = 0; g < kSinkGrp; ++g) {
        const int s = s0 + g;
        if (s >= S || s >= VP - 1) break;
        // species term 2^y of the level opacity (level_kappa_df_cb) and its temperature slope
        const float4 fb = __ldg(reinterpret_cast<const float4*>(sf + s) + 1);  // wT, log2 n
        if (fb.z == kNoSpecies) continue;
        const dfx lo = {make_float2(t0a[g].x, t0b[g].x), make_float2(t0a[g].y, t0b[g].y)};
        const dfx hi = {make_float2(t1a[g].x, t1b[g].x), make_float2(t1a[g].y, t1b[g].y)};
        // lo + (hi - lo) wT + log2 n, as the forward pass forms it (level_kappa_df_cb)
        const dfx diff = dfx_sub(hi, lo);
        const dfx y = dfx_fma(diff, dfx_bcast(df2{fb.x, fb.y}), dfx_add(lo, dfx_bcast(df2{fb.z, fb.w})));
        int2 n;
        const dfx m = dfx_exp2(y, n, et.hi, et.lo);
        const float2 d = __ldg(dwl + s);
        const dfx slope = dfx_mul(diff, dfx_bcast(df2{d.x, d.y}));
        const bool nar_a = n.x > -100 && n.x < 100, nar_b = n.y > -100 && n.y < 100;
        if (nar_a && nar_b) {
          const dfx t = dfx_ldexp_normal(m, n);
          if (use_a) acc[s] = df_fma(gKa, dfx_get(t, 0), acc[s]);
          if (use_b) acc[s] = df_fma(gKb, dfx_get(t, 1), acc[s]);
          if (d.x != 0.0f) dk = dfx_fma(t, slope, dk);
        } else {
          // a term outside the float exponent range: the single-wavenumber steps per element
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            if (!(e ? use_b : use_a)) continue;
            const df2 me = dfx_get(m, e), se = dfx_get(slope, e), gKe = e ? gKb : gKa;
            const int ne = e ? n.y : n.x;
            if (ne > -100 && ne < 100) {
              const df2 t = df_ldexp(me, ne);
              acc[s] = df_fma(gKe, t, acc[s]);
              if (d.x != 0.0f) {
                const df2 dke = df_fma(t, se, dfx_get(dk, e));
                (e ? dk.hi.y : dk.hi.x) = dke.hi;
                (e ? dk.lo.y : dk.lo.x) = dke.lo;
              }
            } else {
              const double tw = df_to_double(me) * pow2d(ne);
              double& g64 = e ? gK64b : gK64a;
              if (g64 == 0.0) g64 = df_to_double(gKe);
              acc[s] = df_add(acc[s], df_from_double(g64 * tw));
              if (d.x != 0.0f) (e ? dkwb : dkwa) += tw * df_to_double(se);
            }
          }
        }
      }
    }
    // H- continuum: d log L / d (level coefficient c) = sum_k gK row_c (the rows after the
    // Rayleigh rows), accumulators S .. S + kHmTerms - 1
    if (a.hm_v0) {
#pragma unroll
      for (int j = 0; j < VP - 1; ++j) {  // compile-time accumulator index j = S + c
        if (j < S || j >= S + kHmTerms) continue;
        const float2* row = dm.rayleigh_df + (size_t)(dm.R_ray + j - S) * N;
        const float2 ra = __ldg(row + ka), rb = __ldg(row + kb);
        if (use_a) acc[j] = df_fma(gKa, df2{ra.x, ra.y}, acc[j]);
        if (use_b) acc[j] = df_fma(gKb, df2{rb.x, rb.y}, acc[j]);
      }
    }
    // opacity part of d log L / dT: gK d kappa / dT (level-table values are log2: d 2^y / dy = 2^y ln 2)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      if (!(e ? use_b : use_a)) continue;
      const df2 gKe = e ? gKb : gKa;
      acc[VP - 1] = df_add(acc[VP - 1], df_mul(gKe, df_mul(dfx_get(dk, e), df2{kLn2Hi, kLn2Lo})));
      const double dkw = e ? dkwb : dkwa;
      if (dkw != 0.0) acc[VP - 1] = df_add(acc[VP - 1], df_from_double(df_to_double(gKe) * dkw * 0.693147180559945309));
    }
  }
  const df2 r = warp_reduce_scatter<VP>(acc, lane);
  if (lane % G == 0) red[warp][lane / G] = df_to_double(r);
  __syncthreads();
  // value slot j < S: species j; S .. S + 6 with the H- continuum: its coefficients (values
  // hm_v0 ..); slot VP-1: temperature (value S of the partial sums)
  const bool hm_slot = a.hm_v0 && tid >= S && tid < S + kHmTerms;
  if (tid < VP && (tid < S || tid == VP - 1 || hm_slot)) {
    double sum = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) sum += red[w][tid];
    const int v = tid < S ? tid : hm_slot ? a.hm_v0 + tid - S : S;
    a.partial[(((size_t)b * L + l) * a.V + v) * a.tiles_total + a.tile0 + blockIdx.z] = sum;
  }
}

// ------------------------------------------------------------------ parameter tangents
// One block per evaluation. sg[L][V] = the partial sums reduced over the tiles;
// then thread th < P forms d log L / d param_th = sum over levels of the sinks
// times the tangents of ln n_s, T, lev.dz and lev.cloud along param_th
// (EmissionModel::calcAtmosphereStructure src/forward_model/emission/emission.cpp:158-189,
// Atmosphere::calcAltitude src/forward_model/atmosphere/atmosphere.cpp:288-307,
// GreyCloudModel src/cloud_model/grey_cloud_model.cpp:59-195,
// EmissionModel::radiusDistanceScaling emission.cpp:108-120).
__global__ void __launch_bounds__(kAdjThreads) atmosphere_adjoint_kernel(
    DeviceModel dm, const double* __restrict__ params, int P, const LevelInfo* __restrict__ lev,
    const EvalInfo* __restrict__ ev, const double* __restrict__ partial, int V, int tiles,
    const double* __restrict__ seed, double* __restrict__ grad) {
  extern __shared__ double sg[];
  const AtmosphereConfig& c = *dm.cfg;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int L = c.L, S = c.S;
  if (ev[b].neglect) return;
  const double inv = seed[b * 3 + 1];
  for (int idx = warp; idx < L * V; idx += nw) {
    const double* p = partial + ((size_t)b * L * V + idx) * tiles;
    double s = 0.0;
    for (int j = lane; j < tiles; j += 32) s += p[j];
    s = warp_sum_d(s);
    if (lane == 0) sg[idx] = s * inv;
  }
  __syncthreads();
  // thread (th, ch): parameter th, levels of chunk ch; chunk sums added in chunk order
  __shared__ double part[kAdjThreads];
  const int nch = max(1, (int)blockDim.x / P);
  const int th = tid % P, ch = tid / P;
  double acc = 0.0;
  if (ch < nch) {
    const double* par = params + (size_t)b * P;
    const double* gen = par;
    const int ng = c.nparam_general, nc = c.nparam_chem, nt = c.nparam_temp;
    const double* chem = par + ng;
    const double* temp = chem + nc;
    const double* cloud = temp + nt;

    double X[kSpeciesCount], dX[kSpeciesCount], mmw, dmmw;
    chemistry_tangent(c, chem, (th >= ng && th < ng + nc) ? th - ng : -1, X, dX, mmw, dmmw);
    // per opacity species: n_s = prod over the species and its collision partners of
    // n_total X_j, n_total = p / (k T): d ln n_s = sum_j dX_j / X_j - np_s dT / T
    double dlnX[kMaxTableSpecies];
    int np[kMaxTableSpecies];
    for (int s = 0; s < S; ++s) {
      const int js[3] = {c.sp_index[s], c.sp_partner[s][0], c.sp_partner[s][1]};
      double v = 0.0;
      int n = 0;
      bool zero = false;
      for (int u = 0; u < 3; ++u) {
        if (js[u] < 0) continue;
        ++n;
        if (X[js[u]] == 0.0) zero = true;
        else v += dX[js[u]] / X[js[u]];
      }
      dlnX[s] = v;
      np[s] = zero ? -1 : n;  // -1: zero density, the species contributes nothing
    }
    // temperature: T = poly(dof, log10 p), dof_i = temp_0 temp_1 ... temp_i (a constant profile: T = temp_0)
    const int tm = th - ng - nc;
    const bool temp_theta = tm >= 0 && tm < nt;
    double ddof[kMaxPolyDof];
    if (temp_theta && c.temp_poly) {
      for (int i = 0; i < c.pp_ndof; ++i) {
        double v = 0.0;
        if (i >= tm) {
          v = 1.0;
          for (int j = 0; j <= i; ++j)
            if (j != tm) v *= temp[j];
        }
        ddof[i] = v;
      }
    }
    auto dT_at = [&](int l) -> double {
      if (!temp_theta) return 0.0;
      return c.temp_poly ? poly_value(c, ddof, dm.log10p[l]) : (tm == 0 ? 1.0 : 0.0);
    };
    const double g = pow(10.0, gen[0]);
    const double dlng = th == 0 ? kLn10 : 0.0;  // d ln g / d log g
    const int ci = ng + nc + nt;                 // cloud optical depth parameter
    const EvalInfo e = ev[b];
    double cloud_d = 0.0;
    if (c.cloud && th == ci && cloud[0] >= 0)
      cloud_d = 1.0 / (double)((unsigned)e.cloud_top - (unsigned)e.cloud_bottom);
    // u = R T / (mmw p 1e6) = 1 / rho and its tangent
    auto u_at = [&](int l, double& du) {
      const double T = lev[(size_t)b * L + l].T;
      const double u = kGasConst * T / (mmw * dm.pressure[l] * 1e6);
      du = u * (dT_at(l) / T - dmmw / mmw);
      return u;
    };
    const int l0 = ch * L / nch, l1 = (ch + 1) * L / nch;
    double du_prev = 0.0, u_prev = l0 >= 1 ? u_at(l0 - 1, du_prev) : 0.0;
    for (int l = l0; l < l1; ++l) {
      const double T = lev[(size_t)b * L + l].T;
      const double dT = dT_at(l);
      const double dlnT = dT / T;
      const double* sgl = sg + (size_t)l * V;
      for (int s = 0; s < S; ++s)
        if (np[s] >= 0) acc = fma(sgl[s], dlnX[s] - np[s] * dlnT, acc);
      acc = fma(sgl[S], dT, acc);
      if (c.hm) {
        // H- continuum coefficients (atmosphere_kernel): h_0 = n(H-), h_i = (5040/T)^((i+1)/2)
        // n(e-) k T n(H) for i >= 1 (zero, and held there, when n(H-) = 0); n_j = X_j p / (k T)
        const double* sh = sgl + S + 3 + (c.cloud_kind == 1 ? 1 : c.cloud_kind == 2 ? 3 : 0);
        const double nt = dm.pressure[l] * 1.e6 / kBoltzmann / T, dnt = -nt * dlnT;
        const double nHm = X[SP_Hm] * nt, ne = X[SP_e] * nt, nH = X[SP_H] * nt;
        const double dnHm = dX[SP_Hm] * nt + X[SP_Hm] * dnt;
        const double dne = dX[SP_e] * nt + X[SP_e] * dnt, dnH = dX[SP_H] * nt + X[SP_H] * dnt;
        acc = fma(sh[0], dnHm, acc);
        if (nHm != 0.0)
          for (int i = 1; i < kHmTerms; ++i) {
            const double ex = (i + 1) / 2.0;
            const double f = pow(5040.0 / T, ex);
            const double dh = kBoltzmann * (f * (dne * T * nH + ne * dT * nH + ne * T * dnH) - ex * f * dlnT * ne * T * nH);
            acc = fma(sh[i], dh, acc);
          }
      }
      // layer thickness Delta_l = 0.5 (p_{l-1} - p_l) 1e6 (u_l + u_{l-1}) / g (lev[l-1].dz)
      const double u = kGasConst * T / (mmw * dm.pressure[l] * 1e6);
      const double du = u * (dlnT - dmmw / mmw);
      if (l >= 1) {
        const double pf = 0.5 * (dm.pressure[l - 1] * 1e6 - dm.pressure[l] * 1e6) / g;
        acc = fma(sg[(size_t)(l - 1) * V + S + 1], pf * ((du + du_prev) - (u + u_prev) * dlng), acc);
      }
      u_prev = u;
      du_prev = du;
      // grey cloud: tau_c / (top - bottom) on layers bottom < l <= top, l < L - 1
      if (cloud_d != 0.0 && (unsigned)l <= (unsigned)e.cloud_top && (unsigned)l > (unsigned)e.cloud_bottom &&
          l < L - 1)
        acc = fma(sgl[S + 2], cloud_d, acc);
    }
    // non-grey cloud shape parameters (after the optical depth): value S + 3 + c of level 0
    if (ch == 0 && c.cloud && c.cloud_kind) {
      const int cs = th - ci - 1;
      if (cs >= 0 && cs < (c.cloud_kind == 1 ? 1 : 3)) acc += sg[S + 3 + cs];
    }
    // radius-distance scaling (R_J / d)^2 f, once (chunk 0); the secondary eclipse has
    // none (its R_p / R_s and stellar derivatives come from the likelihood adjoint)
    if (ch == 0 && dm.star_model == 0) {
      const double gsc = seed[b * 3 + 2] / e.scaling;
      if (th == 1) acc += gsc * (kRJupiter / gen[2]) * (kRJupiter / gen[2]);
      if (th == 2) acc += gsc * (-2.0 * e.scaling / gen[2]);
    }
  }
  part[tid] = acc;
  __syncthreads();
  if (tid < P) {
    double tot = 0.0;
    for (int q = 0; q < nch; ++q) tot += part[q * P + tid];
    grad[(size_t)b * P + tid] += tot;
  }
}

// ------------------------------------------------------------------ host side
void free_grad_workspace(Model& m) {
  GradWorkspace& g = m.gws;
  cudaFree(g.taps.dwT);
  cudaFree(g.taps.istore);
  cudaFree(g.taps.em_layer);
  cudaFree(g.em_gK);
  cudaFree(g.gS);
  cudaFree(g.seed);
  cudaFree(g.partial);
  cudaFree(g.taps.tr_geo);
  cudaFree(g.taps.tr_c);
  cudaFree(g.taps.tr_T);
  cudaFree(g.taps.tr_qs);
  cudaFree(g.taps.tr_us);
  cudaFree(g.taps.tr_I);
  cudaFree(g.taps.tr_ts);
  cudaFree(g.taps.tr_dk);
  cudaFree(g.tr_gc);
  cudaFree(g.tr_gz);
  cudaFree(g.tr_rp);
  cudaFree(g.tr_cs);
  cudaFree(g.taps.tr_d);
  cudaFree(g.tr_gd);
  g = GradWorkspace{};
}

namespace {

int value_slots(int V) { return V <= 8 ? 8 : V <= 16 ? 16 : 32; }

size_t adjoint_smem(const Model& m) { return (size_t)2 * m.acfg.S * kAdjThreads * (sizeof(float2) + sizeof(double)); }

// split: the double-float path's per-(level, wavenumber) layer data and d log L / d kappa
size_t grad_bytes_per_eval(const Model& m, int tiles, int V, bool split) {
  const size_t L = m.L, N = m.N, S = std::max(m.acfg.S, 1), M = std::max(m.M, 1);
  return L * 2 * N * 8 + L * S * sizeof(float2) + M * 8 + 3 * 8 + L * (size_t)V * tiles * 8 +
         (split ? L * N * (sizeof(float4) + sizeof(float2)) : 0);
}

void ensure_grad_workspace(Model& m, int chunk, int tiles, int V, bool split) {
  GradWorkspace& g = m.gws;
  if (chunk <= g.capacity && tiles == g.tiles && (!split || g.em_gK)) return;
  BGB_CUDA(cudaDeviceSynchronize());
  free_grad_workspace(m);
  const size_t B = chunk, L = m.L, N = m.N, S = std::max(m.acfg.S, 1), M = std::max(m.M, 1);
  BGB_CUDA(cudaMalloc(&g.taps.dwT, B * L * S * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.taps.istore, B * L * 2 * N * sizeof(double)));
  if (split) {
    BGB_CUDA(cudaMalloc(&g.taps.em_layer, B * L * N * sizeof(float4)));
    BGB_CUDA(cudaMalloc(&g.em_gK, B * L * N * sizeof(float2)));
  }
  BGB_CUDA(cudaMalloc(&g.gS, B * M * sizeof(double)));
  BGB_CUDA(cudaMalloc(&g.seed, B * 3 * sizeof(double)));
  BGB_CUDA(cudaMalloc(&g.partial, B * L * (size_t)V * tiles * sizeof(double)));
  g.capacity = chunk;
  g.tiles = tiles;
}

template <bool DF, int VP>
void launch_emission_adjoint(const Model& m, dim3 grid, size_t smem, cudaStream_t st, const AdjointArgs& a) {
  if (smem > 48 * 1024)
    BGB_CUDA(cudaFuncSetAttribute(emission_adjoint_kernel<DF, VP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  emission_adjoint_kernel<DF, VP><<<grid, kAdjThreads, smem, st>>>(m.dm, a);
}

}  // namespace

// adjoint_transmission.cu
size_t transmission_grad_bytes_per_eval(const Model& m, int V, bool store);
void alloc_transmission_grad(Model& m, int chunk, int V, bool store);
void transmission_adjoint_chunk(Model& m, const double* params_chunk, int nb, cudaStream_t st, double* grad_chunk,
                                int V);

static void launch_gradient_transmission(Model& m, const double* params_dev, int batch, cudaStream_t st,
                                         double* loglike_dev, double* grad_dev, uint8_t* neglect_dev) {
  if (m.precision != 0) throw Error(BEAR_ERR_UNSUPPORTED, "the transmission gradient runs in precision mode 0");
  const int S = m.acfg.S, R = m.acfg.R, L = m.L, P = m.acfg.nparam_total;
  // level values: species, Rayleigh / H- terms, temperature, altitude, cloud extinction, then
  // the sums along the non-grey cloud's shape parameters
  const int NC = m.acfg.cloud_kind == 1 ? 1 : m.acfg.cloud_kind == 2 ? 3 : 0;
  const int V = S + R + 3 + NC;
  if (V > 32) throw Error(BEAR_ERR_UNSUPPORTED, "the gradient supports at most 29 table and Rayleigh species");
  if (P > 128) throw Error(BEAR_ERR_UNSUPPORTED, "the gradient supports at most 128 parameters");
  if (L > 32767) throw Error(BEAR_ERR_UNSUPPORTED, "too many levels");
  const size_t S1 = std::max(S, 1), M = std::max(m.M, 1);
  // the forward pass stores the opacity terms for the adjoint when chunks of at least
  // min(batch, 8) evaluations still fit the memory budget; else the adjoint recomputes them
  const size_t extra = L * S1 * sizeof(float2) + M * 8 + 3 * 8;
  const size_t per_store = transmission_grad_bytes_per_eval(m, V, true) + extra;
  // (with A > 1 impact parameters per layer the adjoint always recomputes them)
  const bool store = m.annuli <= 1 && m.grad_budget / per_store >= std::min<size_t>((size_t)batch, 8);
  const size_t per_eval = store ? per_store : transmission_grad_bytes_per_eval(m, V, false) + extra;
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)batch, m.grad_budget / per_eval));
  BGB_CUDA(cudaSetDevice(m.device));
  ensure_workspace(m, chunk);
  GradWorkspace& g = m.gws;
  if (chunk > g.capacity || g.tiles != -1 || g.tr_store != store) {
    BGB_CUDA(cudaDeviceSynchronize());
    free_grad_workspace(m);
    BGB_CUDA(cudaMalloc(&g.taps.dwT, (size_t)chunk * L * S1 * sizeof(float2)));
    BGB_CUDA(cudaMalloc(&g.gS, (size_t)chunk * M * sizeof(double)));
    BGB_CUDA(cudaMalloc(&g.seed, (size_t)chunk * 3 * sizeof(double)));
    alloc_transmission_grad(m, chunk, V, store);
    g.capacity = chunk;
    g.tiles = -1;  // transmission layout
  }
  const Workspace& w = m.ws;
  for (int c0 = 0; c0 < batch; c0 += chunk) {
    const int nb = std::min(chunk, batch - c0);
    const double* pc = params_dev + (size_t)c0 * P;
    double* gc = grad_dev + (size_t)c0 * P;
    launch_forward_taps(m, pc, nb, st, neglect_dev ? neglect_dev + c0 : nullptr, loglike_dev + c0, g.taps);
    obs_adjoint_kernel<<<nb, 256, 0, st>>>(m.dm, pc, P, w.ev, w.obs, g.gS, g.seed, gc, 1);
    BGB_CUDA(cudaGetLastError());
    transmission_adjoint_chunk(m, pc, nb, st, gc, V);
  }
}

void launch_gradient(Model& m, const double* params_dev, int batch, cudaStream_t st, double* loglike_dev,
                     double* grad_dev, uint8_t* neglect_dev) {
  if (m.hm && m.precision != 0) throw Error(BEAR_ERR_UNSUPPORTED, "H- continuum gradients run in precision mode 0");
  if (m.acfg.cloud_kind && m.precision != 0)
    throw Error(BEAR_ERR_UNSUPPORTED, "power-law and KH cloud gradients run in precision mode 0");
  if (m.transmission) {
    launch_gradient_transmission(m, params_dev, batch, st, loglike_dev, grad_dev, neglect_dev);
    return;
  }
  const int S = m.acfg.S, L = m.L, P = m.acfg.nparam_total;
  // level values: species, temperature, layer thickness, cloud, then (level 0 only) the
  // derivatives along the non-grey cloud's shape parameters
  const int NC = m.acfg.cloud_kind == 1 ? 1 : m.acfg.cloud_kind == 2 ? 3 : 0;
  const int V = S + 3 + NC + (m.hm ? kHmTerms : 0);  // the H- coefficients last
  if (V > 32) throw Error(BEAR_ERR_UNSUPPORTED, "the gradient supports at most 29 table species");
  if (P > kAdjThreads) throw Error(BEAR_ERR_UNSUPPORTED, "the gradient supports at most 128 parameters");
  const bool df = m.precision == 0;
  // tile slots of the partial sums: the fused kernel's (128 wavenumbers each) or the sweep
  // kernel's (256 wavenumbers each), then
  // in the double-float path the sink kernel's (kSinkKPT x 128 wavenumbers each)
  const int tiles_a = (int)((m.N + (df ? 2 : 1) * kAdjThreads - 1) / ((df ? 2 : 1) * kAdjThreads));
  const int tiles_b = df ? (int)((m.N + kSinkKPT * kAdjThreads - 1) / (kSinkKPT * kAdjThreads)) : 0;
  const int tiles = tiles_a + tiles_b;
  const size_t per_eval = grad_bytes_per_eval(m, tiles, V, df);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)batch, m.grad_budget / per_eval));
  BGB_CUDA(cudaSetDevice(m.device));
  ensure_workspace(m, chunk);
  ensure_grad_workspace(m, chunk, tiles, V, df);
  const GradWorkspace& g = m.gws;
  const Workspace& w = m.ws;
  const size_t smem = adjoint_smem(m);
  const size_t smem_atm = (size_t)L * V * sizeof(double);
  if (smem > 227 * 1024 || smem_atm > 227 * 1024)
    throw Error(BEAR_ERR_UNSUPPORTED, "model too large for the adjoint kernels' shared memory");
  if (smem_atm > 48 * 1024)
    BGB_CUDA(cudaFuncSetAttribute(atmosphere_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_atm));
  const int VP = value_slots(V);
  const int VPB = value_slots(S + 1 + (m.hm ? kHmTerms : 0));
  for (int c0 = 0; c0 < batch; c0 += chunk) {
    const int nb = std::min(chunk, batch - c0);
    const double* pc = params_dev + (size_t)c0 * P;
    double* gc = grad_dev + (size_t)c0 * P;
    launch_forward_taps(m, pc, nb, st, neglect_dev ? neglect_dev + c0 : nullptr, loglike_dev + c0, g.taps);
    obs_adjoint_kernel<<<nb, 256, 0, st>>>(m.dm, pc, P, w.ev, w.obs, g.gS, g.seed, gc, 0);
    BGB_CUDA(cudaGetLastError());
    AdjointArgs a{w.lev, w.ls, w.lsdf, w.ev, g.taps.dwT, g.taps.istore, g.gS, g.seed, g.partial, V};
    const dim3 grid(nb, tiles_a);
    if (df) {
      BGB_CUDA(cudaMemsetAsync(g.partial, 0, (size_t)nb * L * V * tiles * sizeof(double), st));
      SweepArgs sa{w.lev, w.ev, g.taps.istore, g.taps.em_layer, g.gS, g.seed, g.em_gK, g.partial, V, tiles};
      if (m.acfg.cloud_kind) emission_adjoint_sweep_kernel<true><<<grid, kAdjThreads, 0, st>>>(m.dm, sa);
      else emission_adjoint_sweep_kernel<false><<<grid, kAdjThreads, 0, st>>>(m.dm, sa);
      BGB_CUDA(cudaGetLastError());
      if (S > 0) {
        SinkArgs ka{w.lsdf, g.taps.dwT, g.em_gK, g.partial, V, tiles, tiles_a, m.hm ? S + 3 + NC : 0};
        const dim3 gridb(nb, L, tiles_b);
        if (VPB == 8) emission_adjoint_sinks_kernel<8><<<gridb, kAdjThreads, 0, st>>>(m.dm, ka);
        else if (VPB == 16) emission_adjoint_sinks_kernel<16><<<gridb, kAdjThreads, 0, st>>>(m.dm, ka);
        else emission_adjoint_sinks_kernel<32><<<gridb, kAdjThreads, 0, st>>>(m.dm, ka);
      }
    } else {
      if (VP == 8) launch_emission_adjoint<false, 8>(m, grid, smem, st, a);
      else if (VP == 16) launch_emission_adjoint<false, 16>(m, grid, smem, st, a);
      else launch_emission_adjoint<false, 32>(m, grid, smem, st, a);
    }
    BGB_CUDA(cudaGetLastError());
    atmosphere_adjoint_kernel<<<nb, kAdjThreads, smem_atm, st>>>(m.dm, pc, P, w.lev, w.ev, g.partial, V, tiles,
                                                                 g.seed, gc);
    BGB_CUDA(cudaGetLastError());
  }
}

}  // namespace bgb
