// Adjoint (reverse-mode) gradient of the log-likelihood of transmission models.
//
// Forward model per evaluation and wavenumber (TransmissionModel
// src/forward_model/transmission/transmission_spectrum.cpp:32-154):
//   chi_l  = kappa_l + sum_r sigma_r n_{r,l} + cloud_l            extinction
//   c_i    = chi_i + chi_{i+1}
//   tau_t  = sum_{i=t}^{I_t} G[t][i] c_i                            (I_t: the tau > 10 cut-off)
//   T_t    = exp(-tau_t),  h = sum_t (R + z_t)(1 - T_t) wz_t,  wz_t = z_{t+1} - z_{t-1} (z_1 - z_0 at t = 0)
//   depth  = (h + R^2) / R_s^2 1e6
// with G[t][i] = S_t(i+1) - S_t(i), S_t(j) = sqrt((R + z_j)^2 - (R + z_t)^2) (S_t(t) = 0).
//
// Kernel chain for one chunk of evaluations (the likelihood adjoint and the seed
// normaliser come from adjoint.cu):
//   tr_geometry_adjoint_kernel  per evaluation, before the forward radiative transfer:
//                               P[t][j] = dG[t][j-1]/dz_j = (R + z_j)/S_t(j) (stored as
//                               [j][t]), Q[t][i] = dG[t][i]/dz_t and the path lengths G
//                               transposed ([j][t]) for pass 2a
//   transmission_kernel<STORE>  (engine.cu) the forward pass itself also stores, per (level,
//                               wavenumber), the ray transmission T_t, the cut-off index, the
//                               pair sums c and the ray sum of c dG/dz_t
//   tr_adjoint_pass2a           per (level j, wavenumber), g_tau_t = d log L / d tau_t and the
//                               cut-off indices staged in shared memory: d log L / d c_j =
//                               sum_t g_tau_t G[t][j], d log L / d z_j (geometry and effective
//                               height) and d log L / dR
//   tr_adjoint_pass2b           per (evaluation, level), threads striding the wavenumbers: the
//                               level sinks (log number densities of the table and Rayleigh
//                               species, temperature, altitude, cloud extinction) from the stored
//                               or recomputed opacity terms, one block reduction per level
//   tr_atmosphere_adjoint_kernel per evaluation: the level sinks, forward-mode
//                               tangents of the level physics (temperature, chemistry,
//                               hydrostatic altitudes as prefix sums, cloud extinction),
//                               planet and star radii
// Double-float arithmetic on the FP32 pipe throughout except the effective-height
// terms and the per-evaluation tangents (FP64); the ray transmissions T_t are the
// forward pass's double-float values.
// Discrete decisions (table brackets, cut-off index, cloud layers) are held fixed.

#include <algorithm>
#include <cmath>
#include <string>

#include "adjoint_common.cuh"
#include "bulk_copy.cuh"
#include "dfloat2x.cuh"

namespace bgb {


// d log L / d depth_k normalised (the seed): sum_r W_rk gS_r times the evaluation's normaliser
__device__ __forceinline__ double tr_seed(const DeviceModel& dm, const double* __restrict__ gS,
                                          const double* __restrict__ seed, int b, int k) {
  const double* g = gS + (size_t)b * dm.M;
  double gF = 0.0;
  const int e1 = __ldg(&dm.col_ptr[k + 1]);
  for (int e = __ldg(&dm.col_ptr[k]); e < e1; ++e) gF = fma(__ldg(&dm.col_w[e]), g[__ldg(&dm.col_row[e])], gF);
  return gF * seed[b * 3];
}

// ------------------------------------------------------------------ geometry derivatives
__global__ void tr_geometry_adjoint_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                           const EvalInfo* __restrict__ ev, const float2* __restrict__ geom,
                                           float2* __restrict__ geo) {
  const int b = blockIdx.x, L = dm.L;
  const LevelInfo* lv = lev + (size_t)b * L;
  const double R = ev[b].radius;
  float2* PT = geo + (size_t)b * 3 * L * L;  // [j][t]: P transposed, for the per-level sums of pass 2a
  float2* Q = PT + (size_t)L * L;
  float2* GT = Q + (size_t)L * L;            // [j][t]: the forward path lengths G transposed
  const float2* G = geom + (size_t)b * L * L;
  // 1 / S_t(j) for j > t (0 for j <= t or a degenerate zero path)
  auto rS = [&](int t, int j) -> double {
    if (j <= t) return 0.0;
    const double bt = R + lv[t].z, a = R + lv[j].z;
    const double s = sqrt(__dsub_rn(__dmul_rn(a, a), __dmul_rn(bt, bt)));
    return s > 0.0 ? 1.0 / s : 0.0;
  };
  auto put = [](float2* p, double v) {
    const df2 d = df_from_double(v);
    *p = make_float2(d.hi, d.lo);
  };
  // grid: evaluations x blocks of elements
  for (int idx = blockIdx.y * blockDim.x + threadIdx.x; idx < L * L; idx += gridDim.y * blockDim.x) {
    const int t = idx / L, i = idx % L;
    const double zt = lv[t].z;
    put(PT + (size_t)i * L + t, (R + lv[i].z) * rS(t, i));
    GT[(size_t)i * L + t] = __ldg(&G[idx]);
    double q = 0.0;
    if (i >= t && i < L - 1) q = (R + zt) * (rS(t, i) - rS(t, i + 1));
    put(Q + idx, q);
  }
}

// With A impact parameters per layer (ray k = t A + jj of layer t, impact radius
// b_k = R + zb_k, zb_k = z_t + (z_{t+1} - z_t) jj / A, path lengths G_k[i] = s_{i+1} - s_i,
// s_i = sqrt((R + z_i)^2 - b_k^2), the first segment G_k[t] = s_{t+1}): per evaluation
//   PT[j][k] = ds_j / dz_j = (R + z_j) / s_j  (j > t, else 0)
//   GT[j][k] = G_k[j]                          (t <= j <= L - 2, else 0)
//   Q[t][i][jj] = dG_k[i] / db_k = b_k (1 / s_i [i > t] - 1 / s_{i+1})   (the forward's layout)
__global__ void tr_geometry_adjoint_annuli_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                  const EvalInfo* __restrict__ ev, const float2* __restrict__ geom,
                                                  const double* __restrict__ rays, float2* __restrict__ geo) {
  const int b = blockIdx.x, L = dm.L, A = dm.annuli, K = (L - 1) * A;
  const LevelInfo* lv = lev + (size_t)b * L;
  const double R = ev[b].radius;
  const double* zb = rays + (size_t)b * 2 * (K + 1);
  float2* PT = geo + (size_t)b * 3 * L * K;
  float2* GT = PT + (size_t)L * K;
  float2* Q = GT + (size_t)L * K;
  const float2* G = geom + (size_t)b * (L - 1) * L * A;
  auto put = [](float2* p, double v) {
    const df2 d = df_from_double(v);
    *p = make_float2(d.hi, d.lo);
  };
  for (size_t idx = (size_t)blockIdx.y * blockDim.x + threadIdx.x; idx < (size_t)K * L;
       idx += (size_t)gridDim.y * blockDim.x) {
    const int kr = (int)(idx / L), i = (int)(idx % L);
    const int t = kr / A, jj = kr - t * A;
    const double bt = R + zb[kr], bb = __dmul_rn(bt, bt);
    auto rS = [&](int j) -> double {  // 1 / s_j (0 at and below the tangent layer's base)
      if (j <= t) return 0.0;
      const double a = R + lv[j].z;
      const double sj = sqrt(__dsub_rn(__dmul_rn(a, a), bb));
      return sj > 0.0 ? 1.0 / sj : 0.0;
    };
    put(PT + (size_t)i * K + kr, i > t ? (R + lv[i].z) * rS(i) : 0.0);
    const size_t at = ((size_t)t * L + i) * A + jj;
    const bool seg = i >= t && i < L - 1;
    GT[(size_t)i * K + kr] = seg ? G[at] : make_float2(0.0f, 0.0f);
    put(Q + at, seg ? bt * (rS(i) - rS(i + 1)) : 0.0);
  }
}

// ------------------------------------------------------------------ pass 2a
struct TrArgs {
  const LevelInfo* lev;
  const LevelSpeciesDF* lsdf;
  const double* ray_n;
  const EvalInfo* ev;
  const float2* geom;
  const float2* geo;
  const float2* dwT;
  const double* gS;
  const double* seed;
  const float2* c;
  float2* T;  // ray transmissions (rewritten in place with d log L / d tau by the annuli pass 2a)
  float2* qs;  // read, then overwritten with the direct altitude sink z1_t
  float2* us;  // written with A_t = (R + z_t)(1 - T_t)
  const short* I;
  float2* gc;
  float2* gz;
  double* rp;
  double* partial;
  int V;
  const float2* ts;  // stored opacity terms (nullptr: recompute them)
  const float2* dk;  // stored temperature-slope sums
  const double* cs;  // non-grey cloud: per evaluation the wavelength factor and its NC shape derivatives
  int nc;            // NC (0: grey cloud or none)
  // A > 1 impact parameters per layer: the rays' altitudes and weights (the forward
  // geometry's), the extinction differences and d log L / d of them
  const double* rays = nullptr;
  const float2* d = nullptr;
  float2* gd = nullptr;
};

// The cloud values of level l at wavenumber k from g_x = d log L / d chi_l: value q0 = 0 (the
// cloud extinction) is g_x times the wavelength factor of a non-grey cloud (g_x itself for
// the grey one), values q0 = 1 .. NC the sums along the shape parameters,
// g_x cloud_l df_k / dtheta (cloud_l the level's grey-part cloud extinction).
__device__ __forceinline__ df2 tr_cloud_value(const TrArgs& a, int q0, int b, size_t N, int k, df2 gx,
                                              double cloud_l) {
  if (!a.cs) return q0 == 0 ? gx : df2{0.0f, 0.0f};
  const double* row = a.cs + (size_t)b * (1 + a.nc) * N + (size_t)q0 * N + k;
  if (q0 == 0) return df_mul(gx, df_from_double(__ldg(row)));
  return df_from_double(df_to_double(gx) * cloud_l * __ldg(row));
}

// The wavelength factor of the evaluation's non-grey cloud and its derivatives along the
// shape parameters at every wavenumber (the forward pass's cloud_shape, FP64).
__global__ void tr_cloud_shape_kernel(DeviceModel dm, const EvalInfo* __restrict__ ev, double* __restrict__ cs,
                                      int nc) {
  const int b = blockIdx.x, k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= dm.N) return;
  const size_t N = dm.N;
  double* row = cs + (size_t)b * (1 + nc) * N;
  row[k] = cloud_shape(dm, ev[b], k);
  double d[3];
  cloud_shape_tangent(dm, ev[b], k, d);
  for (int c = 0; c < nc; ++c) row[(size_t)(1 + c) * N + k] = d[c];
}

// Block: 32 wavenumbers (lanes) x 4 groups; group w takes levels j = w, w+4, ...
// From the forward pass's stores, with g_h = d log L / dh (the normalised seed times
// 1e6 / R_s^2) and F_t = (R + z_t) wz_t:
//   g_tau_t = g_h F_t T_t                 staged with the cut-off indices in shared
//                                          memory (float2 [L][32] then short [L][32]; 24
//                                          warps per SM at 100 levels: 14.8 -> ~12.5 ms at
//                                          B = 64 once m(j) no longer took a third array)
//   g_c_j   = sum_{t <= j <= I_t} g_tau_t G[t][j]                      (j <= L-2)
//   g_z_j   = sum_{t < j} g_tau_t P[t][j] (c_{j-1} [j-1 <= I_t] - c_j [j <= I_t])
//           + g_h (1 - T_j) wz_j + g_tau_j qs_j + g_h (A_{j-1} - A_{j+1}) (- A_0 at j = 0),
//             A_t = (R + z_t)(1 - T_t)   (wz_t = z_{t+1} - z_{t-1}; z_1 - z_0 at t = 0)
//   dlogL/dR = sum_j g_z_j + 2 R g_h (depth = (h + R^2) / R_s^2): every radius in the path
//             lengths and the effective-height weights is R + z_j, so their derivative along R
//             is the sum of their derivatives along the z_j
// Two wavenumbers per lane (k and k + 32 of a 64-wavenumber tile) with paired FP32
// double-float instructions (dfloat2x.cuh), eight groups of levels: every per-element step is
// the one-wavenumber step, and a ray that does not reach level j (or a sum it does not enter)
// contributes a zeroed g_tau, which leaves a double-float sum unchanged, so each wavenumber's
// g_c and g_z equal the one-wavenumber results.
constexpr int kPass2aGroups = 8;

__global__ void __launch_bounds__(32 * kPass2aGroups, 3) tr_adjoint_pass2a(DeviceModel dm, TrArgs a) {
  constexpr int NG = kPass2aGroups;
  extern __shared__ __align__(16) unsigned char tr2a_smem[];
  __shared__ float2 rp_part[32 * NG];
  const int L = dm.L;
  float4* gt_s = reinterpret_cast<float4*>(tr2a_smem);                // [L][32] paired g_tau
  float2* fz_s = reinterpret_cast<float2*>(gt_s + (size_t)L * 32);     // [L]: R + z_t
  float2* fw_s = fz_s + L;                                             // [L]: wz_t
  float2* ff_s = fw_s + L;                                             // [L]: (R + z_t) wz_t
  short2* I_s = reinterpret_cast<short2*>(ff_s + L);                   // [L][32] paired cut-off indices
  // grid (tiles, evaluations): the blocks an SM runs together mostly share one evaluation, so
  // its path-length rows stay in L1
  const int b = blockIdx.y, lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
  const int kk0 = blockIdx.x * 64 + lane, kk1 = kk0 + 32;
  const bool act0 = kk0 < dm.N, act1 = kk1 < dm.N;
  const int k0 = act0 ? kk0 : dm.N - 1, k1 = act1 ? kk1 : dm.N - 1;
  const size_t N = dm.N;
  const size_t col0 = (size_t)b * L * N + k0, col1 = (size_t)b * L * N + k1;
  const LevelInfo* lv = a.lev + (size_t)b * L;
  const double Rp = a.ev[b].radius, Rs = a.ev[b].star_radius;
  // per-level geometry factors of the effective height (FP64 once per block)
  for (int t = threadIdx.x; t < L - 1; t += blockDim.x) {
    const double zt = __ldg(&lv[t].z);
    const double wz = (__ldg(&lv[t + 1].z) - zt) + (t >= 1 ? zt - __ldg(&lv[t - 1].z) : 0.0);
    const df2 z = df_from_double(Rp + zt), w = df_from_double(wz), f = df_from_double((Rp + zt) * wz);
    fz_s[t] = make_float2(z.hi, z.lo);
    fw_s[t] = make_float2(w.hi, w.lo);
    ff_s[t] = make_float2(f.hi, f.lo);
  }
  __syncthreads();
  const dfx gh = dfx_make(df_from_double(act0 ? tr_seed(dm, a.gS, a.seed, b, k0) * 1e6 / (Rs * Rs) : 0.0),
                          df_from_double(act1 ? tr_seed(dm, a.gS, a.seed, b, k1) * 1e6 / (Rs * Rs) : 0.0));
  const dfx zx = {f2(0.0f), f2(0.0f)};
  const dfx one = dfx_bcast(df_make(1.0f));
  // both elements of a per-(level, wavenumber) array at level t
  auto ld = [&](const float2* arr, int t) {
    const float2 v0 = arr[col0 + (size_t)t * N], v1 = arr[col1 + (size_t)t * N];
    return dfx{make_float2(v0.x, v1.x), make_float2(v0.y, v1.y)};
  };
  auto st = [&](float2* arr, int t, const dfx& v) {
    if (act0) arr[col0 + (size_t)t * N] = make_float2(v.hi.x, v.lo.x);
    if (act1) arr[col1 + (size_t)t * N] = make_float2(v.hi.y, v.lo.y);
  };
  auto sm = [](const float2* arr, int i) {
    const float2 v = arr[i];
    return dfx_bcast(df2{v.x, v.y});
  };
  // per tangent level: g_tau_t = g_h F_t T_t (staged), A_t = (R + z_t)(1 - T_t) and the direct
  // sink z1_t = g_h (1 - T_t) wz_t + g_tau_t qs_t, written over the ray sum qs_t and into a.us
  dfx rp = zx;
  for (int t = grp; t < L - 1; t += NG) {
    const dfx T = ld(a.T, t), omT = dfx_sub(one, T);
    const dfx gt = dfx_mul(dfx_mul(gh, sm(ff_s, t)), T);
    const dfx base = dfx_mul(dfx_mul(gh, omT), sm(fw_s, t));
    const dfx z1 = dfx_add(base, dfx_mul(gt, ld(a.qs, t)));
    const dfx A = dfx_mul(sm(fz_s, t), omT);
    gt_s[t * 32 + lane] = make_float4(gt.hi.x, gt.hi.y, gt.lo.x, gt.lo.y);
    I_s[t * 32 + lane] = make_short2(a.I[col0 + (size_t)t * N], a.I[col1 + (size_t)t * N]);
    st(a.qs, t, z1);
    st(a.us, t, A);
  }
  if (grp == 0) rp = dfx_add(rp, dfx_mul(gh, dfx_bcast(df_from_double(2.0 * Rp))));  // depth = (h + R^2) / R_s^2
  __syncthreads();
  if (act0) {
    // m(j): the lowest tangent level whose ray reaches level j. Ray t covers levels
    // t..I_t + 1 (I_t >= t), so in ascending t the covered levels form a growing prefix
    // (reaching L - 1 at t = L - 2 at the latest); m(j) is the t whose ray first extends it
    // to j, found per element while the thread's levels j ascend
    int tp0 = 0, cov0 = -1, m0 = 0, tp1 = 0, cov1 = -1, m1 = 0;
    // per level j the rays' path lengths G[t][j] and P[t][j], contiguous in t
    const float2* PT = a.geo + (size_t)b * 3 * L * L;
    const float2* GT = PT + (size_t)2 * L * L;
    for (int j = grp; j < L; j += NG) {
      const dfx cj1 = j >= 1 ? ld(a.c, j - 1) : zx;
      const dfx cj = j <= L - 2 ? ld(a.c, j) : zx;
      const dfx dcc = dfx_sub(cj1, cj);
      // g_z part: sum over rays through j of g_tau P (x dcc), over rays ending at j - 1 (x c_{j-1})
      dfx gc = zx, pin = zx, pend = zx;
      const int tmax = min(j, L - 2);
      while (cov0 < j && tp0 <= L - 2) {
        cov0 = max(cov0, min((int)I_s[tp0 * 32 + lane].x + 1, L - 1));
        m0 = tp0++;
      }
      while (cov1 < j && tp1 <= L - 2) {
        cov1 = max(cov1, min((int)I_s[tp1 * 32 + lane].y + 1, L - 1));
        m1 = tp1++;
      }
      // from the lowest m(j) of the warp's wavenumbers, so the path-length loads stay uniform
      const unsigned mask = __activemask();
      const int t0 = (int)__reduce_min_sync(mask, (unsigned)min(m0, m1));
      auto ray = [&](int t, short2 I, float2 g, float2 p, float4 q) {
        // per element: the ray of tangent level t reaches level j (I >= j - 1); it passes
        // through j (sum g_c and P "in") or ends at j - 1 (P "end")
        const bool r0 = I.x >= j - 1, r1 = I.y >= j - 1;
        const bool in0 = r0 && I.x >= j && j <= L - 2, in1 = r1 && I.y >= j && j <= L - 2;
        const dfx gtau = {make_float2(q.x, q.y), make_float2(q.z, q.w)};
        if (in0 || in1) gc = dfx_fma(dfx_select(in0, in1, gtau, zx), dfx_bcast(df2{g.x, g.y}), gc);
        if (t < j) {
          const bool e0 = r0 && !in0, e1 = r1 && !in1;
          const dfx pp = dfx_bcast(df2{p.x, p.y});
          if (in0 || in1) pin = dfx_fma(dfx_select(in0, in1, gtau, zx), pp, pin);
          if (e0 || e1) pend = dfx_fma(dfx_select(e0, e1, gtau, zx), pp, pend);
        }
      };
      const float2* Gj = GT + (size_t)j * L;
      const float2* Pj = PT + (size_t)j * L;
      int t = t0;
      // two rays per step, their loads issued together (same sums, same order)
      for (; t + 1 <= tmax; t += 2) {
        const short2 I0 = I_s[t * 32 + lane], I1 = I_s[(t + 1) * 32 + lane];
        const float2 g0 = __ldg(&Gj[t]), g1 = __ldg(&Gj[t + 1]), p0 = __ldg(&Pj[t]), p1 = __ldg(&Pj[t + 1]);
        const float4 q0 = gt_s[t * 32 + lane], q1 = gt_s[(t + 1) * 32 + lane];
        ray(t, I0, g0, p0, q0);
        ray(t + 1, I1, g1, p1, q1);
      }
      if (t <= tmax) ray(t, I_s[t * 32 + lane], __ldg(&Gj[t]), __ldg(&Pj[t]), gt_s[t * 32 + lane]);
      const dfx gzp = dfx_fma(pin, dcc, dfx_mul(pend, cj1));
      // direct terms of the effective height: z1_j + g_h (A_{j-1} - A_{j+1}) (- A_0 at j = 0)
      dfx nb = zx;
      if (j >= 1) nb = ld(a.us, j - 1);
      if (j + 1 <= L - 2) nb = dfx_sub(nb, ld(a.us, j + 1));
      if (j == 0) nb = dfx_sub(nb, ld(a.us, 0));
      dfx gzt = dfx_fma(gh, nb, gzp);
      if (j <= L - 2) gzt = dfx_add(gzt, ld(a.qs, j));
      st(a.gc, j, gc);
      st(a.gz, j, gzt);
      // (an element past N reads wavenumber N - 1's stored sinks: left out)
      rp = dfx_add(rp, dfx_select(true, act1, gzt, zx));
    }
  }
  const df2 rps = df_add(dfx_get(rp, 0), dfx_get(rp, 1));
  rp_part[threadIdx.x] = make_float2(rps.hi, rps.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < 32 * NG; ++q) s += df_to_double(df2{rp_part[q].x, rp_part[q].y});
    a.rp[(size_t)b * gridDim.x + blockIdx.x] = s;
  }
}

// Pass 2a with A impact parameters per layer (K = (L - 1) A rays; geometry in
// tr_geometry_adjoint_annuli_kernel). Ray k of layer t_k with weight w_k = jj / A has
//   tau_k = G_k[t] (c_t + w_k d_t) + sum_{i = t+1}^{I_k} G_k[i] c_i,  d_t = chi_{t+1} - chi_t,
//   h = sum_k rw_k (1 - T_k),  rw_k = (R + zb_k)((zb_{k+1} - zb_k) + (zb_k - zb_{k-1})).
// Block: 64 wavenumbers (two per lane, paired double-floats) x 8 warps, three phases:
//   1. per ray: g_tau_k = g_h rw_k T_k (over T_k), A_k = (R + zb_k)(1 - T_k), and
//      z1_k = g_h (1 - T_k) wz_k + g_tau_k qs_k (over qs_k; qs_k = dtau_k / db_k)
//   2. per ray: D_k = d log L / d zb_k = z1_k + g_h (A_{k-1} - A_{k+1}) (- A_0 at k = 0)
//   3. per level j, over the rays that reach it (from the lowest one, as in tr_adjoint_pass2a):
//      g_c_j = sum g_tau_k G_k[j] (segment j in the ray), g_d_j = sum_{t_k = j} g_tau_k w_k G_k[j],
//      g_z_j = sum_{t_k < j} g_tau_k P_k[j] (c'_{j-1} [j-1 <= I_k] - c_j [j <= I_k])
//              + sum_{t_k = j} (1 - w_k) D_k + sum_{t_k = j-1} w_k D_k (+ g_h A_{K-1} at j = L - 1),
//      c'_{j-1} = c_{j-1} + w_k d_{j-1} for the rays of layer j - 1 (their first segment);
//      d log L / dR = sum_j g_z_j + 2 R g_h as in tr_adjoint_pass2a.
// The per-ray arrays are [b][k][N]; lanes past N work on wavenumber N - 1 with a zero seed
// and store nothing.
__global__ void __launch_bounds__(32 * kPass2aGroups, 2) tr_adjoint_pass2a_annuli(DeviceModel dm, TrArgs a) {
  constexpr int NG = kPass2aGroups;
  __shared__ float2 rp_part[32 * NG];
  const int L = dm.L, A = dm.annuli, K = (L - 1) * A;
  const int b = blockIdx.y, lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
  const int kk0 = blockIdx.x * 64 + lane, kk1 = kk0 + 32;
  const bool act0 = kk0 < dm.N, act1 = kk1 < dm.N;
  const int k0 = act0 ? kk0 : dm.N - 1, k1 = act1 ? kk1 : dm.N - 1;
  const size_t N = dm.N;
  const size_t col0 = (size_t)b * L * N + k0, col1 = (size_t)b * L * N + k1;    // per-level rows
  const size_t rcol0 = (size_t)b * K * N + k0, rcol1 = (size_t)b * K * N + k1;  // per-ray rows
  const double Rp = a.ev[b].radius, Rs = a.ev[b].star_radius;
  const double* zb = a.rays + (size_t)b * 2 * (K + 1);
  const double* rw = zb + (K + 1);
  const dfx gh = dfx_make(df_from_double(act0 ? tr_seed(dm, a.gS, a.seed, b, k0) * 1e6 / (Rs * Rs) : 0.0),
                          df_from_double(act1 ? tr_seed(dm, a.gS, a.seed, b, k1) * 1e6 / (Rs * Rs) : 0.0));
  const dfx zx = {f2(0.0f), f2(0.0f)};
  const dfx one = dfx_bcast(df_make(1.0f));
  auto pair = [](float2 v0, float2 v1) { return dfx{make_float2(v0.x, v1.x), make_float2(v0.y, v1.y)}; };
  auto ld = [&](const float2* arr, int t) { return pair(arr[col0 + (size_t)t * N], arr[col1 + (size_t)t * N]); };
  auto ldr = [&](const float2* arr, int k) { return pair(arr[rcol0 + (size_t)k * N], arr[rcol1 + (size_t)k * N]); };
  auto put = [&](float2* arr, size_t c0, size_t c1, const dfx& v) {
    if (act0) arr[c0] = make_float2(v.hi.x, v.lo.x);
    if (act1) arr[c1] = make_float2(v.hi.y, v.lo.y);
  };
  auto bc = [](double x) { return dfx_bcast(df_from_double(x)); };
  // the per-ray stores are rewritten in place: T -> g_tau, us -> A, qs -> z1, then qs -> D
  float2* gtau_r = a.T;
  for (int kr = grp; kr < K; kr += NG) {
    const dfx T = ldr(a.T, kr), omT = dfx_sub(one, T);
    const double z = zb[kr];
    const double wz = (zb[kr + 1] - z) + (kr >= 1 ? z - zb[kr - 1] : 0.0);
    const dfx gt = dfx_mul(dfx_mul(gh, bc(rw[kr])), T);
    const dfx z1 = dfx_add(dfx_mul(dfx_mul(gh, omT), bc(wz)), dfx_mul(gt, ldr(a.qs, kr)));
    const size_t o = (size_t)kr * N;
    put(gtau_r, rcol0 + o, rcol1 + o, gt);
    put(a.us, rcol0 + o, rcol1 + o, dfx_mul(bc(Rp + z), omT));
    put(a.qs, rcol0 + o, rcol1 + o, z1);
  }
  __syncthreads();
  for (int kr = grp; kr < K; kr += NG) {
    dfx nb = zx;
    if (kr >= 1) nb = ldr(a.us, kr - 1);
    if (kr + 1 <= K - 1) nb = dfx_sub(nb, ldr(a.us, kr + 1));
    if (kr == 0) nb = dfx_sub(nb, ldr(a.us, 0));
    const size_t o = (size_t)kr * N;
    put(a.qs, rcol0 + o, rcol1 + o, dfx_fma(gh, nb, ldr(a.qs, kr)));
  }
  __syncthreads();
  const float2* PT = a.geo + (size_t)b * 3 * L * K;
  const float2* GT = PT + (size_t)L * K;
  dfx rp = zx;
  // the lowest ray reaching level j, per element (ray k covers levels t_k .. I_k + 1)
  int tp0 = 0, cov0 = -1, m0 = 0, tp1 = 0, cov1 = -1, m1 = 0;
  for (int j = grp; j < L; j += NG) {
    const dfx cj1 = j >= 1 ? ld(a.c, j - 1) : zx;
    const dfx cj = j <= L - 2 ? ld(a.c, j) : zx;
    const dfx dj1 = j >= 1 ? ld(a.d, j - 1) : zx;
    dfx gc = zx, gd = zx, pin = zx, pend = zx, pw = zx, dd = zx;
    while (cov0 < j && tp0 <= K - 1) {
      cov0 = max(cov0, min((int)a.I[rcol0 + (size_t)tp0 * N] + 1, L - 1));
      m0 = tp0++;
    }
    while (cov1 < j && tp1 <= K - 1) {
      cov1 = max(cov1, min((int)a.I[rcol1 + (size_t)tp1 * N] + 1, L - 1));
      m1 = tp1++;
    }
    const int kmin = (int)__reduce_min_sync(0xffffffffu, (unsigned)min(m0, m1));
    const int kmax = j <= L - 2 ? min((j + 1) * A, K) - 1 : K - 1;
    const float2* Gj = GT + (size_t)j * K;
    const float2* Pj = PT + (size_t)j * K;
    auto ray = [&](int t, short I0, short I1, const dfx& gtau, float2 g, float2 p) {
      // segment j in the ray (and j <= L - 2), segment j - 1 in the ray
      const bool in0 = I0 >= j && j <= L - 2, in1 = I1 >= j && j <= L - 2;
      if (in0 || in1) gc = dfx_fma(dfx_select(in0, in1, gtau, zx), dfx_bcast(df2{g.x, g.y}), gc);
      if (t < j) {
        const bool e0 = I0 >= j - 1 && !in0, e1 = I1 >= j - 1 && !in1;
        const dfx pp = dfx_bcast(df2{p.x, p.y});
        if (in0 || in1) pin = dfx_fma(dfx_select(in0, in1, gtau, zx), pp, pin);
        if (e0 || e1) pend = dfx_fma(dfx_select(e0, e1, gtau, zx), pp, pend);
      }
    };
    // two rays per step, their loads issued together (same sums, same order); t and jj of
    // ray kr kept as counters
    int t = kmin / A, jj = kmin - t * A;
    int kr = kmin;
    for (; kr + 1 <= kmax; kr += 2) {
      const size_t o0 = (size_t)kr * N, o1 = o0 + N;
      const short Ia0 = a.I[rcol0 + o0], Ia1 = a.I[rcol1 + o0], Ib0 = a.I[rcol0 + o1], Ib1 = a.I[rcol1 + o1];
      const dfx ga = ldr(gtau_r, kr), gb = ldr(gtau_r, kr + 1);
      const float2 g0 = __ldg(&Gj[kr]), g1 = __ldg(&Gj[kr + 1]), p0 = __ldg(&Pj[kr]), p1 = __ldg(&Pj[kr + 1]);
      const int tb = jj + 1 == A ? t + 1 : t;
      ray(t, Ia0, Ia1, ga, g0, p0);
      ray(tb, Ib0, Ib1, gb, g1, p1);
      jj += 2;
      while (jj >= A) {
        jj -= A;
        ++t;
      }
    }
    if (kr <= kmax)
      ray(t, a.I[rcol0 + (size_t)kr * N], a.I[rcol1 + (size_t)kr * N], ldr(gtau_r, kr), __ldg(&Gj[kr]), __ldg(&Pj[kr]));
    // the first segments: rays of layer j (g_d, and (1 - w) D) and of layer j - 1 (w P, w D)
    if (j <= L - 2)
      for (int jj = 0; jj < A; ++jj) {
        const int kr = j * A + jj;
        const double w = (double)jj / A;
        const dfx gtau = ldr(gtau_r, kr);
        const float2 g = __ldg(&Gj[kr]);
        gd = dfx_fma(dfx_mul(gtau, bc(w)), dfx_bcast(df2{g.x, g.y}), gd);
        dd = dfx_fma(bc(1.0 - w), ldr(a.qs, kr), dd);
      }
    if (j >= 1)
      for (int jj = 0; jj < A; ++jj) {
        const int kr = (j - 1) * A + jj;
        const double w = (double)jj / A;
        const float2 p = __ldg(&Pj[kr]);
        pw = dfx_fma(dfx_mul(ldr(gtau_r, kr), bc(w)), dfx_bcast(df2{p.x, p.y}), pw);
        dd = dfx_fma(bc(w), ldr(a.qs, kr), dd);
      }
    if (j == L - 1) dd = dfx_fma(gh, ldr(a.us, K - 1), dd);  // zb_K = z_{L-1}
    const dfx gz = dfx_add(dfx_add(dfx_fma(pin, dfx_sub(cj1, cj), dfx_mul(pend, cj1)), dfx_mul(pw, dj1)), dd);
    if (j <= L - 2) {
      put(a.gc, col0 + (size_t)j * N, col1 + (size_t)j * N, gc);
      put(a.gd, col0 + (size_t)j * N, col1 + (size_t)j * N, gd);
    }
    put(a.gz, col0 + (size_t)j * N, col1 + (size_t)j * N, gz);
    rp = dfx_add(rp, dfx_select(act0, act1, gz, zx));
  }
  if (grp == 0) rp = dfx_add(rp, dfx_mul(gh, bc(2.0 * Rp)));  // depth = (h + R^2) / R_s^2
  const df2 rps = df_add(dfx_get(rp, 0), dfx_get(rp, 1));
  rp_part[threadIdx.x] = make_float2(rps.hi, rps.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < 32 * NG; ++q) s += df_to_double(df2{rp_part[q].x, rp_part[q].y});
    a.rp[(size_t)b * gridDim.x + blockIdx.x] = s;
  }
}

// ------------------------------------------------------------------ pass 2b
// Level sinks: one block per (evaluation, level). The kTrSinkThreads threads stride the
// wavenumbers and accumulate, as double-floats in registers, v = 0..S-1 d log L / d ln n_s
// (table species), S..S+R-1 d log L / d ln n_r (Rayleigh species), S+R temperature,
// S+R+1 z_l and S+R+2 the cloud extinction of level l; one block reduction in a fixed order
// (warp reduce-scatter, then the warps' sums in warp order) writes partial[b][l][v] (times
// the evaluation's seed normaliser in the parameter pass). The opacity terms come from the
// forward pass's stores (a.ts, a.dk) where present, else they are recomputed from the level
// table in the same order (per-thread shared slots). Dynamic shared memory: float2 [S][T],
// double [S][T] (T = kTrSinkThreads), then the level's Rayleigh number densities float2 [R].
constexpr int kTrSinkThreads = 128;

// CLOUD: a non-grey cloud (the cloud value weighted by the wavelength factor, and the
// values along its shape parameters; tr_cloud_value).
template <int VP, bool PAIRS, bool CLOUD = false>
__global__ void __launch_bounds__(kTrSinkThreads, VP == 32 ? 4 : 6) tr_adjoint_pass2b(DeviceModel dm, TrArgs a) {
  constexpr int G = 32 / VP, NW = kTrSinkThreads / 32;
  __shared__ ExpTables et;
  __shared__ float2 red[NW][VP];
  extern __shared__ __align__(16) unsigned char tr2_smem[];
  const int S = dm.S, R = dm.R, L = dm.L;
  const int b = blockIdx.x, l = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float2* td = reinterpret_cast<float2*>(tr2_smem) + tid;                                  // [S][T]
  double* tw = reinterpret_cast<double*>(tr2_smem + (size_t)S * kTrSinkThreads * sizeof(float2)) + tid;
  float2* rn_s = reinterpret_cast<float2*>(tr2_smem + (size_t)S * kTrSinkThreads * (sizeof(float2) + sizeof(double)));
  load_exp_tables(et);
  for (int r = tid; r < R; r += kTrSinkThreads) {
    const df2 d = df_from_double(__ldg(&a.ray_n[((size_t)b * L + l) * R + r]));
    rn_s[r] = make_float2(d.hi, d.lo);
  }
  __syncthreads();
  const size_t N = dm.N;
  const LevelSpeciesDF* sfl = a.lsdf + ((size_t)b * L + l) * S;
  const float2* dwl = a.dwT + ((size_t)b * L + l) * S;
  const size_t row = ((size_t)b * L + l) * N;  // [b][l][k] of k = 0
  const float2* tsl = a.ts + ((size_t)b * L + l) * S * N;  // [s][N] (stored mode)
  const double cloud_l = CLOUD ? __ldg(&a.lev[(size_t)b * L + l].cloud) : 0.0;
  df2 v[VP];
#pragma unroll
  for (int q = 0; q < VP; ++q) v[q] = df2{0.0f, 0.0f};
  // one wavenumber's contribution (the recompute path, and every wavenumber when the
  // wavenumbers are not taken in pairs)
  auto one = [&](int k, df2 gx, float2 gz, float2 dks) {
    // opacity terms and their temperature slope (level-table values are log2 units)
    df2 dk = {0.0f, 0.0f};
    double dkw = 0.0;
    bool wide = false;
    const bool stored = !isnan(dks.x);
    if (stored) {
      dk = df2{dks.x, dks.y};
    } else {
      level_kappa_df_cb<2>(dm.ltab, N, sfl, S, k, et, [&](int s, df2 t, double t_w, bool is_wide, df2 lo, df2 hi) {
        const float2 d = __ldg(dwl + s);
        td[(size_t)s * kTrSinkThreads] = make_float2(t.hi, t.lo);
        tw[(size_t)s * kTrSinkThreads] = t_w;
        if (d.x != 0.0f) {
          const df2 slope = df_mul(df_sub(hi, lo), df2{d.x, d.y});
          if (is_wide) dkw += t_w * df_to_double(slope);
          else dk = df_add(dk, df_mul(t, slope));
        }
        wide = wide || is_wide;
      });
    }
    df2 gT = df_mul(gx, df_mul(dk, df2{kLn2Hi, kLn2Lo}));
    if (wide) gT = df_add(gT, df_from_double(df_to_double(gx) * dkw * 0.693147180559945309));
#pragma unroll
    for (int q = 0; q < VP; ++q) {
      df2 x = {0.0f, 0.0f};
      if (q < S) {
        const float2 t = stored ? __ldg(tsl + (size_t)q * N + k) : td[(size_t)q * kTrSinkThreads];
        x = df_mul(gx, df2{t.x, t.y});
        if (wide) x = df_add(x, df_from_double(df_to_double(gx) * tw[(size_t)q * kTrSinkThreads]));
      } else if (q < S + R) {
        const float2 sr = __ldg(&dm.rayleigh_df[(size_t)(q - S) * N + k]);
        const float2 nr = rn_s[q - S];
        x = df_mul(gx, df_mul(df2{sr.x, sr.y}, df2{nr.x, nr.y}));
      } else if (q == S + R) {
        x = gT;
      } else if (q == S + R + 1) {
        x = df2{gz.x, gz.y};
      } else if (CLOUD ? q >= S + R + 2 && q <= S + R + 2 + a.nc : q == S + R + 2) {
        x = CLOUD ? tr_cloud_value(a, q - S - R - 2, b, N, k, gx, cloud_l) : gx;
      }
      v[q] = df_add(v[q], x);
    }
  };
  auto load_gx = [&](int k) {
    df2 gx = {0.0f, 0.0f};
    if (l <= L - 2) {
      const float2 c0 = a.gc[row + k];
      gx = df2{c0.x, c0.y};
    }
    if (l >= 1) {
      const float2 c1 = a.gc[row - N + k];
      gx = df_add(gx, df2{c1.x, c1.y});
    }
    if (a.gd) {  // A > 1: the first segments' c_t + w d_t, d_t = chi_{t+1} - chi_t
      if (l >= 1) {
        const float2 d1 = a.gd[row - N + k];
        gx = df_add(gx, df2{d1.x, d1.y});
      }
      if (l <= L - 2) {
        const float2 d0 = a.gd[row + k];
        gx = df_sub(gx, df2{d0.x, d0.y});
      }
    }
    return gx;
  };
  const float2 no_store = make_float2(__int_as_float(0x7fc00000), 0.0f);
  if (!PAIRS) {
    for (int k = tid; k < (int)N; k += kTrSinkThreads)
      one(k, load_gx(k), a.gz[row + k], a.ts ? a.dk[row + k] : no_store);
  } else {
    // N even: wavenumbers in adjacent pairs, every read 16 bytes; where both terms of a pair
    // are stored they are combined directly (the same sums in the same order as one() twice)
    auto ld4 = [](const float2* p) { return __ldg(reinterpret_cast<const float4*>(p)); };
    for (int k0 = 2 * tid; k0 < (int)N; k0 += 2 * kTrSinkThreads) {
      df2 gx0 = {0.0f, 0.0f}, gx1 = {0.0f, 0.0f};
      if (l <= L - 2) {
        const float4 c = ld4(a.gc + row + k0);
        gx0 = df2{c.x, c.y};
        gx1 = df2{c.z, c.w};
      }
      if (l >= 1) {
        const float4 c = ld4(a.gc + row - N + k0);
        gx0 = df_add(gx0, df2{c.x, c.y});
        gx1 = df_add(gx1, df2{c.z, c.w});
      }
      if (a.gd) {
        if (l >= 1) {
          const float4 c = ld4(a.gd + row - N + k0);
          gx0 = df_add(gx0, df2{c.x, c.y});
          gx1 = df_add(gx1, df2{c.z, c.w});
        }
        if (l <= L - 2) {
          const float4 c = ld4(a.gd + row + k0);
          gx0 = df_sub(gx0, df2{c.x, c.y});
          gx1 = df_sub(gx1, df2{c.z, c.w});
        }
      }
      const float4 gz = ld4(a.gz + row + k0);
      const float4 dks = a.ts ? ld4(a.dk + row + k0) : make_float4(no_store.x, 0.0f, no_store.x, 0.0f);
      if (isnan(dks.x) || isnan(dks.z)) {
#pragma unroll 1
        for (int w = 0; w < 2; ++w)
          one(k0 + w, w ? gx1 : gx0, w ? make_float2(gz.z, gz.w) : make_float2(gz.x, gz.y),
              w ? make_float2(dks.z, dks.w) : make_float2(dks.x, dks.y));
        continue;
      }
      const df2 gT0 = df_mul(gx0, df_mul(df2{dks.x, dks.y}, df2{kLn2Hi, kLn2Lo}));
      const df2 gT1 = df_mul(gx1, df_mul(df2{dks.z, dks.w}, df2{kLn2Hi, kLn2Lo}));
#pragma unroll
      for (int q = 0; q < VP; ++q) {
        df2 x0 = {0.0f, 0.0f}, x1 = {0.0f, 0.0f};
        if (q < S) {
          const float4 t = ld4(tsl + (size_t)q * N + k0);
          x0 = df_mul(gx0, df2{t.x, t.y});
          x1 = df_mul(gx1, df2{t.z, t.w});
        } else if (q < S + R) {
          const float4 sr = ld4(dm.rayleigh_df + (size_t)(q - S) * N + k0);
          const float2 nr = rn_s[q - S];
          x0 = df_mul(gx0, df_mul(df2{sr.x, sr.y}, df2{nr.x, nr.y}));
          x1 = df_mul(gx1, df_mul(df2{sr.z, sr.w}, df2{nr.x, nr.y}));
        } else if (q == S + R) {
          x0 = gT0;
          x1 = gT1;
        } else if (q == S + R + 1) {
          x0 = df2{gz.x, gz.y};
          x1 = df2{gz.z, gz.w};
        } else if (CLOUD ? q >= S + R + 2 && q <= S + R + 2 + a.nc : q == S + R + 2) {
          x0 = CLOUD ? tr_cloud_value(a, q - S - R - 2, b, N, k0, gx0, cloud_l) : gx0;
          x1 = CLOUD ? tr_cloud_value(a, q - S - R - 2, b, N, k0 + 1, gx1, cloud_l) : gx1;
        }
        v[q] = df_add(df_add(v[q], x0), x1);
      }
    }
  }
  const df2 r = warp_reduce_scatter<VP>(v, lane);
  if (lane % G == 0) red[warp][lane / G] = make_float2(r.hi, r.lo);
  __syncthreads();
  if (tid < a.V) {
    df2 sum = {red[0][tid].x, red[0][tid].y};
#pragma unroll
    for (int w = 1; w < NW; ++w) sum = df_add(sum, df2{red[w][tid].x, red[w][tid].y});
    a.partial[((size_t)b * L + l) * a.V + tid] = df_to_double(sum);
  }
}

// ------------------------------------------------------------------ parameter tangents
// One block per evaluation. sg[L][V] = the level sinks of pass 2b (partial[b][l][v]); then
// thread th < P forms d log L / d param_th = sum over levels of the sinks times the
// tangents of ln n (table and Rayleigh species), T, z_l and the cloud extinction
// chi_cloud,l = tau_layer(l-1) / (z_l - z_{l-1}) (CloudModel::convertOpticalDepth
// src/cloud_model/cloud_model.h:67-88), plus the planet radius (d log L / dR from
// pass 1) and the stellar radius (depth ~ 1 / R_s^2: -2 / R_s sum_k g_k depth_k).
// TransmissionModel::calcAtmosphereStructure src/forward_model/transmission/transmission.cpp:150-194,
// Atmosphere::calcAltitude src/forward_model/atmosphere/atmosphere.cpp:288-307.
__global__ void __launch_bounds__(128) tr_atmosphere_adjoint_kernel(
    DeviceModel dm, const double* __restrict__ params, int P, const LevelInfo* __restrict__ lev,
    const EvalInfo* __restrict__ ev, const double* __restrict__ partial, int V, int tiles,
    const double* __restrict__ rp, int rp_tiles, const double* __restrict__ seed, double* __restrict__ grad) {
  extern __shared__ double sg[];
  __shared__ double s_rp;
  const AtmosphereConfig& c = *dm.cfg;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int L = c.L, S = c.S, R = c.R;
  if (ev[b].neglect) return;
  const double inv = seed[b * 3 + 1];
  for (int idx = tid; idx < L * V; idx += blockDim.x) sg[idx] = partial[((size_t)b * L * V + idx) * tiles] * inv;
  if (warp == 0) {
    double s = 0.0;
    for (int q = lane; q < rp_tiles; q += 32) s += rp[(size_t)b * rp_tiles + q];
    s = warp_sum_d(s);
    if (lane == 0) s_rp = s * inv;
  }
  __syncthreads();
  // thread (th, ch): parameter th over the levels of chunk ch; the altitude tangent, a prefix
  // sum over levels, starts each chunk from the chunks below it (two passes), and the chunk
  // sums are added in chunk order
  __shared__ double part[128];
  const int nch = max(1, (int)blockDim.x / P);
  const int th = tid % P, ch = tid / P;
  const bool work = ch < nch;
  const int l0 = ch * L / nch, l1 = (ch + 1) * L / nch;
  const double* par = params + (size_t)b * P;
  const double* gen = par;
  const int ng = c.nparam_general, nc = c.nparam_chem, nt = c.nparam_temp;
  const double* chem = par + ng;
  const double* temp = chem + nc;
  const double* cloud = temp + nt;
  double X[kSpeciesCount], dX[kSpeciesCount], mmw, dmmw;
  chemistry_tangent(c, chem, (th >= ng && th < ng + nc) ? th - ng : -1, X, dX, mmw, dmmw);
  if (c.fit_mmw) {  // mean molecular weight as a free parameter (general parameter 3)
    mmw = gen[3];
    dmmw = th == 3 ? 1.0 : 0.0;
  }
  const int tm = th - ng - nc;
  const bool temp_theta = tm >= 0 && tm < nt;
  double ddof[kMaxPolyDof];
  if (temp_theta && c.temp_poly) {
    for (int i = 0; i < c.pp_ndof; ++i) {
      double v = 0.0;
      if (i >= tm) {
        v = 1.0;
        for (int q = 0; q <= i; ++q)
          if (q != tm) v *= temp[q];
      }
      ddof[i] = v;
    }
  }
  const double g = pow(10.0, gen[0]);
  const double dlng = th == 0 ? kLn10 : 0.0;
  const int ci = ng + nc + nt;
  const EvalInfo e = ev[b];
  double cloud_d = 0.0;
  if (c.cloud && th == ci && cloud[0] >= 0)
    cloud_d = 1.0 / (double)((unsigned)e.cloud_top - (unsigned)e.cloud_bottom);
  auto in_cloud = [&](int layer) {
    return (unsigned)layer <= (unsigned)e.cloud_top && (unsigned)layer > (unsigned)e.cloud_bottom && layer < L - 1;
  };
  // per species: d ln n = sum_j dX_j / X_j - (1 + partners) d ln T
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
    np[s] = zero ? -1 : n;
  }
  auto dT_at = [&](int l) -> double {
    if (!temp_theta) return 0.0;
    return c.temp_poly ? poly_value(c, ddof, dm.log10p[l]) : (tm == 0 ? 1.0 : 0.0);
  };
  // u = R T / (mmw p 1e6) and its tangent at level l
  auto u_at = [&](int l, double& du) {
    const double T = lev[(size_t)b * L + l].T;
    const double u = kGasConst * T / (mmw * dm.pressure[l] * 1e6);
    du = u * (dT_at(l) / T - dmmw / mmw);
    return u;
  };
  // The altitude tangent dz_l = dz_{l-1} + A_l + B_l dz_{l-1} for the layer l - 1 -> l:
  // constant gravity (Delta_l = 0.5 (p_{l-1} - p_l) 1e6 (u_l + u_{l-1}) / g): B_l = 0,
  // A_l = 0.5 (p_{l-1} - p_l) 1e6 ((du_l + du_{l-1}) - (u_l + u_{l-1}) d ln g) / g; variable
  // gravity (g_l = g R^2 / (R + z_{l-1})^2, Atmosphere::calcAltitudeVariableGravity
  // src/forward_model/atmosphere/atmosphere.cpp:311-334, R the planet radius): with the
  // forward's Delta_l = z_l - z_{l-1}, B_l = 2 Delta_l / (R + z_{l-1}) and
  // A_l = Delta_l ((du_l + du_{l-1}) / (u_l + u_{l-1}) - d ln g - 2 dR / R + 2 dR / (R + z_{l-1})).
  const double R0 = gen[1], dR0 = th == 1 ? 1.0 : 0.0;
  auto ddelta = [&](int l, double u, double du, double u_prev, double du_prev, double& B) {
    if (!c.var_g) {
      B = 0.0;
      const double pf = 0.5 * (dm.pressure[l - 1] * 1e6 - dm.pressure[l] * 1e6) / g;
      return pf * ((du + du_prev) - (u + u_prev) * dlng);
    }
    const double zp = lev[(size_t)b * L + l - 1].z, dzv = lev[(size_t)b * L + l].z - zp;
    B = 2.0 * dzv / (R0 + zp);
    return dzv * ((du + du_prev) / (u + u_prev) - dlng - 2.0 * dR0 / R0 + 2.0 * dR0 / (R0 + zp));
  };
  // pass 1: the chunk's affine map of the altitude tangent, dz_end = M dz_start + C
  __shared__ double part_m[128];
  double u_prev = 0.0, du_prev = 0.0;
  if (work) {
    double Mc = 1.0, Cc = 0.0;
    if (l0 >= 1) u_prev = u_at(l0 - 1, du_prev);
    double up = u_prev, dup = du_prev;
    for (int l = l0; l < l1; ++l) {
      double du;
      const double u = u_at(l, du);
      if (l >= 1) {
        double B;
        const double A = ddelta(l, u, du, up, dup, B);
        Cc = c.var_g ? fma(1.0 + B, Cc, A) : Cc + A;
        Mc *= 1.0 + B;
      }
      up = u;
      dup = du;
    }
    part[tid] = Cc;
    part_m[tid] = Mc;
  }
  __syncthreads();
  double dz = 0.0, dz_prev = 0.0, acc = 0.0;
  if (work)
    for (int q = 0; q < ch; ++q) dz = c.var_g ? fma(part_m[q * P + th], dz, part[q * P + th]) : dz + part[q * P + th];
  __syncthreads();
  for (int l = l0; work && l < l1; ++l) {
    const LevelInfo li = lev[(size_t)b * L + l];
    const double dT = dT_at(l);
    const double dlnT = dT / li.T;
    const double* sgl = sg + (size_t)l * V;
    for (int s = 0; s < S; ++s)
      if (np[s] >= 0) acc = fma(sgl[s], dlnX[s] - np[s] * dlnT, acc);
    for (int r = 0; r < c.R_ray; ++r) {
      const int jr = c.ray_index[r];
      if (X[jr] != 0.0) acc = fma(sgl[S + r], dX[jr] / X[jr] - dlnT, acc);
    }
    if (c.hm && X[SP_Hm] != 0.0) {
      // H- continuum: values S + R_ray + i are d log L / d ln h_i for the coefficients
      // h_0 = n(H-) and h_i = (5040/T)^((i+1)/2) n(e-) k T n(H) (atmosphere_kernel); n_j = X_j p / (k T).
      // A zero H or e- abundance makes h_i (i >= 1) zero, and its derivative is taken as zero.
      acc = fma(sgl[S + c.R_ray], dX[SP_Hm] / X[SP_Hm] - dlnT, acc);
      if (X[SP_e] != 0.0 && X[SP_H] != 0.0) {
        const double dln = dX[SP_e] / X[SP_e] + dX[SP_H] / X[SP_H];
        for (int i = 1; i < kHmTerms; ++i) acc = fma(sgl[S + c.R_ray + i], dln - (1.0 + (i + 1) / 2.0) * dlnT, acc);
      }
    }
    acc = fma(sgl[S + R], dT, acc);
    // z_l = z_{l-1} + Delta_l, Delta_l = 0.5 (p_{l-1} - p_l) 1e6 (u_l + u_{l-1}) / g, u = R T / (mmw p 1e6)
    double du;
    const double u = u_at(l, du);
    dz_prev = dz;
    if (l >= 1) {
      double B;
      const double A = ddelta(l, u, du, u_prev, du_prev, B);
      dz = c.var_g ? fma(1.0 + B, dz, A) : dz + A;
    }
    u_prev = u;
    du_prev = du;
    acc = fma(sgl[S + R + 1], dz, acc);
    // cloud extinction tau_layer(l-1) / (z_l - z_{l-1})
    if (c.cloud && l >= 1 && in_cloud(l - 1)) {
      const double zl1 = lev[(size_t)b * L + l - 1].z;
      const double h = li.z - zl1;
      double d = -li.cloud * (dz - dz_prev) / h;
      if (cloud_d != 0.0 && in_cloud(l - 1)) d += cloud_d / h;
      acc = fma(sgl[S + R + 2], d, acc);
    }
  }
  // non-grey cloud shape parameters (after the optical depth): values S + R + 3 + c summed over levels
  if (work && c.cloud && c.cloud_kind) {
    const int cs = th - ci - 1;
    if (cs >= 0 && cs < (c.cloud_kind == 1 ? 1 : 3))
      for (int l = l0; l < l1; ++l) acc += sg[(size_t)l * V + S + R + 3 + cs];
  }
  if (work && ch == 0) {
    if (th == 1) acc += s_rp;                                      // planet radius
    if (th == 2) acc += -2.0 / e.star_radius * seed[b * 3 + 2];    // stellar radius
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
size_t transmission_grad_bytes_per_eval(const Model& m, int V, bool store) {
  const size_t L = m.L, N = m.N, K = transmission_rays(m);
  const size_t tiles = (N + 31) / 32;
  const size_t terms = store ? L * N * ((size_t)m.acfg.S + 1) * sizeof(float2) : 0;
  const size_t cs = m.acfg.cloud_kind ? (m.acfg.cloud_kind == 1 ? 2 : 4) * N * sizeof(double) : 0;
  // per ray T, qs, us, I; per level c, g_c, g_z (and with A > 1 d, g_d)
  const size_t rays = std::max(K, L);
  const size_t levels = (m.annuli > 1 ? 5 : 3) * L * N * sizeof(float2);
  return rays * N * (3 * sizeof(float2) + sizeof(short)) + levels + 3 * L * rays * sizeof(float2) +
         L * (size_t)V * 8 + tiles * 8 + terms + cs;
}

void alloc_transmission_grad(Model& m, int chunk, int V, bool store) {
  GradWorkspace& g = m.gws;
  const size_t B = chunk, L = m.L, N = m.N;
  g.tr_store = store;
  if (store) {
    // two spare entries at the end of the arrays the level-sink pass streams (whole 16-byte
    // units of an odd-length last row)
    BGB_CUDA(cudaMalloc(&g.taps.tr_ts, (B * L * (size_t)m.acfg.S * N + 2) * sizeof(float2)));
    BGB_CUDA(cudaMalloc(&g.taps.tr_dk, (B * L * N + 2) * sizeof(float2)));
  }
  // per-ray arrays: one row per level (rays at the levels) or per ray (A > 1)
  const size_t n = B * L * N, tiles = (N + 31) / 32, nr = B * std::max<size_t>(transmission_rays(m), L) * N;
  BGB_CUDA(cudaMalloc(&g.taps.tr_c, n * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.taps.tr_T, nr * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.taps.tr_qs, nr * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.taps.tr_us, nr * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.taps.tr_I, nr * sizeof(short)));
  BGB_CUDA(cudaMalloc(&g.taps.tr_geo, nr / N * 3 * L * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.tr_gc, (n + 2) * sizeof(float2)));
  BGB_CUDA(cudaMalloc(&g.tr_gz, (n + 2) * sizeof(float2)));
  if (m.annuli > 1) {
    BGB_CUDA(cudaMalloc(&g.taps.tr_d, n * sizeof(float2)));
    BGB_CUDA(cudaMalloc(&g.tr_gd, (n + 2) * sizeof(float2)));
  }
  BGB_CUDA(cudaMalloc(&g.tr_rp, B * tiles * sizeof(double)));
  BGB_CUDA(cudaMalloc(&g.partial, B * L * (size_t)V * sizeof(double)));
  if (m.acfg.cloud_kind) {
    const size_t nc = m.acfg.cloud_kind == 1 ? 1 : 3;
    BGB_CUDA(cudaMalloc(&g.tr_cs, B * (1 + nc) * N * sizeof(double)));
  }
}

// ------------------------------------------------------------------ pass 2b, streamed
// tr_adjoint_pass2b's sums (its stored-terms path) with the rows it reads streamed through
// shared memory by bulk asynchronous copies: per (evaluation, level) block and tile of
// kStreamTile wavenumbers the S opacity-term rows, the R Rayleigh cross-section rows, g_z,
// the temperature-slope sums and the two g_c rows (STAGES tiles in flight: three where two
// blocks per SM fit, else two). With PAIRS (N even) thread tid takes the pair k0 + 2 tid,
// k0 + 2 tid + 1 of each tile, as tr_adjoint_pass2b<VP, true> does; otherwise the single
// wavenumbers k0 + tid and k0 + 128 + tid, as tr_adjoint_pass2b<VP, false> does (rows of odd
// length start on 8-byte boundaries: each copy starts at the 16-byte unit holding its first
// entry, and the arrays end with a spare 16-byte unit). Every sum receives the same terms
// in the same order as in that kernel, so the partial sums are equal bit for bit. A pair with a
// term outside the float range (no stored slope) recomputes its terms from the level table
// as that kernel does. If a copy does not complete within the bounded wait, the block's
// partial sums are set to NaN (the gradient of that evaluation reads NaN) and the block
// returns after waiting, bounded again, for its copies in flight.
// Block: kTrSinkThreads consumer threads (one pair each per tile) and one producer warp whose
// first lane refills a stage as soon as the four consumer warps released it (no block-wide
// barrier inside the loop). For 64 evaluations of 100 levels x 33976 points (16 segments, 96
// KB of stages per block, two blocks per SM) it reads 24.0 GB in 5.9 ms (4.1 TB/s); the
// register-streamed tr_adjoint_pass2b took 9.3 ms and a version refilling stages after a
// block barrier 8.2 ms.
constexpr int kStreamTile = 256;  // wavenumbers per tile (128 pairs, one per thread)
constexpr int kStreamMaxSeg = 40;  // segments per tile: S + R + 4 with S + R <= 36

// level_kappa_df_cb's term of one species (same arithmetic): t (zero if outside the float
// range, then w holds it in FP64 and wide is set), lo and hi the level-table values
__device__ __forceinline__ void species_term_df(const float2* __restrict__ ltab, size_t N,
                                                const LevelSpeciesDF* __restrict__ f, int k, const ExpTables& et,
                                                df2& t, double& w, bool& wide, df2& lo, df2& hi) {
  const df2 z = {0.0f, 0.0f};
  t = z;
  w = 0.0;
  wide = false;
  lo = hi = z;
  const int4 rw = __ldg(reinterpret_cast<const int4*>(f));
  const float4 fb = __ldg(reinterpret_cast<const float4*>(f) + 1);  // wT, log2 n
  if (fb.z == kNoSpecies) return;
  const float2 t0 = __ldg(ltab + (size_t)rw.x * N + k), t1 = __ldg(ltab + (size_t)rw.y * N + k);
  lo = df2{t0.x, t0.y};
  hi = df2{t1.x, t1.y};
  const df2 y = df_fma(df_sub(hi, lo), df2{fb.x, fb.y}, df_add(lo, df2{fb.z, fb.w}));
  int n;
  const df2 m = df_exp2(y, n, et.hi, et.lo);
  if (n > -100 && n < 100) {
    t = df_ldexp(m, n);
  } else {
    w = df_to_double(m) * pow2d(n);
    wide = true;
  }
}

// tr_adjoint_pass2b's one() for a wavenumber without a stored slope sum (a term outside the
// float range): the S species contributions gx t_s (+ the FP64 part) into xs, and the
// temperature contribution returned; kept out of line so that the streamed kernel's
// common path carries no per-species arrays.
__device__ __noinline__ df2 tr_sink_recompute(const DeviceModel& dm, const LevelSpeciesDF* __restrict__ sfl,
                                              const float2* __restrict__ dwl, int k, const ExpTables& et, df2 gx,
                                              df2* xs) {
  const int S = dm.S;
  const size_t N = dm.N;
  df2 dk = {0.0f, 0.0f};
  double dkw = 0.0;
  bool wide = false;
  double tw[32];
  for (int q = 0; q < S; ++q) {
    bool is_wide;
    df2 lo, hi;
    species_term_df(dm.ltab, N, sfl + q, k, et, xs[q], tw[q], is_wide, lo, hi);
    const float2 d = __ldg(dwl + q);
    if (d.x != 0.0f) {
      const df2 slope = df_mul(df_sub(hi, lo), df2{d.x, d.y});
      if (is_wide) dkw += tw[q] * df_to_double(slope);
      else dk = df_add(dk, df_mul(xs[q], slope));
    }
    wide = wide || is_wide;
  }
  df2 gT = df_mul(gx, df_mul(dk, df2{kLn2Hi, kLn2Lo}));
  if (wide) gT = df_add(gT, df_from_double(df_to_double(gx) * dkw * 0.693147180559945309));
  for (int q = 0; q < S; ++q) {
    df2 x = df_mul(gx, xs[q]);
    if (wide) x = df_add(x, df_from_double(df_to_double(gx) * tw[q]));
    xs[q] = x;
  }
  return gT;
}

template <int VP, int STAGES, bool PAIRS>
__global__ void __launch_bounds__(kTrSinkThreads + 32, 2) tr_adjoint_pass2b_stream(DeviceModel dm, TrArgs a, int nseg) {
  static_assert(kStreamTile == 2 * kTrSinkThreads, "two wavenumbers per thread and tile");
  constexpr int G = 32 / VP, NW = kTrSinkThreads / 32;
  constexpr int SEG = kStreamTile + 2;  // entries per staged segment (one spare 16-byte unit)
  __shared__ ExpTables et;
  __shared__ float2 red[NW][VP];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES];
  __shared__ float2 rn_s[32];
  __shared__ volatile int abort_s, issued_s;
  __shared__ const float2* seg_src[kStreamMaxSeg];  // 16-byte unit holding the row's first entry
  __shared__ int seg_sh[kStreamMaxSeg];             // entries before the row's first in that unit
  extern __shared__ __align__(16) unsigned char tr2s_smem[];
  float2* stage = reinterpret_cast<float2*>(tr2s_smem);  // [STAGES][nseg][SEG]
  const int S = dm.S, R = dm.R, L = dm.L;
  const int b = blockIdx.x, l = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t N = dm.N;
  const size_t bl = (size_t)b * L + l;
  const size_t row = bl * N;  // [b][l][k] of k = 0
  const LevelSpeciesDF* sfl = a.lsdf + bl * S;
  const float2* dwl = a.dwT + bl * S;
  // segment order: S term rows, R Rayleigh rows, g_z, slope sums, g_c of levels l and l - 1
  const int sGZ = S + R, sDK = S + R + 1, sC0 = S + R + 2, sC1 = S + R + 3;
  const bool has_c0 = l <= L - 2, has_c1 = l >= 1;
  const int ntiles = (int)((N + kStreamTile - 1) / kStreamTile);
  // first entry of each segment's row in its array (tiles start at even offsets)
  auto row_start = [&](int seg) -> size_t {
    if (seg < S) return (bl * S + seg) * N;
    if (seg < S + R) return (size_t)(seg - S) * N;
    if (seg == sC1) return row - N;
    return row;
  };
  auto array_of = [&](int seg) -> const float2* {
    if (seg < S) return a.ts;
    if (seg < S + R) return dm.rayleigh_df;
    if (seg == sGZ) return a.gz;
    if (seg == sDK) return a.dk;
    return a.gc;
  };
  auto used = [&](int seg) { return !((seg == sC0 && !has_c0) || (seg == sC1 && !has_c1)); };
  load_exp_tables(et);
  for (int r = tid; r < R; r += blockDim.x) {
    const df2 d = df_from_double(__ldg(&a.ray_n[bl * R + r]));
    rn_s[r] = make_float2(d.hi, d.lo);
  }
  if (tid == 0) {
    abort_s = 0;
    issued_s = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NW);
    }
    fence_barrier_init();
  }
  for (int seg = tid; seg < nseg; seg += blockDim.x) {
    const size_t o = row_start(seg);
    seg_sh[seg] = (int)(o & 1);
    seg_src[seg] = array_of(seg) + (o & ~(size_t)1);
  }
  __syncthreads();
  if (warp == NW) {
    // producer warp (one lane): refill each stage once the consumer warps released it
    if (lane == 0) {
      for (int it = 0; it < ntiles; ++it) {
        const int st = it % STAGES;
        if (it >= STAGES) {
          if (!mbar_wait_bounded(&empty[st], (uint32_t)((it / STAGES - 1) & 1))) {
            abort_s = 1;
            break;
          }
          fence_proxy_async_smem();
        }
        if (abort_s) break;
        const size_t k0 = (size_t)it * kStreamTile;
        const int len = (int)min((size_t)kStreamTile, N - k0);
        // each copy: whole 16-byte units from the one holding the tile's first entry
        uint32_t total = 0;
        for (int seg = 0; seg < nseg; ++seg)
          if (used(seg)) total += (uint32_t)((seg_sh[seg] + len + 1) & ~1) * (uint32_t)sizeof(float2);
        mbar_expect_tx(&full[st], total);
        float2* base = stage + (size_t)st * nseg * SEG;
        for (int seg = 0; seg < nseg; ++seg) {
          if (!used(seg)) continue;
          const uint32_t bytes = (uint32_t)((seg_sh[seg] + len + 1) & ~1) * (uint32_t)sizeof(float2);
          bulk_g2s(base + (size_t)seg * SEG, seg_src[seg] + k0, bytes, &full[st]);
        }
        issued_s = it + 1;
      }
    }
  } else {
    df2 v[VP];
#pragma unroll
    for (int q = 0; q < VP; ++q) v[q] = df2{0.0f, 0.0f};
    const df2 z = {0.0f, 0.0f};
    for (int it = 0; it < ntiles; ++it) {
      const int st = it % STAGES;
      if (!mbar_wait_bounded(&full[st], (uint32_t)((it / STAGES) & 1))) abort_s = 1;
      if (abort_s) break;
      const float2* base = stage + (size_t)st * nseg * SEG;
      const int k0 = it * kStreamTile;
      // entry idx of the tile in segment seg (past the copy's leading entry, if any)
      auto sg2 = [&](int seg, int idx) { return base[seg * SEG + seg_sh[seg] + idx]; };
      // one wavenumber (tr_adjoint_pass2b's one(), stored or recomputed terms)
      auto single = [&](int k, int idx) {
        df2 gx = z;
        if (has_c0) {
          const float2 c = sg2(sC0, idx);
          gx = df2{c.x, c.y};
        }
        if (has_c1) {
          const float2 c = sg2(sC1, idx);
          gx = df_add(gx, df2{c.x, c.y});
        }
        const float2 gz = sg2(sGZ, idx), dke = sg2(sDK, idx);
        const bool stored = !isnan(dke.x);
        df2 xs[32];  // recomputed species contributions (rare path)
        const df2 gT = stored ? df_mul(gx, df_mul(df2{dke.x, dke.y}, df2{kLn2Hi, kLn2Lo}))
                              : tr_sink_recompute(dm, sfl, dwl, k, et, gx, xs);
#pragma unroll
        for (int q = 0; q < VP; ++q) {
          df2 x = z;
          if (q < S) {
            if (stored) {
              const float2 t = sg2(q, idx);
              x = df_mul(gx, df2{t.x, t.y});
            } else {
              x = xs[q];
            }
          } else if (q < S + R) {
            const float2 sr = sg2(q, idx);
            const float2 nr = rn_s[q - S];
            x = df_mul(gx, df_mul(df2{sr.x, sr.y}, df2{nr.x, nr.y}));
          } else if (q == S + R) {
            x = gT;
          } else if (q == S + R + 1) {
            x = df2{gz.x, gz.y};
          } else if (q == S + R + 2) {
            x = gx;
          }
          v[q] = df_add(v[q], x);
        }
      };
      if (!PAIRS) {
        if (k0 + tid < (int)N) single(k0 + tid, tid);
        if (k0 + kTrSinkThreads + tid < (int)N) single(k0 + kTrSinkThreads + tid, kTrSinkThreads + tid);
      } else if (k0 + 2 * tid < (int)N) {
        auto sg4 = [&](int seg) { return reinterpret_cast<const float4*>(base + (size_t)seg * SEG)[tid]; };
        const float4 dks = sg4(sDK);
        if (isnan(dks.x) || isnan(dks.z)) {
          // a term outside the float range: per wavenumber, in order
          single(k0 + 2 * tid, 2 * tid);
          single(k0 + 2 * tid + 1, 2 * tid + 1);
        } else {
          df2 gx0 = z, gx1 = z;
          if (has_c0) {
            const float4 c = sg4(sC0);
            gx0 = df2{c.x, c.y};
            gx1 = df2{c.z, c.w};
          }
          if (has_c1) {
            const float4 c = sg4(sC1);
            gx0 = df_add(gx0, df2{c.x, c.y});
            gx1 = df_add(gx1, df2{c.z, c.w});
          }
          const float4 gz = sg4(sGZ);
          const df2 gT0 = df_mul(gx0, df_mul(df2{dks.x, dks.y}, df2{kLn2Hi, kLn2Lo}));
          const df2 gT1 = df_mul(gx1, df_mul(df2{dks.z, dks.w}, df2{kLn2Hi, kLn2Lo}));
#pragma unroll
          for (int q = 0; q < VP; ++q) {
            df2 x0 = z, x1 = z;
            if (q < S) {
              const float4 t = sg4(q);
              x0 = df_mul(gx0, df2{t.x, t.y});
              x1 = df_mul(gx1, df2{t.z, t.w});
            } else if (q < S + R) {
              const float4 sr = sg4(q);
              const float2 nr = rn_s[q - S];
              x0 = df_mul(gx0, df_mul(df2{sr.x, sr.y}, df2{nr.x, nr.y}));
              x1 = df_mul(gx1, df_mul(df2{sr.z, sr.w}, df2{nr.x, nr.y}));
            } else if (q == S + R) {
              x0 = gT0;
              x1 = gT1;
            } else if (q == S + R + 1) {
              x0 = df2{gz.x, gz.y};
              x1 = df2{gz.z, gz.w};
            } else if (q == S + R + 2) {
              x0 = gx0;
              x1 = gx1;
            }
            v[q] = df_add(df_add(v[q], x0), x1);
          }
        }
      }
      // this warp is done with the stage
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);
    }
    const df2 r = warp_reduce_scatter<VP>(v, lane);
    if (lane % G == 0) red[warp][lane / G] = make_float2(r.hi, r.lo);
  }
  __syncthreads();
  if (abort_s) {
    // wait (bounded) for the copies still in flight, then mark the block's sums invalid
    if (tid == 0)
      for (int it = max(0, issued_s - STAGES); it < issued_s; ++it)
        mbar_wait_bounded(&full[it % STAGES], (uint32_t)((it / STAGES) & 1));
    __syncthreads();
    if (tid < a.V) a.partial[bl * a.V + tid] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  if (tid < a.V) {
    df2 sum = {red[0][tid].x, red[0][tid].y};
#pragma unroll
    for (int w = 1; w < NW; ++w) sum = df_add(sum, df2{red[w][tid].x, red[w][tid].y});
    a.partial[bl * a.V + tid] = df_to_double(sum);
  }
}

// The adjoint kernels of one chunk, after the storing forward pass and the likelihood adjoint.
void transmission_adjoint_chunk(Model& m, const double* params_chunk, int nb, cudaStream_t st, double* grad_chunk,
                                int V) {
  const DeviceModel& dm = m.dm;
  const Workspace& w = m.ws;
  const GradWorkspace& g = m.gws;
  const ForwardTaps& tp = g.taps;
  const int L = m.L, S = m.acfg.S, P = m.acfg.nparam_total;
  const size_t N = m.N;
  const int tiles2a = (int)((N + 63) / 64);  // pass 2a: 64 wavenumbers per block (the d log L / dR partials)
  TrArgs a{w.lev, w.lsdf, w.ray_n, w.ev, reinterpret_cast<const float2*>(w.geom), tp.tr_geo, tp.dwT, g.gS,
           g.seed, tp.tr_c, tp.tr_T, tp.tr_qs, tp.tr_us, tp.tr_I, g.tr_gc, g.tr_gz, g.tr_rp, g.partial, V,
           tp.tr_ts, tp.tr_dk, g.tr_cs, m.acfg.cloud_kind == 1 ? 1 : m.acfg.cloud_kind == 2 ? 3 : 0};
  a.rays = w.rays;
  a.d = tp.tr_d;
  a.gd = g.tr_gd;
  if (g.tr_cs) {
    tr_cloud_shape_kernel<<<dim3(nb, (unsigned)((N + 255) / 256)), 256, 0, st>>>(dm, w.ev, g.tr_cs, a.nc);
    BGB_CUDA(cudaGetLastError());
  }
  if (m.annuli > 1) {
    tr_adjoint_pass2a_annuli<<<dim3(tiles2a, nb), 32 * kPass2aGroups, 0, st>>>(dm, a);
  } else {
    const size_t sm2a = (size_t)L * 32 * (sizeof(float4) + sizeof(short2)) + (size_t)3 * L * sizeof(float2);
    if (sm2a > 48 * 1024)
      BGB_CUDA(cudaFuncSetAttribute(tr_adjoint_pass2a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2a));
    tr_adjoint_pass2a<<<dim3(tiles2a, nb), 32 * kPass2aGroups, sm2a, st>>>(dm, a);
  }
  BGB_CUDA(cudaGetLastError());
  const size_t sm2 = (size_t)S * kTrSinkThreads * (sizeof(float2) + sizeof(double)) + (size_t)m.acfg.R * sizeof(float2);
  const int VP = V <= 8 ? 8 : V <= 16 ? 16 : 32;
  auto go2 = [&](auto kernel) {
    if (sm2 > 48 * 1024) BGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
    kernel<<<dim3(nb, L), kTrSinkThreads, sm2, st>>>(dm, a);
  };
  // wavenumbers in pairs (16-byte reads) when N is even; with the opacity terms stored, the
  // rows streamed through shared memory by bulk copies (16-byte aligned rows need N even)
  const bool pairs = (N % 2) == 0;
  // three stages of tiles in flight where two blocks per SM still fit, else two
  const int nseg = S + m.acfg.R + 4;
  const size_t stage_bytes = (size_t)nseg * (kStreamTile + 2) * sizeof(float2);
  const int stages = 3 * stage_bytes <= 110 * 1024 ? 3 : 2;
  const size_t sms = stages * stage_bytes;
  if (!g.tr_cs && tp.tr_ts && m.acfg.R <= 32 && nseg <= kStreamMaxSeg && sms <= 200 * 1024) {
    auto gos = [&](auto kernel) {
      BGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sms));
      kernel<<<dim3(nb, L), kTrSinkThreads + 32, sms, st>>>(dm, a, nseg);
    };
    if (stages == 3) {
      if (VP == 8) pairs ? gos(tr_adjoint_pass2b_stream<8, 3, true>) : gos(tr_adjoint_pass2b_stream<8, 3, false>);
      else if (VP == 16) pairs ? gos(tr_adjoint_pass2b_stream<16, 3, true>) : gos(tr_adjoint_pass2b_stream<16, 3, false>);
      else pairs ? gos(tr_adjoint_pass2b_stream<32, 3, true>) : gos(tr_adjoint_pass2b_stream<32, 3, false>);
    } else {
      if (VP == 8) pairs ? gos(tr_adjoint_pass2b_stream<8, 2, true>) : gos(tr_adjoint_pass2b_stream<8, 2, false>);
      else if (VP == 16) pairs ? gos(tr_adjoint_pass2b_stream<16, 2, true>) : gos(tr_adjoint_pass2b_stream<16, 2, false>);
      else pairs ? gos(tr_adjoint_pass2b_stream<32, 2, true>) : gos(tr_adjoint_pass2b_stream<32, 2, false>);
    }
  } else if (g.tr_cs) {  // non-grey cloud
    if (VP == 8) pairs ? go2(tr_adjoint_pass2b<8, true, true>) : go2(tr_adjoint_pass2b<8, false, true>);
    else if (VP == 16) pairs ? go2(tr_adjoint_pass2b<16, true, true>) : go2(tr_adjoint_pass2b<16, false, true>);
    else pairs ? go2(tr_adjoint_pass2b<32, true, true>) : go2(tr_adjoint_pass2b<32, false, true>);
  } else if (VP == 8) pairs ? go2(tr_adjoint_pass2b<8, true>) : go2(tr_adjoint_pass2b<8, false>);
  else if (VP == 16) pairs ? go2(tr_adjoint_pass2b<16, true>) : go2(tr_adjoint_pass2b<16, false>);
  else pairs ? go2(tr_adjoint_pass2b<32, true>) : go2(tr_adjoint_pass2b<32, false>);
  BGB_CUDA(cudaGetLastError());
  const size_t sma = (size_t)L * V * sizeof(double);
  if (sma > 48 * 1024)
    BGB_CUDA(cudaFuncSetAttribute(tr_atmosphere_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma));
  tr_atmosphere_adjoint_kernel<<<nb, 128, sma, st>>>(dm, params_chunk, P, w.lev, w.ev, g.partial, V, 1, g.tr_rp,
                                                     tiles2a, g.seed, grad_chunk);
  BGB_CUDA(cudaGetLastError());
}

}  // namespace bgb
