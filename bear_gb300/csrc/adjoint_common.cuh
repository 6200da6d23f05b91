// Helpers shared by the adjoint kernels (adjoint.cu for emission,
// adjoint_transmission.cu for transmission): error checking, accumulator types
// (double-float or FP64), the warp reduce-scatter of per-level sinks.
#pragma once

#include <string>

#include "../../include/bear_gb300.h"
#include "level_physics.cuh"
#include "model.h"
#include "rt_common.cuh"

namespace bgb {

constexpr int kAdjThreads = 128;  // threads (wavenumbers) per block of the emission adjoint kernel
constexpr double kLn10 = 2.302585092994045684;

// ------------------------------------------------------------------ accumulators
// The per-level sinks are summed either as double-floats (FP32 pipe) or in FP64.
__device__ __forceinline__ df2 acc_add(df2 a, df2 b) { return df_add(a, b); }
__device__ __forceinline__ double acc_add(double a, double b) { return a + b; }
__device__ __forceinline__ df2 acc_shfl_xor(df2 v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ double acc_shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double acc_to_double(df2 v) { return df_to_double(v); }
__device__ __forceinline__ double acc_to_double(double v) { return v; }

template <bool DF>
struct AccType {
  typedef double type;
  static __device__ __forceinline__ double from(double x) { return x; }
  static __device__ __forceinline__ double zero() { return 0.0; }
};
template <>
struct AccType<true> {
  typedef df2 type;
  static __device__ __forceinline__ df2 from(double x) { return df_from_double(x); }
  static __device__ __forceinline__ df2 zero() { return df2{0.0f, 0.0f}; }
};

// Warp reduce-scatter of VP values (VP = 8, 16 or 32): each halving step keeps
// half of the values, sends the other half to the partner lane and adds what
// comes back, so the warp does VP - 1 additions per lane instead of 5 VP.
// Afterwards lane j holds the warp total of value j / (32 / VP).
template <int VP, class A>
__device__ __forceinline__ A warp_reduce_scatter(A (&v)[VP], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    const int cnt = VP >> s;
    if (cnt >= 2) {
      const int h = cnt / 2;
      const bool upper = (lane & o) != 0;
#pragma unroll
      for (int i = 0; i < h; ++i) {
        const A send = upper ? v[i] : v[i + h];
        const A keep = upper ? v[i + h] : v[i];
        v[i] = acc_add(keep, acc_shfl_xor(send, o));
      }
    } else {
      v[0] = acc_add(v[0], acc_shfl_xor(v[0], o));
    }
  }
  return v[0];
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------------------------ level tangents
// Mixing ratios X_j = n_j / n_total after the chemistry modules (level independent
// for isoprofile and background chemistry) and their derivative along chemistry
// parameter tc (-1: none). IsoprofileChemistry::calcChemicalComposition
// src/chemistry/isoprofile_chemistry.cpp:87-119, BackgroundChemistry
// src/chemistry/background_chemistry.cpp:72-137, Chemistry::meanMolecularWeight
// src/chemistry/chemistry.h:47-59.
static __device__ void chemistry_tangent(const AtmosphereConfig& c, const double* chem, int tc, double* X, double* dX,
                                  double& mmw, double& dmmw) {
  for (int j = 0; j < kSpeciesCount; ++j) {
    X[j] = 0.0;
    dX[j] = 0.0;
  }
  X[SP_TOTAL] = 1.0;
  mmw = dmmw = 0.0;
  int pidx = 0;
  for (int m = 0; m < c.nchem; ++m) {
    if (c.chem_kind[m] == 0) {
      for (int j = 0; j < c.chem_nsp[m]; ++j) {
        X[c.chem_sp[m][j]] = chem[pidx + j];
        dX[c.chem_sp[m][j]] = (tc == pidx + j) ? 1.0 : 0.0;
      }
      if (!c.chem_na_free[m]) {
        X[SP_Na] = X[SP_K] * 16.2181;
        dX[SP_Na] = dX[SP_K] * 16.2181;
      }
      pidx += c.chem_nsp[m];
    } else {
      double bg = 1.0, dbg = 0.0;
      for (int j = 1; j < kSpeciesCount; ++j) {
        const bool other = c.chem_bg_h2he[m] ? (j != SP_H2 && j != SP_He) : (j != c.chem_bg_sp[m]);
        if (other) {
          bg -= X[j];
          dbg -= dX[j];
        }
      }
      if (bg < 0) bg = dbg = 0.0;
      if (c.chem_bg_h2he[m]) {
        const double f2 = kSolarH2 / (kSolarH2 + kSolarHe), fe = kSolarHe / (kSolarH2 + kSolarHe);
        X[SP_H2] = bg * f2;
        dX[SP_H2] = dbg * f2;
        X[SP_He] = bg * fe;
        dX[SP_He] = dbg * fe;
      } else {
        X[c.chem_bg_sp[m]] = bg;
        dX[c.chem_bg_sp[m]] = dbg;
      }
    }
    mmw = dmmw = 0.0;
    for (int j = 1; j < kSpeciesCount; ++j) {
      mmw += X[j] * kMolWeight[j];
      dmmw += dX[j] * kMolWeight[j];
    }
  }
}

}  // namespace bgb
