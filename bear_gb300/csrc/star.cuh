// Stellar spectrum of the secondary-eclipse (occultation) model on the device:
// the blackbody flux at one wavenumber and the trilinear interpolation of a
// stellar-spectrum grid over (T_eff, log g, [M/H]).
#pragma once

#include "model.h"
#include "physics.cuh"

namespace bgb {

// pi B_nu(T_eff) 1e-3 (StarBlackBody::calcFlux src/forward_model/stellar_spectrum/star_blackbody.cpp:35-47:
// the Planck function in W m^-2 cm), FP64.
__device__ __forceinline__ double star_blackbody_fp64(const DeviceModel& dm, int k, double teff) {
  return __ldg(&dm.planck_c1[k]) / (exp(__ldg(&dm.planck_c2[k]) / teff) - 1.0) * kPi * 1e-3;
}

// The same in double-float arithmetic (about 48 significant bits); invT = 1 / T_eff.
__device__ __forceinline__ double star_blackbody_df(const DeviceModel& dm, int k, df2 invT, const ExpTables& et) {
  const float2 c1 = __ldg(&dm.planck_c1_df[k]), c2 = __ldg(&dm.planck_c2l_df[k]);
  return planck_df(df2{c1.x, c1.y}, df2{c2.x, c2.y}, invT, et.hi, et.lo) * kPi * 1e-3;
}

// d/dT_eff of pi B_nu(T_eff) 1e-3: B x e^x / (e^x - 1) / T_eff, x = c2 / T_eff (FP64).
__device__ __forceinline__ double star_blackbody_dT(const DeviceModel& dm, int k, double teff) {
  const double x = __ldg(&dm.planck_c2[k]) / teff;
  const double em1 = expm1(x);
  const double B = __ldg(&dm.planck_c1[k]) / em1 * kPi * 1e-3;
  return B * x * ((em1 + 1.0) / em1) / teff;
}

// Cell of a stellar-grid parameter: the reference clamps the value to the nodes,
// takes (0, 0) / (n-1, n-1) at the ends, the node itself twice when it is hit
// exactly, else the bracketing pair (StellarSpectrumGrid::findClosestGridPoints and
// calcFlux src/forward_model/stellar_spectrum/stellar_spectrum_grid.cpp:245-298), and the
// weight (x - x0) / (x1 - x0), 0 when x == x0 (aux::triLinearInterpolation
// src/additional/aux_functions.cpp:290-318). dw receives d weight / d x (0 outside the
// open cell, where the clamp or an exact node fixes the weight).
__device__ __forceinline__ void star_axis_cell(const double* __restrict__ nodes, int n, double x, int& i0,
                                               int& i1, double& w, double& dw) {
  double xc = x;
  const bool below = xc < nodes[0], above = xc > nodes[n - 1];
  if (below) xc = nodes[0];
  if (above) xc = nodes[n - 1];
  dw = 0.0;
  if (xc <= nodes[0]) {
    i0 = i1 = 0;
  } else if (xc >= nodes[n - 1]) {
    i0 = i1 = n - 1;
  } else {
    int j = 0;
    while (nodes[j] < xc) ++j;  // lower_bound: first node >= x
    i1 = j;
    i0 = nodes[j] != xc ? j - 1 : j;
  }
  const double x0 = nodes[i0], x1 = nodes[i1];
  w = (xc - x0) / (x1 - x0);
  if (xc == x0) w = 0.0;
  else dw = 1.0 / (x1 - x0);
}

// Eight corner spectra and the three weights of one parameter set (sp: T_eff, log g, [M/H]);
// corner order c000, c100, c010, c110, c001, c101, c011, c111 (x = T_eff, y = log g, z = [M/H]).
struct StarCell {
  int c[8];
  double w[3];
  double dw[3];
};

__device__ __forceinline__ StarCell star_grid_cell(const DeviceModel& dm, const double* sp) {
  const int n0 = dm.star_n[0], n1 = dm.star_n[1], n2 = dm.star_n[2];
  int t[2], g[2], q[2];
  StarCell s;
  star_axis_cell(dm.star_axes, n0, sp[0], t[0], t[1], s.w[0], s.dw[0]);
  star_axis_cell(dm.star_axes + n0, n1, sp[1], g[0], g[1], s.w[1], s.dw[1]);
  star_axis_cell(dm.star_axes + n0 + n1, n2, sp[2], q[0], q[1], s.w[2], s.dw[2]);
  for (int i = 0; i < 8; ++i) s.c[i] = (t[i & 1] * n1 + g[(i >> 1) & 1]) * n2 + q[i >> 2];
  return s;
}

// Trilinear interpolation in the reference's operation order; v[i] = value of corner i.
__device__ __forceinline__ double star_trilinear(const double v[8], const double w[3]) {
  const double xd = w[0], yd = w[1], zd = w[2];
  const double c00 = v[0] * (1. - xd) + v[1] * xd;
  const double c01 = v[4] * (1. - xd) + v[5] * xd;
  const double c10 = v[2] * (1. - xd) + v[3] * xd;
  const double c11 = v[6] * (1. - xd) + v[7] * xd;
  const double c0 = c00 * (1. - yd) + c10 * yd;
  const double c1 = c01 * (1. - yd) + c11 * yd;
  return c0 * (1. - zd) + c1 * zd;
}

// Derivatives of the trilinear value along the three weights.
__device__ __forceinline__ void star_trilinear_dw(const double v[8], const double w[3], double d[3]) {
  const double xd = w[0], yd = w[1], zd = w[2];
  const double c00 = v[0] * (1. - xd) + v[1] * xd, c01 = v[4] * (1. - xd) + v[5] * xd;
  const double c10 = v[2] * (1. - xd) + v[3] * xd, c11 = v[6] * (1. - xd) + v[7] * xd;
  const double c0 = c00 * (1. - yd) + c10 * yd, c1 = c01 * (1. - yd) + c11 * yd;
  const double e00 = v[1] - v[0], e01 = v[5] - v[4], e10 = v[3] - v[2], e11 = v[7] - v[6];
  const double e0 = e00 * (1. - yd) + e10 * yd, e1 = e01 * (1. - yd) + e11 * yd;
  d[0] = e0 * (1. - zd) + e1 * zd;
  d[1] = (c10 - c00) * (1. - zd) + (c11 - c01) * zd;
  d[2] = c1 - c0;
}

}  // namespace bgb
