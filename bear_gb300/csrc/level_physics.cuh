// Level physics shared by the atmosphere kernel (atmosphere.cu) and its
// tangent/adjoint counterpart (adjoint.cu): the piecewise-polynomial
// temperature profile and the molecular weights of the chemical species.
// Functions have internal linkage, so each translation unit compiles its own
// copy with its own floating-point flags.
#pragma once

#include "model.h"

namespace bgb {

// PiecewisePolynomial::getValue src/additional/piecewise_poly.cpp:154-181 and
// Element::getValue / lagrangeBase :202-229. Linear in dof.
static __device__ double poly_value(const AtmosphereConfig& c, const double* dof, double x) {
  if (x > c.pp_dof_vertices[0] || x < c.pp_dof_vertices[c.pp_ndof - 1]) return 0.0;
  for (int i = 0; i < c.pp_ndof; ++i)
    if (c.pp_dof_vertices[i] == x) return dof[i];
  const int nd = c.pp_ndof_el;
  int el = 0;
  for (int e = 0; e < c.pp_nel; ++e)
    if (c.pp_el_vert[e * nd] > x && c.pp_el_vert[e * nd + nd - 1] < x) {
      el = e;
      break;
    }
  const double xl = c.pp_el_vert[el * nd], xr = c.pp_el_vert[el * nd + nd - 1];
  const double r = 2.0 * (x - xl) / (xr - xl) - 1.0;
  double y = 0;
  for (int i = 0; i < nd; ++i) {
    double l = 1;
    for (int j = 0; j < nd; ++j) {
      if (i == j) continue;
      l *= (r - c.pp_ref[j]) / (c.pp_ref[i] - c.pp_ref[j]);
    }
    y += dof[el * (nd - 1) + i] * l;
  }
  return y;
}

// Molecular weights in species-id order (src/chemistry/chem_species.h:30-90).
static __device__ __constant__ double kMolWeight[kSpeciesCount] = {
    0.0,      1.00784, 4.002602, 12.0107, 15.999,   55.845,   55.845,  40.078,  47.867,
    47.867,   2.01588, 18.01528, 44.01,   28.0101,  16.04246, 27.0253, 17.03052, 26.04,
    28.0134,  22.98977, 39.0983, 34.09099, 1.00784, 63.8664,  66.9409, 56.853,  34.08,
    40.3044,  42.981,  56.0774,  54.0040, 26.3209,  41.0859,  48.87484, 17.008,
    5.4857990907e-4, 50.9415, 50.9415, 54.938044, 28.085, 51.996, 51.996, 44.08, 60.08,
    64.066,   76.139};

// Chemistry::meanMolecularWeight src/chemistry/chemistry.h:47-59
static __device__ double mean_molecular_weight(const double* n) {
  double mu = 0;
  for (int j = 0; j < kSpeciesCount; ++j) mu += n[j] / n[SP_TOTAL] * kMolWeight[j];
  return mu;
}

// Solar H2 and He abundances of BackgroundChemistry
// (src/chemistry/background_chemistry.cpp:72-137).
constexpr double kSolarH2 = 0.5;
constexpr double kSolarHe = 0.085114;

}  // namespace bgb
