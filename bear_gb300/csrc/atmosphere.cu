// Device-side atmosphere: temperature profile, chemistry, hydrostatic altitude,
// grey cloud and the opacity-table stencils, one thread block per evaluation.
//
// Compiled with --fmad=false: every product and sum is rounded separately,
// like the reference's host code, so that the discrete decisions made here
// (temperature clamp, table brackets, cloud layer indices) agree bit for bit
// with the reference on the same parameters.

#include "model.h"
#include "dfloat.cuh"
#include "level_physics.cuh"

namespace bgb {


// One block per evaluation, blockDim.x >= L. Dynamic shared memory: 4 L doubles.
// dwT (optional, B x L x S) receives the temperature derivative of each stencil's
// temperature weight.
__global__ void __launch_bounds__(kMaxLevels) atmosphere_kernel(DeviceModel dm, const double* __restrict__ params, int P,
                                  LevelInfo* __restrict__ lev, LevelSpecies* __restrict__ ls,
                                  LevelSpeciesDF* __restrict__ lsdf, double* __restrict__ ray_n,
                                  EvalInfo* __restrict__ ev, float2* __restrict__ dwT) {
  const AtmosphereConfig& c = *dm.cfg;
  const int b = blockIdx.x;
  const int l = threadIdx.x;
  const int L = c.L, S = c.S;
  extern __shared__ double smem[];
  double* sT = smem;
  double* smmw = smem + L;
  double* sz = smem + 2 * L;
  double* sH = smem + 3 * L;
  __shared__ int s_neglect;
  __shared__ int s_top, s_bottom;
  __shared__ double s_cloud_layer;
  if (l == 0) s_neglect = 0;
  __syncthreads();

  const double* par = params + (size_t)b * P;
  const double* gen = par;
  const double* chem = par + c.nparam_general;
  const double* temp = chem + c.nparam_chem;
  const double* cloud = temp + c.nparam_temp;
  // EmissionModel::calcAtmosphereStructure src/forward_model/emission/emission.cpp:158-189,
  // TransmissionModel::calcAtmosphereStructure src/forward_model/transmission/transmission.cpp:150-194
  const double g = pow(10.0, gen[0]);

  int neglect = 0;
  if (l < L) {
    const double p = dm.pressure[l];
    // temperature: PiecewisePolynomialTemperature::calcProfile
    // src/temperature/piecewise_poly_temperature.cpp:49-84, ConstantTemperature
    // src/temperature/constant_temperature.h:37-44
    double T;
    if (c.temp_poly) {
      double dof[kMaxPolyDof];
      dof[0] = temp[0];
      for (int i = 1; i < c.pp_ndof; ++i) dof[i] = dof[i - 1] * temp[i];
      T = poly_value(c, dof, dm.log10p[l]);
      if (T < 50) {
        T = 50;
        neglect = 1;
      }
    } else {
      T = temp[0];
    }
    // chemistry modules in configuration order
    double n[kSpeciesCount];
    for (int j = 0; j < kSpeciesCount; ++j) n[j] = 0.0;
    double mmw = 0.0;
    int pidx = 0;
    for (int m = 0; m < c.nchem; ++m) {
      if (c.chem_kind[m] == 0) {
        // IsoprofileChemistry::calcChemicalComposition src/chemistry/isoprofile_chemistry.cpp:87-119
        n[SP_TOTAL] = p * 1.e6 / kBoltzmann / T;
        for (int j = 0; j < c.chem_nsp[m]; ++j) n[c.chem_sp[m][j]] = n[SP_TOTAL] * chem[pidx + j];
        if (!c.chem_na_free[m]) n[SP_Na] = n[SP_K] * 16.2181;
        mmw = mean_molecular_weight(n);
        // Chemistry::checkMixingRatios src/chemistry/chemistry.h:61-76
        double sum = 0;
        for (int j = 1; j < kSpeciesCount; ++j) sum += n[j] / n[SP_TOTAL];
        if (sum > 1 + 1e-10) neglect = 1;
        pidx += c.chem_nsp[m];
      } else {
        // BackgroundChemistry::calcChemicalComposition src/chemistry/background_chemistry.cpp:72-137
        const double sh2 = kSolarH2, she = kSolarHe;
        const double sh2he = sh2 + she;
        n[SP_TOTAL] = p * 1.e6 / kBoltzmann / T;
        double bg = 1.0;
        for (int j = 1; j < kSpeciesCount; ++j) {
          if (c.chem_bg_h2he[m]) {
            if (j != SP_H2 && j != SP_He) bg -= n[j] / n[SP_TOTAL];
          } else if (j != c.chem_bg_sp[m]) {
            bg -= n[j] / n[SP_TOTAL];
          }
        }
        if (bg < 0) {
          neglect = 1;
          bg = 0;
        }
        if (c.chem_bg_h2he[m]) {
          const double xh2 = bg * sh2 / sh2he;
          const double xhe = bg * she / sh2he;
          n[SP_H2] = n[SP_TOTAL] * xh2;
          n[SP_He] = n[SP_TOTAL] * xhe;
        } else {
          n[c.chem_bg_sp[m]] = n[SP_TOTAL] * bg;
        }
        mmw = mean_molecular_weight(n);
      }
    }
    if (c.transmission && c.fit_mmw) mmw = gen[3];  // Atmosphere::calcAtmosphereStructure :126-187
    sT[l] = T;
    smmw[l] = mmw;
    // number densities of the opacity species (OpacitySpecies::calcTransportCoefficients
    // src/transport_coeff/opacity_species.cpp:407-410: index species times collision partners)
    for (int s = 0; s < S; ++s) {
      double nd = n[c.sp_index[s]];
      if (c.sp_partner[s][0] >= 0) nd *= n[c.sp_partner[s][0]];
      if (c.sp_partner[s][1] >= 0) nd *= n[c.sp_partner[s][1]];
      ls[((size_t)b * L + l) * S + s].n = nd;
      // log2 of the density for the double-float path; a zero density skips the
      // species like the reference's early return (opacity_species.cpp:412)
      LevelSpeciesDF& f = lsdf[((size_t)b * L + l) * S + s];
      if (nd > 0) {
        const df2 lg = df_from_double(log2(nd));
        f.lg2n_hi = lg.hi;
        f.lg2n_lo = lg.lo;
      } else {
        f.lg2n_hi = kNoSpecies;
        f.lg2n_lo = 0.0f;
      }
    }
    double* rn = ray_n + ((size_t)b * L + l) * c.R;
    for (int r = 0; r < c.R_ray; ++r) rn[r] = n[c.ray_index[r]];
    if (c.hm) {
      // H- continuum coefficients (GasHm::calcContinuumAbsorption src/transport_coeff/h_m.cpp:36-53:
      // kappa_bf n(H-) + kappa_ff P_e n(H), P_e = n(e-) k T; nothing when n(H-) = 0)
      double* hc = rn + c.R_ray;
      const double nhm = n[SP_Hm];
      hc[0] = nhm;
      const double pn = n[SP_e] * kBoltzmann * T * n[SP_H];
      for (int i = 1; i < kHmTerms; ++i) hc[i] = nhm == 0.0 ? 0.0 : pow(5040.0 / T, (i + 1) / 2.0) * pn;
    }
    if (neglect) atomicOr(&s_neglect, 1);
  }
  __syncthreads();

  // hydrostatic altitude: Atmosphere::calcAltitude src/forward_model/atmosphere/atmosphere.cpp:288-307,
  // calcAltitudeVariableGravity :311-334; scale height calcScaleHeight :353-360.
  double dz_l = 0.0;
  if (l >= 1 && l < L && !c.var_g) {
    const double rho_i = smmw[l] * dm.pressure[l] * 1e6 / (kGasConst * sT[l]);
    const double rho_m = smmw[l - 1] * dm.pressure[l - 1] * 1e6 / (kGasConst * sT[l - 1]);
    dz_l = (1.0 / (rho_i * g) + 1.0 / (rho_m * g)) * 0.5 * (dm.pressure[l - 1] * 1e6 - dm.pressure[l] * 1e6);
  }
  if (l < L) sH[l] = dz_l;  // staged through sH
  __syncthreads();
  if (l == 0) {
    sz[0] = 0.0;
    if (!c.var_g) {
      for (int i = 1; i < L; ++i) sz[i] = sz[i - 1] + sH[i];
    } else {
      const double R0 = gen[1];
      for (int i = 1; i < L; ++i) {
        const double rho_i = smmw[i] * dm.pressure[i] * 1e6 / (kGasConst * sT[i]);
        const double rho_m = smmw[i - 1] * dm.pressure[i - 1] * 1e6 / (kGasConst * sT[i - 1]);
        const double lr = R0 + sz[i - 1];
        const double ratio = R0 / lr;
        const double gi = g * (ratio * ratio);
        const double dz = (1.0 / (rho_i * gi) + 1.0 / (rho_m * gi)) * 0.5 * (dm.pressure[i - 1] * 1e6 - dm.pressure[i] * 1e6);
        sz[i] = sz[i - 1] + dz;
      }
    }
  }
  __syncthreads();
  if (l < L) sH[l] = kGasConst * sT[l] / (smmw[l] * g);
  __syncthreads();

  // grey cloud: GreyCloudModel::opticalProperties / cloudPosition
  // src/cloud_model/grey_cloud_model.cpp:59-195
  if (l == 0) {
    int top = 0, bottom = 0;
    double per = 0.0;
    if (c.cloud) {
      // power law and KH clouds place the layers like the grey cloud
      // (src/cloud_model/power_law_cloud_model.cpp:69-121, kh_cloud_model.cpp:69-133)
      const int it = c.cloud_kind == 0 ? 1 : c.cloud_kind == 1 ? 2 : 4;
      double tau = cloud[0];
      const double ptop = cloud[it];
      const double pbot = c.cloud_fb ? 0.0 : ptop * cloud[it + 1];
      if (tau < 0) tau = 0;
      unsigned ti = 0, bi = 0;
      for (int i = 0; i < L - 1; ++i)
        if ((dm.pressure[i] > ptop && dm.pressure[i + 1] < ptop) || dm.pressure[i] == ptop) ti = i;
      if (c.cloud_fb) {
        if (ptop < dm.pressure[L - 1]) ti = L - 1;
        double ba = sz[ti] - sH[ti];
        if (ba < 0) ba = 0;
        for (int i = 0; i < L - 1; ++i)
          if ((sz[i] < ba && sz[i + 1] > ba) || sz[i] == ba) bi = i;
        if (ti == bi) bi -= 2;
        if (ti == bi) bi -= 2;
        if (ti < 2) { ti = 2; bi = 0; }
      } else {
        for (int i = 0; i < L - 1; ++i)
          if ((dm.pressure[i] > pbot && dm.pressure[i + 1] < pbot) || dm.pressure[i] == pbot) bi = i;
        if (ptop <= dm.pressure[L - 1]) ti = L - 1;
        if (pbot >= dm.pressure[0]) bi = 0;
        if (ti == bi) bi -= 2;
        if (ti < 2) { ti = 2; bi = 0; }
      }
      per = tau / (double)(ti - bi);
      top = (int)ti;
      bottom = (int)bi;
    }
    s_top = top;
    s_bottom = bottom;
    s_cloud_layer = per;
    EvalInfo e;
    if (c.occultation) {
      // OccultationModel::calcModelGPU src/forward_model/secondary_eclipse/secondary_eclipse.cpp:262-285:
      // the planet's spectrum unscaled; radius holds R_p / R_s
      e.scaling = 1.0;
      e.radius = gen[1];
      e.star_radius = 0.0;
    } else {
      // EmissionModel::radiusDistanceScaling src/forward_model/emission/emission.cpp:108-120
      double sc = kRJupiter / gen[2];
      e.scaling = sc * sc * gen[1];
      e.radius = gen[1];
      e.star_radius = gen[2];
    }
    // Retrieval::logLikelihood error inflation src/retrieval/retrieval.cpp:332-335
    e.inflation = c.error_inflation ? pow(10.0, par[P - 1]) : 0.0;
    e.neglect = s_neglect;
    e.cloud_top = top;
    e.cloud_bottom = bottom;
    e.pad = 0;
    for (int i = 0; i < 4; ++i) e.cs[i] = 0.0;
    if (c.cloud && c.cloud_kind == 1) {
      e.cs[0] = cloud[1];                          // exponent
      e.cs[3] = pow(c.cloud_ref_wl, cloud[1]);     // reference_value
    } else if (c.cloud && c.cloud_kind == 2) {
      const double q0 = cloud[1], a0 = cloud[2];
      e.cs[0] = q0;
      e.cs[1] = a0;
      e.cs[2] = 2 * kPi * cloud[3];                // 2 pi particle size
      const double xr = e.cs[2] / c.cloud_ref_wl;  // reference size parameter
      e.cs[3] = q0 * pow(xr, -a0) + pow(xr, 0.2);  // reference_q
    }
    ev[b] = e;
  }
  __syncthreads();

  if (l < L) {
    const double T = sT[l];
    LevelInfo li;
    li.T = T;
    li.invT = 1.0 / T;
    li.z = sz[l];
    li.dz = (l + 1 < L) ? sz[l + 1] - sz[l] : 0.0;
    double cl = 0.0;
    if (c.cloud) {
      // layer l holds tau / (top - bottom) for bottom < l <= top (and l < L - 1)
      const unsigned top = (unsigned)s_top, bottom = (unsigned)s_bottom;
      auto layer_tau = [&](int j) -> double {
        return ((unsigned)j <= top && (unsigned)j > bottom && j < L - 1) ? s_cloud_layer : 0.0;
      };
      if (!c.transmission) cl = layer_tau(l);
      else if (l >= 1) cl = layer_tau(l - 1) / (sz[l] - sz[l - 1]);  // CloudModel::convertOpticalDepth src/cloud_model/cloud_model.h:67-88
    }
    li.cloud = cl;
    const df2 it = df_from_double(li.invT);
    li.invT_hi = it.hi;
    li.invT_lo = it.lo;
    const df2 dh = df_from_double(0.5 * li.dz);
    li.dzh_hi = dh.hi;
    li.dzh_lo = dh.lo;
    const df2 cd = df_from_double(cl);
    li.cloud_hi = cd.hi;
    li.cloud_lo = cd.lo;
    lev[(size_t)b * L + l] = li;
    // table stencils: OpacitySpecies::findClosestDataPoints src/transport_coeff/opacity_species.cpp:160-273
    for (int s = 0; s < S; ++s) {
      const double* Tn = dm.table_T + c.sp_T_off[s];
      const int nT = c.sp_nT[s];
      int lo = 0, up = 0;
      if (T < Tn[0]) {
        lo = up = 0;
      } else if (T > Tn[nT - 1]) {
        lo = up = nT - 1;
      } else {
        for (int i = 0; i < nT; ++i) {
          if (Tn[i] == T) { lo = up = i; break; }
          if (Tn[i] < T && Tn[i + 1] > T) { lo = i; up = i + 1; break; }
        }
      }
      LevelSpecies& e = ls[((size_t)b * L + l) * S + s];
      const int ilo = c.sp_pb_off[s] + lo * L + l;
      const int iup = c.sp_pb_off[s] + up * L + l;
      e.row[0] = dm.pb_row0[ilo];
      e.row[1] = dm.pb_row1[ilo];
      e.row[2] = dm.pb_row0[iup];
      e.row[3] = dm.pb_row1[iup];
      e.wp_lo = dm.pb_w[ilo];
      e.wp_hi = dm.pb_w[iup];
      e.wT = (lo != up) ? (T - Tn[lo]) / (Tn[up] - Tn[lo]) : 0.0;
      LevelSpeciesDF& f = lsdf[((size_t)b * L + l) * S + s];
      const df2 t = df_from_double(e.wT);
      f.lrow[0] = ilo;  // level-table rows: the pressure-bracket indices
      f.lrow[1] = iup;
      f.pad[0] = f.pad[1] = 0;
      f.wT_hi = t.hi;
      f.wT_lo = t.lo;
      // d wT / dT for the adjoint (0 when T is clamped to the end of the table)
      if (dwT) {
        const df2 dw = df_from_double(lo != up ? 1.0 / (Tn[up] - Tn[lo]) : 0.0);
        dwT[((size_t)b * L + l) * S + s] = make_float2(dw.hi, dw.lo);
      }
    }
  }
}

}  // namespace bgb
