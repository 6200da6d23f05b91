// Contribution functions of emission and secondary-eclipse models (post-processing).
//
// Reference: contributionFunctionDevice src/CUDA_kernels/contribution_function_kernels.cu:21-66,
// driven by EmissionModel::postProcessContributionFunctions
// src/forward_model/emission/emission_post_process.cpp:330-376 (and its secondary-eclipse
// twin src/forward_model/secondary_eclipse/secondary_eclipse_post_process.cpp:255-305).
// Per wavenumber, from the top level down, with the gas absorption (no cloud):
//   dtau_i = (z_i - z_{i-1}) (kappa_i + kappa_{i-1}) / 2,  t_i = exp(-dtau_i)
//   CF_i   = 2 pi B(T_i) (1 - t_i) prod_{j > i} t_j      (i = L-1 .. 1; CF_0 = 0)
// Each level's CF is then binned through the observations with wavelength
// integration (is_flux = false in the reference), here on the host with the
// observation operator composed for that mode.
//
// Differences from the reference: its opacities are stored as floats
// (OpacityCalculation::absorption_coeff_gpu), ours are double-float (FP64 in precision
// mode 1), so results agree to float rounding of the opacity; its level-0 row is
// never written (uninitialised device memory), ours is 0.

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/bear_gb300.h"
#include "model.h"
#include "rt_common.cuh"

namespace bgb {

template <bool DF>
__global__ void __launch_bounds__(128) contribution_kernel(DeviceModel dm, const LevelInfo* __restrict__ lev,
                                                           const LevelSpecies* __restrict__ ls,
                                                           const LevelSpeciesDF* __restrict__ lsdf,
                                                           const double* __restrict__ ray_n,
                                                           double* __restrict__ cf) {
  __shared__ ExpTables et;
  if (DF) load_exp_tables(et);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= dm.N) return;
  const int L = dm.L, S = dm.S;
  const size_t N = dm.N;
  auto kappa = [&](int l) {
    double v;
    if (DF) {
      const Kappa kp = level_kappa_df(dm.ltab, N, lsdf + (size_t)l * S, S, k, et);
      v = df_to_double(kp.v) + kp.wide;
    } else {
      v = level_absorption_fp64(dm.table64, N, ls + (size_t)l * S, S, k);
    }
    // H- continuum rows (absorption); Rayleigh rows are scattering and stay out
    for (int r = dm.R_ray; r < dm.R; ++r) v += __ldg(&dm.rayleigh[(size_t)r * N + k]) * ray_n[(size_t)l * dm.R + r];
    return v;
  };
  const double c1 = __ldg(&dm.planck_c1[k]), c2 = __ldg(&dm.planck_c2[k]);
  double tcum = 1.0;
  double kap_up = kappa(L - 1);
  for (int i = L - 1; i > 0; --i) {
    const double kap_lo = kappa(i - 1);
    const double dtau = lev[i - 1].dz * (kap_up + kap_lo) / 2.;
    const double t = exp(-dtau);
    const double B = c1 / (exp(c2 / lev[i].T) - 1.0);
    cf[(size_t)i * N + k] = 2 * kPi * B * (1.0 - t) * tcum;
    tcum *= t;
    kap_up = kap_lo;
  }
  cf[k] = 0.0;
}

// Contribution functions of the evaluation held in the model's workspace (batch row 0,
// left there by a plain-path evaluation on the same stream). spectrum (L x N) and bins
// (L x M, each level's bins in the caller's order) are host buffers; either may be null.
void contribution_functions(Model& m, cudaStream_t st, double* spectrum, double* bins) {
  if (m.transmission) throw Error(BEAR_ERR_UNSUPPORTED, "contribution functions exist for emission and secondary-eclipse models");
  const size_t L = m.L, N = m.N;
  BGB_CUDA(cudaSetDevice(m.device));
  if (!m.d_cf) {
    BGB_CUDA(cudaMalloc(&m.d_cf, L * N * sizeof(double)));
    m.allocations.push_back(m.d_cf);
  }
  const Workspace& w = m.ws;
  const unsigned grid = (unsigned)((N + 127) / 128);
  if (m.precision == 1) contribution_kernel<false><<<grid, 128, 0, st>>>(m.dm, w.lev, w.ls, w.lsdf, w.ray_n, m.d_cf);
  else contribution_kernel<true><<<grid, 128, 0, st>>>(m.dm, w.lev, w.ls, w.lsdf, w.ray_n, m.d_cf);
  BGB_CUDA(cudaGetLastError());
  std::vector<double> hr(L * N);
  BGB_CUDA(cudaMemcpyAsync(hr.data(), m.d_cf, L * N * sizeof(double), cudaMemcpyDeviceToHost, st));
  BGB_CUDA(cudaStreamSynchronize(st));
  if (spectrum) std::copy(hr.begin(), hr.end(), spectrum);
  if (!bins) return;
  if (m.cf_W.empty()) {
    // observation operators with wavelength integration (the reference bins contribution
    // functions with is_flux = false)
    for (const auto& o : m.obs) {
      std::vector<int> k0, len;
      std::vector<long long> off;
      compose_operator_rows(m, o, false, m.cf_W, k0, len, off);
      for (int b = 0; b < o.n; ++b) {
        m.cf_k0.push_back(k0[b]);
        m.cf_len.push_back(len[b]);
        m.cf_off.push_back(off[b]);
        m.cf_out.push_back(o.out_offset + (o.ascending ? o.n - 1 - b : b));
      }
    }
  }
  const size_t M = m.M;
  for (size_t l = 0; l < L; ++l) {
    const double* F = hr.data() + l * N;
    for (size_t r = 0; r < M; ++r) {
      const double* wr = m.cf_W.data() + m.cf_off[r];
      double s = 0.0;
      for (int j = 0; j < m.cf_len[r]; ++j) s += wr[j] * F[m.cf_k0[r] + j];
      bins[l * M + (size_t)m.cf_out[r]] = s;
    }
  }
}

}  // namespace bgb
