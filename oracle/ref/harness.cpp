// Driver that runs the reference's own FP64 CPU likelihood path on a case
// directory and writes its outputs as raw float64 files. Test infrastructure:
// it is compiled against the reference sources by oracle/ref/Makefile and is
// used only to produce golden vectors and to pin the C oracle.
//
// Case directory layout (written by oracle/refcase.py):
//   config.txt        "key value..." lines (same keys as the product config)
//   observations.txt  one block per observation (see read_observations)
//   params.txt        "P S" then S rows of P physical parameters
// Outputs written into the same directory:
//   ref_grid.bin      N model wavenumbers  (SpectralGrid::wavenumber_list)
//   ref_spectrum.bin  S x N high-res spectrum (ForwardModel::calcModel, true)
//   ref_obs.bin       S x M binned spectrum (all observations concatenated)
//   ref_loglike.bin   S log-likelihoods (Retrieval::computeLikelihood)
//   ref_neglect.bin   S neglect flags as float64
//   ref_setup.txt     per observation: band edge indices, convolution windows
// With --priors the driver instead reads priors.txt ("type description unit n p0 [p1]"
// per parameter, unit "-" for none; linked priors give the 1-based index they follow)
// and cube.txt ("P S" then S hypercube rows), builds the Retrieval with those priors and
// writes Retrieval::convertCubeParameters (src/retrieval/multinest_loglike.cpp:41-97)
// of every row: ref_prior_parameter.bin and ref_prior_physical.bin (S x P).
//
// Objects are built the way pyBeAR builds them
// (python/src/bear_python_wrapper.cpp:114-129): GlobalConfig 7-argument
// constructor, EmissionModelConfig / TransmissionModelConfig, ObservationInput
// and PriorConfig, then Retrieval(config, model_config, observations, priors).

#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "case_io.h"
#include "forward_model/forward_model.h"
#include "retrieval/priors.h"
#include "retrieval/retrieval.h"

namespace {

void write_bin(const std::string& path, const std::vector<double>& v) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) throw std::runtime_error("cannot write " + path);
  if (!v.empty()) std::fwrite(v.data(), sizeof(double), v.size(), fp);
  std::fclose(fp);
}

std::vector<bear::PriorConfig> read_priors(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::vector<bear::PriorConfig> out;
  std::string type, desc, unit;
  size_t n = 0;
  while (f >> type >> desc >> unit >> n) {
    std::vector<double> p(n);
    for (auto& x : p) f >> x;
    if (unit == "-")
      out.emplace_back(type, desc, p);
    else
      out.emplace_back(type, desc, p, unit);
  }
  return out;
}

int run_priors(const std::string& dir) {
  refcase::RefCase rc = refcase::load_case(dir);
  std::vector<bear::PriorConfig> priors = read_priors(dir + "priors.txt");
  std::ifstream cf(dir + "cube.txt");
  size_t P = 0, S = 0;
  cf >> P >> S;
  std::vector<std::vector<double>> cube(S, std::vector<double>(P));
  for (auto& row : cube)
    for (auto& x : row) cf >> x;
  bear::Retrieval retrieval(rc.cfg, rc.model_cfg, rc.obs, priors);
  std::vector<double> par_all, phys_all;
  for (auto& row : cube) {
    std::vector<double> c = row;
    auto pp = retrieval.convertCubeParameters(c);
    par_all.insert(par_all.end(), pp.first.begin(), pp.first.end());
    phys_all.insert(phys_all.end(), pp.second.begin(), pp.second.end());
  }
  write_bin(dir + "ref_prior_parameter.bin", par_all);
  write_bin(dir + "ref_prior_physical.bin", phys_all);
  rc.release();
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: bear_ref_harness <case_dir/> [--repeat K | --priors]\n";
    return 2;
  }
  std::string dir = argv[1];
  if (dir.back() != '/') dir += "/";
  if (argc >= 3 && std::string(argv[2]) == "--priors") return run_priors(dir);
  int repeat = 0;
  if (argc >= 4 && std::string(argv[2]) == "--repeat") repeat = std::stoi(argv[3]);

  refcase::RefCase rc = refcase::load_case(dir);
  auto& obs_in = rc.obs;
  auto& params = rc.params;
  const size_t P = params.empty() ? 0 : params[0].size();

  std::vector<bear::PriorConfig> priors;
  for (size_t i = 0; i < P; ++i)
    priors.emplace_back("delta", "p" + std::to_string(i), std::vector<double>{0.0});

  bear::Retrieval retrieval(rc.cfg, rc.model_cfg, obs_in, priors);

  write_bin(dir + "ref_grid.bin", retrieval.spectral_grid.wavenumber_list);

  {
    std::ofstream su(dir + "ref_setup.txt");
    su.precision(17);
    for (auto& o : retrieval.observations) {
      auto& sb = o.spectral_bands;
      su << "observation " << o.nbPoints() << " " << sb.obs_index_range.first << " "
         << sb.obs_index_range.second << " " << o.filter_response_normalisation << "\n";
      for (auto& e : sb.edge_indices) su << "edge " << e[0] << " " << e[1] << "\n";
      for (auto& c : sb.convolution_quadrature_intervals) su << "conv " << c[0] << " " << c[1] << "\n";
    }
  }

  std::vector<double> spec_all, obs_all, ll_all, neglect_all;
  for (auto& p : params) {
    bear::ForwardModelOutput out = retrieval.computeModel(p, true);
    spec_all.insert(spec_all.end(), out.spectrum.begin(), out.spectrum.end());
    for (auto& o : out.spectrum_obs) obs_all.insert(obs_all.end(), o.begin(), o.end());
    neglect_all.push_back(out.neglect_model ? 1.0 : 0.0);
    ll_all.push_back(retrieval.computeLikelihood(p));
  }
  write_bin(dir + "ref_spectrum.bin", spec_all);
  write_bin(dir + "ref_obs.bin", obs_all);
  write_bin(dir + "ref_loglike.bin", ll_all);
  write_bin(dir + "ref_neglect.bin", neglect_all);

  if (repeat > 0) {
    // timing mode: mean wall time of computeLikelihood over `repeat` calls
    auto& p = params[0];
    retrieval.computeLikelihood(p);
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < repeat; ++i) retrieval.computeLikelihood(p);
    auto t1 = std::chrono::steady_clock::now();
    double s = std::chrono::duration<double>(t1 - t0).count() / repeat;
    std::printf("ref_seconds_per_eval %.9f\n", s);
  }

  rc.release();
  return 0;
}
