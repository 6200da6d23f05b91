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
//
// Objects are built the way pyBeAR builds them
// (python/src/bear_python_wrapper.cpp:114-129): GlobalConfig 7-argument
// constructor, EmissionModelConfig / TransmissionModelConfig, ObservationInput
// and PriorConfig, then Retrieval(config, model_config, observations, priors).

#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "config/global_config.h"
#include "forward_model/emission/emission.h"
#include "forward_model/forward_model.h"
#include "forward_model/transmission/transmission.h"
#include "forward_model/secondary_eclipse/secondary_eclipse.h"
#include "observations/observations.h"
#include "retrieval/priors.h"
#include "retrieval/retrieval.h"

namespace {

struct KV {
  std::multimap<std::string, std::vector<std::string>> items;
  std::vector<std::string> get(const std::string& k) const {
    auto it = items.find(k);
    if (it == items.end()) return {};
    return it->second;
  }
  std::vector<std::vector<std::string>> all(const std::string& k) const {
    std::vector<std::vector<std::string>> out;
    auto r = items.equal_range(k);
    for (auto it = r.first; it != r.second; ++it) out.push_back(it->second);
    return out;
  }
  std::string str(const std::string& k, const std::string& d = "") const {
    auto v = get(k);
    return v.empty() ? d : v[0];
  }
};

KV read_config(const std::string& path) {
  KV kv;
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string key, tok;
    if (!(ss >> key) || key[0] == '#') continue;
    std::vector<std::string> vals;
    while (ss >> tok) vals.push_back(tok);
    kv.items.emplace(key, vals);
  }
  return kv;
}

std::vector<bear::ObservationInput> read_observations(const std::string& path) {
  // block header:
  // observation <name> <type> <n> <has_fwhm> <has_weight> <n_filter> <detector> <modifier>
  // then n rows: spectroscopy -> wl data err [fwhm] [weight]
  //              others       -> wl_a wl_b data err [fwhm] [weight]
  // then n_filter rows: wavelength response
  std::vector<bear::ObservationInput> obs;
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::string tag;
  while (f >> tag) {
    if (tag != "observation") throw std::runtime_error("bad observation block");
    std::string name, type, detector, modifier;
    size_t n, has_fwhm, has_weight, n_filter;
    f >> name >> type >> n >> has_fwhm >> has_weight >> n_filter >> detector >> modifier;
    bear::ObservationInput in;
    in.name = name;
    in.type = type;
    for (size_t i = 0; i < n; ++i) {
      if (type == "spectroscopy") {
        double w;
        f >> w;
        in.wavelengths.push_back(w);
      } else {
        double a, b;
        f >> a >> b;
        in.bin_wavelength_edges.push_back({a, b});
      }
      double d, e;
      f >> d >> e;
      in.data.push_back(d);
      in.data_error.push_back(e);
      if (has_fwhm) { double x; f >> x; in.instrument_profile_fwhm.push_back(x); }
      if (has_weight) { double x; f >> x; in.likelihood_weight.push_back(x); }
    }
    if (n_filter > 0) {
      std::vector<double> wl, resp;
      for (size_t i = 0; i < n_filter; ++i) {
        double a, b;
        f >> a >> b;
        wl.push_back(a);
        resp.push_back(b);
      }
      in.filter_response = {wl, resp};
      in.filter_detector_type = detector;
    }
    in.spectrum_modifier_id = (modifier == "-") ? "" : modifier;
    obs.push_back(in);
  }
  return obs;
}

void write_bin(const std::string& path, const std::vector<double>& v) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) throw std::runtime_error("cannot write " + path);
  if (!v.empty()) std::fwrite(v.data(), sizeof(double), v.size(), fp);
  std::fclose(fp);
}

std::vector<std::string> tail(const std::vector<std::string>& v, size_t from) {
  return std::vector<std::string>(v.begin() + std::min(from, v.size()), v.end());
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: bear_ref_harness <case_dir/> [--repeat K]\n";
    return 2;
  }
  std::string dir = argv[1];
  if (dir.back() != '/') dir += "/";
  int repeat = 0;
  if (argc >= 4 && std::string(argv[2]) == "--repeat") repeat = std::stoi(argv[3]);

  KV kv = read_config(dir + "config.txt");
  const std::string model = kv.str("forward_model");

  bear::GlobalConfig cfg(false, model, kv.str("cross_section_path"),
                         kv.str("spectral_discretisation", "const_wavenumber"),
                         std::stod(kv.str("spectral_resolution", "1")), "", "");
  cfg.wavenumber_file_path = kv.str("wavenumber_file");
  cfg.use_error_inflation = kv.str("error_inflation", "0") == "1";

  auto bounds = kv.get("atmos_boundaries");
  const int nb_grid = std::stoi(kv.str("nb_grid_points"));
  auto temp = kv.get("temperature_profile");
  std::vector<std::string> chem_models;
  std::vector<std::vector<std::string>> chem_params;
  for (auto& c : kv.all("chemistry")) {
    chem_models.push_back(c[0]);
    chem_params.push_back(tail(c, 1));
  }
  std::vector<std::string> cloud_models;
  std::vector<std::vector<std::string>> cloud_params;
  for (auto& c : kv.all("cloud")) {
    cloud_models.push_back(c[0]);
    cloud_params.push_back(tail(c, 1));
  }
  std::vector<std::string> op_symbol, op_folder;
  for (auto& o : kv.all("opacity")) {
    op_symbol.push_back(o[0]);
    op_folder.push_back(o.size() > 1 ? o[1] : "");
  }

  bear::GenericConfig* model_cfg = nullptr;
  bear::EmissionModelConfig* em = nullptr;
  bear::TransmissionModelConfig* tm = nullptr;
  bear::OccultationConfig* om = nullptr;
  if (model == "secondary_eclipse" || model == "Secondary_eclipse" || model == "se") {
    auto rt = kv.get("radiative_transfer");
    if (rt.empty()) rt = {"scm"};
    auto star = kv.get("stellar_spectrum");
    om = new bear::OccultationConfig(nb_grid, std::stod(bounds[0]), std::stod(bounds[1]), temp[0],
                                     tail(temp, 1), rt[0], tail(rt, 1), chem_models, chem_params,
                                     op_symbol, op_folder, star[0], tail(star, 1), cloud_models,
                                     cloud_params);
    model_cfg = om;
  } else if (model == "emission") {
    auto rt = kv.get("radiative_transfer");
    if (rt.empty()) rt = {"scm"};
    em = new bear::EmissionModelConfig(nb_grid, std::stod(bounds[0]), std::stod(bounds[1]),
                                       temp[0], tail(temp, 1), rt[0], tail(rt, 1), chem_models,
                                       chem_params, op_symbol, op_folder, cloud_models,
                                       cloud_params);
    model_cfg = em;
  } else if (model == "transmission") {
    tm = new bear::TransmissionModelConfig(
        kv.str("fit_mean_molecular_weight", "0") == "1", kv.str("fit_scale_height", "0") == "1",
        kv.str("variable_gravity", "0") == "1", nb_grid, std::stod(bounds[0]),
        std::stod(bounds[1]), temp[0], tail(temp, 1), chem_models, chem_params, op_symbol,
        op_folder, cloud_models, cloud_params, std::vector<std::string>(),
        std::vector<std::vector<std::string>>());
    model_cfg = tm;
  } else {
    std::cerr << "unsupported forward model " << model << "\n";
    return 2;
  }

  auto obs_in = read_observations(dir + "observations.txt");

  std::ifstream pf(dir + "params.txt");
  size_t P = 0, S = 0;
  pf >> P >> S;
  std::vector<std::vector<double>> params(S, std::vector<double>(P));
  for (auto& row : params)
    for (auto& x : row) pf >> x;

  std::vector<bear::PriorConfig> priors;
  for (size_t i = 0; i < P; ++i)
    priors.emplace_back("delta", "p" + std::to_string(i), std::vector<double>{0.0});

  bear::Retrieval retrieval(&cfg, model_cfg, obs_in, priors);

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

  delete em;
  delete tm;
  delete om;
  return 0;
}
