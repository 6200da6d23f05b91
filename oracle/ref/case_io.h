// Reading of a golden-case directory into the reference's own configuration objects,
// shared by the reference driver (harness.cpp) and the binding check
// (tests/binding_check.cpp). Test infrastructure, compiled against the reference's
// headers.
//
// Case directory layout (written by oracle/refcase.py):
//   config.txt        "key value..." lines (same keys as the product config)
//   observations.txt  one block per observation (see read_observations)
//   params.txt        "P S" then S rows of P physical parameters
//
// Objects are built the way pyBeAR builds them
// (python/src/bear_python_wrapper.cpp:114-129): GlobalConfig 7-argument
// constructor, EmissionModelConfig / TransmissionModelConfig / OccultationConfig and
// ObservationInput.
#ifndef BEAR_ORACLE_REF_CASE_IO_H
#define BEAR_ORACLE_REF_CASE_IO_H

#include <algorithm>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "config/global_config.h"
#include "forward_model/emission/emission.h"
#include "forward_model/secondary_eclipse/secondary_eclipse.h"
#include "forward_model/transmission/transmission.h"
#include "observations/observations.h"

namespace refcase {

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

inline KV read_config(const std::string& path) {
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

inline std::vector<bear::ObservationInput> read_observations(const std::string& path) {
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

inline std::vector<std::string> tail(const std::vector<std::string>& v, size_t from) {
  return std::vector<std::string>(v.begin() + std::min(from, v.size()), v.end());
}

// The reference's configuration objects of one case (owned; released by release()).
// GenericConfig has no virtual destructor, so the model config is kept with its type.
struct RefCase {
  std::string model;
  bear::GlobalConfig* cfg = nullptr;
  bear::GenericConfig* model_cfg = nullptr;  // one of em, tm, om
  bear::EmissionModelConfig* em = nullptr;
  bear::TransmissionModelConfig* tm = nullptr;
  bear::OccultationConfig* om = nullptr;
  std::vector<bear::ObservationInput> obs;
  std::vector<std::vector<double>> params;
  void release() {
    delete cfg;
    delete em;
    delete tm;
    delete om;
    cfg = nullptr;
    model_cfg = nullptr;
    em = nullptr;
    tm = nullptr;
    om = nullptr;
  }
};

// config.txt, observations.txt and params.txt of case directory `dir` (with a trailing '/').
inline RefCase load_case(const std::string& dir) {
  KV kv = read_config(dir + "config.txt");
  const std::string model = kv.str("forward_model");
  RefCase rc;
  rc.model = model;
  rc.cfg = new bear::GlobalConfig(false, model, kv.str("cross_section_path"),
                         kv.str("spectral_discretisation", "const_wavenumber"),
                         std::stod(kv.str("spectral_resolution", "1")), "", "");
  rc.cfg->wavenumber_file_path = kv.str("wavenumber_file");
  rc.cfg->use_error_inflation = kv.str("error_inflation", "0") == "1";

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

  if (model == "secondary_eclipse" || model == "Secondary_eclipse" || model == "se") {
    auto rt = kv.get("radiative_transfer");
    if (rt.empty()) rt = {"scm"};
    auto star = kv.get("stellar_spectrum");
    rc.model_cfg = rc.om = new bear::OccultationConfig(nb_grid, std::stod(bounds[0]), std::stod(bounds[1]), temp[0],
                                     tail(temp, 1), rt[0], tail(rt, 1), chem_models, chem_params,
                                     op_symbol, op_folder, star[0], tail(star, 1), cloud_models,
                                     cloud_params);
  } else if (model == "emission") {
    auto rt = kv.get("radiative_transfer");
    if (rt.empty()) rt = {"scm"};
    rc.model_cfg = rc.em = new bear::EmissionModelConfig(nb_grid, std::stod(bounds[0]), std::stod(bounds[1]),
                                       temp[0], tail(temp, 1), rt[0], tail(rt, 1), chem_models,
                                       chem_params, op_symbol, op_folder, cloud_models,
                                       cloud_params);
  } else if (model == "transmission") {
    rc.model_cfg = rc.tm = new bear::TransmissionModelConfig(
        kv.str("fit_mean_molecular_weight", "0") == "1", kv.str("fit_scale_height", "0") == "1",
        kv.str("variable_gravity", "0") == "1", nb_grid, std::stod(bounds[0]),
        std::stod(bounds[1]), temp[0], tail(temp, 1), chem_models, chem_params, op_symbol,
        op_folder, cloud_models, cloud_params, std::vector<std::string>(),
        std::vector<std::vector<std::string>>());
  } else {
    throw std::runtime_error("unsupported forward model " + model);
  }
  rc.obs = read_observations(dir + "observations.txt");
  std::ifstream pf(dir + "params.txt");
  size_t P = 0, S = 0;
  pf >> P >> S;
  rc.params.assign(S, std::vector<double>(P));
  for (auto& row : rc.params)
    for (auto& x : row) pf >> x;
  return rc;
}

}  // namespace refcase

#endif  // BEAR_ORACLE_REF_CASE_IO_H
