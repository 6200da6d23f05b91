// Check of the reference-side C++ binding (bear_gb300/binding/gb300_model.h), compiled
// against the reference's own headers and linked with its objects and libbeargb300.so by
// tests/test_cpp_binding.py. It builds the reference's Retrieval from a golden-case
// directory the way pyBeAR does, renders the engine configuration from the same
// configuration objects (gb300_config_text), builds a Gb300Model on the Retrieval's
// spectral grid and observations (host set-up only, no GPU) and prints what the two
// models report: parameter counts, spectral grid, observation sizes, and whether the
// selectForwardModel branch recognises its prefix. Exit status 0 when they agree.

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "case_io.h"
#include "gb300_model.h"
#include "retrieval/priors.h"
#include "retrieval/retrieval.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: binding_check <case_dir/>\n");
    return 2;
  }
  std::string dir = argv[1];
  if (dir.back() != '/') dir += "/";
  refcase::RefCase rc = refcase::load_case(dir);
  const size_t P = rc.params.empty() ? 0 : rc.params[0].size();
  std::vector<bear::PriorConfig> priors;
  for (size_t i = 0; i < P; ++i) priors.emplace_back("delta", "p" + std::to_string(i), std::vector<double>{0.0});
  bear::Retrieval retrieval(rc.cfg, rc.model_cfg, rc.obs, priors);

  const std::string text = bear::gb300_config_text(*rc.cfg, rc.model, rc.model_cfg);
  bear::Gb300Model gm(rc.cfg, &retrieval.spectral_grid, retrieval.observations, text, rc.obs, 0, true);

  int bad = 0;
  const size_t ref_params = retrieval.nbParameters() - (rc.cfg->use_error_inflation ? 1 : 0);
  std::printf("parameters %zu %zu\n", gm.parametersNumber(), ref_params);
  bad += gm.parametersNumber() != ref_params;

  const std::vector<double>& ref_nu = retrieval.spectral_grid.wavenumber_list;
  std::vector<double> nu(ref_nu.size());
  bad += bear_model_wavenumbers(gm.engine(), nu.data()) != BEAR_OK;
  double worst = 0.0;
  for (size_t k = 0; k < nu.size(); ++k) worst = std::fmax(worst, std::fabs(nu[k] - ref_nu[k]));
  std::printf("points %zu max_abs_wavenumber_difference %.3g\n", nu.size(), worst);
  bad += worst != 0.0;

  for (size_t i = 0; i < retrieval.observations.size(); ++i) {
    int n = 0;
    bad += bear_model_observation_size(gm.engine(), (int)i, &n) != BEAR_OK;
    std::printf("observation %zu %d %zu\n", i, n, retrieval.observations[i].nbPoints());
    bad += (size_t)n != retrieval.observations[i].nbPoints();
  }

  bear::ForwardModel* sel = bear::selectGb300Model("gb300:" + rc.model, rc.model_cfg, rc.cfg,
                                                   &retrieval.spectral_grid, retrieval.observations, rc.obs, 0,
                                                   true);
  bear::ForwardModel* none = bear::selectGb300Model(rc.model, rc.model_cfg, rc.cfg, &retrieval.spectral_grid,
                                                    retrieval.observations, rc.obs, 0, true);
  std::printf("select %d %d\n", sel != nullptr, none != nullptr);
  bad += sel == nullptr || none != nullptr;
  delete sel;

  std::printf("%s\n", bad ? "binding MISMATCH" : "binding ok");
  rc.release();
  return bad ? 1 : 0;
}
