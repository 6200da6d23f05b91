/*
 * gb300_model.h -- the reference-side binding: a BeAR ForwardModel whose spectra come
 * from the GB300 engine (libbeargb300.so, C ABI in include/bear_gb300.h).
 *
 * This header is compiled inside BeAR (C++11, against BeAR's own headers with
 * -I<BeAR>/src) by a maintainer who adds the engine as a forward model. It replaces the
 * model construction of Retrieval::selectForwardModel
 * (src/retrieval/select_forward_model.cpp:38-120) and implements the ForwardModel
 * interface (src/forward_model/forward_model.h:61-144):
 *
 *   calcModelGPU(params, spectrum_dev, spectrum_obs_dev)   -> bear_forward
 *   calcModelCPU(params, spectrum, spectrum_obs)           -> bear_compute_model (host
 *       buffers; the GPU computes), observations returned in BeAR's internal order
 *   parametersNumber()                                     -> bear_model_info (without the
 *       error-inflation exponent, which Retrieval adds as an extra prior)
 *
 * gb300_config_text() renders the engine's configuration from the GlobalConfig and the
 * model config object the Retrieval was given (EmissionModelConfig,
 * TransmissionModelConfig or OccultationConfig), so the same inputs build both models.
 *
 * The constructor runs the engine's host set-up (spectral grid, observation operators,
 * tables); the device upload happens on construction, or on the first evaluation when
 * defer_upload is true (so a model can be built and inspected on a machine without a GPU).
 * Errors from the engine are thrown as bear::InvalidInput with the engine's message.
 */
#ifndef BEAR_GB300_BINDING_GB300_MODEL_H
#define BEAR_GB300_BINDING_GB300_MODEL_H

#include <algorithm>
#include <sstream>
#include <string>
#include <vector>

#include "additional/exceptions.h"
#include "config/global_config.h"
#include "forward_model/emission/emission.h"
#include "forward_model/forward_model.h"
#include "forward_model/secondary_eclipse/secondary_eclipse.h"
#include "forward_model/transmission/transmission.h"
#include "observations/observations.h"
#include "spectral_grid/spectral_grid.h"

#include "bear_gb300.h"

namespace bear {

namespace gb300_detail {

inline void check(int rc, const char* what) {
  if (rc != BEAR_OK) throw InvalidInput(std::string("GB300 engine: ") + what, bear_last_error());
}

inline std::string number(double x) {
  std::ostringstream s;
  s.precision(17);
  s << x;
  return s.str();
}

inline void words(std::ostringstream& out, const std::string& key, const std::string& first,
                  const std::vector<std::string>& rest) {
  out << key << " " << first;
  for (size_t i = 0; i < rest.size(); ++i) out << " " << rest[i];
  out << "\n";
}

template <class Config>
void atmosphere_lines(std::ostringstream& out, const Config& c) {
  out << "nb_grid_points " << c.nb_grid_points << "\n";
  out << "atmos_boundaries " << number(c.atmos_boundaries[0]) << " " << number(c.atmos_boundaries[1]) << "\n";
  words(out, "temperature_profile", c.temperature_profile_model, c.temperature_profile_parameters);
}

template <class Config>
void species_lines(std::ostringstream& out, const Config& c) {
  for (size_t i = 0; i < c.chemistry_model.size(); ++i)
    words(out, "chemistry", c.chemistry_model[i], c.chemistry_parameters[i]);
  for (size_t i = 0; i < c.cloud_model.size(); ++i)
    words(out, "cloud", c.cloud_model[i], c.cloud_model_parameters[i]);
  for (size_t i = 0; i < c.opacity_species_symbol.size(); ++i) {
    out << "opacity " << c.opacity_species_symbol[i];
    if (i < c.opacity_species_folder.size() && !c.opacity_species_folder[i].empty())
      out << " " << c.opacity_species_folder[i];
    out << "\n";
  }
}

}  // namespace gb300_detail

// The engine's configuration text for a Retrieval's GlobalConfig and model config
// (the arguments Retrieval::selectForwardModel receives).
inline std::string gb300_config_text(const GlobalConfig& config, const std::string& model_description,
                                     GenericConfig* model_config) {
  static const char* const kDiscretisation[3] = {"const_wavenumber", "const_wavelength", "const_resolution"};
  std::ostringstream out;
  std::string path = config.cross_section_file_path;
  if (!path.empty() && path[path.size() - 1] != '/') path += "/";
  out << "forward_model " << model_description << "\n";
  out << "cross_section_path " << path << "\n";
  out << "wavenumber_file " << config.wavenumber_file_path << "\n";
  out << "spectral_discretisation " << kDiscretisation[std::min(config.spectral_disecretisation, 2u)] << "\n";
  out << "spectral_resolution " << gb300_detail::number(config.spectral_resolution) << "\n";
  out << "error_inflation " << (config.use_error_inflation ? 1 : 0) << "\n";
  if (EmissionModelConfig* e = dynamic_cast<EmissionModelConfig*>(model_config)) {
    gb300_detail::atmosphere_lines(out, *e);
    gb300_detail::words(out, "radiative_transfer", e->radiative_transfer_model, e->radiative_transfer_parameters);
    gb300_detail::species_lines(out, *e);
  } else if (TransmissionModelConfig* t = dynamic_cast<TransmissionModelConfig*>(model_config)) {
    if (!t->modules.empty())
      throw InvalidInput("GB300 engine", "transmission spectrum modules are not supported");
    gb300_detail::atmosphere_lines(out, *t);
    out << "fit_mean_molecular_weight " << (t->fit_mean_molecular_weight ? 1 : 0) << "\n";
    out << "fit_scale_height " << (t->fit_scale_height ? 1 : 0) << "\n";
    out << "variable_gravity " << (t->use_variable_gravity ? 1 : 0) << "\n";
    gb300_detail::species_lines(out, *t);
  } else if (OccultationConfig* o = dynamic_cast<OccultationConfig*>(model_config)) {
    gb300_detail::atmosphere_lines(out, *o);
    gb300_detail::words(out, "radiative_transfer", o->radiative_transfer_model, o->radiative_transfer_parameters);
    gb300_detail::words(out, "stellar_spectrum", o->stellar_spectrum_model, o->stellar_model_parameters);
    gb300_detail::species_lines(out, *o);
  } else {
    throw InvalidInput("GB300 engine", "unsupported model configuration for " + model_description);
  }
  return out.str();
}

class Gb300Model : public ForwardModel {
 public:
  // config, spectral_grid, observations: as every ForwardModel receives them;
  // config_text: gb300_config_text(*config, model_description, model_config);
  // observation_input: the ObservationInput list the Retrieval was built from.
  Gb300Model(GlobalConfig* config, SpectralGrid* spectral_grid, std::vector<Observation>& observations,
             const std::string& config_text, const std::vector<ObservationInput>& observation_input,
             int device = 0, bool defer_upload = false)
      : ForwardModel(config, spectral_grid, observations) {
    gb300_detail::check(bear_model_create(config_text.c_str(), device, &model_), "bear_model_create");
    try {
      for (size_t i = 0; i < observation_input.size(); ++i) add_observation(observation_input[i]);
      gb300_detail::check(bear_model_prepare(model_), "bear_model_prepare");
      int n = 0, m = 0, p = 0, k = 0;
      gb300_detail::check(bear_model_info(model_, &n, &m, &p, &k), "bear_model_info");
      // the engine counts the error-inflation exponent (the last physical parameter when
      // GlobalConfig::use_error_inflation is set); ForwardModel::parametersNumber does not,
      // Retrieval adds it as an extra prior (src/retrieval/retrieval.cpp:92-96)
      nb_param_ = p - (config->use_error_inflation ? 1 : 0);
      nb_points_ = n;
      if ((size_t)n != spectral_grid->nbSpectralPoints())
        throw InvalidInput("GB300 engine", "the engine sampled a different spectral grid than BeAR");
      if (!defer_upload) upload();
    } catch (...) {
      bear_model_destroy(model_);
      throw;
    }
  }

  ~Gb300Model() { bear_model_destroy(model_); }

  // ForwardModel::calcModelGPU (src/forward_model/forward_model.h:76-79): spectrum
  // (N doubles) and one device buffer per observation, BeAR's internal order.
  virtual bool calcModelGPU(const std::vector<double>& physical_parameters, double* spectrum,
                            std::vector<double*>& spectrum_obs) {
    upload();
    int neglect = 0;
    gb300_detail::check(bear_forward(model_, physical_parameters.data(), (int)physical_parameters.size(), spectrum,
                                     spectrum_obs.empty() ? NULL : &spectrum_obs[0], &neglect, NULL),
                        "bear_forward");
    return neglect != 0;
  }

  // ForwardModel::calcModelCPU (forward_model.h:70-73) with host outputs computed on the GPU;
  // the observations come back in BeAR's internal (descending-wavelength) order, which
  // ForwardModel::calcModel then reverses for ascending inputs.
  virtual bool calcModelCPU(const std::vector<double>& physical_parameters, std::vector<double>& spectrum,
                            std::vector<std::vector<double> >& spectrum_obs) {
    upload();
    size_t total = 0;
    for (size_t i = 0; i < observations.size(); ++i) total += observations[i].nbPoints();
    std::vector<double> obs(std::max<size_t>(total, 1));
    spectrum.assign((size_t)nb_points_, 0.0);
    int neglect = 0;
    gb300_detail::check(bear_compute_model(model_, physical_parameters.data(), (int)physical_parameters.size(),
                                           &spectrum[0], &obs[0], &neglect, NULL),
                        "bear_compute_model");
    spectrum_obs.resize(observations.size());
    size_t off = 0;
    for (size_t i = 0; i < observations.size(); ++i) {
      const size_t n = observations[i].nbPoints();
      spectrum_obs[i].assign(obs.begin() + off, obs.begin() + off + n);
      if (observations[i].ascending_wavelengths) std::reverse(spectrum_obs[i].begin(), spectrum_obs[i].end());
      off += n;
    }
    return neglect != 0;
  }

  virtual size_t parametersNumber() { return (size_t)nb_param_; }

  // post-processing stays with BeAR's own models
  virtual void postProcess(const std::vector<std::vector<double> >&, const size_t, bool&) {
    throw InvalidInput("GB300 engine", "post-processing is done with BeAR's own forward models");
  }
  virtual void postProcess(GenericConfig*, const std::vector<std::vector<double> >&, const size_t, bool&) {
    throw InvalidInput("GB300 engine", "post-processing is done with BeAR's own forward models");
  }
  virtual bool testModel(const std::vector<double>&) { return true; }

  // the engine's log-likelihood of one parameter set (Retrieval::computeLikelihood's value)
  double logLikelihood(const std::vector<double>& physical_parameters) {
    upload();
    double ll = 0.0;
    gb300_detail::check(bear_loglike(model_, physical_parameters.data(), (int)physical_parameters.size(), &ll, NULL),
                        "bear_loglike");
    return ll;
  }

  bear_model* engine() { return model_; }

 private:
  void add_observation(const ObservationInput& o) {
    std::vector<double> ce = o.wavelengths;
    if (ce.empty())
      for (size_t i = 0; i < o.bin_wavelength_edges.size(); ++i) {
        ce.push_back(o.bin_wavelength_edges[i][0]);
        ce.push_back(o.bin_wavelength_edges[i][1]);
      }
    const bool filter = o.filter_response.size() == 2 && !o.filter_response[0].empty();
    gb300_detail::check(
        bear_model_add_observation(
            model_, o.name.c_str(), o.type.c_str(), (int)o.data.size(), ce.empty() ? NULL : &ce[0],
            o.data.empty() ? NULL : &o.data[0], o.data_error.empty() ? NULL : &o.data_error[0],
            o.likelihood_weight.empty() ? NULL : &o.likelihood_weight[0],
            o.instrument_profile_fwhm.empty() ? NULL : &o.instrument_profile_fwhm[0],
            filter ? (int)o.filter_response[0].size() : 0, filter ? &o.filter_response[0][0] : NULL,
            filter ? &o.filter_response[1][0] : NULL, o.filter_detector_type.c_str(),
            o.spectrum_modifier_id.c_str()),
        "bear_model_add_observation");
  }

  void upload() {
    if (uploaded_) return;
    gb300_detail::check(bear_model_finalize(model_), "bear_model_finalize");
    uploaded_ = true;
  }

  bear_model* model_ = NULL;
  int nb_param_ = 0;
  int nb_points_ = 0;
  bool uploaded_ = false;
};

// The branch a maintainer adds to Retrieval::selectForwardModel
// (src/retrieval/select_forward_model.cpp:38): "gb300:<model>" builds the engine for
// <model> from the same configuration objects; other descriptions return NULL and the
// reference's own selection continues.
inline ForwardModel* selectGb300Model(const std::string& model_description, GenericConfig* model_config,
                                      GlobalConfig* config, SpectralGrid* spectral_grid,
                                      std::vector<Observation>& observations,
                                      const std::vector<ObservationInput>& observation_input, int device = 0,
                                      bool defer_upload = false) {
  const std::string prefix = "gb300:";
  if (model_description.compare(0, prefix.size(), prefix) != 0) return NULL;
  const std::string model = model_description.substr(prefix.size());
  return new Gb300Model(config, spectral_grid, observations, gb300_config_text(*config, model, model_config),
                        observation_input, device, defer_upload);
}

}  // namespace bear

#endif  // BEAR_GB300_BINDING_GB300_MODEL_H
