// Host-side set-up of the likelihood engine: configuration, spectral grid,
// observation operators, opacity tables. Everything here is evaluated once per
// model; the per-evaluation work runs on the GPU (engine.cu).
//
// The integer decisions (grid points, band-edge indices, convolution windows,
// table brackets) must match the reference exactly, so this file is compiled
// without FMA contraction and follows the reference's operation order.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/bear_gb300.h"
#include "model.h"

namespace bgb {

const char* const kSpeciesSymbol[kSpeciesCount] = {
    "Total", "H",   "He",  "C",    "O",   "Fe",  "Fe+", "Ca",  "Ti",   "Ti+", "H2",  "H2O",
    "CO2",   "CO",  "CH4", "HCN",  "NH3", "C2H2", "N2", "Na",  "K",    "H2S", "H-",  "TiO",
    "VO",    "FeH", "SH",  "MgO",  "AlO", "CaO", "CrH", "MgH", "CaH",  "TiH", "OH",  "e-",
    "V",     "V+",  "Mn",  "Si",   "Cr",  "Cr+", "SiO", "SiO2", "SO2", "CS2"};
const double kSpeciesMolWeight[kSpeciesCount] = {
    0.0,      1.00784, 4.002602, 12.0107, 15.999,   55.845,   55.845,  40.078,  47.867,
    47.867,   2.01588, 18.01528, 44.01,   28.0101,  16.04246, 27.0253, 17.03052, 26.04,
    28.0134,  22.98977, 39.0983, 34.09099, 1.00784, 63.8664,  66.9409, 56.853,  34.08,
    40.3044,  42.981,  56.0774,  54.0040, 26.3209,  41.0859,  48.87484, 17.008,
    5.4857990907e-4, 50.9415, 50.9415, 54.938044, 28.085, 51.996, 51.996, 44.08, 60.08,
    64.066,   76.139};

int species_id(const std::string& s) {
  for (int i = 0; i < kSpeciesCount; ++i)
    if (s == kSpeciesSymbol[i]) return i;
  return -1;
}

static Error invalid(const std::string& s) { return Error(BEAR_ERR_INVALID_INPUT, s); }
static Error unsupported(const std::string& s) { return Error(BEAR_ERR_UNSUPPORTED, s); }

// ------------------------------------------------------------------ config text
void parse_config(Model& m, const std::string& text) {
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::vector<std::string> t;
    std::string w;
    while (ls >> w) t.push_back(w);
    if (t.empty() || t[0][0] == '#') continue;
    const std::string& k = t[0];
    auto need = [&](size_t n) {
      if (t.size() < n) throw invalid("config line '" + line + "' is incomplete");
    };
    if (k == "forward_model") {
      need(2);
      // Retrieval::selectForwardModel src/retrieval/select_forward_model.cpp:38-150
      if (t[1] == "emission") m.transmission = false;
      else if (t[1] == "transmission") m.transmission = true;
      else if (t[1] == "secondary_eclipse" || t[1] == "Secondary_eclipse" || t[1] == "se") m.occultation = true;
      else
        throw unsupported("forward model " + t[1] + " is not supported (emission, transmission, secondary_eclipse)");
    } else if (k == "cross_section_path") {
      m.xsec_path = t.size() > 1 ? t[1] : "";
    } else if (k == "wavenumber_file") {
      m.wn_file = t.size() > 1 ? t[1] : "";
    } else if (k == "spectral_discretisation") {
      need(2);
      // GlobalConfig::GlobalConfig src/config/global_config.cpp:37-74
      if (t[1] == "const_wavenumber") m.discretisation = 0;
      else if (t[1] == "const_wavelength") m.discretisation = 1;
      else if (t[1] == "const_resolution") m.discretisation = 2;
      else throw invalid("Spectral discretisation parameter: " + t[1] + " unknown!");
    } else if (k == "spectral_resolution") {
      need(2);
      m.resolution = std::stod(t[1]);
    } else if (k == "error_inflation") {
      need(2);
      m.error_inflation = std::stoi(t[1]) != 0;
    } else if (k == "nb_grid_points") {
      need(2);
      m.L = std::stoi(t[1]);
    } else if (k == "atmos_boundaries") {
      need(3);
      m.pbot = std::stod(t[1]);
      m.ptop = std::stod(t[2]);
    } else if (k == "temperature_profile") {
      need(2);
      // selectTemperatureProfile src/temperature/select_temperature_profile.h:52-161
      if (t[1] == "poly") {
        if (t.size() != 4) throw invalid("Piesewise polynomial temperature profile requires exactly two parameters!");
        m.temp_poly = true;
        m.poly_elements = std::stoi(t[2]);
        m.poly_order = std::stoi(t[3]);
        if (m.poly_order > 6) throw invalid("Piecewise polynomials are only available up to 6th order");
      } else if (t[1] == "const") {
        m.temp_poly = false;
      } else {
        throw unsupported("temperature profile " + t[1] + " is not supported (poly, const)");
      }
    } else if (k == "stellar_spectrum") {
      need(2);
      // selectStellarModel src/forward_model/stellar_spectrum/select_stellar_model.h:52-122
      if (t[1] == "blackbody") {
        if (t.size() != 2) throw invalid("Stellar blackbody model requires no parameters!");
        m.star_model = 1;
      } else if (t[1] == "file" || t[1] == "grid") {
        if (t.size() != 3)
          throw invalid(t[1] == "file" ? "Stellar model requires one parameter (the file path)!"
                                       : "Stellar grid model requires one parameter (the parameter file path)!");
        m.star_model = t[1] == "file" ? 2 : 3;
        m.star_path = t[2];
      } else {
        throw invalid("Stellar model " + t[1] + " unknown!");
      }
    } else if (k == "radiative_transfer") {
      need(2);
      if (t[1] != "scm") throw unsupported("radiative transfer " + t[1] + " is not supported (scm)");
    } else if (k == "chemistry") {
      need(2);
      ChemModule c;
      if (t[1] == "iso" || t[1] == "isoprofile") {
        // IsoprofileChemistry::IsoprofileChemistry src/chemistry/isoprofile_chemistry.cpp:30-84
        c.kind = 0;
        for (size_t i = 2; i < t.size(); ++i) {
          int id = species_id(t[i]);
          if (id < 0) throw invalid("Chemical species " + t[i] + " not found in the list of species");
          c.sp.push_back(id);
          if (id == SP_Na) c.na_free = true;
        }
      } else if (t[1] == "bg" || t[1] == "background") {
        // BackgroundChemistry::BackgroundChemistry src/chemistry/background_chemistry.cpp:31-69
        need(3);
        c.kind = 1;
        if (t[2] == "H2He") c.bg_h2he = true;
        else {
          c.bg_sp = species_id(t[2]);
          if (c.bg_sp < 0) throw invalid("Chemical species " + t[2] + " not found in the list of species");
        }
      } else {
        throw unsupported("chemistry " + t[1] + " is not supported (iso, bg)");
      }
      if (m.chem.size() >= (size_t)kMaxChemModules) throw unsupported("too many chemistry modules");
      if (c.sp.size() > (size_t)kSpeciesCount) throw invalid("too many species in one chemistry module");
      m.chem.push_back(c);
    } else if (k == "cloud") {
      need(2);
      if (t[1] == "none") continue;
      // selectCloudModel src/cloud_model/select_cloud_model.h:42-100
      if (m.cloud) throw unsupported("only one cloud model is supported");
      if (t[1] == "grey") {
        m.cloud_kind = 0;
        m.cloud_fb = (t.size() == 3 && t[2] == "fb");
      } else if (t[1] == "power_law" || t[1] == "KHnongrey") {
        // PowerLawCloudModel / KHCloudModel ctors: the reference wavelength, then optionally "fb"
        if (t.size() < 3)
          throw invalid("Expected at least one parameter for the " + t[1] + " cloud model, but only found 0");
        m.cloud_kind = t[1] == "power_law" ? 1 : 2;
        m.cloud_ref_wl = std::stod(t[2]);
        m.cloud_fb = (t.size() == 4 && t[3] == "fb");
      } else {
        throw unsupported("cloud model " + t[1] + " is not supported (grey, power_law, KHnongrey)");
      }
      m.cloud = true;
    } else if (k == "opacity") {
      need(2);
      m.opac_cfg.emplace_back(t[1], t.size() > 2 ? t[2] : "");
    } else if (k == "fit_mean_molecular_weight") {
      need(2);
      m.fit_mmw = std::stoi(t[1]) != 0;
    } else if (k == "fit_scale_height") {
      need(2);
      m.fit_sh = std::stoi(t[1]) != 0;
    } else if (k == "variable_gravity") {
      need(2);
      m.var_g = std::stoi(t[1]) != 0;
    } else if (k == "transmission_annuli") {
      need(2);
      m.annuli = std::stoi(t[1]);
      if (m.annuli < 1 || m.annuli > 64) throw invalid("transmission_annuli must be in [1, 64]");
    } else {
      throw invalid("unknown config key " + k);
    }
  }
  if (m.fit_sh) throw unsupported("fit_scale_height is not supported");
  if (m.occultation && m.star_model == 0) throw invalid("the secondary-eclipse model needs a stellar_spectrum");
  if (!m.occultation && m.star_model != 0) throw invalid("stellar_spectrum applies to the secondary-eclipse model only");
  if (m.L < 2 || m.L > kMaxLevels) throw invalid("nb_grid_points must be in [2, 512]");
  if (!(m.pbot > m.ptop) || !(m.ptop > 0)) throw invalid("atmos_boundaries must be bottom > top > 0");
}

static void reverse_vec(std::vector<double>& v) { std::reverse(v.begin(), v.end()); }

// ------------------------------------------------------------------ observations
// Observation::init(ObservationInput) src/observations/observations.cpp:42-111
void add_observation(Model& m, const char* name, const char* type, int n, const double* ce,
                     const double* data, const double* error, const double* weight,
                     const double* fwhm, int nfilter, const double* fwl, const double* fresp,
                     const char* detector, const char* modifier) {
  if (m.prepared) throw Error(BEAR_ERR_STATE, "observations must be added before prepare / finalize");
  if (n < 1) throw invalid("observation without data points");
  ObservationSetup o;
  o.name = name ? name : "";
  std::string mod = modifier ? modifier : "";
  // setSpectrumModifier :374-392
  if (mod.empty() || mod == "none") o.nb_modifier = 0;
  else if (mod == "shift_const") o.nb_modifier = 1;
  else throw invalid("Observation modifier " + mod + " unknown.");
  std::string ty = type ? type : "";
  // selectBandType src/spectral_grid/spectral_band_type.h:49-80
  if (ty == "spectroscopy" || ty == "Spectroscopy") o.type = 0;
  else if (ty == "photometry" || ty == "Photometry") o.type = 1;
  else if (ty == "band-spectroscopy" || ty == "Band-spectroscopy") o.type = 2;
  else throw invalid("Unsupported band type *" + ty + "* for observation " + o.name);
  o.n = n;
  o.data.assign(data, data + n);
  o.error.assign(error, error + n);
  o.weight.assign(n, 1.0);
  if (weight) o.weight.assign(weight, weight + n);
  if (fwhm) o.fwhm.assign(fwhm, fwhm + n);
  if (nfilter > 0) {
    std::string det = detector ? detector : "";
    if (det == "Energy") det = "energy";
    if (det == "Photon") det = "photon";
    if (det != "energy" && det != "photon") throw invalid("Unsupported detector type *" + det + "*");
    o.photon = det == "photon";
    o.nfilter = nfilter;
    o.filter_wl.assign(fwl, fwl + nfilter);
    o.filter_resp.assign(fresp, fresp + nfilter);
    if (o.filter_wl.front() < o.filter_wl.back()) {
      reverse_vec(o.filter_wl);
      reverse_vec(o.filter_resp);
    }
  }
  o.edges.resize(n);
  o.centers.resize(n);
  if (o.type == 0) {
    std::vector<double> wl(ce, ce + n);
    // areWavelengthsAscending(vector<double>) :127-151
    o.ascending = false;
    if (n > 1 && wl[0] < wl[1]) {
      o.ascending = true;
      reverse_vec(wl);
      reverse_vec(o.data);
      reverse_vec(o.error);
      reverse_vec(o.fwhm);
      reverse_vec(o.weight);
    }
    o.centers = wl;
    // calcBinEdges :188-221
    for (int i = 0; i < n; ++i) {
      if (i == 0) {
        if (n < 2) throw invalid("a spectroscopy observation needs at least two points");
        o.edges[0][1] = wl[0] - (wl[i] - wl[i + 1]) * 0.5;
        o.edges[0][0] = wl[0] + (wl[i] - wl[i + 1]) * 0.5;
      } else if (i == n - 1) {
        o.edges[n - 1][1] = wl[i] - (wl[i - 1] - wl[i]) * 0.5;
        o.edges[n - 1][0] = wl[i] + (wl[i - 1] - wl[i]) * 0.5;
      } else {
        o.edges[i][0] = wl[i - 1] - (wl[i - 1] - wl[i]) * 0.5;
        o.edges[i][1] = wl[i] - (wl[i] - wl[i + 1]) * 0.5;
      }
    }
  } else {
    for (int i = 0; i < n; ++i) o.edges[i] = {ce[2 * i], ce[2 * i + 1]};
    // areWavelengthsAscending(vector<vector<double>>) :156-184
    o.ascending = false;
    if (n > 1 && o.edges.front()[0] < o.edges.back()[0]) {
      o.ascending = true;
      std::reverse(o.edges.begin(), o.edges.end());
      reverse_vec(o.data);
      reverse_vec(o.error);
      reverse_vec(o.fwhm);
      reverse_vec(o.weight);
    }
    for (auto& e : o.edges)
      if (e[0] < e[1]) std::swap(e[0], e[1]);
    // calcBinCenters :224-233
    for (int i = 0; i < n; ++i) o.centers[i] = o.edges[i][0] - (o.edges[i][0] - o.edges[i][1]) * 0.5;
  }
  // setObservationEdges :237-251
  if (!o.fwhm.empty()) {
    o.wl_edges[0] = o.edges.front()[0] + 5.0 * o.fwhm.front() / 2.355;
    o.wl_edges[1] = o.edges.back()[1] - 5.0 * o.fwhm.back() / 2.355;
  } else {
    o.wl_edges[0] = o.edges.front()[0];
    o.wl_edges[1] = o.edges.back()[1];
  }
  // SpectralBands::init src/spectral_grid/spectral_band.cpp:38-63
  o.edge_nu.resize(n);
  for (int i = 0; i < n; ++i) o.edge_nu[i] = {1.0 / o.edges[i][0] * 1e4, 1.0 / o.edges[i][1] * 1e4};
  o.obs_nu_range[0] = 1.0 / o.wl_edges[0] * 1e4;
  o.obs_nu_range[1] = 1.0 / o.wl_edges[1] * 1e4;
  m.obs.push_back(std::move(o));
}

// ------------------------------------------------------------------ spectral grid
// SpectralGrid::findClosestIndex{,Asc,Desc} src/spectral_grid/spectral_grid.cpp:323-385.
// Past the end the reference reads beyond its vector; the last index is used here.
static size_t find_closest(double x, const std::vector<double>& d, size_t start) {
  const size_t n = d.size();
  if (n < 2) return 0;
  size_t it;
  if (d[0] < d[1]) it = std::lower_bound(d.begin() + start, d.end(), x) - d.begin();
  else if (d[0] > d[1]) it = std::lower_bound(d.begin() + start, d.end(), x, std::greater<double>()) - d.begin();
  else return 0;
  if (it == start) return start;
  if (it == n) return n - 1;
  if (std::fabs(x - d[it - 1]) < std::fabs(x - d[it])) return it - 1;
  return it;
}

static void load_wavenumbers(Model& m) {
  // SpectralGrid::loadWavenumberList :87-119; createHeliosWavenumberList :75-84
  std::ifstream f(m.wn_file);
  if (!f) {
    size_t n = (size_t)(90000.0 / 0.01 + 1);
    m.nu_full.resize(n);
    for (size_t i = 0; i < n; ++i) m.nu_full[i] = i * 0.01;
  } else {
    size_t n = 0;
    f >> n;
    m.nu_full.resize(n);
    for (auto& v : m.nu_full) f >> v;
    if (!f) throw Error(BEAR_ERR_FILE, "malformed wavenumber file " + m.wn_file);
  }
  m.wl_full.resize(m.nu_full.size());
  for (size_t i = 0; i < m.nu_full.size(); ++i) m.wl_full[i] = 1.0 / m.nu_full[i] * 1e4;
}

static void sample_grid(Model& m) {
  // SpectralGrid::sampleSpectralGrid :123-157
  std::vector<std::array<double, 2>> e;
  for (auto& o : m.obs) e.push_back({1.0 / o.wl_edges[0] * 1e4, 1.0 / o.wl_edges[1] * 1e4});
  std::stable_sort(e.begin(), e.end(), [](const std::array<double, 2>& a, const std::array<double, 2>& b) { return a[0] < b[0]; });
  std::vector<std::array<double, 2>> we{e[0]};
  for (size_t i = 1; i < e.size(); ++i) {
    if (e[i][0] > we.back()[0] && e[i][1] < we.back()[1]) continue;
    if (e[i][0] < we.back()[1] && e[i][1] > we.back()[1]) we.back()[1] = e[i][1];
    else we.push_back(e[i]);
  }
  const size_t nfull = m.nu_full.size();
  // findBinEdges :390-416
  std::vector<std::array<size_t, 2>> ei(we.size());
  for (size_t i = 0; i < we.size(); ++i) {
    size_t l = std::lower_bound(m.nu_full.begin(), m.nu_full.end(), we[i][0]) - m.nu_full.begin();
    size_t r = std::lower_bound(m.nu_full.begin(), m.nu_full.end(), we[i][1]) - m.nu_full.begin();
    if (l >= nfull || r >= nfull)
      throw invalid("observation range outside of the wavenumber list");
    ei[i][0] = l;
    if (m.nu_full[ei[i][0]] > we[i][0]) {
      if (ei[i][0] == 0) throw invalid("observation range outside of the wavenumber list");
      ei[i][0] -= 1;
    }
    ei[i][1] = r;
  }
  // createHighResGrid :239-304 with the three discretisations :161-236
  std::vector<int> inc(nfull, 0);
  for (auto& r : ei) {
    inc[r[0]] = 1;
    size_t last = r[0];
    for (size_t j = r[0]; j < r[1]; ++j) {
      if (m.discretisation == 0) {
        const double next = m.nu_full[last] + m.resolution;
        if (next == m.nu_full[j] || m.nu_full[j + 1] > next) { inc[j] = 1; last = j; }
      } else if (m.discretisation == 1) {
        const double next = m.wl_full[last] - m.resolution;
        if (next == m.wl_full[j] || m.wl_full[j + 1] < next) { inc[j] = 1; last = j; }
      } else {
        const double next = m.wl_full[last] * (1 - 1. / m.resolution);
        if (next == m.wl_full[j] || m.wl_full[j + 1] < next) { inc[j] = 1; last = j; }
      }
      inc[r[1]] = 1;
    }
  }
  for (auto& o : m.obs) {
    size_t start = 0;
    double last_nu = 0;
    for (int b = 0; b < o.n; ++b) {
      if (last_nu > o.edge_nu[b][0]) start = 0;
      size_t i1 = find_closest(o.edge_nu[b][0], m.nu_full, start);
      size_t i2 = find_closest(o.edge_nu[b][1], m.nu_full, start);
      inc[i1] = 1;
      inc[i2] = 1;
      last_nu = o.edge_nu[b][1];
      start = i2;
    }
  }
  m.index_list.clear();
  for (size_t i = 0; i < nfull; ++i)
    if (inc[i] == 1) m.index_list.push_back(i);
  m.N = m.index_list.size();
  m.nu.resize(m.N);
  m.wl.resize(m.N);
  for (size_t i = 0; i < m.N; ++i) {
    m.nu[i] = m.nu_full[m.index_list[i]];
    m.wl[i] = m.wl_full[m.index_list[i]];
  }
  // SpectralBands::setBandEdgeIndices src/spectral_grid/spectral_band.cpp:80-121 and init :66-76
  for (auto& o : m.obs) {
    o.edge_idx.resize(o.n);
    size_t start = 0;
    double last_nu = 0;
    for (int b = 0; b < o.n; ++b) {
      if (last_nu > o.edge_nu[b][0]) start = 0;
      size_t i1 = find_closest(o.edge_nu[b][0], m.nu, start);
      size_t i2 = find_closest(o.edge_nu[b][1], m.nu, start);
      if (i1 > m.N - 1 || i2 > m.N - 1) throw invalid("Edge wavenumber index not found!");
      if (i1 == i2) throw invalid("The spectral resolution of the opacity grid is too small!");
      o.edge_idx[b] = {i1, i2};
      last_nu = o.edge_nu[b][1];
      start = i2;
    }
    o.range_lo = find_closest(o.obs_nu_range[0], m.nu, 0);
    o.range_hi = find_closest(o.obs_nu_range[1], m.nu, 0);
  }
}

// SpectralGrid::interpolateToWavelengthGrid src/spectral_grid/spectral_grid_interpolate.cpp:60-172
static std::vector<double> interp_to_wavelengths(std::vector<double> x, std::vector<double> y,
                                                 const double* newx, size_t nn) {
  if (x.size() > 1 && x[0] < x[1]) {
    reverse_vec(x);
    reverse_vec(y);
  }
  std::vector<double> out(nn, 0.0);
  const size_t nd = x.size();
  size_t x_start = 0;
  for (size_t i = 0; i < nn; ++i) {
    if (newx[i] > x.front()) continue;
    if (newx[i] < x.back()) break;
    size_t it = x_start;
    while (it < nd && !(x[it] <= newx[i])) ++it;
    if (it >= nd) break;
    const size_t index = it;
    if (x[it] == newx[i]) out[i] = y[index];
    else out[i] = y[index - 1] + (y[index] - y[index - 1]) * (newx[i] - x[it - 1]) / (x[it] - x[it - 1]);
    if (x_start > 0) x_start = index - 1;
  }
  return out;
}

static double normal_dist(double sigma, double x) {
  // aux::normalDistribution(sigma, x) src/additional/aux_functions.cpp:344-351
  const double c = std::sqrt(1.0 / (2.0 * kPi));
  return c / sigma * std::exp(-x * x / (2.0 * sigma * sigma));
}

// Builds the instrument profile and filter (src/spectral_grid/spectral_band.cpp:127-154,
// src/spectral_grid/spectral_band_convolve.cpp:44-95, src/observations/
// observations_filter_response.cpp:122-160) and folds filter, convolution and bin
// integration into one banded linear operator per bin:
//   bin_b = sum_k W[b,k] F[k],
// F being the high-resolution spectrum in native units. The composition is exact for
// F >= 0 (emission fluxes and transit depths), where the absolute values the reference
// takes of each convolved point and each wavelength-space bin integral only flip signs.
static void build_observation_operator(Model& m, ObservationSetup& o) {
  const size_t N = m.N;
  o.has_profile = false;
  if (!o.fwhm.empty() && (int)o.fwhm.size() == o.n) {
    const size_t nhr = o.range_hi - o.range_lo + 1;
    std::vector<double> prof = interp_to_wavelengths(o.centers, o.fwhm, m.wl.data() + o.range_lo, nhr);
    o.sigma.assign(N, 0.0);
    for (size_t i = 0; i < nhr; ++i) o.sigma[i + o.range_lo] = prof[i] / 2.355;
    o.conv.resize(nhr);
    for (size_t i = 0; i < nhr; ++i) {
      const size_t idx = i + o.range_lo;
      o.conv[i] = {o.range_lo, o.range_hi};
      const double cut = 5.0 * o.sigma[idx];
      if (cut == 0) o.conv[i] = {idx, idx};
      else {
        o.conv[i][0] = find_closest(m.wl[idx] + cut, m.wl, 0);
        o.conv[i][1] = find_closest(m.wl[idx] - cut, m.wl, o.conv[i][0]);
      }
    }
    o.has_profile = true;
  }
  if (o.nfilter) {
    o.filter_grid = interp_to_wavelengths(o.filter_wl, o.filter_resp, m.wl.data(), N);
    o.filter_weight.assign(N, 1.0);
    if (o.photon)
      for (size_t i = 0; i < N; ++i) o.filter_weight[i] = m.wl[i];
    std::vector<double> y = o.filter_resp;
    if (o.photon)
      for (size_t i = 0; i < y.size(); ++i) y[i] *= o.filter_wl[i];
    double s = 0.0;
    if (y.size() == 1) s = y[0];
    else {
      for (size_t i = 1; i < y.size(); ++i) s += (o.filter_wl[i] - o.filter_wl[i - 1]) * (y[i] + y[i - 1]);
      s *= 0.5;
    }
    if (s < 0) s = std::fabs(s);
    o.filter_norm = s;
    if (o.has_profile)
      for (double r : o.filter_grid)
        if (r < 0) throw unsupported("negative filter response combined with an instrument profile");
  }
  compose_operator_rows(m, o, !m.transmission, m.W, o.row_k0, o.row_len, o.row_off);
}

// The rows of one observation's composite operator (filter, convolution, bin integration)
// for flux (is_flux: wavenumber integral over the band) or wavelength integration,
// appended to W; k0 / len / off receive each row's first wavenumber, length and offset.
void compose_operator_rows(const Model& m, const ObservationSetup& o, bool is_flux, std::vector<double>& W,
                           std::vector<int>& row_k0, std::vector<int>& row_len, std::vector<long long>& row_off) {
  auto filt = [&](size_t k) -> double {
    return o.nfilter ? o.filter_grid[k] * o.filter_weight[k] / o.filter_norm : 1.0;
  };
  row_k0.resize(o.n);
  row_len.resize(o.n);
  row_off.resize(o.n);
  for (int b = 0; b < o.n; ++b) {
    const size_t i0 = o.edge_idx[b][0], i1 = o.edge_idx[b][1];
    // band integration weights on the (convolved) points i0..i1
    std::vector<double> bw(i1 - i0 + 1, 0.0);
    double scale;
    if (is_flux) {
      // bandIntegrateSpectrumFlux src/spectral_grid/spectral_band_integrate.cpp:66-80
      const double wl_l = 1.0 / m.nu[i0] * 1e4, wl_r = 1.0 / m.nu[i1] * 1e4;
      for (size_t i = i0 + 1; i < i1 + 1; ++i) {
        const double d = m.nu[i] - m.nu[i - 1];
        bw[i - i0] += d;
        bw[i - 1 - i0] += d;
      }
      scale = 0.5 / (wl_l - wl_r);
    } else {
      // bandIntegrateSpectrum :85-107 (absolute value of a negative wavelength integral)
      for (size_t i = i0 + 1; i < i1 + 1; ++i) {
        const double d = m.wl[i] - m.wl[i - 1];
        bw[i - i0] += d;
        bw[i - 1 - i0] += d;
      }
      scale = -0.5;
      if (!o.nfilter) scale /= (m.wl[i0] - m.wl[i1]);
    }
    // k range of the composite row
    size_t klo = i0, khi = i1;
    if (o.has_profile) {
      for (size_t i = i0; i <= i1; ++i) {
        if (i < o.range_lo || i > o.range_hi) continue;
        const auto& c = o.conv[i - o.range_lo];
        klo = std::min(klo, c[0]);
        khi = std::max(khi, c[1]);
      }
    }
    std::vector<double> row(khi - klo + 1, 0.0);
    for (size_t i = i0; i <= i1; ++i) {
      const double wb = bw[i - i0] * scale;
      if (wb == 0.0) continue;
      if (!o.has_profile) {
        row[i - klo] += wb * filt(i);
        continue;
      }
      if (i < o.range_lo || i > o.range_hi) continue;  // convolved spectrum is zero outside the range
      const auto& c = o.conv[i - o.range_lo];
      // SpectralBands::convolveSpectrum :116-144
      if (c[0] == c[1] || o.sigma[i] == 0) {
        row[i - klo] += wb * filt(i);
        continue;
      }
      const size_t s = c[0], e = c[1];
      if (e - s == 1) {
        row[s - klo] += wb * filt(s) * normal_dist(o.sigma[i], std::fabs(m.wl[i] - m.wl[s]));
        continue;
      }
      // |0.5 sum (x_j - x_{j-1}) (y_j + y_{j-1})| with x descending -> -0.5 * ...
      for (size_t j = s; j < e; ++j) {
        double cw = 0.0;
        if (j > s) cw += m.wl[j] - m.wl[j - 1];
        if (j + 1 < e) cw += m.wl[j + 1] - m.wl[j];
        const double g = normal_dist(o.sigma[i], std::fabs(m.wl[i] - m.wl[j]));
        row[j - klo] += wb * (-0.5 * cw) * g * filt(j);
      }
    }
    row_k0[b] = (int)klo;
    row_len[b] = (int)row.size();
    row_off[b] = (long long)W.size();
    W.insert(W.end(), row.begin(), row.end());
  }
}

// ------------------------------------------------------------------ opacity tables
// OpacitySpecies::readFileList src/transport_coeff/opacity_species.cpp:66-122,
// orderDataList :129-156, CrossSectionFile::loadFile
// src/transport_coeff/cross_section_file.cpp:33-68, SampledData::sampleCrossSections
// src/transport_coeff/sampled_data.cpp:48-87.
static void load_table(Model& m, OpacitySpecies& op, const std::string& folder) {
  const std::string list = m.xsec_path + folder + "/filelist.dat";
  std::ifstream f(list);
  if (!f) throw Error(BEAR_ERR_FILE, "No line absorption data found: " + list);
  std::string line;
  std::getline(f, line);
  std::istringstream first(line);
  std::string storage;
  op.mass = 0;
  first >> op.mass >> storage;
  const bool log_storage = storage == "log";
  struct Entry { double p, T; std::string file; };
  std::vector<Entry> entries;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    Entry e;
    if (ls >> e.p >> e.T >> e.file) entries.push_back(e);
  }
  if (entries.empty()) throw Error(BEAR_ERR_FILE, "empty cross-section list " + list);
  for (auto& e : entries)
    if (std::find(op.T.begin(), op.T.end(), e.T) == op.T.end()) op.T.push_back(e.T);
  std::sort(op.T.begin(), op.T.end());
  const size_t nT = op.T.size();
  op.P.assign(nT, {});
  op.logP.assign(nT, {});
  op.row.assign(nT, {});
  std::vector<float> buf;
  for (size_t t = 0; t < nT; ++t) {
    std::vector<const Entry*> rows;
    for (auto& e : entries)
      if (e.T == op.T[t]) rows.push_back(&e);
    std::stable_sort(rows.begin(), rows.end(), [](const Entry* a, const Entry* b) { return a->p < b->p; });
    for (const Entry* e : rows) {
      op.P[t].push_back(e->p);
      op.logP[t].push_back(std::log10(e->p));
      const std::string path = m.xsec_path + folder + "/" + e->file;
      std::ifstream df(path, std::ios::binary | std::ios::ate);
      if (!df) throw Error(BEAR_ERR_FILE, "cross section file " + path + " not found");
      const size_t nd = (size_t)df.tellg() / sizeof(float);
      df.seekg(0);
      buf.resize(nd);
      df.read(reinterpret_cast<char*>(buf.data()), nd * sizeof(float));
      const int row = (int)m.n_rows++;
      op.row[t].push_back(row);
      m.table_host.resize((size_t)m.n_rows * m.N);
      double* r = m.table_host.data() + (size_t)row * m.N;
      for (size_t k = 0; k < m.N; ++k) r[k] = 0.0;
      for (size_t k = 0; k < m.N; ++k) {
        if (m.index_list[k] > nd - 1) break;
        double v = buf[m.index_list[k]];
        if (log_storage) v = std::pow(10.0, v);
        r[k] = v;
      }
      for (size_t k = 0; k < m.N; ++k) {
        if (op.mass > 0) r[k] *= op.mass / 6.022140857e23;
        if (r[k] < 1e-200) r[k] = 1e-200;
      }
      for (size_t k = 0; k < m.N; ++k) r[k] = std::log10(r[k]);
    }
  }
}

// Rayleigh cross sections src/transport_coeff/species_rayleigh_cross_sections.cpp:25-234 and
// OpacitySpecies::generalRayleighCrossSection src/transport_coeff/opacity_species.cpp:528-537:
// H2, He (all wavelengths), H (Lee & Kim 2002 expansion), CO, CO2, CH4, H2O (zero beyond
// 2 micron; H2O from the refractive index of water at standard conditions).
static void tabulate_rayleigh(Model& m, OpacitySpecies& op) {
  const int sp = op.index;
  if (sp != SP_H2 && sp != SP_He && sp != SP_H && sp != SP_CO && sp != SP_CO2 && sp != SP_CH4 && sp != SP_H2O)
    throw unsupported(std::string("Rayleigh scattering of ") + kSpeciesSymbol[sp] +
                      " is not supported (H2, He, H, CO, CO2, CH4, H2O)");
  op.rayleigh.assign(m.N, 0.0);
  for (size_t j = 0; j < m.N; ++j) {
    const double nu = m.nu[j], wl = m.wl[j];
    double n = 1.0, nref = 2.546899e19, king = 1.0;
    if (sp == SP_H2) {
      n = (13.58e-5 * (1. + 7.52e-3 / std::pow(wl, 2))) + 1.;
      nref = 2.651629e19;
    } else if (sp == SP_He) {
      n = (2283. + 1.8102e13 / (1.5342e10 - nu * nu)) * 1e-8 + 1;
    } else if (sp == SP_H) {
      const double f = 0.0912 / wl;  // Lyman limit / wavelength
      op.rayleigh[j] = 8.41e-25 * std::pow(f, 4) + 3.37e-24 * std::pow(f, 6) + 4.71e-22 * std::pow(f, 14);
      continue;
    } else {
      if (wl > 2.0) continue;
      const double nu2 = nu * nu;
      if (sp == SP_CO) {
        n = (22851. + 0.456e14 / (71427.0 * 71427.0 - nu2)) * 1e-8 + 1;
      } else if (sp == SP_CO2) {
        king = 1.1364 + 25.3e-12 * nu2;
        n = (5799.25 / (128908.9 * 128908.9 - nu2) + 120.05 / (89223.8 * 89223.8 - nu2) +
             5.3334 / (75037.5 * 75037.5 - nu2) + 4.3244 / (67837.7 * 67837.7 - nu2) +
             0.1218145e-6 / (2418.136 * 2418.136 - nu2)) * 1.1427e3 + 1.0;
      } else if (sp == SP_CH4) {
        n = (46662. + 4.02e-6 * nu2) * 1e-8 + 1;
      } else {  // H2O
        static const double a[8] = {0.244257733, 0.974634476e-2, -0.373234996e-2, 0.268678472e-3,
                                    0.158920570e-2, 0.245934259e-2, 0.900704920, -0.166626219e-1};
        const double delta = 1.0, theta = 1.0, luv = 0.229202, lir = 5.432937;
        nref = 3.34279671749673e+22;
        king = (6 + 3 * 3e-4) / (6 - 7 * 3e-4);
        const double lam = wl / 0.589;
        const double af = delta * (a[0] + a[1] * delta + a[2] * theta + a[3] * lam * lam * theta +
                                   a[4] * std::pow(lam, -2) + a[5] / (lam * lam - luv * luv) +
                                   a[6] / (lam * lam - lir * lir) + a[7] * delta * delta);
        n = std::pow(((2 * af + 1) / (1 - af)), 0.5);
      }
    }
    op.rayleigh[j] = 24. * std::pow(kPi, 3) * std::pow(nu, 4) / (nref * nref) *
                     std::pow((n * n - 1) / (n * n + 2), 2) * king;
  }
}

// GasHm::boundFreeAbsorption and freeFreeAbsorption src/transport_coeff/h_m.cpp:56-137: the
// wavelength-dependent parts. Row 0: the photo-detachment cross section (threshold 1.6419 um,
// valid above 0.125 um); rows 1-6: the free-free polynomials lambda^2 A + B + C/lambda + ...
// + F/lambda^4 of each power (5040/T)^((i+1)/2), with the coefficient set above 0.3645 um or
// from 0.1823 to 0.3645 um, times 1e-29 (zero outside).
static void tabulate_hm(Model& m) {
  static const double lambda_0 = 1.6419;
  static const double Cn[7] = {0.0, 152.519, 49.534, -118.858, 92.536, -34.194, 4.982};
  static const double A1[7] = {0.0, 0.0, 2483.3460, -3449.8890, 2200.0400, -696.2710, 88.2830};
  static const double B1[7] = {0.0, 0.0, 285.8270, -1158.3820, 2427.7190, -1841.4000, 444.5170};
  static const double C1[7] = {0.0, 0.0, -2054.2910, 8746.5230, -13651.1050, 8624.9700, -1863.8650};
  static const double D1[7] = {0.0, 0.0, 2827.7760, -11485.6320, 16755.5240, -10051.5300, 2095.2880};
  static const double E1[7] = {0.0, 0.0, -1341.5370, 5303.6090, -7510.4940, 4400.0670, -901.7880};
  static const double F1[7] = {0.0, 0.0, 208.9520, -812.9390, 1132.7380, -655.0200, 132.9850};
  static const double A2[7] = {0.0, 518.1021, 473.2636, -482.2089, 115.5291, 0.0, 0.0};
  static const double B2[7] = {0.0, -734.8666, 1443.4137, -737.1616, 169.6374, 0.0, 0.0};
  static const double C2[7] = {0.0, 1021.1775, -1977.3395, 1096.8827, -245.6490, 0.0, 0.0};
  static const double D2[7] = {0.0, -479.0721, 922.3575, -521.1341, 114.2430, 0.0, 0.0};
  static const double E2[7] = {0.0, 93.1373, -178.9275, 101.7963, -21.9972, 0.0, 0.0};
  static const double F2[7] = {0.0, -6.4285, 12.3600, -7.0571, 1.5097, 0.0, 0.0};
  const size_t N = m.N;
  m.hm_rows.assign((size_t)kHmTerms * N, 0.0);
  for (size_t k = 0; k < N; ++k) {
    const double l = m.wl[k];
    if (l <= lambda_0 && l >= 0.125) {
      double f = 0;
      for (int i = 1; i < 7; ++i) f += Cn[i] * std::pow((1.0 / l - 1.0 / lambda_0), (i - 1) / 2.0);
      m.hm_rows[k] = 1e-18 * l * l * l * std::pow(1.0 / l - 1.0 / lambda_0, 1.5) * f;
    }
    const double *A = nullptr, *B = nullptr, *C = nullptr, *D = nullptr, *E = nullptr, *F = nullptr;
    if (l > 0.3645) { A = A1; B = B1; C = C1; D = D1; E = E1; F = F1; }
    else if (l >= 0.1823) { A = A2; B = B2; C = C2; D = D2; E = E2; F = F2; }
    if (!A) continue;
    for (int i = 1; i < 7; ++i)
      m.hm_rows[(size_t)i * N + k] =
          (l * l * A[i] + B[i] + C[i] / l + D[i] / l / l + E[i] / l / l / l + F[i] / l / l / l / l) * 1e-29;
  }
}

static void setup_opacity(Model& m) {
  // TransportCoefficients::addOpacitySpecies src/transport_coeff/transport_coeff.cpp:98-237
  m.hm = false;
  m.hm_rows.clear();
  m.n_rows = 0;
  m.table_host.clear();
  for (size_t i = 0; i < m.opac_cfg.size(); ++i) {
    const std::string& s = m.opac_cfg[i].first;
    const std::string& fo = m.opac_cfg[i].second;
    OpacitySpecies op;
    if (s == "CIA-H2-H2") { op.index = SP_H2; op.partners = {SP_H2}; }
    else if (s == "CIA-H2-He") { op.index = SP_H2; op.partners = {SP_He}; }
    else if (s == "CIA-H-He") { op.index = SP_H; op.partners = {SP_He}; }
    else if (s == "H-") {
      // GasHm: no tables, a continuum computed from T, n(H-), n(H) and n(e-)
      if (m.hm) throw invalid("the H- continuum is listed twice");
      m.hm = true;
      tabulate_hm(m);
      continue;
    }
    else if (fo == "Rayleigh") {
      op.index = species_id(s);
      if (op.index < 0) throw invalid("Opacity species " + s + " has not been found");
      op.kind = 1;
      tabulate_rayleigh(m, op);
      m.rayleigh_species.push_back((int)m.opac.size());
      m.opac.push_back(std::move(op));
      continue;
    } else {
      op.index = species_id(s);
      if (op.index < 0) throw invalid("Opacity species " + s + " has not been found");
    }
    op.kind = 0;
    load_table(m, op, fo);
    m.table_species.push_back((int)m.opac.size());
    m.opac.push_back(std::move(op));
  }
  if ((int)m.table_species.size() > kMaxTableSpecies) throw unsupported("too many opacity species");
  if ((int)m.rayleigh_species.size() > kMaxRayleigh) throw unsupported("too many Rayleigh species");
}

// ------------------------------------------------------------------ atmosphere constants
static void setup_atmosphere(Model& m) {
  AtmosphereConfig& a = m.acfg;
  std::memset(&a, 0, sizeof a);
  const int L = m.L;
  // Atmosphere::createPressureGrid src/forward_model/atmosphere/atmosphere.cpp:365-383
  m.p.assign(L, 0.0);
  const double minp = m.ptop, maxp = m.pbot;
  m.p[0] = std::log10(maxp);
  const double step = (std::log10(maxp) - std::log10(minp)) / (L - 1.0);
  for (int i = 1; i < L - 1; ++i) m.p[i] = m.p[i - 1] - step;
  for (int i = 0; i < L - 1; ++i) m.p[i] = std::pow(10.0, m.p[i]);
  m.p[L - 1] = minp;
  m.log10p.resize(L);
  for (int i = 0; i < L; ++i) m.log10p[i] = std::log10(m.p[i]);
  a.L = L;
  a.transmission = m.transmission;
  a.occultation = m.occultation;
  a.temp_poly = m.temp_poly;
  if (m.temp_poly) {
    // PiecewisePolynomial src/additional/piecewise_poly.cpp:36-121 (node table :36-44)
    static const double gl[7][5] = {{0.0},
                                     {-1.0, 1.0},
                                     {-1.0, 0.0, 1.0},
                                     {-1.0, -0.447214, 0.447214, 1.0},
                                     {-1.0, -0.654654, 0.654654, 1.0},
                                     {-1.0, -0.654654, 0.0, 0.654654, 1.0},
                                     {-1.0, -7.65055 - 0.285232, 0.285232, 0.765055, 1.0}};
    static const int gn[7] = {1, 2, 3, 4, 4, 5, 5};
    const int order = std::min(std::max(m.poly_order, 1), 6);
    const int nel = std::max(m.poly_elements, 1);
    const int nd = gn[order];
    if (nel * (nd - 1) + 1 > kMaxPolyDof || nel * nd > kMaxPolyDof * 8)
      throw unsupported("too many piecewise-polynomial elements");
    a.pp_nel = nel;
    a.pp_ndof_el = nd;
    for (int i = 0; i < nd; ++i) a.pp_ref[i] = gl[order][i];
    const double lb0 = std::log10(m.pbot), lb1 = std::log10(m.ptop);
    const double size = (lb0 - lb1) / nel;
    std::vector<double> edges(nel + 1);
    edges.front() = lb0;
    edges.back() = lb1;
    for (int i = 1; i < nel; ++i) edges[i] = edges[i - 1] - size;
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < nd; ++i)
        a.pp_el_vert[e * nd + i] = edges[e] + (1.0 + a.pp_ref[i]) / 2.0 * (edges[e + 1] - edges[e]);
    int c = 0;
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < nd - 1; ++i) a.pp_dof_vertices[c++] = a.pp_el_vert[e * nd + i];
    a.pp_dof_vertices[c++] = a.pp_el_vert[(nel - 1) * nd + nd - 1];
    a.pp_ndof = c;
    m.nparam_temp = nel * order + 1;  // PiecewisePolynomialTemperature ctor :33-43
  } else {
    m.nparam_temp = 1;
  }
  a.nchem = (int)m.chem.size();
  for (int c = 0; c < a.nchem; ++c) {
    a.chem_kind[c] = m.chem[c].kind;
    a.chem_nsp[c] = (int)m.chem[c].sp.size();
    for (size_t j = 0; j < m.chem[c].sp.size(); ++j) a.chem_sp[c][j] = m.chem[c].sp[j];
    a.chem_na_free[c] = m.chem[c].na_free;
    a.chem_bg_h2he[c] = m.chem[c].bg_h2he;
    a.chem_bg_sp[c] = m.chem[c].bg_sp;
  }
  a.cloud = m.cloud;
  a.cloud_fb = m.cloud_fb;
  a.cloud_kind = m.cloud ? m.cloud_kind : 0;
  a.cloud_ref_wl = m.cloud_ref_wl;
  a.fit_mmw = m.fit_mmw;
  // variable gravity applies to transmission models only: the emission and secondary-eclipse
  // models compute their structure with constant gravity (EmissionModel::calcAtmosphereStructure
  // src/forward_model/emission/emission.cpp:178-185, OccultationModel::calcAtmosphereStructure
  // src/forward_model/secondary_eclipse/secondary_eclipse.cpp:165-172 pass false)
  a.var_g = m.var_g && m.transmission;
  // table species: temperature nodes and the (parameter-independent) pressure bracket of
  // every level for every temperature row (OpacitySpecies::findClosestDataPoints
  // src/transport_coeff/opacity_species.cpp:204-269)
  a.S = (int)m.table_species.size();
  m.table_T.clear();
  m.pb_row0.clear();
  m.pb_row1.clear();
  m.pb_w.clear();
  for (int s = 0; s < a.S; ++s) {
    const OpacitySpecies& op = m.opac[m.table_species[s]];
    a.sp_index[s] = op.index;
    a.sp_partner[s][0] = op.partners.size() > 0 ? op.partners[0] : -1;
    a.sp_partner[s][1] = op.partners.size() > 1 ? op.partners[1] : -1;
    a.sp_nT[s] = (int)op.T.size();
    a.sp_T_off[s] = (int)m.table_T.size();
    a.sp_pb_off[s] = (int)m.pb_row0.size();
    for (double T : op.T) m.table_T.push_back(T);
    for (size_t t = 0; t < op.T.size(); ++t) {
      const std::vector<double>& P = op.P[t];
      const int np = (int)P.size();
      for (int l = 0; l < L; ++l) {
        const double p = m.p[l];
        int q0 = 0, q1 = 0;
        if (p < P.front()) q0 = q1 = 0;
        else if (p > P.back()) q0 = q1 = np - 1;
        else {
          for (int i = 0; i < np; ++i) {
            if (P[i] == p) { q0 = q1 = i; break; }
            else if (P[i] < p && P[i + 1] > p) { q0 = i; q1 = i + 1; break; }
          }
        }
        m.pb_row0.push_back(op.row[t][q0]);
        m.pb_row1.push_back(op.row[t][q1]);
        double w = 0.0;
        if (q0 != q1) w = (m.log10p[l] - op.logP[t][q0]) / (op.logP[t][q1] - op.logP[t][q0]);
        m.pb_w.push_back(w);
      }
    }
  }
  a.R_ray = (int)m.rayleigh_species.size();
  for (int r = 0; r < a.R_ray; ++r) a.ray_index[r] = m.opac[m.rayleigh_species[r]].index;
  a.hm = m.hm;
  a.R = a.R_ray + (m.hm ? kHmTerms : 0);
}

// ------------------------------------------------------------------ stellar spectrum
static std::vector<float> read_floats(const std::string& path, const char* what) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) throw Error(BEAR_ERR_FILE, std::string(what) + " " + path + " not found");
  const std::streamoff n = f.tellg() / (std::streamoff)sizeof(float);
  std::vector<float> v((size_t)n);
  f.seekg(0);
  f.read(reinterpret_cast<char*>(v.data()), n * (std::streamoff)sizeof(float));
  return v;
}

// StarSpectrumFile::readSpectrum src/forward_model/stellar_spectrum/star_file_spectrum.cpp:85-130:
// "wavelength flux" lines (W m^-2 um^-1), converted to W m^-2 cm (x wl^2 / 1e4) and
// interpolated linearly onto the model's wavelengths (zero outside the file's range).
static void load_star_file(Model& m) {
  std::ifstream f(m.star_path);
  if (!f) throw Error(BEAR_ERR_FILE, "stellar spectrum file " + m.star_path + " not found");
  std::vector<double> x, y;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    double a, b;
    if (!(ls >> a >> b)) continue;
    x.push_back(a);
    y.push_back(b);
  }
  if (x.size() < 2) throw invalid("stellar spectrum file " + m.star_path + " has fewer than two points");
  for (size_t i = 0; i < y.size(); ++i) y[i] = y[i] * x[i] * x[i] / 10000.;
  m.star_hr = interp_to_wavelengths(x, y, m.wl.data(), m.N);
}

// StellarSpectrumGrid src/forward_model/stellar_spectrum/stellar_spectrum_grid.cpp:42-210:
// <folder>grid_parameters.dat holds the T_eff, log g and [M/H] nodes (one line each), the
// name of the float32 wavelength file, then one "T_eff log_g [M/H] file" line per spectrum
// (float32 fluxes). Every spectrum is sampled onto the model grid here
// (SampledStellarSpectrum::sampleSpectrum sampled_stellar_spectrum.cpp:47-80: x wl^2 / 1e4,
// linear interpolation, values below 1e-37 raised to 1e-37), once, instead of on first use.
// As in the reference, a folder path without a trailing '/' is extended with '+'.
static void load_star_grid(Model& m) {
  std::string folder = m.star_path;
  if (folder.empty() || folder.back() != '/') folder += "+";
  const std::string pfile = folder + "grid_parameters.dat";
  std::ifstream f(pfile);
  if (!f) throw Error(BEAR_ERR_FILE, "stellar grid parameter file " + pfile + " not found");
  std::vector<double> axis[3];
  std::string line;
  for (int a = 0; a < 3; ++a) {
    std::getline(f, line);
    std::istringstream ls(line);
    double v;
    while (ls >> v) axis[a].push_back(v);
    if (axis[a].empty()) throw invalid("stellar grid " + pfile + ": an empty parameter line");
    for (size_t i = 1; i < axis[a].size(); ++i)
      if (!(axis[a][i] > axis[a][i - 1])) throw invalid("stellar grid " + pfile + ": nodes must ascend");
  }
  std::string wl_name;
  f >> wl_name;
  std::getline(f, line);
  std::vector<std::string> entries;
  while (std::getline(f, line)) entries.push_back(line);
  const size_t n0 = axis[0].size(), n1 = axis[1].size(), n2 = axis[2].size();
  if (entries.size() != n0 * n1 * n2)
    throw invalid("Stellar spectrum grid is inconsistent. The number of files does not correspond to the number "
                  "of given effective temperatures, log g, and metallicities!");
  const std::vector<float> wlf = read_floats(folder + wl_name, "stellar grid wavelength file");
  std::vector<double> gwl(wlf.begin(), wlf.end());
  m.star_hr.assign(n0 * n1 * n2 * m.N, 0.0);
  std::vector<char> seen(n0 * n1 * n2, 0);
  for (const std::string& e : entries) {
    std::istringstream ls(e);
    double v[3];
    std::string name;
    if (!(ls >> v[0] >> v[1] >> v[2] >> name)) throw invalid("stellar grid " + pfile + ": bad line '" + e + "'");
    size_t idx[3];
    for (int a = 0; a < 3; ++a) {
      auto it = std::find(axis[a].begin(), axis[a].end(), v[a]);
      if (it == axis[a].end()) throw invalid("stellar grid " + pfile + ": a spectrum off the parameter nodes");
      idx[a] = (size_t)(it - axis[a].begin());
    }
    const size_t c = (idx[0] * n1 + idx[1]) * n2 + idx[2];
    if (seen[c]) throw invalid("Stellar spectra grid seems to be incomplete. Possibly duplicates?");
    seen[c] = 1;
    const std::vector<float> fl = read_floats(folder + name, "stellar grid spectrum");
    if (fl.size() != gwl.size())
      throw invalid("spectrum file " + folder + name + " has an incorrect number of spectral points");
    std::vector<double> y(fl.size());
    for (size_t i = 0; i < y.size(); ++i) y[i] = (double)fl[i] * gwl[i] * gwl[i] / 10000.;
    std::vector<double> s = interp_to_wavelengths(gwl, y, m.wl.data(), m.N);
    for (double& q : s)
      if (q < 1e-37) q = 1e-37;
    std::copy(s.begin(), s.end(), m.star_hr.begin() + c * m.N);
  }
  m.star_axes.clear();
  for (int a = 0; a < 3; ++a) {
    m.star_n[a] = (int)axis[a].size();
    m.star_axes.insert(m.star_axes.end(), axis[a].begin(), axis[a].end());
  }
}

// Stellar spectra through the observation operator: the binned stellar flux of every
// operator row (the binning is linear, so the grid model interpolates these instead of
// binning an interpolated spectrum).
static void setup_star(Model& m) {
  m.star_hr.clear();
  m.star_bin.clear();
  if (m.star_model == 2) load_star_file(m);
  else if (m.star_model == 3) load_star_grid(m);
  else return;
  const size_t ns = m.star_hr.size() / m.N;
  m.star_bin.assign(ns * (size_t)m.M, 0.0);
  for (size_t c = 0; c < ns; ++c) {
    const double* F = m.star_hr.data() + c * m.N;
    size_t r = 0;
    for (const auto& o : m.obs)
      for (int b = 0; b < o.n; ++b, ++r) {
        double s = 0.0;
        const double* w = m.W.data() + o.row_off[b];
        for (int j = 0; j < o.row_len[b]; ++j) s += w[j] * F[o.row_k0[b] + j];
        m.star_bin[c * m.M + r] = s;
      }
  }
}

void finalize_host(Model& m) {
  if (m.prepared) throw Error(BEAR_ERR_STATE, "model already prepared");
  if (m.obs.empty()) throw invalid("No observations given");
  load_wavenumbers(m);
  sample_grid(m);
  m.W.clear();
  m.M = 0;
  for (auto& o : m.obs) {
    o.out_offset = m.M;
    m.M += o.n;
  }
  setup_opacity(m);
  for (auto& o : m.obs) build_observation_operator(m, o);
  setup_star(m);
  setup_atmosphere(m);
  // parameter layout: EmissionModel::extractParameters src/forward_model/emission/emission.cpp:123-153,
  // TransmissionModel::extractParameters src/forward_model/transmission/transmission.cpp:110-146,
  // OccultationModel::extractParameters src/forward_model/secondary_eclipse/secondary_eclipse.cpp:115-150
  // ([log g, R_p / R_s] and the stellar model's parameters; both counted as general here)
  m.nparam_general = 3 + ((m.transmission && m.fit_mmw) ? 1 : 0);
  if (m.occultation) m.nparam_general = 2 + (m.star_model == 1 ? 1 : m.star_model == 3 ? 3 : 0);
  m.nparam_chem = 0;
  for (auto& c : m.chem) m.nparam_chem += c.kind == 0 ? (int)c.sp.size() : 0;
  m.nparam_cloud = m.cloud ? (m.cloud_fb ? 2 : 3) + (m.cloud_kind == 1 ? 1 : m.cloud_kind == 2 ? 3 : 0) : 0;
  m.nparam_mod = 0;
  for (auto& o : m.obs) m.nparam_mod += o.nb_modifier;
  m.nparam_total = m.nparam_general + m.nparam_chem + m.nparam_temp + m.nparam_cloud + m.nparam_mod;
  AtmosphereConfig& a = m.acfg;
  a.nparam_general = m.nparam_general;
  a.nparam_chem = m.nparam_chem;
  a.nparam_temp = m.nparam_temp;
  a.nparam_cloud = m.nparam_cloud;
  a.nparam_mod = m.nparam_mod;
  a.nparam_total = m.nparam_total + (m.error_inflation ? 1 : 0);
  a.error_inflation = m.error_inflation;
}

}  // namespace bgb
