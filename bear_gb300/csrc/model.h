// Internal declarations of the GB300 likelihood engine (host set-up + device
// kernels). The public boundary is include/bear_gb300.h.
#pragma once

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace bgb {

// ----------------------------------------------------------------- constants
// Physical constants in cgs units, src/additional/physical_const.h:28-52.
constexpr double kPlanckH = 6.62606896e-27;
constexpr double kLightC = 2.99792458e10;
constexpr double kBoltzmann = 1.3806504e-16;
constexpr double kGravConst = 6.673e-8;
constexpr double kGasConst = 8.314472e7;
constexpr double kRJupiter = 7.1492e9;
constexpr double kPi = 3.14159265358979323846;

// Chemical species table, src/chemistry/chem_species.h:30-90. The id order is
// significant: the mean molecular weight is summed over it in this order.
constexpr int kSpeciesCount = 46;
enum SpeciesId : int {
  SP_TOTAL = 0, SP_H = 1, SP_He = 2, SP_H2 = 10, SP_H2O = 11, SP_CO2 = 12, SP_CO = 13, SP_CH4 = 14,
  SP_Na = 19, SP_K = 20, SP_Hm = 22, SP_e = 35
};
extern const char* const kSpeciesSymbol[kSpeciesCount];
extern const double kSpeciesMolWeight[kSpeciesCount];
int species_id(const std::string& symbol);

constexpr int kMaxLevels = 512;
constexpr int kMaxChemModules = 4;
constexpr int kMaxTableSpecies = 32;
constexpr int kMaxRayleigh = 8;
constexpr int kMaxPolyDof = 64;

// ----------------------------------------------------------------- device-side model description
// Everything the per-evaluation kernels need that does not depend on the
// parameters. Lives in device memory; kernels receive a pointer.
struct AtmosphereConfig {
  int L;                       // levels, index 0 = bottom (highest pressure)
  int transmission;            // 0 emission, 1 transmission
  int occultation;             // 1: secondary eclipse (emission with spectrum scaling 1)
  int nparam_general, nparam_chem, nparam_temp, nparam_cloud, nparam_mod, nparam_total;
  int error_inflation;
  // temperature: 0 const, 1 piecewise polynomial in log10 p
  int temp_poly, pp_nel, pp_ndof_el, pp_ndof;
  double pp_ref[8];
  double pp_dof_vertices[kMaxPolyDof];
  double pp_el_vert[kMaxPolyDof * 8];
  // chemistry modules applied in order
  int nchem;
  int chem_kind[kMaxChemModules];     // 0 isoprofile, 1 background
  int chem_nsp[kMaxChemModules];
  int chem_sp[kMaxChemModules][kSpeciesCount];
  int chem_na_free[kMaxChemModules];
  int chem_bg_h2he[kMaxChemModules];
  int chem_bg_sp[kMaxChemModules];
  // cloud: grey placement (kind 0), times a wavelength shape for the power-law (1) and
  // KH non-grey (2) clouds; parameters [tau, (exponent | q0, a0, size), p_top, (bottom factor)]
  int cloud, cloud_fb, cloud_kind;
  double cloud_ref_wl;
  // transmission options
  int fit_mmw, var_g;
  // opacity species with tables (line lists and CIA)
  int S;
  int sp_index[kMaxTableSpecies];
  int sp_partner[kMaxTableSpecies][2];  // -1 if unused
  int sp_nT[kMaxTableSpecies];
  int sp_T_off[kMaxTableSpecies];       // offset into table_T
  int sp_pb_off[kMaxTableSpecies];      // offset into pb_* arrays: [t][level]
  // linear opacity terms: R_ray Rayleigh species (scattering), then, with hm, the kHmTerms
  // terms of the H- continuum (absorption); R = R_ray + (hm ? kHmTerms : 0)
  int R, R_ray, hm;
  int ray_index[kMaxRayleigh];
};

// H- continuum (GasHm src/transport_coeff/h_m.cpp:36-137) as kHmTerms linear terms: row 0
// the bound-free cross section (coefficient n(H-)), rows 1-6 the free-free polynomials
// in wavelength (coefficients (5040/T)^((i+1)/2) 1e-29 P_e n(H)); all zero when n(H-) = 0.
constexpr int kHmTerms = 7;

// Per (evaluation, level, table species): the four table rows of the
// interpolation stencil and its weights, plus the species' number density
// (product with collision partners for CIA).
struct __align__(16) LevelSpecies {
  int row[4];      // (T_lo, p_lo), (T_lo, p_hi), (T_hi, p_lo), (T_hi, p_hi): absolute row numbers
  double wp_lo;    // log-p weight on the T_lo rows
  double wp_hi;    // log-p weight on the T_hi rows
  double wT;       // temperature weight
  double n;        // number density (cm^-3, or cm^-6 for CIA pairs)
};

// Companion of LevelSpecies for the double-float opacity path: the two rows of
// the level table (the log-p interpolation at this level is precomputed for every
// temperature node) at the lower and upper temperature node, the temperature
// weight and log2 of the number density (lg2n_hi = kNoSpecies when the density is
// zero and the species is skipped), as double-floats.
struct __align__(16) LevelSpeciesDF {
  int lrow[2];
  int pad[2];
  float wT_hi, wT_lo, lg2n_hi, lg2n_lo;
};
constexpr float kNoSpecies = -1.0e30f;

// Per (evaluation, level).
struct __align__(16) LevelInfo {
  double T;        // temperature
  double invT;     // 1 / T
  double z;        // altitude (cm)
  double dz;       // z[l+1] - z[l] (0 on the top level)
  double cloud;    // emission: grey-cloud optical depth of layer l; transmission: cloud extinction at level l
  float invT_hi, invT_lo;    // 1 / T as a double-float
  float dzh_hi, dzh_lo;      // dz / 2 as a double-float
  float cloud_hi, cloud_lo;  // cloud as a double-float
};

// Per evaluation.
struct __align__(16) EvalInfo {
  double scaling;      // emission: (R_J / d)^2 f
  double radius;       // transmission: bottom (planet) radius
  double star_radius;  // transmission: stellar radius
  double inflation;    // 10^b error inflation (0 if off)
  int neglect;
  int cloud_top, cloud_bottom;
  int pad;
  // non-grey cloud shape: power law {exponent, -, -, ref_wl^exponent};
  // KH {q0, a0, 2 pi size, Q(reference size parameter)}
  double cs[4];
};

// One parameter's prior on the device (Retrieval's PriorConfig list). a, b: uniform
// bounds (ordered), log10 of the log-uniform bounds (ordered), Gaussian mean and
// standard deviation, or the delta value; link: the linked parameter (linked priors).
enum PriorType : int { kPriorUniform = 0, kPriorLogUniform = 1, kPriorGaussian = 2, kPriorDelta = 3, kPriorLinked = 4 };
constexpr int kMaxPriors = 256;
struct DevicePrior {
  int type;
  int link;
  double a, b, unit;
};

// Device pointers and sizes for the kernels (passed by value).
struct DeviceModel {
  const AtmosphereConfig* cfg;
  int L, S, R, N, M, P, nobs;
  // grid
  const double* nu;           // N
  const double* wl;           // N
  const double* planck_c1;    // N: 2 h c^2 nu^3
  const double* planck_c2;    // N: h nu c / k
  const float2* planck_c1_df; // N: 2 h c^2 nu^3 as double-float
  const float2* planck_c2l_df;// N: (h nu c / k) log2(e) as double-float
  const float2* ltab;         // level table: per (species, temperature node, level) the
                              // log-p-interpolated cross section in log2 units, x N, double-float
                              // (row = the pressure-bracket index sp_pb_off[s] + t L + l)
  // atmosphere constants
  const double* pressure;     // L (bar)
  const double* log10p;       // L
  // tables
  const double* table64;      // rows x N, log10 cross sections
  const double* table_T;      // all species' temperature nodes
  const int* pb_row0;         // per species [nT][L]: absolute row of the lower pressure node
  const int* pb_row1;         // upper pressure node
  const double* pb_w;         // log-p weight
  const double* rayleigh;     // R x N: Rayleigh cross sections, then the H- continuum rows
  const float2* rayleigh_df;  // R x N as double-floats
  int R_ray;                  // Rayleigh rows (the rest, R - R_ray, are H- continuum rows)
  int cloud_kind;             // 0 grey (or no cloud), 1 power law, 2 KH non-grey
  int annuli;                 // transmission: impact parameters per layer (1: the reference's tangent rays)
  // observation operator: M rows, internal (descending-wavelength) order
  const int* row_k0;
  const int* row_len;
  const long long* row_off;
  const double* W;
  const int* row_obs;
  const int* row_out;         // index in the caller-order output
  const double* row_data;
  const double* row_err2;
  const double* row_weight;
  const double* row_logterm;  // -0.5 log(2 pi sigma^2) (no inflation)
  const int* obs_mod_param;   // per observation: parameter index of the shift, or -1
  const int* obs_row_start;   // nobs + 1: first operator row of each observation
  // tangent-ray cut-off of the transmission sums (the reference's tau > 10): FP64 bit
  // pattern (tau >= 0 compares as an integer) and double-float split
  long long tau_cut_bits;
  float tau_cut_hi, tau_cut_lo;
  // transposed observation operator (adjoint): per wavenumber the rows that read it
  const int* col_ptr;         // N + 1
  const int* col_row;         // nnz
  const double* col_w;        // nnz
  // secondary eclipse: the stellar spectrum (star_model 1 blackbody at T_eff = params[2],
  // 2 file, 3 grid over (T_eff, log g, [M/H]) = params[2..4]); 0 for other models
  int star_model;
  int star_n[3];              // grid: nodes per axis
  const double* star_axes;    // grid: star_n[0] + star_n[1] + star_n[2] ascending nodes
  const double* star_hr;      // file: N; grid: spectra x N, spectrum (t, g, m) at (t n1 + g) n2 + m
  const double* star_bin;     // file: M; grid: spectra x M: the stellar spectrum through each row
};

// Work buffers for a batch of evaluations.
struct Workspace {
  int capacity = 0;
  double* params = nullptr;    // B x P (plain path staging)
  LevelInfo* lev = nullptr;    // B x L
  LevelSpecies* ls = nullptr;  // B x L x S
  LevelSpeciesDF* lsdf = nullptr;  // B x L x S
  double* ray_n = nullptr;     // B x L x R number densities of the Rayleigh species
  EvalInfo* ev = nullptr;      // B
  double* spectrum = nullptr;  // B x N native units
  double* obs = nullptr;       // B x M internal order
  double* loglike = nullptr;   // B
  double* geom = nullptr;      // transmission path lengths B x L x L (B x K x L with K = (L-1) A annuli)
  double* rays = nullptr;      // transmission: B x 2 (K + 1): ray altitudes, effective-height weights
};

// Extra outputs of the forward pass that the adjoint reads back.
struct ForwardTaps {
  float2* dwT = nullptr;     // B x L x S: d wT / dT of every stencil (double-float)
  double* istore = nullptr;  // emission, B x L x 2 x N: Gauss-angle intensities after every level
  float4* em_layer = nullptr;  // emission, B x L x N: layer optical depth and (k_l + k_{l-1}) / 2
                               // as double-floats (layer l between levels l-1 and l; l = 0 unused)
  // transmission, per (evaluation, level, wavenumber) as double-floats unless noted
  float2* tr_geo = nullptr;  // per evaluation 3 x L x L: dG/dz_j (P, transposed), dG/dz_t (Q),
                             // the path lengths G transposed
  float2* tr_c = nullptr;    // extinction pair sums chi_i + chi_{i+1}
  float2* tr_T = nullptr;    // tangent-ray transmission T_t
  float2* tr_qs = nullptr;   // sum_i c_i Q[t][i] over the ray's terms
  float2* tr_us = nullptr;   // pass 2a: A_t = (R + z_t)(1 - T_t)
  short* tr_I = nullptr;     // last level index inside the cut-off
  // (with A impact parameters per layer tr_T, tr_qs, tr_us and tr_I hold one row per ray,
  // K = (L - 1) A rows, and tr_geo 3 x L x K per evaluation)
  float2* tr_d = nullptr;    // A > 1: extinction differences chi_{i+1} - chi_i
  // transmission, when the gradient's memory budget allows (else the adjoint recomputes them):
  float2* tr_ts = nullptr;   // B x L x S x N: each table species' opacity term n_s sigma_s
  float2* tr_dk = nullptr;   // B x L x N: sum_s term_s (hi_s - lo_s) d wT_s / dT; x = NaN where a
                             // term lies outside the float range (the adjoint recomputes there)
};

// Work buffers of the gradient for a chunk of evaluations.
struct GradWorkspace {
  int capacity = 0;
  int tiles = 0;             // wavenumber tiles of the adjoint kernel (partials per level value)
  ForwardTaps taps;
  double* gS = nullptr;      // B x M: d log L / d binned model
  double* seed = nullptr;    // B x 3: seed normaliser, its inverse, sum_r gS_r (s_r - shift_r)
  double* partial = nullptr; // B x L x V x tiles per-block sinks of the adjoint kernel(s)
  float2* em_gK = nullptr;   // emission, B x L x N: d log L / d kappa per level (double-float)
  // transmission adjoint, per (evaluation, level, wavenumber), double-floats
  float2* tr_gc = nullptr;    // d log L / d (chi_j + chi_{j+1})
  float2* tr_gz = nullptr;    // d log L / d z_j
  float2* tr_gd = nullptr;    // A > 1: d log L / d (chi_{j+1} - chi_j) (the first, partial ray segments)
  double* tr_rp = nullptr;    // per (evaluation, tile) partial d log L / d R_p
  double* tr_cs = nullptr;    // non-grey cloud: B x (1 + NC) x N wavelength factor and its shape derivatives
  bool tr_store = false;      // the forward pass stores the opacity terms (taps.tr_ts, tr_dk)
};

// ----------------------------------------------------------------- host model
struct ObservationSetup {
  std::string name;
  int type = 0;  // 0 spectroscopy, 1 photometry, 2 band-spectroscopy
  int n = 0;
  bool ascending = false;
  int nb_modifier = 0;
  int out_offset = 0;   // offset in the concatenated outputs
  std::vector<double> data, error, weight, fwhm, centers;
  std::vector<std::array<double, 2>> edges, edge_nu;
  double wl_edges[2] = {0, 0};
  double obs_nu_range[2] = {0, 0};
  size_t range_lo = 0, range_hi = 0;
  std::vector<std::array<size_t, 2>> edge_idx;
  bool has_profile = false;
  std::vector<double> sigma;
  std::vector<std::array<size_t, 2>> conv;
  int nfilter = 0;
  bool photon = false;
  std::vector<double> filter_wl, filter_resp, filter_grid, filter_weight;
  double filter_norm = 0;
  // composite operator rows (internal order)
  std::vector<int> row_k0, row_len;
  std::vector<long long> row_off;
};

struct OpacitySpecies {
  int kind = 0;  // 0 tabulated (line list / CIA), 1 Rayleigh only
  int index = 0;
  std::vector<int> partners;
  double mass = 0;
  std::vector<double> T;                    // ascending
  std::vector<std::vector<double>> P, logP; // per T, ascending
  std::vector<std::vector<int>> row;        // absolute packed row per (t, q)
  std::vector<double> rayleigh;             // N (kind 1)
};

struct ChemModule {
  int kind = 0;  // 0 iso, 1 background
  std::vector<int> sp;
  bool na_free = false;
  bool bg_h2he = false;
  int bg_sp = -1;
};

// Device copies of a model's opacity tables (FP64 table, level table, stencil
// brackets). Models on the same device with the same table files, spectral grid
// and pressure grid share one set (engine.cu keeps a registry).
struct TableSet;

struct Model {
  // configuration
  bool transmission = false;
  std::string xsec_path, wn_file;
  int discretisation = 0;
  double resolution = 1.0;
  bool error_inflation = false;
  int L = 0;
  double pbot = 0, ptop = 0;
  bool temp_poly = false;
  int poly_elements = 0, poly_order = 0;
  std::vector<ChemModule> chem;
  bool cloud = false, cloud_fb = false;
  int cloud_kind = 0;             // 0 grey, 1 power_law, 2 KHnongrey
  double cloud_ref_wl = 0.0;      // reference wavelength (micron) of the non-grey clouds
  bool fit_mmw = false, fit_sh = false, var_g = false;
  int annuli = 1;                 // transmission impact parameters per layer (not in the reference)
  bool occultation = false;
  bool hm = false;                // H- continuum configured
  int star_model = 0;             // 1 blackbody, 2 file, 3 grid
  std::string star_path;          // file path (2) or grid folder (3)
  std::vector<std::pair<std::string, std::string>> opac_cfg;
  // set-up products
  std::vector<ObservationSetup> obs;
  std::vector<double> nu_full, wl_full;
  std::vector<size_t> index_list;
  std::vector<double> nu, wl;
  size_t N = 0;
  std::vector<double> p, log10p;
  std::vector<OpacitySpecies> opac;  // config order
  std::vector<int> table_species;    // indices into opac with kind 0
  std::vector<int> rayleigh_species; // indices into opac with kind 1
  long long n_rows = 0;
  long long n_lrows = 0;             // rows of the level table
  std::vector<double> table_host;    // n_rows x N (freed after upload)
  std::vector<double> W;             // concatenated operator weights
  std::vector<double> hm_rows;       // kHmTerms x N wavelength parts of the H- continuum
  // stellar spectrum of the secondary-eclipse model (file: 1 spectrum; grid: all)
  std::vector<double> star_hr;       // spectra x N on the model grid
  std::vector<double> star_bin;      // spectra x M through the observation rows
  std::vector<double> star_axes;
  int star_n[3] = {0, 0, 0};
  int M = 0;
  int nparam_general = 0, nparam_chem = 0, nparam_temp = 0, nparam_cloud = 0, nparam_mod = 0;
  int nparam_total = 0;
  AtmosphereConfig acfg{};
  std::vector<int> pb_row0, pb_row1;
  std::vector<double> pb_w, table_T;
  bool prepared = false;
  bool finalized = false;
  // device
  int device = 0;
  int precision = 0;  // 0: double-float opacity + table exponentials, 1: FP64 libm kernels
  int rt_threads = 0, obs_threads = 0;
  int tuned_rt = 0;           // autotuned radiative-transfer launch shape for batches > 1 (0: default)
  unsigned ws_generation = 0; // bumped whenever the workspace is reallocated (captured graphs check it)
  DeviceModel dm{};
  std::vector<void*> allocations;
  size_t device_bytes = 0;
  AtmosphereConfig* d_cfg = nullptr;
  double* d_table64 = nullptr;
  std::shared_ptr<TableSet> tables;   // shared device tables
  bool tables_shared = false;         // true when another model created them
  Workspace ws;
  GradWorkspace gws;
  size_t grad_budget = size_t(32) << 30;  // bytes of gradient work buffers per chunk
  DevicePrior* d_priors = nullptr;  // prior table (bear_model_set_priors)
  // contribution functions: device L x N buffer and the wavelength-integration operator
  // (rows in internal order, cf_out = caller-order index), built on first use
  double* d_cf = nullptr;
  std::vector<double> cf_W;
  std::vector<int> cf_k0, cf_len, cf_out;
  std::vector<long long> cf_off;
  int n_priors = 0;
  double* h_pinned = nullptr;  // pinned staging for the plain path
  size_t h_pinned_bytes = 0;
  // stage timing (bear_model_set_profiling)
  bool profiling = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ev_recorded = false;
};

// model_setup.cpp
void parse_config(Model& m, const std::string& text);
void add_observation(Model& m, const char* name, const char* type, int n, const double* ce,
                     const double* data, const double* error, const double* weight,
                     const double* fwhm, int nfilter, const double* fwl, const double* fresp,
                     const char* detector, const char* modifier);
void finalize_host(Model& m);
void compose_operator_rows(const Model& m, const ObservationSetup& o, bool is_flux, std::vector<double>& W,
                           std::vector<int>& row_k0, std::vector<int>& row_len, std::vector<long long>& row_off);

// engine.cu
// transmission rays per evaluation: L - 1 tangent rays, (L - 1) A with annuli
inline int transmission_rays(const Model& m) { return (m.L - 1) * std::max(m.annuli, 1); }
void upload_model(Model& m);
void ensure_workspace(Model& m, int batch);
void release_model(Model& m);
void launch_forward(Model& m, const double* params_dev, int batch, cudaStream_t stream,
                    bool want_loglike, uint8_t* neglect_dev, double* loglike_dev);
void launch_spectrum_output(Model& m, double* out_dev, cudaStream_t stream);
size_t table_bytes(const Model& m);  // device bytes of the model's (possibly shared) tables
void set_tau_cutoff(Model& m, double tau);
void stage_times(Model& m, float* ms3);
// noalloc.cu
void loglike_noalloc(Model& m, const double* params_dev, double* loglike_dev, uint8_t* neglect_dev,
                     cudaStream_t stream);
long long stencil_rows(Model& m, int batch);
void launch_forward_taps(Model& m, const double* params_dev, int batch, cudaStream_t stream,
                         uint8_t* neglect_dev, double* loglike_dev, const ForwardTaps& taps);
// contribution.cu
void contribution_functions(Model& m, cudaStream_t stream, double* spectrum, double* bins);
// priors.cu
void set_priors(Model& m, int n, const int* type, const double* a, const double* b, const double* unit,
                const int* link);
void launch_prior_transform(Model& m, const double* cube_dev, int batch, double* params_dev, cudaStream_t stream);
// adjoint.cu
void launch_gradient(Model& m, const double* params_dev, int batch, cudaStream_t stream,
                     double* loglike_dev, double* grad_dev, uint8_t* neglect_dev);
void free_grad_workspace(Model& m);

struct Error : std::exception {
  int code;
  std::string msg;
  Error(int c, std::string s) : code(c), msg(std::move(s)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

// Throws Error(BEAR_ERR_CUDA) with the failing call and CUDA's message (the
// BEAR_ERR_* codes come from include/bear_gb300.h, which users of the macro include).
#define BGB_CUDA(x)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess)                                                                  \
      throw Error(BEAR_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));         \
  } while (0)


}  // namespace bgb
