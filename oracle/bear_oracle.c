/*
 * bear_oracle.c -- FP64 CPU restatement of the reference's per-likelihood
 * forward-model path. TEST INFRASTRUCTURE ONLY: it is the checker the GPU
 * engine is compared against (tests, smoke check, and the CPU-baseline leg of
 * the benchmark). Nothing in the product links or calls it.
 *
 * Each function names the reference function it restates (file:line, paths
 * inside the reference project). The operation order follows the reference so
 * that the same libm calls see the same arguments; FMA contraction is disabled
 * at build time (-ffp-contract=off) so results agree across x86-64 and aarch64.
 *
 * Pinned against the reference itself: tests/golden/ holds outputs of the
 * reference's CPU path (built from its sources by oracle/ref/Makefile) and
 * tests/test_oracle_golden.py checks this file against them.
 */
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ constants
 * src/additional/physical_const.h:28-52 */
#define K_PLANCK_H 6.62606896e-27
#define K_LIGHT_C 2.99792458e10
#define K_BOLTZMANN 1.3806504e-16
#define K_GRAV 6.673e-8
#define K_GAS 8.314472e7
#define K_RJUP 7.1492e9
#define K_MJUP 1.89813e30
#define K_PI 3.14159265358979323846

/* species table: src/chemistry/chem_species.h:30-90 (id order matters: the
 * mean molecular weight sums over it in this order) */
enum {
  SP_TOTAL, SP_H, SP_He, SP_C, SP_O, SP_Fe, SP_Fep, SP_Ca, SP_Ti, SP_Tip, SP_H2, SP_H2O, SP_CO2,
  SP_CO, SP_CH4, SP_HCN, SP_NH3, SP_C2H2, SP_N2, SP_Na, SP_K, SP_H2S, SP_Hm, SP_TiO, SP_VO,
  SP_FeH, SP_SH, SP_MgO, SP_AlO, SP_CaO, SP_CrH, SP_MgH, SP_CaH, SP_TiH, SP_OH, SP_e, SP_V,
  SP_Vp, SP_Mn, SP_Si, SP_Cr, SP_Crp, SP_SiO, SP_SiO2, SP_SO2, SP_CS2, SP_COUNT
};
static const char* SP_SYMBOL[SP_COUNT] = {
  "Total", "H", "He", "C", "O", "Fe", "Fe+", "Ca", "Ti", "Ti+", "H2", "H2O", "CO2", "CO", "CH4",
  "HCN", "NH3", "C2H2", "N2", "Na", "K", "H2S", "H-", "TiO", "VO", "FeH", "SH", "MgO", "AlO",
  "CaO", "CrH", "MgH", "CaH", "TiH", "OH", "e-", "V", "V+", "Mn", "Si", "Cr", "Cr+", "SiO",
  "SiO2", "SO2", "CS2"};
static const double SP_MW[SP_COUNT] = {
  0.0, 1.00784, 4.002602, 12.0107, 15.999, 55.845, 55.845, 40.078, 47.867, 47.867, 2.01588,
  18.01528, 44.01, 28.0101, 16.04246, 27.0253, 17.03052, 26.04, 28.0134, 22.98977, 39.0983,
  34.09099, 1.00784, 63.8664, 66.9409, 56.853, 34.08, 40.3044, 42.981, 56.0774, 54.0040,
  26.3209, 41.0859, 48.87484, 17.008, 5.4857990907e-4, 50.9415, 50.9415, 54.938044, 28.085,
  51.996, 51.996, 44.08, 60.08, 64.066, 76.139};

static int species_id(const char* s) {
  for (int i = 0; i < SP_COUNT; ++i)
    if (strcmp(SP_SYMBOL[i], s) == 0) return i;
  return -1;
}

/* ------------------------------------------------------------------ helpers */
static char g_err[512];
static void set_err(const char* fmt, ...) {
  va_list ap; va_start(ap, fmt); vsnprintf(g_err, sizeof g_err, fmt, ap); va_end(ap);
}
const char* orc_last_error(void) { return g_err; }

/* ------------------------------------------------------------------ model */
enum { BAND_SPEC = 0, BAND_PHOT = 1, BAND_BANDSPEC = 2 };

typedef struct {
  int type;
  int n;                     /* data points */
  int ascending;
  double* data; double* error; double* weight; /* internal (descending-wavelength) order */
  double* fwhm; int nfwhm;
  double (*edges)[2];        /* bin edges in wavelength, [0] > [1] */
  double* centers;
  double wl_edges[2];        /* Observation::wavelength_edges */
  double (*edge_nu)[2];
  double obs_nu_range[2];
  size_t range_lo, range_hi;  /* obs_index_range */
  size_t (*edge_idx)[2];
  double* sigma;             /* instrument_profile_sigma over the model grid (0 outside) */
  size_t (*conv)[2];          /* per point in the obs range */
  int has_profile;
  /* filter */
  int nfilter; double* filter_wl; double* filter_resp; int photon;
  double* filter_on_grid; double* filter_weight; double filter_norm;
  int nb_modifier;
  int out_offset;            /* offset into the concatenated user-order output */
} obs_t;

typedef struct {
  int kind;                  /* 0 line/CIA table, 1 Rayleigh only, 2 H- continuum */
  int index;                 /* species_index */
  int partner[2]; int npartner;
  double mass;
  int nT; double* T;         /* ascending */
  int* nP; double** P; double** logP;  /* per T, ascending */
  double*** rows;            /* rows[t][p] -> N log10 cross sections */
  double* rayleigh;          /* N */
  double* hm_bf;             /* N: H- bound-free cross section (kind 2) */
  double* hm_ff[7];          /* [1..6] x N: the free-free polynomials in wavelength (kind 2) */
} opac_t;

typedef struct orc_model {
  /* global */
  int transmission;
  int occultation;           /* secondary eclipse (OccultationModel) */
  int annuli;                /* impact parameters per layer of the transit integral (1: the reference) */
  int star_model;            /* 1 blackbody (T_eff parameter), 2 file, 3 grid (T_eff, log g, [M/H]) */
  char star_file[1024];      /* file path (2) or grid folder (3) */
  double* star_flux;         /* N, file stellar spectrum on the model grid */
  double* star_grid;         /* spectra x N, grid spectra on the model grid, (t, g, m) row-major */
  double* star_axis[3];
  int star_n[3];
  char xsec_path[1024], wn_file[1024];
  int discretisation; double resolution; int error_inflation;
  /* model */
  int L; double pbot, ptop;
  int temp_poly; int poly_elements, poly_order;
  int nchem; int chem_kind[8]; int chem_nsp[8]; int chem_sp[8][SP_COUNT]; int chem_bg_h2he[8]; int chem_bg_sp[8];
  int chem_na_free[8];
  int cloud; int cloud_fb;
  int cloud_kind;            /* 0 grey, 1 power_law, 2 KHnongrey */
  double cloud_ref_wl;       /* reference wavelength (um) of the non-grey clouds */
  int fit_mmw, fit_sh, var_g;
  int nopac; opac_t opac[64];
  char opac_sym[64][64], opac_folder[64][512];
  /* observations */
  int nobs; obs_t obs[64];
  /* grid */
  double* nu_full; double* wl_full; size_t nfull;
  size_t* index_list; double* nu; double* wl; size_t N;
  /* atmosphere constants */
  double* p;                 /* pressure grid [L] */
  /* piecewise polynomial (src/additional/piecewise_poly.cpp) */
  int pp_nel, pp_order, pp_ndof_el; double* pp_dof_vertices; int pp_ndof;
  double* pp_el_vert;        /* [nel][ndof_el] */
  double pp_ref[8];
  int nparam_general, nparam_chem, nparam_temp, nparam_cloud, nparam_mod, nparam_total;
  int M;                     /* total obs points */
  int finalized;
  double tau_cut;            /* tangent-ray cut-off (the reference's 10) */
} orc_model;

/* ------------------------------------------------------------------ config parsing */
static int tokenize(char* line, char** tok, int maxtok) {
  int n = 0; char* s = line;
  while (*s && n < maxtok) {
    while (*s && isspace((unsigned char)*s)) ++s;
    if (!*s) break;
    tok[n++] = s;
    while (*s && !isspace((unsigned char)*s)) ++s;
    if (*s) *s++ = 0;
  }
  return n;
}

orc_model* orc_create(const char* text) {
  orc_model* m = (orc_model*)calloc(1, sizeof(orc_model));
  m->resolution = 1.0;
  m->tau_cut = 10;
  char* buf = strdup(text);
  char* save = NULL;
  for (char* line = strtok_r(buf, "\n", &save); line; line = strtok_r(NULL, "\n", &save)) {
    char* tok[128]; int nt = tokenize(line, tok, 128);
    if (nt == 0 || tok[0][0] == '#') continue;
    const char* k = tok[0];
    if (!strcmp(k, "forward_model")) {
      if (nt < 2) goto bad;
      if (!strcmp(tok[1], "transmission")) m->transmission = 1;
      else if (!strcmp(tok[1], "secondary_eclipse") || !strcmp(tok[1], "Secondary_eclipse") || !strcmp(tok[1], "se"))
        m->occultation = 1;  /* selectForwardModel src/retrieval/select_forward_model.cpp:69 */
      else if (strcmp(tok[1], "emission")) { set_err("unsupported forward model %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "cross_section_path")) { snprintf(m->xsec_path, sizeof m->xsec_path, "%s", nt > 1 ? tok[1] : ""); }
    else if (!strcmp(k, "wavenumber_file")) { snprintf(m->wn_file, sizeof m->wn_file, "%s", nt > 1 ? tok[1] : ""); }
    else if (!strcmp(k, "spectral_discretisation")) {
      if (nt < 2) goto bad;
      if (!strcmp(tok[1], "const_wavenumber")) m->discretisation = 0;
      else if (!strcmp(tok[1], "const_wavelength")) m->discretisation = 1;
      else if (!strcmp(tok[1], "const_resolution")) m->discretisation = 2;
      else { set_err("unknown discretisation %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "spectral_resolution")) { m->resolution = atof(tok[1]); }
    else if (!strcmp(k, "error_inflation")) { m->error_inflation = atoi(tok[1]); }
    else if (!strcmp(k, "nb_grid_points")) { m->L = atoi(tok[1]); }
    else if (!strcmp(k, "atmos_boundaries")) { m->pbot = atof(tok[1]); m->ptop = atof(tok[2]); }
    else if (!strcmp(k, "temperature_profile")) {
      if (!strcmp(tok[1], "poly")) { m->temp_poly = 1; m->poly_elements = atoi(tok[2]); m->poly_order = atoi(tok[3]); }
      else if (!strcmp(tok[1], "const")) m->temp_poly = 0;
      else { set_err("unsupported temperature profile %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "stellar_spectrum")) {
      /* selectStellarModel src/forward_model/stellar_spectrum/select_stellar_model.h */
      if (nt < 2) goto bad;
      if (!strcmp(tok[1], "blackbody")) m->star_model = 1;
      else if ((!strcmp(tok[1], "file") || !strcmp(tok[1], "grid")) && nt >= 3) {
        m->star_model = !strcmp(tok[1], "file") ? 2 : 3;
        snprintf(m->star_file, sizeof m->star_file, "%s", tok[2]);
      }
      else { set_err("unsupported stellar spectrum %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "radiative_transfer")) {
      if (strcmp(tok[1], "scm")) { set_err("unsupported radiative transfer %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "chemistry")) {
      int c = m->nchem++;
      if (!strcmp(tok[1], "iso") || !strcmp(tok[1], "isoprofile")) {
        m->chem_kind[c] = 0; m->chem_nsp[c] = 0; m->chem_na_free[c] = 0;
        for (int i = 2; i < nt; ++i) {
          int id = species_id(tok[i]);
          if (id < 0) { set_err("unknown species %s", tok[i]); goto fail; }
          m->chem_sp[c][m->chem_nsp[c]++] = id;
          if (id == SP_Na) m->chem_na_free[c] = 1;
        }
      } else if (!strcmp(tok[1], "bg") || !strcmp(tok[1], "background")) {
        m->chem_kind[c] = 1; m->chem_nsp[c] = 0;
        if (!strcmp(tok[2], "H2He")) m->chem_bg_h2he[c] = 1;
        else { m->chem_bg_h2he[c] = 0; m->chem_bg_sp[c] = species_id(tok[2]); if (m->chem_bg_sp[c] < 0) { set_err("unknown bg species"); goto fail; } }
      } else { set_err("unsupported chemistry %s", tok[1]); goto fail; }
    } else if (!strcmp(k, "cloud")) {
      if (!strcmp(tok[1], "none")) continue;
      /* selectCloudModel src/cloud_model/select_cloud_model.h:42-100 */
      if (!strcmp(tok[1], "grey")) {
        m->cloud_kind = 0; m->cloud_fb = (nt >= 3 && !strcmp(tok[2], "fb"));
      } else if (!strcmp(tok[1], "power_law") || !strcmp(tok[1], "KHnongrey")) {
        /* PowerLawCloudModel / KHCloudModel ctors: reference wavelength, optional "fb" */
        if (nt < 3) { set_err("the %s cloud needs a reference wavelength", tok[1]); goto fail; }
        m->cloud_kind = !strcmp(tok[1], "power_law") ? 1 : 2;
        m->cloud_ref_wl = atof(tok[2]);
        m->cloud_fb = (nt == 4 && !strcmp(tok[3], "fb"));
      } else { set_err("unsupported cloud %s", tok[1]); goto fail; }
      m->cloud = 1;
    } else if (!strcmp(k, "opacity")) {
      int o = m->nopac++;
      snprintf(m->opac_sym[o], 64, "%s", tok[1]);
      snprintf(m->opac_folder[o], 512, "%s", nt > 2 ? tok[2] : "");
    } else if (!strcmp(k, "fit_mean_molecular_weight")) m->fit_mmw = atoi(tok[1]);
    else if (!strcmp(k, "fit_scale_height")) m->fit_sh = atoi(tok[1]);
    else if (!strcmp(k, "variable_gravity")) m->var_g = atoi(tok[1]);
    else if (!strcmp(k, "transmission_annuli")) m->annuli = atoi(tok[1]);
    continue;
  bad:
    set_err("malformed config line for %s", k); goto fail;
  }
  free(buf);
  if (m->fit_sh) { set_err("fit_scale_height is not supported"); free(m); return NULL; }
  if (m->L < 2 || m->L > 512) { set_err("nb_grid_points must be in [2, 512]"); free(m); return NULL; }
  return m;
fail:
  free(buf); free(m); return NULL;
}

/* ------------------------------------------------------------------ observations
 * Observation::init(ObservationInput) src/observations/observations.cpp:42-111 */
static void reverse_d(double* a, int n) { for (int i = 0; i < n / 2; ++i) { double t = a[i]; a[i] = a[n - 1 - i]; a[n - 1 - i] = t; } }

int orc_add_observation(orc_model* m, const char* name, const char* type, int n,
                        const double* ce, const double* data, const double* error,
                        const double* weight, const double* fwhm, int nfilter,
                        const double* fwl, const double* fresp, const char* detector,
                        const char* modifier) {
  (void)name;
  obs_t* o = &m->obs[m->nobs++];
  memset(o, 0, sizeof *o);
  /* setSpectrumModifier src/observations/observations.cpp:374-392 */
  if (!modifier || !modifier[0] || !strcmp(modifier, "none")) o->nb_modifier = 0;
  else if (!strcmp(modifier, "shift_const")) o->nb_modifier = 1;
  else { set_err("unknown modifier %s", modifier); return -1; }
  if (!strcmp(type, "spectroscopy") || !strcmp(type, "Spectroscopy")) o->type = BAND_SPEC;
  else if (!strcmp(type, "photometry") || !strcmp(type, "Photometry")) o->type = BAND_PHOT;
  else if (!strcmp(type, "band-spectroscopy") || !strcmp(type, "Band-spectroscopy")) o->type = BAND_BANDSPEC;
  else { set_err("unsupported band type %s", type); return -1; }
  o->n = n;
  o->data = (double*)malloc(n * sizeof(double)); memcpy(o->data, data, n * sizeof(double));
  o->error = (double*)malloc(n * sizeof(double)); memcpy(o->error, error, n * sizeof(double));
  o->weight = (double*)malloc(n * sizeof(double));
  for (int i = 0; i < n; ++i) o->weight[i] = weight ? weight[i] : 1.0;
  o->nfwhm = fwhm ? n : 0;
  o->fwhm = (double*)malloc((n ? n : 1) * sizeof(double));
  if (fwhm) memcpy(o->fwhm, fwhm, n * sizeof(double));
  if (nfilter > 0) {
    o->nfilter = nfilter;
    o->filter_wl = (double*)malloc(nfilter * sizeof(double)); memcpy(o->filter_wl, fwl, nfilter * sizeof(double));
    o->filter_resp = (double*)malloc(nfilter * sizeof(double)); memcpy(o->filter_resp, fresp, nfilter * sizeof(double));
    if (!strcmp(detector, "energy") || !strcmp(detector, "Energy")) o->photon = 0;
    else if (!strcmp(detector, "photon") || !strcmp(detector, "Photon")) o->photon = 1;
    else { set_err("unsupported detector type %s", detector); return -1; }
    if (o->filter_wl[0] < o->filter_wl[nfilter - 1]) { reverse_d(o->filter_wl, nfilter); reverse_d(o->filter_resp, nfilter); }
  }
  o->edges = (double(*)[2])malloc((n ? n : 1) * sizeof(double[2]));
  o->centers = (double*)malloc((n ? n : 1) * sizeof(double));
  if (o->type == BAND_SPEC) {
    double* wl = (double*)malloc(n * sizeof(double)); memcpy(wl, ce, n * sizeof(double));
    /* areWavelengthsAscending(vector<double>) :127-151 */
    o->ascending = 0;
    if (n > 1) {
      if (wl[0] < wl[1]) {
        o->ascending = 1;
        reverse_d(wl, n); reverse_d(o->data, n); reverse_d(o->error, n);
        if (o->nfwhm) reverse_d(o->fwhm, o->nfwhm);
        reverse_d(o->weight, n);
      }
    }
    memcpy(o->centers, wl, n * sizeof(double));
    /* calcBinEdges :188-221 */
    for (int i = 0; i < n; ++i) {
      if (i == 0) {
        o->edges[0][1] = wl[0] - (wl[i] - wl[i + 1]) * 0.5;
        o->edges[0][0] = wl[0] + (wl[i] - wl[i + 1]) * 0.5;
      } else if (i == n - 1) {
        o->edges[n - 1][1] = wl[i] - (wl[i - 1] - wl[i]) * 0.5;
        o->edges[n - 1][0] = wl[i] + (wl[i - 1] - wl[i]) * 0.5;
      } else {
        o->edges[i][0] = wl[i - 1] - (wl[i - 1] - wl[i]) * 0.5;
        o->edges[i][1] = wl[i] - (wl[i] - wl[i + 1]) * 0.5;
      }
    }
    free(wl);
  } else {
    for (int i = 0; i < n; ++i) { o->edges[i][0] = ce[2 * i]; o->edges[i][1] = ce[2 * i + 1]; }
    /* areWavelengthsAscending(vector<vector<double>>) :156-184 */
    o->ascending = 0;
    if (n > 1 && o->edges[0][0] < o->edges[n - 1][0]) {
      o->ascending = 1;
      for (int i = 0; i < n / 2; ++i) {
        double a0 = o->edges[i][0], a1 = o->edges[i][1];
        o->edges[i][0] = o->edges[n - 1 - i][0]; o->edges[i][1] = o->edges[n - 1 - i][1];
        o->edges[n - 1 - i][0] = a0; o->edges[n - 1 - i][1] = a1;
      }
      reverse_d(o->data, n); reverse_d(o->error, n);
      if (o->nfwhm) reverse_d(o->fwhm, o->nfwhm);
      reverse_d(o->weight, n);
    }
    for (int i = 0; i < n; ++i)
      if (o->edges[i][0] < o->edges[i][1]) { double t = o->edges[i][0]; o->edges[i][0] = o->edges[i][1]; o->edges[i][1] = t; }
    /* calcBinCenters :224-233 */
    for (int i = 0; i < n; ++i) o->centers[i] = o->edges[i][0] - (o->edges[i][0] - o->edges[i][1]) * 0.5;
  }
  /* setObservationEdges :237-251 */
  if (o->nfwhm) {
    o->wl_edges[0] = o->edges[0][0] + 5.0 * o->fwhm[0] / 2.355;
    o->wl_edges[1] = o->edges[n - 1][1] - 5.0 * o->fwhm[o->nfwhm - 1] / 2.355;
  } else {
    o->wl_edges[0] = o->edges[0][0];
    o->wl_edges[1] = o->edges[n - 1][1];
  }
  /* SpectralBands::init :38-63 (wavelengthToWavenumber = 1.0/x * 1e4) */
  o->edge_nu = (double(*)[2])malloc((n ? n : 1) * sizeof(double[2]));
  for (int i = 0; i < n; ++i) { o->edge_nu[i][0] = 1.0 / o->edges[i][0] * 1e4; o->edge_nu[i][1] = 1.0 / o->edges[i][1] * 1e4; }
  o->obs_nu_range[0] = 1.0 / o->wl_edges[0] * 1e4;
  o->obs_nu_range[1] = 1.0 / o->wl_edges[1] * 1e4;
  return 0;
}

/* ------------------------------------------------------------------ spectral grid
 * src/spectral_grid/spectral_grid.cpp */
static size_t lower_bound_asc(const double* a, size_t lo, size_t hi, double x) {
  while (lo < hi) { size_t mid = lo + (hi - lo) / 2; if (a[mid] < x) lo = mid + 1; else hi = mid; }
  return lo;
}
static size_t lower_bound_desc(const double* a, size_t lo, size_t hi, double x) {
  /* std::lower_bound with std::greater: first element e with !(e > x) */
  while (lo < hi) { size_t mid = lo + (hi - lo) / 2; if (a[mid] > x) lo = mid + 1; else hi = mid; }
  return lo;
}
/* findClosestIndex{,Asc,Desc} :323-385. When the search runs past the end the
 * reference reads one element beyond the vector; the last index is returned here. */
static size_t find_closest(double x, const double* data, size_t n, size_t start) {
  size_t it;
  if (n < 2) return 0;
  if (data[0] < data[1]) it = lower_bound_asc(data, start, n, x);
  else if (data[0] > data[1]) it = lower_bound_desc(data, start, n, x);
  else return 0;
  if (it == start) return start;
  if (it == n) return n - 1;
  if (fabs(x - data[it - 1]) < fabs(x - data[it])) return it - 1;
  return it;
}

static int load_wavenumbers(orc_model* m) {
  /* loadWavenumberList :87-119, createHeliosWavenumberList :75-84 */
  FILE* f = fopen(m->wn_file, "r");
  if (!f) {
    m->nfull = (size_t)(90000.0 / 0.01 + 1);
    m->nu_full = (double*)malloc(m->nfull * sizeof(double));
    for (size_t i = 0; i < m->nfull; ++i) m->nu_full[i] = i * 0.01;
  } else {
    unsigned long long n = 0;
    if (fscanf(f, "%llu", &n) != 1) { fclose(f); set_err("bad wavenumber file"); return -1; }
    m->nfull = n;
    m->nu_full = (double*)malloc(n * sizeof(double));
    for (size_t i = 0; i < n; ++i) if (fscanf(f, "%lf", &m->nu_full[i]) != 1) { fclose(f); set_err("short wavenumber file"); return -1; }
    fclose(f);
  }
  m->wl_full = (double*)malloc(m->nfull * sizeof(double));
  for (size_t i = 0; i < m->nfull; ++i) m->wl_full[i] = 1.0 / m->nu_full[i] * 1e4;
  return 0;
}

typedef struct { double a, b; } pair_d;

static int sample_grid(orc_model* m) {
  /* sampleSpectralGrid :123-157 */
  int no = m->nobs;
  pair_d* e = (pair_d*)malloc(no * sizeof(pair_d));
  for (int i = 0; i < no; ++i) { e[i].a = 1.0 / m->obs[i].wl_edges[0] * 1e4; e[i].b = 1.0 / m->obs[i].wl_edges[1] * 1e4; }
  /* std::sort by a; ties keep an unspecified order in the reference; use a stable insertion sort */
  for (int i = 1; i < no; ++i) { pair_d t = e[i]; int j = i - 1; while (j >= 0 && e[j].a > t.a) { e[j + 1] = e[j]; --j; } e[j + 1] = t; }
  pair_d* we = (pair_d*)malloc(no * sizeof(pair_d)); int nw = 1; we[0] = e[0];
  for (int i = 1; i < no; ++i) {
    if (e[i].a > we[nw - 1].a && e[i].b < we[nw - 1].b) continue;
    if (e[i].a < we[nw - 1].b && e[i].b > we[nw - 1].b) we[nw - 1].b = e[i].b;
    else we[nw++] = e[i];
  }
  /* findBinEdges :390-416 */
  size_t (*ei)[2] = (size_t(*)[2])malloc(nw * sizeof(size_t[2]));
  for (int i = 0; i < nw; ++i) {
    size_t l = lower_bound_asc(m->nu_full, 0, m->nfull, we[i].a);
    size_t r = lower_bound_asc(m->nu_full, 0, m->nfull, we[i].b);
    ei[i][0] = l;
    if (m->nu_full[ei[i][0]] > we[i].a) ei[i][0] -= 1;
    ei[i][1] = r;
  }
  /* createHighResGrid :239-304 */
  int* inc = (int*)calloc(m->nfull, sizeof(int));
  for (int i = 0; i < nw; ++i) {
    inc[ei[i][0]] = 1;
    size_t last = ei[i][0];
    for (size_t j = ei[i][0]; j < ei[i][1]; ++j) {
      if (m->discretisation == 0) {        /* :161-184 */
        const double next = m->nu_full[last] + m->resolution;
        if (next == m->nu_full[j] || m->nu_full[j + 1] > next) { inc[j] = 1; last = j; }
      } else if (m->discretisation == 1) { /* :187-210 */
        const double next = m->wl_full[last] - m->resolution;
        if (next == m->wl_full[j] || m->wl_full[j + 1] < next) { inc[j] = 1; last = j; }
      } else {                             /* :213-236 */
        const double next = m->wl_full[last] * (1 - 1. / m->resolution);
        if (next == m->wl_full[j] || m->wl_full[j + 1] < next) { inc[j] = 1; last = j; }
      }
      inc[ei[i][1]] = 1;
    }
  }
  for (int k = 0; k < no; ++k) {
    obs_t* o = &m->obs[k];
    size_t start = 0; double last_nu = 0;
    for (int b = 0; b < o->n; ++b) {
      if (last_nu > o->edge_nu[b][0]) start = 0;
      size_t i1 = find_closest(o->edge_nu[b][0], m->nu_full, m->nfull, start);
      size_t i2 = find_closest(o->edge_nu[b][1], m->nu_full, m->nfull, start);
      inc[i1] = 1; inc[i2] = 1;
      last_nu = o->edge_nu[b][1];
      start = i2;
    }
  }
  m->N = 0;
  for (size_t i = 0; i < m->nfull; ++i) m->N += inc[i] == 1;
  m->index_list = (size_t*)malloc(m->N * sizeof(size_t));
  m->nu = (double*)malloc(m->N * sizeof(double));
  m->wl = (double*)malloc(m->N * sizeof(double));
  size_t c = 0;
  for (size_t i = 0; i < m->nfull; ++i)
    if (inc[i] == 1) { m->index_list[c] = i; m->nu[c] = m->nu_full[i]; m->wl[c] = m->wl_full[i]; ++c; }
  free(inc); free(ei); free(we); free(e);

  /* SpectralBands::setBandEdgeIndices src/spectral_grid/spectral_band.cpp:80-121, init :66-76 */
  for (int k = 0; k < no; ++k) {
    obs_t* o = &m->obs[k];
    o->edge_idx = (size_t(*)[2])malloc((o->n ? o->n : 1) * sizeof(size_t[2]));
    size_t start = 0; double last_nu = 0;
    for (int b = 0; b < o->n; ++b) {
      if (last_nu > o->edge_nu[b][0]) start = 0;
      size_t i1 = find_closest(o->edge_nu[b][0], m->nu, m->N, start);
      size_t i2 = find_closest(o->edge_nu[b][1], m->nu, m->N, start);
      if (i1 > m->N - 1 || i2 > m->N - 1) { set_err("Edge wavenumber index not found"); return -1; }
      if (i1 == i2) { set_err("The spectral resolution of the opacity grid is too small"); return -1; }
      o->edge_idx[b][0] = i1; o->edge_idx[b][1] = i2;
      last_nu = o->edge_nu[b][1];
      start = i2;
    }
    o->range_lo = find_closest(o->obs_nu_range[0], m->nu, m->N, 0);
    o->range_hi = find_closest(o->obs_nu_range[1], m->nu, m->N, 0);
  }
  return 0;
}

/* SpectralGrid::interpolateToWavelengthGrid(x, y, new_x, log)
 * src/spectral_grid/spectral_grid_interpolate.cpp:110-172 (log = false) */
static void interp_to_wavelengths(const double* dx, const double* dy, int nd, const double* newx,
                                  size_t nn, double* out) {
  double* x = (double*)malloc(nd * sizeof(double)); double* y = (double*)malloc(nd * sizeof(double));
  memcpy(x, dx, nd * sizeof(double)); memcpy(y, dy, nd * sizeof(double));
  if (x[0] < x[1]) { reverse_d(x, nd); reverse_d(y, nd); }
  for (size_t i = 0; i < nn; ++i) out[i] = 0.0;
  size_t x_start = 0;
  for (size_t i = 0; i < nn; ++i) {
    if (newx[i] > x[0]) continue;
    if (newx[i] < x[nd - 1]) break;
    size_t it = x_start;
    while (it < (size_t)nd && !(x[it] <= newx[i])) ++it;
    size_t index = it;
    if (x[it] == newx[i]) out[i] = y[index];
    else out[i] = y[index - 1] + (y[index] - y[index - 1]) * (newx[i] - x[it - 1]) / (x[it] - x[it - 1]);
    if (x_start > 0) x_start = index - 1;
  }
  free(x); free(y);
}

static void setup_observation_operators(orc_model* m) {
  for (int k = 0; k < m->nobs; ++k) {
    obs_t* o = &m->obs[k];
    /* setInstrumentProfileFWHW src/spectral_grid/spectral_band.cpp:127-154 */
    o->has_profile = 0;
    if (o->nfwhm && o->nfwhm == o->n) {
      size_t nhr = o->range_hi - o->range_lo + 1;
      double* prof = (double*)malloc(nhr * sizeof(double));
      interp_to_wavelengths(o->centers, o->fwhm, o->n, m->wl + o->range_lo, nhr, prof);
      o->sigma = (double*)calloc(m->N, sizeof(double));
      for (size_t i = 0; i < nhr; ++i) o->sigma[i + o->range_lo] = prof[i] / 2.355;
      free(prof);
      /* setConvolutionQuadratureIntervals src/spectral_grid/spectral_band_convolve.cpp:44-95 */
      o->conv = (size_t(*)[2])malloc(nhr * sizeof(size_t[2]));
      for (size_t i = 0; i < nhr; ++i) {
        size_t idx = i + o->range_lo;
        o->conv[i][0] = o->range_lo; o->conv[i][1] = o->range_hi;
        const double cut = 5.0 * o->sigma[idx];
        if (cut == 0) { o->conv[i][0] = idx; o->conv[i][1] = idx; }
        else {
          o->conv[i][0] = find_closest(m->wl[idx] + cut, m->wl, m->N, 0);
          o->conv[i][1] = find_closest(m->wl[idx] - cut, m->wl, m->N, o->conv[i][0]);
        }
      }
      o->has_profile = 1;
    }
    /* setFilterResponseFunction src/observations/observations_filter_response.cpp:122-143,
     * the whole-grid interpolateToWavelengthGrid(x, y, log) :60-106 */
    if (o->nfilter) {
      o->filter_on_grid = (double*)malloc(m->N * sizeof(double));
      interp_to_wavelengths(o->filter_wl, o->filter_resp, o->nfilter, m->wl, m->N, o->filter_on_grid);
      o->filter_weight = (double*)malloc(m->N * sizeof(double));
      for (size_t i = 0; i < m->N; ++i) o->filter_weight[i] = o->photon ? m->wl[i] : 1.0;
      /* filterResponseNormalisation :147-160 */
      double* y = (double*)malloc(o->nfilter * sizeof(double));
      for (int i = 0; i < o->nfilter; ++i) y[i] = o->photon ? o->filter_resp[i] * o->filter_wl[i] : o->filter_resp[i];
      double s = 0;
      if (o->nfilter == 1) s = y[0] / 0.5;
      else for (int i = 1; i < o->nfilter; ++i) s += (o->filter_wl[i] - o->filter_wl[i - 1]) * (y[i] + y[i - 1]);
      s *= 0.5;
      if (s < 0) s = fabs(s);
      o->filter_norm = s;
      free(y);
    }
  }
}

/* ------------------------------------------------------------------ opacity tables */
static int load_rows(orc_model* m, opac_t* op, const char* folder) {
  /* readFileList src/transport_coeff/opacity_species.cpp:66-122, orderDataList :129-156 */
  char path[2048];
  snprintf(path, sizeof path, "%s%s/filelist.dat", m->xsec_path, folder);
  FILE* f = fopen(path, "r");
  if (!f) { set_err("No line absorption data: %s", path); return -1; }
  char line[4096];
  if (!fgets(line, sizeof line, f)) { fclose(f); set_err("empty filelist %s", path); return -1; }
  char stor[64] = "";
  op->mass = 0; sscanf(line, "%lf %63s", &op->mass, stor);
  int logst = !strcmp(stor, "log");
  int cap = 256, cnt = 0;
  double* Ps = (double*)malloc(cap * sizeof(double)); double* Ts = (double*)malloc(cap * sizeof(double));
  char** names = (char**)malloc(cap * sizeof(char*));
  while (fgets(line, sizeof line, f)) {
    double pp, tt; char nm[1024];
    if (sscanf(line, "%lf %lf %1023s", &pp, &tt, nm) != 3) continue;
    if (cnt == cap) { cap *= 2; Ps = (double*)realloc(Ps, cap * sizeof(double)); Ts = (double*)realloc(Ts, cap * sizeof(double)); names = (char**)realloc(names, cap * sizeof(char*)); }
    Ps[cnt] = pp; Ts[cnt] = tt; names[cnt] = strdup(nm); ++cnt;
  }
  fclose(f);
  /* distinct temperatures, ascending */
  double* tl = (double*)malloc(cnt * sizeof(double)); int nT = 0;
  for (int i = 0; i < cnt; ++i) { int found = 0; for (int j = 0; j < nT; ++j) if (tl[j] == Ts[i]) found = 1; if (!found) tl[nT++] = Ts[i]; }
  for (int i = 1; i < nT; ++i) { double t = tl[i]; int j = i - 1; while (j >= 0 && tl[j] > t) { tl[j + 1] = tl[j]; --j; } tl[j + 1] = t; }
  op->nT = nT; op->T = tl;
  op->nP = (int*)calloc(nT, sizeof(int)); op->P = (double**)calloc(nT, sizeof(double*));
  op->logP = (double**)calloc(nT, sizeof(double*)); op->rows = (double***)calloc(nT, sizeof(double**));
  float* buf = NULL; size_t bufn = 0;
  for (int t = 0; t < nT; ++t) {
    int np = 0; for (int i = 0; i < cnt; ++i) if (Ts[i] == tl[t]) ++np;
    int* idx = (int*)malloc(np * sizeof(int)); np = 0;
    for (int i = 0; i < cnt; ++i) if (Ts[i] == tl[t]) idx[np++] = i;
    for (int i = 1; i < np; ++i) { int x = idx[i]; int j = i - 1; while (j >= 0 && Ps[idx[j]] > Ps[x]) { idx[j + 1] = idx[j]; --j; } idx[j + 1] = x; }
    op->nP[t] = np; op->P[t] = (double*)malloc(np * sizeof(double)); op->logP[t] = (double*)malloc(np * sizeof(double));
    op->rows[t] = (double**)malloc(np * sizeof(double*));
    for (int q = 0; q < np; ++q) {
      int i = idx[q];
      op->P[t][q] = Ps[i]; op->logP[t][q] = log10(Ps[i]);
      /* CrossSectionFile::loadFile src/transport_coeff/cross_section_file.cpp:33-68 and
       * SampledData::sampleCrossSections src/transport_coeff/sampled_data.cpp:48-87 */
      snprintf(path, sizeof path, "%s%s/%s", m->xsec_path, folder, names[i]);
      FILE* df = fopen(path, "rb");
      if (!df) { set_err("cross section file %s not found", path); return -1; }
      fseek(df, 0, SEEK_END); long bytes = ftell(df); fseek(df, 0, SEEK_SET);
      size_t nd = (size_t)(bytes / (long)sizeof(float));
      if (nd > bufn) { buf = (float*)realloc(buf, nd * sizeof(float)); bufn = nd; }
      if (fread(buf, sizeof(float), nd, df) != nd) { fclose(df); set_err("short read %s", path); return -1; }
      fclose(df);
      double* r = (double*)malloc(m->N * sizeof(double));
      /* points past the end of the file keep 0 (then the 1e-200 floor) */
      size_t kend = 0;
      while (kend < m->N && m->index_list[kend] <= nd - 1) ++kend;
      const long long nk = (long long)m->N;
#pragma omp parallel for schedule(static)
      for (long long k = 0; k < nk; ++k) {
        double v = 0.0;
        if ((size_t)k < kend) {
          v = buf[m->index_list[k]];
          if (logst) v = pow(10.0, v);
        }
        if (op->mass > 0) v *= op->mass / 6.022140857e23;
        if (v < 1e-200) v = 1e-200;
        r[k] = log10(v);
      }
      op->rows[t][q] = r;
    }
    free(idx);
  }
  free(buf);
  for (int i = 0; i < cnt; ++i) free(names[i]);
  free(names); free(Ps); free(Ts);
  return 0;
}

/* Rayleigh cross sections, src/transport_coeff/species_rayleigh_cross_sections.cpp:25-234 and
 * generalRayleighCrossSection src/transport_coeff/opacity_species.cpp:528-537 */
static double rayleigh_general(double nref, double n, double king, double nu) {
  return 24. * pow(K_PI, 3) * pow(nu, 4) / (nref * nref) * pow((n * n - 1) / (n * n + 2), 2) * king;
}
static int tabulate_rayleigh(orc_model* m, opac_t* op, int sp) {
  op->rayleigh = (double*)malloc(m->N * sizeof(double));
  for (size_t j = 0; j < m->N; ++j) {
    const double nu = m->nu[j], wl = m->wl[j];
    double king = 1.0, n = 1.0, nref = 1.0;
    if (sp == SP_H2) {
      n = (13.58e-5 * (1. + 7.52e-3 / pow(wl, 2))) + 1.;
      nref = 2.651629e19;
    } else if (sp == SP_He) {
      n = (2283. + 1.8102e13 / (1.5342e10 - nu * nu)) * 1e-8 + 1;
      nref = 2.546899e19;
    } else if (sp == SP_H) {
      /* GasHRayleigh: Lee & Kim 2002 low-energy expansion */
      const double f = 0.0912 / wl;
      op->rayleigh[j] = 8.41e-25 * pow(f, 4) + 3.37e-24 * pow(f, 6) + 4.71e-22 * pow(f, 14);
      continue;
    } else if (sp == SP_CO || sp == SP_CO2 || sp == SP_CH4 || sp == SP_H2O) {
      op->rayleigh[j] = 0.0;
      if (wl > 2.0) continue;  /* these are zero beyond 2 micron */
      const double nu2 = nu * nu;
      nref = 2.546899e19;
      if (sp == SP_CO) {
        n = (22851. + 0.456e14 / (71427.0 * 71427.0 - nu2)) * 1e-8 + 1;
      } else if (sp == SP_CO2) {
        king = 1.1364 + 25.3e-12 * nu2;
        n = (5799.25 / (128908.9 * 128908.9 - nu2) + 120.05 / (89223.8 * 89223.8 - nu2)
             + 5.3334 / (75037.5 * 75037.5 - nu2) + 4.3244 / (67837.7 * 67837.7 - nu2)
             + 0.1218145e-6 / (2418.136 * 2418.136 - nu2)) * 1.1427e3 + 1.0;
      } else if (sp == SP_CH4) {
        n = (46662. + 4.02e-6 * nu2) * 1e-8 + 1;
      } else {
        /* GasH2ORayleigh: water at STP (delta = theta = 1) */
        static const double a[8] = {0.244257733, 0.974634476e-2, -0.373234996e-2, 0.268678472e-3,
                                    0.158920570e-2, 0.245934259e-2, 0.900704920, -0.166626219e-1};
        const double delta = 1.0, theta = 1.0, luv = 0.229202, lir = 5.432937;
        nref = 3.34279671749673e+22;
        king = (6 + 3 * 3e-4) / (6 - 7 * 3e-4);
        const double lam = wl / 0.589;
        const double af = delta * (a[0] + a[1] * delta + a[2] * theta + a[3] * lam * lam * theta
                                   + a[4] * pow(lam, -2) + a[5] / (lam * lam - luv * luv)
                                   + a[6] / (lam * lam - lir * lir) + a[7] * delta * delta);
        n = pow(((2 * af + 1) / (1 - af)), 0.5);
      }
    } else {
      set_err("Rayleigh scattering for this species is not restated in the oracle");
      return -1;
    }
    op->rayleigh[j] = rayleigh_general(nref, n, king, nu);
  }
  return 0;
}

/* GasHm src/transport_coeff/h_m.cpp:36-137: the wavelength-dependent parts of the H-
 * bound-free cross section (photo-detachment threshold 1.6419 um, valid above 0.125 um)
 * and of the free-free polynomials (two coefficient sets, above 0.3645 um and from
 * 0.1823 to 0.3645 um); the temperature factors are applied per level. */
static void tabulate_hm(orc_model* m, opac_t* op) {
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
  const size_t N = m->N;
  op->hm_bf = (double*)calloc(N, sizeof(double));
  for (int i = 1; i < 7; ++i) op->hm_ff[i] = (double*)calloc(N, sizeof(double));
  for (size_t k = 0; k < N; ++k) {
    const double l = m->wl[k];
    if (l <= lambda_0 && l >= 0.125) {
      double f = 0;
      for (int i = 1; i < 7; ++i) f += Cn[i] * pow((1.0 / l - 1.0 / lambda_0), (i - 1) / 2.0);
      op->hm_bf[k] = 1e-18 * l * l * l * pow(1.0 / l - 1.0 / lambda_0, 1.5) * f;
    }
    const double *A = NULL, *B = NULL, *C = NULL, *D = NULL, *E = NULL, *F = NULL;
    if (l > 0.3645) { A = A1; B = B1; C = C1; D = D1; E = E1; F = F1; }
    else if (l >= 0.1823) { A = A2; B = B2; C = C2; D = D2; E = E2; F = F2; }
    if (A)
      for (int i = 1; i < 7; ++i)
        op->hm_ff[i][k] = l * l * A[i] + B[i] + C[i] / l + D[i] / l / l + E[i] / l / l / l + F[i] / l / l / l / l;
  }
}

static int setup_opacity(orc_model* m) {
  /* TransportCoefficients::addOpacitySpecies src/transport_coeff/transport_coeff.cpp:98-237 */
  for (int i = 0; i < m->nopac; ++i) {
    opac_t* op = &m->opac[i];
    const char* s = m->opac_sym[i]; const char* fo = m->opac_folder[i];
    op->npartner = 0;
    if (!strcmp(s, "CIA-H2-H2")) { op->kind = 0; op->index = SP_H2; op->partner[op->npartner++] = SP_H2; }
    else if (!strcmp(s, "CIA-H2-He")) { op->kind = 0; op->index = SP_H2; op->partner[op->npartner++] = SP_He; }
    else if (!strcmp(s, "CIA-H-He")) { op->kind = 0; op->index = SP_H; op->partner[op->npartner++] = SP_He; }
    else if (!strcmp(s, "H-")) { op->kind = 2; op->index = SP_Hm; tabulate_hm(m, op); continue; }
    else if (!strcmp(fo, "Rayleigh")) {
      int sp = species_id(s);
      if (sp < 0) { set_err("unknown Rayleigh species %s", s); return -1; }
      op->kind = 1; op->index = sp;
      if (tabulate_rayleigh(m, op, sp)) return -1;
      continue;
    } else {
      int sp = species_id(s);
      if (sp < 0) { set_err("Opacity species %s not found", s); return -1; }
      op->kind = 0; op->index = sp;
    }
    if (load_rows(m, op, fo)) return -1;
  }
  return 0;
}

/* ------------------------------------------------------------------ atmosphere setup */
static void setup_atmosphere(orc_model* m) {
  /* Atmosphere::createPressureGrid src/forward_model/atmosphere/atmosphere.cpp:365-383 */
  int L = m->L;
  m->p = (double*)calloc(L, sizeof(double));
  const double minp = m->ptop, maxp = m->pbot;
  m->p[0] = log10(maxp);
  const double step = (log10(maxp) - log10(minp)) / (L - 1.0);
  for (int i = 1; i < L - 1; ++i) m->p[i] = m->p[i - 1] - step;
  for (int i = 0; i < L - 1; ++i) m->p[i] = pow(10.0, m->p[i]);
  m->p[L - 1] = minp;
  if (m->temp_poly) {
    /* PiecewisePolynomial ctor / createElementGrid src/additional/piecewise_poly.cpp:49-121 */
    static const double gl1[] = {-1.0, 1.0}, gl2[] = {-1.0, 0.0, 1.0},
                        gl3[] = {-1.0, -0.447214, 0.447214, 1.0}, gl4[] = {-1.0, -0.654654, 0.654654, 1.0},
                        gl5[] = {-1.0, -0.654654, 0.0, 0.654654, 1.0},
                        gl6[] = {-1.0, -7.65055 - 0.285232, 0.285232, 0.765055, 1.0};
    static const double* nodes[] = {NULL, gl1, gl2, gl3, gl4, gl5, gl6};
    static const int nn[] = {1, 2, 3, 4, 4, 5, 5};
    int order = m->poly_order < 1 ? 1 : (m->poly_order > 6 ? 6 : m->poly_order);
    int nel = m->poly_elements < 1 ? 1 : m->poly_elements;
    m->pp_nel = nel; m->pp_order = order; m->pp_ndof_el = nn[order];
    for (int i = 0; i < nn[order]; ++i) m->pp_ref[i] = nodes[order][i];
    double lb0 = log10(m->pbot), lb1 = log10(m->ptop);
    double size = (lb0 - lb1) / nel;
    double* edges = (double*)malloc((nel + 1) * sizeof(double));
    edges[0] = lb0; edges[nel] = lb1;
    for (int i = 1; i < nel; ++i) edges[i] = edges[i - 1] - size;
    m->pp_el_vert = (double*)malloc(nel * nn[order] * sizeof(double));
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < nn[order]; ++i)
        m->pp_el_vert[e * nn[order] + i] = edges[e] + (1.0 + m->pp_ref[i]) / 2.0 * (edges[e + 1] - edges[e]);
    m->pp_ndof = nel * (nn[order] - 1) + 1;
    m->pp_dof_vertices = (double*)malloc(m->pp_ndof * sizeof(double));
    int c = 0;
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < nn[order] - 1; ++i) m->pp_dof_vertices[c++] = m->pp_el_vert[e * nn[order] + i];
    m->pp_dof_vertices[c++] = m->pp_el_vert[(nel - 1) * nn[order] + nn[order] - 1];
    free(edges);
    m->nparam_temp = nel * order + 1;
  } else {
    m->nparam_temp = 1;
  }
}

/* StarSpectrumFile src/forward_model/stellar_spectrum/star_file_spectrum.cpp:40-120:
 * "wavelength(um) flux(W m-2 um-1)" lines, flux * wl^2 / 1e4, interpolated to the grid */
static int load_star_file(orc_model* m) {
  FILE* f = fopen(m->star_file, "r");
  if (!f) { set_err("stellar spectrum file %s not found", m->star_file); return -1; }
  size_t cap = 1024, n = 0;
  double* x = (double*)malloc(cap * sizeof(double));
  double* y = (double*)malloc(cap * sizeof(double));
  char line[512];
  while (fgets(line, sizeof line, f)) {
    double a, b;
    if (sscanf(line, "%lf %lf", &a, &b) != 2) continue;
    if (n == cap) { cap *= 2; x = (double*)realloc(x, cap * sizeof(double)); y = (double*)realloc(y, cap * sizeof(double)); }
    x[n] = a; y[n] = b * a * a / 10000.; ++n;
  }
  fclose(f);
  if (n < 2) { free(x); free(y); set_err("stellar spectrum file %s has fewer than two points", m->star_file); return -1; }
  m->star_flux = (double*)calloc(m->N, sizeof(double));
  interp_to_wavelengths(x, y, (int)n, m->wl, m->N, m->star_flux);
  free(x); free(y);
  return 0;
}

static float* read_float_file(const char* path, size_t* n) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  *n = (size_t)bytes / sizeof(float);
  float* v = (float*)malloc((*n ? *n : 1) * sizeof(float));
  if (fread(v, sizeof(float), *n, f) != *n) { free(v); fclose(f); return NULL; }
  fclose(f);
  return v;
}

/* StellarSpectrumGrid src/forward_model/stellar_spectrum/stellar_spectrum_grid.cpp:42-210 and
 * SampledStellarSpectrum::sampleSpectrum sampled_stellar_spectrum.cpp:47-80: every grid
 * spectrum (float32, W m-2 um-1 on the grid's float32 wavelengths) x wl^2 / 1e4, interpolated
 * to the model grid, values below 1e-37 raised to 1e-37. A folder without a trailing '/' gets
 * a '+' appended, as in the reference. */
static int load_star_grid(orc_model* m) {
  char folder[1100], path[2200], line[4096];
  snprintf(folder, sizeof folder, "%s%s", m->star_file,
           (m->star_file[0] && m->star_file[strlen(m->star_file) - 1] == '/') ? "" : "+");
  snprintf(path, sizeof path, "%sgrid_parameters.dat", folder);
  FILE* f = fopen(path, "r");
  if (!f) { set_err("stellar grid parameter file %s not found", path); return -1; }
  for (int a = 0; a < 3; ++a) {
    if (!fgets(line, sizeof line, f)) { fclose(f); set_err("stellar grid %s truncated", path); return -1; }
    m->star_axis[a] = (double*)malloc(256 * sizeof(double));
    int n = 0, used = 0; double v; char* c = line;
    while (n < 256 && sscanf(c, "%lf%n", &v, &used) == 1) { m->star_axis[a][n++] = v; c += used; }
    m->star_n[a] = n;
  }
  char wlname[1024];
  if (fscanf(f, "%1023s", wlname) != 1) { fclose(f); set_err("stellar grid %s truncated", path); return -1; }
  if (!fgets(line, sizeof line, f)) line[0] = 0;
  const int n0 = m->star_n[0], n1 = m->star_n[1], n2 = m->star_n[2];
  snprintf(path, sizeof path, "%s%s", folder, wlname);
  size_t nwl = 0;
  float* wlf = read_float_file(path, &nwl);
  if (!wlf) { fclose(f); set_err("stellar grid wavelength file %s not found", path); return -1; }
  double* gwl = (double*)malloc(nwl * sizeof(double));
  double* y = (double*)malloc(nwl * sizeof(double));
  for (size_t i = 0; i < nwl; ++i) gwl[i] = wlf[i];
  m->star_grid = (double*)calloc((size_t)n0 * n1 * n2 * m->N, sizeof(double));
  int count = 0;
  while (fgets(line, sizeof line, f)) {
    double t, g, q; char name[1024];
    if (sscanf(line, "%lf %lf %lf %1023s", &t, &g, &q, name) != 4) continue;
    int it = -1, ig = -1, iq = -1;
    for (int i = 0; i < n0; ++i) if (m->star_axis[0][i] == t) it = i;
    for (int i = 0; i < n1; ++i) if (m->star_axis[1][i] == g) ig = i;
    for (int i = 0; i < n2; ++i) if (m->star_axis[2][i] == q) iq = i;
    if (it < 0 || ig < 0 || iq < 0) { fclose(f); set_err("stellar grid: spectrum off the nodes"); return -1; }
    snprintf(path, sizeof path, "%s%s", folder, name);
    size_t nf = 0;
    float* fl = read_float_file(path, &nf);
    if (!fl || nf != nwl) { fclose(f); set_err("stellar grid spectrum %s missing or of the wrong size", path); return -1; }
    for (size_t i = 0; i < nwl; ++i) y[i] = (double)fl[i] * gwl[i] * gwl[i] / 10000.;
    free(fl);
    double* out = m->star_grid + ((size_t)(it * n1 + ig) * n2 + iq) * m->N;
    interp_to_wavelengths(gwl, y, (int)nwl, m->wl, m->N, out);
    for (size_t i = 0; i < m->N; ++i) if (out[i] < 1e-37) out[i] = 1e-37;
    ++count;
  }
  fclose(f);
  free(wlf); free(gwl); free(y);
  if (count != n0 * n1 * n2) { set_err("stellar grid is inconsistent"); return -1; }
  return 0;
}

/* StellarSpectrumGrid::findClosestGridPoints stellar_spectrum_grid.cpp:245-270 */
static void star_closest(const double* g, int n, double x, int* i0, int* i1) {
  if (x <= g[0]) { *i0 = *i1 = 0; return; }
  if (x >= g[n - 1]) { *i0 = *i1 = n - 1; return; }
  int j = 0;
  while (g[j] < x) ++j;
  *i1 = j;
  *i0 = g[j] != x ? j - 1 : j;
}

/* StellarSpectrumGrid::calcFlux stellar_spectrum_grid.cpp:275-330 with
 * aux::triLinearInterpolation src/additional/aux_functions.cpp:290-318 */
static void star_grid_flux(const orc_model* m, const double* sp, double* out) {
  double x[3]; int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    const double* g = m->star_axis[a]; const int n = m->star_n[a];
    x[a] = sp[a];
    if (x[a] < g[0]) x[a] = g[0];
    if (x[a] > g[n - 1]) x[a] = g[n - 1];
    star_closest(g, n, x[a], &lo[a], &hi[a]);
  }
  const int n1 = m->star_n[1], n2 = m->star_n[2];
  #define ORC_SG(t, g, q) (m->star_grid + ((size_t)((t) * n1 + (g)) * n2 + (q)) * m->N)
  const double* c000 = ORC_SG(lo[0], lo[1], lo[2]); const double* c100 = ORC_SG(hi[0], lo[1], lo[2]);
  const double* c010 = ORC_SG(lo[0], hi[1], lo[2]); const double* c110 = ORC_SG(hi[0], hi[1], lo[2]);
  const double* c001 = ORC_SG(lo[0], lo[1], hi[2]); const double* c101 = ORC_SG(hi[0], lo[1], hi[2]);
  const double* c011 = ORC_SG(lo[0], hi[1], hi[2]); const double* c111 = ORC_SG(hi[0], hi[1], hi[2]);
  #undef ORC_SG
  const double x0 = m->star_axis[0][lo[0]], x1 = m->star_axis[0][hi[0]];
  const double y0 = m->star_axis[1][lo[1]], y1 = m->star_axis[1][hi[1]];
  const double z0 = m->star_axis[2][lo[2]], z1 = m->star_axis[2][hi[2]];
  double xd = (x[0] - x0) / (x1 - x0); if (x[0] == x0) xd = 0;
  double yd = (x[1] - y0) / (y1 - y0); if (x[1] == y0) yd = 0;
  double zd = (x[2] - z0) / (z1 - z0); if (x[2] == z0) zd = 0;
  for (size_t i = 0; i < m->N; ++i) {
    const double c00 = c000[i] * (1. - xd) + c100[i] * xd;
    const double c01 = c001[i] * (1. - xd) + c101[i] * xd;
    const double c10 = c010[i] * (1. - xd) + c110[i] * xd;
    const double c11 = c011[i] * (1. - xd) + c111[i] * xd;
    const double c0 = c00 * (1. - yd) + c10 * yd;
    const double c1 = c01 * (1. - yd) + c11 * yd;
    out[i] = c0 * (1. - zd) + c1 * zd;
  }
}

int orc_finalize(orc_model* m) {
  if (m->nobs == 0) { set_err("no observations"); return -1; }
  if (m->annuli < 0 || m->annuli > 64) { set_err("transmission_annuli must be in [1, 64]"); return -1; }
  if (load_wavenumbers(m)) return -1;
  if (sample_grid(m)) return -1;
  setup_observation_operators(m);
  if (setup_opacity(m)) return -1;
  setup_atmosphere(m);
  m->nparam_general = 3 + (m->transmission && (m->fit_mmw || m->fit_sh) ? 1 : 0);
  if (m->occultation) {
    /* OccultationModel: [log g, R_p / R_s] then the stellar model's parameters
     * (src/forward_model/secondary_eclipse/secondary_eclipse.cpp:72,115-150) */
    if (m->star_model == 0) { set_err("the secondary-eclipse model needs a stellar spectrum"); return -1; }
    m->nparam_general = 2 + (m->star_model == 1 ? 1 : m->star_model == 3 ? 3 : 0);
    if (m->star_model == 2 && load_star_file(m)) return -1;
    if (m->star_model == 3 && load_star_grid(m)) return -1;
  }
  m->nparam_chem = 0;
  for (int c = 0; c < m->nchem; ++c) m->nparam_chem += m->chem_kind[c] == 0 ? m->chem_nsp[c] : 0;
  /* grey [tau, p_top, (bottom factor)]; power_law [tau, exponent, p_top, (...)];
   * KHnongrey [tau, q0, a0, particle size, p_top, (...)] */
  m->nparam_cloud = m->cloud ? (m->cloud_fb ? 2 : 3) + (m->cloud_kind == 1 ? 1 : m->cloud_kind == 2 ? 3 : 0) : 0;
  m->nparam_mod = 0; m->M = 0;
  for (int k = 0; k < m->nobs; ++k) { m->nparam_mod += m->obs[k].nb_modifier; m->obs[k].out_offset = m->M; m->M += m->obs[k].n; }
  m->nparam_total = m->nparam_general + m->nparam_chem + m->nparam_temp + m->nparam_cloud + m->nparam_mod;
  m->finalized = 1;
  return 0;
}

int orc_nb_spectral_points(const orc_model* m) { return (int)m->N; }
int orc_nb_obs_points(const orc_model* m) { return m->M; }
int orc_nb_parameters(const orc_model* m) { return m->nparam_total + (m->error_inflation ? 1 : 0); }
void orc_grid(const orc_model* m, double* nu) { memcpy(nu, m->nu, m->N * sizeof(double)); }

/* ------------------------------------------------------------------ per-eval atmosphere */
typedef struct {
  double* T; double* z; double* H; double* mmw; double* nd; /* nd[L][SP_COUNT] */
  int neglect;
} atm_t;

/* PiecewisePolynomial::getValue src/additional/piecewise_poly.cpp:154-181,
 * Element::getValue / lagrangeBase :202-229 */
static double pp_value(const orc_model* m, const double* dof, double x) {
  if (x > m->pp_dof_vertices[0] || x < m->pp_dof_vertices[m->pp_ndof - 1]) return 0.0;
  for (int i = 0; i < m->pp_ndof; ++i) if (m->pp_dof_vertices[i] == x) return dof[i];
  int el = 0;
  const int nd = m->pp_ndof_el;
  for (int e = 0; e < m->pp_nel; ++e)
    if (m->pp_el_vert[e * nd] > x && m->pp_el_vert[e * nd + nd - 1] < x) { el = e; break; }
  const double xl = m->pp_el_vert[el * nd], xr = m->pp_el_vert[el * nd + nd - 1];
  const double r = 2.0 * (x - xl) / (xr - xl) - 1.0;
  double y = 0;
  for (int i = 0; i < nd; ++i) {
    double l = 1;
    for (int j = 0; j < nd; ++j) { if (i == j) continue; l *= (r - m->pp_ref[j]) / (m->pp_ref[i] - m->pp_ref[j]); }
    y += dof[el * (nd - 1) + i] * l;
  }
  return y;
}

static void mean_molecular_weight(int L, const double* nd, double* mmw) {
  /* Chemistry::meanMolecularWeight src/chemistry/chemistry.h:47-59 */
  for (int i = 0; i < L; ++i) {
    double mu = 0;
    for (int j = 0; j < SP_COUNT; ++j) mu += nd[i * SP_COUNT + j] / nd[i * SP_COUNT + SP_TOTAL] * SP_MW[j];
    mmw[i] = mu;
  }
}

static int atmosphere(const orc_model* m, const double* tparam, const double* cparam, double g,
                      double bottom_radius, double fixed_mmw, atm_t* a) {
  /* Atmosphere::calcAtmosphereStructure src/forward_model/atmosphere/atmosphere.cpp:63-187 */
  const int L = m->L;
  int neglect = 0;
  if (m->temp_poly) {
    /* PiecewisePolynomialTemperature::calcProfile src/temperature/piecewise_poly_temperature.cpp:49-84 */
    double dof[64];
    dof[0] = tparam[0];
    for (int i = 1; i < m->nparam_temp; ++i) dof[i] = dof[i - 1] * tparam[i];
    for (int i = 0; i < L; ++i) a->T[i] = pp_value(m, dof, log10(m->p[i]));
    for (int i = 0; i < L; ++i) if (a->T[i] < 50) { a->T[i] = 50; neglect = 1; }
  } else {
    for (int i = 0; i < L; ++i) a->T[i] = tparam[0]; /* src/temperature/constant_temperature.h:37-44 */
  }
  memset(a->nd, 0, sizeof(double) * L * SP_COUNT);
  for (int i = 0; i < L; ++i) a->mmw[i] = 0.0;
  int pidx = 0;
  for (int c = 0; c < m->nchem; ++c) {
    if (m->chem_kind[c] == 0) {
      /* IsoprofileChemistry::calcChemicalComposition src/chemistry/isoprofile_chemistry.cpp:87-119 */
      const double solar_na_k = 16.2181;
      for (int i = 0; i < L; ++i) {
        double* n = a->nd + i * SP_COUNT;
        n[SP_TOTAL] = m->p[i] * 1.e6 / K_BOLTZMANN / a->T[i];
        for (int j = 0; j < m->chem_nsp[c]; ++j) n[m->chem_sp[c][j]] = n[SP_TOTAL] * cparam[pidx + j];
        if (!m->chem_na_free[c]) n[SP_Na] = n[SP_K] * solar_na_k;
      }
      mean_molecular_weight(L, a->nd, a->mmw);
      /* checkMixingRatios src/chemistry/chemistry.h:61-76 */
      for (int i = 0; i < L; ++i) {
        double s = 0; const double* n = a->nd + i * SP_COUNT;
        for (int j = 0; j < SP_COUNT; ++j) if (j != SP_TOTAL) s += n[j] / n[SP_TOTAL];
        if (s > 1 + 1e-10) { neglect = 1; break; }
      }
      pidx += m->chem_nsp[c];
    } else {
      /* BackgroundChemistry::calcChemicalComposition src/chemistry/background_chemistry.cpp:72-137 */
      const double sh2 = 0.5, she = 0.085114, sh2he = sh2 + she;
      for (int i = 0; i < L; ++i) a->nd[i * SP_COUNT + SP_TOTAL] = m->p[i] * 1.e6 / K_BOLTZMANN / a->T[i];
      for (int i = 0; i < L; ++i) {
        double* n = a->nd + i * SP_COUNT;
        double bg = 1.0;
        for (int j = 0; j < SP_COUNT; ++j) {
          if (j == SP_TOTAL) continue;
          if (m->chem_bg_h2he[c]) { if (j != SP_H2 && j != SP_He) bg -= n[j] / n[SP_TOTAL]; }
          else if (j != m->chem_bg_sp[c]) bg -= n[j] / n[SP_TOTAL];
        }
        if (bg < 0) { neglect = 1; bg = 0; }
        if (m->chem_bg_h2he[c]) {
          const double xh2 = bg * sh2 / sh2he, xhe = bg * she / sh2he;
          n[SP_H2] = n[SP_TOTAL] * xh2; n[SP_He] = n[SP_TOTAL] * xhe;
          continue;
        }
        n[m->chem_bg_sp[c]] = n[SP_TOTAL] * bg;
      }
      mean_molecular_weight(L, a->nd, a->mmw);
    }
  }
  if (fixed_mmw > 0) for (int i = 0; i < L; ++i) a->mmw[i] = fixed_mmw;
  /* calcAltitude :288-307 / calcAltitudeVariableGravity :311-334 */
  double* rho = (double*)malloc(L * sizeof(double));
  for (int i = 0; i < L; ++i) rho[i] = a->mmw[i] * m->p[i] * 1e6 / (K_GAS * a->T[i]);
  a->z[0] = 0.0;
  for (int i = 1; i < L; ++i) {
    double gi = g;
    /* transmission models only (emission.cpp:178-185 and secondary_eclipse.cpp:165-172 pass false) */
    if (m->var_g && m->transmission) { const double lr = bottom_radius + a->z[i - 1]; gi = g * pow(bottom_radius / lr, 2.0); }
    double dz = (1.0 / (rho[i] * gi) + 1.0 / (rho[i - 1] * gi)) * 0.5 * (m->p[i - 1] * 1e6 - m->p[i] * 1e6);
    a->z[i] = a->z[i - 1] + dz;
  }
  free(rho);
  /* calcScaleHeight :353-360 */
  for (int i = 0; i < L; ++i) a->H[i] = K_GAS * a->T[i] / (a->mmw[i] * g);
  a->neglect = neglect;
  return neglect;
}

/* GreyCloudModel::cloudPosition (both variants) src/cloud_model/grey_cloud_model.cpp:112-195 */
static void cloud_position(const orc_model* m, const atm_t* a, double ptop, double pbottom,
                           int fb, unsigned* top, unsigned* bottom) {
  const int L = m->L;
  unsigned ti = 0, bi = 0;
  for (int i = 0; i < L - 1; ++i)
    if ((m->p[i] > ptop && m->p[i + 1] < ptop) || m->p[i] == ptop) ti = i;
  if (fb) {
    if (ptop < m->p[L - 1]) ti = L - 1;
    double ba = a->z[ti] - a->H[ti];
    if (ba < 0) ba = 0;
    for (int i = 0; i < L - 1; ++i)
      if ((a->z[i] < ba && a->z[i + 1] > ba) || a->z[i] == ba) bi = i;
    if (ti == bi) bi -= 2;
    if (ti == bi) bi -= 2;
    if (ti < 2) { ti = 2; bi = 0; }
  } else {
    for (int i = 0; i < L - 1; ++i)
      if ((m->p[i] > pbottom && m->p[i + 1] < pbottom) || m->p[i] == pbottom) bi = i;
    if (ptop <= m->p[L - 1]) ti = L - 1;
    if (pbottom >= m->p[0]) bi = 0;
    if (ti == bi) bi -= 2;
    if (ti < 2) { ti = 2; bi = 0; }
  }
  *top = ti; *bottom = bi;
}

/* ------------------------------------------------------------------ opacity per eval */
static int find_closest_points(const opac_t* op, double p, double T, int* t0, int* q0, int* t1, int* q1,
                               int* t2, int* q2, int* t3, int* q3) {
  /* OpacitySpecies::findClosestDataPoints src/transport_coeff/opacity_species.cpp:160-273 */
  int lo = 0, up = 0;
  if (T < op->T[0]) { lo = up = 0; }
  else if (T > op->T[op->nT - 1]) { lo = up = op->nT - 1; }
  else {
    for (int i = 0; i < op->nT; ++i) {
      if (op->T[i] == T) { lo = up = i; break; }
      else if (op->T[i] < T && op->T[i + 1] > T) { lo = i; up = i + 1; break; }
    }
  }
  int tt[2] = {lo, up}; int a[2] = {0, 0}, b[2] = {0, 0};
  for (int k = 0; k < 2; ++k) {
    const int t = tt[k]; const int np = op->nP[t];
    if (p < op->P[t][0]) { a[k] = b[k] = 0; }
    else if (p > op->P[t][np - 1]) { a[k] = b[k] = np - 1; }
    else {
      for (int i = 0; i < np; ++i) {
        if (op->P[t][i] == p) { a[k] = b[k] = i; break; }
        else if (op->P[t][i] < p && op->P[t][i + 1] > p) { a[k] = i; b[k] = i + 1; break; }
      }
    }
  }
  *t0 = lo; *q0 = a[0]; *t1 = lo; *q1 = b[0]; *t2 = up; *q2 = a[1]; *t3 = up; *q3 = b[1];
  return 0;
}

/* OpacitySpecies::calcAbsorptionCrossSections :277-345 + calcTransportCoefficients :400-455;
 * adds into absorption[nu*L + level] and scattering[nu*L + level] */
static void species_coefficients(const orc_model* m, const opac_t* op, const double* n, double T,
                                 double p, int level, double* absorption, double* scattering) {
  const size_t N = m->N; const int L = m->L;
  double nd = n[op->index];
  for (int k = 0; k < op->npartner; ++k) nd *= n[op->partner[k]];
  if (nd == 0) return;
  if (op->kind == 0) {
    int t0, q0, t1, q1, t2, q2, t3, q3;
    find_closest_points(op, p, T, &t0, &q0, &t1, &q1, &t2, &q2, &t3, &q3);
    const double* r0 = op->rows[t0][q0]; const double* r1 = op->rows[t1][q1];
    const double* r2 = op->rows[t2][q2]; const double* r3 = op->rows[t3][q3];
    const int same01 = (t0 == t1 && q0 == q1), same23 = (t2 == t3 && q2 == q3), same02 = (t0 == t2 && q0 == q2);
    const double lp = log10(p);
    const double lp0 = op->logP[t0][q0], lp1 = op->logP[t1][q1], lp2 = op->logP[t2][q2], lp3 = op->logP[t3][q3];
    const double T0 = op->T[t0], T2 = op->T[t2];
    #pragma omp parallel for
    for (long i = 0; i < (long)N; ++i) {
      double cs;
      if (same01 && same02 && same23) cs = pow(10.0, r0[i]);
      else {
        double lower = r0[i], upper = r2[i];
        if (!same01) lower = r0[i] + (r1[i] - r0[i]) * (lp - lp0) / (lp1 - lp0);
        if (!same23) upper = r2[i] + (r3[i] - r2[i]) * (lp - lp2) / (lp3 - lp2);
        if (!same02) cs = lower + (upper - lower) * (T - T0) / (T2 - T0);
        else cs = lower;
        cs = pow(10.0, cs);
      }
      absorption[i * L + level] += cs * nd;
    }
  }
  if (op->kind == 1) {
    const double ns = n[op->index];
    #pragma omp parallel for
    for (long i = 0; i < (long)N; ++i) scattering[i * L + level] += op->rayleigh[i] * ns;
  }
  if (op->kind == 2) {
    /* GasHm::calcContinuumAbsorption h_m.cpp:36-53 with freeFreeAbsorption :88-137 */
    double pw[7];
    for (int i = 1; i < 7; ++i) pw[i] = pow(5040.0 / T, (i + 1) / 2.0);
    const double pe = n[SP_e] * K_BOLTZMANN * T, nh = n[SP_H], nhm = n[SP_Hm];
    #pragma omp parallel for
    for (long i = 0; i < (long)N; ++i) {
      double x = 0;
      for (int j = 1; j < 7; ++j) x += pw[j] * op->hm_ff[j][i];
      const double kff = x * 1e-29;
      absorption[i * L + level] += op->hm_bf[i] * nhm + kff * pe * nh;
    }
  }
}

/* ------------------------------------------------------------------ radiative transfer */
static double planck_wn(double T, double nu) {
  /* aux::planckFunctionWavenumber src/additional/aux_functions.cpp:272-278 */
  return 2. * K_PLANCK_H * K_LIGHT_C * K_LIGHT_C * nu * nu * nu
       / (exp(K_PLANCK_H * nu * K_LIGHT_C / K_BOLTZMANN / T) - 1.0);
}

/* ShortCharacteristics::calcSpectrum src/radiative_transfer/short_characteristics.cpp:39-125 */
static double sc_point(const orc_model* m, const double* kappa, const double* cloud_tau, const double* cnum,
                       const double* cden, const atm_t* a, size_t nu_i) {
  const int L = m->L;
  const double mu[2] = {0.211324865405187, 0.788675134594813};
  const double w[2] = {0.5, 0.5};
  double tau[512], B[512];
  for (int i = 0; i < L - 1; ++i) tau[i] = (a->z[i + 1] - a->z[i]) * (kappa[i + 1] + kappa[i]) / 2.;
  if (cloud_tau)
    for (int i = 0; i < L - 1; ++i) tau[i] += cnum ? cloud_tau[i] * cnum[nu_i] / cden[nu_i] : cloud_tau[i];
  for (int i = 0; i < L; ++i) B[i] = planck_wn(a->T[i], m->nu[nu_i]);
  double I1 = B[0], I2 = B[0];
  for (int i = 0; i < L - 1; ++i) {
    if (tau[i] == 0) continue;
    const double d1 = tau[i] / mu[0];
    const double a1 = exp(-d1);
    I1 = I1 * a1;
    const double b1 = 1.0 + (a1 - 1.0) / d1;
    const double g1 = -a1 - (a1 - 1.0) / d1;
    I1 += b1 * B[i + 1] + g1 * B[i];
    const double d2 = tau[i] / mu[1];
    const double a2 = exp(-d2);
    I2 = I2 * a2;
    const double b2 = 1.0 + (a2 - 1.0) / d2;
    const double g2 = -a2 - (a2 - 1.0) / d2;
    I2 += b2 * B[i + 1] + g2 * B[i];
  }
  return 2.0 * K_PI * (I1 * mu[0] * w[0] + I2 * mu[1] * w[1]) * 1e-3;
}

/* TransmissionModel::tangentPathsTransmission / tangentOpticalDepth /
 * integrateEffectiveTangentHeight / distanceToTangentCenter
 * src/forward_model/transmission/transmission_spectrum.cpp:32-154 */
/* The transit depth with A impact parameters per layer (A = 1 is the reference's
 * formula, transit_point below): in layer t, b_k = R + zb_k with
 * zb_k = z_t + (z_{t+1} - z_t) j / A, j = 0..A-1, plus the top level. A ray's first,
 * partial segment from its tangent point to level t+1 uses the extinction interpolated
 * linearly in altitude at zb_k, chi_t + (chi_{t+1} - chi_t) j / A; the other segments
 * and the tau > cut-off rule are the reference's; the effective height is the same
 * trapezoid over the finer grid of impact parameters. Not in the reference. */
static double transit_point_annuli(const orc_model* m, const double* chi, const atm_t* a, double R, double Rs) {
  const int L = m->L, A = m->annuli, K = (L - 1) * A;
  double* zb = (double*)malloc((K + 1) * sizeof(double));
  double* trans = (double*)malloc((K + 1) * sizeof(double));
  for (int k = 0; k < K; ++k) {
    const int t = k / A, j = k % A;
    zb[k] = a->z[t] + (a->z[t + 1] - a->z[t]) * j / A;
  }
  zb[K] = a->z[L - 1];
  trans[K] = 1;
  for (int k = K - 1; k >= 0; --k) {
    const int t = k / A, j = k % A;
    const double b = R + zb[k];
    const double chib = chi[t] + (chi[t + 1] - chi[t]) * j / A;
    const double a1 = R + a->z[t + 1];
    double tau = sqrt(a1 * a1 - b * b) * (chib + chi[t + 1]);
    if (!(tau > m->tau_cut))
      for (int i = t + 1; i < L - 1; ++i) {
        const double u1 = R + a->z[i + 1], u0 = R + a->z[i];
        tau += (sqrt(u1 * u1 - b * b) - sqrt(u0 * u0 - b * b)) * (chi[i] + chi[i + 1]);
        if (tau > m->tau_cut) break;
      }
    trans[k] = exp(-tau);
  }
  double h = 0;
  for (int k = 0; k < K; ++k)
    h += 2. * ((R + zb[k]) * (1. - trans[k]) + (R + zb[k + 1]) * (1. - trans[k + 1])) * (zb[k + 1] - zb[k]) * 0.5;
  free(zb); free(trans);
  h = sqrt(h + R * R) - R;
  const double rp = h + R;
  return rp * rp / Rs / Rs * 1e6;
}

static double transit_point(const orc_model* m, const double* chi, const atm_t* a, double R, double Rs) {
  if (m->annuli > 1) return transit_point_annuli(m, chi, a, R, Rs);
  const int L = m->L;
  double trans[512];
  trans[L - 1] = 1;
  for (int t = L - 2; t > -1; --t) {
    double tau = 0;
    for (int i = t; i < L - 1; ++i) {
      const double b = R + a->z[t];
      const double a1 = R + a->z[i + 1], a0 = R + a->z[i];
      const double path = sqrt(a1 * a1 - b * b) - sqrt(a0 * a0 - b * b);
      tau += path * (chi[i] + chi[i + 1]);
      if (tau > m->tau_cut) break;
    }
    trans[t] = exp(-tau);
  }
  double h = 0;
  for (int i = 0; i < L - 1; ++i)
    h += 2. * ((R + a->z[i]) * (1. - trans[i]) + (R + a->z[i + 1]) * (1. - trans[i + 1])) * (a->z[i + 1] - a->z[i]) * 0.5;
  h = sqrt(h + R * R) - R;
  const double rp = h + R;
  return rp * rp / Rs / Rs * 1e6;
}

/* ------------------------------------------------------------------ observation operator */
static double normal_dist(double sigma, double x) {
  /* aux::normalDistribution(sigma, x) src/additional/aux_functions.cpp:344-351 */
  const double c = sqrt(1.0 / (2.0 * K_PI));
  return c / sigma * exp(-x * x / (2.0 * sigma * sigma));
}

/* Observation::processModelSpectrum src/observations/observations.cpp:290-304 with
 * applyFilterResponseFunction, SpectralBands::convolveSpectrum
 * (src/spectral_grid/spectral_band_convolve.cpp:100-144) and bandIntegrateSpectrum
 * (src/spectral_grid/spectral_band_integrate.cpp:39-107); writes internal-order bins */
static void process_observation(const orc_model* m, const obs_t* o, const double* spectrum, int is_flux, double* bands) {
  const size_t N = m->N;
  double* filt = (double*)malloc(N * sizeof(double));
  if (o->nfilter) for (size_t i = 0; i < N; ++i) filt[i] = spectrum[i] * o->filter_on_grid[i] * o->filter_weight[i] / o->filter_norm;
  else memcpy(filt, spectrum, N * sizeof(double));
  double* conv = filt;
  if (o->has_profile) {
    conv = (double*)calloc(N, sizeof(double));
    #pragma omp parallel for
    for (long ii = (long)o->range_lo; ii < (long)o->range_hi + 1; ++ii) {
      const size_t i = (size_t)ii, ci = i - o->range_lo;
      if (o->conv[ci][0] == o->conv[ci][1] || o->sigma[i] == 0) { conv[i] = filt[i]; continue; }
      const size_t s = o->conv[ci][0], e = o->conv[ci][1];
      /* quadratureTrapezoidal over x = wl[s..e), y = filt[s..e) * N(sigma, |wl_i - x|) */
      const size_t n = e - s;
      double sum = 0.0;
      if (n == 1) sum = filt[s] * normal_dist(o->sigma[i], fabs(m->wl[i] - m->wl[s])) / 0.5;
      double yprev = filt[s] * normal_dist(o->sigma[i], fabs(m->wl[i] - m->wl[s]));
      for (size_t j = s + 1; j < e; ++j) {
        const double y = filt[j] * normal_dist(o->sigma[i], fabs(m->wl[i] - m->wl[j]));
        sum += (m->wl[j] - m->wl[j - 1]) * (y + yprev);
        yprev = y;
      }
      conv[i] = fabs(sum * 0.5);
    }
  }
  for (int b = 0; b < o->n; ++b) {
    const size_t i0 = o->edge_idx[b][0], i1 = o->edge_idx[b][1];
    double sum = 0.0;
    if (is_flux) {
      const double wl_l = 1.0 / m->nu[i0] * 1e4, wl_r = 1.0 / m->nu[i1] * 1e4;
      for (size_t i = i0 + 1; i < i1 + 1; ++i) sum += (m->nu[i] - m->nu[i - 1]) * (conv[i] + conv[i - 1]);
      bands[b] = sum * 0.5 / (wl_l - wl_r);
    } else {
      const double wl_r = m->wl[i1], wl_l = m->wl[i0];
      for (size_t i = i0 + 1; i < i1 + 1; ++i) sum += (m->wl[i] - m->wl[i - 1]) * (conv[i] + conv[i - 1]);
      double v = fabs(sum * 0.5);
      if (!o->nfilter) v /= (wl_l - wl_r);
      bands[b] = v;
    }
  }
  if (conv != filt) free(conv);
  free(filt);
}

/* ------------------------------------------------------------------ forward model */
/* EmissionModel::calcModelCPU src/forward_model/emission/emission.cpp:194-228 and
 * TransmissionModel::calcModelCPU src/forward_model/transmission/transmission.cpp:199-251,
 * then ForwardModel::calcModel's order reversal src/forward_model/forward_model.cpp:119-123.
 * spectrum: N (emission: per micron after changeSpectrumUnits; transmission: ppm);
 * obs: M in the caller's (input) order. */
int orc_forward(const orc_model* m, const double* par, int P, double* spectrum, double* obs_out, int* neglect_out) {
  if (!m->finalized) { set_err("model not finalized"); return -1; }
  if (P < m->nparam_total) { set_err("expected %d parameters, got %d", m->nparam_total, P); return -1; }
  const int L = m->L; const size_t N = m->N;
  const double* gen = par;
  const double* chem = par + m->nparam_general;
  const double* temp = chem + m->nparam_chem;
  const double* cloud = temp + m->nparam_temp;
  const double* mods = cloud + m->nparam_cloud;

  atm_t a;
  a.T = (double*)malloc(L * sizeof(double)); a.z = (double*)malloc(L * sizeof(double));
  a.H = (double*)malloc(L * sizeof(double)); a.mmw = (double*)malloc(L * sizeof(double));
  a.nd = (double*)malloc((size_t)L * SP_COUNT * sizeof(double));
  const double g = pow(10, gen[0]);
  int neglect;
  if (!m->transmission) {
    /* EmissionModel::calcAtmosphereStructure :158-189; the derived-mass neglect flag is
     * overwritten by the atmosphere's return value there, so it is not computed here */
    neglect = atmosphere(m, temp, chem, g, 1.0, 0.0, &a);
  } else {
    neglect = atmosphere(m, temp, chem, g, gen[1], (m->fit_mmw ? gen[3] : 0.0), &a);
  }

  /* OpacityCalculation::calculate src/transport_coeff/opacity_calc.h:154-243 */
  double* absorption = (double*)calloc(N * L, sizeof(double));
  double* scattering = (double*)calloc(N * L, sizeof(double));
  for (int l = 0; l < L; ++l)
    for (int s = 0; s < m->nopac; ++s)
      species_coefficients(m, &m->opac[s], a.nd + (size_t)l * SP_COUNT, a.T[l], m->p[l], l, absorption, scattering);

  double* cloud_tau = NULL;   /* [L-1] layer optical depth of the grey placement */
  double *cnum = NULL, *cden = NULL;  /* non-grey clouds: layer depth x cnum / cden per nu */
  if (m->cloud) {
    /* GreyCloudModel::opticalProperties src/cloud_model/grey_cloud_model.cpp:59-106;
     * PowerLawCloudModel::opticalProperties power_law_cloud_model.cpp:69-121 and
     * KHCloudModel::opticalProperties kh_cloud_model.cpp:69-133 place the cloud the same way */
    const int it = m->cloud_kind == 0 ? 1 : m->cloud_kind == 1 ? 2 : 4;
    double tau_c = cloud[0], ptop = cloud[it], pbot = 0;
    if (!m->cloud_fb) pbot = ptop * cloud[it + 1];
    if (m->cloud_kind) {
      cnum = (double*)malloc(N * sizeof(double)); cden = (double*)malloc(N * sizeof(double));
      if (m->cloud_kind == 1) {
        const double expo = cloud[1], ref = pow(m->cloud_ref_wl, expo);
        for (size_t i = 0; i < N; ++i) { cnum[i] = pow(m->wl[i], expo); cden[i] = ref; }
      } else {
        const double q0 = cloud[1], a0 = cloud[2], r = cloud[3];
        const double xr = 2 * K_PI * r / m->cloud_ref_wl;
        const double refq = q0 * pow(xr, -a0) + pow(xr, 0.2);
        for (size_t i = 0; i < N; ++i) {
          const double x = 2 * K_PI * r / m->wl[i];
          cnum[i] = refq;
          cden[i] = q0 * pow(x, -a0) + pow(x, 0.2);
        }
      }
    }
    if (tau_c < 0) tau_c = 0;
    unsigned ti, bi;
    cloud_position(m, &a, ptop, pbot, m->cloud_fb, &ti, &bi);
    cloud_tau = (double*)calloc(L, sizeof(double));
    const double per = tau_c / (double)(ti - bi);
    for (unsigned i = ti; i > bi; --i) if ((int)i < L - 1) cloud_tau[i] = per;
  }

  double* spec = (double*)malloc(N * sizeof(double));
  double* star = NULL;
  if (m->occultation) {
    /* OccultationModel::calcModelCPU src/forward_model/secondary_eclipse/secondary_eclipse.cpp:183-246:
     * planet emission without the radius-distance scaling, stellar spectrum from the model */
    #pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)N; ++i) spec[i] = sc_point(m, absorption + (size_t)i * L, cloud_tau, cnum, cden, &a, (size_t)i);
    star = (double*)malloc(N * sizeof(double));
    if (m->star_model == 3) star_grid_flux(m, gen + 2, star);
    else
      for (size_t i = 0; i < N; ++i)  /* StarBlackBody::calcFlux star_blackbody.cpp:35-47 */
        star[i] = m->star_model == 1 ? planck_wn(gen[2], m->nu[i]) * K_PI * 1e-3 : m->star_flux[i];
  } else if (!m->transmission) {
    const double scaling = (K_RJUP / gen[2]) * (K_RJUP / gen[2]) * gen[1];
    #pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)N; ++i) spec[i] = sc_point(m, absorption + (size_t)i * L, cloud_tau, cnum, cden, &a, (size_t)i);
    for (size_t i = 0; i < N; ++i) spec[i] *= scaling;
  } else {
    const double R = gen[1], Rs = gen[2];
    double* ext = NULL;
    if (cloud_tau) {
      /* CloudModel::convertOpticalDepth src/cloud_model/cloud_model.h:67-88 */
      ext = (double*)calloc(L, sizeof(double));
      for (int j = 1; j < L; ++j) ext[j] = cloud_tau[j - 1] / (a.z[j] - a.z[j - 1]);
    }
    #pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)N; ++i) {
      double chi[512];
      for (int l = 0; l < L; ++l) {
        double e = ext ? ext[l] : 0.0;
        if (cnum && l > 0) e = cloud_tau[l - 1] * cnum[i] / cden[i] / (a.z[l] - a.z[l - 1]);
        chi[l] = absorption[(size_t)i * L + l] + scattering[(size_t)i * L + l] + e;
      }
      spec[i] = transit_point(m, chi, &a, R, Rs);
    }
    free(ext);
  }

  /* convertSpectrumToObservation + applyObservationModifier src/forward_model/forward_model.cpp:131-180 */
  int mi = 0;
  for (int k = 0; k < m->nobs; ++k) {
    const obs_t* o = &m->obs[k];
    double* bands = (double*)malloc((o->n ? o->n : 1) * sizeof(double));
    process_observation(m, o, spec, !m->transmission, bands);
    if (m->occultation) {
      /* occultation depth: binned planet / binned star x (R_p / R_s)^2 x 1e6 */
      double* sb = (double*)malloc((o->n ? o->n : 1) * sizeof(double));
      process_observation(m, o, star, 1, sb);
      for (int b = 0; b < o->n; ++b) bands[b] = bands[b] / sb[b] * gen[1] * gen[1] * 1e6;
      free(sb);
    }
    if (o->nb_modifier) { const double c = mods[mi]; if (c != 0) for (int b = 0; b < o->n; ++b) bands[b] += c; mi += o->nb_modifier; }
    for (int b = 0; b < o->n; ++b) obs_out[o->out_offset + b] = o->ascending ? bands[o->n - 1 - b] : bands[b];
    free(bands);
  }
  if (m->occultation) {
    for (size_t i = 0; i < N; ++i) spec[i] = spec[i] / star[i] * gen[1] * gen[1] * 1e6;
  } else if (!m->transmission) {
    /* RadiativeTransfer::changeSpectrumUnits src/radiative_transfer/radiative_transfer.h:58-60 */
    for (size_t i = 0; i < N; ++i) spec[i] = spec[i] / m->wl[i] / m->wl[i] * 10000.0;
  }
  free(star);
  if (spectrum) memcpy(spectrum, spec, N * sizeof(double));
  *neglect_out = neglect;
  free(spec); free(absorption); free(scattering); free(cloud_tau); free(cnum); free(cden);
  free(a.T); free(a.z); free(a.H); free(a.mmw); free(a.nd);
  return 0;
}

/* Contribution functions: contributionFunctionDevice
 * src/CUDA_kernels/contribution_function_kernels.cu:21-66 as driven by
 * EmissionModel::postProcessContributionFunctions src/forward_model/emission/emission_post_process.cpp:330-376
 * (secondary eclipse: secondary_eclipse_post_process.cpp:255-305): gas absorption only, from
 * the top down, CF_i = 2 pi B(T_i) (1 - exp(-dtau_i)) x the transmission above; level 0 is
 * left 0 here (never written by the reference). hr: L x N; bins: L x M, each level binned with
 * wavelength integration (is_flux = false) and in the caller's order. The reference keeps its
 * opacities as floats on the GPU; this restatement is FP64 throughout. */
int orc_contribution(const orc_model* m, const double* par, int P, double* hr, double* bins) {
  if (!m->finalized) { set_err("model not finalized"); return -1; }
  if (m->transmission) { set_err("contribution functions exist for emission models only"); return -1; }
  if (P < m->nparam_total) { set_err("expected %d parameters, got %d", m->nparam_total, P); return -1; }
  const int L = m->L; const size_t N = m->N;
  const double* gen = par;
  const double* chem = par + m->nparam_general;
  const double* temp = chem + m->nparam_chem;
  atm_t a;
  a.T = (double*)malloc(L * sizeof(double)); a.z = (double*)malloc(L * sizeof(double));
  a.H = (double*)malloc(L * sizeof(double)); a.mmw = (double*)malloc(L * sizeof(double));
  a.nd = (double*)malloc((size_t)L * SP_COUNT * sizeof(double));
  atmosphere(m, temp, chem, pow(10, gen[0]), 1.0, 0.0, &a);
  double* absorption = (double*)calloc(N * L, sizeof(double));
  double* scattering = (double*)calloc(N * L, sizeof(double));
  for (int l = 0; l < L; ++l)
    for (int s = 0; s < m->nopac; ++s)
      species_coefficients(m, &m->opac[s], a.nd + (size_t)l * SP_COUNT, a.T[l], m->p[l], l, absorption, scattering);
  double* cf = (double*)calloc(N * L, sizeof(double));
  #pragma omp parallel for
  for (long k = 0; k < (long)N; ++k) {
    double tcum = 1.0;
    for (int i = L - 1; i > 0; --i) {
      const double dz = a.z[i] - a.z[i - 1];
      const double dtau = dz * (absorption[(size_t)k * L + i] + absorption[(size_t)k * L + i - 1]) / 2.;
      const double t = exp(-dtau);
      cf[(size_t)i * N + k] = 2 * K_PI * planck_wn(a.T[i], m->nu[k]) * (1.0 - t) * tcum;
      tcum *= t;
    }
  }
  if (hr) memcpy(hr, cf, N * L * sizeof(double));
  if (bins) {
    for (int l = 0; l < L; ++l)
      for (int k = 0; k < m->nobs; ++k) {
        const obs_t* o = &m->obs[k];
        double* bands = (double*)malloc((o->n ? o->n : 1) * sizeof(double));
        process_observation(m, o, cf + (size_t)l * N, 0, bands);
        for (int b = 0; b < o->n; ++b) bins[(size_t)l * m->M + o->out_offset + b] = o->ascending ? bands[o->n - 1 - b] : bands[b];
        free(bands);
      }
  }
  free(cf); free(absorption); free(scattering);
  free(a.T); free(a.z); free(a.H); free(a.mmw); free(a.nd);
  return 0;
}

/* Retrieval::logLikelihood src/retrieval/retrieval.cpp:314-369 */
int orc_loglike(const orc_model* m, const double* par, int P, double* loglike, double* obs_out) {
  double* obs = obs_out ? obs_out : (double*)malloc((m->M ? m->M : 1) * sizeof(double));
  int neglect = 0;
  if (orc_forward(m, par, P, NULL, obs, &neglect)) { if (!obs_out) free(obs); return -1; }
  double infl = 0;
  if (m->error_inflation) infl = pow(10, par[P - 1]);
  double ll = 0;
  for (int k = 0; k < m->nobs; ++k) {
    const obs_t* o = &m->obs[k];
    for (int j = 0; j < o->n; ++j) {
      const double mod = o->ascending ? obs[o->out_offset + o->n - 1 - j] : obs[o->out_offset + j];
      const double es = o->error[j] * o->error[j] + infl;
      const double d = o->data[j] - mod;
      ll += (-0.5 * log(es * 2.0 * K_PI) - 0.5 * d * d / es) * o->weight[j];
    }
  }
  if (neglect) ll = -1e30;
  *loglike = ll;
  if (!obs_out) free(obs);
  return 0;
}

/* Optical depth at which tangent-ray sums stop (the reference's 10; INFINITY:
 * none). Test infrastructure: gradient checks by central differences use the
 * smooth model without the cut-off. */
int orc_set_tau_cutoff(orc_model* m, double tau) {
  if (!m || !(tau > 0)) return 1;
  m->tau_cut = tau;
  return 0;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n; return 1;
#endif
}

/* setup dump for parity checks of the integer setup: per observation
 * [range_lo, range_hi, n, edge pairs..., conv pairs...] */
int orc_obs_setup(const orc_model* m, int k, long* out, int cap) {
  const obs_t* o = &m->obs[k];
  int c = 0;
  if (cap < 3) return -1;
  out[c++] = (long)o->range_lo; out[c++] = (long)o->range_hi; out[c++] = o->n;
  for (int b = 0; b < o->n && c + 2 <= cap; ++b) { out[c++] = (long)o->edge_idx[b][0]; out[c++] = (long)o->edge_idx[b][1]; }
  if (o->has_profile) {
    size_t nhr = o->range_hi - o->range_lo + 1;
    for (size_t i = 0; i < nhr && c + 2 <= cap; ++i) { out[c++] = (long)o->conv[i][0]; out[c++] = (long)o->conv[i][1]; }
  }
  return c;
}

void orc_destroy(orc_model* m) {
  if (!m) return;
  for (int i = 0; i < m->nopac; ++i) {
    opac_t* op = &m->opac[i];
    for (int t = 0; t < op->nT; ++t) {
      if (op->rows && op->rows[t]) {
        for (int q = 0; q < op->nP[t]; ++q) free(op->rows[t][q]);
        free(op->rows[t]);
      }
      if (op->P) free(op->P[t]);
      if (op->logP) free(op->logP[t]);
    }
    free(op->rows); free(op->P); free(op->logP); free(op->nP); free(op->T);
    free(op->rayleigh); free(op->hm_bf);
    for (int j = 1; j < 7; ++j) free(op->hm_ff[j]);
  }
  for (int i = 0; i < m->nobs; ++i) {
    obs_t* o = &m->obs[i];
    free(o->data); free(o->error); free(o->weight); free(o->fwhm); free(o->edges); free(o->centers);
    free(o->edge_nu); free(o->edge_idx); free(o->sigma); free(o->conv); free(o->filter_wl);
    free(o->filter_resp); free(o->filter_on_grid); free(o->filter_weight);
  }
  free(m->nu_full); free(m->wl_full); free(m->index_list); free(m->nu); free(m->wl); free(m->p);
  free(m->pp_dof_vertices); free(m->pp_el_vert); free(m->star_flux); free(m->star_grid);
  for (int a = 0; a < 3; ++a) free(m->star_axis[a]);
  free(m);
}
