/*
 * bear_gb300.h -- C ABI of the GB300 likelihood engine (libbeargb300.so).
 *
 * The engine evaluates BeAR's per-likelihood forward-model path on one GPU:
 * opacity assembly from tabulated cross sections, short-characteristics
 * emission or slant-path transmission radiative transfer, the observation
 * operator (filter, instrument-profile convolution, bin integration) and the
 * Gaussian log-likelihood. All signatures use plain pointers and sizes; device
 * pointers are CUDA device addresses, streams are cudaStream_t passed as void*.
 *
 * Each entry point names the reference interface it replaces (paths inside the
 * BeAR project).
 *
 * Status: every function returns 0 on success or a BEAR_ERR_* code; the
 * message of the last failure on the calling thread is bear_last_error().
 * No function calls exit(); invalid physics is reported per evaluation through
 * the neglect flag (the reference then reports log L = -1e30).
 *
 * Threading: a model is used by one host thread / one stream at a time. Batch
 * calls are stream-ordered and allocate nothing once a batch size has been
 * seen (work buffers grow on first use of a larger batch).
 *
 * Devices: every call that touches the GPU makes the model's device (the one
 * given to bear_model_create) current while it runs and restores the caller's
 * current device before returning. Streams passed in must belong to the
 * model's device.
 */
#ifndef BEAR_GB300_H
#define BEAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  BEAR_OK = 0,
  BEAR_ERR_INVALID_INPUT = 1, /* reference: InvalidInput (src/additional/exceptions.h:29-50) */
  BEAR_ERR_FILE = 2,          /* reference: FileNotFound */
  BEAR_ERR_CUDA = 3,          /* reference: gpuErrchk -> exit (src/CUDA_kernels/error_check.h:29-37) */
  BEAR_ERR_UNSUPPORTED = 4,   /* module outside the engine's scope */
  BEAR_ERR_STATE = 5,         /* call order (e.g. evaluation before finalize) */
  BEAR_ERR_SIZE = 6           /* argument sizes do not match the model */
};

typedef struct bear_model bear_model;

/* Message of the last failed call on this thread (never NULL). */
const char* bear_last_error(void);

/* --------------------------------------------------------------- set-up
 * Replaces the model construction of Retrieval::Retrieval(GlobalConfig*,
 * GenericConfig*, vector<ObservationInput>, vector<PriorConfig>)
 * (src/retrieval/retrieval.cpp:70-104): GlobalConfig + Emission/Transmission/
 * Occultation ModelConfig are given as line-based text ("key value ..." per line,
 * keys: forward_model (emission, transmission, secondary_eclipse), cross_section_path,
 * wavenumber_file, spectral_discretisation, spectral_resolution, error_inflation,
 * nb_grid_points, atmos_boundaries, temperature_profile, radiative_transfer,
 * chemistry, cloud, opacity, fit_mean_molecular_weight, fit_scale_height,
 * variable_gravity, stellar_spectrum (secondary eclipse: blackbody | file <path> |
 * grid <folder/>, src/forward_model/stellar_spectrum/select_stellar_model.h:52-122)). */
int bear_model_create(const char* config_text, int device, bear_model** out);

/* One ObservationInput (src/observations/observations.h:42-92,
 * Observation::init src/observations/observations.cpp:42-111).
 * type: "spectroscopy" (centers_or_edges = n wavelengths) or "photometry" /
 * "band-spectroscopy" (centers_or_edges = n x 2 bin edges). weight, fwhm may
 * be NULL; n_filter = 0 means no filter response. */
int bear_model_add_observation(bear_model* m, const char* name, const char* type, int n,
                               const double* centers_or_edges, const double* data,
                               const double* error, const double* weight, const double* fwhm,
                               int n_filter, const double* filter_wavelength,
                               const double* filter_response, const char* detector,
                               const char* modifier);

/* Builds the spectral grid (SpectralGrid::sampleSpectralGrid,
 * src/spectral_grid/spectral_grid.cpp:123-157), the observation operators
 * (src/spectral_grid/spectral_band*.cpp, src/observations/*), loads and
 * uploads the opacity tables (src/transport_coeff/opacity_species.cpp:44-156,
 * sampled_data.cpp:48-87) and the device constants. */
int bear_model_finalize(bear_model* m);

/* The host half of bear_model_finalize (grid, observation operators, tables)
 * without touching a GPU. bear_model_finalize calls it when needed. After it,
 * the size and set-up queries below work; evaluations need finalize. */
int bear_model_prepare(bear_model* m);

/* Set-up of observation k as integers: [obs_index_range.first, .second, n,
 * n pairs of band-edge indices (SpectralBands::edge_indices), then one pair of
 * convolution limits per point of the observation range
 * (SpectralBands::convolution_quadrature_intervals) when an instrument profile
 * is present]. Returns the number of values written through *written. */
int bear_model_observation_setup(const bear_model* m, int k, long long* out, int capacity,
                                 int* written);

/* Row r (internal order, observations concatenated) of the composite
 * observation operator: bin_r = sum_j weights[j] * spectrum[k0 + j], j < len.
 * *weights points into the model's host memory (valid until destroy). */
int bear_model_operator_row(const bear_model* m, int r, int* k0, int* len, const double** weights);

/* Sizes: spectral points N, total observation points M, physical parameters P
 * (ForwardModel::parametersNumber + 1 with error inflation), observations. */
int bear_model_info(const bear_model* m, int* nb_spectral_points, int* nb_obs_points,
                    int* nb_parameters, int* nb_observations);
/* SpectralGrid::wavenumber_list (src/spectral_grid/spectral_grid.h:41). */
int bear_model_wavenumbers(const bear_model* m, double* out);
/* Observation::nbPoints of observation k. */
int bear_model_observation_size(const bear_model* m, int k, int* n);
/* Bytes of device memory held by the model (tables, operators, work buffers;
 * tables shared with other models are counted in each). */
int bear_model_device_bytes(const bear_model* m, size_t* bytes);
/* Whether the model's device opacity tables were created by another model on the
 * same device (same table files, spectral grid and pressure grid) and are shared,
 * and their size. No reference counterpart. */
int bear_model_table_sharing(const bear_model* m, int* shared, size_t* table_bytes);
void bear_model_destroy(bear_model* m);

/* --------------------------------------------------------------- plain path
 * ForwardModel::calcModelGPU(params, spectrum_dev, spectrum_obs_dev)
 * (src/forward_model/forward_model.h:76-79; Emission
 * src/forward_model/emission/emission.cpp:234-265, Transmission
 * src/forward_model/transmission/transmission.cpp:257-321).
 * params: host, nb_params physical parameters. spectrum_dev: device, N
 * doubles (emission: W m^-2 um^-1 after the unit change; transmission: ppm),
 * or NULL. obs_dev: array (host memory) of nb_observations device pointers,
 * each receiving that observation's binned model in the reference's internal
 * (descending-wavelength) order, or NULL. neglect: host, set to the model's
 * neglect flag. Synchronises the stream before returning (the reference's
 * calcModelGPU is synchronous). */
int bear_forward(bear_model* m, const double* params, int nb_params, double* spectrum_dev,
                 double* const* obs_dev, int* neglect, void* stream);

/* ForwardModel::calcModel(params, return_high_res) (src/forward_model/
 * forward_model.cpp:60-127) with host outputs: spectrum (N, may be NULL) and
 * obs (M, concatenated, each observation in the caller's original order). */
int bear_compute_model(bear_model* m, const double* params, int nb_params, double* spectrum,
                       double* obs, int* neglect, void* stream);

/* Retrieval::computeLikelihood (src/retrieval/retrieval.cpp:295-310,
 * logLikelihoodGPU :374-421): host params, host log-likelihood (-1e30 when
 * the model is neglected). */
int bear_loglike(bear_model* m, const double* params, int nb_params, double* loglike,
                 void* stream);

/* --------------------------------------------------------------- batched path
 * No reference counterpart (the reference evaluates one point per MultiNest
 * callback, src/retrieval/multinest_loglike.cpp:152-186). params_dev: device,
 * batch x nb_params row-major; loglike_dev: device, batch; neglect_dev:
 * device, batch bytes (NULL allowed). Stream-ordered, no synchronisation. */
int bear_loglike_batch(bear_model* m, const double* params_dev, int batch, int nb_params,
                       double* loglike_dev, uint8_t* neglect_dev, void* stream);

/* Contribution functions of one parameter set (emission and secondary-eclipse models;
 * EmissionModel::postProcessContributionFunctions
 * src/forward_model/emission/emission_post_process.cpp:330-376, kernel
 * src/CUDA_kernels/contribution_function_kernels.cu:21-66): per level i the share
 * 2 pi B(T_i) (1 - exp(-dtau_i)) exp(-sum of dtau above) of the gas absorption layer
 * below it (level 0: 0). cf_spectrum (host, levels x spectral points) and cf_bins
 * (host, levels x observation points, each level in the order of bear_compute_model's
 * observations, binned by wavelength integration as the reference does) may be NULL.
 * Level 0 is the bottom of the atmosphere. Transmission models: BEAR_ERR_UNSUPPORTED. */
int bear_contribution_functions(bear_model* m, const double* params, int nb_params, double* cf_bins,
                                double* cf_spectrum, void* stream);

/* --------------------------------------------------------------- priors on the device
 * The reference converts MultiNest's hypercube coordinates to parameters on the host,
 * one point at a time (Retrieval::convertHypercubeParameters
 * src/retrieval/multinest_loglike.cpp:59-97, prior classes src/retrieval/prior_types.h:89-256).
 * Here a batch of live points stays in device memory: cube -> parameters -> log L.
 *
 * bear_model_set_priors: one prior per model parameter (n = the model's parameter
 * count, the error exponent included when error inflation is on), as the PriorConfig
 * list of Retrieval::Retrieval: type[i] 0 uniform (a, b = bounds), 1 log-uniform
 * (a, b = bounds > 0), 2 Gaussian (a = mean, b = standard deviation; erf_inv as the
 * reference), 3 delta (a = value), 4 linked (link[i] = the 0-based parameter whose
 * prior and cube coordinate it takes; never another linked one; the value is used
 * without a unit, as in the reference). unit[i]: the unit factor (NULL: all 1), e.g.
 * 7.1492e9 for "Rj" (src/retrieval/prior_types.h:57-82). a, b, link may be NULL
 * where no prior needs them.
 * bear_prior_transform_batch: cube (batch x nb_params, device, in [0, 1]) to physical
 * parameters (batch x nb_params, device).
 * bear_loglike_cube_batch: the transform, then bear_loglike_batch on the result
 * (params_dev receives the physical parameters). */
int bear_model_set_priors(bear_model* m, int n, const int* type, const double* a, const double* b,
                          const double* unit, const int* link);
int bear_prior_transform_batch(bear_model* m, const double* cube_dev, int batch, int nb_params,
                               double* params_dev, void* stream);
int bear_loglike_cube_batch(bear_model* m, const double* cube_dev, int batch, int nb_params, double* params_dev,
                            double* loglike_dev, uint8_t* neglect_dev, void* stream);

/* Gradient of the log-likelihood with respect to the physical parameters (the
 * reference's parameter vector: ratios for the temperature knots, linear mixing
 * ratios) by the engine's adjoint kernels, with the log-likelihood itself.
 * No reference counterpart (the reference has no derivatives). grad_dev:
 * device, batch x nb_params; loglike_dev: device, batch; neglect_dev: device,
 * batch bytes (NULL allowed). Neglected models get -1e30 and a zero gradient.
 * Discrete choices of the model (table brackets, cloud layer indices, the
 * transmission tau cut-off indices) are held fixed, so d/d cloud-top pressure
 * is 0. Emission, secondary-eclipse and transmission models (grey, power-law and
 * KH clouds, the H- continuum, variable gravity, A impact parameters per
 * layer); transmission, H- and non-grey cloud gradients run in precision mode 0
 * (else BEAR_ERR_UNSUPPORTED). Stream-ordered. Evaluations run in chunks whose work buffers fit the gradient
 * memory budget. */
int bear_loglike_grad_batch(bear_model* m, const double* params_dev, int batch, int nb_params,
                            double* loglike_dev, double* grad_dev, uint8_t* neglect_dev,
                            void* stream);

/* Optical depth at which a transmission tangent-ray sum stops (the reference's
 * tau > 10, src/forward_model/transmission/transmission_spectrum.cpp:136-137,
 * the default; INFINITY: no cut-off). The cut-off makes log L a step function of
 * the parameters wherever a ray's partial sum crosses it; gradient checks by
 * finite differences therefore use the smooth model without it. Applies to
 * later launches (not to graphs captured before). */
int bear_model_set_tau_cutoff(bear_model* m, double tau);

/* Device memory the gradient's work buffers may use per chunk of evaluations
 * (0 = default, 32 GiB). No reference counterpart. */
int bear_model_set_gradient_memory(bear_model* m, long long bytes);

/* --------------------------------------------------------------- autotuner and captured batches
 * No reference counterpart. bear_model_autotune times the radiative-transfer
 * kernel's launch shapes (emission: 64 / 128 / 256 threads per block;
 * transmission: 160, 176, 208, 192, 224, 32, 64, see bear_model_set_launch: wavenumbers
 * per block, levels per thread and species per table-read group) on this batch with CUDA events,
 * keeps the fastest for later batched calls (an explicit bear_model_set_launch
 * takes precedence) and reports it. Synchronous; results do not depend on the
 * choice (each wavenumber is computed by the same code). */
int bear_model_autotune(bear_model* m, const double* params_dev, int batch, int nb_params, void* stream,
                        int* rt_threads_out);

/* A captured batch: the batched kernel sequence (atmosphere, radiative transfer,
 * observation + likelihood) for fixed device buffers params_dev (batch x
 * nb_params), loglike_dev (batch) and neglect_dev (batch bytes, NULL allowed),
 * captured once into a CUDA graph. Write new parameters into params_dev, then
 * bear_batch_graph_launch replays the kernels on the given stream. The graph uses
 * the model's work buffers as they were at capture: a launch after they were
 * reallocated (a larger batch or gradient chunk on the same model) fails with
 * BEAR_ERR_STATE; precision and launch settings changed later do not affect it.
 * Destroy graphs before their model. */
typedef struct bear_batch_graph bear_batch_graph;
int bear_batch_graph_create(bear_model* m, const double* params_dev, int batch, int nb_params,
                            double* loglike_dev, uint8_t* neglect_dev, bear_batch_graph** out);
/* The same captured from the hypercube: prior transform (into params_dev) + forward. */
int bear_batch_graph_create_cube(bear_model* m, const double* cube_dev, int batch, int nb_params,
                                 double* params_dev, double* loglike_dev, uint8_t* neglect_dev,
                                 bear_batch_graph** out);
int bear_batch_graph_launch(bear_batch_graph* g, void* stream);
int bear_batch_graph_destroy(bear_batch_graph* g);

/* Arithmetic of the opacity assembly (applies to every evaluation path):
 * 0 (default) = double-float (hi + lo float pairs, ~48 bits) on the FP32 pipe
 * with table-driven exponentials; radiative-transfer recurrences, tangent-ray
 * sums and the likelihood stay FP64. 1 = every step in FP64 with the CUDA
 * math library (the validation path). */
int bear_model_set_precision(bear_model* m, int mode);

/* Launch shape of the radiative-transfer kernel (emission: threads =
 * wavenumbers per block, 64 / 128 / 256; transmission: 16 / 32 / 64 wavenumbers
 * per block with four threads each, or two wavenumbers per thread group: 160 (32
 * wavenumbers per block, eight threads per pair, two species per table-read group),
 * 176 (one species per group), 208 (four), 224 (four threads per pair: twice the
 * levels per thread), 192 (64 wavenumbers per block); any other value the default
 * 160; the FP64 path runs 32 in place of the paired shapes; 0 = default or the
 * autotuned shape) and
 * threads per block of the observation + likelihood kernel (0 = 256). An explicit
 * setting overrides bear_model_autotune. Every shape gives the same bits. */
int bear_model_set_launch(bear_model* m, int rt_threads, int obs_threads);

/* Allocation-free log-likelihood of one parameter set. No counterpart in the
 * reference. For host applications that cannot call cudaMalloc during the call:
 * those whose device memory belongs to another framework's pool or to a fixed
 * budget set at start-up, and per-point sampler callbacks that must not block in
 * the allocator. params_dev: device, nb_params doubles; loglike_dev: device,
 * 1 double (-1e30 when neglected); neglect_dev: device, 1 byte (NULL allowed).
 * The per-evaluation work buffers live in a fixed 2 MiB device array that every
 * GPU loading the library holds until exit; models needing more scratch than
 * that are rejected with BEAR_ERR_SIZE. The first call for a model's device
 * looks up the array's address with cudaGetSymbolAddress (with the model's
 * device current): make it before any stream capture. The address is kept for
 * the life of the process, so the entry point must not be used after
 * cudaDeviceReset. All calls on a device share the array: calls that may
 * overlap on the GPU race and must be serialised by the caller. Stream-ordered;
 * does not synchronise. */
int bear_loglike_noalloc(bear_model* m, const double* params_dev, int nb_params,
                         double* loglike_dev, uint8_t* neglect_dev, void* stream);

/* --------------------------------------------------------------- measurement
 * No reference counterpart. With profiling on, every evaluation call records
 * CUDA events around its three stages (atmosphere, radiative transfer,
 * observation operator + likelihood) on the launching stream;
 * bear_model_stage_times waits for the last call's events and returns the
 * three durations in milliseconds. */
int bear_model_set_profiling(bear_model* m, int on);
int bear_model_stage_times(bear_model* m, float* ms3);

/* Table layout and the number of distinct table rows referenced by the
 * stencils of the last `batch` evaluations (for algorithmic-byte accounting;
 * copies the stencils to the host and synchronises). */
int bear_model_table_info(const bear_model* m, int* levels, int* table_species,
                          int* rayleigh_species, long long* table_rows);
int bear_model_stencil_rows(bear_model* m, int batch, long long* distinct_rows);

#ifdef __cplusplus
}
#endif

#endif /* BEAR_GB300_H */
