// C ABI of the engine (include/bear_gb300.h): argument checking, error
// translation and the plain-path orchestration around the device kernels.

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bear_gb300.h"
#include "model.h"

struct bear_model {
  bgb::Model m;
};

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    f();
    return BEAR_OK;
  } catch (const bgb::Error& e) {
    return fail(e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(BEAR_ERR_INVALID_INPUT, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(BEAR_ERR_INVALID_INPUT, e.what());
  }
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw bgb::Error(BEAR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Makes the model's device current for the duration of a call and restores the
// caller's device afterwards, so a call made while another GPU is current still
// launches on the GPU that holds the model's buffers. cudaSetDevice is only
// called when the devices differ.
class DeviceScope {
 public:
  explicit DeviceScope(int device) {
    check_cuda(cudaGetDevice(&previous_), "cudaGetDevice");
    if (previous_ != device) {
      check_cuda(cudaSetDevice(device), "cudaSetDevice");
      switched_ = true;
    }
  }
  ~DeviceScope() {
    if (switched_) cudaSetDevice(previous_);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;

 private:
  int previous_ = 0;
  bool switched_ = false;
};

void require_ready(const bear_model* h) {
  if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
  if (!h->m.finalized) throw bgb::Error(BEAR_ERR_STATE, "model is not finalized");
}

void require_prepared(const bear_model* h) {
  if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
  if (!h->m.prepared) throw bgb::Error(BEAR_ERR_STATE, "model is not prepared");
}

void require_params(const bear_model* h, int nb_params) {
  if (nb_params != h->m.acfg.nparam_total)
    throw bgb::Error(BEAR_ERR_SIZE, "expected " + std::to_string(h->m.acfg.nparam_total) +
                                        " parameters, got " + std::to_string(nb_params));
}

// Stage host parameters into the workspace and run one evaluation.
void run_plain(bear_model* h, const double* params, int nb_params, cudaStream_t st) {
  bgb::Model& m = h->m;
  require_params(h, nb_params);
  if (!params) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null parameters");
  if ((size_t)nb_params * sizeof(double) > m.h_pinned_bytes)
    throw bgb::Error(BEAR_ERR_SIZE, "too many parameters for the staging buffer");
  bgb::ensure_workspace(m, 1);
  std::memcpy(m.h_pinned, params, nb_params * sizeof(double));
  check_cuda(cudaMemcpyAsync(m.ws.params, m.h_pinned, nb_params * sizeof(double), cudaMemcpyHostToDevice, st),
             "parameter upload");
  bgb::launch_forward(m, m.ws.params, 1, st, true, nullptr, m.ws.loglike);
}

}  // namespace

extern "C" {

const char* bear_last_error(void) { return g_last_error.c_str(); }

int bear_model_create(const char* config_text, int device, bear_model** out) {
  if (!out) return fail(BEAR_ERR_INVALID_INPUT, "null output handle");
  *out = nullptr;
  bear_model* h = new bear_model();
  int rc = guarded([&] {
    if (!config_text) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null config text");
    h->m.device = device;
    bgb::parse_config(h->m, config_text);
  });
  if (rc != BEAR_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return BEAR_OK;
}

int bear_model_add_observation(bear_model* h, const char* name, const char* type, int n,
                               const double* ce, const double* data, const double* error,
                               const double* weight, const double* fwhm, int n_filter,
                               const double* fwl, const double* fresp, const char* detector,
                               const char* modifier) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (!ce || !data || !error) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "observation arrays missing");
    if (n_filter > 0 && (!fwl || !fresp)) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "filter arrays missing");
    bgb::add_observation(h->m, name, type, n, ce, data, error, weight, fwhm, n_filter, fwl, fresp,
                         detector, modifier);
  });
}

int bear_model_prepare(bear_model* h) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (!h->m.prepared) {
      bgb::finalize_host(h->m);
      h->m.prepared = true;
    }
  });
}

int bear_model_finalize(bear_model* h) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (h->m.finalized) throw bgb::Error(BEAR_ERR_STATE, "model already finalized");
    const DeviceScope on_model_device(h->m.device);
    if (!h->m.prepared) {
      bgb::finalize_host(h->m);
      h->m.prepared = true;
    }
    bgb::upload_model(h->m);
    h->m.finalized = true;
  });
}

int bear_model_observation_setup(const bear_model* h, int k, long long* out, int cap, int* written) {
  return guarded([&] {
    require_prepared(h);
    const bgb::Model& m = h->m;
    if (k < 0 || k >= (int)m.obs.size()) throw bgb::Error(BEAR_ERR_SIZE, "observation index out of range");
    const bgb::ObservationSetup& o = m.obs[k];
    std::vector<long long> v{(long long)o.range_lo, (long long)o.range_hi, (long long)o.n};
    for (auto& e : o.edge_idx) { v.push_back((long long)e[0]); v.push_back((long long)e[1]); }
    if (o.has_profile)
      for (auto& c : o.conv) { v.push_back((long long)c[0]); v.push_back((long long)c[1]); }
    if ((int)v.size() > cap) throw bgb::Error(BEAR_ERR_SIZE, "capacity too small: need " + std::to_string(v.size()));
    std::copy(v.begin(), v.end(), out);
    *written = (int)v.size();
  });
}

int bear_model_operator_row(const bear_model* h, int r, int* k0, int* len, const double** weights) {
  return guarded([&] {
    require_prepared(h);
    const bgb::Model& m = h->m;
    if (r < 0 || r >= m.M) throw bgb::Error(BEAR_ERR_SIZE, "operator row out of range");
    for (const auto& o : m.obs) {
      if (r < o.out_offset + o.n) {
        const int j = r - o.out_offset;
        *k0 = o.row_k0[j];
        *len = o.row_len[j];
        *weights = m.W.data() + o.row_off[j];
        return;
      }
    }
  });
}

int bear_model_info(const bear_model* h, int* N, int* M, int* P, int* nobs) {
  return guarded([&] {
    require_prepared(h);
    if (N) *N = (int)h->m.N;
    if (M) *M = h->m.M;
    if (P) *P = h->m.acfg.nparam_total;
    if (nobs) *nobs = (int)h->m.obs.size();
  });
}

int bear_model_wavenumbers(const bear_model* h, double* out) {
  return guarded([&] {
    require_prepared(h);
    std::memcpy(out, h->m.nu.data(), h->m.N * sizeof(double));
  });
}

int bear_model_observation_size(const bear_model* h, int k, int* n) {
  return guarded([&] {
    require_prepared(h);
    if (k < 0 || k >= (int)h->m.obs.size()) throw bgb::Error(BEAR_ERR_SIZE, "observation index out of range");
    *n = h->m.obs[k].n;
  });
}

int bear_model_device_bytes(const bear_model* h, size_t* bytes) {
  return guarded([&] {
    require_ready(h);
    const bgb::Model& m = h->m;
    size_t ws = 0;
    if (m.ws.capacity) {
      const size_t B = m.ws.capacity, L = m.L, S = std::max(m.acfg.S, 1), N = m.N;
      ws = B * (L * sizeof(bgb::LevelInfo) + L * S * sizeof(bgb::LevelSpecies) + N * 8 + m.M * 8 + 64);
      if (m.transmission) ws += B * L * L * 8;
    }
    *bytes = m.device_bytes + ws;
  });
}

void bear_model_destroy(bear_model* h) {
  if (!h) return;
  if (h->m.finalized) {
    int previous = 0;
    const bool have_previous = cudaGetDevice(&previous) == cudaSuccess;
    bgb::release_model(h->m);
    if (have_previous) cudaSetDevice(previous);
  }
  delete h;
}

int bear_model_set_precision(bear_model* h, int mode) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (mode != 0 && mode != 1) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "precision mode must be 0 or 1");
    h->m.precision = mode;
  });
}

int bear_model_set_tau_cutoff(bear_model* h, double tau) {
  return guarded([&] {
    require_ready(h);
    if (!(tau > 0)) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "the cut-off must be positive (inf: none)");
    bgb::set_tau_cutoff(h->m, tau);
  });
}

int bear_model_set_gradient_memory(bear_model* h, long long bytes) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (bytes < 0) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "bytes must be non-negative");
    h->m.grad_budget = bytes ? (size_t)bytes : (size_t(32) << 30);
  });
}

int bear_model_set_launch(bear_model* h, int rt_threads, int obs_threads) {
  return guarded([&] {
    if (!h) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null model");
    if (rt_threads < 0 || rt_threads > 256 || rt_threads % 16) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "rt_threads must be a multiple of 16 up to 256");
    if (obs_threads < 0 || obs_threads > 1024 || obs_threads % 32) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "obs_threads must be a multiple of 32 up to 1024");
    h->m.rt_threads = rt_threads;
    h->m.obs_threads = obs_threads;
  });
}

int bear_model_set_profiling(bear_model* h, int on) {
  return guarded([&] {
    require_ready(h);
    h->m.profiling = on != 0;
    h->m.ev_recorded = false;
  });
}

int bear_model_stage_times(bear_model* h, float* ms3) {
  return guarded([&] {
    require_ready(h);
    if (!ms3) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null output");
    bgb::stage_times(h->m, ms3);
  });
}

int bear_model_table_sharing(const bear_model* h, int* shared, size_t* table_bytes) {
  return guarded([&] {
    require_ready(h);
    if (shared) *shared = h->m.tables_shared ? 1 : 0;
    if (table_bytes) *table_bytes = bgb::table_bytes(h->m);
  });
}

int bear_model_table_info(const bear_model* h, int* levels, int* table_species, int* rayleigh_species,
                          long long* table_rows) {
  return guarded([&] {
    require_prepared(h);
    if (levels) *levels = h->m.L;
    if (table_species) *table_species = h->m.acfg.S;
    if (rayleigh_species) *rayleigh_species = h->m.acfg.R_ray;
    if (table_rows) *table_rows = h->m.n_rows;
  });
}

int bear_model_stencil_rows(bear_model* h, int batch, long long* rows) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    if (!rows) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null output");
    *rows = bgb::stencil_rows(h->m, batch);
  });
}

int bear_forward(bear_model* h, const double* params, int nb_params, double* spectrum_dev,
                 double* const* obs_dev, int* neglect, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    bgb::Model& m = h->m;
    cudaStream_t st = (cudaStream_t)stream;
    run_plain(h, params, nb_params, st);
    if (spectrum_dev) bgb::launch_spectrum_output(m, spectrum_dev, st);
    if (obs_dev) {
      for (size_t o = 0; o < m.obs.size(); ++o) {
        if (!obs_dev[o]) continue;
        check_cuda(cudaMemcpyAsync(obs_dev[o], m.ws.obs + m.obs[o].out_offset, m.obs[o].n * sizeof(double),
                                   cudaMemcpyDeviceToDevice, st), "observation output");
      }
    }
    bgb::EvalInfo ev;
    check_cuda(cudaMemcpyAsync(&ev, m.ws.ev, sizeof ev, cudaMemcpyDeviceToHost, st), "neglect flag");
    check_cuda(cudaStreamSynchronize(st), "forward model");
    if (neglect) *neglect = ev.neglect;
  });
}

int bear_compute_model(bear_model* h, const double* params, int nb_params, double* spectrum,
                       double* obs, int* neglect, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    bgb::Model& m = h->m;
    cudaStream_t st = (cudaStream_t)stream;
    run_plain(h, params, nb_params, st);
    std::vector<double> internal(std::max(m.M, 1));
    if (spectrum) {
      bgb::launch_spectrum_output(m, m.ws.spectrum + 0, st);  // in place: plain path owns row 0
      check_cuda(cudaMemcpyAsync(spectrum, m.ws.spectrum, m.N * sizeof(double), cudaMemcpyDeviceToHost, st),
                 "spectrum download");
    }
    check_cuda(cudaMemcpyAsync(internal.data(), m.ws.obs, m.M * sizeof(double), cudaMemcpyDeviceToHost, st),
               "observation download");
    bgb::EvalInfo ev;
    check_cuda(cudaMemcpyAsync(&ev, m.ws.ev, sizeof ev, cudaMemcpyDeviceToHost, st), "neglect flag");
    check_cuda(cudaStreamSynchronize(st), "compute model");
    if (obs) {
      // ForwardModel::calcModel reverses observations given in ascending wavelength order
      // (src/forward_model/forward_model.cpp:119-123)
      for (const auto& o : m.obs)
        for (int j = 0; j < o.n; ++j)
          obs[o.out_offset + (o.ascending ? o.n - 1 - j : j)] = internal[o.out_offset + j];
    }
    if (neglect) *neglect = ev.neglect;
  });
}

int bear_loglike(bear_model* h, const double* params, int nb_params, double* loglike, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    bgb::Model& m = h->m;
    cudaStream_t st = (cudaStream_t)stream;
    run_plain(h, params, nb_params, st);
    check_cuda(cudaMemcpyAsync(m.h_pinned, m.ws.loglike, sizeof(double), cudaMemcpyDeviceToHost, st),
               "log-likelihood download");
    check_cuda(cudaStreamSynchronize(st), "log-likelihood");
    *loglike = m.h_pinned[0];
  });
}

int bear_loglike_batch(bear_model* h, const double* params_dev, int batch, int nb_params,
                       double* loglike_dev, uint8_t* neglect_dev, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!params_dev || !loglike_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    bgb::launch_forward(h->m, params_dev, batch, (cudaStream_t)stream, true, neglect_dev, loglike_dev);
  });
}

int bear_loglike_noalloc(bear_model* h, const double* params_dev, int nb_params, double* loglike_dev,
                         uint8_t* neglect_dev, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (!params_dev || !loglike_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    bgb::loglike_noalloc(h->m, params_dev, loglike_dev, neglect_dev, (cudaStream_t)stream);
  });
}

int bear_contribution_functions(bear_model* h, const double* params, int nb_params, double* cf_bins,
                                double* cf_spectrum, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    if (h->m.transmission)
      throw bgb::Error(BEAR_ERR_UNSUPPORTED, "contribution functions exist for emission and secondary-eclipse models");
    const cudaStream_t st = (cudaStream_t)stream;
    run_plain(h, params, nb_params, st);
    bgb::contribution_functions(h->m, st, cf_spectrum, cf_bins);
  });
}

int bear_model_set_priors(bear_model* h, int n, const int* type, const double* a, const double* b,
                          const double* unit, const int* link) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    if (n < 0 || (n > 0 && !type)) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null prior table");
    bgb::set_priors(h->m, n, type, a, b, unit, link);
  });
}

int bear_prior_transform_batch(bear_model* h, const double* cube_dev, int batch, int nb_params,
                               double* params_dev, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!cube_dev || !params_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    bgb::launch_prior_transform(h->m, cube_dev, batch, params_dev, (cudaStream_t)stream);
  });
}

int bear_loglike_cube_batch(bear_model* h, const double* cube_dev, int batch, int nb_params, double* params_dev,
                            double* loglike_dev, uint8_t* neglect_dev, void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!cube_dev || !params_dev || !loglike_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    const cudaStream_t st = (cudaStream_t)stream;
    bgb::launch_prior_transform(h->m, cube_dev, batch, params_dev, st);
    bgb::launch_forward(h->m, params_dev, batch, st, true, neglect_dev, loglike_dev);
  });
}

int bear_loglike_grad_batch(bear_model* h, const double* params_dev, int batch, int nb_params,
                            double* loglike_dev, double* grad_dev, uint8_t* neglect_dev,
                            void* stream) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!params_dev || !loglike_dev || !grad_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    bgb::launch_gradient(h->m, params_dev, batch, (cudaStream_t)stream, loglike_dev, grad_dev, neglect_dev);
  });
}

}  // extern "C"

// ------------------------------------------------------------------ autotuner and captured batches
// Not in the reference (it evaluates one point per call). The autotuner times the
// radiative-transfer kernel's launch shapes on the caller's batch with CUDA events
// and keeps the fastest for batched calls; the batch graph captures the batched
// kernel sequence once and replays it.

struct bear_batch_graph {
  bear_model* h = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned generation = 0;
};

extern "C" {

int bear_model_autotune(bear_model* h, const double* params_dev, int batch, int nb_params, void* stream,
                        int* rt_threads_out) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 2) throw bgb::Error(BEAR_ERR_SIZE, "autotuning needs a batch of at least 2");
    if (!params_dev) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null device buffer");
    bgb::Model& m = h->m;
    const cudaStream_t st = (cudaStream_t)stream;
    // emission: threads (wavenumbers) per block; transmission: wavenumbers per block
    const std::vector<int> cand = !m.transmission ? std::vector<int>{64, 128, 256}
                                  : m.annuli > 1  ? std::vector<int>{32, 16, 64}
                                                  : std::vector<int>{160, 176, 208, 192, 224, 32, 64};
    const int saved_rt = m.rt_threads;
    const bool saved_prof = m.profiling;
    m.rt_threads = 0;
    m.profiling = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int best = 0;
    float best_ms = 0.0f;
    try {
      check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
      check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
      for (int c : cand) {
        m.tuned_rt = c;
        bgb::launch_forward(m, params_dev, batch, st, true, nullptr, nullptr);  // warm-up
        check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");
        for (int r = 0; r < 3; ++r) bgb::launch_forward(m, params_dev, batch, st, true, nullptr, nullptr);
        check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        if (best == 0 || ms < best_ms) {
          best = c;
          best_ms = ms;
        }
      }
    } catch (...) {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      m.rt_threads = saved_rt;
      m.profiling = saved_prof;
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m.tuned_rt = best;
    m.rt_threads = saved_rt;
    m.profiling = saved_prof;
    if (rt_threads_out) *rt_threads_out = best;
  });
}

}  // extern "C"

namespace {

// Captures launch(stream) for a batch of the model into a graph (every allocation
// happens before the capture).
template <class F>
void capture_batch(bear_model* h, int batch, bear_batch_graph** out, F&& launch) {
  bgb::Model& m = h->m;
  check_cuda(cudaSetDevice(m.device), "cudaSetDevice");
  bgb::ensure_workspace(m, batch);  // every allocation happens before the capture
  const bool saved_prof = m.profiling;
  m.profiling = false;
  cudaStream_t s = nullptr;
  check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    cudaStreamDestroy(s);
    m.profiling = saved_prof;
    check_cuda(ce, "cudaStreamBeginCapture");
  }
  try {
    launch(s);
  } catch (...) {
    cudaStreamEndCapture(s, &graph);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(s);
    m.profiling = saved_prof;
    throw;
  }
  m.profiling = saved_prof;
  ce = cudaStreamEndCapture(s, &graph);
  cudaStreamDestroy(s);
  check_cuda(ce, "cudaStreamEndCapture");
  auto* g = new bear_batch_graph;
  g->h = h;
  g->graph = graph;
  g->generation = m.ws_generation;
  ce = cudaGraphInstantiate(&g->exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    delete g;
    check_cuda(ce, "cudaGraphInstantiate");
  }
  *out = g;
}

}  // namespace

extern "C" {

int bear_batch_graph_create(bear_model* h, const double* params_dev, int batch, int nb_params,
                            double* loglike_dev, uint8_t* neglect_dev, bear_batch_graph** out) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!params_dev || !loglike_dev || !out) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null buffer");
    capture_batch(h, batch, out, [&](cudaStream_t s) {
      bgb::launch_forward(h->m, params_dev, batch, s, true, neglect_dev, loglike_dev);
    });
  });
}

int bear_batch_graph_create_cube(bear_model* h, const double* cube_dev, int batch, int nb_params,
                                 double* params_dev, double* loglike_dev, uint8_t* neglect_dev,
                                 bear_batch_graph** out) {
  return guarded([&] {
    require_ready(h);
    const DeviceScope on_model_device(h->m.device);
    require_params(h, nb_params);
    if (batch < 1) throw bgb::Error(BEAR_ERR_SIZE, "batch must be positive");
    if (!cube_dev || !params_dev || !loglike_dev || !out) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null buffer");
    if (h->m.n_priors != h->m.acfg.nparam_total) throw bgb::Error(BEAR_ERR_STATE, "no priors set (bear_model_set_priors)");
    capture_batch(h, batch, out, [&](cudaStream_t s) {
      bgb::launch_prior_transform(h->m, cube_dev, batch, params_dev, s);
      bgb::launch_forward(h->m, params_dev, batch, s, true, neglect_dev, loglike_dev);
    });
  });
}

int bear_batch_graph_launch(bear_batch_graph* g, void* stream) {
  return guarded([&] {
    if (!g || !g->exec) throw bgb::Error(BEAR_ERR_INVALID_INPUT, "null graph");
    if (g->generation != g->h->m.ws_generation)
      throw bgb::Error(BEAR_ERR_STATE, "the model's work buffers were reallocated after the capture; recreate the graph");
    const DeviceScope on_model_device(g->h->m.device);
    check_cuda(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "cudaGraphLaunch");
  });
}

int bear_batch_graph_destroy(bear_batch_graph* g) {
  return guarded([&] {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
  });
}

}  // extern "C"
