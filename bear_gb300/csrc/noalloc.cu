// Single-evaluation log-likelihood that allocates no memory at call time.
//
// Who needs this: host applications that cannot call cudaMalloc while they run.
// Some own all device memory through another framework's pool or a fixed budget
// set at start-up, so an allocation made behind their back either fails or
// breaks their accounting; others call the likelihood from a real-time callback
// (for example a sampler's per-point likelihood hook) that must not block on the
// allocator. The regular entry points grow a per-model workspace with cudaMalloc
// the first time a batch size is seen; this one instead keeps the per-evaluation
// work buffers (level and stencil records, the high-resolution spectrum, the
// binned spectrum, the transmission path lengths) in one fixed array in device
// memory declared below.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds kNoAllocScratchBytes of it until the process exits, whether or
// not this entry point is used. Host code cannot use the array's name as a
// device address; its address is looked up with cudaGetSymbolAddress once per
// device, with that device current, on the first call made for a model on that
// device. Make that first call before any stream capture starts. The address is
// kept for the life of the process: after cudaDeviceReset it is stale, and this
// entry point must not be called again in that process.
//
// Every call on a device shares the same array, and each call overwrites what
// the previous one left there: every element a call reads is written earlier in
// the same call, so nothing needs clearing. Calls whose executions can overlap
// on the GPU (different streams without ordering between them, or different
// models on the same device) race on the array and must be serialised by the
// caller.

#include <mutex>
#include <string>

#include "../../include/bear_gb300.h"
#include "model.h"

namespace bgb {

constexpr size_t kNoAllocScratchBytes = size_t(2) << 20;  // 2 MiB per device

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

void launch_forward_into(Model& m, const double* params_dev, const Workspace& w, cudaStream_t st,
                         uint8_t* neglect_dev, double* loglike_dev);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Carves the single-evaluation work buffers out of the scratch array; returns
// the bytes needed (and fills w when base is not null).
size_t layout(const Model& m, unsigned char* base, Workspace* w) {
  const size_t L = m.L, S = std::max(m.acfg.S, 1), R = std::max(m.acfg.R, 1);
  const size_t N = m.N, M = std::max(m.M, 1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align256(off + bytes);
    return base ? base + at : nullptr;
  };
  unsigned char* lev = take(L * sizeof(LevelInfo));
  unsigned char* ls = take(L * S * sizeof(LevelSpecies));
  unsigned char* lsdf = take(L * S * sizeof(LevelSpeciesDF));
  unsigned char* rn = take(L * R * sizeof(double));
  unsigned char* ev = take(sizeof(EvalInfo));
  unsigned char* spec = take(N * sizeof(double));
  unsigned char* obs = take(M * sizeof(double));
  const size_t K = m.transmission ? (size_t)transmission_rays(m) : 0;
  unsigned char* geom = m.transmission ? take(std::max(K, L) * L * sizeof(double)) : nullptr;
  unsigned char* rays = m.transmission ? take(2 * (K + 1) * sizeof(double)) : nullptr;
  if (base) {
    *w = Workspace{};
    w->capacity = 1;
    w->lev = reinterpret_cast<LevelInfo*>(lev);
    w->ls = reinterpret_cast<LevelSpecies*>(ls);
    w->lsdf = reinterpret_cast<LevelSpeciesDF*>(lsdf);
    w->ray_n = reinterpret_cast<double*>(rn);
    w->ev = reinterpret_cast<EvalInfo*>(ev);
    w->spectrum = reinterpret_cast<double*>(spec);
    w->obs = reinterpret_cast<double*>(obs);
    w->geom = reinterpret_cast<double*>(geom);
    w->rays = reinterpret_cast<double*>(rays);
  }
  return off;
}

// Address of the scratch array on `device`, which the caller has made current
// (the C ABI switches to the model's device for the whole call).
unsigned char* scratch_for_device(int device) {
  if (device < 0 || device >= kMaxDevices) throw Error(BEAR_ERR_INVALID_INPUT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[device]) {
    int current = -1;
    cudaError_t e = cudaGetDevice(&current);
    if (e != cudaSuccess) throw Error(BEAR_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (current != device) throw Error(BEAR_ERR_STATE, "the model's device is not current");
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      throw Error(BEAR_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[device] = ptr;
  }
  return static_cast<unsigned char*>(g_scratch_addr[device]);
}

}  // namespace

void loglike_noalloc(Model& m, const double* params_dev, double* loglike_dev, uint8_t* neglect_dev,
                     cudaStream_t st) {
  const size_t need = layout(m, nullptr, nullptr);
  if (need > kNoAllocScratchBytes)
    throw Error(BEAR_ERR_SIZE, "this model needs " + std::to_string(need) +
                                   " bytes of per-evaluation scratch; the allocation-free entry point is limited to " +
                                   std::to_string(kNoAllocScratchBytes) + " bytes");
  unsigned char* base = scratch_for_device(m.device);
  Workspace w;
  layout(m, base, &w);
  launch_forward_into(m, params_dev, w, st, neglect_dev, loglike_dev);
}

}  // namespace bgb
