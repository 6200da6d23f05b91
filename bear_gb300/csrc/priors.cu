// Prior transform on the device: unit-hypercube coordinates of a batch of live
// points to the physical parameter vector the likelihood takes, so that a batched
// sampler keeps its live points in HBM (cube -> parameters -> log L with no host
// round trip).
//
// Reference: Retrieval::convertHypercubeParameters src/retrieval/multinest_loglike.cpp:59-97
// with the prior classes of src/retrieval/prior_types.h:89-256 and the linked-prior
// set-up of Priors::setupLinkedPriors src/retrieval/priors.cpp:246-280:
//   uniform      lo + u (hi - lo)                         (bounds swapped if reversed)
//   log-uniform  10^(log10 lo + u (log10 hi - log10 lo))
//   gaussian     mu + sigma sqrt(2) erfinv(2 u - 1)       (the reference: boost::math::erf_inv)
//   delta        value
//   linked       the linked prior's value at the linked parameter's cube coordinate
// each times the prior's unit factor. A linked prior carries no unit of its own and
// BasicPrior::parameterPhysicalValue multiplies by the linked prior object's unit
// (1), so a linked parameter's physical value is its linked prior's value without
// the unit, as in the reference.

#include <cmath>
#include <string>
#include <vector>

#include "../../include/bear_gb300.h"
#include "model.h"

namespace bgb {

__global__ void prior_transform_kernel(const DevicePrior* __restrict__ pr, int P, const double* __restrict__ cube,
                                       long long n, double* __restrict__ params) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long b = i / P;
  const int j = (int)(i - b * P);
  const DevicePrior p = pr[j];
  const bool linked = p.type == kPriorLinked;
  const DevicePrior q = linked ? pr[p.link] : p;
  const double u = cube[b * P + (linked ? p.link : j)];
  double v;
  switch (q.type) {
    case kPriorUniform: v = q.a + u * (q.b - q.a); break;
    case kPriorLogUniform: v = pow(10.0, q.a + u * (q.b - q.a)); break;
    case kPriorGaussian: v = q.a + q.b * sqrt(2.0) * erfinv(2. * u - 1.); break;
    default: v = q.a; break;  // delta
  }
  params[i] = linked ? v : v * p.unit;
}

// Priors::addSingle / setupLinkedPriors src/retrieval/priors.cpp:101-280: parameter
// counts per type, bounds ordered, log10 of the log-uniform bounds, links 1-based in
// the reference's config (here 0-based) and never to another linked prior.
void set_priors(Model& m, int n, const int* type, const double* a, const double* b, const double* unit,
                const int* link) {
  if (n != m.acfg.nparam_total)
    throw Error(BEAR_ERR_SIZE, "Found " + std::to_string(n) + " priors config but expected " +
                                   std::to_string(m.acfg.nparam_total));
  std::vector<DevicePrior> v((size_t)n);
  for (int i = 0; i < n; ++i) {
    DevicePrior& p = v[i];
    p.type = type[i];
    p.link = -1;
    p.unit = unit ? unit[i] : 1.0;
    p.a = a ? a[i] : 0.0;
    p.b = b ? b[i] : 0.0;
    switch (p.type) {
      case kPriorUniform:
        if (p.b < p.a) std::swap(p.a, p.b);
        break;
      case kPriorLogUniform:
        if (!(p.a > 0.0) || !(p.b > 0.0)) throw Error(BEAR_ERR_INVALID_INPUT, "log-uniform prior bounds must be positive");
        p.a = std::log10(p.a);
        p.b = std::log10(p.b);
        if (p.b < p.a) std::swap(p.a, p.b);
        break;
      case kPriorGaussian:
      case kPriorDelta:
        break;
      case kPriorLinked:
        if (!link || link[i] < 0 || link[i] >= n)
          throw Error(BEAR_ERR_INVALID_INPUT, "Linked prior " + std::to_string(i) + " wrong index for link!");
        if (type[link[i]] == kPriorLinked)
          throw Error(BEAR_ERR_INVALID_INPUT, "Linked prior " + std::to_string(i) +
                                                  " Can not link prior to another linked prior!");
        p.link = link[i];
        break;
      default:
        throw Error(BEAR_ERR_INVALID_INPUT, "Prior type " + std::to_string(p.type) + " unknown!");
    }
  }
  BGB_CUDA(cudaSetDevice(m.device));
  if (!m.d_priors) {
    BGB_CUDA(cudaMalloc(&m.d_priors, (size_t)kMaxPriors * sizeof(DevicePrior)));
    m.allocations.push_back(m.d_priors);
  }
  if (n > kMaxPriors) throw Error(BEAR_ERR_UNSUPPORTED, "too many parameters for the device prior table");
  BGB_CUDA(cudaMemcpy(m.d_priors, v.data(), (size_t)n * sizeof(DevicePrior), cudaMemcpyHostToDevice));
  m.n_priors = n;
}

void launch_prior_transform(Model& m, const double* cube_dev, int batch, double* params_dev, cudaStream_t st) {
  if (m.n_priors != m.acfg.nparam_total) throw Error(BEAR_ERR_STATE, "no priors set (bear_model_set_priors)");
  const long long n = (long long)batch * m.n_priors;
  if (n == 0) return;
  prior_transform_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(m.d_priors, m.n_priors, cube_dev, n, params_dev);
  BGB_CUDA(cudaGetLastError());
}

}  // namespace bgb
