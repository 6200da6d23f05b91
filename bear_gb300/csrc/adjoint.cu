// Adjoint (reverse-mode) gradient of the log-likelihood.
#include "../../include/bear_gb300.h"
#include "model.h"

namespace bgb {

void launch_gradient(Model& m, const double* params_dev, int batch, cudaStream_t st,
                     double* loglike_dev, double* grad_dev, uint8_t* neglect_dev) {
  (void)m; (void)params_dev; (void)batch; (void)st; (void)loglike_dev; (void)grad_dev; (void)neglect_dev;
  throw Error(BEAR_ERR_UNSUPPORTED, "gradient not available");
}

}  // namespace bgb
