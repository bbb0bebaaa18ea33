// v2c_newton.cu -- per-marker visco-elasto-plastic + RSF Newton and the
// network that proposes its initial guess.
#include "v2c_newton.h"

namespace v2c {

cudaError_t newton_init(NewtonState &s, long cap) {
  s.cap = cap;
  return cudaMalloc((void **)&s.d_mlp, sizeof(float) * V2C_MLP_NPARAM);
}

void newton_free(NewtonState &s) {
  if (s.d_mlp) cudaFree(s.d_mlp);
  s.d_mlp = nullptr;
}

}  // namespace v2c

extern "C" int v2c_rsf_newton(v2c_ctx *ctx, const double *states_dev, long n, int guess,
                              double *out_dev, int32_t *iters_dev) {
  (void)ctx; (void)states_dev; (void)n; (void)guess; (void)out_dev; (void)iters_dev;
  return V2C_ERR_UNSUPPORTED;
}
extern "C" int v2c_mlp_load(v2c_ctx *ctx, const float *params_host) {
  (void)ctx; (void)params_host;
  return V2C_ERR_UNSUPPORTED;
}
extern "C" int v2c_mlp_save(v2c_ctx *ctx, float *params_host) {
  (void)ctx; (void)params_host;
  return V2C_ERR_UNSUPPORTED;
}
extern "C" int v2c_mlp_train(v2c_ctx *ctx, const double *states_dev, const double *targets_dev,
                             long n, int epochs, int batch, float lr, uint64_t seed,
                             float *final_loss) {
  (void)ctx; (void)states_dev; (void)targets_dev; (void)n; (void)epochs; (void)batch; (void)lr;
  (void)seed; (void)final_loss;
  return V2C_ERR_UNSUPPORTED;
}
