// v2c_newton.h -- state of the per-marker VEP+RSF Newton and its network.
#pragma once
#include <cuda_runtime.h>

#include "v2c_internal.cuh"

namespace v2c {

struct NewtonState {
  float *d_mlp = nullptr;  // packed network parameters (V2C_MLP_NPARAM)
  int have_mlp = 0;
  long cap = 0;
  float *d_guess = nullptr;  // network outputs [2][guess_cap] for v2c_rsf_newton
  long guess_cap = 0;
};

cudaError_t newton_init(NewtonState &s, long cap);
void newton_free(NewtonState &s);

}  // namespace v2c

struct v2c_ctx;
v2c::NewtonState *v2c_ctx_newton(v2c_ctx *ctx);
cudaStream_t v2c_ctx_stream(v2c_ctx *ctx);
unsigned long long *v2c_ctx_stat(v2c_ctx *ctx);
const v2c_params *v2c_ctx_params(v2c_ctx *ctx);
void v2c_ctx_prof_begin(v2c_ctx *ctx, int group, cudaEvent_t *a);
void v2c_ctx_prof_end(v2c_ctx *ctx, int group, cudaEvent_t a);
void v2c_ctx_count_launches(v2c_ctx *ctx, long k);
