// v2c_newton.cu -- the per-marker VEP+RSF Newton on state arrays, and the
// network that proposes its start: inference, feature statistics, training
// (forward + backward on the tensor cores, deterministic gradient reduction,
// Adam).  No counterpart in the reference.
//
// Training.  One CTA of 128 threads takes 128 samples (32 per warp).  Each
// warp runs the forward pass and the backward pass through the layers with
// mma.sync (BF16 operands, FP32 accumulate), keeping activations in
// registers, and writes its activations and pre-activation gradients to
// shared memory (BF16).  The CTA then forms the weight gradients as GEMMs
// over its 128 samples (again mma.sync) and writes one partial gradient per
// CTA; a second kernel sums the partials in CTA order (no atomics, so the
// result does not depend on scheduling) and applies Adam to the FP32 master
// weights.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "v2c_mlp.cuh"
#include "v2c_newton.h"
#include "v2c_rsf.cuh"

namespace v2c {

cudaError_t newton_init(NewtonState &s, long cap) {
  s.cap = cap;
  cudaError_t e = cudaMalloc((void **)&s.d_mlp, sizeof(float) * V2C_MLP_NPARAM);
  if (e != cudaSuccess) return e;
  return cudaMemset(s.d_mlp, 0, sizeof(float) * V2C_MLP_NPARAM);
}

void newton_free(NewtonState &s) {
  if (s.d_mlp) cudaFree(s.d_mlp);
  if (s.d_guess) cudaFree(s.d_guess);
  s.d_mlp = nullptr;
  s.d_guess = nullptr;
  s.guess_cap = 0;
}

namespace {

constexpr int NT = 128;  // threads per CTA (4 warps)
constexpr int NG = MLP_OXM;  // trainable parameters (W1 b1 W2 b2 W3 b3)

__device__ __forceinline__ void warp_add(unsigned long long *p, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(V2C_FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(p, v);
}
// largest value over the warp, one atomic per warp (non-negative doubles
// order like their bit patterns)
__device__ __forceinline__ void warp_max_bits(unsigned long long *p, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_down_sync(V2C_FULL, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0 && v) atomicMax(p, v);
}

// state column k of sample i (column-major [V2C_RS_N][n])
__device__ __forceinline__ double st_at(const double *S, long n, int k, long i) {
  return S[(long)k * n + i];
}

__device__ __forceinline__ void state_of(const double *S, long n, long i, double W, RsfIn &in,
                                         double &vold) {
  vold = st_at(S, n, V2C_RS_VOLD, i);
  in.a = ff_from_double(st_at(S, n, V2C_RS_A, i));
  in.b = ff_from_double(st_at(S, n, V2C_RS_B, i));
  in.L = ff_from_double(st_at(S, n, V2C_RS_L, i));
  in.V0 = ff_from_double(st_at(S, n, V2C_RS_V0, i));
  in.mu0 = ff_from_double(st_at(S, n, V2C_RS_MU0, i));
  in.sn = ff_from_double(st_at(S, n, V2C_RS_SN, i));
  in.dt = ff_from_double(st_at(S, n, V2C_RS_DT, i));
  in.phio = ff_from_double(st_at(S, n, V2C_RS_PHIOLD, i));
  in.tau_old = ff_from_double(st_at(S, n, V2C_RS_TAUOLD, i));
  in.edot = ff_from_double(st_at(S, n, V2C_RS_EDOT, i));
  in.eta = ff_from_double(st_at(S, n, V2C_RS_ETA, i));
  in.G = ff_from_double(st_at(S, n, V2C_RS_G, i));
  in.W = ff_from_double(W);
}

// ---------------------------------------------------------- solve states
// one instantiation per (arithmetic, start) pair; the learned start comes
// from the network's outputs guess[i] (k_infer), so this kernel keeps the
// plain start's occupancy
template <bool FP64, bool LEARNED>
__global__ void __launch_bounds__(NT, 4) k_solve_states(const double *S, long n, double W,
                                                        const float *guess, double rtol, int maxit,
                                                        double *out, int32_t *iters,
                                                        unsigned long long *stat) {
  const bool learned = LEARNED;
  const bool fp64 = FP64;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (NT / 32);
  for (long base = ((long)blockIdx.x * (NT / 32) + wl) * 32; base < n; base += nwarps * 32) {
    const long i = base + lane;
    const bool valid = i < n;
    RsfIn in;
    double vold = 1e-9;
    if (valid) state_of(S, n, i, W, in, vold);
    const float u_plain = (vold > 0) ? logf((float)vold) : -30.f;
    // split form: states whose load is certainly below the floor's yield
    // are done with one FP32 evaluation
    bool at_floor = false;
    float A_floor = 0.f;
    if (valid && !fp64) at_floor = rsf_floor_certain(rsf32_of(in), A_floor);
    const float u0 = (learned && valid) ? guess[i] : u_plain;
    unsigned long long it = 0, fb = 0, nc = 0, resbits = 0;
    if (valid) {
      // the FP64 form starts from the FP64 log of the previous slip rate
      const double u_plain64 = (fp64 && vold > 0) ? log(vold) : (double)u_plain;
      RsfResult r = at_floor ? rsf_floor_result(in, A_floor)
                  : fp64     ? rsf_solve64(in, learned ? (double)u0 : u_plain64, rtol, maxit)
                             : rsf_solve_split(in, rsf32_of(in), u0, rtol, maxit);
      it = r.it32 + r.itff + r.it64;
      if (!r.ok && learned && u0 != u_plain) {
        RsfResult r2 = fp64 ? rsf_solve64(in, u_plain64, rtol, maxit)
                            : rsf_solve_split(in, rsf32_of(in), u_plain, rtol, maxit);
        it += r2.it32 + r2.itff + r2.it64;
        fb = 1;
        r = r2;
      }
      if (!r.ok) nc = 1;
      out[(long)V2C_RO_V * n + i] = r.V;
      out[(long)V2C_RO_PHI * n + i] = r.phi;
      // tau_y = sn a A + 4.3303e6 V at the solution (calc_RSF.c:128), FP64
      out[(long)V2C_RO_TAU * n + i] =
          ff_to_double(in.sn) * ff_to_double(in.a) * r.A + RSF_ETA_RAD * r.V;
      out[(long)V2C_RO_RES * n + i] = r.res;
      if (iters) iters[i] = r.ok ? (int32_t)it : -(int32_t)it;
      if (r.res > 0) resbits = (unsigned long long)__double_as_longlong(r.res);
    }
    warp_max_bits(stat + ST_NEWTON_MAXRES_BITS, resbits);
    warp_add(stat + ST_NEWTON_ITERS, it);
    warp_add(stat + ST_NEWTON_FALLBACK, fb);
    warp_add(stat + ST_NEWTON_NONCONV, nc);
  }
}

// The learned start of every state (the k_guess rule of the MIC step):
// the plain start where its FP32 residual ratio is below RSF_NET_MIN_RES,
// else the better of it and the network's proposal, the network evaluated
// by a warp only when one of its states needs it.
__global__ void __launch_bounds__(NT) k_learned_start(const double *S, long n, double W,
                                                      const float *mlp, float *u0_out) {
  __shared__ MlpSmem M;
  mlp_load_smem(M, mlp);
  __syncthreads();
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (NT / 32);
  for (long base = ((long)blockIdx.x * (NT / 32) + wl) * 32; base < n; base += nwarps * 32) {
    const long i = base + lane;
    RsfIn in;
    double vold = 1e-9;
    float rp = 0.f, up = 0.f, u_plain = 0.f;
    bool need = false;
    if (i < n) {
      state_of(S, n, i, W, in, vold);
      u_plain = (vold > 0) ? logf((float)vold) : -30.f;
      float A_floor;
      const Rsf32 q = rsf32_of(in);
      if (!rsf_floor_certain(q, A_floor)) {
        rp = rsf_start_residual(q, u_plain, up);
        need = !(rp <= RSF_NET_MIN_RES);
      }
    }
    float u0 = u_plain;
    if (__any_sync(V2C_FULL, need)) {
      float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (need) rsf_features(in, f);
#pragma unroll
      for (int k = 0; k < 8; k++) M.xin[wl][lane][k] = f[k];
      __syncwarp();
      mlp_warp_forward(M, wl);
      float un;
      if (need && rsf_start_residual(rsf32_of(in), M.yout[wl][lane][0], un) < rp) u0 = un;
      __syncwarp();
    }
    if (i < n) u0_out[i] = u0;
  }
}

// network outputs (log V, phi) for every state
__global__ void __launch_bounds__(NT) k_infer(const double *S, long n, double W, const float *mlp,
                                              float *out) {
  __shared__ MlpSmem M;
  mlp_load_smem(M, mlp);
  __syncthreads();
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (NT / 32);
  for (long base = ((long)blockIdx.x * (NT / 32) + wl) * 32; base < n; base += nwarps * 32) {
    const long i = base + lane;
    float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
      RsfIn in;
      double vold;
      state_of(S, n, i, W, in, vold);
      rsf_features(in, f);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) M.xin[wl][lane][k] = f[k];
    __syncwarp();
    mlp_warp_forward(M, wl);
    if (i < n) {
      out[i] = M.yout[wl][lane][0];
      out[n + i] = M.yout[wl][lane][1];
    }
    __syncwarp();
  }
}

// ------------------------------------------------------- training inputs
// X[n][8] features, Y[n][2] = (log V, phi) targets, both FP32
__global__ void k_features(const double *S, const double *T, long n, double W, float *X, float *Y) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  RsfIn in;
  double vold;
  state_of(S, n, i, W, in, vold);
  float f[8];
  rsf_features(in, f);
#pragma unroll
  for (int k = 0; k < 8; k++) X[i * 8 + k] = f[k];
  Y[i * 2 + 0] = (float)log(T[i]);
  Y[i * 2 + 1] = (float)T[n + i];
}

// column means and standard deviations, FP64, one block per column,
// fixed-order tree
__global__ void k_colstats(const float *A, long n, int ncol, double *mean, double *sd) {
  __shared__ double s1[256], s2[256];
  const int c = blockIdx.x;
  double a = 0, b = 0;
  for (long i = threadIdx.x; i < n; i += 256) {
    double v = A[i * ncol + c];
    a += v;
    b += v * v;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) { s1[threadIdx.x] += s1[threadIdx.x + o]; s2[threadIdx.x] += s2[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double m = s1[0] / n;
    double var = s2[0] / n - m * m;
    mean[c] = m;
    sd[c] = var > 1e-12 ? sqrt(var) : 1.0;
  }
}

// --------------------------------------------------------------- training
struct TrainSmem {
  __nv_bfloat16 w1[64][16], w2[64][64], w2t[64][64], w3[8][64], w3t[64][2];
  float b1[64], b2[64], b3[2], xm[8], xis[8], ym[2], yis[2];
  __nv_bfloat16 X[128][16];    // normalised inputs (K padded)
  __nv_bfloat16 H1[128][64], H2[128][64], D1[128][64], D2[128][64];
  float DY[128][2];
  float loss[4];
};

__device__ __forceinline__ uint32_t pk(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  __nv_bfloat162 h;
  h.x = lo;
  h.y = hi;
  return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }

// forward + backward for this CTA's 128 samples; partial gradient to part
__global__ void __launch_bounds__(NT) k_train_step(const float *P, const float *Xall,
                                                   const float *Yall, const int32_t *order,
                                                   long n, long first, int bsz, float *part,
                                                   float *loss_part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, wl = tid >> 5, g = lane >> 2, t = lane & 3;
  // weights (BF16 operand images) and normalisation
  for (int i = tid; i < 64 * 16; i += NT) {
    int r = i / 16, c = i % 16;
    S.w1[r][c] = __float2bfloat16(c < 8 ? P[MLP_OW1 + r * 8 + c] : 0.f);
  }
  for (int i = tid; i < 64 * 64; i += NT) {
    __nv_bfloat16 v = __float2bfloat16(P[MLP_OW2 + i]);
    S.w2[i / 64][i % 64] = v;
    S.w2t[i % 64][i / 64] = v;
  }
  for (int i = tid; i < 8 * 64; i += NT) {
    int r = i / 64, c = i % 64;
    __nv_bfloat16 v = __float2bfloat16(r < 2 ? P[MLP_OW3 + r * 64 + c] : 0.f);
    S.w3[r][c] = v;
    if (r < 2) S.w3t[c][r] = v;
  }
  if (tid < 64) { S.b1[tid] = P[MLP_OB1 + tid]; S.b2[tid] = P[MLP_OB2 + tid]; }
  if (tid < 8) { S.xm[tid] = P[MLP_OXM + tid]; S.xis[tid] = 1.f / P[MLP_OXS + tid]; }
  if (tid < 2) { S.b3[tid] = P[MLP_OB3 + tid]; S.ym[tid] = P[MLP_OYM + tid]; S.yis[tid] = 1.f / P[MLP_OYS + tid]; }
  __syncthreads();
  // this CTA's samples
  const long s0 = first + (long)blockIdx.x * 128;
  {
    const int r = tid;  // one sample per thread
    long s = s0 + r;
    bool ok = (long)blockIdx.x * 128 + r < bsz;
    long idx = ok ? order[s % n] : 0;
#pragma unroll
    for (int k = 0; k < 16; k++)
      S.X[r][k] = __float2bfloat16(ok && k < 8 ? (Xall[idx * 8 + k] - S.xm[k]) * S.xis[k] : 0.f);
  }
  __syncthreads();

  float lsum = 0.f;
  const float inv_b = 1.f / (float)bsz;
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    const int r0 = wl * 32 + mt * 16 + g, r1 = r0 + 8;
    const uint32_t xa0 = pk(S.X[r0][2 * t], S.X[r0][2 * t + 1]);
    const uint32_t xa1 = pk(S.X[r1][2 * t], S.X[r1][2 * t + 1]);
    uint32_t h1[4][4], h2[4][4];
    // layer 1
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4];
      d[0] = d[2] = S.b1[nt * 8 + 2 * t];
      d[1] = d[3] = S.b1[nt * 8 + 2 * t + 1];
      mma_bf16(d, xa0, xa1, 0u, 0u, lds_u32(&S.w1[nt * 8 + g][2 * t]), lds_u32(&S.w1[nt * 8 + g][2 * t + 8]));
      const int kk = nt >> 1, hi = nt & 1;
      h1[kk][hi * 2 + 0] = pack_bf16(tanh_fast(d[0]), tanh_fast(d[1]));
      h1[kk][hi * 2 + 1] = pack_bf16(tanh_fast(d[2]), tanh_fast(d[3]));
    }
    // layer 2
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4];
      d[0] = d[2] = S.b2[nt * 8 + 2 * t];
      d[1] = d[3] = S.b2[nt * 8 + 2 * t + 1];
#pragma unroll
      for (int kk = 0; kk < 4; kk++)
        mma_bf16(d, h1[kk][0], h1[kk][1], h1[kk][2], h1[kk][3],
                 lds_u32(&S.w2[nt * 8 + g][kk * 16 + 2 * t]), lds_u32(&S.w2[nt * 8 + g][kk * 16 + 2 * t + 8]));
      const int kk = nt >> 1, hi = nt & 1;
      h2[kk][hi * 2 + 0] = pack_bf16(tanh_fast(d[0]), tanh_fast(d[1]));
      h2[kk][hi * 2 + 1] = pack_bf16(tanh_fast(d[2]), tanh_fast(d[3]));
    }
    // layer 3
    float y[4];
    y[0] = y[2] = (t == 0) ? S.b3[0] : 0.f;
    y[1] = y[3] = (t == 0) ? S.b3[1] : 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
      mma_bf16(y, h2[kk][0], h2[kk][1], h2[kk][2], h2[kk][3],
               lds_u32(&S.w3[g][kk * 16 + 2 * t]), lds_u32(&S.w3[g][kk * 16 + 2 * t + 8]));
    // loss 0.5 mean over samples of the summed squared normalised error
    float dy[4] = {0, 0, 0, 0};
    if (t == 0) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = h ? r1 : r0;
        const long s = s0 + r;
        const bool ok = (long)blockIdx.x * 128 + r < bsz;
        const long idx = ok ? order[s % n] : 0;
        const float t0 = (Yall[idx * 2 + 0] - S.ym[0]) * S.yis[0];
        const float t1 = (Yall[idx * 2 + 1] - S.ym[1]) * S.yis[1];
        const float e0 = ok ? y[2 * h] - t0 : 0.f, e1 = ok ? y[2 * h + 1] - t1 : 0.f;
        lsum += 0.5f * (e0 * e0 + e1 * e1);
        dy[2 * h] = e0 * inv_b;
        dy[2 * h + 1] = e1 * inv_b;
        S.DY[r][0] = dy[2 * h];
        S.DY[r][1] = dy[2 * h + 1];
      }
    }
    // dH2 = dY W3 (A: dY padded to K=16, only k=0,1 live in lanes t==0)
    const uint32_t da0 = (t == 0) ? pack_bf16(dy[0], dy[1]) : 0u;
    const uint32_t da1 = (t == 0) ? pack_bf16(dy[2], dy[3]) : 0u;
    uint32_t d2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4] = {0, 0, 0, 0};
      const uint32_t b0 = (t == 0) ? lds_u32(&S.w3t[nt * 8 + g][0]) : 0u;
      mma_bf16(d, da0, da1, 0u, 0u, b0, 0u);
      // dZ2 = dH2 (1 - H2^2), H2 from the layer-3 A fragments
      const int kk = nt >> 1, hi = nt & 1;
      const __nv_bfloat162 ha = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][hi * 2 + 0]);
      const __nv_bfloat162 hb = *reinterpret_cast<__nv_bfloat162 *>(&h2[kk][hi * 2 + 1]);
      const float z0 = d[0] * (1.f - bf(ha.x) * bf(ha.x)), z1 = d[1] * (1.f - bf(ha.y) * bf(ha.y));
      const float z2 = d[2] * (1.f - bf(hb.x) * bf(hb.x)), z3 = d[3] * (1.f - bf(hb.y) * bf(hb.y));
      d2[kk][hi * 2 + 0] = pack_bf16(z0, z1);
      d2[kk][hi * 2 + 1] = pack_bf16(z2, z3);
      // keep H2 and dZ2 for the weight gradients
      const int c = nt * 8 + 2 * t;
      *reinterpret_cast<uint32_t *>(&S.H2[r0][c]) = h2[kk][hi * 2 + 0];
      *reinterpret_cast<uint32_t *>(&S.H2[r1][c]) = h2[kk][hi * 2 + 1];
      *reinterpret_cast<uint32_t *>(&S.D2[r0][c]) = d2[kk][hi * 2 + 0];
      *reinterpret_cast<uint32_t *>(&S.D2[r1][c]) = d2[kk][hi * 2 + 1];
    }
    // dH1 = dZ2 W2, dZ1 = dH1 (1 - H1^2)
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4] = {0, 0, 0, 0};
#pragma unroll
      for (int kk = 0; kk < 4; kk++)
        mma_bf16(d, d2[kk][0], d2[kk][1], d2[kk][2], d2[kk][3],
                 lds_u32(&S.w2t[nt * 8 + g][kk * 16 + 2 * t]), lds_u32(&S.w2t[nt * 8 + g][kk * 16 + 2 * t + 8]));
      const int kk = nt >> 1, hi = nt & 1;
      const __nv_bfloat162 ha = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][hi * 2 + 0]);
      const __nv_bfloat162 hb = *reinterpret_cast<__nv_bfloat162 *>(&h1[kk][hi * 2 + 1]);
      const float z0 = d[0] * (1.f - bf(ha.x) * bf(ha.x)), z1 = d[1] * (1.f - bf(ha.y) * bf(ha.y));
      const float z2 = d[2] * (1.f - bf(hb.x) * bf(hb.x)), z3 = d[3] * (1.f - bf(hb.y) * bf(hb.y));
      const int c = nt * 8 + 2 * t;
      *reinterpret_cast<uint32_t *>(&S.H1[r0][c]) = h1[kk][hi * 2 + 0];
      *reinterpret_cast<uint32_t *>(&S.H1[r1][c]) = h1[kk][hi * 2 + 1];
      *reinterpret_cast<uint32_t *>(&S.D1[r0][c]) = pack_bf16(z0, z1);
      *reinterpret_cast<uint32_t *>(&S.D1[r1][c]) = pack_bf16(z2, z3);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(V2C_FULL, lsum, o);
  if (lane == 0) S.loss[wl] = lsum;
  __syncthreads();

  // ---- weight gradients over the CTA's 128 samples (K = samples)
  // A[m][k] = D[k][m] (transposed activation gradient), B[k][n] = act[k][n]
  float *out = part + (long)blockIdx.x * NG;
  // dW2[o][i] = sum_s D2[s][o] H1[s][i]: 4 m-tiles x 8 n-tiles, 8 per warp
  for (int tile = wl; tile < 32; tile += 4) {
    const int mt = tile >> 3, nt = tile & 7;
    float d[4] = {0, 0, 0, 0};
#pragma unroll
    for (int kk = 0; kk < 8; kk++) {
      const int k0 = kk * 16 + 2 * t, m0 = mt * 16 + g;
      const uint32_t a0 = pk(S.D2[k0][m0], S.D2[k0 + 1][m0]);
      const uint32_t a1 = pk(S.D2[k0][m0 + 8], S.D2[k0 + 1][m0 + 8]);
      const uint32_t a2 = pk(S.D2[k0 + 8][m0], S.D2[k0 + 9][m0]);
      const uint32_t a3 = pk(S.D2[k0 + 8][m0 + 8], S.D2[k0 + 9][m0 + 8]);
      const int n0 = nt * 8 + g;
      const uint32_t b0 = pk(S.H1[k0][n0], S.H1[k0 + 1][n0]);
      const uint32_t b1 = pk(S.H1[k0 + 8][n0], S.H1[k0 + 9][n0]);
      mma_bf16(d, a0, a1, a2, a3, b0, b1);
    }
    const int m0 = mt * 16 + g, c = nt * 8 + 2 * t;
    out[MLP_OW2 + m0 * 64 + c] = d[0];
    out[MLP_OW2 + m0 * 64 + c + 1] = d[1];
    out[MLP_OW2 + (m0 + 8) * 64 + c] = d[2];
    out[MLP_OW2 + (m0 + 8) * 64 + c + 1] = d[3];
  }
  // dW1[o][k] = sum_s D1[s][o] X[s][k]: 4 m-tiles x 1 n-tile (k < 8)
  {
    const int mt = wl;
    float d[4] = {0, 0, 0, 0};
#pragma unroll
    for (int kk = 0; kk < 8; kk++) {
      const int k0 = kk * 16 + 2 * t, m0 = mt * 16 + g;
      const uint32_t a0 = pk(S.D1[k0][m0], S.D1[k0 + 1][m0]);
      const uint32_t a1 = pk(S.D1[k0][m0 + 8], S.D1[k0 + 1][m0 + 8]);
      const uint32_t a2 = pk(S.D1[k0 + 8][m0], S.D1[k0 + 9][m0]);
      const uint32_t a3 = pk(S.D1[k0 + 8][m0 + 8], S.D1[k0 + 9][m0 + 8]);
      const uint32_t b0 = pk(S.X[k0][g], S.X[k0 + 1][g]);
      const uint32_t b1 = pk(S.X[k0 + 8][g], S.X[k0 + 9][g]);
      mma_bf16(d, a0, a1, a2, a3, b0, b1);
    }
    const int m0 = mt * 16 + g, c = 2 * t;
    out[MLP_OW1 + m0 * 8 + c] = d[0];
    out[MLP_OW1 + m0 * 8 + c + 1] = d[1];
    out[MLP_OW1 + (m0 + 8) * 8 + c] = d[2];
    out[MLP_OW1 + (m0 + 8) * 8 + c + 1] = d[3];
  }
  // dW3[j][i] = sum_s DY[s][j] H2[s][i] and the biases: plain FP32 sums in
  // sample order (small)
  for (int q = tid; q < 2 * 64 + 64 + 64 + 2; q += NT) {
    float acc = 0.f;
    if (q < 128) {
      const int j = q / 64, i = q % 64;
      for (int s = 0; s < 128; s++) acc += S.DY[s][j] * bf(S.H2[s][i]);
      out[MLP_OW3 + j * 64 + i] = acc;
    } else if (q < 192) {
      const int o = q - 128;
      for (int s = 0; s < 128; s++) acc += bf(S.D2[s][o]);
      out[MLP_OB2 + o] = acc;
    } else if (q < 256) {
      const int o = q - 192;
      for (int s = 0; s < 128; s++) acc += bf(S.D1[s][o]);
      out[MLP_OB1 + o] = acc;
    } else {
      const int j = q - 256;
      for (int s = 0; s < 128; s++) acc += S.DY[s][j];
      out[MLP_OB3 + j] = acc;
    }
  }
  if (tid == 0) loss_part[blockIdx.x] = S.loss[0] + S.loss[1] + S.loss[2] + S.loss[3];
}

// sum the per-CTA partials in CTA order; Adam on the FP32 master weights
// (or, with adam == 0, just return the gradient)
__global__ void k_reduce_adam(const float *part, int nparts, float *P, float *m1, float *m2,
                              float lr, float b1c, float b2c, int adam, float *grad_out) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NG) return;
  float gsum = 0.f;
  for (int c = 0; c < nparts; c++) gsum += part[(long)c * NG + p];
  if (grad_out) grad_out[p] = gsum;
  if (!adam) return;
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  m1[p] = beta1 * m1[p] + (1.f - beta1) * gsum;
  m2[p] = beta2 * m2[p] + (1.f - beta2) * gsum * gsum;
  const float mh = m1[p] / b1c, vh = m2[p] / b2c;
  P[p] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_sum_loss(const float *lp, int np, float *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < np; i++) s += lp[i];
    *out = s;
  }
}

uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

}  // namespace
}  // namespace v2c

using namespace v2c;

#define CKR(call)                                    \
  do {                                               \
    if ((call) != cudaSuccess) return V2C_ERR_CUDA;  \
  } while (0)

extern "C" int v2c_rsf_newton(v2c_ctx *ctx, const double *states_dev, long n, int guess,
                              double *out_dev, int32_t *iters_dev) {
  if (!ctx || (!states_dev && n > 0) || (!out_dev && n > 0) || n < 0) return V2C_ERR_ARG;
  if (guess == V2C_GUESS_LEARNED && !v2c_ctx_newton(ctx)->have_mlp) return V2C_ERR_STATE;
  if (n == 0) return V2C_OK;
  const v2c_params *p = v2c_ctx_params(ctx);
  cudaStream_t st = v2c_ctx_stream(ctx);
  long warps = (n + 31) / 32;
  long blocks = (warps + 3) / 4;
  if (blocks > 152 * 16) blocks = 152 * 16;
  cudaEvent_t ev;
  v2c_ctx_prof_begin(ctx, V2C_PROF_NEWTON, &ev);
  const bool fp64 = p->newton_precision == V2C_NEWTON_FP64;
  const bool learned = guess == V2C_GUESS_LEARNED;
  NewtonState *ns = v2c_ctx_newton(ctx);
  if (learned) {
    if (ns->guess_cap < n) {
      if (ns->d_guess) cudaFree(ns->d_guess);
      ns->d_guess = nullptr;
      ns->guess_cap = 0;
      CKR(cudaMalloc((void **)&ns->d_guess, sizeof(float) * 2 * n));
      ns->guess_cap = n;
    }
    k_learned_start<<<(unsigned)blocks, NT, 0, st>>>(states_dev, n, p->faultwidth, ns->d_mlp,
                                                     ns->d_guess);
    v2c_ctx_count_launches(ctx, 1);
  }
  auto kern = fp64 ? (learned ? k_solve_states<true, true> : k_solve_states<true, false>)
                   : (learned ? k_solve_states<false, true> : k_solve_states<false, false>);
  kern<<<(unsigned)blocks, NT, 0, st>>>(states_dev, n, p->faultwidth, ns->d_guess, p->newton_rtol,
                                        p->newton_maxit, out_dev, iters_dev, v2c_ctx_stat(ctx));
  v2c_ctx_prof_end(ctx, V2C_PROF_NEWTON, ev);
  v2c_ctx_count_launches(ctx, 1);
  CKR(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_mlp_load(v2c_ctx *ctx, const float *params_host) {
  if (!ctx || !params_host) return V2C_ERR_ARG;
  NewtonState *s = v2c_ctx_newton(ctx);
  CKR(cudaMemcpy(s->d_mlp, params_host, sizeof(float) * V2C_MLP_NPARAM, cudaMemcpyHostToDevice));
  s->have_mlp = 1;
  return V2C_OK;
}

extern "C" int v2c_mlp_save(v2c_ctx *ctx, float *params_host) {
  if (!ctx || !params_host) return V2C_ERR_ARG;
  NewtonState *s = v2c_ctx_newton(ctx);
  CKR(cudaStreamSynchronize(v2c_ctx_stream(ctx)));
  CKR(cudaMemcpy(params_host, s->d_mlp, sizeof(float) * V2C_MLP_NPARAM, cudaMemcpyDeviceToHost));
  return V2C_OK;
}

namespace {
// shared by training and the gradient check
struct TrainBufs {
  float *X = nullptr, *Y = nullptr, *part = nullptr, *lpart = nullptr, *m1 = nullptr,
        *m2 = nullptr, *loss = nullptr, *grad = nullptr;
  int32_t *order = nullptr;
  double *stats = nullptr;
  ~TrainBufs() {
    void *p[] = {X, Y, part, lpart, m1, m2, loss, grad, order, stats};
    for (void *q : p)
      if (q) cudaFree(q);
  }
};

int prepare(v2c_ctx *ctx, const double *S, const double *T, long n, int batch, TrainBufs &b,
            bool set_norm) {
  cudaStream_t st = v2c_ctx_stream(ctx);
  const v2c_params *p = v2c_ctx_params(ctx);
  int nparts = (batch + 127) / 128;
  CKR(cudaMalloc((void **)&b.X, sizeof(float) * n * 8));
  CKR(cudaMalloc((void **)&b.Y, sizeof(float) * n * 2));
  CKR(cudaMalloc((void **)&b.part, sizeof(float) * (size_t)nparts * NG));
  CKR(cudaMalloc((void **)&b.lpart, sizeof(float) * nparts));
  CKR(cudaMalloc((void **)&b.m1, sizeof(float) * NG));
  CKR(cudaMalloc((void **)&b.m2, sizeof(float) * NG));
  CKR(cudaMalloc((void **)&b.loss, sizeof(float)));
  CKR(cudaMalloc((void **)&b.grad, sizeof(float) * NG));
  CKR(cudaMalloc((void **)&b.order, sizeof(int32_t) * n));
  CKR(cudaMalloc((void **)&b.stats, sizeof(double) * 20));
  CKR(cudaMemsetAsync(b.m1, 0, sizeof(float) * NG, st));
  CKR(cudaMemsetAsync(b.m2, 0, sizeof(float) * NG, st));
  k_features<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(S, T, n, p->faultwidth, b.X, b.Y);
  v2c_ctx_count_launches(ctx, 1);
  if (set_norm) {
    k_colstats<<<8, 256, 0, st>>>(b.X, n, 8, b.stats, b.stats + 8);
    k_colstats<<<2, 256, 0, st>>>(b.Y, n, 2, b.stats + 16, b.stats + 18);
    v2c_ctx_count_launches(ctx, 2);
    double h[20];
    CKR(cudaMemcpyAsync(h, b.stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    float f[20];
    for (int i = 0; i < 20; i++) f[i] = (float)h[i];
    NewtonState *s = v2c_ctx_newton(ctx);
    CKR(cudaMemcpy(s->d_mlp + MLP_OXM, f, sizeof(float) * 8, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(s->d_mlp + MLP_OXS, f + 8, sizeof(float) * 8, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(s->d_mlp + MLP_OYM, f + 16, sizeof(float) * 2, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(s->d_mlp + MLP_OYS, f + 18, sizeof(float) * 2, cudaMemcpyHostToDevice));
  }
  return V2C_OK;
}

cudaError_t train_smem_attr() {
  return cudaFuncSetAttribute(k_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(TrainSmem));
}
}  // namespace

extern "C" int v2c_mlp_train(v2c_ctx *ctx, const double *states_dev, const double *targets_dev,
                             long n, int epochs, int batch, float lr, uint64_t seed,
                             float *final_loss) {
  if (!ctx || !states_dev || !targets_dev || n < 128 || epochs < 1 || batch < 128) return V2C_ERR_ARG;
  if (n > INT32_MAX) return V2C_ERR_CAPACITY;
  batch = (batch / 128) * 128;
  cudaStream_t st = v2c_ctx_stream(ctx);
  NewtonState *s = v2c_ctx_newton(ctx);
  TrainBufs b;
  int rc = prepare(ctx, states_dev, targets_dev, n, batch, b, true);
  if (rc) return rc;
  // Xavier-uniform initialisation from the seed
  std::vector<float> P(V2C_MLP_NPARAM, 0.f);
  CKR(cudaMemcpy(P.data(), s->d_mlp, sizeof(float) * V2C_MLP_NPARAM, cudaMemcpyDeviceToHost));
  uint64_t rs = seed;
  auto uni = [&](float lim) {
    return (float)((double)(splitmix(rs) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * lim;
  };
  for (int i = 0; i < 64 * 8; i++) P[MLP_OW1 + i] = uni(sqrtf(6.f / (8 + 64)));
  for (int i = 0; i < 64 * 64; i++) P[MLP_OW2 + i] = uni(sqrtf(6.f / (64 + 64)));
  for (int i = 0; i < 2 * 64; i++) P[MLP_OW3 + i] = uni(sqrtf(6.f / (64 + 2)));
  for (int i = 0; i < 64; i++) P[MLP_OB1 + i] = P[MLP_OB2 + i] = 0.f;
  P[MLP_OB3] = P[MLP_OB3 + 1] = 0.f;
  CKR(cudaMemcpy(s->d_mlp, P.data(), sizeof(float) * V2C_MLP_NPARAM, cudaMemcpyHostToDevice));
  CKR(train_smem_attr());
  // shuffled sample order per epoch (host Fisher-Yates from the seed)
  std::vector<int32_t> order(n);
  const int nparts = batch / 128;
  const long steps_per_epoch = (n + batch - 1) / batch;
  long step = 0;
  float last = 0.f;
  for (int ep = 0; ep < epochs; ep++) {
    for (long i = 0; i < n; i++) order[i] = (int32_t)i;
    for (long i = n - 1; i > 0; i--) {
      long j = (long)(splitmix(rs) % (uint64_t)(i + 1));
      std::swap(order[i], order[j]);
    }
    CKR(cudaMemcpyAsync(b.order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    for (long k = 0; k < steps_per_epoch; k++) {
      step++;
      const float b1c = 1.f - powf(0.9f, (float)step), b2c = 1.f - powf(0.999f, (float)step);
      // cosine decay of the learning rate over the run
      const float frac = (float)step / (float)(epochs * steps_per_epoch);
      const float lr_t = lr * 0.5f * (1.f + cosf(3.14159265f * frac));
      k_train_step<<<nparts, NT, sizeof(TrainSmem), st>>>(s->d_mlp, b.X, b.Y, b.order, n,
                                                           k * (long)batch, batch, b.part, b.lpart);
      k_reduce_adam<<<(NG + 255) / 256, 256, 0, st>>>(b.part, nparts, s->d_mlp, b.m1, b.m2, lr_t,
                                                      b1c, b2c, 1, nullptr);
      v2c_ctx_count_launches(ctx, 2);
    }
    k_sum_loss<<<1, 32, 0, st>>>(b.lpart, nparts, b.loss);
    CKR(cudaMemcpyAsync(&last, b.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
  }
  CKR(cudaGetLastError());
  s->have_mlp = 1;
  if (final_loss) *final_loss = last / (float)batch;
  return V2C_OK;
}

extern "C" int v2c_mlp_grad(v2c_ctx *ctx, const double *states_dev, const double *targets_dev,
                            long n, float *grad_host, float *loss) {
  if (!ctx || !states_dev || !targets_dev || !grad_host || n < 1 || n > 128 * 1024) return V2C_ERR_ARG;
  if (!v2c_ctx_newton(ctx)->have_mlp) return V2C_ERR_STATE;
  cudaStream_t st = v2c_ctx_stream(ctx);
  NewtonState *s = v2c_ctx_newton(ctx);
  const int batch = (int)((n + 127) / 128 * 128);
  TrainBufs b;
  int rc = prepare(ctx, states_dev, targets_dev, n, batch, b, false);
  if (rc) return rc;
  std::vector<int32_t> order(n);
  for (long i = 0; i < n; i++) order[i] = (int32_t)i;
  CKR(cudaMemcpyAsync(b.order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
  CKR(train_smem_attr());
  const int nparts = batch / 128;
  // k_train_step normalises by the batch; pass the true count
  k_train_step<<<nparts, NT, sizeof(TrainSmem), st>>>(s->d_mlp, b.X, b.Y, b.order, n, 0, (int)n,
                                                       b.part, b.lpart);
  k_reduce_adam<<<(NG + 255) / 256, 256, 0, st>>>(b.part, nparts, s->d_mlp, b.m1, b.m2, 0.f, 1.f,
                                                  1.f, 0, b.grad);
  k_sum_loss<<<1, 32, 0, st>>>(b.lpart, nparts, b.loss);
  v2c_ctx_count_launches(ctx, 3);
  CKR(cudaMemcpyAsync(grad_host, b.grad, sizeof(float) * NG, cudaMemcpyDeviceToHost, st));
  float l = 0.f;
  CKR(cudaMemcpyAsync(&l, b.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  CKR(cudaStreamSynchronize(st));
  CKR(cudaGetLastError());
  if (loss) *loss = l / (float)n;
  return V2C_OK;
}

extern "C" int v2c_mlp_infer(v2c_ctx *ctx, const double *states_dev, long n, float *out_dev) {
  if (!ctx || !states_dev || !out_dev || n < 0) return V2C_ERR_ARG;
  if (!v2c_ctx_newton(ctx)->have_mlp) return V2C_ERR_STATE;
  if (n == 0) return V2C_OK;
  long blocks = ((n + 31) / 32 + 3) / 4;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_infer<<<(unsigned)blocks, NT, 0, v2c_ctx_stream(ctx)>>>(states_dev, n, v2c_ctx_params(ctx)->faultwidth,
                                                           v2c_ctx_newton(ctx)->d_mlp, out_dev);
  v2c_ctx_count_launches(ctx, 1);
  CKR(cudaGetLastError());
  return V2C_OK;
}
