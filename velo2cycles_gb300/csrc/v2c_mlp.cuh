// v2c_mlp.cuh -- the 8 -> 64 -> 64 -> 2 tanh network that proposes the
// start of the per-marker Newton, evaluated by one warp for 32 states on the
// tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulate).
//
// Fragment layout of m16n8k16 (g = lane/4, t = lane%4):
//   A (16x16, row): a0 = (g, 2t..2t+1)  a1 = (g+8, 2t..)  a2 = (g, 2t+8..)  a3 = (g+8, 2t+8..)
//   B (16x8, col):  b0 = (k 2t..2t+1, n g)  b1 = (k 2t+8.., n g)
//   C (16x8):       c0,c1 = (g, 2t..2t+1)   c2,c3 = (g+8, 2t..2t+1)
// The C fragments of n-tiles 2k and 2k+1 are exactly the A fragment of
// k-step k of the next layer, so the layers chain in registers.
//
// Packed parameter vector (host, FP32; see V2C_MLP_NPARAM):
//   W1[64][8] b1[64] W2[64][64] b2[64] W3[2][64] b3[2] xmean[8] xstd[8]
//   ymean[2] ystd[2]
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace v2c {

constexpr int MLP_H = 64;
enum {
  MLP_OW1 = 0, MLP_OB1 = MLP_OW1 + 64 * 8, MLP_OW2 = MLP_OB1 + 64, MLP_OB2 = MLP_OW2 + 64 * 64,
  MLP_OW3 = MLP_OB2 + 64, MLP_OB3 = MLP_OW3 + 2 * 64, MLP_OXM = MLP_OB3 + 2,
  MLP_OXS = MLP_OXM + 8, MLP_OYM = MLP_OXS + 8, MLP_OYS = MLP_OYM + 2, MLP_NP = MLP_OYS + 2
};

// Shared-memory image of the network used by inference.  Weight rows are
// padded (16 -> 24 and 64 -> 72 BF16) so that the eight rows a B-fragment
// load touches (one per lane group g) fall in distinct banks.
constexpr int MLP_W1S = 24, MLP_W2S = 72;
struct MlpSmem {
  __nv_bfloat16 w1[64][MLP_W1S];   // K padded 8 -> 16 with zeros
  __nv_bfloat16 w2[64][MLP_W2S];
  __nv_bfloat16 w3[8][MLP_W2S];    // N padded 2 -> 8 with zeros
  float b1[64], b2[64], b3[2];
  float xm[8], xis[8], ym[2], ys[2];
  float xin[4][32][9];             // per-warp feature staging (4 warps), padded
  float yout[4][32][2];
};

__device__ __forceinline__ void mlp_load_smem(MlpSmem &S, const float *P) {
  for (int i = threadIdx.x; i < 64 * 16; i += blockDim.x) {
    int r = i / 16, c = i % 16;
    S.w1[r][c] = __float2bfloat16(c < 8 ? P[MLP_OW1 + r * 8 + c] : 0.f);
  }
  for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x)
    S.w2[i / 64][i % 64] = __float2bfloat16(P[MLP_OW2 + i]);
  for (int i = threadIdx.x; i < 8 * 64; i += blockDim.x) {
    int r = i / 64, c = i % 64;
    S.w3[r][c] = __float2bfloat16(r < 2 ? P[MLP_OW3 + r * 64 + c] : 0.f);
  }
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    S.b1[i] = P[MLP_OB1 + i];
    S.b2[i] = P[MLP_OB2 + i];
  }
  if (threadIdx.x < 8) {
    S.xm[threadIdx.x] = P[MLP_OXM + threadIdx.x];
    S.xis[threadIdx.x] = 1.f / P[MLP_OXS + threadIdx.x];
  }
  if (threadIdx.x < 2) {
    S.b3[threadIdx.x] = P[MLP_OB3 + threadIdx.x];
    S.ym[threadIdx.x] = P[MLP_OYM + threadIdx.x];
    S.ys[threadIdx.x] = P[MLP_OYS + threadIdx.x];
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t lds_u32(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

// One warp evaluates the network for the 32 feature rows this warp staged
// in S.xin[wl] (raw features, normalised here); results land in
// S.yout[wl][row][0..1], denormalised.  The two 16-row m-tiles go through
// the layers one after the other (fewer live registers than both at once).
// All 32 lanes must call it.
__device__ __forceinline__ void mlp_warp_forward(MlpSmem &S, int wl) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
  for (int mt = 0; mt < 2; mt++) {
    const int r0 = mt * 16 + g, r1 = r0 + 8;
    // layer 1: X (16x16, K padded) times W1^T
    const uint32_t xa0 = pack_bf16((S.xin[wl][r0][2 * t] - S.xm[2 * t]) * S.xis[2 * t],
                                   (S.xin[wl][r0][2 * t + 1] - S.xm[2 * t + 1]) * S.xis[2 * t + 1]);
    const uint32_t xa1 = pack_bf16((S.xin[wl][r1][2 * t] - S.xm[2 * t]) * S.xis[2 * t],
                                   (S.xin[wl][r1][2 * t + 1] - S.xm[2 * t + 1]) * S.xis[2 * t + 1]);
    uint32_t h1[4][4];  // A fragments of layer 2, one per k-step
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4];
      d[0] = d[2] = S.b1[nt * 8 + 2 * t];
      d[1] = d[3] = S.b1[nt * 8 + 2 * t + 1];
      mma_bf16(d, xa0, xa1, 0u, 0u, lds_u32(&S.w1[nt * 8 + g][2 * t]),
               lds_u32(&S.w1[nt * 8 + g][2 * t + 8]));
      const int kk = nt >> 1, hi = nt & 1;
      h1[kk][hi * 2 + 0] = pack_bf16(tanh_fast(d[0]), tanh_fast(d[1]));
      h1[kk][hi * 2 + 1] = pack_bf16(tanh_fast(d[2]), tanh_fast(d[3]));
    }
    // layer 2
    uint32_t h2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4];
      d[0] = d[2] = S.b2[nt * 8 + 2 * t];
      d[1] = d[3] = S.b2[nt * 8 + 2 * t + 1];
#pragma unroll
      for (int kk = 0; kk < 4; kk++)
        mma_bf16(d, h1[kk][0], h1[kk][1], h1[kk][2], h1[kk][3],
                 lds_u32(&S.w2[nt * 8 + g][kk * 16 + 2 * t]),
                 lds_u32(&S.w2[nt * 8 + g][kk * 16 + 2 * t + 8]));
      const int kk = nt >> 1, hi = nt & 1;
      h2[kk][hi * 2 + 0] = pack_bf16(tanh_fast(d[0]), tanh_fast(d[1]));
      h2[kk][hi * 2 + 1] = pack_bf16(tanh_fast(d[2]), tanh_fast(d[3]));
    }
    // layer 3 (2 outputs in an 8-wide tile)
    float d[4];
    d[0] = d[2] = (t == 0) ? S.b3[0] : 0.f;
    d[1] = d[3] = (t == 0) ? S.b3[1] : 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
      mma_bf16(d, h2[kk][0], h2[kk][1], h2[kk][2], h2[kk][3],
               lds_u32(&S.w3[g][kk * 16 + 2 * t]), lds_u32(&S.w3[g][kk * 16 + 2 * t + 8]));
    if (t == 0) {
      S.yout[wl][r0][0] = d[0] * S.ys[0] + S.ym[0];
      S.yout[wl][r0][1] = d[1] * S.ys[1] + S.ym[1];
      S.yout[wl][r1][0] = d[2] * S.ys[0] + S.ym[0];
      S.yout[wl][r1][1] = d[3] * S.ys[1] + S.ym[1];
    }
  }
  __syncwarp();
}

}  // namespace v2c
