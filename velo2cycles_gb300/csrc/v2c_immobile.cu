// v2c_immobile.cu -- the marker bookkeeping of immobile markers after the
// move (moveandrotatemarkers.c:88-171), in reference marker order.
//
// An immobile marker (type >= 100) that moved inside the model spawns a
// mobile marker of type - 100 there; the reference appends the spawned
// markers after the last marker in the order of its marker loop, then lets
// the mobile markers left outside the model, in marker order, take the
// appended markers from the last one back.  The move kernel records, per
// reference marker number (id), whether the marker spawned (with the spawn
// position) or is a mobile marker outside the model.  Here:
//   * exclusive scans over ids give each spawn its append rank j and each
//     out-of-model marker its rank k (A spawns and O such markers in all);
//   * the out-of-model marker of rank k < min(A, O) takes spawn A-1-k: type,
//     position, and the resets the reference applies (temperature, markd,
//     strain, stresses, pressure, strain rates);
//   * spawns j < A - min(A, O) become new markers n + j (array index and
//     id), with the spawn's resets and every other field zero (the
//     reference's slots past the last marker have never held a marker).
// The markers stay where they are in the arrays; the next cell sort orders
// them.  This is the routine as written for one thread (the reference's
// OpenMP build appends through a reduction variable that starts from 0 in
// each thread, so there the spawns overwrite markers 0, 1, ...).
#include "v2c_kernels.h"

namespace v2c {

namespace {

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_imm_inv(const int32_t *id, long n, int32_t *inv) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) inv[id[i]] = (int32_t)i;
}

__global__ void k_imm_src(ImmBufs b, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n && b.spawn[k]) b.src[b.spawn_rank[k]] = (int32_t)k;
}

// the resets a spawned or refilled marker gets (moveandrotatemarkers.c:
// 101-119, 150-167)
__device__ __forceinline__ void reset_fields(const Markers &m, long i) {
  m.tk[i] = 0.f; m.tk_lo[i] = 0.f;
  m.e[i] = 0.f; m.sxx[i] = 0.f; m.sxy[i] = 0.f; m.p[i] = 0.f;
  m.exx[i] = 0.f; m.exy[i] = 0.f;
}

__global__ void k_imm_refill(Markers m, ImmBufs b, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n || !b.out[k]) return;
  const int A = b.spawn_rank[n], O = b.out_rank[n];
  const int K = A < O ? A : O;
  const int r = b.out_rank[k];
  if (r >= K) return;
  const int src = b.src[A - 1 - r];
  const long i = b.inv[k], s = b.inv[src];
  m.type[i] = (int8_t)(m.type[s] - 100);
  m.cell_out[i] = b.sp_cell[src];
  m.u_out[i] = b.sp_u[src];
  m.v_out[i] = b.sp_v[src];
  reset_fields(m, i);
  m.flags[i] |= MFLAG_DNEG;
}

__global__ void k_imm_append(Markers m, ImmBufs b, long n) {
  const long j = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int A = b.spawn_rank[n], O = b.out_rank[n];
  const int keep = A - (A < O ? A : O);
  if (j >= keep) return;
  const int src = b.src[j];
  const long i = n + j, s = b.inv[src];
  m.type[i] = (int8_t)(m.type[s] - 100);
  m.cell_out[i] = b.sp_cell[src];
  m.u_out[i] = b.sp_u[src];
  m.v_out[i] = b.sp_v[src];
  m.id[i] = (int32_t)i;
  m.flags[i] = MFLAG_DNEG;
  reset_fields(m, i);
  m.mv[i] = 0.f; m.mv_lo[i] = 0.f;
  m.vx[i] = 0.f; m.vy[i] = 0.f; m.phi[i] = 0.f; m.coh[i] = 0.f; m.slipv[i] = 0.f;
  m.mnu[i] = 0.f; m.mkt[i] = 0.f; m.mro[i] = 0.f;
}

}  // namespace

int launch_immobile_compact(const Markers &m, long n, long cap, ImmBufs &b, long *added,
                            cudaStream_t st) {
  *added = 0;
  if (n <= 0) return V2C_OK;
  launch_scan(b.spawn, n, b.spawn_rank, b.blocksum, st);
  launch_scan(b.out, n, b.out_rank, b.blocksum, st);
  int32_t h[2] = {0, 0};
  if (cudaMemcpyAsync(&h[0], b.spawn_rank + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(&h[1], b.out_rank + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return V2C_ERR_CUDA;
  const long A = h[0], O = h[1];
  if (A == 0) return V2C_OK;
  const long keep = A - (A < O ? A : O);
  if (n + keep > cap) return V2C_ERR_CAPACITY;  // the reference's "Space out in markx[]"
  k_imm_inv<<<nblk(n, 256), 256, 0, st>>>(m.id, n, b.inv);
  k_imm_src<<<nblk(n, 256), 256, 0, st>>>(b, n);
  k_imm_refill<<<nblk(n, 256), 256, 0, st>>>(m, b, n);
  if (keep > 0) k_imm_append<<<nblk(keep, 256), 256, 0, st>>>(m, b, n);
  *added = keep;
  return cudaGetLastError() == cudaSuccess ? V2C_OK : V2C_ERR_CUDA;
}

}  // namespace v2c
