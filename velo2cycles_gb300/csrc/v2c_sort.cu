// v2c_sort.cu -- cell assignment and the counting sort by cell.
//
// Cell assignment (upload) bisects the FP64 grid lines exactly like
// nxsearch/nysearch (interpolation.c:1536-1573), so the integer cell of
// every marker is bit-identical to the reference's.  The counting sort
// orders by cell, within a cell by quarter class q = 2 (v > 1/2) + (u > 1/2)
// and within a class by array index: counts by integer atomics
// (order-independent), exclusive scan, scatter of (q, index) keys into
// per-cell slots, then each cell's keys are ranked, which fixes the order
// whatever order the atomics handed the slots out in.  The sweeps that
// scatter to nodes read each quarter class as one contiguous run.
#include <climits>

#include "v2c_kernels.h"

namespace v2c {

namespace {

__global__ void k_assign(Grid g, const double *x, const double *y, long n, Markers m) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xi = x[i], yi = y[i];
  int ix = nsearch64(g.gx, g.xn, xi), iy = nsearch64(g.gy, g.yn, yi);
  double u = (xi - g.gx[ix]) / (g.gx[ix + 1] - g.gx[ix]);
  double v = (yi - g.gy[iy]) / (g.gy[iy + 1] - g.gy[iy]);
  m.cell_in[i] = ix * g.ncy + iy;
  m.u_in[i] = offset32(u);
  m.v_in[i] = offset32(v);
  m.id[i] = (int32_t)i;
}

// Markers of one cell are mostly adjacent in memory, so the lanes of a warp
// share few cells: one atomic per distinct cell in the warp (the leader adds
// the group's size), each lane's slot is the group's base plus its rank
// among the group's lanes.
__global__ void k_count(const int32_t *cell, long n, int32_t *counts, int32_t *slot) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = i < n;
  const int c = valid ? cell[i] : -1;
  const unsigned act = __ballot_sync(V2C_FULL, valid);
  if (!valid) return;
  const unsigned grp = __match_any_sync(act, c);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(grp) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counts + c, __popc(grp));
  base = __shfl_sync(grp, base, leader);
  slot[i] = base + __popc(grp & ((1u << lane) - 1));
}

// exclusive scan, three passes: per-block scan of 4 elements per thread
constexpr int SB = 1024, SE = 4;
__global__ void k_scan_block(const int32_t *in, long m, int32_t *out, int32_t *bsum) {
  __shared__ int32_t sh[SB];
  long base = (long)blockIdx.x * SB * SE + (long)threadIdx.x * SE;
  int32_t v[SE], s = 0;
#pragma unroll
  for (int k = 0; k < SE; k++) {
    v[k] = (base + k < m) ? in[base + k] : 0;
    s += v[k];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < SB; off <<= 1) {
    int32_t t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int32_t run = sh[threadIdx.x] - s;
#pragma unroll
  for (int k = 0; k < SE; k++) {
    if (base + k < m) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == SB - 1) bsum[blockIdx.x] = sh[SB - 1];
}

__global__ void k_scan_sums(int32_t *bsum, long nb, int32_t *total_out) {
  // single block, sequential chunks of SB
  __shared__ int32_t sh[SB];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long c0 = 0; c0 < nb; c0 += SB) {
    long i = c0 + threadIdx.x;
    int32_t v = (i < nb) ? bsum[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < SB; off <<= 1) {
      int32_t t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += sh[SB - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(int32_t *out, long m, const int32_t *bsum) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < m) out[i] += bsum[i / (SB * SE)];
}

// key of marker i: quarter class in bits 30-31, array index below
__global__ void k_slots(const int32_t *cell, const float *u, const float *v, long n,
                        const int32_t *start, const int32_t *slot, uint32_t *tmp) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t q = (v[i] > 0.5f ? 2u : 0u) + (u[i] > 0.5f ? 1u : 0u);
    tmp[start[cell[i]] + slot[i]] = (q << 30) | (uint32_t)i;
  }
}

constexpr uint32_t KEY_INDEX = (1u << 30) - 1;

// One warp orders the L <= 32 distinct keys of a cell's slots, held one per
// lane in val (lanes >= L hold 0xffffffff, which sorts last: array indices
// stay below 2^30 - 1, so no key equals it), writes their indices in
// ascending key order and returns the counts of quarter classes 0, 1, 2
// (same value in every lane).  The bitonic network is skipped when the
// keys are in order already: a cell whose markers one warp of the count
// pass met keeps their slots in array order, and array order is class
// order for markers that have kept their cell and class since the markers
// were last stored in sorted order.
__device__ __forceinline__ int4 rank_small(uint32_t val, int32_t *perm, int L, int lane) {
  uint32_t key = val;
  const uint32_t next = __shfl_down_sync(V2C_FULL, val, 1);
  if (!__all_sync(V2C_FULL, lane >= L - 1 || val < next)) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const uint32_t other = __shfl_xor_sync(V2C_FULL, key, j);
        const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
        key = keep_min ? min(key, other) : max(key, other);
      }
  }
  const bool in = lane < L;
  const uint32_t q = key >> 30;
  int4 cnt;
  cnt.x = __popc(__ballot_sync(V2C_FULL, in && q == 0));
  cnt.y = __popc(__ballot_sync(V2C_FULL, in && q == 1));
  cnt.z = __popc(__ballot_sync(V2C_FULL, in && q == 2));
  cnt.w = 0;
  if (in) perm[lane] = (int32_t)(key & KEY_INDEX);
  return cnt;
}

// The same for a cell of L > 32 keys (read from tmp): each key's rank is
// the number of the cell's keys below it.
__device__ __noinline__ int4 rank_large(const uint32_t *tmp, int32_t *perm, int L, int lane) {
  int4 cnt = make_int4(0, 0, 0, 0);
  for (int b = 0; b < L; b += 32) {
    const int jj = b + lane;
    const uint32_t val = (jj < L) ? tmp[jj] : 0xffffffffu;
    int rank = 0;
    for (int b2 = 0; b2 < L; b2 += 32) {
      const uint32_t other = (b2 + lane < L) ? tmp[b2 + lane] : 0xffffffffu;
#pragma unroll 8
      for (int k = 0; k < 32; k++) rank += (__shfl_sync(V2C_FULL, other, k) < val);
    }
    const bool in = jj < L;
    const uint32_t q = val >> 30;
    cnt.x += __popc(__ballot_sync(V2C_FULL, in && q == 0));
    cnt.y += __popc(__ballot_sync(V2C_FULL, in && q == 1));
    cnt.z += __popc(__ballot_sync(V2C_FULL, in && q == 2));
    if (in) perm[rank] = (int32_t)(val & KEY_INDEX);
  }
  return cnt;
}

// One warp per RG consecutive cells: their starts in one read, each cell's
// keys read while the previous cell is ranked, their quarter class starts
// written together; the largest cell count goes to the status counter once
// per block.
constexpr int RG = 8;
__global__ void k_rank(const int32_t *start, long ncell, const uint32_t *tmp, int32_t *perm,
                       int4 *qstart, unsigned long long *stat) {
  __shared__ int bmax;
  if (threadIdx.x == 0) bmax = 0;
  __syncthreads();
  const long c0 = ((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5) * RG;
  const int lane = threadIdx.x & 31;
  if (c0 < ncell) {
    const int sv = (lane <= RG && c0 + lane <= ncell) ? start[c0 + lane] : 0;
    const int ng = (int)min((long)RG, ncell - c0);
    int s = __shfl_sync(V2C_FULL, sv, 0), L = __shfl_sync(V2C_FULL, sv, 1) - s;
    uint32_t val = (lane < L && L <= 32) ? tmp[s + lane] : 0xffffffffu;
    int4 myq = make_int4(0, 0, 0, 0);
    int lmax = 0;
    for (int g = 0; g < ng; g++) {
      // the next cell's keys
      int s1 = 0, L1 = 0;
      uint32_t val1 = 0xffffffffu;
      if (g + 1 < ng) {
        s1 = __shfl_sync(V2C_FULL, sv, g + 1);
        L1 = __shfl_sync(V2C_FULL, sv, g + 2) - s1;
        if (lane < L1 && L1 <= 32) val1 = tmp[s1 + lane];
      }
      lmax = max(lmax, L);
      int4 cnt = make_int4(0, 0, 0, 0);
      if (L > 32) cnt = rank_large(tmp + s, perm + s, L, lane);
      else if (L > 0) cnt = rank_small(val, perm + s, L, lane);
      if (lane == g)
        myq = make_int4(s, s + cnt.x, s + cnt.x + cnt.y, s + cnt.x + cnt.y + cnt.z);
      s = s1; L = L1; val = val1;
    }
    if (lane < ng) qstart[c0 + lane] = myq;
    if (lane == 0) {
      if (lmax > 0) atomicMax(&bmax, lmax);
      if (c0 + ng == ncell) {
        const int e = start[ncell];
        qstart[ncell] = make_int4(e, e, e, e);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && bmax > 0) atomicMax(stat + ST_MAX_CELL, (unsigned long long)bmax);
}

__global__ void k_f64_to_f32(const double *src, float *dst, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}
// FP64 -> float pair hi + lo (hi the nearest float, lo the nearest float to
// the remainder)
__global__ void k_f64_to_pair(const double *src, float *hi, float *lo, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) {
    const double d = src[i];
    const float h = (float)d;
    hi[i] = h;
    lo[i] = (float)(d - (double)h);
  }
}
__global__ void k_unperm_pair(const float *hi, const float *lo, const int32_t *id, double *out,
                              long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[id[i]] = (double)hi[i] + (double)lo[i];
}
template <class T>
__global__ void k_gather(const T *src, const int32_t *perm, T *dst, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[perm[i]];
}
__global__ void k_unperm_f32(const float *src, const int32_t *id, double *out, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[id[i]] = (double)src[i];
}
template <class T>
__global__ void k_unperm(const T *src, const int32_t *id, T *out, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[id[i]] = src[i];
}
__global__ void k_positions(Grid g, Markers m, long n, double *x, double *y) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = m.cell_in[i];
  int ix = c / g.ncy, iy = c - ix * g.ncy;
  int k = m.id[i];
  x[k] = g.gx[ix] + (double)m.u_in[i] * (g.gx[ix + 1] - g.gx[ix]);
  y[k] = g.gy[iy] + (double)m.v_in[i] * (g.gy[iy + 1] - g.gy[iy]);
}

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_assign(const Grid &g, const double *x, const double *y, long n, Markers m,
                   unsigned long long *stat, cudaStream_t st) {
  (void)stat;
  if (n > 0) k_assign<<<nblk(n, 256), 256, 0, st>>>(g, x, y, n, m);
}

long scan_blocks(long m) { return (m + SB * SE - 1) / (SB * SE); }

void launch_scan(const int32_t *in, long m, int32_t *out, int32_t *blocksum, cudaStream_t st) {
  const long nb = scan_blocks(m);
  if (nb > 0) k_scan_block<<<(unsigned)nb, SB, 0, st>>>(in, m, out, blocksum);
  k_scan_sums<<<1, SB, 0, st>>>(blocksum, nb, out + m);
  if (m > 0) k_scan_add<<<nblk(m, 256), 256, 0, st>>>(out, m, blocksum);
}

void launch_sort(const int32_t *cell, const float *u, const float *v, long n, long ncell,
                 SortBufs &b, unsigned long long *stat, cudaStream_t st) {
  cudaMemsetAsync(b.counts, 0, sizeof(int32_t) * ncell, st);
  if (n > 0) k_count<<<nblk(n, 256), 256, 0, st>>>(cell, n, b.counts, b.slot);
  long nb = (ncell + SB * SE - 1) / (SB * SE);
  k_scan_block<<<(unsigned)nb, SB, 0, st>>>(b.counts, ncell, b.start, b.blocksum);
  k_scan_sums<<<1, SB, 0, st>>>(b.blocksum, nb, b.start + ncell);
  k_scan_add<<<nblk(ncell, 256), 256, 0, st>>>(b.start, ncell, b.blocksum);
  uint32_t *keys = reinterpret_cast<uint32_t *>(b.tmp);
  if (n > 0) k_slots<<<nblk(n, 256), 256, 0, st>>>(cell, u, v, n, b.start, b.slot, keys);
  k_rank<<<nblk((ncell + RG - 1) / RG * 32, 256), 256, 0, st>>>(b.start, ncell, keys, b.perm,
                                                                 b.qstart, stat);
}

void launch_f64_to_f32(const double *src, float *dst, long n, cudaStream_t st) {
  if (n > 0) k_f64_to_f32<<<nblk(n, 256), 256, 0, st>>>(src, dst, n);
}
void launch_f64_to_pair(const double *src, float *hi, float *lo, long n, cudaStream_t st) {
  if (n > 0) k_f64_to_pair<<<nblk(n, 256), 256, 0, st>>>(src, hi, lo, n);
}
void launch_unpermute_pair(const float *hi, const float *lo, const int32_t *id, double *out,
                           long n, cudaStream_t st) {
  if (n > 0) k_unperm_pair<<<nblk(n, 256), 256, 0, st>>>(hi, lo, id, out, n);
}
void launch_gather_f32(const float *src, const int32_t *perm, float *dst, long n, cudaStream_t st) {
  if (n > 0) k_gather<float><<<nblk(n, 256), 256, 0, st>>>(src, perm, dst, n);
}
void launch_gather_i32(const int32_t *src, const int32_t *perm, int32_t *dst, long n, cudaStream_t st) {
  if (n > 0) k_gather<int32_t><<<nblk(n, 256), 256, 0, st>>>(src, perm, dst, n);
}
void launch_gather_i8(const int8_t *src, const int32_t *perm, int8_t *dst, long n, cudaStream_t st) {
  if (n > 0) k_gather<int8_t><<<nblk(n, 256), 256, 0, st>>>(src, perm, dst, n);
}
void launch_gather_u8(const uint8_t *src, const int32_t *perm, uint8_t *dst, long n, cudaStream_t st) {
  if (n > 0) k_gather<uint8_t><<<nblk(n, 256), 256, 0, st>>>(src, perm, dst, n);
}
void launch_unpermute_f32(const float *src, const int32_t *id, double *out, long n, cudaStream_t st) {
  if (n > 0) k_unperm_f32<<<nblk(n, 256), 256, 0, st>>>(src, id, out, n);
}
void launch_unpermute_f64(const double *src, const int32_t *id, double *out, long n, cudaStream_t st) {
  if (n > 0) k_unperm<double><<<nblk(n, 256), 256, 0, st>>>(src, id, out, n);
}
void launch_unpermute_i32(const int32_t *src, const int32_t *id, int32_t *out, long n, cudaStream_t st) {
  if (n > 0) k_unperm<int32_t><<<nblk(n, 256), 256, 0, st>>>(src, id, out, n);
}
void launch_unpermute_u8(const uint8_t *src, const int32_t *id, uint8_t *out, long n, cudaStream_t st) {
  if (n > 0) k_unperm<uint8_t><<<nblk(n, 256), 256, 0, st>>>(src, id, out, n);
}
void launch_unpermute_i8(const int8_t *src, const int32_t *id, int8_t *out, long n, cudaStream_t st) {
  if (n > 0) k_unperm<int8_t><<<nblk(n, 256), 256, 0, st>>>(src, id, out, n);
}
void launch_positions(const Grid &g, const Markers &m, long n, double *x, double *y,
                      cudaStream_t st) {
  if (n > 0) k_positions<<<nblk(n, 256), 256, 0, st>>>(g, m, n, x, y);
}

}  // namespace v2c
