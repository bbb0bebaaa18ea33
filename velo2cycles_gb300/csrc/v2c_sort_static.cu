// v2c_sort_static.cu -- cell assignment + stable counting sort by cell that
// allocates nothing (v2c_sort_cells_static in include/v2c.h).
//
// Same results as the context path (k_assign + the counting sort of
// v2c_sort.cu): the cell of every marker from the FP64 bisection of
// nxsearch/nysearch (interpolation.c:1536-1573), and the markers of each
// cell in ascending array index.  The difference is where the scratch lives.
// The context path keeps per-cell counters and per-marker slot/rank buffers
// in memory it allocates at v2c_create; this variant keeps its only scratch,
// the per-cell counters and the scan's block sums, in the file-scope array
// g_scratch below, and orders each cell's segment of the caller's perm in
// place, so it needs no per-marker scratch at all.
//
// g_scratch is one array per device (module-scope __device__ storage).
// Calls that overlap on one device -- two streams, two host threads, or a
// call on one stream while another is still running on another -- race on
// it and produce wrong counts; calls must be ordered (one stream, or events).
#include <climits>
#include <cstdio>
#include <mutex>

#include "v2c_internal.cuh"

namespace v2c {

namespace {

constexpr int SB = 1024, SE = 4;  // scan: 1024 threads x 4 counters per block
constexpr long MAX_CELLS = V2C_STATIC_SORT_MAX_CELLS;
constexpr long MAX_BLOCKS = (MAX_CELLS + SB * SE - 1) / (SB * SE);
constexpr long SCRATCH_WORDS = MAX_CELLS + MAX_BLOCKS;  // counters, then block sums

// 4 Mi counters + 1 Ki block sums = 16 MiB + 4 KiB per device.  The counters
// must be zero before the counting pass and again before the fill pass; every
// call zeroes them itself on its stream, so nothing has to be zero on entry.
static __device__ __align__(256) int32_t g_scratch[SCRATCH_WORDS];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
int32_t *g_scratch_ptr[MAX_DEVICES] = {};

__global__ void k_assign_count(const double *gx, int xn, const double *gy, int yn,
                               const double *x, const double *y, long n, int32_t *cell,
                               int32_t *count) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ix = nsearch64(gx, xn, x[i]), iy = nsearch64(gy, yn, y[i]);
  const int c = ix * (yn - 1) + iy;
  cell[i] = c;
  atomicAdd(count + c, 1);
}

__global__ void k_scan_block_s(const int32_t *in, long m, int32_t *out, int32_t *bsum) {
  __shared__ int32_t sh[SB];
  const long base = (long)blockIdx.x * SB * SE + (long)threadIdx.x * SE;
  int32_t v[SE], s = 0;
#pragma unroll
  for (int k = 0; k < SE; k++) {
    v[k] = (base + k < m) ? in[base + k] : 0;
    s += v[k];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < SB; off <<= 1) {
    const int32_t t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
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

// exclusive scan of at most SB block sums in one block; the total goes to
// *total (start[ncell])
__global__ void k_scan_sums_s(int32_t *bsum, int nb, int32_t *total) {
  __shared__ int32_t sh[SB];
  const int32_t v = (threadIdx.x < nb) ? bsum[threadIdx.x] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < SB; off <<= 1) {
    const int32_t t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (threadIdx.x < nb) bsum[threadIdx.x] = sh[threadIdx.x] - v;
  if (threadIdx.x == SB - 1) *total = sh[SB - 1];
}

__global__ void k_scan_add_s(int32_t *out, long m, const int32_t *bsum) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < m) out[i] += bsum[i / (SB * SE)];
}

// every marker takes a slot in its cell's segment (slot order is whatever
// the atomics give; k_order_cells makes it index order)
__global__ void k_fill(const int32_t *cell, long n, const int32_t *start, int32_t *cursor,
                       int32_t *perm) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  perm[start[c] + atomicAdd(cursor + c, 1)] = (int32_t)i;
}

// One warp per cell sorts the cell's segment of perm ascending, in place.
// Up to 32 entries: rank in registers, then write.  Longer segments: a
// bitonic network in the form whose every compare puts the smaller value at
// the lower position (first stage of each merge compares a with its mirror
// in the block), so positions past the segment act as +infinity and are
// never touched.  Every position is in one pair per stage; __syncwarp()
// orders the stages' global-memory accesses among the warp's lanes.
__global__ void k_order_cells(const int32_t *start, long ncell, int32_t *perm) {
  const long c = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;  // uniform across the warp
  const int s = start[c], L = start[c + 1] - s;
  if (L < 2) return;
  int32_t *p = perm + s;
  if (L <= 32) {
    const int32_t v = (lane < L) ? p[lane] : INT_MAX;
    int rank = 0;
#pragma unroll
    for (int k = 0; k < 32; k++) rank += (__shfl_sync(V2C_FULL, v, k) < v);
    __syncwarp();
    if (lane < L) p[rank] = v;  // marker indices are distinct
    return;
  }
  int P = 64;
  while (P < L) P <<= 1;
  for (int k = 2; k <= P; k <<= 1) {
    const int h = k >> 1;
    for (int i = lane; i < P / 2; i += 32) {
      const int blk = i / h, off = i - blk * h;
      const int a = blk * k + off, b = blk * k + k - 1 - off;
      if (b < L) {
        const int32_t va = p[a], vb = p[b];
        if (va > vb) { p[a] = vb; p[b] = va; }
      }
    }
    __syncwarp();
    for (int j = k >> 2; j >= 1; j >>= 1) {
      for (int i = lane; i < P / 2; i += 32) {
        const int blk = i / j, off = i - blk * j;
        const int a = blk * 2 * j + off, b = a + j;
        if (b < L) {
          const int32_t va = p[a], vb = p[b];
          if (va > vb) { p[a] = vb; p[b] = va; }
        }
      }
      __syncwarp();
    }
  }
}

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

// Set-up, once per device, with that device current: the device address of
// g_scratch.  This may load the module on the device, so a caller that
// captures streams makes its first call on each device before capturing.
int scratch_for_current_device(int32_t **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return V2C_ERR_CUDA;
  if (dev < 0 || dev >= MAX_DEVICES) return V2C_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "v2c_sort_cells_static: cudaGetSymbolAddress failed on device %d: %s\n",
              dev, cudaGetErrorString(e));
      return V2C_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<int32_t *>(p);
  }
  *out = g_scratch_ptr[dev];
  return V2C_OK;
}

}  // namespace

}  // namespace v2c

using namespace v2c;

extern "C" int v2c_sort_cells_static(const double *gx_dev, long xnumx, const double *gy_dev,
                                     long ynumy, const double *x_dev, const double *y_dev,
                                     long n, int32_t *cell_dev, int32_t *perm_dev,
                                     int32_t *start_dev, void *cuda_stream) {
  // sizes first: nothing below the limits reaches the device.  Each factor
  // is bounded before the product is formed, so no size overflows `long` or
  // the int the kernels take.
  if (xnumx < 2 || ynumy < 2 || n < 0 || n > INT_MAX) return V2C_ERR_ARG;
  if (xnumx - 1 > MAX_CELLS || ynumy - 1 > MAX_CELLS / (xnumx - 1)) {
    fprintf(stderr,
            "v2c_sort_cells_static: %ld x %ld grid lines give more than the %ld cells "
            "(V2C_STATIC_SORT_MAX_CELLS) its fixed scratch holds; use the context path\n",
            xnumx, ynumy, MAX_CELLS);
    return V2C_ERR_CAPACITY;
  }
  const long ncell = (xnumx - 1) * (ynumy - 1);
  if (!gx_dev || !gy_dev || !start_dev || (n > 0 && (!x_dev || !y_dev || !cell_dev || !perm_dev)))
    return V2C_ERR_ARG;
  // An error another caller left pending would be reported as this call's
  // own by the checks after each launch below: refuse to start instead, and
  // leave that error in place for its owner.
  if (cudaPeekAtLastError() != cudaSuccess) {
    fprintf(stderr, "v2c_sort_cells_static: an earlier CUDA error is pending (%s); not started\n",
            cudaGetErrorString(cudaPeekAtLastError()));
    return V2C_ERR_CUDA;
  }
  int32_t *scratch = nullptr;
  if (int rc = scratch_for_current_device(&scratch)) return rc;
  int32_t *count = scratch, *bsum = scratch + MAX_CELLS;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  // status of the launch just queued (nothing was pending on entry)
  auto launched = []() { return cudaGetLastError() == cudaSuccess; };

  if (cudaMemsetAsync(count, 0, sizeof(int32_t) * ncell, st) != cudaSuccess) return V2C_ERR_CUDA;
  if (n > 0) {
    k_assign_count<<<nblk(n, 256), 256, 0, st>>>(gx_dev, (int)xnumx, gy_dev, (int)ynumy, x_dev,
                                                 y_dev, n, cell_dev, count);
    if (!launched()) return V2C_ERR_CUDA;
  }
  const long nb = (ncell + SB * SE - 1) / (SB * SE);
  k_scan_block_s<<<(unsigned)nb, SB, 0, st>>>(count, ncell, start_dev, bsum);
  if (!launched()) return V2C_ERR_CUDA;
  k_scan_sums_s<<<1, SB, 0, st>>>(bsum, (int)nb, start_dev + ncell);
  if (!launched()) return V2C_ERR_CUDA;
  k_scan_add_s<<<nblk(ncell, 256), 256, 0, st>>>(start_dev, ncell, bsum);
  if (!launched()) return V2C_ERR_CUDA;
  if (n > 0) {
    if (cudaMemsetAsync(count, 0, sizeof(int32_t) * ncell, st) != cudaSuccess) return V2C_ERR_CUDA;
    k_fill<<<nblk(n, 256), 256, 0, st>>>(cell_dev, n, start_dev, count, perm_dev);
    if (!launched()) return V2C_ERR_CUDA;
    k_order_cells<<<nblk(ncell * 32, 256), 256, 0, st>>>(start_dev, ncell, perm_dev);
    if (!launched()) return V2C_ERR_CUDA;
  }
  return V2C_OK;
}
