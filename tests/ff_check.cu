// Test program for velo2cycles_gb300/csrc/v2c_ff.cuh (built and run by
// tests/test_gpu_ff.py): float-float exp, log, div and sqrt of the FP64
// inputs in a binary file, each result written as (hi, lo) float pairs.
//   ff_check <in.bin> <out.bin>
// in.bin: int64 n, then n doubles x, then n doubles y.
// out.bin: for each of exp(x), log(|x|), x/y, sqrt(|x|): n (hi, lo) pairs.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../velo2cycles_gb300/csrc/v2c_ff.cuh"

using namespace v2c;

__global__ void k_check(const double *x, const double *y, long n, float2 *out) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ff a = ff_from_double(x[i]), b = ff_from_double(y[i]);
  const ff aa = ff_from_double(fabs(x[i]));
  ff r[4] = {ff_exp(a), ff_log(aa), ff_div(a, b), ff_sqrt(aa)};
  for (int k = 0; k < 4; k++) out[k * n + i] = make_float2(r[k].hi, r[k].lo);
}

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  long long n = 0;
  if (fread(&n, 8, 1, f) != 1 || n <= 0 || n > (1 << 24)) return 4;
  std::vector<double> h(2 * n);
  if (fread(h.data(), 8, 2 * n, f) != (size_t)(2 * n)) return 5;
  fclose(f);
  double *d;
  float2 *o;
  if (cudaMalloc(&d, 16 * n) != cudaSuccess || cudaMalloc(&o, 32 * n) != cudaSuccess) return 6;
  cudaMemcpy(d, h.data(), 16 * n, cudaMemcpyHostToDevice);
  k_check<<<(unsigned)((n + 255) / 256), 256>>>(d, d + n, n, o);
  std::vector<float2> ho(4 * n);
  if (cudaMemcpy(ho.data(), o, 32 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  FILE *g = fopen(argv[2], "wb");
  if (!g) return 8;
  fwrite(ho.data(), 8, 4 * n, g);
  fclose(g);
  cudaFree(d);
  cudaFree(o);
  return 0;
}
