// v2c_temp.cu -- the marker part of solve_temperature
// (temperature_iterate.c:181-412), after the host's thermal solve.
//
// Node TK holds the solved temperature, TK2 the one before the solve.  Three
// passes over the cell-sorted markers:
//   1. per marker: fluid markers (type 50..99) take the solved temperature;
//      rock markers (type < 50) strictly inside the model start from the old
//      one when their temperature is not positive (at least tdeep), get the
//      subgrid diffusion towards it (heatdif > 0) and the solution's change;
//      the diffusion change and its weight are kept per sorted position;
//   2. per cell: the weighted diffusion changes of the cell's markers summed
//      in sorted order with two-sum compensation and normalised, stored at the
//      cell's upper-left node (the reference adds each marker to that one
//      node only, temperature_iterate.c:306-335);
//   3. per marker: the antidiffusion, minus that node value times the
//      marker's weight at the node.
// Marker temperatures are float pairs (tk + tk_lo) and are updated in FP64
// (a few FP64 operations per marker, outside the MIC step): the viscosity
// amplifies a temperature error about fifty-fold.  The node temperatures
// are read from their FP64 copies when the host uploaded TK and TK2 since
// the last marker2nodes, so a marker that takes the solved temperature, or
// its change TK - TK2, takes it at FP64 precision.
#include <math.h>

#include "v2c_kernels.h"

namespace v2c {

namespace {

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

// strictly inside the model (temperature_iterate.c:202,223): the FP64
// position decides only in the cells on the model's edge
__device__ __forceinline__ bool inside_model(const Grid &g, int ix, int iy, float u, float v) {
  bool in = true;
  if (ix == 0 || ix == g.ncx - 1) {
    const double x = g.gx[ix] + (double)u * (g.gx[ix + 1] - g.gx[ix]);
    in = in && x > 0 && x < g.xsize;
  }
  if (iy == 0 || iy == g.ncy - 1) {
    const double y = g.gy[iy] + (double)v * (g.gy[iy + 1] - g.gy[iy]);
    in = in && y > 0 && y < g.ysize;
  }
  return in;
}

__global__ void k_temp_markers(TempArgs a) {
  const Grid &g = a.g;
  const long yn = g.yn;
  const float *tk = a.N.f(V2C_NF_TK), *tk2 = a.N.f(V2C_NF_TK2);
  const float *kt = a.N.f(V2C_NF_KT), *cp = a.N.f(V2C_NF_CP), *ro = a.N.f(V2C_NF_RO);
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < a.n;
       s += (long)gridDim.x * blockDim.x) {
    a.dtk1[s] = 0.f;
    a.wt[s] = 0.f;
    const int idx = __ldg(a.perm + s);
    const int c = a.m.cell_in[idx];
    const int ix = c / g.ncy, iy = c - ix * g.ncy;
    const float u = a.m.u_in[idx], v = a.m.v_in[idx];
    const int t = a.m.type[idx];
    if (t >= 100 || !inside_model(g, ix, iy, u, v)) continue;
    // interpolate_temperature (interpolation.c:1492-1533) in the marker's cell
    const long m3 = (long)ix * yn + iy;
    const float d0 = (1.f - u) * (1.f - v), d1 = (1.f - u) * v, d2 = u * (1.f - v), d3 = u * v;
    double TK, TK2;
    if (a.tk64 && a.tk2_64) {
      const double *p = a.tk64, *q = a.tk2_64;
      TK = (double)d0 * p[m3] + (double)d1 * p[m3 + 1] + (double)d2 * p[m3 + yn] +
           (double)d3 * p[m3 + yn + 1];
      TK2 = (double)d0 * q[m3] + (double)d1 * q[m3 + 1] + (double)d2 * q[m3 + yn] +
            (double)d3 * q[m3 + yn + 1];
    } else {
      TK = d0 * tk[m3] + d1 * tk[m3 + 1] + d2 * tk[m3 + yn] + d3 * tk[m3 + yn + 1];
      TK2 = d0 * tk2[m3] + d1 * tk2[m3 + 1] + d2 * tk2[m3 + yn] + d3 * tk2[m3 + yn + 1];
    }
    double mk;
    if (t >= 50) {
      mk = TK;
    } else {
    mk = (double)a.m.tk[idx] + (double)a.m.tk_lo[idx];
    if (mk <= 0.0) mk = TK2 < a.tdeep64 ? a.tdeep64 : TK2;  // newly arrived marker
    if (a.heatdif != 0.f) {
      const float wx = __ldg(g.wx + ix), wy = __ldg(g.wy + iy);
      // node order of the reference's loop: m1 outer, m2 inner
      const float mkt = kt[m3] * d0 + kt[m3 + 1] * d1 + kt[m3 + yn] * d2 + kt[m3 + yn + 1] * d3;
      const float mrocp = cp[m3] * ro[m3] * d0 + cp[m3 + 1] * ro[m3 + 1] * d1 +
                          cp[m3 + yn] * ro[m3 + yn] * d2 + cp[m3 + yn + 1] * ro[m3 + yn + 1] * d3;
      float e = -a.heatdif * mkt / mrocp * 2.f * (1.f / (wx * wx) + 1.f / (wy * wy)) * a.dt;
      if (e < -150.f) e = -150.f;
      const float dtk1 = -(float)(TK2 - mk) * expm1f(e);  // dtk (1 - exp(e))
      mk += dtk1;
      a.dtk1[s] = dtk1;
      a.wt[s] = d0 / (wx * wy);
    }
    mk += TK - TK2;
    }
    const float hi = (float)mk;
    a.m.tk[idx] = hi;
    a.m.tk_lo[idx] = (float)(mk - (double)hi);
  }
}

// per cell: the normalised diffusion change at its upper-left node
__global__ void k_temp_cells(TempArgs a) {
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= a.ncell) return;
  const int b = __ldg(a.start + c), e = __ldg(a.start + c + 1);
  Acc w, d;
  w.zero();
  d.zero();
  for (int s = b; s < e; s++) {
    const float ws = a.wt[s];
    if (ws != 0.f) {
      w.add(ws);
      d.add(a.dtk1[s] * ws);
    }
  }
  const float ws = w.value();
  const int ix = (int)(c / a.g.ncy), iy = (int)(c - (long)ix * a.g.ncy);
  a.tol[(long)ix * a.g.yn + iy] = ws != 0.f ? d.value() / ws : 0.f;
}

__global__ void k_temp_anti(TempArgs a) {
  const Grid &g = a.g;
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < a.n;
       s += (long)gridDim.x * blockDim.x) {
    if (a.wt[s] == 0.f) continue;  // rock markers inside the model only
    const int idx = __ldg(a.perm + s);
    const int c = a.m.cell_in[idx];
    const int ix = c / g.ncy, iy = c - ix * g.ncy;
    const float t = a.tol[(long)ix * g.yn + iy];
    if (t != 0.f) {
      const float u = a.m.u_in[idx], v = a.m.v_in[idx];
      const double mk = (double)a.m.tk[idx] + (double)a.m.tk_lo[idx] -
                        (double)(t * ((1.f - u) * (1.f - v)));
      const float hi = (float)mk;
      a.m.tk[idx] = hi;
      a.m.tk_lo[idx] = (float)(mk - (double)hi);
    }
  }
}

}  // namespace

void launch_temperature(const TempArgs &a, cudaStream_t st) {
  cudaMemsetAsync(a.tol, 0, sizeof(float) * a.g.nn, st);
  if (a.n <= 0) return;
  const unsigned gb = nblk(a.n, 256) < 152 * 16 ? nblk(a.n, 256) : 152 * 16;
  k_temp_markers<<<gb, 256, 0, st>>>(a);
  if (a.heatdif == 0.f) return;
  k_temp_cells<<<nblk(a.ncell, 256), 256, 0, st>>>(a);
  k_temp_anti<<<gb, 256, 0, st>>>(a);
}

}  // namespace v2c
