// v2c_internal.cuh -- device data layout and shared helpers of the GB300
// marker-in-cell step.
//
// HBM layout (one context):
//  * markers, structure of arrays, physically sorted by cell at upload and
//    updated in place afterwards; a per-step permutation `perm` lists them in
//    (cell, array index) order.  Position = int32 cell (ix*(ynumy-1)+iy) +
//    FP32 in-cell offsets (u, v); u, v in [0,1) inside the grid, outside
//    [0,1] only for markers beyond the domain edge.  cell/u/v are double
//    buffered so a kernel can move markers while neighbouring tiles still
//    read the old positions.
//  * node fields, FP32, [V2C_NF_N][nodenum], y fastest (m3 = m1*ynumy+m2),
//    the reference's own layout; they are converted to and from FP64 only
//    when they cross the C ABI.  (GB300 runs FP64 -- conversions included --
//    at 1/64 of the FP32 rate, so FP64 inside the per-marker and per-node
//    loops would dominate the step.)
//  * grid: FP64 lines plus FP32 cell widths for cell-local arithmetic.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/v2c.h"

#define V2C_FULL 0xffffffffu

namespace v2c {

// ------------------------------------------------------------ rock table
// FP32 copies and derived constants of the per-type coefficients.
// The _LO entries are the low words of float pairs (hi + lo, ~48 bits) for
// the constants of the Arrhenius exponent, whose rounding to FP32 alone would
// change the viscosity by several parts in 1e6 (see ductile_visc32).
enum {
  RK_GG = 0, RK_INV_GG, RK_NU, RK_LNNU, RK_DH, RK_DV, RK_LNSS, RK_MM,
  RK_RO, RK_BB, RK_AA, RK_CP, RK_KT, RK_HT, RK_KF, RK_KP, RK_LN_N0, RK_LN_N1,
  RK_N0, RK_N1, RK_KIND, RK_IM,
  RK_DH_LO, RK_DV_LO,      // activation energy and volume, low words
  RK_LNK, RK_LNK_LO,       // ln(0.5 nu / ss^(mm-1)), the diffusion-creep prefactor
  RK_LNG, RK_LNG_LO,       // ln G
  RK_SS, RK_SS_LO,         // ss
  RK_EM, RK_EM_LO,         // (mm-1)/mm
  RK_MM1, RK_MM1_LO,       // mm-1
  RK_LNSS_LO,              // low word of ln ss
  RK_N
};
enum { VISC_NEWTON = 0, VISC_POWER = 1, VISC_STICKY = 2, VISC_UNDEF = 3 };

struct Rock {
  const float *f;  // [RK_N][V2C_MAXTMR]
  __device__ __forceinline__ float operator()(int k, int t) const {
    return __ldg(f + k * V2C_MAXTMR + t);
  }
};

// --------------------------------------------------------------- markers
struct Markers {
  int32_t *cell_in, *cell_out;
  float *u_in, *u_out, *v_in, *v_out;
  int32_t *id;
  int8_t *type;
  uint8_t *flags;  // bit0: out-of-grid reset (markd = markw = -1)
  // tk + tk_lo is the temperature as a float pair: the power-law viscosity
  // depends on exp(E/RT) with E/RT up to ~50, so a temperature rounded to
  // FP32 (6e-8) alone would move it by ~3e-6
  float *tk, *e, *p, *sxx, *sxy, *exx, *exy, *vx, *vy, *phi, *coh, *slipv;
  float *tk_lo;
  // markv as a float pair: the y anchor of an immobile marker (type >= 100,
  // whose markk holds the x anchor), moveandrotatemarkers.c:127-133
  float *mv, *mv_lo;
  float *mnu, *mkt, *mro;  // per-step results of the marker physics kernel
};
// RESET: out-of-grid reset, markd = markw = -1; DNEG: markd = -1 only (a
// marker appended or refilled by the immobile-marker rule)
enum { MFLAG_RESET = 1, MFLAG_DNEG = 2 };

// ------------------------------------------------------------------ grid
struct Grid {
  const double *gx, *gy;  // lines
  const float *wx, *wy;   // cell widths (ncx, ncy)
  int xn, yn, ncx, ncy;
  long nn;
  double xsize, ysize;
};

struct Nodes {
  float *base;
  long nn;
  __host__ __device__ __forceinline__ float *f(int k) const { return base + (long)k * nn; }
};

// scalar parameters the kernels read, converted once per call on the host
struct Scal {
  v2c_params p;
  int antid;        // timesum > 0 && antidiffinter == 1
  int phi_reset0;   // timesum == timestep (calc_RSF.c:287)
  int sticky_cap;   // stickymod == 1 && timesum > 4e7
  float dt;
  float sticky_nu;  // markgg[2]*timestep/100
  float ln_nubeg, ln_nuend;
  // FP32 copies of the double parameters that per-marker and per-node code
  // reads, rounded once here: in a kernel every double->float conversion or
  // double compare issues on the FP64 pipe, 1/64 of the FP32 rate on this GPU
  float fault_y_f, fault_slope_f;
  float fault_hw1_f;  // (float)fault_hw + 1: far-field test margin
  float a_hr_f, b_hr_f, L_hr_f, V0_hr_f;
  float tdeep_f, zdeep_f;
  float zdeep_lo_f;   // (float)zdeep - 1 - 1e-6 |zdeep|: coarse depth test
  float eps2_f, nstress_f, nubeg_f, nuend_f, faultwidth_f;
  float dt_hi, dt_lo, W_hi, W_lo, sn_hi, sn_lo;  // float-float timestep, faultwidth, nstress
  float lndt_hi, lndt_lo;  // ln timestep as a float pair (-inf when timestep <= 0)
  float eps2_lo, tdeep_lo; // low words of the temperatures markers are reset to
  int sppe_nstress;   // timesum == 0 && reloadfromDP == 0 && compressiblemode == 1
  int timesum_pos;    // timesum > 0
  int timesum_zero;   // timesum == 0
};

// ----------------------------------------------------- compensated sums
// Neumaier two-sum accumulator in FP32: (s, c) carries a sum to about twice
// FP32 precision; value() rounds it once.
struct Acc {
  float s, c;
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    float e = (fabsf(s) >= fabsf(x)) ? (s - t) + x : (x - t) + s;
    c += e;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

// The centre-node weight factor 1 - 2|f - 1/2| of an in-cell offset f
// (interpolation.c:620-622), written as 2f below the middle and 2(1 - f)
// above it: the same value, exact in FP32 (1 - f is exact for f >= 1/2),
// where the literal form loses the low bits of a marker near the cell edge
// -- whose weight is then tiny but whose viscosity may be 1e6 times its
// neighbours' and decide the node's average.
__device__ __forceinline__ float tent(float f) { return f < 0.5f ? 2.f * f : 2.f * (1.f - f); }

// --------------------------------------------------- cell-local geometry
// Offsets of the grid lines i-1 .. i+2 relative to line i, in FP32.
struct Axis {
  int i;      // cell index along the axis
  float X;    // position relative to line i, metres
  float w;    // width of cell i
  float gm1, g1, g2;  // line offsets of i-1, i+1, i+2
  __device__ __forceinline__ float G(int k) const {
    return k <= -1 ? gm1 : (k == 0 ? 0.f : (k == 1 ? g1 : g2));
  }
};

__device__ __forceinline__ Axis make_axis(const float *w, int nc, int i, float X) {
  Axis a;
  a.i = i;
  a.X = X;
  a.w = __ldg(w + i);
  a.gm1 = (i > 0) ? -__ldg(w + i - 1) : -a.w;
  a.g1 = a.w;
  a.g2 = (i + 1 < nc) ? a.w + __ldg(w + i + 1) : 2.f * a.w;
  return a;
}

// Move a local position to the cell containing it (FP32 cell walk).  Cells
// are clamped to [0, nc-1]; returns false when more than `maxsteps` cells
// would be crossed (the caller then falls back to an FP64 search).
__device__ __forceinline__ bool relocate(const float *w, int nc, int &i, float &X,
                                         int maxsteps) {
  for (int s = 0; s < maxsteps; s++) {
    float wi = __ldg(w + i);
    if (X >= wi && i < nc - 1) {
      X -= wi;
      i++;
    } else if (X < 0.f && i > 0) {
      i--;
      X += __ldg(w + i);
    } else {
      return true;
    }
  }
  float wi = __ldg(w + i);
  return !((X >= wi && i < nc - 1) || (X < 0.f && i > 0));
}

// nxsearch (interpolation.c:1536-1554) in FP64: largest l with g[l] <= x,
// clamped to n-2.
__device__ __forceinline__ int nsearch64(const double *g, int n, double x) {
  int lo = 0, hi = n - 1;
  do {
    int c = (lo + hi) / 2;
    if (__ldg(g + c) > x) hi = c; else lo = c;
  } while (hi - lo > 1);
  return lo > n - 2 ? n - 2 : lo;
}

// Offset within a cell rounded to FP32 without crossing 0.5 or 1.0: the
// scatter kernels branch on u < 0.5 / u > 0.5 and the in-grid tests on
// u < 1, so the FP32 offset must land on the same side as the FP64 one.
__device__ __forceinline__ float offset32(double u) {
  float f = (float)u;
  if (u < 0.5 && f >= 0.5f) f = nextafterf(0.5f, 0.f);
  if (u > 0.5 && f <= 0.5f) f = nextafterf(0.5f, 1.f);
  if (u < 1.0 && f >= 1.0f) f = nextafterf(1.0f, 0.f);
  if (u > 1.0 && f <= 1.0f) f = nextafterf(1.0f, 2.f);
  if (u > 0.0 && f <= 0.0f) f = 1e-30f;
  if (u < 0.0 && f >= 0.0f) f = -1e-30f;
  return f;
}

// ---------------------------------------------------------- device status
// Counters read back by v2c_get_status (64-bit, integer atomics only).
enum {
  ST_OUT_OF_GRID = 0, ST_FAR_MOVES, ST_NAN, ST_NEWTON_ITERS, ST_NEWTON_FALLBACK,
  ST_NEWTON_NONCONV, ST_NEWTON_MAXRES_BITS, ST_MAX_CELL, ST_N
};

}  // namespace v2c
