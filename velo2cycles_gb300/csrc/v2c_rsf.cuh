// v2c_rsf.cuh -- per-marker visco-elasto-plastic + rate-and-state Newton.
//
// No counterpart in the reference, which couples stress and slip rate only
// through its global Picard loop (momentum_continuity_iterate.c:49-124).
// The per-marker problem is built from the reference's own formulas:
//   ageing-law state after dt    phi(V)      calc_RSF.c:96-103
//   regularised RSF yield        tau_y(V)    calc_RSF.c:128 (+ radiation
//                                            damping 4.3303e6 V, :109-116)
//   visco-plastic viscosity      eta_vp(V)   calc_RSF.c:142
//   Maxwell stress update        tau = 2 eta_vp Z edot + (1-Z) tau_old,
//                                Z = G dt/(G dt + eta_vp)
//                                (momentum_continuity_addmatrix_checkerror.c:380-393)
// "Maxwell stress = yield stress" multiplies out, with T* = tau_old +
// 2 G dt edot, c1 = 1 + G dt/eta and klin = 4.3303e6 c1 + 2 G dt/W, to
//   F(V) = sn a c1 asinh(V/(2V0) e^((mu0 + b phi(V))/a)) + klin V - T* = 0,
// solved for u = log V by Newton safeguarded with the bracket
// [log 1e-40, log(T*/klin)] (F < 0 at the floor, F > 0 at the top because
// asinh > 0).  Relative residual |F| / (F + T*).
//
// Precision split: iterate in FP32 until the FP32 residual stalls near its
// rounding floor, then polish in FP64 to the 1e-10 tolerance.  The FP64
// evaluation follows the oracle (oracle/v2c_oracle.c) expression for
// expression.
#pragma once
#include <math.h>

namespace v2c {

struct RsfState {
  double a, b, L, V0, mu0, sn, dt, phio, Ts, c1, klin;
};

__device__ __forceinline__ void rsf_setup(RsfState &q, double a, double b, double L, double V0,
                                          double mu0, double sn, double dt, double phio,
                                          double tau_old, double edot, double eta, double G,
                                          double W) {
  q.a = a; q.b = b; q.L = L; q.V0 = V0; q.mu0 = mu0; q.sn = sn; q.dt = dt; q.phio = phio;
  q.Ts = tau_old + 2.0 * G * dt * edot;
  q.c1 = 1.0 + G * dt / eta;
  q.klin = 4.3303e+06 * q.c1 + 2.0 * G * dt / W;
}

// FP32 residual F, dF/du and the scale F + T* at u = log V
struct Rsf32 {
  float a, b, L, V0, mu0, sn, dt, phio, ephio, Ts, snac1, klin, lg2V0;
};
__device__ __forceinline__ Rsf32 rsf32_of(const RsfState &q) {
  Rsf32 r;
  r.a = (float)q.a; r.b = (float)q.b; r.L = (float)q.L; r.V0 = (float)q.V0;
  r.mu0 = (float)q.mu0; r.sn = (float)q.sn; r.dt = (float)q.dt; r.phio = (float)q.phio;
  r.ephio = expf(r.phio);
  r.Ts = (float)q.Ts;
  r.snac1 = (float)(q.sn * q.a * q.c1);
  r.klin = (float)q.klin;
  r.lg2V0 = logf(2.f * r.V0);
  return r;
}
__device__ __forceinline__ float rsf_eval32(const Rsf32 &q, float u, float &dF, float &lhs,
                                            float &phi) {
  const float V = __expf(u);
  const float x = V * q.dt / q.L;
  float g, dg;
  if (x <= 1e-6f) {
    g = q.ephio * (1.f - x) + q.V0 * q.dt / q.L;
    dg = -q.ephio * x;
  } else {
    const float r = q.V0 / V, ex = __expf(-x);
    g = r + (q.ephio - r) * ex;
    dg = -r + r * ex - (q.ephio - r) * ex * x;
  }
  phi = __logf(g);
  const float dph = dg / g;
  const float w = u - q.lg2V0 + (q.mu0 + q.b * phi) / q.a;
  const float A = (w > 20.f) ? w + 0.693147180559945f : asinhf(__expf(w));
  const float dA = rsqrtf(1.f + __expf(-2.f * w));
  lhs = q.snac1 * A + q.klin * V;
  dF = q.snac1 * dA * (1.f + q.b / q.a * dph) + q.klin * V;
  return lhs - q.Ts;
}

// FP64 residual, as the oracle's rsf_eval
__device__ __forceinline__ double rsf_eval64(const RsfState &q, double u, double &dF,
                                             double &rel, double &phi) {
  const double V = exp(u);
  const double x = V * q.dt / q.L;
  const double ephio = exp(q.phio);
  double g, dg;
  if (x <= 1e-6) {
    g = ephio * (1 - x) + q.V0 * q.dt / q.L;
    dg = -ephio * x;
  } else {
    const double r = q.V0 / V, ex = exp(-x);
    g = r + (ephio - r) * ex;
    dg = -r + r * ex - (ephio - r) * ex * x;
  }
  phi = log(g);
  const double dph = dg / g;
  const double w = u - log(2.0 * q.V0) + (q.mu0 + q.b * phi) / q.a;
  const double A = (w > 20.0) ? w + 0.69314718055994530942 + 0.25 * exp(-2.0 * w) : asinh(exp(w));
  const double dA = 1.0 / sqrt(1.0 + exp(-2.0 * w));
  const double lhs = q.sn * q.a * q.c1 * A + q.klin * V;
  const double F = lhs - q.Ts;
  dF = q.sn * q.a * q.c1 * dA * (1.0 + q.b / q.a * dph) + q.klin * V;
  rel = fabs(F) / lhs;
  return F;
}

struct RsfResult {
  double V, res;
  float phi;
  int it32, it64;
  bool ok;
};

// FP32 safeguarded Newton from u0; returns the last FP32 iterate.  A step
// below the floor before F(floor) < 0 is known goes to the floor itself.
__device__ __forceinline__ float rsf_newton32(const Rsf32 &q, float u0, float ulo, float uhi,
                                              int maxit, int &iters) {
  const float floor_u = ulo;
  float u = fminf(fmaxf(u0, ulo + 1e-3f * (uhi - ulo)), uhi - 1e-3f * (uhi - ulo));
  if (!(u == u)) u = 0.5f * (ulo + uhi);
  bool lo_known = false;
  iters = 0;
  for (int it = 0; it < maxit; it++) {
    float dF, lhs, phi;
    const float F = rsf_eval32(q, u, dF, lhs, phi);
    iters++;
    // FP32 rounding floor of the residual is a few 1e-7 of lhs
    if (fabsf(F) <= 2e-6f * lhs) break;
    if (u == floor_u && F >= 0.f) break;  // the FP64 polish confirms the floor
    if (F < 0.f) { ulo = u; lo_known = true; } else uhi = u;
    float un = u - F / dF;
    if (!lo_known && dF > 0.f && !(un > ulo)) un = floor_u;
    else if (!(dF > 0.f) || !(un > ulo) || !(un < uhi)) un = 0.5f * (ulo + uhi);
    if (fabsf(un - u) <= 1e-6f * fmaxf(1.f, fabsf(u))) { u = un; break; }
    u = un;
  }
  return u;
}

// FP64 polish from u to the relative tolerance, same rules as the oracle
__device__ __forceinline__ bool rsf_polish64(const RsfState &q, double u, double rtol, int maxit,
                                             double &V, double &res, float &phi, int &iters) {
  const double floor_u = log(1e-40);
  double ulo = floor_u, uhi = log(q.Ts / q.klin);
  if (!(u > ulo + 1e-6)) u = floor_u;  // an FP32 floor iterate is the floor
  if (!(u < uhi)) u = uhi - (uhi - ulo) * 1e-3;
  bool lo_known = false;
  iters = 0;
  res = 1.0;
  for (int it = 0; it < maxit; it++) {
    double dF, rel, ph;
    const double F = rsf_eval64(q, u, dF, rel, ph);
    iters++;
    if (rel <= rtol) {
      V = exp(u); res = rel; phi = (float)ph;
      return true;
    }
    if (u == floor_u && F >= 0) {
      V = 1e-40; res = 0; phi = (float)ph;
      return true;
    }
    if (F < 0) { ulo = u; lo_known = true; } else uhi = u;
    double un = u - F / dF;
    if (!lo_known && dF > 0 && !(un > ulo)) un = floor_u;
    else if (!(dF > 0) || !(un > ulo) || !(un < uhi)) un = 0.5 * (ulo + uhi);
    u = un;
    res = rel;
  }
  V = exp(u);
  return false;
}

// Full solve from a start u0 (FP32 phase then FP64 polish).  Degenerate
// loads (T* <= 0, or the 1e-40 floor already above the load) return the
// floor with zero iterations, as the oracle does.
__device__ __forceinline__ RsfResult rsf_solve(const RsfState &q, float u0, double rtol,
                                               int maxit) {
  RsfResult r;
  r.it32 = r.it64 = 0;
  r.ok = true;
  r.res = 0;
  r.phi = (float)q.phio;
  if (!(q.Ts > 0)) { r.V = 1e-40; return r; }
  const double uhi = log(q.Ts / q.klin), ulo = log(1e-40);
  if (uhi <= ulo) { r.V = 1e-40; return r; }
  const Rsf32 q32 = rsf32_of(q);
  const float u32 = rsf_newton32(q32, u0, (float)ulo, (float)uhi, maxit, r.it32);
  r.ok = rsf_polish64(q, (double)u32, rtol, maxit, r.V, r.res, r.phi, r.it64);
  return r;
}

}  // namespace v2c
