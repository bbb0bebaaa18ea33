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
// Two forms:
//  * FP64 (rsf_newton64): the whole Newton in FP64, step for step the
//    oracle's v2c_oracle_rsf_newton1 -- the straightforward GPU form.
//  * split (rsf_solve_split): FP32 Newton until the FP32 residual reaches its
//    rounding floor, then Newton steps with the residual evaluated in
//    float-float (v2c_ff.cuh, ~48 bits, relative error ~1e-13) until
//    |F|/(F+T*) <= rtol; the converged residual is formed in FP64 from the
//    float-float terms.  GB300 runs FP64 at 1/64 of the FP32 rate, so the
//    FP64 transcendentals are what the split form removes.  If the
//    float-float phase does not converge in a few steps, the FP64 Newton
//    finishes from its last iterate.
#pragma once
#include <math.h>

#include "v2c_ff.cuh"

namespace v2c {

constexpr double RSF_ETA_RAD = 4.3303e+06;  // radiation damping, calc_RSF.c:109-116
constexpr double RSF_LOG_FLOOR = -92.103403719761836;  // log(1e-40)

// ----------------------------------------------------------------- inputs
// One state in float-float (exact copies of FP64 or FP32 inputs).
struct RsfIn {
  ff a, b, L, V0, mu0, sn, dt, phio, tau_old, edot, eta, G, W;
};

// ------------------------------------------------------------ FP64 form
struct RsfState {
  double a, b, L, V0, mu0, sn, dt, phio, Ts, c1, klin;
};

__device__ __forceinline__ void rsf_setup64(RsfState &q, const RsfIn &in) {
  q.a = ff_to_double(in.a); q.b = ff_to_double(in.b); q.L = ff_to_double(in.L);
  q.V0 = ff_to_double(in.V0); q.mu0 = ff_to_double(in.mu0); q.sn = ff_to_double(in.sn);
  q.dt = ff_to_double(in.dt); q.phio = ff_to_double(in.phio);
  const double G = ff_to_double(in.G), eta = ff_to_double(in.eta);
  q.Ts = ff_to_double(in.tau_old) + 2.0 * G * q.dt * ff_to_double(in.edot);
  q.c1 = 1.0 + G * q.dt / eta;
  q.klin = RSF_ETA_RAD * q.c1 + 2.0 * G * q.dt / ff_to_double(in.W);
}

// F, dF/du, relative residual, phi and the friction term A = asinh(..) at
// u = log V; the oracle's rsf_eval expression for expression
__device__ __forceinline__ double rsf_eval64(const RsfState &q, double u, double &dF,
                                             double &rel, double &phi, double &A) {
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
  A = (w > 20.0) ? w + 0.69314718055994530942 + 0.25 * exp(-2.0 * w) : asinh(exp(w));
  const double dA = 1.0 / sqrt(1.0 + exp(-2.0 * w));
  const double lhs = q.sn * q.a * q.c1 * A + q.klin * V;
  const double F = lhs - q.Ts;
  dF = q.sn * q.a * q.c1 * dA * (1.0 + q.b / q.a * dph) + q.klin * V;
  rel = fabs(F) / lhs;
  return F;
}

struct RsfResult {
  double V, res, A;  // slip rate, relative residual, friction term at V
  float Vf;          // slip rate in FP32 (what a marker stores)
  float phi;
  int it32, itff, it64;
  bool ok;
};

// Safeguarded FP64 Newton from u (the oracle's v2c_oracle_rsf_newton1
// rules).  `snap_floor`: an iterate handed over from the FP32 phase at the
// floor is taken as the floor itself.
// Kept out of line: the split form reaches it only as a rare fallback, and
// its FP64 library code would otherwise crowd the hot loop's instructions.
static __device__ __noinline__ void rsf_newton64(const RsfState &q, double u, double rtol, int maxit,
                                          bool snap_floor, RsfResult &r) {
  r.it64 = 0;
  r.ok = false;
  double ulo = RSF_LOG_FLOOR, uhi = log(q.Ts / q.klin);
  const double floor_u = ulo;
  if (snap_floor && !(u > ulo + 1e-6)) u = floor_u;
  else if (!(u > ulo)) u = ulo + 0.5 * (uhi - ulo) * 1e-3;
  if (!(u < uhi)) u = uhi - (uhi - ulo) * 1e-3;
  bool lo_known = false;
  double rel = 1.0;
  for (int it = 0; it < maxit; it++) {
    double dF, ph, A;
    const double F = rsf_eval64(q, u, dF, rel, ph, A);
    r.it64++;
    r.phi = (float)ph;
    r.A = A;
    if (rel <= rtol) { r.V = exp(u); r.Vf = (float)r.V; r.res = rel; r.ok = true; return; }
    if (u == floor_u && F >= 0) { r.V = 1e-40; r.Vf = 1e-40f; r.res = 0; r.ok = true; return; }
    if (F < 0) { ulo = u; lo_known = true; } else uhi = u;
    double un = u - F / dF;
    if (!lo_known && dF > 0 && !(un > ulo)) un = floor_u;
    else if (!(dF > 0) || !(un > ulo) || !(un < uhi)) un = 0.5 * (ulo + uhi);
    u = un;
  }
  r.V = exp(u);
  r.Vf = (float)r.V;
  r.res = rel;
}

// Degenerate loads: T* <= 0, or the floor already above the load.
static __device__ __noinline__ bool rsf_degenerate(double Ts, double klin) {
  return !(Ts > 0) || !(log(Ts / klin) > RSF_LOG_FLOOR);
}

// Out-of-line FP64 pieces of the split form (rarely taken).
static __device__ __noinline__ bool rsf_degenerate_in(const RsfIn &in) {
  RsfState s;
  rsf_setup64(s, in);
  return rsf_degenerate(s.Ts, s.klin);
}
static __device__ __noinline__ void rsf_finish64(const RsfIn &in, double u, double rtol, int maxit,
                                          RsfResult &r) {
  RsfState s;
  rsf_setup64(s, in);
  rsf_newton64(s, u, rtol, maxit, true, r);
}

// Whole FP64 solve from the start u0.
__device__ __forceinline__ RsfResult rsf_solve64(const RsfIn &in, double u0, double rtol,
                                                 int maxit) {
  RsfResult r{};
  RsfState q;
  rsf_setup64(q, in);
  r.phi = in.phio.hi;
  if (rsf_degenerate(q.Ts, q.klin)) { r.V = 1e-40; r.Vf = 1e-40f; r.ok = true; return r; }
  rsf_newton64(q, u0, rtol, maxit, false, r);
  return r;
}

// ------------------------------------------------- float-float residual
struct RsfFF {
  ff Ts, klin, snac1, ephio, V0dtL, dtL, V0s, ln2V0, mu0, b, inv_a;
};

// 2^64 and 2^-64: V is carried as Vs = V 2^64 so that V down to the 1e-40
// floor stays a normal float
#define V2C_TWO64 1.8446744073709552e19f
#define V2C_TWOM64 5.4210108624275222e-20f

__device__ __forceinline__ void rsf_setup_ff(RsfFF &q, const RsfIn &in) {
  const ff Gdt = ff_mul(in.G, in.dt);
  q.Ts = ff_add(in.tau_old, ff_scale(ff_mul(Gdt, in.edot), 2.f));
  const ff c1 = ff_add_f(ff_div(Gdt, in.eta), 1.f);
  q.klin = ff_add(ff_mul_f(c1, 4330300.f), ff_scale(ff_div(Gdt, in.W), 2.f));
  q.snac1 = ff_mul(ff_mul(in.sn, in.a), c1);
  q.ephio = ff_exp(in.phio);
  q.dtL = ff_div(in.dt, in.L);
  q.V0dtL = ff_mul(in.V0, q.dtL);
  q.V0s = ff_scale(in.V0, V2C_TWO64);
  q.ln2V0 = ff_log(ff_scale(in.V0, 2.f));
  q.mu0 = in.mu0;
  q.b = in.b;
  q.inv_a = ff_div(ff_f(1.f), in.a);
}

// F and lhs = F + T* at u (float-float); phi and A at u.  Mirrors
// rsf_eval64 term by term.
__device__ __forceinline__ ff rsf_eval_ff(const RsfFF &q, ff u, ff &lhs, ff &phi, ff &A,
                                          ff &Vs) {
  Vs = ff_exp(ff_add(u, ff_scale(ff_ln2(), 64.f)));
  const ff x = ff_scale(ff_mul(Vs, q.dtL), V2C_TWOM64);
  ff g;
  if (x.hi <= 1e-6f) {
    g = ff_add(ff_mul(q.ephio, ff_add_f(ff_neg(x), 1.f)), q.V0dtL);
  } else {
    const ff r = ff_div(q.V0s, Vs);
    const ff ex = ff_exp(ff_neg(x));
    g = ff_add(r, ff_mul(ff_sub(q.ephio, r), ex));
  }
  phi = ff_log(g);
  const ff w = ff_add(ff_sub(u, q.ln2V0), ff_mul(ff_add(q.mu0, ff_mul(q.b, phi)), q.inv_a));
  if (w.hi > 9.f) {
    // asinh(e^w) = w + ln 2 + log((1 + sqrt(1 + t))/2), t = e^-2w < 1.6e-8:
    // the last term is s - s^2/2 with s = t / (2 (sqrt(1+t) + 1))
    const float t = expf(-2.f * w.hi);
    const float s = t / (2.f * (sqrtf(1.f + t) + 1.f));
    A = ff_add_f(ff_add(w, ff_ln2()), s - 0.5f * s * s);
  } else if (w.hi < -4.f) {
    // asinh(z) = z (1 - z^2/6 + 3 z^4/40 - ...), z = e^w < 0.0184
    const ff z = ff_exp(w);
    const float z2 = z.hi * z.hi;
    A = ff_add(z, ff_mul_f(z, z2 * (-1.f / 6.f + z2 * (3.f / 40.f))));
  } else {
    const ff z = ff_exp(w);
    A = ff_log(ff_add(z, ff_sqrt(ff_add_f(ff_mul(z, z), 1.f))));
  }
  const ff klinV = ff_scale(ff_mul(q.klin, Vs), V2C_TWOM64);
  lhs = ff_add(ff_mul(q.snac1, A), klinV);
  return ff_sub(lhs, q.Ts);
}

// Network inputs (the oracle's rsf_features), in FP32: log10 of the
// demanded friction T*/(sn c1) and of the linear stiffness klin/(sn c1),
// 100 a, 100 (b-a), mu0, phi_old, log10 dt/L, log10 V0.  All zero when
// T* <= 0 (a degenerate load, solved without the network).
__device__ __forceinline__ void rsf_features(const RsfIn &in, float *f) {
  const float Gdt = in.G.hi * in.dt.hi;
  const float Ts = in.tau_old.hi + 2.f * Gdt * in.edot.hi;
  const float c1 = 1.f + Gdt / in.eta.hi;
  const float klin = 4330300.f * c1 + 2.f * Gdt / in.W.hi;
  const float snc1 = in.sn.hi * c1;
  if (!(Ts > 0.f)) {
#pragma unroll
    for (int k = 0; k < 8; k++) f[k] = 0.f;
    return;
  }
  // fast-math logs and quotients: these are network inputs, a few ulp off
  // change nothing the network can resolve
  f[0] = __log10f(__fdividef(Ts, snc1));
  f[1] = __log10f(__fdividef(klin, snc1));
  f[2] = in.a.hi * 100.f;
  f[3] = (in.b.hi - in.a.hi) * 100.f;
  f[4] = in.mu0.hi;
  f[5] = in.phio.hi;
  f[6] = __log10f(__fdividef(in.dt.hi, in.L.hi));
  f[7] = __log10f(in.V0.hi);
}

// ------------------------------------------------------- FP32 residual
struct Rsf32 {
  float a, b, L, V0, mu0, dt, ephio, Ts, snac1, klin, lg2V0, uhi;
};
// FP32 constants straight from the inputs (no float-float set-up needed
// for the FP32 phase)
__device__ __forceinline__ Rsf32 rsf32_of(const RsfIn &in) {
  Rsf32 r;
  r.a = in.a.hi; r.b = in.b.hi; r.L = in.L.hi; r.V0 = in.V0.hi; r.mu0 = in.mu0.hi;
  r.dt = in.dt.hi;
  const float Gdt = in.G.hi * in.dt.hi;
  r.Ts = in.tau_old.hi + 2.f * Gdt * in.edot.hi;
  const float c1 = 1.f + Gdt / in.eta.hi;
  r.klin = 4330300.f * c1 + 2.f * Gdt / in.W.hi;
  r.snac1 = in.sn.hi * in.a.hi * c1;
  r.ephio = expf(in.phio.hi);
  r.lg2V0 = logf(2.f * in.V0.hi);
  r.uhi = logf(r.Ts / r.klin);
  return r;
}
__device__ __forceinline__ float rsf_eval32(const Rsf32 &q, float u, float &dF, float &lhs) {
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
  const float phi = __logf(g);
  const float dph = dg / g;
  const float w = u - q.lg2V0 + (q.mu0 + q.b * phi) / q.a;
  const float A = (w > 20.f) ? w + 0.693147180559945f : asinhf(__expf(w));
  const float dA = rsqrtf(1.f + __expf(-2.f * w));
  lhs = q.snac1 * A + q.klin * V;
  dF = q.snac1 * dA * (1.f + q.b / q.a * dph) + q.klin * V;
  return lhs - q.Ts;
}

// FP32 safeguarded Newton from u0; returns the last iterate and the FP32
// derivative there.  A step below the floor before F(floor) < 0 is known
// goes to the floor itself.
__device__ __forceinline__ float rsf_newton32(const Rsf32 &q, float u0, float ulo, float uhi,
                                              int maxit, int &iters, float &dFu) {
  const float floor_u = ulo;
  float u = fminf(fmaxf(u0, ulo + 1e-3f * (uhi - ulo)), uhi - 1e-3f * (uhi - ulo));
  if (!(u == u)) u = 0.5f * (ulo + uhi);
  bool lo_known = false;
  iters = 0;
  dFu = 0.f;
  for (int it = 0; it < maxit; it++) {
    float dF, lhs;
    const float F = rsf_eval32(q, u, dF, lhs);
    iters++;
    dFu = dF;
    // FP32 rounding floor of the residual is a few 1e-7 of lhs
    if (fabsf(F) <= 1e-6f * lhs) break;
    if (u == floor_u && F >= 0.f) break;  // the finishing phase confirms the floor
    if (F < 0.f) { ulo = u; lo_known = true; } else uhi = u;
    float un = u - F / dF;
    if (!lo_known && dF > 0.f && !(un > ulo)) un = floor_u;
    else if (!(dF > 0.f) || !(un > ulo) || !(un < uhi)) un = 0.5f * (ulo + uhi);
    if (fabsf(un - u) <= 1e-6f * fmaxf(1.f, fabsf(u))) { u = un; break; }
    u = un;
  }
  return u;
}

// True when F(floor) > 0 is certain from the FP32 residual alone (margin
// 1e-3 of the scale, two orders above the FP32 evaluation error): the load
// cannot drive slip above the 1e-40 floor, and the floor is the solution
// (the rule of the FP64 form at the floor).
// A_floor: the friction term asinh(..) at the floor (FP32), for tau_y.
__device__ __forceinline__ bool rsf_floor_certain(const Rsf32 &q, float &A_floor) {
  A_floor = 0.f;
  if (!(q.Ts > 0.f) || !(q.uhi > (float)RSF_LOG_FLOOR)) return false;  // degenerate: FP64 decides
  float dF, lhs;
  const float F = rsf_eval32(q, (float)RSF_LOG_FLOOR, dF, lhs);
  A_floor = lhs / q.snac1;  // klin V is below 1e-30 of lhs at the floor
  return F >= 1e-3f * lhs;
}

// The start u0 clamped into the FP32 Newton's bracket, as rsf_newton32
// does, and the FP32 residual ratio |F|/lhs there.
__device__ __forceinline__ float rsf_start_residual(const Rsf32 &q, float u0, float &u) {
  const float ulo = (float)RSF_LOG_FLOOR, uhi = q.uhi;
  u = fminf(fmaxf(u0, ulo + 1e-3f * (uhi - ulo)), uhi - 1e-3f * (uhi - ulo));
  float dF, lhs;
  const float F = rsf_eval32(q, u, dF, lhs);
  const float r = fabsf(F) / lhs;
  return r == r ? r : INFINITY;
}

// The learned start, evaluated only where it can pay: the network's
// proposal costs a few Newton iterations' worth of work, so a state whose
// plain start (the previous slip rate) already has an FP32 residual ratio
// below RSF_NET_MIN_RES -- a couple of Newton steps from the FP32 floor --
// keeps it; elsewhere the proposal is taken if its residual is smaller
// than the plain start's, so the chosen start is never the worse of the
// two.
constexpr float RSF_NET_MIN_RES = 1e-2f;

// Split solve from the start u0 (FP32 phase, float-float phase, FP64
// fallback).  q32 = rsf32_of(in).
__device__ __forceinline__ RsfResult rsf_solve_split(const RsfIn &in, const Rsf32 &q32, float u0,
                                                     double rtol, int maxit) {
  RsfResult r{};
  r.phi = in.phio.hi;
  const float floor32 = (float)RSF_LOG_FLOOR;
  if (!(q32.Ts > 0.f) || !(q32.uhi > floor32)) {
    // degenerate in FP32: decided in FP64 as the FP64 form does
    if (rsf_degenerate_in(in)) { r.V = 1e-40; r.Vf = 1e-40f; r.ok = true; return r; }
  }
  float dF32;
  const float u32 = rsf_newton32(q32, u0, floor32, q32.uhi, maxit, r.it32, dF32);
  RsfFF q;
  rsf_setup_ff(q, in);
  const ff floor_u = ff_from_double(RSF_LOG_FLOOR);
  ff u = (u32 <= floor32 + 1e-6f) ? floor_u : ff_f(u32);
  // the ratio |F|/(F+T*) needs a few significant digits: F and F+T* come
  // from the float-float evaluation, the ratio is taken in FP32.  Accepted
  // at 3/4 of the tolerance: the float-float ratio and the FP64 one at the
  // same slip rate differ by up to ~1.3e-11 (measured on 20 000 states of
  // the C3 distributions), and the returned root must meet rtol in FP64.
  const float rtolf = 0.75f * (float)rtol;
  for (int k = 0; k < 4; k++) {
    ff lhs, phi, A, Vs;
    const ff F = rsf_eval_ff(q, u, lhs, phi, A, Vs);
    r.itff++;
    const float rel = fabsf(F.hi) / lhs.hi;
    r.phi = phi.hi;
    if (rel <= rtolf) {
      r.A = ff_to_double(A);
      r.V = ff_to_double(Vs) * 5.4210108624275222e-20;
      r.Vf = Vs.hi * V2C_TWOM64;
      r.res = rel;
      r.ok = true;
      return r;
    }
    const bool at_floor = u.hi == floor_u.hi && u.lo == floor_u.lo;
    if (at_floor && F.hi >= 0.f) {
      r.V = 1e-40; r.Vf = 1e-40f; r.res = 0; r.ok = true;
      return r;
    }
    if (!(dF32 > 0.f)) break;
    u = ff_add_f(u, -F.hi / dF32);
  }
  // the FP64 Newton finishes
  rsf_finish64(in, ff_to_double(u), rtol, maxit, r);
  return r;
}

// The floor as a result (one FP32 residual evaluation)
__device__ __forceinline__ RsfResult rsf_floor_result(const RsfIn &in, float A_floor) {
  RsfResult r{};
  r.phi = in.phio.hi;
  r.A = A_floor;
  r.V = 1e-40;
  r.Vf = 1e-40f;
  r.res = 0;
  r.it32 = 1;
  r.ok = true;
  return r;
}

}  // namespace v2c
