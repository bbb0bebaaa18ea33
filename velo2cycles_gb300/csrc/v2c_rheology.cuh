// v2c_rheology.cuh -- per-marker property evaluation in FP32.
//
// Follows recalc_marker_properties.c:1-83, dencalcomp and ductilevisc
// (density_ductilevisc_calc.c:2-223) and calc_frictionpara (calc_RSF.c:
// 224-295).  The ductile viscosity keeps the reference's creep Newton
// iteration and stopping rule, but runs it on viscosities divided by the
// diffusion-creep viscosity (so eta_diff = 1): the Arrhenius factor
// exp((E+PV)/RT) reaches exp(150) in the reference and overflows FP32, while
// the ratios the iteration actually needs stay O(1).
#pragma once
#include "v2c_ff.cuh"
#include "v2c_internal.cuh"

namespace v2c {

// dencalcomp: density and the adiabatic coefficient
__device__ __forceinline__ void density32(const Rock &R, int densimod, int t, float T,
                                          float mpb, float &mro, float &mbb) {
  float bb = R(RK_BB, t), aa = R(RK_AA, t);
  mbb = bb / (1.f - bb * (T - 298.15f));
  mro = R(RK_RO, t);
  if (densimod != 0) mro = mro * (1.f - bb * (T - 298.15f)) * (1.f + aa * (mpb - 1.f) * 1e-3f);
}

// thermal conductivity, recalc_marker_properties.c:59-62
__device__ __forceinline__ float conductivity32(const Rock &R, int t, float T, float mpb) {
  float kf = R(RK_KF, t), kp = R(RK_KP, t);
  float k = (R(RK_KT, t) + kf / (T + 77.f)) * expf(kp * mpb);
  if (k < 0.f) k = -k / (1.f + kf * (T - kp) / kp);
  return k;
}

// ductilevisc.  Returns NaN for a type that fits no branch (the reference
// leaves its result undefined there).  sig2 = sxx^2 + sxy^2 (the squared
// stress invariant) and mpb (pressure, bar) arrive as float pairs: the
// dislocation viscosity goes as sigin^(1-n) and the Arrhenius factor as
// e^(V P/(R T)), with V P/(R T) up to ~7 in the mantle, so their FP32
// roundings alone would be a few 1e-7 of the viscosity.
//
// Precision.  The viscosity is e^s0 times an O(1) ratio, with s0 = ln of
// the diffusion-creep viscosity, up to ~60: an FP32 s0 alone (ulp 4e-6)
// would carry several parts in 1e6.  s0 = ln(0.5 k1) + (E + PV)/(RT) is
// therefore formed as a float pair from the float-pair temperature
// (T, Tlo) and the per-type constant pairs of the rock table.
//
// The creep iteration.  The reference iterates on the dislocation-creep
// viscosity with an approximate derivative, so it converges linearly (about
// a dozen steps, up to ~30), and its result is the iterate where the
// relative change of mnu0 first drops below 1e-6 in log10.  Run directly in
// FP32, every step carries a rounding error of a few 1e-7 of the iterate:
// the iterates drift by up to ~2e-6 from the FP64 ones, and the stopping
// test, which compares changes of ~2e-6, stops a step early or late for a
// few per cent of the markers.  Here, with d = eta_disl / eta_diff and
// B(d) = g + d (1 + g) the reference's prefactor term, its residual is
// f2(d) = d - (q B(d))^em (q = ss/sigin, em = (mm-1)/mm, g = G dt/eta_diff):
//   1. d*, close to the root of f2, by an FP32 Newton with the exact
//      derivative;
//   2. R0 = f2(d*) in float-float, from float pairs of q, g and em;
//   3. the reference's iteration replayed from its start d0 = q^(mm-1)
//      (float-float) in the deviation e = d - d*:
//        f2(d* + e) = R0 + e - (q B*)^em expm1(em log1p(e (1 + g)/B*)),
//      every term of which FP32 holds to a few 1e-7 of e rather than of d,
//      as it does the steps and the change that the stopping test reads.
// The viscosity is e^s0 d/(1 + d) at the step the replay stops, in
// float-float, rounded once to FP32 (through the exponent s0 + ln(d/(1+d))
// where it is near a limit or e^s0 is beyond the FP32 range).
__device__ __forceinline__ float ductile_visc32(const Rock &R, const Scal &S, int t,
                                                ff sig2, float T, float Tlo, ff mpb) {
  int kind = (int)R(RK_KIND, t);
  if (kind == VISC_STICKY) {
    float nu = R(RK_NU, t);
    if (S.sticky_cap && nu > S.sticky_nu) nu = S.sticky_nu;
    return nu;
  }
  if (kind == VISC_NEWTON) return R(RK_NU, t);
  if (kind != VISC_POWER) return __int_as_float(0x7fc00000);

  const float mm = R(RK_MM, t);
  // (E + PV)/(RT), density_ductilevisc_calc.c:116-120, capped at 150
  const ff num = ff_add(ff{R(RK_DH, t), R(RK_DH_LO, t)}, ff_mul(ff{R(RK_DV, t), R(RK_DV_LO, t)}, mpb));
  const ff den = ff_mul(ff{T, Tlo}, ff{8.31400012969970703125f, -1.2969971407983394e-07f});
  ff le1 = den.hi != 0.f ? ff_div_fast(num, den) : ff_f(num.hi / den.hi);
  if (le1.hi > 150.f || (le1.hi == 150.f && le1.lo > 0.f)) le1 = ff_f(150.f);
  // ln of the diffusion-creep viscosity 0.5 k1 e1, k1 = nu / ss^(mm-1)
  const ff s0 = ff_add(ff{R(RK_LNK, t), R(RK_LNK_LO, t)}, le1);
  ff rat = ff_f(1.f);  // eta / eta_diff = d/(1 + d); sigin == 0: eta = eta_diff
  if (sig2.hi > 0.f) {
    const ff em_ff{R(RK_EM, t), R(RK_EM_LO, t)};
    const float em = em_ff.hi;
    // ln q = ln ss - ln sigin, q = ss / sigin
    const ff lnq = ff_sub(ff{R(RK_LNSS, t), R(RK_LNSS_LO, t)}, ff_scale(ff_log(sig2), 0.5f));
    const float q = __expf(lnq.hi);
    // G dt / eta_diff (0 without elasticity or time step); below 6e-6 its
    // FP32 value is within 1e-11 of itself, far inside what R0 needs
    ff g_ff = ff_f(0.f);
    if (R(RK_LNG, t) > -INFINITY && S.lndt_hi > -INFINITY) {
      const ff lng = ff_sub(ff_add(ff{R(RK_LNG, t), R(RK_LNG_LO, t)}, ff{S.lndt_hi, S.lndt_lo}), s0);
      g_ff = lng.hi < -12.f ? ff_f(expf(lng.hi) * (1.f + lng.lo)) : ff_exp(lng);
    }
    const float g = g_ff.hi, g1p = 1.f + g;
    // the reference's start, eta_disl / eta_diff = q^(mm-1) at the marker's
    // stress, in float-float: an FP32 start would change where the replay
    // stops in ~0.1 % of the markers
    const ff d0_ff = ff_exp(ff_mul(ff{R(RK_MM1, t), R(RK_MM1_LO, t)}, lnq));
    const float d0 = d0_ff.hi;
    // 1. d*: Newton on f2 with its exact derivative (fast intrinsics: only
    //    its closeness to the root matters, R0 below is exact at it)
    float ds = d0;
    for (int it = 0; it < 16; it++) {
      const float B = fmaf(ds, g1p, g);
      const float f1c = exp2f(em * __log2f(q * B));  // (q B)^em
      const float fp = 1.f - em * __fdividef(f1c, B) * g1p;
      float dn = ds - __fdividef(ds - f1c, fp);
      if (!(dn > 0.f)) dn = 0.5f * ds;
      const bool conv = fabsf(dn - ds) <= 1e-6f * ds;
      ds = dn;
      if (conv) break;
    }
    // 2. R0 = f2(d*) and (q B*)^em in float-float
    const ff Bs_ff = ff_add(ff_mul_f(ff_add_f(g_ff, 1.f), ds), g_ff);
    const ff c0f1s_ff = ff_exp(ff_mul(em_ff, ff_add(lnq, ff_log(Bs_ff))));
    const ff R0 = ff_add_f(ff_neg(c0f1s_ff), ds);
    const float c0f1s = c0f1s_ff.hi, Bs = Bs_ff.hi, r0 = R0.hi;
    // 3. the reference's iteration in e = d - d*
    const float invS = __expf(-s0.hi);
    const float p2fac = 2.f * s0.hi * invS;
    // the extra derivative term p2 (below) is at most invS e^max(p2fac,0)
    // (d >= 0); under half an ulp of gm it cannot change gm + p2 in FP32
    const float p2max = invS * __expf(fmaxf(p2fac, 0.f));
    // |log10(m_k / m_k-1)| < 1e-6  <=>  10^-1e-6 - 1 < m_k / m_k-1 - 1 < 10^1e-6 - 1
    const float TLO = -2.30258242e-6f, THI = 2.30258771e-6f;
    const ff e0 = ff_add_f(d0_ff, -ds);
    float e = e0.hi + e0.lo, e_prev = 0.f, d_prev = 1.f;
    // per-step constants: B(d)/B* - 1 = x = e (1 + g)/B*; c0 B^em / B
    // = (c0 B*^em / B*) (1 + g1)/(1 + x)
    const float inv_Bs = __fdividef(1.f, Bs);
    const float kx = g1p * inv_Bs, kc = c0f1s * inv_Bs;
    // Near the stop (|x| < 1/32) both powers come from the binomial series
    // of (1 + x)^a - 1 = h = a x (1 + c1 x (1 + c2 x (1 + c3 x (1 + c4 x)))),
    // a = em - 1, c_k = (a - k)/(k + 1), within 1.4e-8 of itself there:
    // (1 + x)^em - 1 = x + h (1 + x) and c0 B^em / B = kc (1 + h), without a
    // division.
    const float a1 = em - 1.f;
    const float c1 = 0.5f * (a1 - 1.f), c2 = (a1 - 2.f) * (1.f / 3.f);
    const float c3 = 0.25f * (a1 - 3.f), c4 = 0.2f * (a1 - 4.f);
    for (int counter = 1; counter <= 50; counter++) {
      const float e_old = e;
      const float d_old = ds + e_old;
      const float m = __fdividef(d_old, d_old + 1.f);   // mnu0 / eta_diff
      const float gm = g + m;
      // B(d)/B* - 1: below -1 the reference's iteration has gone to a
      // negative prefactor, whose power is NaN there and is NaN here (log1pf)
      const float x = e_old * kx;
      float g1, cfB;  // (B(d)/B*)^em - 1 and c0 B^em / B
      if (fabsf(x) < 0.03125f) {
        const float h =
            a1 * x * fmaf(c1 * x, fmaf(c2 * x, fmaf(c3 * x, fmaf(c4, x, 1.f), 1.f), 1.f), 1.f);
        g1 = fmaf(h, 1.f + x, x);
        cfB = fmaf(kc, h, kc);
      } else {
        g1 = expm1f(em * log1pf(x));
        cfB = __fdividef(kc * (1.f + g1), 1.f + x);
      }
      const float f2 = (e_old - c0f1s * g1) + r0;       // f2(d* + e)
      // pow(eta_diff, 2/(eta_diff+eta_disl_old)) / eta_diff, the reference's
      // extra term of the derivative (density_ductilevisc_calc.c:190-191)
      const float p2 = (invS > 1e-30f && !(p2max < gm * 0x1p-25f))
                           ? __expf(__fdividef(p2fac, 1.f + d_old)) * invS : 0.f;
      const float df = 1.f - em * cfB * (gm + p2);
      e = e_old - __fdividef(f2, df);
      // relative change of mnu0 from the previous step: (d - d_prev) /
      // (d_prev (1 + d)), tested without the division (the denominator > 0)
      const float D = d_prev * (1.f + d_old), dd = e_old - e_prev;
      if (counter > 3 && dd > TLO * D && dd < THI * D) break;
      e_prev = e_old;
      d_prev = d_old;
    }
    // d/(1 + d) at the last step, d = d* + e as a float pair
    ff d_ff;
    d_ff.hi = two_sum(ds, e, d_ff.lo);
    rat = ff_div_fast(d_ff, ff_add_f(d_ff, 1.f));
  }
  // limits nubeg/nuend then the per-type limits, in that order; an FP32
  // estimate of ln nu (within 1e-5) decides all but the values near a limit
  const float lest = s0.hi + __logf(rat.hi);
  float nu;
  if (lest < S.ln_nubeg - 1e-3f) nu = S.nubeg_f;
  else if (lest > S.ln_nuend + 1e-3f) nu = S.nuend_f;
  else if (s0.hi < 80.f && lest > S.ln_nubeg + 1e-3f && lest < S.ln_nuend - 1e-3f) {
    nu = ff_round(ff_mul(ff_exp(s0), rat));
  } else {
    const ff lnv = ff_add(s0, ff_log(rat));
    if (lnv.hi < S.ln_nubeg) nu = S.nubeg_f;
    else if (lnv.hi > S.ln_nuend) nu = S.nuend_f;
    else nu = ff_round(ff_exp(lnv));
  }
  if (nu < R(RK_N0, t)) nu = R(RK_N0, t);
  if (nu > R(RK_N1, t)) nu = R(RK_N1, t);
  return nu;
}

// calc_frictionpara: RSF parameters of a marker; returns the updated state
// phi.  x, y are FP64 positions (the band and zone limits are sharp
// thresholds, so they are tested on the same FP64 value the reference sees).
struct Fric {
  float a, b, L, V0, mu0;
};
// Out of line: the marker physics calls it only near the frictional band
// (FP64 position test) and for sticky air.
static __device__ __noinline__ float friction_marker(const v2c_params &p, int phi_reset0,
                                                 double x, double y, int t, float phi,
                                                 Fric &f) {
  double d = y - (p.fault_y + p.fault_slope * x);
  double radius = d >= 0 ? d : -d;
  if (t > 0) {
    if (radius <= p.fault_hw) {
      double a, b, L, V0;
      if (x > p.end_updip && x < p.start_downdip) {
        a = p.a_vw; b = p.b_vw; L = p.L_vw; V0 = p.V0_vw;
      } else if (x > p.start_updip && x < p.end_updip && p.half_range > 0) {
        double fr = (x - (p.start_updip - p.xstpx / 2)) / (2 * p.half_range);
        a = p.a_vs + fr * (p.a_vw - p.a_vs); b = p.b_vs + fr * (p.b_vw - p.b_vs);
        L = p.L_vs + fr * (p.L_vw - p.L_vs); V0 = p.V0_vs + fr * (p.V0_vw - p.V0_vs);
      } else if (x >= p.start_downdip && x < p.end_downdip && p.half_range > 0) {
        double fr = (x - (p.start_downdip - p.xstpx / 2)) / (2 * p.half_range);
        a = p.a_vw - fr * (p.a_vw - p.a_vs); b = p.b_vw - fr * (p.b_vw - p.b_vs);
        L = p.L_vw - fr * (p.L_vw - p.L_vs); V0 = p.V0_vw - fr * (p.V0_vw - p.V0_vs);
      } else {
        a = p.a_vs; b = p.b_vs; L = p.L_vs; V0 = p.V0_vs;
      }
      f.a = (float)a; f.b = (float)b; f.L = (float)L; f.V0 = (float)V0; f.mu0 = 0.2f;
      if (phi_reset0) phi = 0.f;
    } else {
      phi = 50.f;
      f.a = (float)p.a_hr; f.b = (float)p.b_hr; f.L = (float)p.L_hr;
      f.V0 = (float)p.V0_hr; f.mu0 = 0.6f;
    }
  } else {
    f.a = 1.f; f.b = 0.01f; f.L = 0.2f; f.V0 = (float)p.V0_hr; f.mu0 = 0.6f;
  }
  return phi;
}

// ----------------------------------------------- interpolation stencils
// Bilinear weights of a point given as cell-local axes, following the four
// staggered stencils of interpolation.c.  Each returns the node index of
// the upper-left stencil node and the weights (e, n).

// basic (shear) nodes, interpolation.c:1067-1080: m10 clamped to [1, xn-3]
// Stencil weights use the fast reciprocal division (__fdividef, 2 ulp): the
// denominators are cell widths, far inside its range.
__device__ __forceinline__ long stencil_basic(const Grid &g, const Axis &ax, const Axis &ay,
                                              float &e, float &n) {
  int m10 = ax.i, m20 = ay.i;
  if (m10 < 1) m10 = 1;
  if (m10 > g.xn - 3) m10 = g.xn - 3;
  if (m20 < 1) m20 = 1;
  if (m20 > g.yn - 3) m20 = g.yn - 3;
  int kx = m10 - ax.i, ky = m20 - ay.i;
  e = __fdividef(ax.X - ax.G(kx), ax.G(kx + 1) - ax.G(kx));
  n = __fdividef(ay.X - ay.G(ky), ay.G(ky + 1) - ay.G(ky));
  return (long)m10 * g.yn + m20;
}

// pressure (cell-centre) nodes, interpolation.c:1216-1229 and :1940-1950.
// xhi/yhi: point in the upper half of its cell (x > cell midpoint).
__device__ __forceinline__ long stencil_centre(const Grid &g, const Axis &ax, const Axis &ay,
                                               bool xhi, bool yhi, float &e, float &n) {
  int m10 = ax.i + (xhi ? 1 : 0), m20 = ay.i + (yhi ? 1 : 0);
  if (m10 > g.xn - 2) m10 = g.xn - 2;
  if (m20 > g.yn - 2) m20 = g.yn - 2;
  if (m10 < 1) m10 = 1;
  if (m20 < 1) m20 = 1;
  int kx = m10 - ax.i, ky = m20 - ay.i;
  e = __fdividef(ax.X - (ax.G(kx - 1) + ax.G(kx)) * 0.5f, (ax.G(kx + 1) - ax.G(kx - 1)) * 0.5f);
  n = __fdividef(ay.X - (ay.G(ky - 1) + ay.G(ky)) * 0.5f, (ay.G(ky + 1) - ay.G(ky - 1)) * 0.5f);
  return (long)m10 * g.yn + m20;
}

// vx nodes, interpolation.c:1377-1391: ylo = point in the upper half in y
// is false (y below the cell midpoint)
__device__ __forceinline__ long stencil_vx(const Grid &g, const Axis &ax, const Axis &ay,
                                           bool ylo, int xclamp_hi, float &e, float &n) {
  int m10 = ax.i, m20 = ay.i - (ylo ? 1 : 0);
  if (m10 < 0) m10 = 0;
  if (m10 > xclamp_hi) m10 = xclamp_hi;
  if (m20 < 0) m20 = 0;
  if (m20 > g.yn - 3) m20 = g.yn - 3;
  int kx = m10 - ax.i, ky = m20 - ay.i;
  e = __fdividef(ax.X - ax.G(kx), ax.G(kx + 1) - ax.G(kx));
  n = __fdividef(ay.X - (ay.G(ky) + ay.G(ky + 1)) * 0.5f, (ay.G(ky + 2) - ay.G(ky)) * 0.5f);
  return (long)m10 * g.yn + m20;
}

// vy nodes, interpolation.c:1434-1448
__device__ __forceinline__ long stencil_vy(const Grid &g, const Axis &ax, const Axis &ay,
                                           bool xlo, int yclamp_hi, float &e, float &n) {
  int m10 = ax.i - (xlo ? 1 : 0), m20 = ay.i;
  if (m10 < 0) m10 = 0;
  if (m10 > g.xn - 3) m10 = g.xn - 3;
  if (m20 < 0) m20 = 0;
  if (m20 > yclamp_hi) m20 = yclamp_hi;
  int kx = m10 - ax.i, ky = m20 - ay.i;
  e = __fdividef(ax.X - (ax.G(kx) + ax.G(kx + 1)) * 0.5f, (ax.G(kx + 2) - ax.G(kx)) * 0.5f);
  n = __fdividef(ay.X - ay.G(ky), ay.G(ky + 1) - ay.G(ky));
  return (long)m10 * g.yn + m20;
}

__device__ __forceinline__ float bil(const float *f, long m3, long yn, float e, float n) {
  float d0 = (1.f - e) * (1.f - n), d1 = (1.f - e) * n, d2 = e * (1.f - n), d3 = e * n;
  return d0 * __ldg(f + m3) + d1 * __ldg(f + m3 + 1) + d2 * __ldg(f + m3 + yn) +
         d3 * __ldg(f + m3 + yn + 1);
}

// bilinear interpolation as a float pair: the first node's value plus the
// FP32 change across the stencil (for a smooth field such as the pressure
// the change is a small part of the value, so its rounding is too)
__device__ __forceinline__ ff bil_ff(const float *f, long m3, long yn, float e, float n) {
  const float f0 = __ldg(f + m3), f1 = __ldg(f + m3 + 1), f2 = __ldg(f + m3 + yn),
              f3 = __ldg(f + m3 + yn + 1);
  const float d10 = f1 - f0, d20 = f2 - f0, dd = (f3 - f2) - d10;
  const float d = fmaf(e, fmaf(n, dd, d20), n * d10);
  ff r;
  r.hi = two_sum(f0, d, r.lo);
  return r;
}

// bil(f) - bil(g) as one interpolation of the node differences (the same
// bilinear form, so the same value in exact arithmetic): f and g are
// consecutive states of one field that agree in their leading digits, and
// their FP32 node differences are exact where they are within a factor 2
__device__ __forceinline__ float bil_diff(const float *f, const float *g, long m3, long yn,
                                          float e, float n) {
  float d0 = (1.f - e) * (1.f - n), d1 = (1.f - e) * n, d2 = e * (1.f - n), d3 = e * n;
  return d0 * (__ldg(f + m3) - __ldg(g + m3)) + d1 * (__ldg(f + m3 + 1) - __ldg(g + m3 + 1)) +
         d2 * (__ldg(f + m3 + yn) - __ldg(g + m3 + yn)) +
         d3 * (__ldg(f + m3 + yn + 1) - __ldg(g + m3 + yn + 1));
}

}  // namespace v2c
