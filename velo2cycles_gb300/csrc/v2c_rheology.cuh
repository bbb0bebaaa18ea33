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
// leaves its result undefined there).
__device__ __forceinline__ float ductile_visc32(const Rock &R, const Scal &S, int t,
                                                float sigin, float T, float mpb) {
  int kind = (int)R(RK_KIND, t);
  if (kind == VISC_STICKY) {
    float nu = R(RK_NU, t);
    if (S.sticky_cap && nu > S.sticky_nu) nu = S.sticky_nu;
    return nu;
  }
  if (kind == VISC_NEWTON) return R(RK_NU, t);
  if (kind != VISC_POWER) return __int_as_float(0x7fc00000);

  const float mm = R(RK_MM, t);
  const float LN_HALF = -0.693147180559945f;
  float le1 = (R(RK_DH, t) + R(RK_DV, t) * mpb) / (8.314f * T);
  if (le1 > 150.f) le1 = 150.f;
  // ln of the diffusion-creep viscosity 0.5 k1 e1, k1 = nu / ss^(mm-1)
  float s0 = LN_HALF + R(RK_LNNU, t) - (mm - 1.f) * R(RK_LNSS, t) + le1;
  float lnv = s0;  // sigin == 0: eta = eta_diff
  if (sigin > 0.f) {
    // eta_disl / eta_diff = (ss / sigin)^(mm-1)
    const float d0 = exp2f((mm - 1.f) * (R(RK_LNSS, t) - logf(sigin)) * 1.44269504089f);
    const float g = __expf(__logf(R(RK_GG, t) * S.dt) - s0);  // G dt / eta_diff
    const float invS = __expf(-s0);
    const float em = (mm - 1.f) / mm;
    const float c0 = exp2f(__log2f(d0) / mm);     // coeff / eta_diff^(1/mm)
    const float emc0 = em * c0;
    const float p2fac = 2.f * s0 * invS;
    // |log10(m_k / m_k-1)| < 1e-6  <=>  10^-1e-6 < m_k / m_k-1 < 10^1e-6
    const float RLO = 0.99999769741f, RHI = 1.00000230259f;
    // the extra derivative term p2 (below) is at most invS e^max(p2fac,0)
    // (dold >= 0); under half an ulp of gm it cannot change gm + p2 in FP32
    const float p2max = invS * __expf(fmaxf(p2fac, 0.f));
    float dnew = d0, m_prev = 1.f;
    for (int counter = 1; counter <= 50; counter++) {
      const float dold = dnew;
      const float m = __fdividef(dnew, dnew + 1.f);    // mnu0 / eta_diff
      const float gm = g + m;
      const float base = (1.f + dold) * gm;            // prefactor (G dt + mnu0) / eta_diff
      const float f1 = exp2f(em * __log2f(base));      // base^((mm-1)/mm)
      const float f2 = dold - c0 * f1;
      // pow(eta_diff, 2/(eta_diff+eta_disl_old)) / eta_diff, the reference's
      // extra term of the derivative (density_ductilevisc_calc.c:190-191)
      const float p2 = (invS > 1e-30f && !(p2max < gm * 0x1p-25f))
                           ? __expf(__fdividef(p2fac, 1.f + dold)) * invS : 0.f;
      const float df = 1.f - emc0 * __fdividef(f1, base) * (gm + p2);  // base^(-1/mm) = f1/base
      dnew = dold - __fdividef(f2, df);
      // m / m_prev within (RLO, RHI), m and m_prev positive
      if (counter > 3 && m > RLO * m_prev && m < RHI * m_prev) break;
      m_prev = m;
    }
    lnv = s0 - log1pf(1.f / dnew);
  }
  // limits nubeg/nuend then the per-type limits, in that order
  float nu;
  if (lnv < S.ln_nubeg) nu = S.nubeg_f;
  else if (lnv > S.ln_nuend) nu = S.nuend_f;
  else nu = expf(lnv);
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

}  // namespace v2c
