// v2c_nodes.cu -- node loops of the step, one thread per node, FP32.
//
//  * interpolate_center2basic_old (interpolation.c:1575-1598)
//  * compute_before_solve -> calc_vpvisc (plastic.c:2-56, calc_RSF.c:33-169)
//  * compute_after_solve -> calc_sliprate_after_solve (plastic.c:61-129,
//    calc_RSF.c:172-221), with a deterministic block-tree + fixed-order sum
//    for the RMS misfit
//  * the boundary corrections that end marker2nodes
//    (momentum_continuity_addmatrix_checkerror.c:1002-1184,
//    temperature_iterate.c:828-891): the reference solves them with its
//    frontal Gauss routine; here each boundary row arrives pre-resolved on
//    the host (v2c_set_bonds) as constant + references to unconstrained
//    rows, which is the same linear solution.
//
// The rate-and-state expressions of calc_RSF.c multiply exp(+-(mu0+b phi)/a)
// factors that reach e^+-160 for the host-rock state phi = 50; they are
// evaluated here in log space, which is exact algebra and stays inside FP32
// range.
#include <math.h>

#include "v2c_ff.cuh"
#include "v2c_kernels.h"

namespace v2c {

namespace {

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

// Float-float forms of the exponents of the slip-rate law.  Its exponent
// sums terms of a few hundred that cancel (ln V, (mu + b phi)/a, ln sinh of
// tau/(a sigma)), and the slip rate is e^exponent: in FP32 the sum's
// rounding alone (~1e-5) would be the slip rate's relative error.

// ln sinh x for x > 0 as a float pair (the correction terms in FP32: below
// 2e-9 for x > 10, and log1p of sinh(x)/x - 1 < 0.05 for x < 0.5)
__device__ __forceinline__ ff ff_log_sinh(ff x) {
  if (x.hi > 10.f)
    return ff_add_f(ff_sub(x, ff_ln2()), log1pf(-expf(-2.f * x.hi)));
  if (x.hi > 0.5f)
    return ff_log(ff_scale(ff_sub(ff_exp(x), ff_exp(ff_neg(x))), 0.5f));
  const float x2 = x.hi * x.hi;
  return ff_add_f(ff_log(x), log1pf(x2 * (1.f / 6.f + x2 * (1.f / 120.f + x2 * (1.f / 5040.f)))));
}

// e^E for a float pair E (the low word as a first-order factor)
__device__ __forceinline__ float exp_ff(ff E) { return expf(E.hi) * (1.f + E.lo); }

// A node value formed in float-float and rounded once to FP32: the node
// kernels of a Picard pass feed each other through FP32 node fields, and the
// slip rate magnifies a one-ulp difference of its inputs a hundredfold
// (tau/(a sigma) ~ 100 in the exponent), so each field is rounded from a
// value ~2^-48 accurate rather than from a chain of FP32 roundings.
__device__ __forceinline__ float rn(ff a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ ff ff_quarter_sum(float a, float b, float c, float d) {
  ff s = ff_add_f(ff_f(a), b);
  s = ff_add_f(s, c);
  return ff_scale(ff_add_f(s, d), 0.25f);
}
// a / b, the IEEE FP32 quotient where b is 0 or a non-finite (the reference's
// inf and NaN), else the float-float quotient
__device__ __forceinline__ ff ff_div_ieee(ff a, ff b) {
  if (b.hi == 0.f || !isfinite(b.hi) || !isfinite(a.hi)) return ff_f(a.hi / b.hi);
  return ff_div(a, b);
}

// asinh(e^w) as a float pair (calc_RSF.c:128): w + ln 2 + e^-2w / 4 above
// w = 9 (the next term is below 1e-16 of the result), the series
// x - x^3/6 + 3 x^5/40 for x = e^w below 1e-3, else ln(x + sqrt(x^2 + 1))
__device__ __forceinline__ ff ff_asinh_exp(ff w) {
  if (w.hi > 9.f) return ff_add_f(ff_add(w, ff_ln2()), 0.25f * __expf(-2.f * w.hi));
  const ff x = ff_exp(w);
  if (x.hi < 1e-3f) {
    const float x2 = x.hi * x.hi;
    return ff_mul_f(x, 1.f - x2 * (1.f / 6.f - x2 * 0.075f));
  }
  return ff_log(ff_add(x, ff_sqrt(ff_add_f(ff_mul(x, x), 1.f))));
}

// ageing-law state after dt at slip rate V (calc_RSF.c:96-103), as a float
// pair.  The state (~50 in the host rock) enters the slip rate as e^(b/a
// phi) with b/a up to ~2, so its FP32 evaluation error (a few ulps from the
// logarithms of V0/V and of 1 - e^-x, each of size ~20) would be several
// 1e-6 of the slip rate: the logarithms and the sums run in float-float,
// and only corrections far below an ulp of the state stay in FP32.
// dt is a float pair (dt_hi, dt_lo).
__device__ __forceinline__ ff new_state_ff(float ph, float V, ff dt, float L, float V0) {
  const ff x = ff_div(ff_mul_f(dt, V), ff_f(L));  // V dt / L
  // the reference's test V dt / L <= 1e-6, on the FP64 constant as a pair
  const float c_hi = 9.99999997e-07f, c_lo = 2.52475725e-15f;
  if (x.hi < c_hi || (x.hi == c_hi && x.lo <= c_lo)) {
    // log(e^ph (1 - x) + V0 dt / L) = ph + log1p(-x + V0 dt / L e^-ph)
    const float t = -x.hi + V0 * dt.hi / L * expf(-ph);
    return ff_add_f(ff_f(ph), log1pf(t));
  }
  // log(A + B), A = V0/V (1 - e^-x), B = e^(ph - x)
  const ff la = ff_add(ff_log(ff_div(ff_f(V0), ff_f(V))), ff_log(ff_f(-expm1f(-x.hi))));
  const ff lb = ff_sub(ff_f(ph), x);
  const bool a_big = la.hi > lb.hi || (la.hi == lb.hi && la.lo >= lb.lo);
  const ff hi = a_big ? la : lb, lo = a_big ? lb : la;
  return ff_add_f(hi, log1pf(expf(ff_sub(lo, hi).hi)));
}

// interpolate_center2basic (interpolation.c:1600-1637): means of the four
// pressure nodes around each interior basic node; the plastic and elastic
// strain rates use the reference's per-node terms (IEEE division: a node no
// marker reached has gd = 0 and gives inf as in the reference).  use_dsxx:
// sxx - sxxe is taken from DSXX, which recompute_stress_strainrate wrote
// for the current sxx and sxxe (the FP32 difference cancels at small dt)
__global__ void k_c2b(Grid g, Nodes N, float dt, float dt_lo, int use_dsxx) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  long m2 = m3 % yn, m1 = m3 / yn;
  if (!(m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1)) return;
  const float *exx = N.f(V2C_NF_EXX), *sxx = N.f(V2C_NF_SXX), *sxxe = N.f(V2C_NF_SXXE);
  const float *gd = N.f(V2C_NF_GD), *nd = N.f(V2C_NF_ND_M2C), *pr = N.f(V2C_NF_PR);
  const float *dsxx = N.f(V2C_NF_DSXX);
  const ff dt_ff{dt, dt_lo};
  ff spl = ff_f(0.f), sel = ff_f(0.f);
  const long k[4] = {m3, m3 + 1, m3 + yn, m3 + yn + 1};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const long i = k[q];
    const float e = exx[i], s = sxx[i], s0 = sxxe[i], G = gd[i];
    ff ds;
    if (use_dsxx) ds = ff_f(dsxx[i]);
    else ds.hi = two_sum(s, -s0, ds.lo);
    const ff gdt2 = ff_mul(ff_f(2.f * G), dt_ff);  // 2 G dt
    spl = ff_add(spl, ff_sub(ff_sub(ff_f(e), ff_div_ieee(ds, gdt2)),
                             ff_div_ieee(ff_f(s), ff_f(2.f * nd[i]))));
    sel = ff_add(sel, ff_add_f(ff_mul_f(gdt2, e), s0));
  }
  N.f(V2C_NF_EXXS)[m3] = rn(ff_quarter_sum(exx[k[0]], exx[k[1]], exx[k[2]], exx[k[3]]));
  N.f(V2C_NF_EXXPL)[m3] = rn(ff_scale(spl, 0.25f));
  N.f(V2C_NF_SXXS)[m3] = rn(ff_quarter_sum(sxx[k[0]], sxx[k[1]], sxx[k[2]], sxx[k[3]]));
  N.f(V2C_NF_PRS)[m3] = rn(ff_quarter_sum(pr[k[0]], pr[k[1]], pr[k[2]], pr[k[3]]));
  N.f(V2C_NF_EXXEL)[m3] = rn(ff_scale(sel, 0.25f));
}

// bilinear weight of the centre between lines m1-1 and m1 against the
// clamped basic stencil [m10, m10+1] (interpolation.c:1655-1667): the
// centre lies in cell m1-1 (nxsearch of the midpoint, checked in FP64 for
// a midpoint that rounds onto line m1), so the weight is 1/2 inside and
// clamps to 0 or 1 where the stencil was shifted at the edges
__device__ __forceinline__ int centre_stencil(const double *gl, const float *w, int n, int m1,
                                              float &e) {
  const double x = (gl[m1] + gl[m1 - 1]) / 2;
  int nx = (x >= gl[m1] && m1 <= n - 2) ? m1 : m1 - 1;
  int m10 = nx < 1 ? 1 : (nx > n - 3 ? n - 3 : nx);
  // offset of the midpoint from line m10: half the cell inside, FP64 at the
  // shifted edge stencils (where the weight clamps to 0 or 1)
  const float X = (m10 == nx && nx == m1 - 1) ? 0.5f * __ldg(w + m1 - 1) : (float)(x - gl[m10]);
  e = X / __ldg(w + m10);
  e = fminf(fmaxf(e, 0.f), 1.f);
  return m10;
}

// interpolate_basic2center (interpolation.c:1639-1685): nd at every node
// with m1, m2 >= 1 as the harmonic mean of nu over the basic stencil
__global__ void k_b2c(Grid g, Nodes N, unsigned long long *stat) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  const int m2 = (int)(m3 % yn), m1 = (int)(m3 / yn);
  if (!(m1 >= 1 && m2 >= 1)) return;
  float e, n;
  const int m10 = centre_stencil(g.gx, g.wx, g.xn, m1, e);
  const int m20 = centre_stencil(g.gy, g.wy, g.yn, m2, n);
  const float dm0 = (1.f - e) * (1.f - n), dm1 = (1.f - e) * n, dm2 = e * (1.f - n), dm3 = e * n;
  const float *nu = N.f(V2C_NF_NU);
  const long m4 = (long)m10 * yn + m20;
  const float n0 = nu[m4], n1 = nu[m4 + 1], n2 = nu[m4 + yn], n3 = nu[m4 + yn + 1];
  float nd;
  if (n0 > 0.f && n1 > 0.f && n2 > 0.f && n3 > 0.f && isfinite(n0 + n1 + n2 + n3)) {
    // the harmonic mean in float-float, rounded once
    ff h = ff_div(ff_f(dm0), ff_f(n0));
    h = ff_add(h, ff_div(ff_f(dm1), ff_f(n1)));
    h = ff_add(h, ff_div(ff_f(dm2), ff_f(n2)));
    h = ff_add(h, ff_div(ff_f(dm3), ff_f(n3)));
    nd = rn(ff_div_ieee(ff_f(1.f), h));
  } else {  // a zero or non-finite viscosity: the reference's IEEE result
    nd = 1.f / (dm0 / n0 + dm1 / n1 + dm2 / n2 + dm3 / n3);
  }
  N.f(V2C_NF_ND)[m3] = nd;
  if (!(nd > 0.f)) atomicAdd(stat + ST_NAN, 1ull);  // the reference prints these
}

// nueffcalc (momentum_continuity_addmatrix_checkerror.c:380-393) in
// float-float: Z = G dt / (G dt + nvp), nueff = Z nvp (lower limit nubeg)
__device__ __forceinline__ ff nueff_ff(float nvp, float ggeff, ff dt, float nubeg, ff &Z) {
  const ff gdt = ff_mul_f(dt, ggeff);
  Z = ff_div_ieee(gdt, ff_add_f(gdt, nvp));
  const ff nueff = ff_mul_f(Z, nvp);
  return rn(nueff) < nubeg ? ff_f(nubeg) : nueff;
}

// recompute_stress_strainrate (momentum_continuity_iterate.c:214-262) with
// sxxcalc / sxycalc (momentum_continuity_addmatrix_checkerror.c:446-572):
// strain rates from the node velocities, visco-elastic stresses from the
// node viscosities and the previous elastic stresses, in float-float from
// the FP64 line spacings, each output rounded once.
__global__ void k_recompute(Grid g, Nodes N, float dt, float dt_lo, float nubeg,
                            const double *vx64, const double *vy64) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  const int m2 = (int)(m3 % yn), m1 = (int)(m3 / yn);
  if (!(m1 >= 1 && m2 >= 1)) return;
  const long v0 = m3 - yn - 1, v1 = v0 + 1, v2 = v0 + yn;
  const float *vx = N.f(V2C_NF_VX), *vy = N.f(V2C_NF_VY);
  const ff dt_ff{dt, dt_lo};
  ff Z;
  ff nueff = nueff_ff(N.f(V2C_NF_ND)[m3], N.f(V2C_NF_GD)[m3], dt_ff, nubeg, Z);
  // velocity differences from the FP64 copy where there is one: adjacent
  // velocities agree in their leading digits, which FP32 storage would keep
  // and the differences would lose
  auto dvx = [&](long a, long b) {
    if (vx64) return ff_from_double(__ldg(vx64 + a) - __ldg(vx64 + b));
    ff d;
    d.hi = two_sum(vx[a], -vx[b], d.lo);
    return d;
  };
  auto dvy = [&](long a, long b) {
    if (vy64) return ff_from_double(__ldg(vy64 + a) - __ldg(vy64 + b));
    ff d;
    d.hi = two_sum(vy[a], -vy[b], d.lo);
    return d;
  };
  auto span = [](const double *gl, int i, int j) { return ff_from_double(gl[i] - gl[j]); };
  const ff edotxx = ff_scale(ff_sub(ff_div(dvx(v2, v0), span(g.gx, m1, m1 - 1)),
                                    ff_div(dvy(v1, v0), span(g.gy, m2, m2 - 1))), 0.5f);
  const float s0 = N.f(V2C_NF_SXXE)[m3];
  const ff two_nu_e = ff_scale(ff_mul(nueff, edotxx), 2.f);
  N.f(V2C_NF_EXX)[m3] = rn(edotxx);
  N.f(V2C_NF_SXX)[m3] = rn(ff_add(two_nu_e, ff_mul_f(ff_add_f(ff_neg(Z), 1.f), s0)));
  // the increment itself: at a coseismic dt sxx and sxxe agree to a few
  // FP32 ulps and their difference would be rounding
  N.f(V2C_NF_DSXX)[m3] = rn(ff_sub(two_nu_e, ff_mul_f(Z, s0)));
  if (m1 < g.xn - 1 && m2 < g.yn - 1) {
    nueff = nueff_ff(N.f(V2C_NF_NU)[m3], N.f(V2C_NF_GG)[m3], dt_ff, nubeg, Z);
    const ff exy1 = ff_div(dvx(m3, v2), span(g.gy, m2 + 1, m2 - 1));
    const ff exy2 = ff_div(dvy(m3, v1), span(g.gx, m1 + 1, m1 - 1));
    const ff exy = ff_add(exy1, exy2);
    N.f(V2C_NF_EXY)[m3] = rn(exy);
    N.f(V2C_NF_ESP)[m3] = rn(ff_sub(exy1, exy2));
    N.f(V2C_NF_SXY)[m3] = rn(ff_add(ff_scale(ff_mul(nueff, exy), 2.f),
                                    ff_mul_f(ff_add_f(ff_neg(Z), 1.f), N.f(V2C_NF_SXYE)[m3])));
  }
}

// copyarrays (momentum_continuity_iterate.c:265-281): the solved slip and
// state rates become the final ones
__global__ void k_copyarrays(Grid g, Nodes N) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  const long m2 = m3 % yn, m1 = m3 / yn;
  if (!(m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1)) return;
  const float v = N.f(V2C_NF_RK_SLIPRS_SOLVED)[m3];
  N.f(V2C_NF_SLIPRS)[m3] = v;
  N.f(V2C_NF_RK_SLIPRS_FINAL)[m3] = v;
  N.f(V2C_NF_RK_PHIDTS_FINAL)[m3] = N.f(V2C_NF_RK_PHIDTS_SOLVED)[m3];
}

// accumulated slip of every marker (the per-marker Newton's slip rate)
__global__ void k_marker_slip_acc(const float *slipv, long n, double dt, double *acc) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) acc[i] += dt * (double)slipv[i];
}

// accumulated slip of every interior basic node: acc += dt * slip rate
__global__ void k_slip_acc(Grid g, const float *v, double dt, double *acc) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  const long m2 = m3 % yn, m1 = m3 / yn;
  if (m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1) acc[m3] += dt * (double)v[m3];
}

__global__ void k_c2b_old(Grid g, Nodes N) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const long yn = g.yn;
  long m2 = m3 % yn, m1 = m3 / yn;
  if (m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1) {
    const float *exxe = N.f(V2C_NF_EXXE), *sxxe = N.f(V2C_NF_SXXE), *sppe = N.f(V2C_NF_SPPE);
    N.f(V2C_NF_EXXES)[m3] = rn(ff_quarter_sum(exxe[m3], exxe[m3 + 1], exxe[m3 + yn], exxe[m3 + yn + 1]));
    N.f(V2C_NF_SXXES)[m3] = rn(ff_quarter_sum(sxxe[m3], sxxe[m3 + 1], sxxe[m3 + yn], sxxe[m3 + yn + 1]));
    N.f(V2C_NF_SPPES)[m3] = rn(ff_quarter_sum(sppe[m3], sppe[m3 + 1], sppe[m3 + yn], sppe[m3 + yn + 1]));
  }
}

__global__ void k_before(Grid g, Nodes N, Scal S, float dt, float dt_lo, int rk,
                         unsigned long long *stat) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const v2c_params &p = S.p;
  long m2 = m3 % g.yn, m1 = m3 / g.yn;
  if (!(m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1)) return;
  const float W = (float)p.faultwidth;
  const ff dt_ff{dt, dt_lo};
  const bool nP_const = p.pmode == 0 || p.timesum == 0;
  const ff nP_ff = nP_const ? ff{S.sn_hi, S.sn_lo} : ff_f(N.f(V2C_NF_SPPES)[m3]);
  const float sxxs = N.f(V2C_NF_SXXS)[m3], sxy = N.f(V2C_NF_SXY)[m3];
  const float sigin = sqrtf(sxxs * sxxs + sxy * sxy);
  float nu;
  bool err = false;
  if (sigin > 0.f || p.RSFmode == 0) {
    // calc_vpvisc
    float V = 0.f;
    if (rk == 0) V = (p.RSFmode == 1 || p.timesum > 0) ? N.f(V2C_NF_RK_SLIPRS_FINAL)[m3] : 0.f;
    // later passes take the last solved rate (calc_RSF.c:58-86; the state
    // rates and the rkmod 3 histories it also selects are never used)
    if ((p.rkmod == 0 && rk > 0) || (rk > 0 && rk < 3) || (rk == 3 && p.rkmod == 3))
      V = N.f(V2C_NF_RK_SLIPRS_SOLVED)[m3];
    // V / W as a float pair (the plastic strain rate)
    const ff VW = ff_div(ff_f(V), ff_f(W));
    N.f(V2C_NF_PES)[m3] = rn(ff_add_f(ff_mul(VW, dt_ff), N.f(V2C_NF_PE)[m3]));
    float newstate = 0.f;
    ff sy;  // the yield strength, rounded once for storage
    if (p.RSFmode == 1) {
      const float L = N.f(V2C_NF_LS)[m3], V0 = N.f(V2C_NF_V0S)[m3], ph = N.f(V2C_NF_PHIS)[m3];
      const ff ns = new_state_ff(ph, V, dt_ff, L, V0);
      newstate = ns.hi;
      // radiation damping 4.3303e6 V (an exact FP32 constant)
      ff rad = ff_f(0.f);
      if (p.inertyn == 0) rad.hi = two_prod(4.3303e+06f, V, rad.lo);
      const float a = N.f(V2C_NF_AS)[m3], b = N.f(V2C_NF_BS)[m3], mu = N.f(V2C_NF_MUS_S)[m3];
      if (V == 0.f) {
        // V/V0 e^... = 0: the yield strength is the damping term alone
        sy = rad;
      } else {
        // exponents in float-float (see ff_log_sinh); asinh is odd, so a
        // negative V (an error the flags below report) keeps its sign
        const ff lnVV0 = ff_log(ff_div(ff_f(fabsf(V)), ff_f(V0)));
        if (p.power_law_RSF > 0) {
          sy = V > 0.f ? ff_add(ff_exp(ff_add(ff_add(ff_log(ff_mul_f(nP_ff, mu)),
                                                     ff_mul(ff_div(ff_f(a), ff_f(mu)), lnVV0)),
                                              ff_div(ff_mul_f(ns, b), ff_f(mu)))),
                                rad)
                       : ff_f(__int_as_float(0x7fc00000));
        } else {
          ff as = ff_mul(ff_mul_f(nP_ff, a),
                         ff_asinh_exp(ff_add(ff_sub(lnVV0, ff_ln2()),
                                             ff_div(ff_add_f(ff_mul_f(ns, b), mu), ff_f(a)))));
          if (V < 0.f) as = ff_neg(as);
          sy = ff_add(as, rad);
        }
      }
    } else {
      sy = ff_add_f(ff_mul_f(nP_ff, N.f(V2C_NF_MUS_S)[m3]), N.f(V2C_NF_COHESION)[m3]);
    }
    const float syield = rn(sy);
    const float nm = N.f(V2C_NF_NU_M2C)[m3];
    // nm syield / (2 nm V / W + syield)
    auto vp_of = [&]() {
      return rn(ff_div_ieee(ff_mul_f(sy, nm), ff_add(ff_mul_f(VW, 2.f * nm), sy)));
    };
    float vp;
    if (p.RSFmode == 1) vp = (syield > 0.f) ? vp_of() : nm;
    else vp = vp_of();
    N.f(V2C_NF_PHIS_IT)[m3] = newstate;
    N.f(V2C_NF_SYIELDS)[m3] = syield;
    N.f(V2C_NF_NUVP_IT)[m3] = vp;
    N.f(V2C_NF_SLIPRS)[m3] = V;
    if ((p.timesum > 0 && (isnan(newstate) || isnan(syield) || isnan(vp) || vp == 0.f || isnan(V))) ||
        V < 0.f || syield < 0.f)
      err = true;
    nu = vp;
  } else {
    nu = N.f(V2C_NF_NU_M2C)[m3];
  }
  N.f(V2C_NF_NU)[m3] = nu;
  if (isnan(nu) || nu <= 0.f) err = true;
  if (err) atomicAdd(stat + ST_NAN, 1ull);
}

// per-block partial sums of (syield - sigin)^2 and counts
constexpr int AB = 256;
__global__ void k_after(Grid g, Nodes N, Scal S, float dt, float *part) {
  __shared__ float sd[AB];
  __shared__ float sc[AB];
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  float d2 = 0.f, cnt = 0.f;
  const v2c_params &p = S.p;
  if (m3 < g.nn) {
    long m2 = m3 % g.yn, m1 = m3 / g.yn;
    if (m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < g.yn - 1) {
      const float W = (float)p.faultwidth;
      const bool nps_const = p.pmode == 0 || p.timesum == 0;
      const ff nps_ff = nps_const ? ff{S.sn_hi, S.sn_lo} : ff_f(N.f(V2C_NF_SPPES)[m3]);
      const float sxxs = N.f(V2C_NF_SXXS)[m3], sxy = N.f(V2C_NF_SXY)[m3];
      const float sigin = sqrtf(sxxs * sxxs + sxy * sxy);
      // the stress invariant as a float pair
      const ff sig = ff_sqrt(ff_add(ff_mul(ff_f(sxxs), ff_f(sxxs)), ff_mul(ff_f(sxy), ff_f(sxy))));
      const float a = N.f(V2C_NF_AS)[m3], b = N.f(V2C_NF_BS)[m3], mu = N.f(V2C_NF_MUS_S)[m3];
      const float V0 = N.f(V2C_NF_V0S)[m3], L = N.f(V2C_NF_LS)[m3], ph = N.f(V2C_NF_PHIS_IT)[m3];
      float V;
      if (p.RSFmode == 1) {
        if (sigin > 0.f) {
          // the slip rate's exponent in float-float from the FP32 node
          // values (see ff_log_sinh)
          const ff bpa = ff_div(ff_mul_f(ff_f(ph), b), ff_f(a));  // b phi / a
          ff E;
          if (p.power_law_RSF > 0)
            E = ff_sub(ff_add(ff_log(ff_f(V0)),
                              ff_mul(ff_div(ff_f(mu), ff_f(a)),
                                     ff_log(ff_div(sig, ff_mul_f(nps_ff, mu))))),
                       bpa);
          else
            E = ff_sub(ff_add(ff_log(ff_f(2.f * V0)), ff_log_sinh(ff_div(sig, ff_mul_f(nps_ff, a)))),
                       ff_add(ff_div(ff_f(mu), ff_f(a)), bpa));
          // e^E rounded once; below e^-80 (under the 1e-40 floor's FP32
          // neighbourhood) the FP32 exponential and its subnormals
          V = E.hi > -80.f ? rn(ff_exp(E)) : exp_ff(E);
          const float ex = N.f(V2C_NF_EXXPL)[m3], ey = N.f(V2C_NF_EXY)[m3];
          const float Vslip = sqrtf(ex * ex + ey * ey) * W;
          V = (V <= Vslip) ? V : Vslip;
          if (V < 1e-40f) V = 1e-40f;
        } else {
          V = 0.f;
        }
        N.f(V2C_NF_RK_PHIDTS_SOLVED)[m3] = V0 / L * expf(-ph) - V / L;
      } else {
        const float G = N.f(V2C_NF_GG)[m3], NUVP = N.f(V2C_NF_NU)[m3], NU = N.f(V2C_NF_NU_M2C)[m3];
        const float E2EL = sigin / (NUVP / (G * dt + NUVP));
        const float A = N.f(V2C_NF_SYIELDS)[m3] / E2EL;
        if (A < 1.f) {
          const float nup = G * dt * A / (1.f - A);
          V = W * (sigin / 2.f * (1.f / nup - 1.f / NU));
        } else {
          V = 0.f;
        }
      }
      N.f(V2C_NF_RK_SLIPRS_SOLVED)[m3] = V;
      if (V > 0.f) {
        const float d = rn(ff_sub(ff_f(N.f(V2C_NF_SYIELDS)[m3]), sig));
        N.f(V2C_NF_RK_DELTAS)[m3] = d;
        d2 = d * d;
        cnt = 1.f;
      } else {
        N.f(V2C_NF_RK_DELTAS)[m3] = 0.f;
      }
    }
  }
  sd[threadIdx.x] = d2;
  sc[threadIdx.x] = cnt;
  __syncthreads();
  for (int off = AB / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      sd[threadIdx.x] += sd[threadIdx.x + off];
      sc[threadIdx.x] += sc[threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sd[0];
    part[2 * blockIdx.x + 1] = sc[0];
  }
}

// fold the block partials in block order (single block, fixed order); the
// few thousand partials are summed in FP64
__global__ void k_after_fold(const float *part, long nb, double *out) {
  __shared__ double sd[AB], sc[AB];
  double d = 0, c = 0;
  for (long i = threadIdx.x; i < nb; i += AB) {
    d += part[2 * i];
    c += part[2 * i + 1];
  }
  sd[threadIdx.x] = d;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int off = AB / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      sd[threadIdx.x] += sd[threadIdx.x + off];
      sc[threadIdx.x] += sc[threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sd[0];
    out[1] = sc[0];
  }
}

__global__ void k_bc(BcRows r, Nodes N, float *scratch) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r.n) return;
  float v = r.c[i];
  for (int k = 0; k < r.nref[i]; k++) {
    const int q = i * V2C_BC_MAXREF + k;
    v = v - N.f(r.rfield[q])[r.rnode[q]] * (-r.rcoef[q]);
  }
  scratch[i] = v;
}
__global__ void k_bc_store(BcRows r, Nodes N, const float *scratch) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < r.n) N.f(r.field[i])[r.node[i]] = scratch[i];
}

__global__ void k_to_f32(const double *src, float *dst, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}
__global__ void k_to_f64(const float *src, double *dst, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

// several node fields at once: blockIdx.y picks the field, stage holds
// them one after another (field list order)
struct FieldList {
  int f[V2C_NF_N];
};
__global__ void k_fields_to_f64(const float *base, long nn, FieldList L, double *stage) {
  const float *src = base + (long)L.f[blockIdx.y] * nn;
  double *dst = stage + (long)blockIdx.y * nn;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += (long)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
__global__ void k_fields_to_f32(const double *stage, long nn, FieldList L, float *base) {
  const double *src = stage + (long)blockIdx.y * nn;
  float *dst = base + (long)L.f[blockIdx.y] * nn;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += (long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

FieldList field_list(const int *fields, int count) {
  FieldList L;
  for (int k = 0; k < V2C_NF_N; k++) L.f[k] = k < count ? fields[k] : 0;
  return L;
}

}  // namespace

void launch_c2b_old(const Grid &g, const Nodes &N, cudaStream_t st) {
  k_c2b_old<<<nblk(g.nn, 256), 256, 0, st>>>(g, N);
}

void launch_c2b(const Grid &g, const Nodes &N, double dt, int use_dsxx, cudaStream_t st) {
  const float hi = (float)dt, lo = (float)(dt - (double)hi);
  k_c2b<<<nblk(g.nn, 256), 256, 0, st>>>(g, N, hi, lo, use_dsxx);
}
void launch_recompute(const Grid &g, const Nodes &N, const Scal &S, double dt, const double *vx64,
                      const double *vy64, cudaStream_t st) {
  const float hi = (float)dt, lo = (float)(dt - (double)hi);
  k_recompute<<<nblk(g.nn, 256), 256, 0, st>>>(g, N, hi, lo, S.nubeg_f, vx64, vy64);
}
void launch_copyarrays(const Grid &g, const Nodes &N, cudaStream_t st) {
  k_copyarrays<<<nblk(g.nn, 256), 256, 0, st>>>(g, N);
}
void launch_marker_slip_acc(const float *slipv, long n, double dt, double *acc, cudaStream_t st) {
  if (n > 0) k_marker_slip_acc<<<nblk(n, 256), 256, 0, st>>>(slipv, n, dt, acc);
}
void launch_slip_acc(const Grid &g, const Nodes &N, double dt, double *acc, cudaStream_t st) {
  k_slip_acc<<<nblk(g.nn, 256), 256, 0, st>>>(g, N.f(V2C_NF_RK_SLIPRS_FINAL), dt, acc);
}
void launch_b2c(const Grid &g, const Nodes &N, unsigned long long *stat, cudaStream_t st) {
  k_b2c<<<nblk(g.nn, 256), 256, 0, st>>>(g, N, stat);
}
void launch_before_solve(const Grid &g, const Nodes &N, const Scal &S, double dt, int rk,
                         unsigned long long *stat, cudaStream_t st) {
  const float hi = (float)dt, lo = (float)(dt - (double)hi);
  k_before<<<nblk(g.nn, 256), 256, 0, st>>>(g, N, S, hi, lo, rk, stat);
}

void launch_after_solve(const Grid &g, const Nodes &N, const Scal &S, double dt, int rk,
                        double *red, cudaStream_t st) {
  (void)rk;
  long nb = (g.nn + AB - 1) / AB;
  float *part = (float *)(red + 2);
  k_after<<<(unsigned)nb, AB, 0, st>>>(g, N, S, (float)dt, part);
  k_after_fold<<<1, AB, 0, st>>>(part, nb, red);
}

void launch_bc(const BcRows &rows, const Nodes &N, float *scratch, cudaStream_t st) {
  if (rows.n <= 0) return;
  // all rows read first, then stored: a row never sees another's new value
  k_bc<<<nblk(rows.n, 256), 256, 0, st>>>(rows, N, scratch);
  k_bc_store<<<nblk(rows.n, 256), 256, 0, st>>>(rows, N, scratch);
}

void launch_node_to_f32(const double *src, float *dst, long n, cudaStream_t st) {
  if (n > 0) k_to_f32<<<nblk(n, 256), 256, 0, st>>>(src, dst, n);
}
void launch_node_to_f64(const float *src, double *dst, long n, cudaStream_t st) {
  if (n > 0) k_to_f64<<<nblk(n, 256), 256, 0, st>>>(src, dst, n);
}
void launch_fields_to_f64(const float *base, long nn, const int *fields, int count, double *stage,
                          cudaStream_t st) {
  if (nn <= 0 || count <= 0) return;
  const unsigned bx = nblk(nn, 256) < 152 * 8 ? nblk(nn, 256) : 152 * 8;
  k_fields_to_f64<<<dim3(bx, (unsigned)count), 256, 0, st>>>(base, nn, field_list(fields, count),
                                                             stage);
}
void launch_fields_to_f32(const double *stage, long nn, const int *fields, int count, float *base,
                          cudaStream_t st) {
  if (nn <= 0 || count <= 0) return;
  const unsigned bx = nblk(nn, 256) < 152 * 8 ? nblk(nn, 256) : 152 * 8;
  k_fields_to_f32<<<dim3(bx, (unsigned)count), 256, 0, st>>>(stage, nn, field_list(fields, count),
                                                             base);
}

}  // namespace v2c
