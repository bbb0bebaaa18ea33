/*
 * v2c_oracle.c -- FP64 CPU restatement of the VELO2CYCLEs MIC step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see v2c_oracle.h.  Expressions
 * keep the reference's evaluation order so that, built with
 * -ffp-contract=off like the reference harness, results match the
 * reference bit for bit on the same inputs (tests/test_oracle_pin.py).
 */
#include "v2c_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define RT(s, f, t) ((s)->rt[(long)(f) * V2C_MAXTMR + (t)])
#define AB(a) ((a) >= 0 ? (a) : -(a)) /* ABSV, headevps.c:5 */

/* nxsearch / nysearch, interpolation.c:1536-1573: bisection, ties go left
 * (gx[central] > x moves the right limit), result clamped to n-2. */
long v2c_oracle_nxsearch(const double *g, long n, double x) {
  long lo = 0, hi = n - 1;
  do {
    long c = (lo + hi) / 2;
    if (g[c] > x)
      hi = c;
    else
      lo = c;
  } while (hi - lo > 1);
  if (lo > n - 2) lo = n - 2;
  return lo;
}

/* ---------------------------------------------------------------- helpers */
static long nnodes(const v2c_oracle_state *s) {
  return s->p.xnumx * s->p.ynumy;
}

/* allinterpomp, interpolation.c:1923-1958: pressure at a point from the four
 * surrounding pressure (cell-centre) nodes.  The search happens before the
 * clamp, as in the reference. */
static double interp_pressure(const v2c_oracle_state *s, double x, double y) {
  const double *gx = s->gx, *gy = s->gy, *pr = s->N[V2C_NF_PR];
  long xn = s->p.xnumx, yn = s->p.ynumy;
  long m10 = v2c_oracle_nxsearch(gx, xn, x);
  long m20 = v2c_oracle_nxsearch(gy, yn, y);
  if (x < 0) x = 0; else if (x > s->p.xsize) x = s->p.xsize;
  if (y < 0) y = 0; else if (y > s->p.ysize) y = s->p.ysize;
  if (x > (gx[m10] + gx[m10 + 1]) / 2.0) m10++;
  if (y > (gy[m20] + gy[m20 + 1]) / 2.0) m20++;
  if (m10 < 1) m10 = 1;
  if (m10 > xn - 2) m10 = xn - 2;
  if (m20 < 1) m20 = 1;
  if (m20 > yn - 2) m20 = yn - 2;
  double e = (x - (gx[m10 - 1] + gx[m10]) / 2.0) / ((gx[m10 + 1] - gx[m10 - 1]) / 2.0);
  double n = (y - (gy[m20 - 1] + gy[m20]) / 2.0) / ((gy[m20 + 1] - gy[m20 - 1]) / 2.0);
  long m3 = m10 * yn + m20;
  return (1.0 - e) * (1.0 - n) * pr[m3] + (1.0 - e) * n * pr[m3 + 1] +
         e * (1.0 - n) * pr[m3 + yn] + e * n * pr[m3 + yn + 1];
}

/* dencalcomp, density_ductilevisc_calc.c:2-27 */
static void density(const v2c_oracle_state *s, double mtk, double mpb, int mm2,
                    double *mro, double *mbb, double *maa) {
  double bb = RT(s, V2C_RT_BB, mm2), aa = RT(s, V2C_RT_AA, mm2);
  *mbb = bb / (1.0 - bb * (mtk - 298.15));
  *maa = 1.e-8 * aa / (1.0 + aa * (mpb - 1.0) * 1e-3);
  if (s->p.densimod == 0)
    *mro = RT(s, V2C_RT_RO, mm2);
  else
    *mro = RT(s, V2C_RT_RO, mm2) * (1.0 - bb * (mtk - 298.15)) *
           (1.0 + aa * (mpb - 1.0) * 1e-3);
}

/* ductilevisc, density_ductilevisc_calc.c:29-223, including the creep Newton
 * on the dislocation viscosity (loop :173-200, at most 50 iterations, stop
 * when |log10(eta_k/eta_k-1)| < 1e-6 after more than 3).  A type that fits
 * neither the Newtonian nor the power-law branch leaves the reference's
 * result undefined; NaN is returned for it. */
double v2c_oracle_ductilevisc(const v2c_oracle_state *s, int mm2, double SXY,
                              double SXX, double EXY, double EXX, double mtk,
                              double mpb) {
  const v2c_params *p = &s->p;
  double nueff = NAN;
  double nu = RT(s, V2C_RT_NU, mm2), dh = RT(s, V2C_RT_DH, mm2);
  double dv = RT(s, V2C_RT_DV, mm2), ss = RT(s, V2C_RT_SS, mm2);
  double mm = RT(s, V2C_RT_MM, mm2), gg = RT(s, V2C_RT_GG, mm2);
  (void)EXY;
  (void)EXX;
  if (mm2 == 1) {
    nueff = nu;
    if (p->stickymod == 1 && p->timesum > 4e7) {
      double cap = RT(s, V2C_RT_GG, 2) * p->timestep / 100;
      if (nueff > cap) nueff = cap;
    }
    return nueff;
  }
  if (dh == 0 && dv == 0 && (ss == 0 || mm == 1.0)) return nu;
  if (!(nu > 0 && (dh != 0 || dv != 0) && ss != 0 && mm != 1.0)) return nueff;

  double nunewt = 0, nupowl = 0;
  if (nu) {
    double sigin = pow(SXX * SXX + SXY * SXY, 0.5);
    double e1 = (dh + dv * mpb) / (8.314 * mtk);
    if (e1 > 150.0) e1 = 150.0;
    e1 = exp(e1);
    double k1 = nu / pow(ss, mm - 1.0);
    nunewt = 1.0 / (0.5 * k1 * e1);
    double siginnew = sigin;
    nupowl = 0;
    if (siginnew > 0) nupowl = 1.0 / (0.5 * siginnew * nu * e1 / pow(siginnew, mm));
    if (siginnew > 0) {
      double etadisl = 0.5 * siginnew * nu * e1 / pow(siginnew, mm);
      double etadisl_new = etadisl, etadisl_old;
      double etadiff = 0.5 * k1 * e1;
      double coeff = pow(etadisl, 1.0 / mm);
      double eta_prev = 0, mnu0 = 0;
      int counter = 0, done = 0;
      while (!done && counter < 50) {
        counter++;
        etadisl_old = etadisl_new;
        mnu0 = 1.0 / (1.0 / etadiff + 1.0 / etadisl_new);
        double prefactor = (etadiff + etadisl_old) / etadiff;
        double f1 = pow(prefactor * (gg * p->timestep + mnu0), (mm - 1) / mm);
        double f2 = etadisl_old - coeff * f1;
        double df = 1 - (mm - 1) / (mm * etadiff) * coeff *
                            pow(prefactor * (gg * p->timestep + mnu0), -1 / mm) *
                            ((gg * p->timestep + mnu0) +
                             pow(etadiff, 2 / (etadiff + etadisl_old)));
        etadisl_new = etadisl_old - f2 / df;
        if (counter > 3 && fabs(log10(mnu0 / eta_prev)) < 1.0e-6) done = 1;
        eta_prev = mnu0;
      }
      nupowl = 1 / etadisl_new;
    }
  }
  nueff = 1.0 / (nunewt + nupowl);
  if (nueff < p->nubeg) nueff = p->nubeg;
  if (nueff > p->nuend) nueff = p->nuend;
  if (nueff < RT(s, V2C_RT_N0, mm2)) nueff = RT(s, V2C_RT_N0, mm2);
  if (nueff > RT(s, V2C_RT_N1, mm2)) nueff = RT(s, V2C_RT_N1, mm2);
  return nueff;
}

/* distance from the frictional band centre line, calc_RSF.c:226 */
static double band_radius(const v2c_params *p, double x, double y) {
  double d = y - (p->fault_y + p->fault_slope * x);
  return AB(d);
}

/* calc_frictionpara, calc_RSF.c:224-295: position-dependent RSF parameters
 * of one marker, written to the marker arrays. */
static void friction_marker(v2c_oracle_state *s, long mm1, int mm2) {
  const v2c_params *p = &s->p;
  double x = s->M[V2C_MF_X][mm1], y = s->M[V2C_MF_Y][mm1];
  double radius = band_radius(p, x, y);
  double h2 = p->half_range;
  if (mm2 > 0) {
    if (radius <= p->fault_hw) {
      double a, b, L, V0;
      if (x > p->end_updip && x < p->start_downdip) {
        a = p->a_vw; b = p->b_vw; L = p->L_vw; V0 = p->V0_vw;
      } else if (x > p->start_updip && x < p->end_updip && p->half_range > 0) {
        double f = (x - (p->start_updip - p->xstpx / 2)) / (2 * h2);
        a = p->a_vs + f * (p->a_vw - p->a_vs);
        b = p->b_vs + f * (p->b_vw - p->b_vs);
        L = p->L_vs + f * (p->L_vw - p->L_vs);
        V0 = p->V0_vs + f * (p->V0_vw - p->V0_vs);
      } else if (x >= p->start_downdip && x < p->end_downdip && p->half_range > 0) {
        double f = (x - (p->start_downdip - p->xstpx / 2)) / (2 * h2);
        a = p->a_vw - f * (p->a_vw - p->a_vs);
        b = p->b_vw - f * (p->b_vw - p->b_vs);
        L = p->L_vw - f * (p->L_vw - p->L_vs);
        V0 = p->V0_vw - f * (p->V0_vw - p->V0_vs);
      } else {
        a = p->a_vs; b = p->b_vs; L = p->L_vs; V0 = p->V0_vs;
      }
      s->M[V2C_MF_FRIC_STATIC][mm1] = 0.2;
      s->M[V2C_MF_A][mm1] = a;
      s->M[V2C_MF_B][mm1] = b;
      s->M[V2C_MF_L0][mm1] = L;
      s->M[V2C_MF_L][mm1] = L;
      s->M[V2C_MF_V0][mm1] = V0;
      s->M[V2C_MF_C0][mm1] = 0.0e0;
      if (p->timesum == p->timestep) s->M[V2C_MF_PHI][mm1] = 0.0;
    } else {
      s->M[V2C_MF_PHI][mm1] = 50.0;
      s->M[V2C_MF_FRIC_STATIC][mm1] = 0.6;
      s->M[V2C_MF_A][mm1] = p->a_hr;
      s->M[V2C_MF_B][mm1] = p->b_hr;
      s->M[V2C_MF_L0][mm1] = p->L_hr;
      s->M[V2C_MF_L][mm1] = p->L_hr;
      s->M[V2C_MF_V0][mm1] = p->V0_hr;
    }
  } else {
    s->M[V2C_MF_FRIC_STATIC][mm1] = 0.6;
    s->M[V2C_MF_A][mm1] = 1.0;
    s->M[V2C_MF_B][mm1] = 0.01;
    s->M[V2C_MF_L0][mm1] = 0.2;
    s->M[V2C_MF_V0][mm1] = p->V0_hr;
  }
}

/* calc_frictionpara_nodes, calc_RSF.c:298-350 */
static void friction_node(v2c_oracle_state *s, double x, double y, long m3) {
  const v2c_params *p = &s->p;
  double radius = band_radius(p, x, y);
  double h2 = p->half_range;
  if (radius <= p->fault_hw) {
    double a, b, L, V0;
    if (x > p->end_updip && x < p->start_downdip) {
      a = p->a_vw; b = p->b_vw; L = p->L_vw; V0 = p->V0_vw;
    } else if (x >= p->start_updip && x <= p->end_updip && p->half_range > 0) {
      double f = (x - (p->start_updip)) / (2 * h2);
      a = p->a_vs + f * (p->a_vw - p->a_vs);
      b = p->b_vs + f * (p->b_vw - p->b_vs);
      L = p->L_vs + f * (p->L_vw - p->L_vs);
      V0 = p->V0_vs + f * (p->V0_vw - p->V0_vs);
    } else if (x >= p->start_downdip && x < p->end_downdip && p->half_range > 0) {
      double f = (x - (p->start_downdip)) / (2 * h2);
      a = p->a_vw - f * (p->a_vw - p->a_vs);
      b = p->b_vw - f * (p->b_vw - p->b_vs);
      L = p->L_vw - f * (p->L_vw - p->L_vs);
      V0 = p->V0_vw - f * (p->V0_vw - p->V0_vs);
    } else {
      a = p->a_vs; b = p->b_vs; L = p->L_vs; V0 = p->V0_vs;
    }
    s->N[V2C_NF_MUS_S][m3] = 0.2;
    s->N[V2C_NF_AS][m3] = a;
    s->N[V2C_NF_BS][m3] = b;
    s->N[V2C_NF_LS][m3] = L;
    s->N[V2C_NF_V0S][m3] = V0;
    s->N[V2C_NF_COHESION][m3] = 0.0;
  } else {
    s->N[V2C_NF_MUS_S][m3] = 0.6;
    s->N[V2C_NF_AS][m3] = p->a_hr;
    s->N[V2C_NF_BS][m3] = p->b_hr;
    s->N[V2C_NF_LS][m3] = p->L_hr;
    s->N[V2C_NF_V0S][m3] = p->V0_hr;
  }
}

/* accumulators of the scatter (the private arrays of interpolation.c:170-206
 * merged in marker order) */
enum {
  A_BM = 0, A_RO, A_ET, A_NU, A_PE, A_ND, A_GG, A_GD, A_SPPE, A_COH, A_PHI,
  A_SXXE, A_SXYE, A_EXXE, A_EXYE, A_HT, A_CP, A_KT, A_TK, A_MRX, A_MRY, A_MVX,
  A_MVY, A_SUMSHEAR, A_SOL0, A_SOL0V, A_SOL1C, A_SOL1V, A_N
};

typedef struct {
  double mnu, mgg, me, mro, mbb, mkt, mtk, mbm;
  double xy, exy, coh, phi, ht, cp, xx, exx, p, vx, vy;
} mk_payload;

/* add2basicnode, interpolation.c:2-30 (the dead friction-parameter sums and
 * marker counts it also forms are never read and are not restated) */
static void add_basic(double **A, long m3, double swt, const mk_payload *q) {
  A[A_NU][m3] += q->mnu * swt;
  A[A_GG][m3] += q->mnu / q->mgg * swt;
  A[A_PE][m3] += q->me * swt;
  A[A_SXYE][m3] += q->xy * swt;
  A[A_EXYE][m3] += q->exy * swt;
  A[A_COH][m3] += q->coh * swt;
  A[A_PHI][m3] += q->phi * swt;
  A[A_SUMSHEAR][m3] += swt;
  A[A_RO][m3] += q->mro * swt;
  A[A_ET][m3] += q->mbb * swt;
  A[A_HT][m3] += q->ht * swt;
  A[A_CP][m3] += q->cp * swt;
  A[A_KT][m3] += q->mkt * swt;
  A[A_TK][m3] += q->mtk * swt;
  A[A_SOL0][m3] += swt;
}
/* add2vnode, interpolation.c:33-39 */
static void add_vx(double **A, long m3, double swt, const mk_payload *q) {
  A[A_MVX][m3] += q->vx * q->mro * swt;
  A[A_MRX][m3] += q->mro * swt;
  A[A_SOL0V][m3] += swt;
}
static void add_vy(double **A, long m3, double swt, const mk_payload *q) {
  A[A_MVY][m3] += q->vy * q->mro * swt;
  A[A_MRY][m3] += q->mro * swt;
  A[A_SOL1V][m3] += swt;
}
/* add2centernode, interpolation.c:42-52 */
static void add_centre(double **A, long m3, double swt, const mk_payload *q) {
  A[A_BM][m3] += q->mbm * swt;
  A[A_ND][m3] += q->mnu * swt;
  A[A_GD][m3] += q->mnu / q->mgg * swt;
  A[A_SXXE][m3] += q->xx * swt;
  A[A_EXXE][m3] += q->exx * swt;
  A[A_SPPE][m3] += q->p * swt;
  A[A_SOL1C][m3] += swt;
}

/* the 13-node stencil of interpolationmod 1, interpolation.c:258-538 */
static void scatter_mode1(double **A, long nodenum, long yn, long nx, long ny,
                          double swt1, double cx, double cy,
                          const mk_payload *q) {
  long m3;
  double dx, dy;
  m3 = nx * yn + ny; /* node i,j */
  if (m3 < nodenum) {
    add_basic(A, m3, swt1 * (1.0 - cx) * (1.0 - cy), q);
    add_vx(A, m3, swt1 * (1.0 - cx) * (1.0 - AB(cy - 0.5)), q);
    add_vy(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * (1.0 - cy), q);
    if (cx < 0.5 && cy < 0.5) add_centre(A, m3, swt1 * (1.0 - cx - 0.5) * (1.0 - cy - 0.5), q);
  }
  m3 = nx * yn + ny + 1; /* node i+1,j */
  if (m3 < nodenum) {
    add_basic(A, m3, swt1 * (1.0 - cx) * cy, q);
    if (cy > 0.5) add_vx(A, m3, swt1 * (1 - cx) * (cy - 0.5), q);
    add_vy(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * cy, q);
    if (cx < 0.5) add_centre(A, m3, swt1 * (1.0 - cx - 0.5) * (1.0 - AB(cy - 0.5)), q);
  }
  m3 = (nx + 1) * yn + ny; /* node i,j+1 */
  if (m3 < nodenum) {
    add_basic(A, m3, swt1 * cx * (1.0 - cy), q);
    add_vx(A, m3, swt1 * cx * (1.0 - AB(cy - 0.5)), q);
    if (cx > 0.5) add_vy(A, m3, swt1 * (cx - 0.5) * (1 - cy), q);
    if (cy < 0.5) add_centre(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * (1.0 - cy - 0.5), q);
  }
  m3 = (nx + 1) * yn + ny + 1; /* node i+1,j+1 */
  if (m3 < nodenum) {
    add_basic(A, m3, swt1 * cx * cy, q);
    if (cy > 0.5) add_vx(A, m3, swt1 * cx * (cy - 0.5), q);
    if (cx > 0.5) add_vy(A, m3, swt1 * (cx - 0.5) * cy, q);
    add_centre(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * (1.0 - AB(cy - 0.5)), q);
  }
  m3 = nx * yn + ny + 2;
  if (m3 < nodenum && cx < 0.5 && cy > 0.5) {
    dx = 1.0 - cx - 0.5; dy = cy - 0.5;
    add_centre(A, m3, swt1 * dx * dy, q);
  }
  m3 = (nx + 1) * yn + ny + 2;
  if (m3 < nodenum && cy > 0.5) {
    dx = 1.0 - AB(cx - 0.5); dy = cy - 0.5;
    add_centre(A, m3, swt1 * dx * dy, q);
  }
  m3 = (nx + 2) * yn + ny + 2;
  if (m3 < nodenum && cx > 0.5 && cy > 0.5) {
    dx = cx - 0.5; dy = cy - 0.5;
    add_centre(A, m3, swt1 * dx * dy, q);
  }
  m3 = (nx + 2) * yn + ny + 1;
  if (m3 < nodenum && cx > 0.5) {
    dx = cx - 0.5; dy = 1.0 - AB(cy - 0.5);
    add_centre(A, m3, swt1 * dx * dy, q);
  }
  m3 = (nx + 2) * yn + ny;
  if (m3 < nodenum && cx > 0.5 && cy < 0.5) {
    dx = cx - 0.5; dy = 1.0 - cy - 0.5;
    add_centre(A, m3, swt1 * dx * dy, q);
  }
  if (nx >= 1) {
    m3 = (nx - 1) * yn + ny;
    if (m3 < nodenum && cx < 0.5) add_vy(A, m3, swt1 * (1 - cx - 0.5) * (1 - cy), q);
    m3 = (nx - 1) * yn + ny + 1;
    if (m3 < nodenum && cx < 0.5) add_vy(A, m3, swt1 * (1 - cx - 0.5) * cy, q);
  }
  if (ny >= 1) {
    m3 = nx * yn + ny - 1;
    if (m3 < nodenum && cy < 0.5) add_vx(A, m3, swt1 * (1 - cx) * (1 - cy - 0.5), q);
    m3 = (nx + 1) * yn + ny - 1;
    if (m3 < nodenum && cy < 0.5) add_vx(A, m3, swt1 * cx * (1 - cy - 0.5), q);
  }
}

/* the restricted 1-2|d| kernel of interpolationmod 2, interpolation.c:539-628 */
static void scatter_mode2(double **A, long yn, long nx, long ny, double swt1,
                          double cx, double cy, const mk_payload *q) {
  long m3 = nx * yn + ny;
  if (cx < 0.5 && cy < 0.5) add_basic(A, m3, swt1 * (1.0 - 2.0 * cx) * (1.0 - 2.0 * cy), q);
  if (cx < 0.5) add_vx(A, m3, swt1 * (1.0 - cx) * (1.0 - AB(cy - 0.5)), q);
  if (cy < 0.5) add_vy(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * (1.0 - cy), q);
  m3 = nx * yn + ny + 1;
  if (cx < 0.5 && cy > 0.5) add_basic(A, m3, swt1 * (1.0 - 2.0 * cx) * (2.0 * cy - 1.0), q);
  if (cy > 0.5) add_vy(A, m3, swt1 * (1.0 - AB(cx - 0.5)) * cy, q);
  m3 = (nx + 1) * yn + ny;
  if (cx > 0.5 && cy < 0.5) add_basic(A, m3, swt1 * (2.0 * cx - 1.0) * (1.0 - 2.0 * cy), q);
  if (cx > 0.5) add_vx(A, m3, swt1 * cx * (1.0 - AB(cy - 0.5)), q);
  m3 = (nx + 1) * yn + ny + 1;
  if (cx > 0.5 && cy > 0.5) add_basic(A, m3, swt1 * (2.0 * cx - 1.0) * (2.0 * cy - 1.0), q);
  add_centre(A, m3, swt1 * (1.0 - 2.0 * AB(cx - 0.5)) * (1.0 - 2.0 * AB(cy - 0.5)), q);
}

/* ------------------------------------------------ boundary-condition solve
 * vxvy_boundarycorrection / P_boundarycorrection
 * (momentum_continuity_addmatrix_checkerror.c:1002-1184) and tkrecalc
 * (temperature_iterate.c:828-891) solve, with the frontal Gauss routine
 * gausmat3, a system whose rows are either x_r = value_r or a boundary
 * equation x_r = c + sum_k c_k x_ref(k).  The restatement evaluates the same
 * linear solution by substitution: each row is resolved after the rows it
 * references, references accumulated in increasing row order (the order in
 * which the elimination and back substitution fold them in).  Rows that the
 * reference never adds to the matrix solve to 0. */
typedef struct bc_sys {
  long nrow;
  const signed char *present; /* row added to the matrix */
  const double *value;        /* identity-row value                         */
  const long *bond;           /* bond index per row (0: identity)           */
  long (*ref)(long bondn_entry, long nodenum, long row); /* bondn -> row */
  long nodenum;
  const long *bondn;
  const double *bondv;
  double *x;
  signed char *state; /* 0 todo, 1 in progress, 2 done */
  int err;
} bc_sys;

static double bc_eval(bc_sys *S, long r) {
  if (r < 0 || r >= S->nrow || !S->present[r]) return 0.0;
  if (S->state[r] == 2) return S->x[r];
  if (S->state[r] == 1) { S->err = 1; return 0.0; }
  S->state[r] = 1;
  long b = S->bond[r];
  double v;
  if (!b) {
    v = S->value[r];
  } else {
    long rr[3];
    double cc[3];
    int k = 0;
    for (int n1 = 0; n1 < 3; n1++) {
      long bn = S->bondn[b * 3 + n1];
      if (bn) { rr[k] = S->ref(bn, S->nodenum, r); cc[k] = S->bondv[b * 4 + n1 + 1]; k++; }
    }
    for (int i = 1; i < k; i++) /* increasing row order */
      for (int j = i; j > 0 && rr[j - 1] > rr[j]; j--) {
        long t = rr[j]; rr[j] = rr[j - 1]; rr[j - 1] = t;
        double u = cc[j]; cc[j] = cc[j - 1]; cc[j - 1] = u;
      }
    v = S->bondv[b * 4 + 0];
    for (int i = 0; i < k; i++) v = v - bc_eval(S, rr[i]) * (-cc[i]);
  }
  S->x[r] = v;
  S->state[r] = 2;
  return v;
}

/* parameter number -> row, as the corrections decode bondn[] */
static long ref_vxvy(long bn, long nodenum, long row) {
  if (row < nodenum) return ((bn - 1) - 1) / 3;      /* vx rows */
  return ((bn - 1) - 2) / 3 + nodenum;               /* vy rows */
}
static long ref_p(long bn, long nodenum, long row) { (void)nodenum; (void)row; return (bn - 1) / 3; }
static long ref_t(long bn, long nodenum, long row) { (void)row; return bn - 1 - nodenum * 3; }

static int bc_solve(bc_sys *S) {
  S->state = (signed char *)calloc(S->nrow, 1);
  for (long r = 0; r < S->nrow; r++) bc_eval(S, r);
  free(S->state);
  return S->err;
}

static int bc_corrections(v2c_oracle_state *s) {
  if (!s->bondm) return 0;
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  int err = 0;
  /* velocity rows: vx block [0,nn), vy block [nn,2nn) */
  {
    long nrow = 2 * nn;
    signed char *present = (signed char *)calloc(nrow, 1);
    double *value = (double *)calloc(nrow, sizeof(double));
    long *bond = (long *)calloc(nrow, sizeof(long));
    double *x = (double *)calloc(nrow, sizeof(double));
    for (long m1 = 0; m1 < xn; m1++)
      for (long m2 = 0; m2 < yn; m2++) {
        long m3 = m1 * yn + m2;
        if (m2 < yn - 1) {
          present[m3] = 1;
          value[m3] = s->N[V2C_NF_MVX][m3];
          bond[m3] = s->bondm[m3 * 3 + 1];
        }
        if (m1 < xn - 1) {
          present[nn + m3] = 1;
          value[nn + m3] = s->N[V2C_NF_MVY][m3];
          bond[nn + m3] = s->bondm[m3 * 3 + 2];
        }
      }
    bc_sys S = {nrow, present, value, bond, ref_vxvy, nn, s->bondn, s->bondv, x, NULL, 0};
    err |= bc_solve(&S);
    for (long m1 = 0; m1 < xn; m1++)
      for (long m2 = 0; m2 < yn; m2++) {
        long m3 = m1 * yn + m2;
        s->N[V2C_NF_MVX][m3] = (m2 < yn - 1) ? x[m3] : 0.0;
        s->N[V2C_NF_MVY][m3] = (m1 < xn - 1) ? x[nn + m3] : 0.0;
      }
    free(present); free(value); free(bond); free(x);
  }
  /* pressure rows */
  {
    signed char *present = (signed char *)calloc(nn, 1);
    double *value = (double *)calloc(nn, sizeof(double));
    long *bond = (long *)calloc(nn, sizeof(long));
    double *x = (double *)calloc(nn, sizeof(double));
    for (long m1 = 1; m1 < xn; m1++)
      for (long m2 = 1; m2 < yn; m2++) {
        long m3 = m1 * yn + m2;
        present[m3] = 1;
        value[m3] = s->N[V2C_NF_SPPE][m3];
        bond[m3] = (p->compressiblemode == 1) ? 0 : s->bondm[m3 * 3];
      }
    bc_sys S = {nn, present, value, bond, ref_p, nn, s->bondn, s->bondv, x, NULL, 0};
    err |= bc_solve(&S);
    for (long m3 = 0; m3 < nn; m3++) s->N[V2C_NF_SPPE][m3] = x[m3];
    free(present); free(value); free(bond); free(x);
  }
  if (p->tempmod) {
    signed char *present = (signed char *)malloc(nn);
    memset(present, 1, nn);
    double *x = (double *)calloc(nn, sizeof(double));
    long *bond = (long *)calloc(nn, sizeof(long));
    for (long m3 = 0; m3 < nn; m3++) bond[m3] = s->bondm[3 * nn + m3];
    bc_sys S = {nn, present, s->N[V2C_NF_TK], bond, ref_t, nn, s->bondn, s->bondv, x, NULL, 0};
    err |= bc_solve(&S);
    memcpy(s->N[V2C_NF_TK], x, nn * sizeof(double));
    free(present); free(x); free(bond);
  }
  return err ? V2C_ERR_UNSUPPORTED : 0;
}

/* ============================================================ marker2nodes
 * interpolation.c:55-926 */
/* recalc_marker_properties.c:1-83 for every marker strictly inside the
 * model (interpolation.c:219-240): the ductile viscosity, the thermal
 * conductivity and the pressure in bar each marker is evaluated at, in
 * marker order; markers outside read 0.  The marker state is not changed
 * (the friction update of calc_frictionpara is left out). */
int v2c_oracle_marker_properties(const v2c_oracle_state *s, double *mnu, double *mkt,
                                 double *mpb_out) {
  const v2c_params *p = &s->p;
  double *const *M = s->M;
  for (long mm1 = 0; mm1 < s->n; mm1++) {
    double x = M[V2C_MF_X][mm1], y = M[V2C_MF_Y][mm1];
    double nu = 0, kt = 0, mpb = 0;
    if (x > 0 && y > 0 && x < p->xsize && y < p->ysize) {
      int mm2 = s->t[mm1];
      double mtk = M[V2C_MF_K][mm1];
      mpb = 1e-5 * interp_pressure(s, x, y);
      kt = RT(s, V2C_RT_KT, mm2);
      kt = (kt + RT(s, V2C_RT_KF, mm2) / (mtk + 77.0)) * exp(RT(s, V2C_RT_KP, mm2) * mpb);
      if (kt < 0)
        kt = -kt / (1.0 + RT(s, V2C_RT_KF, mm2) * (mtk - RT(s, V2C_RT_KP, mm2)) /
                              RT(s, V2C_RT_KP, mm2));
      nu = v2c_oracle_ductilevisc(s, mm2, M[V2C_MF_XY][mm1], M[V2C_MF_XX][mm1],
                                  M[V2C_MF_EXY][mm1], M[V2C_MF_EXX][mm1], mtk, mpb);
    }
    if (mnu) mnu[mm1] = nu;
    if (mkt) mkt[mm1] = kt;
    if (mpb_out) mpb_out[mm1] = mpb;
  }
  return V2C_OK;
}

int v2c_oracle_marker2nodes(v2c_oracle_state *s) {
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  double **N = s->N, **M = s->M;
  /* I) arrays the reference zeroes first (:58-153) */
  static const int zero_list[] = {
      V2C_NF_BM, V2C_NF_RO, V2C_NF_ET, V2C_NF_NU, V2C_NF_ND, V2C_NF_WTPHISUM,
      V2C_NF_WTSXXSUM, V2C_NF_WTVXSUM, V2C_NF_WTVYSUM, V2C_NF_PHISUM,
      V2C_NF_SXYSUM, V2C_NF_EXYSUM, V2C_NF_ESUM, V2C_NF_SXXSUM, V2C_NF_EXXSUM,
      V2C_NF_VXSUM, V2C_NF_VYSUM, V2C_NF_PSUM, V2C_NF_GG, V2C_NF_GD,
      V2C_NF_SPPE, V2C_NF_PHIS, V2C_NF_PHIN, V2C_NF_SXYEN, V2C_NF_SXXEN,
      V2C_NF_EXYEN, V2C_NF_EXXEN, V2C_NF_SPPEN, V2C_NF_MUS_S, V2C_NF_AS,
      V2C_NF_BS, V2C_NF_LS, V2C_NF_V0S, V2C_NF_SXXE, V2C_NF_SXYE, V2C_NF_EXXE,
      V2C_NF_EXYE, V2C_NF_STICKY01, V2C_NF_COHESION, V2C_NF_DRO, V2C_NF_DRP,
      V2C_NF_CP, V2C_NF_KT, V2C_NF_HT, V2C_NF_TK, V2C_NF_MRX, V2C_NF_MRY,
      V2C_NF_MVX, V2C_NF_MVY, V2C_NF_MRX0, V2C_NF_MRY0};
  for (size_t i = 0; i < sizeof(zero_list) / sizeof(zero_list[0]); i++)
    memset(N[zero_list[i]], 0, nn * sizeof(double));
  double *A[A_N];
  for (int i = 0; i < A_N; i++) A[i] = (double *)calloc(nn, sizeof(double));

  /* III) marker cycle (:215-630), sequential = the one-thread order */
  for (long mm1 = 0; mm1 < s->n; mm1++) {
    double x = M[V2C_MF_X][mm1], y = M[V2C_MF_Y][mm1];
    if (!(x > 0 && y > 0 && x < p->xsize && y < p->ysize)) continue;
    long nx = v2c_oracle_nxsearch(s->gx, xn, x);
    long ny = v2c_oracle_nxsearch(s->gy, yn, y);
    int mm2 = s->t[mm1];
    mk_payload q;
    q.mbm = 50e9;
    q.mgg = RT(s, V2C_RT_GG, mm2);
    q.mtk = M[V2C_MF_K][mm1];
    double mpb = 1e-5 * interp_pressure(s, x, y);
    /* recalc_marker_properties, recalc_marker_properties.c:1-83 */
    double maa;
    density(s, q.mtk, mpb, mm2, &q.mro, &q.mbb, &maa);
    double mkt = RT(s, V2C_RT_KT, mm2);
    mkt = (mkt + RT(s, V2C_RT_KF, mm2) / (q.mtk + 77.0)) * exp(RT(s, V2C_RT_KP, mm2) * mpb);
    if (mkt < 0)
      mkt = -mkt / (1.0 + RT(s, V2C_RT_KF, mm2) * (q.mtk - RT(s, V2C_RT_KP, mm2)) /
                              RT(s, V2C_RT_KP, mm2));
    q.mkt = mkt;
    q.mnu = v2c_oracle_ductilevisc(s, mm2, M[V2C_MF_XY][mm1], M[V2C_MF_XX][mm1],
                                   M[V2C_MF_EXY][mm1], M[V2C_MF_EXX][mm1], q.mtk, mpb);
    friction_marker(s, mm1, mm2);
    q.me = M[V2C_MF_E][mm1];
    mm2 = s->t[mm1];
    q.xy = M[V2C_MF_XY][mm1];
    q.exy = M[V2C_MF_EXY][mm1];
    q.coh = M[V2C_MF_C][mm1];
    q.phi = M[V2C_MF_PHI][mm1];
    q.ht = RT(s, V2C_RT_HT, mm2);
    q.cp = RT(s, V2C_RT_CP, mm2);
    q.xx = M[V2C_MF_XX][mm1];
    q.exx = M[V2C_MF_EXX][mm1];
    q.p = M[V2C_MF_P][mm1];
    q.vx = M[V2C_MF_VX][mm1];
    q.vy = M[V2C_MF_VY][mm1];
    double celdx = s->gx[nx + 1] - s->gx[nx];
    double celdy = s->gy[ny + 1] - s->gy[ny];
    double swt1 = 1.0 / celdx / celdy;
    celdx = (x - s->gx[nx]) / (s->gx[nx + 1] - s->gx[nx]);
    celdy = (y - s->gy[ny]) / (s->gy[ny + 1] - s->gy[ny]);
    if (p->interpolationmod == 1)
      scatter_mode1(A, nn, yn, nx, ny, swt1, celdx, celdy, &q);
    else if (p->interpolationmod == 2)
      scatter_mode2(A, yn, nx, ny, swt1, celdx, celdy, &q);
  }

  /* nodal normalisation and antidiffusion correction (:714-824) */
  int antid = (p->timesum > 0 && p->antidiffinter == 1);
  for (long m3 = 0; m3 < nn; m3++) {
    long m22 = m3 % yn, m11 = (m3 - m22) / yn;
    double ss = A[A_SUMSHEAR][m3];
    if (ss && m11 >= 1 && m22 >= 1 && m11 < xn - 1 && m22 < yn - 1) {
      N[V2C_NF_PHIN][m3] = A[A_PHI][m3] / ss;
      N[V2C_NF_SXYEN][m3] = A[A_SXYE][m3] / ss;
      N[V2C_NF_EXYEN][m3] = A[A_EXYE][m3] / ss;
      N[V2C_NF_PEN][m3] = A[A_PE][m3] / ss;
      if (antid) {
        N[V2C_NF_PHIS][m3] = N[V2C_NF_PHIS_IT][m3] + (N[V2C_NF_PHIN][m3] - N[V2C_NF_PHIE][m3]);
        N[V2C_NF_SXYE][m3] = N[V2C_NF_SXY][m3] + (N[V2C_NF_SXYEN][m3] - N[V2C_NF_SXYEE][m3]);
        N[V2C_NF_EXYE][m3] = N[V2C_NF_EXY][m3] + (N[V2C_NF_EXYEN][m3] - N[V2C_NF_EXYEE][m3]);
        N[V2C_NF_PE][m3] = N[V2C_NF_PES][m3] + (N[V2C_NF_PEN][m3] - N[V2C_NF_PEE][m3]);
      } else {
        N[V2C_NF_PHIS][m3] = N[V2C_NF_PHIN][m3];
        N[V2C_NF_SXYE][m3] = N[V2C_NF_SXYEN][m3];
        N[V2C_NF_EXYE][m3] = N[V2C_NF_EXYEN][m3];
        N[V2C_NF_PE][m3] = N[V2C_NF_PEN][m3];
      }
      if (N[V2C_NF_PE][m3] < 0) N[V2C_NF_PE][m3] = 0;
      friction_node(s, s->gx[m11], s->gy[m22], m3);
      N[V2C_NF_COHESION][m3] = A[A_COH][m3] / ss;
      N[V2C_NF_NU_M2C][m3] = A[A_NU][m3] / ss;
      N[V2C_NF_GG][m3] = N[V2C_NF_NU_M2C][m3] / (A[A_GG][m3] / ss);
    }
    double s1 = A[A_SOL1C][m3];
    if (s1 && m11 >= 1 && m22 >= 1) {
      N[V2C_NF_SXXEN][m3] = A[A_SXXE][m3] / s1;
      N[V2C_NF_SPPEN][m3] = A[A_SPPE][m3] / s1;
      N[V2C_NF_EXXEN][m3] = A[A_EXXE][m3] / s1;
      if (antid) {
        N[V2C_NF_SXXE][m3] = N[V2C_NF_SXX][m3] + (N[V2C_NF_SXXEN][m3] - N[V2C_NF_SXXEE][m3]);
        N[V2C_NF_SPPE][m3] = N[V2C_NF_PR][m3] + (N[V2C_NF_SPPEN][m3] - N[V2C_NF_SPPEE][m3]);
        N[V2C_NF_EXXE][m3] = N[V2C_NF_EXX][m3] + (N[V2C_NF_EXXEN][m3] - N[V2C_NF_EXXEE][m3]);
      } else {
        N[V2C_NF_SXXE][m3] = N[V2C_NF_SXXEN][m3];
        N[V2C_NF_SPPE][m3] = N[V2C_NF_SPPEN][m3];
        N[V2C_NF_EXXE][m3] = N[V2C_NF_EXXEN][m3];
      }
      if (p->timesum == 0 && p->reloadfromDP == 0 && p->compressiblemode == 1)
        N[V2C_NF_SPPE][m3] = p->nstress;
      N[V2C_NF_ND_M2C][m3] = A[A_ND][m3] / s1;
      N[V2C_NF_GD][m3] = N[V2C_NF_ND_M2C][m3] / (A[A_GD][m3] / s1);
      N[V2C_NF_BM][m3] = A[A_BM][m3] / s1;
      N[V2C_NF_DRO][m3] = 0.0 / s1;
      N[V2C_NF_DRP][m3] = 0.0 / s1;
    }
    if (A[A_SOL0V][m3]) {
      N[V2C_NF_MVXN][m3] = A[A_MVX][m3] / A[A_MRX][m3];
      if (antid)
        N[V2C_NF_MVX][m3] = N[V2C_NF_VX][m3] + (N[V2C_NF_MVXN][m3] - N[V2C_NF_MVXE][m3]);
      else
        N[V2C_NF_MVX][m3] = N[V2C_NF_MVXN][m3];
      N[V2C_NF_MRX][m3] = A[A_MRX][m3] / A[A_SOL0V][m3];
    }
    if (A[A_SOL1V][m3]) {
      N[V2C_NF_MVYN][m3] = A[A_MVY][m3] / A[A_MRY][m3];
      if (antid)
        N[V2C_NF_MVY][m3] = N[V2C_NF_VY][m3] + (N[V2C_NF_MVYN][m3] - N[V2C_NF_MVYE][m3]);
      else
        N[V2C_NF_MVY][m3] = N[V2C_NF_MVYN][m3];
      N[V2C_NF_MRY][m3] = A[A_MRY][m3] / A[A_SOL1V][m3];
    }
    double s0 = A[A_SOL0][m3];
    if (s0) {
      N[V2C_NF_RO][m3] = A[A_RO][m3] / s0;
      N[V2C_NF_ET][m3] = A[A_ET][m3] / s0;
      N[V2C_NF_HT][m3] = A[A_HT][m3] / s0;
      N[V2C_NF_KT][m3] = A[A_KT][m3] / s0;
      N[V2C_NF_CP][m3] = A[A_CP][m3] / s0;
      N[V2C_NF_TK][m3] = A[A_TK][m3] / s0;
    }
  }
  for (int i = 0; i < A_N; i++) free(A[i]);

  /* ghost copy of the state when it diffuses (:827-859) */
  if (p->Dphis > 0) {
    double *phis = N[V2C_NF_PHIS];
    for (long m3 = 0; m3 < nn; m3++) {
      long m22 = m3 % yn, m11 = (m3 - m22) / yn;
      if (m11 == 0 && m22 >= 1 && m22 <= yn - 2)
        phis[m3] = phis[m3 + yn];
      else if (m11 == xn - 1 && m22 >= 1 && m22 <= yn - 2)
        phis[m3] = phis[m3 - yn];
      else if (m22 == 0 && m11 >= 1 && m11 <= xn - 2)
        phis[m3] = phis[m3 + 1];
      else if (m22 == yn - 1 && m11 > 0 && m11 <= xn - 2)
        phis[m3] = phis[m3 - 1];
      else if ((m11 == 0 && m22 == 0) || (m11 == 0 && m22 == yn - 1) ||
               (m11 == xn - 1 && m22 == 0) || (m11 == xn - 1 && m22 == yn - 1))
        phis[m3] = 0;
    }
  }

  /* sticky-air flags, serial over all markers in index order (:866-916).
   * The reference's index can reach nodenum for the last cell; that write
   * falls outside the array and is skipped here. */
  for (long mm1 = 0; mm1 < s->n; mm1++) {
    int t = s->t[mm1];
    if (t != 1 && t != 2) continue;
    double x = M[V2C_MF_X][mm1], y = M[V2C_MF_Y][mm1];
    long nx = v2c_oracle_nxsearch(s->gx, xn, x), ny = v2c_oracle_nxsearch(s->gy, yn, y);
    long m3 = nx * yn + ny + 1;
    double cx = (x - s->gx[nx]) / (s->gx[nx + 1] - s->gx[nx]);
    double cy = (y - s->gy[ny]) / (s->gy[ny + 1] - s->gy[ny]);
    long k = -1;
    if (cx < 0.5 && cy < 0.5) k = m3;
    else if (cx < 0.5 && cy > 0.5) k = m3 + 1;
    else if (cx > 0.5 && cy < 0.5) k = m3 + yn;
    else if (cx > 0.5 && cy > 0.5) k = m3 + yn + 1;
    if (k >= 0 && k < nn) N[V2C_NF_STICKY01][k] = (double)t;
  }
  return bc_corrections(s);
}

/* interpolate_center2basic_old, interpolation.c:1575-1598 */
int v2c_oracle_center2basic_old(v2c_oracle_state *s) {
  long xn = s->p.xnumx, yn = s->p.ynumy, nn = nnodes(s);
  const double *exxe = s->N[V2C_NF_EXXE], *sxxe = s->N[V2C_NF_SXXE], *sppe = s->N[V2C_NF_SPPE];
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1) {
      s->N[V2C_NF_EXXES][m3] = 0.25 * (exxe[m3] + exxe[m3 + 1] + exxe[m3 + yn] + exxe[m3 + yn + 1]);
      s->N[V2C_NF_SXXES][m3] = 0.25 * (sxxe[m3] + sxxe[m3 + 1] + sxxe[m3 + yn] + sxxe[m3 + yn + 1]);
      s->N[V2C_NF_SPPES][m3] = 0.25 * (sppe[m3] + sppe[m3 + 1] + sppe[m3 + yn] + sppe[m3 + yn + 1]);
    }
  }
  return 0;
}

/* interpolate_center2basic, interpolation.c:1600-1637: strain rate, stress,
 * pressure, plastic and elastic strain rate averaged from the four pressure
 * nodes around each interior basic node */
int v2c_oracle_center2basic(v2c_oracle_state *s, double dt) {
  long xn = s->p.xnumx, yn = s->p.ynumy, nn = nnodes(s);
  const double *exx = s->N[V2C_NF_EXX], *sxx = s->N[V2C_NF_SXX], *sxxe = s->N[V2C_NF_SXXE];
  const double *gd = s->N[V2C_NF_GD], *nd = s->N[V2C_NF_ND_M2C], *pr = s->N[V2C_NF_PR];
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (!(m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1)) continue;
    const long k[4] = {m3, m3 + 1, m3 + yn, m3 + yn + 1};
    double epl[4], eel[4];
    for (int q = 0; q < 4; q++) {
      const long i = k[q];
      epl[q] = exx[i] - (sxx[i] - sxxe[i]) / (2 * gd[i] * dt) - sxx[i] / (2 * nd[i]);
      eel[q] = 2 * gd[i] * dt * exx[i] + sxxe[i];
    }
    s->N[V2C_NF_EXXS][m3] = 0.25 * (exx[k[0]] + exx[k[1]] + exx[k[2]] + exx[k[3]]);
    s->N[V2C_NF_EXXPL][m3] = 0.25 * (epl[0] + epl[1] + epl[2] + epl[3]);
    s->N[V2C_NF_SXXS][m3] = 0.25 * (sxx[k[0]] + sxx[k[1]] + sxx[k[2]] + sxx[k[3]]);
    s->N[V2C_NF_PRS][m3] = 0.25 * (pr[k[0]] + pr[k[1]] + pr[k[2]] + pr[k[3]]);
    s->N[V2C_NF_EXXEL][m3] = 0.25 * (eel[0] + eel[1] + eel[2] + eel[3]);
  }
  return 0;
}

/* interpolate_basic2center, interpolation.c:1639-1685: viscosity of each
 * pressure node as the bilinear harmonic mean of the basic-node viscosity
 * nu around the cell centre (weights clamped to the grid) */
int v2c_oracle_basic2center(v2c_oracle_state *s) {
  long xn = s->p.xnumx, yn = s->p.ynumy, nn = nnodes(s);
  const double *gx = s->gx, *gy = s->gy, *nu = s->N[V2C_NF_NU];
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (!(m1 >= 1 && m2 >= 1)) continue;
    double x = (gx[m1] + gx[m1 - 1]) / 2, y = (gy[m2] + gy[m2 - 1]) / 2;
    long m10 = v2c_oracle_nxsearch(gx, xn, x), m20 = v2c_oracle_nxsearch(gy, yn, y);
    if (m10 < 1) m10 = 1;
    if (m10 > xn - 3) m10 = xn - 3;
    if (m20 < 1) m20 = 1;
    if (m20 > yn - 3) m20 = yn - 3;
    double e = (x - gx[m10]) / (gx[m10 + 1] - gx[m10]);
    double n = (y - gy[m20]) / (gy[m20 + 1] - gy[m20]);
    if (e < 0) e = 0.0;
    if (n < 0) n = 0.0;
    if (e > 1) e = 1.0;
    if (n > 1) n = 1.0;
    double dm0 = (1.0 - e) * (1.0 - n), dm1 = (1.0 - e) * n, dm2 = e * (1.0 - n), dm3 = e * n;
    long m4 = m10 * yn + m20;
    s->N[V2C_NF_ND][m3] = 1.0 / (dm0 * 1.0 / nu[m4] + dm1 * 1.0 / nu[m4 + 1] +
                                 dm2 * 1.0 / nu[m4 + yn] + dm3 * 1.0 / nu[m4 + yn + 1]);
  }
  return 0;
}

/* nueffcalc, momentum_continuity_addmatrix_checkerror.c:380-393: the
 * visco-elastic factor Z and the computational viscosity Z*nvp (lower limit
 * nubeg) */
static double nueff_of(const v2c_params *p, double nvp, double ggeff, double dt, double *Z) {
  *Z = ggeff * dt / (ggeff * dt + nvp);
  double nueff = *Z * nvp;
  if (nueff < p->nubeg) nueff = p->nubeg;
  return nueff;
}

/* recompute_stress_strainrate, momentum_continuity_iterate.c:228-271 with
 * sxxcalc and sxycalc (momentum_continuity_addmatrix_checkerror.c:446-481,
 * 528-572): strain rates from the node velocities, visco-elastic stresses
 * from the node viscosities and the previous elastic stresses */
int v2c_oracle_recompute_stress(v2c_oracle_state *s, double dt) {
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  double **N = s->N;
  const double *gx = s->gx, *gy = s->gy, *vx = N[V2C_NF_VX], *vy = N[V2C_NF_VY];
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (!(m1 < xn && m2 < yn && m1 >= 1 && m2 >= 1)) continue;
    long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
    double Z, nueff;
    nueff = nueff_of(p, N[V2C_NF_ND][v3], N[V2C_NF_GD][v3], dt, &Z);
    double edotxx = 0.5 * ((vx[v2] - vx[v0]) / (gx[m1] - gx[m1 - 1]) -
                           (vy[v1] - vy[v0]) / (gy[m2] - gy[m2 - 1]));
    N[V2C_NF_EXX][m3] = edotxx;
    N[V2C_NF_SXX][m3] = 2.0 * nueff * edotxx + N[V2C_NF_SXXE][v3] * (1.0 - Z);
    if (m1 < xn - 1 && m2 < yn - 1) {
      nueff = nueff_of(p, N[V2C_NF_NU][v3], N[V2C_NF_GG][v3], dt, &Z);
      double exy1 = (vx[v3] - vx[v2]) / (gy[m2 + 1] - gy[m2 - 1]);
      double exy2 = (vy[v3] - vy[v1]) / (gx[m1 + 1] - gx[m1 - 1]);
      double edotxy = exy1 + exy2;
      N[V2C_NF_EXY][m3] = edotxy;
      N[V2C_NF_ESP][m3] = exy1 - exy2;
      N[V2C_NF_SXY][m3] = 2.0 * nueff * edotxy + N[V2C_NF_SXYE][v3] * (1.0 - Z);
    }
  }
  return 0;
}

/* copyarrays, momentum_continuity_iterate.c:265-281: the solved slip rate
 * and state rate become the step's final ones (deltaVs, an output-only
 * diagnostic, is not kept) */
int v2c_oracle_copyarrays(v2c_oracle_state *s) {
  long xn = s->p.xnumx, yn = s->p.ynumy, nn = nnodes(s);
  double **N = s->N;
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1) {
      N[V2C_NF_SLIPRS][m3] = N[V2C_NF_RK_SLIPRS_FINAL][m3] = N[V2C_NF_RK_SLIPRS_SOLVED][m3];
      N[V2C_NF_RK_PHIDTS_FINAL][m3] = N[V2C_NF_RK_PHIDTS_SOLVED][m3];
    }
  }
  return 0;
}

/* interpolate_temperature, interpolation.c:1492-1533: solved (TK) and old
 * (TK2) node temperature at a point clamped into the model */
static void temperature_at(const v2c_oracle_state *s, double x, double y, double *TK,
                           double *TK2) {
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy;
  if (x < 0) x = 0; else if (x > p->xsize) x = p->xsize;
  if (y < 0) y = 0; else if (y > p->ysize) y = p->ysize;
  long m10 = v2c_oracle_nxsearch(s->gx, xn, x), m20 = v2c_oracle_nxsearch(s->gy, yn, y);
  if (m10 < 0) m10 = 0;
  if (m10 > xn - 2) m10 = xn - 2;
  if (m20 < 0) m20 = 0;
  if (m20 > yn - 2) m20 = yn - 2;
  double e = (x - s->gx[m10]) / (s->gx[m10 + 1] - s->gx[m10]);
  double n = (y - s->gy[m20]) / (s->gy[m20 + 1] - s->gy[m20]);
  double dm0 = (1.0 - e) * (1.0 - n), dm1 = (1.0 - e) * n, dm2 = e * (1.0 - n), dm3 = e * n;
  long m3 = m10 * yn + m20;
  const double *tk = s->N[V2C_NF_TK], *tk2 = s->N[V2C_NF_TK2];
  *TK = dm0 * tk[m3] + dm1 * tk[m3 + 1] + dm2 * tk[m3 + yn] + dm3 * tk[m3 + yn + 1];
  *TK2 = dm0 * tk2[m3] + dm1 * tk2[m3 + 1] + dm2 * tk2[m3 + yn] + dm3 * tk2[m3 + yn + 1];
}

/* the marker part of solve_temperature, temperature_iterate.c:181-412:
 * fluid markers take the solved temperature; rock markers the subgrid
 * diffusion towards the old temperature, the solution's change, and the
 * antidiffusion of the node-averaged diffusion change, summed at each
 * marker's upper-left node only (the reference's loop bounds) */
int v2c_oracle_marker_temperature(v2c_oracle_state *s, double heatdif) {
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s), n = s->n;
  const double *gx = s->gx, *gy = s->gy, *kt = s->N[V2C_NF_KT], *cp = s->N[V2C_NF_CP];
  const double *ro = s->N[V2C_NF_RO];
  double *mx = s->M[V2C_MF_X], *my = s->M[V2C_MF_Y], *mk = s->M[V2C_MF_K];
  const double dt = p->timestep;
  double *tol0 = calloc(nn, sizeof(double)), *tol1 = calloc(nn, sizeof(double));
  (void)xn;
#define INSIDE(m) (mx[m] > 0 && my[m] > 0 && mx[m] < p->xsize && my[m] < p->ysize)
  for (long m3 = 0; m3 < n; m3++) {
    if (INSIDE(m3) && s->t[m3] >= 50 && s->t[m3] < 100) {
      double TK, TK2;
      temperature_at(s, mx[m3], my[m3], &TK, &TK2);
      mk[m3] = TK;
    }
  }
  const long last = s->phantom ? n : n - 1;
  for (long m3 = 0; m3 <= last; m3++) {
    if (!(INSIDE(m3) && s->t[m3] < 50)) continue;
    long m10 = v2c_oracle_nxsearch(gx, p->xnumx, mx[m3]);
    long m20 = v2c_oracle_nxsearch(gy, p->ynumy, my[m3]);
    double TK, TK2;
    temperature_at(s, mx[m3], my[m3], &TK, &TK2);
    if (mk[m3] <= 0) {
      mk[m3] = TK2;
      if (mk[m3] < p->tdeep) mk[m3] = p->tdeep;
    }
    if (heatdif) {
      double dtk = TK2 - mk[m3];
      double celdx = gx[m10 + 1] - gx[m10], celdy = gy[m20 + 1] - gy[m20];
      double swt1 = 1.0 / celdx / celdy;
      double ex = (mx[m3] - gx[m10]) / (gx[m10 + 1] - gx[m10]);
      double ey = (my[m3] - gy[m20]) / (gy[m20 + 1] - gy[m20]);
      /* the reference's loop order: m1 outer, m2 inner */
      double w[4] = {(1.0 - ex) * (1.0 - ey), (1.0 - ex) * ey, ex * (1.0 - ey), ex * ey};
      long nd[4] = {m10 * yn + m20, m10 * yn + m20 + 1, (m10 + 1) * yn + m20,
                    (m10 + 1) * yn + m20 + 1};
      double mkt = 0, mrocp = 0;
      for (int q = 0; q < 4; q++) {
        mkt += kt[nd[q]] * w[q];
        mrocp += cp[nd[q]] * ro[nd[q]] * w[q];
      }
      double dtk1 = -heatdif * mkt / mrocp * 2.0 * (1.0 / celdx / celdx + 1.0 / celdy / celdy) * dt;
      if (dtk1 < -150.0) dtk1 = -150.0;
      dtk1 = dtk * (1.0 - exp(dtk1));
      mk[m3] += dtk1;
      double ival = (1.0 - ex) * (1.0 - ey) * swt1;
      tol0[nd[0]] += ival;
      tol1[nd[0]] += dtk1 * ival;
    }
    mk[m3] += (TK - TK2);
  }
  if (heatdif) {
    for (long m = 0; m < nn; m++)
      if (tol0[m]) tol1[m] /= tol0[m];
    for (long m3 = 0; m3 <= last; m3++) {
      if (!(INSIDE(m3) && s->t[m3] < 50)) continue;
      long m10 = v2c_oracle_nxsearch(gx, p->xnumx, mx[m3]);
      long m20 = v2c_oracle_nxsearch(gy, p->ynumy, my[m3]);
      double ex = (mx[m3] - gx[m10]) / (gx[m10 + 1] - gx[m10]);
      double ey = (my[m3] - gy[m20]) / (gy[m20 + 1] - gy[m20]);
      long m4 = m10 * yn + m20;
      if (tol1[m4]) mk[m3] -= (tol1[m4] * ((1.0 - ex) * (1.0 - ey)));
    }
  }
#undef INSIDE
  free(tol0);
  free(tol1);
  return 0;
}

/* calc_vpvisc, calc_RSF.c:33-169.  The state rate dphidt it selects per
 * rkmod is never used by the reference (it is only printed on error), nor
 * are the RK_sliprs/RK_phidts histories rkmod 3 stores (calc_RSF.c:72-76,
 * read only into that dphidt at :84-86): the slip rate V is what each
 * pass takes. */
static double vpvisc(v2c_oracle_state *s, int rk, double dt, long m3, double nP,
                     double W, int *err) {
  const v2c_params *p = &s->p;
  double **N = s->N;
  double V = 0, dphidt = 0, newstate = 0, syield = 0, rad = 0, vp = 0;
  if (rk == 0 && p->timesum > 0) {
    V = N[V2C_NF_RK_SLIPRS_FINAL][m3];
    if (p->RSFmode == 1) dphidt = N[V2C_NF_RK_PHIDTS_FINAL][m3];
  } else if (rk == 0 && p->timesum == 0) {
    if (p->RSFmode == 0) V = 0;
    else if (p->RSFmode == 1) {
      V = N[V2C_NF_RK_SLIPRS_FINAL][m3];
      dphidt = N[V2C_NF_RK_PHIDTS_FINAL][m3];
    }
  }
  if ((p->rkmod == 0 && rk > 0) || (rk > 0 && rk < 3)) {
    if (p->rkmod == 1) {
      V = N[V2C_NF_RK_SLIPRS_SOLVED][m3];
      if (p->RSFmode == 1) dphidt = 0.5 * (N[V2C_NF_RK_PHIDTS_FINAL][m3] + N[V2C_NF_RK_PHIDTS_SOLVED][m3]);
    } else {
      V = N[V2C_NF_RK_SLIPRS_SOLVED][m3];
      if (p->RSFmode == 1) dphidt = N[V2C_NF_RK_PHIDTS_SOLVED][m3];
    }
  }
  if (rk == 3 && p->rkmod == 3) {
    V = N[V2C_NF_RK_SLIPRS_SOLVED][m3];
    if (p->RSFmode == 1) dphidt = N[V2C_NF_RK_PHIDTS_SOLVED][m3];  /* (the reference's 1/6 average) */
  }
  (void)dphidt;
  N[V2C_NF_PES][m3] = N[V2C_NF_PE][m3] + V / W * dt;
  if (p->RSFmode == 1) {
    double L = N[V2C_NF_LS][m3], V0 = N[V2C_NF_V0S][m3], ph = N[V2C_NF_PHIS][m3];
    if (V * dt / L <= 1e-6)
      newstate = log(exp(ph) * (1 - V * dt / L) + V0 * dt / L);
    else
      newstate = log(V0 / V + (exp(ph) - V0 / V) * exp(-V * dt / L));
    rad = (p->inertyn == 0) ? 4.3303e+06 * V : 0.0;
    double a = N[V2C_NF_AS][m3], b = N[V2C_NF_BS][m3], mu = N[V2C_NF_MUS_S][m3];
    if (p->power_law_RSF > 0) {
      double sy0 = nP * mu;
      syield = sy0 * pow(V / V0, a / mu) * exp((newstate * b) / mu) + rad;
    } else {
      syield = nP * a * asinh(V / (2 * V0) * exp((mu + newstate * b) / a)) + rad;
    }
  } else {
    syield = nP * N[V2C_NF_MUS_S][m3] + N[V2C_NF_COHESION][m3];
  }
  double nu = N[V2C_NF_NU_M2C][m3];
  if (p->RSFmode == 1)
    vp = (syield > 0) ? nu * syield / (2 * nu * V / W + syield) : nu;
  else
    vp = nu * syield / (2 * nu * V / W + syield);
  N[V2C_NF_PHIS_IT][m3] = newstate;
  N[V2C_NF_SYIELDS][m3] = syield;
  N[V2C_NF_NUVP_IT][m3] = vp;
  N[V2C_NF_SLIPRS][m3] = V;
  if ((p->timesum > 0 && (isnan(newstate) || isnan(syield) || isnan(vp) || vp == 0 || isnan(V))) ||
      V < 0 || syield < 0)
    *err = 1;
  return vp;
}

/* compute_before_solve, plastic.c:2-56 */
int v2c_oracle_compute_before_solve(v2c_oracle_state *s, double dt, int rk) {
  const v2c_params *p = &s->p;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  int err = 0;
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    double W = p->faultwidth;
    double nps = (p->pmode == 0 || p->timesum == 0) ? p->nstress : s->N[V2C_NF_SPPES][m3];
    if (m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1) {
      double sxxs = s->N[V2C_NF_SXXS][m3], sxy = s->N[V2C_NF_SXY][m3];
      double sigin = pow(sxxs * sxxs + sxy * sxy, 0.5);
      double nu;
      if (sigin > 0 || p->RSFmode == 0)
        nu = vpvisc(s, rk, dt, m3, nps, W, &err);
      else
        nu = s->N[V2C_NF_NU_M2C][m3];
      s->N[V2C_NF_NU][m3] = nu;
      if (isnan(nu) || nu <= 0) err = 1;
    }
  }
  return err ? V2C_ERR_NAN : 0;
}

/* compute_after_solve + calc_sliprate_after_solve, plastic.c:61-129 and
 * calc_RSF.c:172-221.  Returns the RMS misfit deltas. */
double v2c_oracle_compute_after_solve(v2c_oracle_state *s, double dt, int rk) {
  const v2c_params *p = &s->p;
  double **N = s->N;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  double deltas = 0.0;
  long count = 0;
  (void)rk;
  for (long m3 = 0; m3 < nn; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    double W = p->faultwidth;
    double nps = (p->pmode == 0 || p->timesum == 0) ? p->nstress : N[V2C_NF_SPPES][m3];
    if (!(m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1)) continue;
    double sxxs = N[V2C_NF_SXXS][m3], sxy = N[V2C_NF_SXY][m3];
    double sigin = pow(sxxs * sxxs + sxy * sxy, 0.5);
    double a = N[V2C_NF_AS][m3], b = N[V2C_NF_BS][m3], mu = N[V2C_NF_MUS_S][m3];
    double V0 = N[V2C_NF_V0S][m3], L = N[V2C_NF_LS][m3], ph = N[V2C_NF_PHIS_IT][m3];
    double EPXX = N[V2C_NF_EXXPL][m3], EXY = N[V2C_NF_EXY][m3];
    if (p->RSFmode == 1) {
      double V;
      if (sigin > 0) {
        if (p->power_law_RSF > 0) {
          double sy0 = nps * mu;
          V = V0 * pow(sigin / sy0, (mu / a)) * exp((-ph * b) / a);
        } else {
          V = 2 * V0 * sinh(sigin / (a * nps)) * exp(-(mu + b * ph) / a);
        }
        double EII = pow(EPXX * EPXX + EXY * EXY, 0.5);
        double Vslip = EII * W;
        V = (V <= Vslip) ? V : Vslip;
        if (V < 1e-40) V = 1e-40;
      } else {
        V = 0;
      }
      N[V2C_NF_RK_SLIPRS_SOLVED][m3] = V;
      N[V2C_NF_RK_PHIDTS_SOLVED][m3] = V0 / L * exp(-ph) - V / L;
    } else {
      double G = N[V2C_NF_GG][m3], NUVP = N[V2C_NF_NU][m3], NU = N[V2C_NF_NU_M2C][m3];
      double E2EL = sigin / (NUVP / (G * dt + NUVP));
      double A = N[V2C_NF_SYIELDS][m3] / E2EL;
      if (A < 1) {
        double nup = G * dt * A / (1.0 - A);
        N[V2C_NF_RK_SLIPRS_SOLVED][m3] = W * (sigin / 2.0 * (1.0 / (nup)-1.0 / NU));
      } else {
        N[V2C_NF_RK_SLIPRS_SOLVED][m3] = 0;
      }
    }
    if (N[V2C_NF_RK_SLIPRS_SOLVED][m3] > 0) {
      double d = N[V2C_NF_SYIELDS][m3] - sigin;
      N[V2C_NF_RK_DELTAS][m3] = d;
      deltas += pow(d, 2);
      count++;
    } else {
      N[V2C_NF_RK_DELTAS][m3] = 0;
    }
  }
  return count > 0 ? pow(deltas / count, 0.5) : 0.0;
}

/* =========================================================== nodes2markers
 * interpolation.c:929-1048 with interpolate_mechanical :1050-1490.  The
 * reference's marker loop runs one index past marknum (:937).  With the
 * marker arrays zero past the end, that extra marker sits at (0,0) with
 * type 0 and back-scatters into the sums of node 0 only (no normalised
 * output reads them).  s->phantom adds it, last, as the reference does. */
typedef struct {
  double EXY, EXYE, SXY, SXYE, PHIS, PHISE, SXX, SXXE, EXX, EXXE, PR, SPPE;
  double VX, MVX, VY, MVY, ESP, ES, ESE;
} mech;

static double bil(const double *f, long m3, long yn, double d0, double d1,
                  double d2, double d3) {
  return d0 * f[m3] + d1 * f[m3 + 1] + d2 * f[m3 + yn] + d3 * f[m3 + yn + 1];
}

static void interpolate_mechanical(v2c_oracle_state *s, double x, double y,
                                   mech *o, double MRO) {
  const v2c_params *p = &s->p;
  double **N = s->N;
  const double *gx = s->gx, *gy = s->gy;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  long m3, m10, m20;
  double e, n, dm0, dm1, dm2, dm3, swt, swt1, celdx, celdy, dx, dy;
  if (x < 0) x = 0; else if (x > p->xsize) x = p->xsize;
  if (y < 0) y = 0; else if (y > p->ysize) y = p->ysize;
  long nx = v2c_oracle_nxsearch(gx, xn, x), ny = v2c_oracle_nxsearch(gy, yn, y);
  int mode = p->interpolationmod, ad = (p->antidiffinter == 1);

  /* basic nodes (:1067-1092) */
  m10 = nx; m20 = ny;
  if (m10 < 1) m10 = 1;
  if (m10 > xn - 3) m10 = xn - 3;
  if (m20 < 1) m20 = 1;
  if (m20 > yn - 3) m20 = yn - 3;
  e = (x - gx[m10]) / (gx[m10 + 1] - gx[m10]);
  n = (y - gy[m20]) / (gy[m20 + 1] - gy[m20]);
  dm0 = (1.0 - e) * (1.0 - n); dm1 = (1.0 - e) * n; dm2 = e * (1.0 - n); dm3 = e * n;
  m3 = m10 * yn + m20;
  o->EXY = bil(N[V2C_NF_EXY], m3, yn, dm0, dm1, dm2, dm3);
  o->EXYE = bil(N[V2C_NF_EXYE], m3, yn, dm0, dm1, dm2, dm3);
  o->SXY = bil(N[V2C_NF_SXY], m3, yn, dm0, dm1, dm2, dm3);
  o->SXYE = bil(N[V2C_NF_SXYE], m3, yn, dm0, dm1, dm2, dm3);
  o->ES = bil(N[V2C_NF_PES], m3, yn, dm0, dm1, dm2, dm3);
  o->ESE = bil(N[V2C_NF_PE], m3, yn, dm0, dm1, dm2, dm3);
  o->ESP = bil(N[V2C_NF_ESP], m3, yn, dm0, dm1, dm2, dm3);
  o->PHISE = bil(N[V2C_NF_PHIS], m3, yn, dm0, dm1, dm2, dm3);
  o->PHIS = bil(N[V2C_NF_PHIS_IT], m3, yn, dm0, dm1, dm2, dm3);

  celdx = gx[nx + 1] - gx[nx];
  celdy = gy[ny + 1] - gy[ny];
  swt1 = 1.0 / celdx / celdy;
  celdx = (x - gx[nx]) / (gx[nx + 1] - gx[nx]);
  celdy = (y - gy[ny]) / (gy[ny + 1] - gy[ny]);
  if (ad) { /* back-scatter to basic nodes (:1094-1210) */
    double *PH = N[V2C_NF_PHISUM], *SY = N[V2C_NF_SXYSUM], *EY = N[V2C_NF_EXYSUM];
    double *ES = N[V2C_NF_ESUM], *WT = N[V2C_NF_WTPHISUM];
    long nodes[4] = {nx * yn + ny, nx * yn + ny + 1, (nx + 1) * yn + ny, (nx + 1) * yn + ny + 1};
    double w[4];
    int use[4];
    if (mode == 1) {
      w[0] = swt1 * (1.0 - celdx) * (1.0 - celdy); use[0] = 1;
      w[1] = swt1 * (1.0 - celdx) * celdy; use[1] = 1;
      w[2] = swt1 * celdx * (1.0 - celdy); use[2] = 1;
      w[3] = swt1 * celdx * celdy; use[3] = 1;
    } else {
      use[0] = celdx < 0.5 && celdy < 0.5; w[0] = swt1 * (1.0 - 2 * celdx) * (1.0 - 2 * celdy);
      use[1] = celdx < 0.5 && celdy > 0.5; w[1] = swt1 * (1.0 - 2.0 * celdx) * (2.0 * celdy - 1.0);
      use[2] = celdx > 0.5 && celdy < 0.5; w[2] = swt1 * (2.0 * celdx - 1.0) * (1.0 - 2.0 * celdy);
      use[3] = celdx > 0.5 && celdy > 0.5; w[3] = swt1 * (2.0 * celdx - 1.0) * (2.0 * celdy - 1.0);
    }
    if (mode == 1 || mode == 2)
      for (int k = 0; k < 4; k++) {
        if (!(nodes[k] < nn && use[k])) continue;
        swt = w[k];
        m3 = nodes[k];
        PH[m3] = PH[m3] + o->PHIS * swt;
        SY[m3] = SY[m3] + o->SXY * swt;
        EY[m3] = EY[m3] + o->EXY * swt;
        ES[m3] = ES[m3] + o->ES * swt;
        WT[m3] = WT[m3] + swt;
      }
  }

  /* pressure nodes (:1211-1239) */
  m10 = nx; m20 = ny;
  if (x > (gx[m10] + gx[m10 + 1]) / 2.0) m10 += 1;
  if (y > (gy[m20] + gy[m20 + 1]) / 2.0) m20 += 1;
  if (m10 > xn - 2) m10 = xn - 2;
  if (m20 > yn - 2) m20 = yn - 2;
  if (m10 < 1) m10 = 1;
  if (m20 < 1) m20 = 1;
  e = (x - (gx[m10 - 1] + gx[m10]) / 2.0) / ((gx[m10 + 1] - gx[m10 - 1]) / 2);
  n = (y - (gy[m20 - 1] + gy[m20]) / 2.0) / ((gy[m20 + 1] - gy[m20 - 1]) / 2);
  dm0 = (1.0 - e) * (1.0 - n); dm1 = (1.0 - e) * n; dm2 = e * (1.0 - n); dm3 = e * n;
  m3 = m10 * yn + m20;
  o->EXX = bil(N[V2C_NF_EXX], m3, yn, dm0, dm1, dm2, dm3);
  o->EXXE = bil(N[V2C_NF_EXXE], m3, yn, dm0, dm1, dm2, dm3);
  o->SXX = bil(N[V2C_NF_SXX], m3, yn, dm0, dm1, dm2, dm3);
  o->SXXE = bil(N[V2C_NF_SXXE], m3, yn, dm0, dm1, dm2, dm3);
  o->PR = bil(N[V2C_NF_PR], m3, yn, dm0, dm1, dm2, dm3);
  o->SPPE = bil(N[V2C_NF_SPPE], m3, yn, dm0, dm1, dm2, dm3);
  if (ad) { /* back-scatter to pressure nodes (:1247-1375) */
    double *PS = N[V2C_NF_PSUM], *SX = N[V2C_NF_SXXSUM], *EX = N[V2C_NF_EXXSUM];
    double *WT = N[V2C_NF_WTSXXSUM];
    long nd[9];
    double w[9];
    int use[9], k = 0;
    if (mode == 1) {
      nd[k] = nx * yn + ny; use[k] = celdx < 0.5 && celdy < 0.5;
      w[k++] = swt1 * (1.0 - celdx - 0.5) * (1.0 - celdy - 0.5);
      nd[k] = nx * yn + ny + 1; use[k] = celdx < 0.5;
      w[k++] = swt1 * (1.0 - celdx - 0.5) * (1.0 - AB(celdy - 0.5));
      nd[k] = (nx + 1) * yn + ny; use[k] = celdy < 0.5;
      w[k++] = swt1 * (1.0 - AB(celdx - 0.5)) * (1.0 - celdy - 0.5);
      nd[k] = (nx + 1) * yn + ny + 1; use[k] = 1;
      w[k++] = swt1 * (1.0 - AB(celdx - 0.5)) * (1.0 - AB(celdy - 0.5));
      nd[k] = nx * yn + ny + 2; use[k] = celdx < 0.5 && celdy > 0.5;
      w[k++] = swt1 * (1.0 - celdx - 0.5) * (celdy - 0.5);
      nd[k] = (nx + 1) * yn + ny + 2; use[k] = celdy > 0.5;
      w[k++] = swt1 * (1.0 - AB(celdx - 0.5)) * (celdy - 0.5);
      nd[k] = (nx + 2) * yn + ny + 2; use[k] = celdx > 0.5 && celdy > 0.5;
      w[k++] = swt1 * (celdx - 0.5) * (celdy - 0.5);
      nd[k] = (nx + 2) * yn + ny + 1; use[k] = celdx > 0.5;
      w[k++] = swt1 * (celdx - 0.5) * (1.0 - AB(celdy - 0.5));
      nd[k] = (nx + 2) * yn + ny; use[k] = celdx > 0.5 && celdy < 0.5;
      w[k++] = swt1 * (celdx - 0.5) * (1.0 - celdy - 0.5);
    } else if (mode == 2) {
      nd[k] = (nx + 1) * yn + ny + 1; use[k] = 1;
      w[k++] = swt1 * (1.0 - 2 * AB(celdx - 0.5)) * (1.0 - 2 * AB(celdy - 0.5));
    }
    for (int i = 0; i < k; i++) {
      if (!(nd[i] < nn && use[i])) continue;
      m3 = nd[i];
      swt = w[i];
      PS[m3] = PS[m3] + o->PR * swt;
      SX[m3] = SX[m3] + o->SXX * swt;
      EX[m3] = EX[m3] + o->EXX * swt;
      WT[m3] = WT[m3] + swt;
    }
  }

  /* vx nodes (:1376-1432) */
  m10 = nx; m20 = ny;
  if (y < (gy[m20] + gy[m20 + 1]) / 2.0) m20 -= 1;
  if (m20 < 0) m20 = 0;
  if (m20 > yn - 3) m20 = yn - 3;
  e = (x - gx[m10]) / (gx[m10 + 1] - gx[m10]);
  n = (y - (gy[m20] + gy[m20 + 1]) / 2.0) / ((gy[m20 + 2] - gy[m20]) / 2);
  dm0 = (1.0 - e) * (1.0 - n); dm1 = (1.0 - e) * n; dm2 = e * (1.0 - n); dm3 = e * n;
  m3 = m10 * yn + m20;
  o->VX = bil(N[V2C_NF_VX], m3, yn, dm0, dm1, dm2, dm3);
  o->MVX = bil(N[V2C_NF_MVX], m3, yn, dm0, dm1, dm2, dm3);
  if (ad && mode == 2) {
    double *VS = N[V2C_NF_VXSUM], *MR = N[V2C_NF_MRX0], *WT = N[V2C_NF_WTVXSUM];
    if (celdx < 0.5) {
      m3 = nx * yn + ny;
      dx = 1.0 - celdx; dy = 1.0 - AB(celdy - 0.5);
      swt = swt1 * dx * dy;
      VS[m3] += o->VX * MRO * swt; MR[m3] += MRO * swt; WT[m3] += swt;
    }
    if (celdx > 0.5) {
      m3 = (nx + 1) * yn + ny;
      dx = celdx; dy = 1.0 - AB(celdy - 0.5);
      swt = swt1 * dx * dy;
      VS[m3] += o->VX * MRO * swt; MR[m3] += MRO * swt; WT[m3] += swt;
    }
  }

  /* vy nodes (:1433-1489) */
  m10 = nx; m20 = ny;
  if (x < (gx[m10] + gx[m10 + 1]) / 2.0) m10 -= 1;
  if (m10 < 0) m10 = 0;
  if (m10 > xn - 3) m10 = xn - 3;
  e = (x - (gx[m10] + gx[m10 + 1]) / 2.0) / ((gx[m10 + 2] - gx[m10]) / 2);
  n = (y - gy[m20]) / (gy[m20 + 1] - gy[m20]);
  dm0 = (1.0 - e) * (1.0 - n); dm1 = (1.0 - e) * n; dm2 = e * (1.0 - n); dm3 = e * n;
  m3 = m10 * yn + m20;
  o->VY = bil(N[V2C_NF_VY], m3, yn, dm0, dm1, dm2, dm3);
  o->MVY = bil(N[V2C_NF_MVY], m3, yn, dm0, dm1, dm2, dm3);
  if (ad && mode == 2) {
    double *VS = N[V2C_NF_VYSUM], *MR = N[V2C_NF_MRY0], *WT = N[V2C_NF_WTVYSUM];
    if (celdy < 0.5) {
      m3 = nx * yn + ny;
      dx = 1.0 - AB(celdx - 0.5); dy = 1.0 - celdy;
      swt = swt1 * dx * dy;
      VS[m3] = VS[m3] + o->VY * MRO * swt; MR[m3] = MR[m3] + MRO * swt; WT[m3] = WT[m3] + swt;
    }
    if (celdy > 0.5) {
      m3 = nx * yn + ny + 1;
      dx = 1.0 - AB(celdx - 0.5); dy = celdy;
      swt = swt1 * dx * dy;
      VS[m3] = VS[m3] + o->VY * MRO * swt; MR[m3] = MR[m3] + MRO * swt; WT[m3] = WT[m3] + swt;
    }
  }
}

int v2c_oracle_nodes2markers(v2c_oracle_state *s) {
  const v2c_params *p = &s->p;
  double **N = s->N, **M = s->M;
  long xn = p->xnumx, yn = p->ynumy, nn = nnodes(s);
  for (long m3 = 0; m3 < s->n; m3++) {
    int m2 = s->t[m3];
    mech o;
    double x = M[V2C_MF_X][m3], y = M[V2C_MF_Y][m3];
    interpolate_mechanical(s, x, y, &o, RT(s, V2C_RT_RO, m2));
    double k = M[V2C_MF_K][m3];
    if (x > 0 && y > 0 && x < p->xsize && y < p->ysize && s->t[m3] < 50 && k <= 0) {
      if (p->antidiffinter == 1) {
        M[V2C_MF_XX][m3] = o.SXX; M[V2C_MF_XY][m3] = o.SXY; M[V2C_MF_P][m3] = o.PR;
        M[V2C_MF_EXX][m3] = o.EXX; M[V2C_MF_EXY][m3] = o.EXY; M[V2C_MF_VX][m3] = o.VX;
        M[V2C_MF_VY][m3] = o.VY; M[V2C_MF_PHI][m3] = o.PHIS; M[V2C_MF_E][m3] = o.ES;
      } else {
        M[V2C_MF_XX][m3] = o.SXXE; M[V2C_MF_XY][m3] = o.SXYE; M[V2C_MF_P][m3] = o.SPPE;
        M[V2C_MF_EXX][m3] = o.EXXE; M[V2C_MF_EXY][m3] = o.EXYE; M[V2C_MF_VX][m3] = o.MVX;
        M[V2C_MF_VY][m3] = o.MVY; M[V2C_MF_PHI][m3] = o.PHISE; M[V2C_MF_E][m3] = o.ESE;
      }
      if (!p->tempmod) M[V2C_MF_K][m3] = p->eps2;
    }
    k = M[V2C_MF_K][m3];
    if (x >= 0 && y >= 0 && x <= p->xsize && y <= p->ysize && s->t[m3] < 50 && k > 0) {
      if (p->antidiffinter == 1) {
        M[V2C_MF_PHI][m3] = o.PHIS; M[V2C_MF_EXX][m3] = o.EXX; M[V2C_MF_EXY][m3] = o.EXY;
        M[V2C_MF_XX][m3] = o.SXX; M[V2C_MF_XY][m3] = o.SXY; M[V2C_MF_P][m3] = o.PR;
        M[V2C_MF_VX][m3] = o.VX; M[V2C_MF_VY][m3] = o.VY; M[V2C_MF_E][m3] = o.ES;
      } else {
        M[V2C_MF_PHI][m3] += (o.PHIS - o.PHISE); M[V2C_MF_EXX][m3] += (o.EXX - o.EXXE);
        M[V2C_MF_EXY][m3] += (o.EXY - o.EXYE); M[V2C_MF_XX][m3] += (o.SXX - o.SXXE);
        M[V2C_MF_XY][m3] += (o.SXY - o.SXYE); M[V2C_MF_P][m3] += (o.PR - o.SPPE);
        M[V2C_MF_VX][m3] += (o.VX - o.MVX); M[V2C_MF_VY][m3] += (o.VY - o.MVY);
        M[V2C_MF_E][m3] += (o.ES - o.ESE);
      }
    }
  }
  if (s->phantom) { /* zero marker at index marknum: back-scatter only */
    mech o;
    interpolate_mechanical(s, 0.0, 0.0, &o, RT(s, V2C_RT_RO, 0));
  }
  if (p->antidiffinter == 1) {
    for (long m3 = 0; m3 < nn; m3++) {
      long m22 = m3 % yn, m11 = (m3 - m22) / yn;
      double w = N[V2C_NF_WTPHISUM][m3];
      if (w && m11 >= 1 && m22 >= 1 && m11 < xn - 1 && m22 < yn - 1) {
        N[V2C_NF_PHIE][m3] = N[V2C_NF_PHISUM][m3] / w;
        N[V2C_NF_SXYEE][m3] = N[V2C_NF_SXYSUM][m3] / w;
        N[V2C_NF_EXYEE][m3] = N[V2C_NF_EXYSUM][m3] / w;
        N[V2C_NF_PEE][m3] = N[V2C_NF_ESUM][m3] / w;
      }
      w = N[V2C_NF_WTSXXSUM][m3];
      if (w && m11 >= 1 && m22 >= 1) {
        N[V2C_NF_SPPEE][m3] = N[V2C_NF_PSUM][m3] / w;
        N[V2C_NF_SXXEE][m3] = N[V2C_NF_SXXSUM][m3] / w;
        N[V2C_NF_EXXEE][m3] = N[V2C_NF_EXXSUM][m3] / w;
      }
      if (N[V2C_NF_WTVXSUM][m3]) N[V2C_NF_MVXE][m3] = N[V2C_NF_VXSUM][m3] / N[V2C_NF_MRX0][m3];
      if (N[V2C_NF_WTVYSUM][m3]) N[V2C_NF_MVYE][m3] = N[V2C_NF_VYSUM][m3] / N[V2C_NF_MRY0][m3];
    }
  }
  return 0;
}

/* ===================================================== moveandrotatemarkers
 * allinteri, interpolation.c:1688-1758: velocity, spin and strain-rate
 * invariant at a point. */
static void allinteri(const v2c_oracle_state *s, double x, double y, double *VX,
                      double *VY, double *ESP, double *EE) {
  const v2c_params *p = &s->p;
  const double *gx = s->gx, *gy = s->gy;
  const double *vx = s->N[V2C_NF_VX], *vy = s->N[V2C_NF_VY];
  const double *exx = s->N[V2C_NF_EXX], *exy = s->N[V2C_NF_EXY], *esp = s->N[V2C_NF_ESP];
  long xn = p->xnumx, yn = p->ynumy, m3, m10, m20;
  double e, n, EXX, EXY, xrat;
  if (x < 0) x = 0; else if (x > p->xsize) x = p->xsize;
  if (y < 0) y = 0; else if (y > p->ysize) y = p->ysize;
  xrat = 2.0 / 3.0;
  if (x < (gx[0] + gx[1]) / 2.0) xrat = 1.0;
  if (x > (gx[xn - 2] + gx[xn - 1]) / 2.0) xrat = 1.0;
  if (y < (gy[0] + gy[1]) / 2.0) xrat = 1.0;
  if (y > (gy[yn - 2] + gy[yn - 1]) / 2.0) xrat = 1.0;
  long nx = v2c_oracle_nxsearch(gx, xn, x), ny = v2c_oracle_nxsearch(gy, yn, y);
  /* exy, esp on basic nodes */
  m10 = nx; m20 = ny;
  if (m10 < 1) m10 = 1;
  if (m10 > xn - 3) m10 = xn - 3;
  if (m20 < 1) m20 = 1;
  if (m20 > yn - 3) m20 = yn - 3;
  e = (x - gx[m10]) / (gx[m10 + 1] - gx[m10]);
  n = (y - gy[m20]) / (gy[m20 + 1] - gy[m20]);
  m3 = m10 * yn + m20;
  EXY = (1.0 - e) * (1.0 - n) * exy[m3] + (1.0 - e) * n * exy[m3 + 1] + e * (1.0 - n) * exy[m3 + yn] + e * n * exy[m3 + yn + 1];
  *ESP = (1.0 - e) * (1.0 - n) * esp[m3] + (1.0 - e) * n * esp[m3 + 1] + e * (1.0 - n) * esp[m3 + yn] + e * n * esp[m3 + yn + 1];
  /* exx and the pressure-node averaged velocities */
  m10 = nx; m20 = ny;
  if (x > (gx[m10] + gx[m10 + 1]) / 2.0) m10++;
  if (y > (gy[m20] + gy[m20 + 1]) / 2.0) m20++;
  if (m10 < 1) m10 = 1;
  if (m10 > xn - 2) m10 = xn - 2;
  if (m20 < 1) m20 = 1;
  if (m20 > yn - 2) m20 = yn - 2;
  e = (x - (gx[m10 - 1] + gx[m10]) / 2.0) / ((gx[m10 + 1] - gx[m10 - 1]) / 2.0);
  n = (y - (gy[m20 - 1] + gy[m20]) / 2.0) / ((gy[m20 + 1] - gy[m20 - 1]) / 2.0);
  m3 = m10 * yn + m20;
  EXX = (1.0 - e) * (1.0 - n) * exx[m3] + (1.0 - e) * n * exx[m3 + 1] + e * (1.0 - n) * exx[m3 + yn] + e * n * exx[m3 + yn + 1];
  *VX = ((1.0 - e) * (1.0 - n) * (vx[m3 - 1] + vx[m3 - yn - 1]) + (1.0 - e) * n * (vx[m3] + vx[m3 - yn]) +
         e * (1.0 - n) * (vx[m3 + yn - 1] + vx[m3 - 1]) + e * n * (vx[m3 + yn] + vx[m3])) *
        0.5 * (1.0 - xrat);
  *VY = ((1.0 - e) * (1.0 - n) * (vy[m3 - yn] + vy[m3 - yn - 1]) + (1.0 - e) * n * (vy[m3 - yn + 1] + vy[m3 - yn]) +
         e * (1.0 - n) * (vy[m3] + vy[m3 - 1]) + e * n * (vy[m3 + 1] + vy[m3])) *
        0.5 * (1.0 - xrat);
  *EE = pow(EXX * EXX + EXY * EXY, 0.5);
  /* staggered vx */
  m10 = nx; m20 = ny;
  if (y < (gy[m20] + gy[m20 + 1]) / 2.0) m20 -= 1;
  if (m10 < 0) m10 = 0;
  if (m10 > xn - 2) m10 = xn - 2;
  if (m20 < 0) m20 = 0;
  if (m20 > yn - 3) m20 = yn - 3;
  e = (x - gx[m10]) / (gx[m10 + 1] - gx[m10]);
  n = (y - (gy[m20] + gy[m20 + 1]) / 2.0) / ((gy[m20 + 2] - gy[m20]) / 2.0);
  m3 = m10 * yn + m20;
  *VX += ((1.0 - e) * (1.0 - n) * vx[m3] + (1.0 - e) * n * vx[m3 + 1] + e * (1.0 - n) * vx[m3 + yn] + e * n * vx[m3 + yn + 1]) * xrat;
  /* staggered vy */
  m10 = nx; m20 = ny;
  if (x < (gx[m10] + gx[m10 + 1]) / 2.0) m10 -= 1;
  if (m10 < 0) m10 = 0;
  if (m10 > xn - 3) m10 = xn - 3;
  if (m20 < 0) m20 = 0;
  if (m20 > yn - 2) m20 = yn - 2;
  e = (x - (gx[m10] + gx[m10 + 1]) / 2.0) / ((gx[m10 + 2] - gx[m10]) / 2.0);
  n = (y - gy[m20]) / (gy[m20 + 1] - gy[m20]);
  m3 = m10 * yn + m20;
  *VY += ((1.0 - e) * (1.0 - n) * vy[m3] + (1.0 - e) * n * vy[m3 + 1] + e * (1.0 - n) * vy[m3 + yn] + e * n * vy[m3 + yn + 1]) * xrat;
}

/* moveandrotatemarkers.c:1-178.  Immobile markers (type >= 100) keep their
 * anchor in markk (x) and markv (y); one that moves inside the model spawns
 * a mobile marker of type - 100 there, appended after the last marker with
 * its temperature, strain, stresses, pressure and strain rates reset, and
 * goes back to its anchor, as it does when it strays more than ystpy from
 * it (:90-136).  Then out-of-model mobile markers, in index order, take the
 * appended markers from the last one back (:141-171).  This is the routine
 * as written for one thread: the reference's OpenMP build makes the append
 * index marknum1 a reduction variable, whose private copies start from 0,
 * so there the spawned markers overwrite markers 0, 1, ... instead. */
int v2c_oracle_move(v2c_oracle_state *s) {
  const v2c_params *p = &s->p;
  double **M = s->M;
  double dt = p->timestep;
  const long cap = s->cap > s->n ? s->cap : s->n;
  long marknum1 = s->n;
  for (long mm1 = 0; mm1 < s->n; mm1++) {
    int mm2 = s->t[mm1];
    double x = M[V2C_MF_X][mm1], y = M[V2C_MF_Y][mm1];
    if (!(((x >= 0 && y >= 0 && x <= p->xsize && y <= p->ysize) || p->outgrid != 1) &&
          !RT(s, V2C_RT_IM, mm2)))
      continue;
    double vx0, vy0, sp0, ee0, vx1, vy1, sp1, ee1, vx2, vy2, sp2, ee2, vx3, vy3, sp3, ee3, vx4, vy4, sp4, ee4;
    if (p->markmod == 1) {
      allinteri(s, x, y, &vx0, &vy0, &sp0, &ee0);
    } else {
      allinteri(s, x, y, &vx1, &vy1, &sp1, &ee1);
      allinteri(s, x + vx1 * dt / 2.0, y + vy1 * dt / 2.0, &vx2, &vy2, &sp2, &ee2);
      allinteri(s, x + vx2 * dt / 2.0, y + vy2 * dt / 2.0, &vx3, &vy3, &sp3, &ee3);
      allinteri(s, x + vx3 * dt, y + vy3 * dt, &vx4, &vy4, &sp4, &ee4);
      vx0 = (vx1 + 2.0 * vx2 + 2.0 * vx3 + vx4) / 6.0;
      vy0 = (vy1 + 2.0 * vy2 + 2.0 * vy3 + vy4) / 6.0;
      if (p->markmod == 2) {
        sp0 = (sp1 + 2.0 * sp2 + 2.0 * sp3 + sp4) / 6.0;
        ee0 = (ee1 + 2.0 * ee2 + 2.0 * ee3 + ee4) / 6.0;
      } else {
        sp0 = sp1;
        ee0 = ee1;
      }
    }
    (void)ee0;
    if (p->outgrid == 2) {
      if (x < 0 || x > p->xsize) vy0 = 0;
      if (y < 0 || y > p->ysize) vx0 = 0;
    }
    x += (dt * vx0);
    y += (dt * vy0);
    if (mm2 >= 100) {
      /* immobile marker (:88-135) */
      if (x >= 0 && y >= 0 && x <= p->xsize && y <= p->ysize) {
        if (marknum1 >= cap) return V2C_ERR_CAPACITY;  /* "Space out in markx[]" */
        const long k = marknum1++;
        s->t[k] = (signed char)(mm2 - 100);
        M[V2C_MF_X][k] = x;
        M[V2C_MF_Y][k] = y;
        M[V2C_MF_K][k] = 0;
        M[V2C_MF_D][k] = -1.0;
        M[V2C_MF_V][k] = 0;
        M[V2C_MF_E][k] = 0;
        M[V2C_MF_XX][k] = 0;
        M[V2C_MF_XY][k] = 0;
        M[V2C_MF_P][k] = 0;
        M[V2C_MF_EXX][k] = 0;
        M[V2C_MF_EXY][k] = 0;
        x = M[V2C_MF_K][mm1];
        y = M[V2C_MF_V][mm1];
      }
      double dx = x - M[V2C_MF_K][mm1];
      double dy = y - M[V2C_MF_V][mm1];
      dy = pow(dx * dx + dy * dy, 0.5);
      if (dy > p->ystpy) {
        x = M[V2C_MF_K][mm1];
        y = M[V2C_MF_V][mm1];
      }
      M[V2C_MF_X][mm1] = x;
      M[V2C_MF_Y][mm1] = y;
      continue;
    }
    M[V2C_MF_X][mm1] = x;
    M[V2C_MF_Y][mm1] = y;
    sp0 *= dt;
    double xx = M[V2C_MF_XX][mm1], xy = M[V2C_MF_XY][mm1];
    if (p->stoksmod == 1) {
      double a = xx * cos(sp0) * cos(sp0) - xx * sin(sp0) * sin(sp0) + xy * sin(2.0 * sp0);
      double b = 0.5 * (-xx - xx) * sin(2.0 * sp0) + xy * cos(2.0 * sp0);
      M[V2C_MF_XX][mm1] = a;
      M[V2C_MF_XY][mm1] = b;
    }
    if (p->stoksmod == 2) {
      double a = xx + xy * 2.0 * sp0;
      double b = xy + 0.5 * (-xx - xx) * 2.0 * sp0;
      M[V2C_MF_XX][mm1] = a;
      M[V2C_MF_XY][mm1] = b;
    }
    if (y > p->zdeep && vy0 < 0 && M[V2C_MF_K][mm1] < p->tdeep) M[V2C_MF_K][mm1] = p->tdeep;
    if (x < 0 || y < 0 || x > p->xsize || y > p->ysize) {
      M[V2C_MF_K][mm1] = 0;
      M[V2C_MF_D][mm1] = -1.0;
      M[V2C_MF_W][mm1] = -1.0;
      M[V2C_MF_E][mm1] = 0;
    }
  }
  /* out-of-model mobile markers take the appended ones, last first */
  for (long mm1 = 0; marknum1 > s->n && mm1 < s->n; mm1++) {
    const double x = M[V2C_MF_X][mm1], y = M[V2C_MF_Y][mm1];
    if ((x < 0 || y < 0 || x > p->xsize || y > p->ysize) && s->t[mm1] < 100) {
      marknum1--;
      s->t[mm1] = s->t[marknum1];
      M[V2C_MF_K][mm1] = 0;
      M[V2C_MF_D][mm1] = -1.0;
      M[V2C_MF_E][mm1] = 0;
      M[V2C_MF_XX][mm1] = 0;
      M[V2C_MF_XY][mm1] = 0;
      M[V2C_MF_P][mm1] = 0;
      M[V2C_MF_EXX][mm1] = 0;
      M[V2C_MF_EXY][mm1] = 0;
      M[V2C_MF_X][mm1] = M[V2C_MF_X][marknum1];
      M[V2C_MF_Y][mm1] = M[V2C_MF_Y][marknum1];
    }
  }
  s->n = marknum1;
  return 0;
}

/* =========================================================================
 * calc_timestep, calc_RSF.c:352-572, in the reference's loop order.  Nodes
 * with b <= 0 reset the state and slip-length limits to maxtmstep
 * (calc_RSF.c:497-501), so those two minima run over the nodes after the
 * last such node; lambda keeps its previous value where chi is NaN
 * (calc_RSF.c:466-481, no branch taken), starting here from 1/5.
 * ========================================================================= */
/* min/max/abs with the reference's comparison order (headevps.c:3-5), which
 * decides what a NaN candidate does to the running extremum */
#define MINV(a, b) ((a) <= (b) ? (a) : (b))
#define MAXV(a, b) ((a) >= (b) ? (a) : (b))
#define ABSV(a) ((a) >= 0 ? (a) : -(a))

int v2c_oracle_calc_timestep(const v2c_oracle_state *s, int oldornew,
                             const v2c_timestep_ctl *c, v2c_timestep_info *o) {
  const v2c_params *p = &s->p;
  const long xn = p->xnumx, yn = p->ynumy, nodenum = xn * yn;
  double *const *N = s->N;
  memset(o, 0, sizeof(*o));
  double maxvel = 0, maxVx = 0;
  o->min_sigin_1 = o->min_sigin_0 = 1e30;
  o->min_visc_1 = o->min_visc_0 = 1e30;
  double dt_f = c->maxtmstep;
  double dtnvp = 1e30, dtd = 1e30, dtphi = 1e30, dtL = 1e30;
  double lambda = 1.0 / 5.0;
  for (long m3 = 0; m3 < nodenum; m3++) {
    long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    if (!(m1 >= 1 && m2 >= 1 && m1 < xn - 1 && m2 < yn - 1)) continue;
    double dx = s->gx[m1 + 1] - s->gx[m1];
    double dy = s->gy[m2 + 1] - s->gy[m2];
    double faultwidth = 2 * 0.5 * (dx + dy);
    double NUVP;
    if (oldornew == 0) {
      if (N[V2C_NF_NU_M2C][m3] > 1.00e+26) {
        double sigin = pow(N[V2C_NF_SXXES][m3] * N[V2C_NF_SXXES][m3] +
                           N[V2C_NF_SXYE][m3] * N[V2C_NF_SXYE][m3], 0.5);
        double V = N[V2C_NF_RK_SLIPRS_FINAL][m3], nu = N[V2C_NF_NU_M2C][m3];
        if (sigin > 0 && V > 0) NUVP = nu * sigin / (2 * nu * V / faultwidth + sigin);
        else NUVP = nu;
      } else {
        NUVP = 5.00e+26;
      }
    } else {
      if (N[V2C_NF_NU_M2C][m3] > 1.00e+26) NUVP = N[V2C_NF_NU][m3];
      else NUVP = 5.00e+26;
    }
    dtnvp = MINV(dtnvp, c->tcnvp * NUVP / N[V2C_NF_GG][m3]);
    /* displacement time step */
    double VXn = oldornew == 1 ? N[V2C_NF_VX][m3] : N[V2C_NF_MVX][m3];
    double VYn = oldornew == 1 ? N[V2C_NF_VY][m3] : N[V2C_NF_MVY][m3];
    if (VXn != 0 && VYn != 0) {
      maxVx = MAXV(maxVx, MAXV(ABSV(VXn), ABSV(VYn)));
      double maxdr = MAXV(ABSV(VXn / dx), ABSV(VYn / dy));
      dtd = MINV(dtd, c->tcd * 1.0 / maxdr);
    }
    /* seismic-cycle time step */
    if (p->RSFmode == 1) {
      double nps = 0;
      if (p->pmode == 0) nps = p->nstress;
      else if (p->pmode == 1) nps = oldornew == 0 ? N[V2C_NF_SPPES][m3] : N[V2C_NF_PRS][m3];
      double bm = N[V2C_NF_BM][m3], gg = N[V2C_NF_GG][m3];
      double as = N[V2C_NF_AS][m3], bs = N[V2C_NF_BS][m3], Ls = N[V2C_NF_LS][m3];
      double v = (3 * bm - 2 * gg) / (2 * (3 * bm + gg));
      double k = 2.0 / 3.14 * (gg / (1 - v)) / p->xstpx;
      double chi = 1.0 / 4.0 * pow(k * Ls / (as * nps) - (bs - as) / as, 2) - k * Ls / (as * nps);
      if (chi > 0) lambda = as * nps / (k * Ls - (bs - as) * nps);
      else if (chi < 0) lambda = 1 - (bs - as) * nps / (k * Ls);
      else if (chi == 0) return V2C_ERR_TIMESTEP;
      lambda = MINV(lambda, 1.0 / 5.0);
      if (bs > 0) {
        if (oldornew == 0 && N[V2C_NF_RK_SLIPRS_FINAL][m3] > 0) {
          double phisc = N[V2C_NF_V0S][m3] / Ls * exp(-N[V2C_NF_PHIS][m3]);
          dtphi = MINV(dtphi, c->tcphih * 1.0 / phisc);
          dtL = MINV(dtL, lambda * Ls / (N[V2C_NF_RK_SLIPRS_FINAL][m3]));
        } else if (oldornew == 1 && N[V2C_NF_RK_SLIPRS_SOLVED][m3] > 0) {
          double phisc = N[V2C_NF_V0S][m3] / Ls * exp(-N[V2C_NF_PHIS_IT][m3]);
          dtphi = MINV(dtphi, c->tcphih * 1.0 / phisc);
          dtL = MINV(dtL, lambda * Ls / (N[V2C_NF_RK_SLIPRS_SOLVED][m3]));
        }
      } else {
        dtphi = c->maxtmstep;
        dtL = c->maxtmstep;
      }
    }
    /* stress and viscosity statistics over sticky-air flags */
    double sigin = pow(N[V2C_NF_SXXS][m3] * N[V2C_NF_SXXS][m3] +
                       N[V2C_NF_SXY][m3] * N[V2C_NF_SXY][m3], 0.5);
    double st = N[V2C_NF_STICKY01][m3], nu = N[V2C_NF_NU][m3];
    if (st == 1 && m1 == 50 && m2 == 50) { o->sigin_P1 = sigin; o->visco_P1 = nu; }
    if (st == 1 && m1 == 500 && m2 == 50) { o->sigin_P2 = sigin; o->visco_P2 = nu; }
    if (st == 2) {
      o->nr_1++;
      o->max_sigin_1 = MAXV(o->max_sigin_1, sigin); o->min_sigin_1 = MINV(o->min_sigin_1, sigin);
      o->sum_sigin_1 += sigin; o->sum2_sigin_1 += pow(sigin, 2);
      o->max_visc_1 = MAXV(o->max_visc_1, nu); o->min_visc_1 = MINV(o->min_visc_1, nu);
      o->sum_visc_1 += log10(nu); o->sum2_visc_1 += pow(log10(nu), 2);
    }
    if (st == 1) {
      o->nr_0++;
      o->max_sigin_0 = MAXV(o->max_sigin_0, sigin); o->min_sigin_0 = MINV(o->min_sigin_0, sigin);
      o->sum_sigin_0 += sigin; o->sum2_sigin_0 += pow(sigin, 2);
      o->max_visc_0 = MAXV(o->max_visc_0, nu); o->min_visc_0 = MINV(o->min_visc_0, nu);
      o->sum_visc_0 += log10(nu); o->sum2_visc_0 += pow(log10(nu), 2);
    }
    if (oldornew == 0 && N[V2C_NF_RK_SLIPRS_FINAL][m3] > 0)
      maxvel = MAXV(maxvel, N[V2C_NF_RK_SLIPRS_FINAL][m3]);
    if (oldornew == 1 && N[V2C_NF_RK_SLIPRS_SOLVED][m3] > 0)
      maxvel = MAXV(maxvel, N[V2C_NF_RK_SLIPRS_SOLVED][m3]);
  }
  dt_f = c->dtfactor * MINV(dt_f, MINV(dtphi, MINV(MINV(dtL, dtnvp), dtd)));
  o->dt_f = dt_f; o->maxvel = maxvel; o->maxVx = maxVx;
  o->dtnvp = dtnvp; o->dtd = dtd; o->dtphi = dtphi; o->dtL = dtL;
  return V2C_OK;
}

/* =========================================================================
 * Per-marker visco-elasto-plastic + RSF Newton (no counterpart in the
 * reference, which couples stress and slip rate only through its global
 * Picard loop).  With T* = tau_old + 2 G dt edot, c1 = 1 + G dt/eta and
 * klin = 4.3303e6 c1 + 2 G dt / W, the condition "Maxwell stress with the
 * visco-plastic viscosity eta_vp(V) equals the yield stress" (eta_vp from
 * calc_RSF.c:142, yield from calc_RSF.c:128, ageing-law state from
 * calc_RSF.c:96-103) is, after multiplying out the denominators,
 *    F(V) = sn a c1 asinh(V/(2V0) exp((mu0 + b phi(V))/a)) + klin V - T* = 0.
 * Unknown u = log V.  The relative residual is |F| / (F + T*).
 * ========================================================================= */
#define ETA_RAD 4.3303e+06

typedef struct {
  double a, b, L, V0, mu0, sn, dt, phio, ephio, Ts, c1, klin;
} rsf_prob;

static void rsf_setup(const double *st, double W, rsf_prob *q) {
  q->a = st[V2C_RS_A]; q->b = st[V2C_RS_B]; q->L = st[V2C_RS_L]; q->V0 = st[V2C_RS_V0];
  q->mu0 = st[V2C_RS_MU0]; q->sn = st[V2C_RS_SN]; q->dt = st[V2C_RS_DT];
  q->phio = st[V2C_RS_PHIOLD];
  q->ephio = exp(q->phio);
  double G = st[V2C_RS_G], eta = st[V2C_RS_ETA];
  q->Ts = st[V2C_RS_TAUOLD] + 2.0 * G * q->dt * st[V2C_RS_EDOT];
  q->c1 = 1.0 + G * q->dt / eta;
  q->klin = ETA_RAD * q->c1 + 2.0 * G * q->dt / W;
}

/* F, dF/du, relative residual; phi and tau_y at V = exp(u) */
static double rsf_eval(const rsf_prob *q, double u, double *dF, double *rel,
                       double *phi, double *tauy) {
  double V = exp(u);
  double x = V * q->dt / q->L;
  double g, dg; /* g and dg/du */
  if (x <= 1e-6) {
    g = q->ephio * (1 - x) + q->V0 * q->dt / q->L;
    dg = -q->ephio * x;
  } else {
    double r = q->V0 / V, ex = exp(-x);
    g = r + (q->ephio - r) * ex;
    dg = -r + r * ex - (q->ephio - r) * ex * x;
  }
  double ph = log(g), dph = dg / g;
  double w = u - log(2.0 * q->V0) + (q->mu0 + q->b * ph) / q->a;
  double A = (w > 20.0) ? w + 0.69314718055994530942 + 0.25 * exp(-2.0 * w) : asinh(exp(w));
  double dA = 1.0 / sqrt(1.0 + exp(-2.0 * w));
  double lhs = q->sn * q->a * q->c1 * A + q->klin * V;
  double F = lhs - q->Ts;
  if (dF) *dF = q->sn * q->a * q->c1 * dA * (1.0 + q->b / q->a * dph) + q->klin * V;
  if (rel) *rel = fabs(F) / lhs;
  if (phi) *phi = ph;
  if (tauy) *tauy = q->sn * q->a * A + ETA_RAD * V;
  return F;
}

double v2c_oracle_rsf_residual(const double *st, double W, double V, double *phi,
                               double *tauy, double *dF_dlogV, double *scale) {
  rsf_prob q;
  rsf_setup(st, W, &q);
  double rel;
  double F = rsf_eval(&q, log(V), dF_dlogV, &rel, phi, tauy);
  if (scale) *scale = F + q.Ts;
  return F;
}

/* safeguarded Newton in u = log V on the bracket [log 1e-40, log(Ts/klin)],
 * bisecting whenever the Newton step leaves the bracket.  A step below the
 * floor before F(floor) < 0 is known evaluates at the floor instead; F >= 0
 * there means the stress cannot drive slip above the floor and the solution
 * is the floor itself (the reference clamps slip rates at 1e-40,
 * calc_RSF.c:196).  Counts residual evaluations as iterations. */
int v2c_oracle_rsf_newton1(const double *st, double W, double u0, double rtol,
                           int maxit, double *V, double *phi, double *tau,
                           double *res) {
  rsf_prob q;
  rsf_setup(st, W, &q);
  double ulo = log(1e-40), uhi;
  if (!(q.Ts > 0)) { *V = 1e-40; *phi = q.phio; *tau = 0; *res = 0; return 0; }
  uhi = log(q.Ts / q.klin);
  if (uhi <= ulo) { /* the floor already carries the load */
    double rel;
    rsf_eval(&q, ulo, NULL, &rel, phi, tau);
    *V = 1e-40; *res = rel; return 1;
  }
  double u = u0;
  if (!(u > ulo)) u = ulo + 0.5 * (uhi - ulo) * 1e-3;
  if (!(u < uhi)) u = uhi - (uhi - ulo) * 1e-3;
  double dF, rel = 1, F;
  const double floor_u = ulo;
  int lo_known = 0; /* F(ulo) < 0 established */
  for (int it = 1; it <= maxit; it++) {
    F = rsf_eval(&q, u, &dF, &rel, phi, tau);
    if (rel <= rtol) { *V = exp(u); *res = rel; return it; }
    if (u == floor_u && F >= 0) { /* root below the 1e-40 floor (calc_RSF.c:196) */
      *V = 1e-40; *res = 0; return it;
    }
    if (F < 0) { ulo = u; lo_known = 1; } else uhi = u;
    double un = u - F / dF;
    if (!lo_known && dF > 0 && !(un > ulo)) un = floor_u; /* test the floor first */
    else if (!(dF > 0) || !(un > ulo) || !(un < uhi)) un = 0.5 * (ulo + uhi);
    u = un;
  }
  *V = exp(u);
  *res = rel;
  return -maxit;
}

long v2c_oracle_rsf_newton(const double *states, long n, double W, double rtol,
                           int maxit, const double *guess_logV, double *out,
                           int *iters) {
  long nonconv = 0;
  for (long i = 0; i < n; i++) {
    double st[V2C_RS_N];
    for (int k = 0; k < V2C_RS_N; k++) st[k] = states[(long)k * n + i];
    double u0 = guess_logV ? guess_logV[i] : log(st[V2C_RS_VOLD]);
    double V, phi, tau, res;
    int it = v2c_oracle_rsf_newton1(st, W, u0, rtol, maxit, &V, &phi, &tau, &res);
    if (it < 0) nonconv++;
    out[(long)V2C_RO_V * n + i] = V;
    out[(long)V2C_RO_PHI * n + i] = phi;
    out[(long)V2C_RO_TAU * n + i] = tau;
    out[(long)V2C_RO_RES * n + i] = res;
    if (iters) iters[i] = it;
  }
  return nonconv;
}

/* network inputs: a dimensionless summary of the state */
void v2c_oracle_rsf_features(const double *states, long n, long i, double *x) {
  double st[V2C_RS_N];
  for (int k = 0; k < V2C_RS_N; k++) st[k] = states[(long)k * n + i];
  rsf_prob q;
  rsf_setup(st, 400.0, &q);
  x[0] = log10(q.Ts / (q.sn * q.c1));              /* demanded friction      */
  x[1] = log10(q.klin / (q.sn * q.c1));            /* linear stiffness / sn  */
  x[2] = q.a * 100.0;
  x[3] = (q.b - q.a) * 100.0;
  x[4] = q.mu0;
  x[5] = q.phio;
  x[6] = log10(q.dt / q.L);
  x[7] = log10(q.V0);
}

/* ------------------------------------------------ MLP 8 -> 64 -> 64 -> 2 */
#define H V2C_MLP_H
static void mlp_offsets(long *oW1, long *ob1, long *oW2, long *ob2, long *oW3,
                        long *ob3, long *oxm, long *oxs, long *oym, long *oys) {
  *oW1 = 0; *ob1 = *oW1 + H * 8; *oW2 = *ob1 + H; *ob2 = *oW2 + H * H;
  *oW3 = *ob2 + H; *ob3 = *oW3 + 2 * H; *oxm = *ob3 + 2; *oxs = *oxm + 8;
  *oym = *oxs + 8; *oys = *oym + 2;
}

double v2c_oracle_mlp_loss_grad(const float *P, const double *X, const double *Y,
                                long n, double *grad) {
  long oW1, ob1, oW2, ob2, oW3, ob3, oxm, oxs, oym, oys;
  mlp_offsets(&oW1, &ob1, &oW2, &ob2, &oW3, &ob3, &oxm, &oxs, &oym, &oys);
  long ng = oxm;
  if (grad) memset(grad, 0, ng * sizeof(double));
  double loss = 0;
  for (long i = 0; i < n; i++) {
    double x[8], h1[H], h2[H], y[2], t[2];
    for (int k = 0; k < 8; k++) x[k] = (X[i * 8 + k] - P[oxm + k]) / P[oxs + k];
    for (int k = 0; k < 2; k++) t[k] = (Y[i * 2 + k] - P[oym + k]) / P[oys + k];
    for (int j = 0; j < H; j++) {
      double a = P[ob1 + j];
      for (int k = 0; k < 8; k++) a += (double)P[oW1 + j * 8 + k] * x[k];
      h1[j] = tanh(a);
    }
    for (int j = 0; j < H; j++) {
      double a = P[ob2 + j];
      for (int k = 0; k < H; k++) a += (double)P[oW2 + j * H + k] * h1[k];
      h2[j] = tanh(a);
    }
    for (int j = 0; j < 2; j++) {
      double a = P[ob3 + j];
      for (int k = 0; k < H; k++) a += (double)P[oW3 + j * H + k] * h2[k];
      y[j] = a;
    }
    double dy[2];
    for (int j = 0; j < 2; j++) {
      double d = y[j] - t[j];
      loss += d * d;
      dy[j] = 2.0 * d / (2.0 * n);
    }
    if (!grad) continue;
    double dh2[H], dh1[H];
    for (int j = 0; j < 2; j++) {
      grad[ob3 + j] += dy[j];
      for (int k = 0; k < H; k++) grad[oW3 + j * H + k] += dy[j] * h2[k];
    }
    for (int k = 0; k < H; k++) {
      double s = 0;
      for (int j = 0; j < 2; j++) s += dy[j] * P[oW3 + j * H + k];
      dh2[k] = s * (1.0 - h2[k] * h2[k]);
    }
    for (int j = 0; j < H; j++) {
      grad[ob2 + j] += dh2[j];
      for (int k = 0; k < H; k++) grad[oW2 + j * H + k] += dh2[j] * h1[k];
    }
    for (int k = 0; k < H; k++) {
      double s = 0;
      for (int j = 0; j < H; j++) s += dh2[j] * P[oW2 + j * H + k];
      dh1[k] = s * (1.0 - h1[k] * h1[k]);
    }
    for (int j = 0; j < H; j++) {
      grad[ob1 + j] += dh1[j];
      for (int k = 0; k < 8; k++) grad[oW1 + j * 8 + k] += dh1[j] * x[k];
    }
  }
  return loss / (2.0 * n);
}

void v2c_oracle_mlp_forward(const float *P, const double *X, long n, double *Y) {
  long oW1, ob1, oW2, ob2, oW3, ob3, oxm, oxs, oym, oys;
  mlp_offsets(&oW1, &ob1, &oW2, &ob2, &oW3, &ob3, &oxm, &oxs, &oym, &oys);
  for (long i = 0; i < n; i++) {
    double x[8], h1[H], h2[H];
    for (int k = 0; k < 8; k++) x[k] = (X[i * 8 + k] - P[oxm + k]) / P[oxs + k];
    for (int j = 0; j < H; j++) {
      double a = P[ob1 + j];
      for (int k = 0; k < 8; k++) a += (double)P[oW1 + j * 8 + k] * x[k];
      h1[j] = tanh(a);
    }
    for (int j = 0; j < H; j++) {
      double a = P[ob2 + j];
      for (int k = 0; k < H; k++) a += (double)P[oW2 + j * H + k] * h1[k];
      h2[j] = tanh(a);
    }
    for (int j = 0; j < 2; j++) {
      double a = P[ob3 + j];
      for (int k = 0; k < H; k++) a += (double)P[oW3 + j * H + k] * h2[k];
      Y[i * 2 + j] = a * P[oys + j] + P[oym + j];
    }
  }
}
#undef H

/* ------------------------------------------------------- Stokes assembly
 * preparematrix (momentum_continuity_addmatrix_checkerror.c:22-213) with
 * contadd (:932-998), xstoksadd (:642-731), ystoksadd (:794-877),
 * sxxcalc_prepare (:395-443), sxycalc_prepare (:483-525), bondadd
 * (:192-211), and the row layout of gausmat4_add (gausevps.c:137-214).
 * Where the reference calls exit(0) (an inconsistent continuity boundary)
 * or would index past the grid (an edge node without a boundary equation)
 * this returns V2C_ERR_UNSUPPORTED. */
#define SK_MAXT 24
typedef struct {
  double c;
  int n;
  long col[SK_MAXT];
  double w[SK_MAXT];
} sk_eq;

static void sk_add(sk_eq *E, long k, double v) {
  if (E->n < SK_MAXT) {
    E->col[E->n] = k;
    E->w[E->n] = v;
  }
  E->n++;
}

typedef struct {
  const v2c_oracle_state *s;
  const v2c_stokes_ctl *c;
  long xn, yn, nn;
  int bad;
} sk_ctx;

static void sk_sxx(sk_ctx *K, sk_eq *E, long m1, long m2, double ynval) {
  const v2c_oracle_state *s = K->s;
  long yn = K->yn;
  long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  double sxxeeff = s->N[V2C_NF_SXXE][v3], Z;
  double nueff = nueff_of(&s->p, s->N[V2C_NF_ND][v3], s->N[V2C_NF_GD][v3], K->c->dt, &Z);
  sk_add(E, v0 * 3 + 1, -ynval * nueff / (s->gx[m1] - s->gx[m1 - 1]));
  sk_add(E, v2 * 3 + 1, +ynval * nueff / (s->gx[m1] - s->gx[m1 - 1]));
  sk_add(E, v0 * 3 + 2, +ynval * nueff / (s->gy[m2] - s->gy[m2 - 1]));
  sk_add(E, v1 * 3 + 2, -ynval * nueff / (s->gy[m2] - s->gy[m2 - 1]));
  E->c -= (1.0 - Z) * ynval * sxxeeff;
}

static void sk_sxy(sk_ctx *K, sk_eq *E, long m1, long m2, double ynval) {
  const v2c_oracle_state *s = K->s;
  long yn = K->yn;
  long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  double sxyeeff = s->N[V2C_NF_SXYE][v3], Z;
  double nueff = nueff_of(&s->p, s->N[V2C_NF_NU][v3], s->N[V2C_NF_GG][v3], K->c->dt, &Z);
  sk_add(E, v2 * 3 + 1, -ynval * 2.0 * nueff / (s->gy[m2 + 1] - s->gy[m2 - 1]));
  sk_add(E, v3 * 3 + 1, +ynval * 2.0 * nueff / (s->gy[m2 + 1] - s->gy[m2 - 1]));
  sk_add(E, v1 * 3 + 2, -ynval * 2.0 * nueff / (s->gx[m1 + 1] - s->gx[m1 - 1]));
  sk_add(E, v3 * 3 + 2, +ynval * 2.0 * nueff / (s->gx[m1 + 1] - s->gx[m1 - 1]));
  E->c -= (1.0 - Z) * ynval * sxyeeff;
}

static void sk_cont(sk_ctx *K, sk_eq *E, long m1, long m2) {
  const v2c_oracle_state *s = K->s;
  long yn = K->yn;
  long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  E->n = 0;
  E->c = 0;
  if (s->p.compressiblemode == 1)
    E->c = s->N[V2C_NF_SPPE][v3] / s->N[V2C_NF_BM][v3] / s->p.timestep;
  sk_add(E, v0 * 3 + 1, -1.0 / (s->gx[m1] - s->gx[m1 - 1]));
  sk_add(E, v2 * 3 + 1, +1.0 / (s->gx[m1] - s->gx[m1 - 1]));
  sk_add(E, v0 * 3 + 2, -1.0 / (s->gy[m2] - s->gy[m2 - 1]));
  sk_add(E, v1 * 3 + 2, +1.0 / (s->gy[m2] - s->gy[m2 - 1]));
  if (s->p.compressiblemode == 1)
    sk_add(E, v3 * 3 + 0, 1.0 / s->N[V2C_NF_BM][v3] / s->p.timestep);
}

static void sk_bond(sk_ctx *K, sk_eq *E, long r) {
  const v2c_oracle_state *s = K->s;
  long B = s->bondm[r];
  E->n = 0;
  E->c = s->bondv[B * 4 + 0];
  sk_add(E, r, 1.0);
  for (int k = 0; k < 3; k++) {
    long bn = s->bondn[B * 3 + k];
    if (bn) {
      if (bn - 1 < 0 || bn - 1 >= 3 * K->nn) K->bad = 1;
      sk_add(E, bn - 1, -s->bondv[B * 4 + k + 1]);
    }
  }
}

static void sk_xstokes(sk_ctx *K, sk_eq *E, long m1, long m2) {
  const v2c_oracle_state *s = K->s;
  const double *gx = s->gx, *gy = s->gy, *ro = s->N[V2C_NF_RO];
  double dt = K->c->dt, GX = K->c->gxkoef;
  int inertyn = s->p.inertyn;
  long yn = K->yn;
  long v0 = m1 * yn + m2, v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  double xkf = (gx[m1 + 1] - gx[m1 - 1]) / 2.0, ykf = gy[m2 + 1] - gy[m2];
  E->n = 0;
  E->c = (-GX - inertyn * s->N[V2C_NF_MVX][v0] / dt) * s->N[V2C_NF_MRX][v0];
  sk_add(E, v1 * 3 + 0, +1.0 / xkf);
  sk_add(E, v3 * 3 + 0, -1.0 / xkf);
  sk_add(E, v0 * 3 + 1, -inertyn * s->N[V2C_NF_MRX][v0] / dt);
  sk_sxx(K, E, m1, m2 + 1, -1.0 / xkf);
  sk_sxx(K, E, m1 + 1, m2 + 1, 1.0 / xkf);
  sk_sxy(K, E, m1, m2, -1.0 / ykf);
  sk_sxy(K, E, m1, m2 + 1, 1.0 / ykf);
  if (K->c->drunkensailor == 1) {
    sk_add(E, v0 * 3 + 1,
           -dt / 2.0 * GX * (ro[v2] + ro[v3] - ro[v0 - yn] - ro[v1 - yn]) /
               (gx[m1 + 1] - gx[m1 - 1]) / 2.0);
    sk_add(E, v0 * 3 + 2,
           -dt / 2.0 * GX * (gx[m1] - gx[m1 - 1]) / (gx[m1 + 1] - gx[m1 - 1]) / 2.0 *
               (ro[v1] - ro[v0]) / (gy[m2 + 1] - gy[m2]));
    sk_add(E, v1 * 3 + 2,
           -dt / 2.0 * GX * (gx[m1] - gx[m1 - 1]) / (gx[m1 + 1] - gx[m1 - 1]) / 2.0 *
               (ro[v1] - ro[v0]) / (gy[m2 + 1] - gy[m2]));
    sk_add(E, (v0 - yn) * 3 + 2,
           -dt / 2.0 * GX * (gx[m1 + 1] - gx[m1]) / (gx[m1 + 1] - gx[m1 - 1]) / 2.0 *
               (ro[v1] - ro[v0]) / (gy[m2 + 1] - gy[m2]));
    sk_add(E, (v1 - yn) * 3 + 2,
           -dt / 2.0 * GX * (gx[m1 + 1] - gx[m1]) / (gx[m1 + 1] - gx[m1 - 1]) / 2.0 *
               (ro[v1] - ro[v0]) / (gy[m2 + 1] - gy[m2]));
  }
}

static void sk_ystokes(sk_ctx *K, sk_eq *E, long m1, long m2) {
  const v2c_oracle_state *s = K->s;
  const double *gx = s->gx, *gy = s->gy, *ro = s->N[V2C_NF_RO];
  double dt = K->c->dt, GY = K->c->gykoef;
  int inertyn = s->p.inertyn;
  long yn = K->yn;
  long v0 = m1 * yn + m2, v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  double xkf = gx[m1 + 1] - gx[m1], ykf = (gy[m2 + 1] - gy[m2 - 1]) / 2.0;
  E->n = 0;
  E->c = (-GY - inertyn * s->N[V2C_NF_MVY][v0] / dt) * s->N[V2C_NF_MRY][v0];
  sk_add(E, v2 * 3 + 0, +1.0 / ykf);
  sk_add(E, v3 * 3 + 0, -1.0 / ykf);
  sk_add(E, v0 * 3 + 2, -inertyn * s->N[V2C_NF_MRY][v0] / dt);
  sk_sxx(K, E, m1 + 1, m2, 1.0 / ykf);
  sk_sxx(K, E, m1 + 1, m2 + 1, -1.0 / ykf);
  sk_sxy(K, E, m1, m2, -1.0 / xkf);
  sk_sxy(K, E, m1 + 1, m2, 1.0 / xkf);
  if (K->c->drunkensailor == 1) {
    sk_add(E, v0 * 3 + 2,
           -dt / 2.0 * GY * (ro[v1] + ro[v3] - ro[v0 - 1] - ro[v2 - 1]) /
               (gy[m2 + 1] - gy[m2 - 1]) / 2.0);
    sk_add(E, v0 * 3 + 1,
           -dt / 2.0 * GY * (gy[m2] - gy[m2 - 1]) / (gy[m2 + 1] - gy[m2 - 1]) / 2.0 *
               (ro[v2] - ro[v0]) / (gx[m1 + 1] - gx[m1]));
    sk_add(E, v2 * 3 + 1,
           -dt / 2.0 * GY * (gy[m2] - gy[m2 - 1]) / (gy[m2 + 1] - gy[m2 - 1]) / 2.0 *
               (ro[v2] - ro[v0]) / (gx[m1 + 1] - gx[m1]));
    sk_add(E, (v0 - 1) * 3 + 1,
           -dt / 2.0 * GY * (gy[m2 + 1] - gy[m2]) / (gy[m2 + 1] - gy[m2 - 1]) / 2.0 *
               (ro[v2] - ro[v0]) / (gx[m1 + 1] - gx[m1]));
    sk_add(E, (v2 - 1) * 3 + 1,
           -dt / 2.0 * GY * (gy[m2 + 1] - gy[m2]) / (gy[m2 + 1] - gy[m2 - 1]) / 2.0 *
               (ro[v2] - ro[v0]) / (gx[m1 + 1] - gx[m1]));
  }
}

/* the continuity form of a vx (k = 2) or vy (k = 3) boundary, addvx
 * :92-108 / addvy :150-166 */
static int sk_cont_bond(sk_ctx *K, sk_eq *E, long r, long m1, long m2, int k) {
  const v2c_oracle_state *s = K->s;
  long B = s->bondm[r], ref = s->bondn[B * 3 + 0];
  long m3 = (ref - 1 - r) / 3, dm1 = 0, dm2 = 0;
  if (m3 >= K->yn) dm1 = 1;
  if (m3 == 1 || m3 > K->yn) dm2 = 1;
  if (m3 < 0 || m3 > K->yn + 1 || !(m1 + dm1) || !(m2 + dm2) || ref - k < 0 ||
      ref - k >= 4 * K->nn || !s->bondm[ref - k])
    return 0;
  if (m1 + dm1 > K->xn - 1 || m2 + dm2 > K->yn - 1) return 0;
  sk_cont(K, E, m1 + dm1, m2 + dm2);
  return 1;
}

static int sk_build(sk_ctx *K, long r, sk_eq *E) {
  const v2c_oracle_state *s = K->s;
  long m3 = r / 3, kind = r % 3, m2 = m3 % K->yn, m1 = (m3 - m2) / K->yn;
  long xn = K->xn, yn = K->yn;
  int scale = 1;
  E->n = 0;
  E->c = 0;
  if (kind == 0) { /* addcont */
    if (m1 && m2) {
      if (!s->bondm[r] || s->p.compressiblemode == 1) sk_cont(K, E, m1, m2);
      else sk_bond(K, E, r);
    } else {
      sk_add(E, r, 1.0);
    }
  } else if (kind == 1) { /* addvx */
    if (m2 < yn - 1) {
      if (!s->bondm[r] ||
          (s->p.timesum > K->c->timebond && m1 > 2 && m2 > 2 && m1 < xn - 4 && m2 < yn - 3)) {
        if (m1 < 1 || m1 > xn - 2 || m2 < 1 || m2 > yn - 3) return 0;
        sk_xstokes(K, E, m1, m2);
        scale = 0;
      } else if (s->bondv[s->bondm[r] * 4 + 1] > 1e+30) {
        if (!sk_cont_bond(K, E, r, m1, m2, 2)) return 0;
      } else {
        sk_bond(K, E, r);
      }
    } else {
      sk_add(E, r, 1.0);
    }
  } else { /* addvy */
    if (m1 < xn - 1) {
      if (!s->bondm[r]) {
        if (m1 < 1 || m1 > xn - 3 || m2 < 1 || m2 > yn - 2) return 0;
        sk_ystokes(K, E, m1, m2);
        scale = 0;
      } else if (s->bondv[s->bondm[r] * 4 + 1] > 1e+30) {
        if (!sk_cont_bond(K, E, r, m1, m2, 3)) return 0;
      } else {
        sk_bond(K, E, r);
      }
    } else {
      sk_add(E, r, 1.0);
    }
  }
  if (E->n > SK_MAXT) return 0;
  if (scale) {
    E->c *= K->c->mukoef;
    for (int i = 0; i < E->n; i++) E->w[i] *= K->c->mukoef;
  }
  return 1;
}

int v2c_oracle_stokes_assemble(const v2c_oracle_state *s, const v2c_stokes_ctl *c, long cap,
                               int *ia, int *ja, double *a, double *b, long *nnz) {
  sk_ctx K = {s, c, s->p.xnumx, s->p.ynumy, s->p.xnumx * s->p.ynumy, 0};
  long rows = 3 * K.nn, pos = 0;
  if (!s->bondm) return V2C_ERR_STATE;
  /* gausmat4_add's column buffer: bufv[] and the marks cur0[] */
  double *bufv = calloc((size_t)rows, sizeof(double));
  char *cur0 = calloc((size_t)rows, 1);
  if (!bufv || !cur0) {
    free(bufv);
    free(cur0);
    return V2C_ERR_CAPACITY;
  }
  int rc = V2C_OK;
  for (long r = 0; r < rows; r++) {
    sk_eq E;
    if (!sk_build(&K, r, &E) || K.bad) {
      rc = V2C_ERR_UNSUPPORTED;
      break;
    }
    long lo = rows, hi = -1;
    for (int i = 0; i < E.n; i++)
      if (E.w[i]) {
        bufv[E.col[i]] = 0.0;
        cur0[E.col[i]] = 1;
      }
    for (int i = 0; i < E.n; i++)
      if (E.w[i]) {
        if (E.col[i] < lo) lo = E.col[i];
        if (E.col[i] > hi) hi = E.col[i];
        bufv[E.col[i]] += E.w[i];
      }
    if (b) b[r] = E.c;
    if (ia) ia[r] = (int)(pos + 1);
    for (long k = lo; k <= hi; k++)
      if (cur0[k]) {
        if (bufv[k]) {
          if (ja && pos < cap) {
            ja[pos] = (int)(k + 1);
            a[pos] = bufv[k];
          }
          pos++;
        }
        bufv[k] = 0.0;
        cur0[k] = 0;
      }
  }
  if (ia && rc == V2C_OK) ia[rows] = (int)(pos + 1);
  free(bufv);
  free(cur0);
  *nnz = pos;
  if (rc == V2C_OK && ja && pos > cap) rc = V2C_ERR_CAPACITY;
  return rc;
}
#undef SK_MAXT
