/*
 * v2c_bind_map.h -- which global array of the reference each C-ABI field id
 * names: V2C_NF_* node fields (headevps.c:95-190, input_RSF.c:3-6),
 * V2C_MF_* marker fields (headevps.c:209-248, input_RSF.c:11) and V2C_RT_*
 * rock-table rows (headevps.c:256-272; markim is an int row and is handled
 * by the caller).
 *
 * Include it inside the reference's translation unit, after headevps.c and
 * input_RSF.c, so that the globals are in scope.  Fields the reference does
 * not have (V2C_MF_SLIPV, V2C_NF_DSXX) map to NULL.
 */
#ifndef V2C_BIND_MAP_H
#define V2C_BIND_MAP_H

#include "v2c.h"

static double *v2c_bind_node_array(int f) {
  switch (f) {
    case V2C_NF_PHIS_IT: return phis_it;
    case V2C_NF_PHIE: return phie;
    case V2C_NF_SXY: return sxy;
    case V2C_NF_SXYEE: return sxyee;
    case V2C_NF_EXY: return exy;
    case V2C_NF_EXYEE: return exyee;
    case V2C_NF_PES: return pes;
    case V2C_NF_PEE: return pee;
    case V2C_NF_SXX: return sxx;
    case V2C_NF_SXXEE: return sxxee;
    case V2C_NF_PR: return pr;
    case V2C_NF_SPPEE: return sppee;
    case V2C_NF_EXX: return exx;
    case V2C_NF_EXXEE: return exxee;
    case V2C_NF_VX: return vx;
    case V2C_NF_MVXE: return mvxe;
    case V2C_NF_VY: return vy;
    case V2C_NF_MVYE: return mvye;
    case V2C_NF_ESP: return esp;
    case V2C_NF_PHIN: return phin;
    case V2C_NF_SXYEN: return sxyen;
    case V2C_NF_EXYEN: return exyen;
    case V2C_NF_PEN: return pen;
    case V2C_NF_PHIS: return phis;
    case V2C_NF_SXYE: return sxye;
    case V2C_NF_EXYE: return exye;
    case V2C_NF_PE: return pe;
    case V2C_NF_MUS_S: return mus_s;
    case V2C_NF_AS: return as;
    case V2C_NF_BS: return bs;
    case V2C_NF_LS: return Ls;
    case V2C_NF_V0S: return V0s;
    case V2C_NF_COHESION: return cohesion;
    case V2C_NF_NU_M2C: return nu_m2c;
    case V2C_NF_GG: return gg;
    case V2C_NF_SXXEN: return sxxen;
    case V2C_NF_SPPEN: return sppen;
    case V2C_NF_EXXEN: return exxen;
    case V2C_NF_SXXE: return sxxe;
    case V2C_NF_SPPE: return sppe;
    case V2C_NF_EXXE: return exxe;
    case V2C_NF_ND_M2C: return nd_m2c;
    case V2C_NF_GD: return gd;
    case V2C_NF_BM: return bm;
    case V2C_NF_DRO: return dro;
    case V2C_NF_DRP: return drp;
    case V2C_NF_MVXN: return mvxn;
    case V2C_NF_MVX: return mvx;
    case V2C_NF_MRX: return mrx;
    case V2C_NF_MVYN: return mvyn;
    case V2C_NF_MVY: return mvy;
    case V2C_NF_MRY: return mry;
    case V2C_NF_RO: return ro;
    case V2C_NF_ET: return et;
    case V2C_NF_HT: return ht;
    case V2C_NF_KT: return kt;
    case V2C_NF_CP: return cp;
    case V2C_NF_TK: return tk;
    case V2C_NF_STICKY01: return sticky01;
    case V2C_NF_NU: return nu;
    case V2C_NF_ND: return nd;
    case V2C_NF_EXXES: return exxes;
    case V2C_NF_SXXES: return sxxes;
    case V2C_NF_SPPES: return sppes;
    case V2C_NF_SXXS: return sxxs;
    case V2C_NF_RK_SLIPRS_FINAL: return RK_sliprs_final;
    case V2C_NF_RK_PHIDTS_FINAL: return RK_phidts_final;
    case V2C_NF_RK_SLIPRS_SOLVED: return RK_sliprs_solved;
    case V2C_NF_RK_PHIDTS_SOLVED: return RK_phidts_solved;
    case V2C_NF_SYIELDS: return syields;
    case V2C_NF_NUVP_IT: return nuvp_it;
    case V2C_NF_SLIPRS: return sliprs;
    case V2C_NF_EXXPL: return exxpl;
    case V2C_NF_RK_DELTAS: return RK_deltas;
    case V2C_NF_PHISUM: return phisum;
    case V2C_NF_WTPHISUM: return wtphisum;
    case V2C_NF_SXYSUM: return sxysum;
    case V2C_NF_EXYSUM: return exysum;
    case V2C_NF_ESUM: return esum;
    case V2C_NF_PSUM: return psum;
    case V2C_NF_SXXSUM: return sxxsum;
    case V2C_NF_EXXSUM: return exxsum;
    case V2C_NF_WTSXXSUM: return wtsxxsum;
    case V2C_NF_VXSUM: return vxsum;
    case V2C_NF_VYSUM: return vysum;
    case V2C_NF_WTVXSUM: return wtvxsum;
    case V2C_NF_WTVYSUM: return wtvysum;
    case V2C_NF_MRX0: return mrx0;
    case V2C_NF_MRY0: return mry0;
    case V2C_NF_PRS: return prs;
    case V2C_NF_EXXS: return exxs;
    case V2C_NF_EXXEL: return exxel;
    case V2C_NF_TK2: return tk2;
  }
  return NULL;
}

static double *v2c_bind_marker_array(int f) {
  switch (f) {
    case V2C_MF_X: return markx;
    case V2C_MF_Y: return marky;
    case V2C_MF_K: return markk;
    case V2C_MF_D: return markd;
    case V2C_MF_E: return marke;
    case V2C_MF_P: return markp;
    case V2C_MF_W: return markw;
    case V2C_MF_EXX: return markexx;
    case V2C_MF_EXY: return markexy;
    case V2C_MF_XX: return markxx;
    case V2C_MF_XY: return markxy;
    case V2C_MF_V: return markv;
    case V2C_MF_VX: return markvx;
    case V2C_MF_VY: return markvy;
    case V2C_MF_C: return markC;
    case V2C_MF_C0: return markC0;
    case V2C_MF_FRIC_STATIC: return fric_static;
    case V2C_MF_PHI: return markphi;
    case V2C_MF_A: return mark_a;
    case V2C_MF_B: return mark_b;
    case V2C_MF_L: return mark_L;
    case V2C_MF_L0: return mark_L0;
    case V2C_MF_V0: return mark_V0;
  }
  return NULL;
}

static double *v2c_bind_rock_row(int f) {
  switch (f) {
    case V2C_RT_GG: return markgg;
    case V2C_RT_NU: return marknu;
    case V2C_RT_DH: return markdh;
    case V2C_RT_DV: return markdv;
    case V2C_RT_SS: return markss;
    case V2C_RT_MM: return markmm;
    case V2C_RT_RO: return markro;
    case V2C_RT_BB: return markbb;
    case V2C_RT_AA: return markaa;
    case V2C_RT_CP: return markcp;
    case V2C_RT_KT: return markkt;
    case V2C_RT_HT: return markht;
    case V2C_RT_KF: return markkf;
    case V2C_RT_KP: return markkp;
    case V2C_RT_N0: return markn0;
    case V2C_RT_N1: return markn1;
  }
  return NULL;
}

#endif
