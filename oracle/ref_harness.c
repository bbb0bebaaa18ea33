/*
 * ref_harness.c -- runs the reference's own hot-path routines on a case file.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh stages the reference C
 * sources (unmodified apart from larger array-size macros in headevps.c)
 * into oracle/_ref/src and compiles this file against them into
 * oracle/_ref/v2c_ref.  Like the reference's own build (src/i2evps.c:12-30)
 * the sources are #included into one translation unit; this file only
 * loads the reference's global arrays from a case file, calls
 *   marker2nodes, interpolate_center2basic_old, compute_before_solve,
 *   compute_after_solve, nodes2markers, moveandrotatemarkers
 * and writes the arrays back.  Stdout (the reference's progress prints) is
 * discarded.
 *
 * Case file (native endianness), written by velo2cycles_gb300/oracle_io.py:
 *   char magic[8] = "V2CCASE1"
 *   int64 xnumx, ynumy, n, bondnum, nthreads, stages, nsteps, warmup
 *   v2c_params
 *   double gx[xnumx], gy[ynumy], rt[V2C_RT_N][V2C_MAXTMR]
 *   double node[V2C_NF_N][nodenum], mark[V2C_MF_N][n]; int8 markt[n]
 *   int64 bondm[nodenum*4], bondn[bondnum*3]; double bondv[bondnum*4]
 * Result file:
 *   char magic[8] = "V2CRES01"; int64 n
 *   double node[V2C_NF_N][nodenum], mark[V2C_MF_N][n]; int8 markt[n]
 *   double seconds[8] (per stage, summed over timed steps), double deltas
 */
#ifndef _GNU_SOURCE
#define _GNU_SOURCE 1
#endif
#include <math.h>
#include <omp.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Pardiso (MKL) is not on the path; its one call site compiles to nothing */
#define PARDISO(...) ((void)0)

#include "headevps.c"
#include "input_RSF.c"
#include "calc_RSF.c"
#include "gausevps.c"
#include "interpolation.c"
#include "density_ductilevisc_calc.c"
#include "moveandrotatemarkers.c"
#include "momentum_continuity_addmatrix_checkerror.c"
#include "temperature_iterate.c"
#include "plastic.c"
#include "recalc_marker_properties.c"

#include "../include/v2c.h"

static double *node_array(int f) {
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
  }
  return NULL;
}

static double *marker_array(int f) {
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

static double *rock_row(int f) {
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

static void rd(void *dst, size_t sz, size_t n, FILE *f) {
  if (n && fread(dst, sz, n, f) != n) { fprintf(stderr, "short read\n"); exit(3); }
}
static void wr(const void *src, size_t sz, size_t n, FILE *f) {
  if (n && fwrite(src, sz, n, f) != n) { fprintf(stderr, "short write\n"); exit(3); }
}

static void set_params(const v2c_params *p) {
  xnumx = p->xnumx; ynumy = p->ynumy; xsize = p->xsize; ysize = p->ysize;
  xstpx = p->xstpx; ystpy = p->ystpy; timesum = p->timesum; timestep = p->timestep;
  interpolationmod = p->interpolationmod; antidiffinter = p->antidiffinter;
  markmod = p->markmod; stoksmod = p->stoksmod; outgrid = p->outgrid;
  densimod = p->densimod; RSFmode = p->RSFmode; power_law_RSF = p->power_law_RSF;
  rkmod = p->rkmod; stickymod = p->stickymod; inertyn = p->inertyn; pmode = p->pmode;
  tempmod = p->tempmod; compressiblemode = p->compressiblemode;
  reloadfromDP = p->reloadfromDP; nubeg = p->nubeg; nuend = p->nuend;
  nstress = p->nstress; Dphis = p->Dphis; zdeep = p->zdeep; tdeep = p->tdeep;
  eps[2] = p->eps2;
  a_vw = p->a_vw; b_vw = p->b_vw; L_vw = p->L_vw; V0_vw = p->V0_vw;
  a_vs = p->a_vs; b_vs = p->b_vs; L_vs = p->L_vs; V0_vs = p->V0_vs;
  a_hr = p->a_hr; b_hr = p->b_hr; L_hr = p->L_hr; V0_hr = p->V0_hr;
  start_updip = p->start_updip; end_updip = p->end_updip;
  start_downdip = p->start_downdip; end_downdip = p->end_downdip;
  half_range = p->half_range;
  nodenum = xnumx * ynumy; nodenum2 = nodenum * 2; nodenum3 = nodenum * 3;
  cellnum = (xnumx - 1) * (ynumy - 1);
  printmod = 0;
  sedimnum = 0;
  sedimcyc = 3;
}

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: v2c_ref case.bin result.bin\n"); return 2; }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 2; }
  char magic[8];
  rd(magic, 1, 8, f);
  if (memcmp(magic, "V2CCASE1", 8)) { fprintf(stderr, "bad case file\n"); return 2; }
  int64_t hdr[8];
  rd(hdr, sizeof(int64_t), 8, f);
  long xn = hdr[0], yn = hdr[1], n = hdr[2], nb = hdr[3];
  int nthreads = (int)hdr[4], stages = (int)hdr[5], nsteps = (int)hdr[6], warmup = (int)hdr[7];
  long nn = xn * yn;
  if (xn > MAXXLN || yn > MAXYLN || n + 1 > MAXMRK || nb + 1 > MAXBON || nn * 4 > MAXPAR) {
    fprintf(stderr, "case exceeds the compiled array sizes\n");
    return 4;
  }
  v2c_params p;
  rd(&p, sizeof(p), 1, f);
  set_params(&p);
  rd(gx, sizeof(double), xn, f);
  rd(gy, sizeof(double), yn, f);
  double *rt = (double *)malloc(sizeof(double) * V2C_RT_N * V2C_MAXTMR);
  rd(rt, sizeof(double), (size_t)V2C_RT_N * V2C_MAXTMR, f);
  for (int r = 0; r < V2C_RT_N; r++) {
    if (r == V2C_RT_IM) {
      for (int t = 0; t < V2C_MAXTMR; t++) markim[t] = (int)rt[r * V2C_MAXTMR + t];
    } else {
      memcpy(rock_row(r), rt + (long)r * V2C_MAXTMR, sizeof(double) * V2C_MAXTMR);
    }
  }
  for (int k = 0; k < V2C_NF_N; k++) rd(node_array(k), sizeof(double), nn, f);
  double *scratch = (double *)malloc(sizeof(double) * (n + 1));
  for (int k = 0; k < V2C_MF_N; k++) {
    double *dst = marker_array(k);
    rd(dst ? dst : scratch, sizeof(double), n, f);
    if (dst) dst[n] = 0.0; /* the extra index nodes2markers reads */
  }
  {
    signed char *t8 = (signed char *)malloc(n + 1);
    rd(t8, 1, n, f);
    for (long i = 0; i < n; i++) markt[i] = (char)t8[i];
    markt[n] = 0;
    free(t8);
  }
  int64_t *b64 = (int64_t *)malloc(sizeof(int64_t) * (nn * 4 + nb * 3 + 3));
  rd(b64, sizeof(int64_t), nn * 4, f);
  for (long i = 0; i < nn * 4; i++) bondm[i] = b64[i];
  rd(b64, sizeof(int64_t), nb * 3, f);
  for (long i = 0; i < nb; i++)
    for (int k = 0; k < 3; k++) bondn[i][k] = b64[i * 3 + k];
  double *bv = (double *)malloc(sizeof(double) * (nb * 4 + 4));
  rd(bv, sizeof(double), nb * 4, f);
  for (long i = 0; i < nb; i++)
    for (int k = 0; k < 4; k++) bondv[i][k] = bv[i * 4 + k];
  bondnum = nb;
  fclose(f);
  marknum = n;

  omp_set_num_threads(nthreads > 0 ? nthreads : 1);
  if (!freopen("/dev/null", "w", stdout)) return 5;

  double secs[8] = {0};
  double deltas = 0;
  for (int step = 0; step < warmup + nsteps; step++) {
    double t0;
    int timed = step >= warmup;
#define STAGE(bit, idx, call)                               \
  if (stages & (1 << bit)) {                                \
    t0 = omp_get_wtime();                                   \
    call;                                                   \
    if (timed) secs[idx] += omp_get_wtime() - t0;           \
  }
    STAGE(0, 0, marker2nodes());
    STAGE(1, 1, interpolate_center2basic_old(timestep));
    STAGE(2, 2, compute_before_solve(timestep, 0));
    STAGE(3, 3, deltas = compute_after_solve(timestep, 0));
    STAGE(4, 4, nodes2markers());
    STAGE(5, 5, moveandrotatemarkers());
#undef STAGE
  }

  FILE *o = fopen(argv[2], "wb");
  if (!o) { perror(argv[2]); return 2; }
  wr("V2CRES01", 1, 8, o);
  int64_t nout = marknum;
  wr(&nout, sizeof(int64_t), 1, o);
  for (int k = 0; k < V2C_NF_N; k++) wr(node_array(k), sizeof(double), nn, o);
  for (int k = 0; k < V2C_MF_N; k++) {
    double *src = marker_array(k);
    if (src) wr(src, sizeof(double), nout, o);
    else {
      memset(scratch, 0, sizeof(double) * nout);
      wr(scratch, sizeof(double), nout, o);
    }
  }
  {
    signed char *t8 = (signed char *)malloc(nout + 1);
    for (long i = 0; i < nout; i++) t8[i] = (signed char)markt[i];
    wr(t8, 1, nout, o);
    free(t8);
  }
  wr(secs, sizeof(double), 8, o);
  wr(&deltas, sizeof(double), 1, o);
  fclose(o);
  return 0;
}
