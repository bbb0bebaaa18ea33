/*
 * v2c_bind.c -- the reference program's MIC routines on the GPU over its
 * own global arrays (usage and data movement: v2c_bind.h).
 *
 * Compiled inside the reference's translation unit after headevps.c and
 * input_RSF.c (the globals named here are the reference's), with
 * -I<repo>/include, and linked with libv2c.so.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "v2c.h"
#include "v2c_bind.h"
#include "v2c_bind_map.h"

/* 0: host marker arrays are refreshed only by v2c_bind_markers_to_host()
 * (the host reads them only to save or post-process); 1: after every call
 * that changes them (a full marker download per call) */
int v2c_bind_sync_markers = 0;

static v2c_ctx *v2c_bind_ctx = NULL;
static int v2c_bind_have_markers = 0;  /* device markers current */
static int v2c_bind_have_model = 0;    /* grid, rock table, bonds set */
static double *v2c_bind_slipv = NULL;  /* the per-marker Newton's slip rate */
static long v2c_bind_slipv_n = 0;

/* node arrays each routine writes (brought back to the host) */
static const int v2c_bind_m2n_out[] = {
    V2C_NF_PHIN, V2C_NF_SXYEN, V2C_NF_EXYEN, V2C_NF_PEN, V2C_NF_PHIS, V2C_NF_SXYE,
    V2C_NF_EXYE, V2C_NF_PE, V2C_NF_MUS_S, V2C_NF_AS, V2C_NF_BS, V2C_NF_LS, V2C_NF_V0S,
    V2C_NF_COHESION, V2C_NF_NU_M2C, V2C_NF_GG, V2C_NF_SXXEN, V2C_NF_SPPEN, V2C_NF_EXXEN,
    V2C_NF_SXXE, V2C_NF_SPPE, V2C_NF_EXXE, V2C_NF_ND_M2C, V2C_NF_GD, V2C_NF_BM, V2C_NF_DRO,
    V2C_NF_DRP, V2C_NF_MVXN, V2C_NF_MVX, V2C_NF_MRX, V2C_NF_MVYN, V2C_NF_MVY, V2C_NF_MRY,
    V2C_NF_RO, V2C_NF_ET, V2C_NF_HT, V2C_NF_KT, V2C_NF_CP, V2C_NF_TK, V2C_NF_STICKY01,
    V2C_NF_NU, V2C_NF_ND, V2C_NF_WTPHISUM, V2C_NF_WTSXXSUM, V2C_NF_WTVXSUM, V2C_NF_WTVYSUM,
    V2C_NF_PHISUM, V2C_NF_SXYSUM, V2C_NF_EXYSUM, V2C_NF_ESUM, V2C_NF_SXXSUM, V2C_NF_EXXSUM,
    V2C_NF_VXSUM, V2C_NF_VYSUM, V2C_NF_PSUM, V2C_NF_MRX0, V2C_NF_MRY0};
static const int v2c_bind_c2b_out[] = {V2C_NF_EXXES, V2C_NF_SXXES, V2C_NF_SPPES};
static const int v2c_bind_before_out[] = {V2C_NF_PES, V2C_NF_PHIS_IT, V2C_NF_SYIELDS,
                                          V2C_NF_NUVP_IT, V2C_NF_SLIPRS, V2C_NF_NU};
static const int v2c_bind_after_out[] = {V2C_NF_RK_PHIDTS_SOLVED, V2C_NF_RK_SLIPRS_SOLVED,
                                         V2C_NF_RK_DELTAS};
static const int v2c_bind_n2m_out[] = {
    V2C_NF_PHISUM, V2C_NF_WTPHISUM, V2C_NF_SXYSUM, V2C_NF_EXYSUM, V2C_NF_ESUM, V2C_NF_PSUM,
    V2C_NF_SXXSUM, V2C_NF_EXXSUM, V2C_NF_WTSXXSUM, V2C_NF_VXSUM, V2C_NF_VYSUM,
    V2C_NF_WTVXSUM, V2C_NF_WTVYSUM, V2C_NF_MRX0, V2C_NF_MRY0, V2C_NF_PHIE, V2C_NF_SXYEE,
    V2C_NF_EXYEE, V2C_NF_PEE, V2C_NF_SPPEE, V2C_NF_SXXEE, V2C_NF_EXXEE, V2C_NF_MVXE,
    V2C_NF_MVYE};
#define V2C_BIND_LEN(a) ((int)(sizeof(a) / sizeof((a)[0])))

static int v2c_bind_ok(int rc, const char *what) {
  if (rc == V2C_OK) return 1;
  printf("v2c_bind: %s failed with status %d\n", what, rc);
  errcheck = 1;
  return 0;
}

/* the scalars of v2c_params from the reference's globals; the frictional
 * band is the reference's fixed one (calc_RSF.c:226-230), W from
 * plastic.c:22, and the per-marker Newton is off (no counterpart) */
static void v2c_bind_params(v2c_params *p) {
  memset(p, 0, sizeof(*p));
  p->xnumx = xnumx; p->ynumy = ynumy; p->xsize = xsize; p->ysize = ysize;
  p->xstpx = xstpx; p->ystpy = ystpy; p->timesum = timesum; p->timestep = timestep;
  p->interpolationmod = interpolationmod; p->antidiffinter = antidiffinter;
  p->markmod = markmod; p->stoksmod = stoksmod; p->outgrid = outgrid;
  p->densimod = densimod; p->RSFmode = RSFmode; p->power_law_RSF = power_law_RSF;
  p->rkmod = rkmod; p->stickymod = stickymod; p->inertyn = inertyn; p->pmode = pmode;
  p->tempmod = tempmod; p->compressiblemode = compressiblemode;
  p->reloadfromDP = reloadfromDP; p->nubeg = nubeg; p->nuend = nuend;
  p->nstress = nstress; p->Dphis = Dphis; p->zdeep = zdeep; p->tdeep = tdeep;
  p->eps2 = eps[2];
  p->a_vw = a_vw; p->b_vw = b_vw; p->L_vw = L_vw; p->V0_vw = V0_vw;
  p->a_vs = a_vs; p->b_vs = b_vs; p->L_vs = L_vs; p->V0_vs = V0_vs;
  p->a_hr = a_hr; p->b_hr = b_hr; p->L_hr = L_hr; p->V0_hr = V0_hr;
  p->start_updip = start_updip; p->end_updip = end_updip;
  p->start_downdip = start_downdip; p->end_downdip = end_downdip;
  p->half_range = half_range;
  p->fault_y = 10.0e3; p->fault_hw = 100.0; p->fault_slope = 0.0;
  p->faultwidth = 400.0;
  p->newton_rtol = 1e-10; p->newton_maxit = 60;
  p->newton_guess = V2C_GUESS_OFF;
  p->newton_precision = V2C_NEWTON_SPLIT;
}

static int v2c_bind_setup(void) {
  v2c_params p;
  v2c_bind_params(&p);
  if (!v2c_bind_ctx) {
    if (!v2c_bind_ok(v2c_create(&p, MAXMRK, NULL, &v2c_bind_ctx), "v2c_create")) return 0;
    v2c_bind_have_model = 0;
    v2c_bind_have_markers = 0;
  }
  if (!v2c_bind_ok(v2c_set_params(v2c_bind_ctx, &p), "v2c_set_params")) return 0;
  if (!v2c_bind_have_model) {
    double *rt = (double *)malloc(sizeof(double) * V2C_RT_N * V2C_MAXTMR);
    if (!rt) return v2c_bind_ok(V2C_ERR_CAPACITY, "rock table");
    for (int r = 0; r < V2C_RT_N; r++)
      for (int t = 0; t < V2C_MAXTMR; t++)
        rt[r * V2C_MAXTMR + t] = (r == V2C_RT_IM) ? (double)markim[t] : v2c_bind_rock_row(r)[t];
    int ok = v2c_bind_ok(v2c_set_grid(v2c_bind_ctx, gx, gy), "v2c_set_grid") &&
             v2c_bind_ok(v2c_set_rock_table(v2c_bind_ctx, rt), "v2c_set_rock_table") &&
             v2c_bind_ok(v2c_set_bonds(v2c_bind_ctx, bondm, &bondn[0][0], &bondv[0][0], bondnum),
                         "v2c_set_bonds");
    free(rt);
    if (!ok) return 0;
    v2c_bind_have_model = 1;
  }
  if (!v2c_bind_have_markers) {
    if (v2c_bind_slipv_n < marknum) {
      free(v2c_bind_slipv);
      v2c_bind_slipv = (double *)calloc(marknum > 0 ? marknum : 1, sizeof(double));
      v2c_bind_slipv_n = marknum;
    }
    const double *f[V2C_MF_N];
    for (int k = 0; k < V2C_MF_N; k++) f[k] = v2c_bind_marker_array(k);
    f[V2C_MF_SLIPV] = v2c_bind_slipv;
    if (!v2c_bind_ok(v2c_upload_markers(v2c_bind_ctx, f, (const signed char *)markt, marknum),
                     "v2c_upload_markers"))
      return 0;
    v2c_bind_have_markers = 1;
  }
  return 1;
}

static int v2c_bind_nodes_up(void) {
  /* every node array the reference has (fields it lacks stay as they are) */
  int fields[V2C_NF_N], nf = 0;
  const double *src[V2C_NF_N];
  for (int k = 0; k < V2C_NF_N; k++) {
    const double *a = v2c_bind_node_array(k);
    if (!a) continue;
    fields[nf] = k;
    src[nf++] = a;
  }
  return v2c_bind_ok(v2c_upload_node_fields(v2c_bind_ctx, nf, fields, src),
                     "v2c_upload_node_fields");
}

static void v2c_bind_nodes_down(const int *fields, int nf) {
  double *dst[V2C_NF_N];
  for (int k = 0; k < nf; k++) dst[k] = v2c_bind_node_array(fields[k]);
  v2c_bind_ok(v2c_download_node_fields(v2c_bind_ctx, nf, fields, dst), "v2c_download_node_fields");
}

void v2c_bind_markers_to_host(void) {
  if (!v2c_bind_ctx || !v2c_bind_have_markers) return;
  if (v2c_bind_slipv_n < marknum) {  /* markers appended by immobile ones */
    double *p = (double *)realloc(v2c_bind_slipv, sizeof(double) * marknum);
    if (!p) { printf("v2c_bind: out of host memory\n"); errcheck = 1; return; }
    memset(p + v2c_bind_slipv_n, 0, sizeof(double) * (marknum - v2c_bind_slipv_n));
    v2c_bind_slipv = p;
    v2c_bind_slipv_n = marknum;
  }
  /* the fields the GPU keeps; markd/markw only where a marker was reset */
  double *f[V2C_MF_N];
  memset(f, 0, sizeof(f));
  static const int keep[] = {V2C_MF_X, V2C_MF_Y, V2C_MF_K, V2C_MF_V, V2C_MF_D, V2C_MF_E, V2C_MF_P,
                             V2C_MF_W, V2C_MF_EXX, V2C_MF_EXY, V2C_MF_XX, V2C_MF_XY,
                             V2C_MF_VX, V2C_MF_VY, V2C_MF_C, V2C_MF_PHI};
  for (int k = 0; k < V2C_BIND_LEN(keep); k++) f[keep[k]] = v2c_bind_marker_array(keep[k]);
  f[V2C_MF_SLIPV] = v2c_bind_slipv;
  v2c_bind_ok(v2c_download_markers(v2c_bind_ctx, f, (signed char *)markt, marknum),
              "v2c_download_markers");
}

void v2c_bind_markers_changed(void) { v2c_bind_have_markers = 0; }
void v2c_bind_model_changed(void) { v2c_bind_have_model = 0; }

void v2c_bind_marker2nodes(void) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return;
  if (!v2c_bind_ok(v2c_marker2nodes(v2c_bind_ctx), "v2c_marker2nodes")) return;
  v2c_bind_nodes_down(v2c_bind_m2n_out, V2C_BIND_LEN(v2c_bind_m2n_out));
  if (v2c_bind_sync_markers) v2c_bind_markers_to_host();
}

double v2c_bind_interpolate_center2basic_old(double dt) {
  (void)dt;  /* the reference's argument is unused as well */
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  if (!v2c_bind_ok(v2c_center2basic_old(v2c_bind_ctx), "v2c_center2basic_old")) return 0;
  v2c_bind_nodes_down(v2c_bind_c2b_out, V2C_BIND_LEN(v2c_bind_c2b_out));
  return 0;
}

double v2c_bind_interpolate_basic2center(void) {
  static const int out[] = {V2C_NF_ND};
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  if (!v2c_bind_ok(v2c_interpolate_basic2center(v2c_bind_ctx), "v2c_interpolate_basic2center"))
    return 0;
  v2c_bind_nodes_down(out, V2C_BIND_LEN(out));
  return 0;
}

double v2c_bind_interpolate_center2basic(double dt) {
  static const int out[] = {V2C_NF_EXXS, V2C_NF_EXXPL, V2C_NF_SXXS, V2C_NF_PRS, V2C_NF_EXXEL};
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  if (!v2c_bind_ok(v2c_interpolate_center2basic(v2c_bind_ctx, dt), "v2c_interpolate_center2basic"))
    return 0;
  v2c_bind_nodes_down(out, V2C_BIND_LEN(out));
  return 0;
}

/* the marker part of solve_temperature (temperature_iterate.c:181-412),
 * after the host's thermal solve has left the solved temperature in tk and
 * the previous one in tk2 */
void v2c_bind_marker_temperature(void) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return;
  if (!v2c_bind_ok(v2c_marker_temperature(v2c_bind_ctx, heatdif), "v2c_marker_temperature"))
    return;
  if (v2c_bind_sync_markers) v2c_bind_markers_to_host();
}

/* preparematrix (momentum_continuity_addmatrix_checkerror.c:22-38): the
 * Stokes matrix assembled on the device into the reference's Pardiso
 * arrays ia, ja, a, b and pos0cur, as gausmat4_add leaves them */
void v2c_bind_preparematrix(double mukoef, double dt, int rk) {
  (void)rk;
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return;
  v2c_stokes_ctl c = {mukoef, dt, GXKOEF, GYKOEF, timebond, drunkensailor};
  long nnz = 0;
  int rc = v2c_stokes_assemble(v2c_bind_ctx, &c, MAXVAL, ia, ja, a, b, &nnz);
  if (rc == V2C_ERR_CAPACITY) { /* the reference's own limit */
    printf("EXIT PROGRAM: Space out in a[] %ld", nnz);
    exit(0);
  }
  if (!v2c_bind_ok(rc, "v2c_stokes_assemble")) return;
  pos0cur = nnz;
}

void v2c_bind_compute_before_solve(double dt, int rk) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return;
  if (!v2c_bind_ok(v2c_compute_before_solve(v2c_bind_ctx, dt, rk), "v2c_compute_before_solve"))
    return;
  v2c_bind_nodes_down(v2c_bind_before_out, V2C_BIND_LEN(v2c_bind_before_out));
}

double v2c_bind_compute_after_solve(double dt, int rk) {
  double deltas = 0;
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  if (!v2c_bind_ok(v2c_compute_after_solve(v2c_bind_ctx, dt, rk, &deltas),
                   "v2c_compute_after_solve"))
    return 0;
  v2c_bind_nodes_down(v2c_bind_after_out, V2C_BIND_LEN(v2c_bind_after_out));
  return deltas;
}

double v2c_bind_nodes2markers(void) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  if (!v2c_bind_ok(v2c_nodes2markers(v2c_bind_ctx), "v2c_nodes2markers")) return 0;
  v2c_bind_nodes_down(v2c_bind_n2m_out, V2C_BIND_LEN(v2c_bind_n2m_out));
  if (v2c_bind_sync_markers) v2c_bind_markers_to_host();
  return 0;
}

void v2c_bind_moveandrotatemarkers(void) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return;
  if (!v2c_bind_ok(v2c_moveandrotatemarkers(v2c_bind_ctx), "v2c_moveandrotatemarkers")) return;
  /* immobile markers append markers: the new count, as the reference sets
   * marknum at the end of its routine (moveandrotatemarkers.c:176) */
  v2c_status st;
  if (v2c_bind_ok(v2c_get_status(v2c_bind_ctx, &st), "v2c_get_status")) {
    if (st.n_markers > MAXMRK) {
      printf("Space out in markx[]");
      exit(0);
    }
    marknum = st.n_markers;
  }
  if (v2c_bind_sync_markers) v2c_bind_markers_to_host();
}

double v2c_bind_calc_timestep(int oldornew) {
  if (!v2c_bind_setup() || !v2c_bind_nodes_up()) return 0;
  v2c_timestep_ctl c = {maxtmstep, dtfactor, tcnvp, tcd, tcphih};
  v2c_timestep_info o;
  int rc = v2c_calc_timestep(v2c_bind_ctx, oldornew, &c, &o);
  if (rc == V2C_ERR_TIMESTEP) {  /* the reference stops here */
    printf("\n Chi is zero in the adaptive time stepping loop \n");
    exit(0);
  }
  if (!v2c_bind_ok(rc, "v2c_calc_timestep")) return 0;
  /* the globals calc_timestep leaves behind (calc_RSF.c:352-572) */
  maxvel = o.maxvel;
  dtnvp = o.dtnvp; dtd = o.dtd; dtphi = o.dtphi; dtL = o.dtL;
  nr_0 = (int)o.nr_0; nr_1 = (int)o.nr_1;
  max_sigin_0 = o.max_sigin_0; min_sigin_0 = o.min_sigin_0;
  sum_sigin_0 = o.sum_sigin_0; sum2_sigin_0 = o.sum2_sigin_0;
  max_visc_0 = o.max_visc_0; min_visc_0 = o.min_visc_0;
  sum_visc_0 = o.sum_visc_0; sum2_visc_0 = o.sum2_visc_0;
  max_sigin_1 = o.max_sigin_1; min_sigin_1 = o.min_sigin_1;
  sum_sigin_1 = o.sum_sigin_1; sum2_sigin_1 = o.sum2_sigin_1;
  max_visc_1 = o.max_visc_1; min_visc_1 = o.min_visc_1;
  sum_visc_1 = o.sum_visc_1; sum2_visc_1 = o.sum2_visc_1;
  sigin_P1 = o.sigin_P1; sigin_P2 = o.sigin_P2; visco_P1 = o.visco_P1; visco_P2 = o.visco_P2;
  return o.dt_f;
}

void v2c_bind_close(void) {
  if (v2c_bind_ctx) v2c_destroy(v2c_bind_ctx);
  v2c_bind_ctx = NULL;
  v2c_bind_have_markers = 0;
  v2c_bind_have_model = 0;
  free(v2c_bind_slipv);
  v2c_bind_slipv = NULL;
  v2c_bind_slipv_n = 0;
}
