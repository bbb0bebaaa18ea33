/*
 * v2c_oracle.h -- CPU restatement of the VELO2CYCLEs marker-in-cell step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark compare the CUDA
 * path against.  The product (velo2cycles_gb300) never links or calls it.
 *
 * It restates, in FP64 and in the reference's arithmetic order, the routines
 * of src/interpolation.c, src/moveandrotatemarkers.c,
 * src/density_ductilevisc_calc.c, src/recalc_marker_properties.c,
 * src/calc_RSF.c and src/plastic.c over explicit arrays instead of the
 * reference's globals.  Each function cites the reference lines it follows.
 * It is pinned against the reference source itself, compiled unmodified by
 * oracle/build_ref.sh (see tests/test_oracle_pin.py).
 */
#ifndef V2C_ORACLE_H
#define V2C_ORACLE_H
#include "../include/v2c.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct v2c_oracle_state {
  v2c_params p;
  const double *gx, *gy;        /* grid lines                               */
  const double *rt;             /* rock table [V2C_RT_N][V2C_MAXTMR]        */
  double *N[V2C_NF_N];          /* node fields, each double[nodenum]        */
  double *M[V2C_MF_N];          /* marker fields, each double[n]            */
  signed char *t;               /* markt                                    */
  long n;                       /* marknum                                  */
  const long *bondm;            /* [nodenum*4] (may be NULL: no corrections) */
  const long *bondn;            /* [bondnum][3]                             */
  const double *bondv;          /* [bondnum][4]                             */
  long bondnum;
  int nthreads;                 /* unused (the restatement is sequential)   */
  int phantom;                  /* 1: nodes2markers also back-scatters the
                                   zero marker one past the end, as the
                                   reference's loop bound m3<=marknum does
                                   (interpolation.c:937)                   */
  long cap;                     /* marker arrays' capacity (>= n; 0: n):
                                   immobile markers append new markers     */
} v2c_oracle_state;

long v2c_oracle_nxsearch(const double *g, long n, double x);
int v2c_oracle_marker2nodes(v2c_oracle_state *s);
int v2c_oracle_center2basic_old(v2c_oracle_state *s);
int v2c_oracle_center2basic(v2c_oracle_state *s, double dt);
int v2c_oracle_basic2center(v2c_oracle_state *s);
int v2c_oracle_recompute_stress(v2c_oracle_state *s, double dt);
int v2c_oracle_copyarrays(v2c_oracle_state *s);
int v2c_oracle_marker_temperature(v2c_oracle_state *s, double heatdif);
/* preparematrix + gausmat4_add: the Stokes matrix as CSR (1-based ia, ja) */
int v2c_oracle_stokes_assemble(const v2c_oracle_state *s, const v2c_stokes_ctl *c, long cap,
                               int *ia, int *ja, double *a, double *b, long *nnz);
int v2c_oracle_compute_before_solve(v2c_oracle_state *s, double dt, int rk);
double v2c_oracle_compute_after_solve(v2c_oracle_state *s, double dt, int rk);
int v2c_oracle_nodes2markers(v2c_oracle_state *s);
int v2c_oracle_move(v2c_oracle_state *s);

/* adaptive time step, calc_RSF.c:352-572; returns V2C_OK or
 * V2C_ERR_TIMESTEP where the reference would stop (chi == 0) */
int v2c_oracle_calc_timestep(const v2c_oracle_state *s, int oldornew,
                             const v2c_timestep_ctl *c, v2c_timestep_info *info);

/* per-marker viscosity, conductivity and pressure (bar) of
 * recalc_marker_properties, 0 outside the model */
int v2c_oracle_marker_properties(const v2c_oracle_state *s, double *mnu, double *mkt,
                                 double *mpb);
/* per-marker ductile viscosity, density_ductilevisc_calc.c:29-223 */
double v2c_oracle_ductilevisc(const v2c_oracle_state *s, int mm2, double SXY,
                              double SXX, double EXY, double EXX, double mtk,
                              double mpb);

/* ----- per-marker visco-elasto-plastic + RSF Newton (extension) ---------- */
/* residual F(V) and dF/dlogV for one state (columns as V2C_RS_*) */
double v2c_oracle_rsf_residual(const double *st, double W, double V,
                               double *phi, double *tauy, double *dF_dlogV,
                               double *scale);
/* safeguarded Newton in log V; returns iterations (negative: no convergence) */
int v2c_oracle_rsf_newton1(const double *st, double W, double logV0,
                           double rtol, int maxit, double *V, double *phi,
                           double *tau, double *res);
/* states column-major [V2C_RS_N][n]; out column-major [V2C_RO_N][n] */
long v2c_oracle_rsf_newton(const double *states, long n, double W,
                           double rtol, int maxit, const double *guess_logV,
                           double *out, int *iters);
/* features of the network, x[8] per state */
void v2c_oracle_rsf_features(const double *states, long n, long i, double *x);

/* ----- MLP 8->64->64->2 (tanh) in FP64, for gradient checks -------------- */
/* params packed as in v2c.h; X[n][8] raw features, Y[n][2] raw targets.
 * Returns the mean-squared loss on normalised targets and, when grad != 0,
 * its gradient w.r.t. the first 64*8+64+64*64+64+2*64+2 parameters. */
double v2c_oracle_mlp_loss_grad(const float *params, const double *X,
                                const double *Y, long n, double *grad);
void v2c_oracle_mlp_forward(const float *params, const double *X, long n,
                            double *Y);

#ifdef __cplusplus
}
#endif
#endif
