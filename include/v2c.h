/*
 * v2c.h -- C ABI of the GB300 marker-in-cell (MIC) step of VELO2CYCLEs.
 *
 * The reference program (src/i2evps.c) calls four routines per time step
 * with no arguments; they read and write fixed-size global arrays declared in
 * src/headevps.c and src/input_RSF.c:
 *
 *   marker2nodes()                  src/interpolation.c:55-926
 *   interpolate_center2basic_old()  src/interpolation.c:1575-1598
 *   nodes2markers()                 src/interpolation.c:929-1048
 *   moveandrotatemarkers()          src/moveandrotatemarkers.c:1-178
 *
 * plus the node loops compute_before_solve / compute_after_solve
 * (src/plastic.c:2-129) inside the Stokes Picard loop.
 *
 * This header replaces that global-array seam with explicit handles:
 * a context owns the device copies of the grid, the rock table, the marker
 * arrays and the node arrays.  Arrays cross the boundary as plain host
 * pointers in the reference's own layout (FP64, node index m3 = m1*ynumy+m2,
 * y fastest; markers indexed by the reference marker number).  Every entry
 * point returns an int status (V2C_OK = 0).  A context is single-stream and
 * not thread-safe; contexts are independent.
 */
#ifndef V2C_H
#define V2C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum {
  V2C_OK = 0,
  V2C_ERR_ARG = 1,          /* bad argument (null pointer, size mismatch)        */
  V2C_ERR_CAPACITY = 2,     /* more markers/nodes than the context was made for  */
  V2C_ERR_CUDA = 3,         /* a CUDA runtime call failed                        */
  V2C_ERR_UNSUPPORTED = 4,  /* configuration outside what the kernels implement  */
  V2C_ERR_NAN = 5,          /* NaN / non-positive viscosity detected (errcheck)  */
  V2C_ERR_NOCONV = 6,       /* per-marker Newton did not converge for some marker */
  V2C_ERR_STATE = 7,        /* call order violated (e.g. no markers uploaded)     */
  V2C_ERR_TIMESTEP = 8      /* chi == 0 in the adaptive time step (the reference
                               stops there, calc_RSF.c:477-481)                */
};

#define V2C_MAXTMR 200 /* rock types, src/headevps.c:15 */

/* ------------------------------------------------------------------ params
 * Scalars and flags the reference keeps as globals.  Defaults in brackets are
 * the shipped configuration (src/mode_RSF.t3c, src/input_RSF.c:13-63). */
typedef struct v2c_params {
  long xnumx, ynumy;        /* grid lines            headevps.c:36            */
  double xsize, ysize;      /* model size, m         headevps.c:40            */
  double xstpx, ystpy;      /* mean grid steps       headevps.c:46            */
  double timesum;           /* time from start, s    headevps.c:446           */
  double timestep;          /* current dt, s         headevps.c:440           */
  int interpolationmod;     /* [2] 1: 13-node stencil, 2: 1-2|d| kernel     */
  int antidiffinter;        /* [1]                                           */
  int markmod;              /* [1] 1 Euler, 0/2 RK4 (2 also averages spin)    */
  int stoksmod;             /* [1] 1 rotation formula, 2 Jaumann              */
  int outgrid;              /* [2]                                           */
  int densimod;             /* [0]                                           */
  int RSFmode;              /* [1]                                           */
  int power_law_RSF;        /* [0]                                           */
  int rkmod;                /* [0] 0 Picard, 1 Lapusta average, 2 RK2, 3 RK4:
                                the slip rate compute_before_solve's pass rk
                                takes (calc_RSF.c:46-86)                    */
  int stickymod;            /* [1]                                           */
  int inertyn;              /* [0] radiation damping on                       */
  int pmode;                /* [0] normal stress = nstress                    */
  int tempmod;              /* [1] tkrecalc after the scatter                 */
  int compressiblemode;     /* [0]                                           */
  int reloadfromDP;         /* [0]                                           */
  double nubeg, nuend;      /* [1e1, 1.667e27] viscosity limits              */
  double nstress;           /* [10e6] effective normal stress, Pa            */
  double Dphis;             /* [0] state diffusion (ghost copy when > 0)     */
  double zdeep, tdeep;      /* markers coming from depth: T reset            */
  double eps2;              /* eps[2]: T given to newly incoming markers     */
  /* rate-and-state parameters, input_RSF.c:30-56 */
  double a_vw, b_vw, L_vw, V0_vw;
  double a_vs, b_vs, L_vs, V0_vs;
  double a_hr, b_hr, L_hr, V0_hr;
  double start_updip, end_updip, start_downdip, end_downdip, half_range;
  /* frictional band: |y - (fault_y + fault_slope*x)| <= fault_hw.  The
   * reference hard-codes fault_y=10e3, fault_hw=100, fault_slope=0
   * (calc_RSF.c:226-230); a non-zero slope gives a dipping megathrust. */
  double fault_y, fault_hw, fault_slope;
  /* per-marker visco-elasto-plastic + RSF Newton (no counterpart in the
   * reference; see v2c_rsf_newton) */
  double faultwidth;        /* [400] m, plastic.c:22                          */
  double newton_rtol;       /* [1e-10] relative residual                      */
  int newton_maxit;         /* [60]                                           */
  int newton_guess;         /* V2C_GUESS_*                                    */
  int newton_precision;     /* V2C_NEWTON_SPLIT [default] or V2C_NEWTON_FP64  */
} v2c_params;

/* initial-guess modes of the per-marker Newton */
enum { V2C_GUESS_PLAIN = 0, V2C_GUESS_LEARNED = 1, V2C_GUESS_OFF = 2 };
/* arithmetic of the per-marker Newton: SPLIT iterates in FP32 and finishes
 * with float-float residuals (FP64 only to form the converged residual and
 * as a fallback); FP64 runs every iteration in FP64.  Both stop at the same
 * relative residual newton_rtol. */
enum { V2C_NEWTON_SPLIT = 0, V2C_NEWTON_FP64 = 1 };

/* -------------------------------------------------------------- rock table
 * Per-type coefficients, each a double[V2C_MAXTMR] row, headevps.c:256-272. */
enum {
  V2C_RT_GG = 0, /* markgg shear modulus            */
  V2C_RT_NU,     /* marknu                          */
  V2C_RT_DH,     /* markdh activation energy        */
  V2C_RT_DV,     /* markdv activation volume        */
  V2C_RT_SS,     /* markss                          */
  V2C_RT_MM,     /* markmm power-law exponent       */
  V2C_RT_RO,     /* markro                          */
  V2C_RT_BB,     /* markbb                          */
  V2C_RT_AA,     /* markaa                          */
  V2C_RT_CP,     /* markcp                          */
  V2C_RT_KT,     /* markkt                          */
  V2C_RT_HT,     /* markht                          */
  V2C_RT_KF,     /* markkf                          */
  V2C_RT_KP,     /* markkp                          */
  V2C_RT_N0,     /* markn0 viscosity lower limit    */
  V2C_RT_N1,     /* markn1 viscosity upper limit    */
  V2C_RT_IM,     /* markim immobility flag (0/1)    */
  V2C_RT_N
};

/* ------------------------------------------------------------ marker fields
 * Same names as the reference arrays (headevps.c:209-248, input_RSF.c:11).
 * The rock type markt is a separate signed char array. */
enum {
  V2C_MF_X = 0, V2C_MF_Y, V2C_MF_K, V2C_MF_D, V2C_MF_E, V2C_MF_P, V2C_MF_W,
  V2C_MF_EXX, V2C_MF_EXY, V2C_MF_XX, V2C_MF_XY, V2C_MF_V, V2C_MF_VX, V2C_MF_VY,
  V2C_MF_C, V2C_MF_C0, V2C_MF_FRIC_STATIC, V2C_MF_PHI, V2C_MF_A, V2C_MF_B,
  V2C_MF_L, V2C_MF_L0, V2C_MF_V0,
  V2C_MF_SLIPV,  /* per-marker slip rate of the marker Newton (extension) */
  V2C_MF_N
};

/* -------------------------------------------------------------- node fields
 * Same names as the reference node arrays (headevps.c:99-190,
 * input_RSF.c:3-6).  Each is a double[nodenum]. */
enum {
  /* state carried between steps / solver outputs read by the MIC step */
  V2C_NF_PHIS_IT = 0, V2C_NF_PHIE, V2C_NF_SXY, V2C_NF_SXYEE, V2C_NF_EXY,
  V2C_NF_EXYEE, V2C_NF_PES, V2C_NF_PEE, V2C_NF_SXX, V2C_NF_SXXEE, V2C_NF_PR,
  V2C_NF_SPPEE, V2C_NF_EXX, V2C_NF_EXXEE, V2C_NF_VX, V2C_NF_MVXE, V2C_NF_VY,
  V2C_NF_MVYE, V2C_NF_ESP,
  /* marker2nodes outputs */
  V2C_NF_PHIN, V2C_NF_SXYEN, V2C_NF_EXYEN, V2C_NF_PEN, V2C_NF_PHIS,
  V2C_NF_SXYE, V2C_NF_EXYE, V2C_NF_PE, V2C_NF_MUS_S, V2C_NF_AS, V2C_NF_BS,
  V2C_NF_LS, V2C_NF_V0S, V2C_NF_COHESION, V2C_NF_NU_M2C, V2C_NF_GG,
  V2C_NF_SXXEN, V2C_NF_SPPEN, V2C_NF_EXXEN, V2C_NF_SXXE, V2C_NF_SPPE,
  V2C_NF_EXXE, V2C_NF_ND_M2C, V2C_NF_GD, V2C_NF_BM, V2C_NF_DRO, V2C_NF_DRP,
  V2C_NF_MVXN, V2C_NF_MVX, V2C_NF_MRX, V2C_NF_MVYN, V2C_NF_MVY, V2C_NF_MRY,
  V2C_NF_RO, V2C_NF_ET, V2C_NF_HT, V2C_NF_KT, V2C_NF_CP, V2C_NF_TK,
  V2C_NF_STICKY01, V2C_NF_NU, V2C_NF_ND,
  /* interpolate_center2basic_old outputs */
  V2C_NF_EXXES, V2C_NF_SXXES, V2C_NF_SPPES,
  /* node RSF update (plastic.c) */
  V2C_NF_SXXS, V2C_NF_RK_SLIPRS_FINAL, V2C_NF_RK_PHIDTS_FINAL,
  V2C_NF_RK_SLIPRS_SOLVED, V2C_NF_RK_PHIDTS_SOLVED, V2C_NF_SYIELDS,
  V2C_NF_NUVP_IT, V2C_NF_SLIPRS, V2C_NF_EXXPL, V2C_NF_RK_DELTAS,
  /* nodes2markers back-scatter sums and outputs */
  V2C_NF_PHISUM, V2C_NF_WTPHISUM, V2C_NF_SXYSUM, V2C_NF_EXYSUM, V2C_NF_ESUM,
  V2C_NF_PSUM, V2C_NF_SXXSUM, V2C_NF_EXXSUM, V2C_NF_WTSXXSUM, V2C_NF_VXSUM,
  V2C_NF_VYSUM, V2C_NF_WTVXSUM, V2C_NF_WTVYSUM, V2C_NF_MRX0, V2C_NF_MRY0,
  /* read by the adaptive time step (calc_RSF.c:455) */
  V2C_NF_PRS,
  /* interpolate_center2basic outputs (with SXXS, EXXPL, PRS above) */
  V2C_NF_EXXS, V2C_NF_EXXEL,
  /* sxx - sxxe of the step as recompute_stress_strainrate forms it
   * (2 nueff exx - Z sxxe, no cancellation); no reference array */
  V2C_NF_DSXX,
  /* node temperature before the thermal solve (solve_temperature saves it
   * as tk2, temperature_iterate.c:62) */
  V2C_NF_TK2,
  V2C_NF_N
};

/* ------------------------------------------------------------ status block */
typedef struct v2c_status {
  long n_markers;           /* markers held by the context                    */
  long n_out_of_grid;       /* markers outside the grid after the last move   */
  long n_far_moves;         /* markers that moved more than one cell          */
  long n_nan;               /* NaN / non-positive values caught (errcheck)     */
  long newton_iters;        /* total Newton iterations in the last solve      */
  long newton_fallbacks;    /* learned guesses rejected for the plain guess   */
  long newton_nonconv;      /* markers that did not reach the tolerance       */
  double newton_max_res;    /* largest relative residual after the last solve */
  long max_cell_count;      /* most markers in one cell after the last sort   */
  long kernel_launches;     /* device kernels launched by this context        */
  int last_error;           /* last non-zero status returned                   */
} v2c_status;

typedef struct v2c_ctx v2c_ctx;

/* ================================================================ life cycle
 * Replaces the static allocation of headevps.c:8-21 (MAXXLN/MAXYLN/MAXMRK):
 * capacities are fixed per context, max_markers below 2^30 (else
 * V2C_ERR_CAPACITY).  stream may be NULL (the per-thread default stream is
 * then not used; the context creates its own).  The context keeps its
 * markers sorted by cell and, within a cell, by quarter (u > 1/2, v > 1/2)
 * and array index; markers keep the reference numbering at the boundary. */
int v2c_create(const v2c_params *p, long max_markers, void *cuda_stream,
               v2c_ctx **out);
int v2c_destroy(v2c_ctx *ctx);
/* Re-read the scalar parameters (timesum, timestep, flags) before a call,
 * as the reference re-reads its globals on every call. */
int v2c_set_params(v2c_ctx *ctx, const v2c_params *p);

/* Grid lines gx[xnumx], gy[ynumy] (headevps.c:95); xsize == gx[xnumx-1]. */
int v2c_set_grid(v2c_ctx *ctx, const double *gx, const double *gy);
/* Rock table rows rt[V2C_RT_N][V2C_MAXTMR] (row-major). */
int v2c_set_rock_table(v2c_ctx *ctx, const double *rt);
/* Boundary-condition equations in the reference layout
 * (headevps.c:205-209): bondm[nodenum*4], bondn[bondnum][3],
 * bondv[bondnum][4].  Used by the boundary corrections that end
 * marker2nodes (momentum_continuity_addmatrix_checkerror.c:1002-1184,
 * temperature_iterate.c:828-891). */
int v2c_set_bonds(v2c_ctx *ctx, const long *bondm, const long *bondn,
                  const double *bondv, long bondnum);

/* =========================================================== marker arrays
 * fields[V2C_MF_N] are host pointers (any may be NULL = not transferred;
 * X, Y and markt are required on upload).  Markers keep the reference
 * numbering at the boundary; the device holds them sorted by cell. */
int v2c_upload_markers(v2c_ctx *ctx, const double *const *fields,
                       const signed char *markt, long n);
int v2c_download_markers(v2c_ctx *ctx, double *const *fields,
                         signed char *markt, long n);
/* Cell index of every marker (reference numbering) as found on the device:
 * ix*(ynumy-1)+iy with ix = nxsearch(x), iy = nysearch(y). */
int v2c_download_cells(v2c_ctx *ctx, int32_t *cell, long n);
/* The per-marker properties the last v2c_marker2nodes evaluated
 * (recalc_marker_properties.c:1-83): ductile viscosity mnu (ductilevisc,
 * density_ductilevisc_calc.c:29-223) and thermal conductivity mkt, n
 * doubles each in reference numbering (either pointer may be NULL).
 * Markers outside the model, which the reference skips, read 0.  Valid
 * from marker2nodes until the markers are uploaded or moved
 * (V2C_ERR_STATE otherwise); synchronous.  The reference keeps these as
 * locals of its marker loop (interpolation.c:229-240) and has no
 * accessor. */
int v2c_download_marker_properties(v2c_ctx *ctx, double *mnu, double *mkt, long n);

/* ============================================================= node arrays
 * One node field (V2C_NF_*) of nodenum doubles, converted to / from the
 * device's FP32.  The download returns when dst is filled.  The upload is
 * asynchronous on the context stream: from pinned host memory the copy runs
 * later, so src must stay unchanged until a call that synchronises the
 * stream (any download, v2c_synchronize).  The velocities VX and VY are also
 * kept in FP64 on the device (allocated at their first upload, 2 x nodenum
 * doubles): recompute_stress_strainrate forms strain rates from their
 * differences, which FP32 storage would round away. */
int v2c_upload_node_field(v2c_ctx *ctx, int field, const double *src);
int v2c_download_node_field(v2c_ctx *ctx, int field, double *dst);
/* count fields at once (fields[k] a V2C_NF_* id, src[k] / dst[k] nodenum
 * doubles each, count <= V2C_NF_N): one conversion kernel over all of them
 * and one copy per field back to back, one synchronisation at the end of
 * the download; the upload is asynchronous as above.  The first call with
 * more fields than any earlier one allocates a device staging area of
 * count x nodenum doubles (synchronising the stream).  No counterpart in
 * the reference, whose node arrays are host memory. */
int v2c_upload_node_fields(v2c_ctx *ctx, int count, const int *fields,
                           const double *const *src);
int v2c_download_node_fields(v2c_ctx *ctx, int count, const int *fields, double *const *dst);
/* The download above without waiting for it: the fields are converted on
 * the context stream after the work enqueued so far (a snapshot: later
 * calls may change them) and copied to dst on a transfer stream of the
 * context, so that the copies run under the kernels the caller enqueues
 * next.  dst (count arrays of nodenum doubles) must be pinned host memory
 * for the copies to overlap, and must not be read before
 * v2c_wait_downloads (or v2c_synchronize) returns.  A second asynchronous
 * download reuses the staging area (count x nodenum doubles, allocated at
 * the first call or when count grows, synchronising both streams) after
 * the first one's copies.  No counterpart in the reference, whose node
 * arrays are host memory. */
int v2c_download_node_fields_async(v2c_ctx *ctx, int count, const int *fields,
                                   double *const *dst);
int v2c_wait_downloads(v2c_ctx *ctx);

/* ======================================================= the MIC step calls
 * Reference equivalents in brackets.  All are asynchronous on the context
 * stream except where a status must be read back (noted). */
int v2c_marker2nodes(v2c_ctx *ctx);                 /* [interpolation.c:55]   */
int v2c_center2basic_old(v2c_ctx *ctx);             /* [interpolation.c:1575] */
/* interpolate_basic2center [interpolation.c:1639]: nd at the pressure nodes
 * (harmonic mean of nu); the Picard loop calls it after compute_before_solve
 * (momentum_continuity_iterate.c:71) */
int v2c_interpolate_basic2center(v2c_ctx *ctx);
/* interpolate_center2basic [interpolation.c:1600]: exxs, exxpl, sxxs, prs and
 * exxel on the basic nodes from the solver's pressure-node fields; called
 * before compute_after_solve (momentum_continuity_iterate.c:87) */
int v2c_interpolate_center2basic(v2c_ctx *ctx, double dt);
/* recompute_stress_strainrate [momentum_continuity_iterate.c:214]: exx, sxx
 * (pressure nodes) and exy, esp, sxy (basic nodes) from the node velocities
 * vx, vy with the visco-elastic update of sxxcalc / sxycalc; the reference
 * runs it after reloading the Stokes solution (:84) */
int v2c_recompute_stress_strainrate(v2c_ctx *ctx, double dt);
/* copyarrays [momentum_continuity_iterate.c:265]: RK_sliprs_final, sliprs
 * and RK_phidts_final from the solved rates, at the end of a step */
int v2c_copyarrays(v2c_ctx *ctx);
int v2c_compute_before_solve(v2c_ctx *ctx, double dt, int rk); /* [plastic.c:2] */
/* returns the RMS of (syield - sigin) in *deltas, [plastic.c:61] (syncs) */
int v2c_compute_after_solve(v2c_ctx *ctx, double dt, int rk, double *deltas);
int v2c_nodes2markers(v2c_ctx *ctx);                /* [interpolation.c:929]  */
int v2c_moveandrotatemarkers(v2c_ctx *ctx);         /* [moveandrotatemarkers.c:1] */
/* nodes2markers followed by moveandrotatemarkers in one marker pass. */
int v2c_nodes2markers_move(v2c_ctx *ctx);

/* ============================================== adaptive time step
 * calc_timestep (calc_RSF.c:352-572): the next time step from the node
 * fields, limited by the visco-plastic Maxwell time (tcnvp), the
 * displacement per step (tcd), the state evolution (tcphih) and the
 * Lapusta et al. (2000) slip length (lambda L / V), and the maximum slip
 * rate; oldornew = 0 before the Stokes solve (mvx/mvy, RK_sliprs_final,
 * phis, sppes), 1 inside the Picard loop (vx/vy, RK_sliprs_solved, phis_it,
 * prs).  Also returns the reference's diagnostic statistics of stress and
 * viscosity over sticky01 == 1 and == 2 nodes.  Synchronises the stream. */
typedef struct v2c_timestep_ctl {
  double maxtmstep;         /* maximum time step, s     headevps.c:339     */
  double dtfactor;          /* [1.0]                    input_RSF.c:17     */
  double tcnvp;             /* [0.2]                    input_RSF.c:18     */
  double tcd;               /* [1e-3]                   input_RSF.c:19     */
  double tcphih;            /* [0.2]                    input_RSF.c:20     */
} v2c_timestep_ctl;
typedef struct v2c_timestep_info {
  double dt_f, maxvel, maxVx, dtnvp, dtd, dtphi, dtL;
  long nr_0, nr_1;
  double max_sigin_0, min_sigin_0, sum_sigin_0, sum2_sigin_0;
  double max_visc_0, min_visc_0, sum_visc_0, sum2_visc_0;
  double max_sigin_1, min_sigin_1, sum_sigin_1, sum2_sigin_1;
  double max_visc_1, min_visc_1, sum_visc_1, sum2_visc_1;
  double sigin_P1, sigin_P2, visco_P1, visco_P2;
} v2c_timestep_info;
int v2c_calc_timestep(v2c_ctx *ctx, int oldornew, const v2c_timestep_ctl *ctl,
                      v2c_timestep_info *info);            /* [calc_RSF.c:352] */

/* ============================================================ restart files
 * The reference's binary restart format (.prn: load_model / save_model,
 * load_save.c:164-527, with the RSF extras of input_RSF.c:94-132), read and
 * written on the host (no GPU needed).  Arrays are the caller's, sized from
 * the info: rt[V2C_RT_N * V2C_MAXTMR] (the rock rows the path uses, markim
 * in V2C_RT_IM), rock_extra[V2C_PRN_ROCK_EXTRA * V2C_MAXTMR] (s0 s1 ll a0 a1
 * b0 b1 e0 e1 f0 f1, which the path does not read), node[V2C_NF_N] (each
 * nodenum doubles; the file holds sxxee sxx exxee exx sxyee sxy exyee exy
 * sppee pr phie phis_it mvxe vx mvye vy pes pee RK_sliprs_final
 * RK_phidts_final), bondm[4 * nodenum], gx[xnumx], gy[ynumy],
 * bondv[4 * bondnum], bondn[3 * bondnum] (equation 0 unused, as in the
 * reference), mark[V2C_MF_N] (each marknum doubles: x y k e xx v xy p exx
 * exy d w vx vy phi L L0 C C0), markt[marknum].  A NULL array is skipped
 * when reading and written as zeros. */
typedef struct v2c_prn_info {
  long xnumx, ynumy, mnumx, mnumy, marknum, bondnum;
  double xsize, ysize, pinit, pkf[4], timestep, timesum, gxkoef, gykoef;
  int rocknum, cycle;
  double timesave[5];
} v2c_prn_info;
#define V2C_PRN_ROCK_EXTRA 11
/* the header; V2C_ERR_UNSUPPORTED when the file's int/long/float/double
 * sizes differ from this machine's or its counts are out of range */
int v2c_prn_read_info(const char *path, v2c_prn_info *info);
/* the whole file into arrays sized from *info (from v2c_prn_read_info);
 * V2C_ERR_CAPACITY when the file's counts differ from *info,
 * V2C_ERR_UNSUPPORTED when bytes remain after the markers */
int v2c_prn_read(const char *path, v2c_prn_info *info, double *rt, double *rock_extra,
                 double *const *node, long *bondm, double *gx, double *gy, double *bondv,
                 long *bondn, double *const *mark, signed char *markt);
int v2c_prn_write(const char *path, const v2c_prn_info *info, const double *rt,
                  const double *rock_extra, const double *const *node, const long *bondm,
                  const double *gx, const double *gy, const double *bondv, const long *bondn,
                  const double *const *mark, const signed char *markt);

/* Marker part of solve_temperature [temperature_iterate.c:181-412], after
 * the host's thermal solve: node TK holds the solved temperature, TK2 the
 * one before it.  Fluid markers (type 50..99) take the interpolated solved
 * temperature; rock markers (type < 50) strictly inside the model start
 * from the old nodal temperature (at least tdeep) when their temperature is
 * not positive, get the subgrid diffusion towards the old nodal
 * temperature when heatdif > 0 (conductivity and rho*cp from the nodes kt,
 * ro, cp, over the step's timestep), the solution's change, and then lose
 * the node-averaged diffusion change again; the reference sums that
 * average at each marker's upper-left node only, here per cell in sorted
 * order (no float atomics). */
int v2c_marker_temperature(v2c_ctx *ctx, double heatdif);

/* ====================================================== Stokes assembly
 * preparematrix [momentum_continuity_addmatrix_checkerror.c:22-213] with
 * gausmat4_add [gausevps.c:137-214]: the continuity and x/y Stokes
 * equations of every node (ghost rows, boundary equations, the continuity
 * form of a vx/vy boundary, the drunken-sailor terms), as the CSR arrays
 * handed to Pardiso: row 3 m3 + 0 is node m3's pressure (continuity)
 * equation, + 1 its vx and + 2 its vy equation; ia[3 nodenum + 1] holds
 * 1-based row starts, ja[nnz] 1-based columns in increasing order within a
 * row, a[nnz] the coefficients (terms of one column summed in equation
 * order, zero terms and zero sums left out), b[3 nodenum] the right-hand
 * side.  Evaluated on the device in FP64 from the device's node fields
 * (nd, gd, sxxe, nu, gg, sxye, mrx, mvx, mry, mvy, ro; sppe and bm in
 * compressible mode) and the boundary equations of v2c_set_bonds; FP64
 * arithmetic in the reference's order, so the arrays equal the reference's
 * for the same node values.
 * Pass ja = a = NULL to only count: *nnz receives the number of
 * coefficients (ia and b are still filled when given).  Returns
 * V2C_ERR_CAPACITY (with *nnz set) when cap < nnz, V2C_ERR_STATE without
 * boundary equations, V2C_ERR_UNSUPPORTED where the reference stops
 * (an inconsistent continuity boundary, addvx/addvy) or where a Stokes or
 * continuity row would reach past the grid (an edge node without a
 * boundary equation). */
typedef struct v2c_stokes_ctl {
  double mukoef;        /* scale of continuity and boundary rows; the reference
                           uses dt*30e5 (momentum_continuity_iterate.c:64)  */
  double dt;            /* time step of the solve, s                        */
  double gxkoef, gykoef;/* gravity, m/s^2 (GXKOEF, GYKOEF, headevps.c:42)   */
  double timebond;      /* interior vx boundary equations apply until this
                           time, s (headevps.c:341)                          */
  int drunkensailor;    /* [1] free-surface stabilisation terms              */
} v2c_stokes_ctl;
int v2c_stokes_assemble(v2c_ctx *ctx, const v2c_stokes_ctl *ctl, long cap, int *ia, int *ja,
                        double *a, double *b, long *nnz);

/* ========================================================= seismic cycle
 * The seismic-cycle workload (no counterpart in the reference: it stands in
 * for the host Stokes solve with prescribed velocities).  Regime 0
 * (interseismic) and 1 (coseismic) each get a velocity field vx, vy
 * (nodenum doubles each); setting regime 0 also zeroes the accumulated
 * slip.  Synchronises. */
int v2c_cycle_set_velocity(v2c_ctx *ctx, int regime, const double *vx, const double *vy);
/* One step of timestep dt with regime r's velocities: marker2nodes,
 * interpolate_center2basic_old, compute_before_solve, interpolate_basic2center,
 * recompute_stress_strainrate, interpolate_center2basic, compute_after_solve
 * (no readback), copyarrays, the accumulated slip of every basic node
 * (+= dt * RK_sliprs_final) and of every marker (+= dt * the Newton's slip
 * rate), nodes2markers, moveandrotatemarkers and the next
 * counting sort; then timesum += dt.  Asynchronous.
 * use_graph: the step is captured once into a CUDA graph per key (regime,
 * dt, the position buffer holding the current positions, every parameter
 * but timesum, and timesum's classes: zero, positive, equal to dt, above
 * 4e7 s, which are all the kernels see of it) and replayed afterwards; at
 * most 8 graphs are kept (the oldest dropped).  The first step of a key
 * runs the capture (no profiling events there); a capture needs no
 * allocation, so it may run at any point after the context is set up. */
int v2c_cycle_step(v2c_ctx *ctx, int regime, double dt, int use_graph);
/* accumulated slip of every node (nodenum doubles).  Synchronises. */
int v2c_cycle_slip(v2c_ctx *ctx, double *out);
/* accumulated slip of every marker, the per-marker Newton's slip rate times
 * dt summed over the cycle steps (n doubles, reference numbering; zero
 * while the Newton is off).  Synchronises. */
int v2c_cycle_marker_slip(v2c_ctx *ctx, double *out, long n);

int v2c_synchronize(v2c_ctx *ctx);
int v2c_get_status(v2c_ctx *ctx, v2c_status *st);

/* Per-kernel timing (instrumentation, no counterpart in the reference): when
 * enabled, every launch group below is bracketed by CUDA events on the
 * context stream; v2c_get_profile synchronises and returns the summed
 * milliseconds and the number of timed launches of one group. */
enum {
  V2C_PROF_M2N = 0,     /* marker2nodes sweep                          */
  V2C_PROF_M2N_TAIL,    /* sticky flags, state ghosts, boundary rows   */
  V2C_PROF_C2B,         /* interpolate_center2basic_old                */
  V2C_PROF_BEFORE,      /* compute_before_solve                        */
  V2C_PROF_AFTER,       /* compute_after_solve                         */
  V2C_PROF_N2M,         /* nodes2markers: gather, update, back-scatter */
  V2C_PROF_SORT,        /* counting sort by cell                       */
  V2C_PROF_NEWTON,      /* marker physics with the per-marker Newton    */
  V2C_PROF_PHYS,        /* marker physics without the Newton            */
  V2C_PROF_MOVE,        /* moveandrotatemarkers                        */
  V2C_PROF_TIMESTEP,    /* calc_timestep                                */
  V2C_PROF_B2C,         /* basic2center, center2basic, recompute stress */
  V2C_PROF_TEMP,        /* marker temperature update                    */
  V2C_PROF_STOKES,      /* Stokes matrix assembly                       */
  V2C_PROF_N
};
int v2c_set_profiling(v2c_ctx *ctx, int on);
int v2c_get_profile(v2c_ctx *ctx, int group, double *ms, long *launches);

/* ================================================ per-marker VEP+RSF Newton
 * No counterpart in the reference (it resolves stress and slip rate only
 * through the global Picard loop, momentum_continuity_iterate.c:49-124).
 * Solves, per state i, for the slip rate V>0 that makes the Maxwell
 * visco-elasto-plastic stress equal the regularised RSF yield stress
 *   F(V) = 2 eta_vp Z edot + (1-Z) tau_old - tau_y(V) = 0,
 *   tau_y(V) = sn a asinh(V/(2V0) exp((mu0 + b phi(V))/a)) + 4.3303e6 V,
 *   phi(V)   = ageing-law update over dt           (calc_RSF.c:96-103),
 *   eta_vp   = eta tau_y /(2 eta V/W + tau_y)     (calc_RSF.c:142),
 *   Z        = G dt /(G dt + eta_vp).
 * States are device pointers of V2C_RS_N float64 columns of length n
 * (column-major, see V2C_RS_*).  Outputs: V, phi(V), tau_y(V), and the
 * Newton iteration count.  guess = V2C_GUESS_PLAIN starts from V_old,
 * V2C_GUESS_LEARNED from the network loaded with v2c_mlp_load and falls back
 * to the plain guess when the learned start does not converge. */
enum {
  V2C_RS_VOLD = 0, V2C_RS_PHIOLD, V2C_RS_A, V2C_RS_B, V2C_RS_L, V2C_RS_V0,
  V2C_RS_MU0, V2C_RS_SN, V2C_RS_DT, V2C_RS_TAUOLD, V2C_RS_EDOT, V2C_RS_ETA,
  V2C_RS_G, V2C_RS_N
};
enum { V2C_RO_V = 0, V2C_RO_PHI, V2C_RO_TAU, V2C_RO_RES, V2C_RO_N };

int v2c_rsf_newton(v2c_ctx *ctx, const double *states_dev, long n, int guess,
                   double *out_dev, int32_t *iters_dev);

/* The per-marker Newton problems the MIC step would solve now, for training
 * the start network on the running model: the state (layout as for
 * v2c_rsf_newton, states_dev[V2C_RS_N][cap]) of every stride-th marker in
 * the context's marker order, computed by the same physics pass as
 * v2c_marker2nodes but changing no marker or node.  A slot whose marker has
 * no problem (outside the model, sticky air, zero viscosity) holds NaN in
 * row V2C_RS_A.  *n_out = slots written = min(cap, ceil(n/stride)).  No
 * counterpart in the reference. */
int v2c_collect_newton_states(v2c_ctx *ctx, long stride, double *states_dev, long cap,
                              long *n_out);

/* Multilayer perceptron 8 -> 64 -> 64 -> 2 that proposes the Newton start.
 * Weights are one packed float32 vector (see V2C_MLP_NPARAM), layout
 * W1[64][8] b1[64] W2[64][64] b2[64] W3[2][64] b3[2] plus the feature
 * normalisation mean[8] std[8] and the output scale mean[2] std[2]. */
#define V2C_MLP_IN 8
#define V2C_MLP_H 64
#define V2C_MLP_OUT 2
#define V2C_MLP_NPARAM (64 * 8 + 64 + 64 * 64 + 64 + 2 * 64 + 2 + 8 + 8 + 2 + 2)
int v2c_mlp_load(v2c_ctx *ctx, const float *params_host);
int v2c_mlp_save(v2c_ctx *ctx, float *params_host);
/* Train on n states (device, as for v2c_rsf_newton) whose Newton solutions
 * are targets_dev[2][n] = (log V, phi).  Hand-written BF16 tensor-core
 * forward/backward + Adam; returns the final mean loss. */
int v2c_mlp_train(v2c_ctx *ctx, const double *states_dev,
                  const double *targets_dev, long n, int epochs, int batch,
                  float lr, uint64_t seed, float *final_loss);
/* Gradient of the training loss at the loaded parameters on n <= 131072
 * states, without updating: grad_host[V2C_MLP_NPARAM - 20] (the trainable
 * parameters, packed as above) and the loss.  For checking the backward
 * pass against an independent implementation. */
int v2c_mlp_grad(v2c_ctx *ctx, const double *states_dev,
                 const double *targets_dev, long n, float *grad_host, float *loss);
/* Network outputs for n states (device): out_dev[2][n] = (log V, phi). */
int v2c_mlp_infer(v2c_ctx *ctx, const double *states_dev, long n, float *out_dev);

/* ============================================ allocation-free cell sort
 * No counterpart in the reference (its marker loops never sort).  Computes,
 * for n markers at device positions x_dev[n], y_dev[n] on the device grid
 * lines gx_dev[xnumx], gy_dev[ynumy], the same cell index as the context
 * path (cell_dev[i] = nxsearch(x)*(ynumy-1) + nysearch(y), bit-exact) and a
 * stable counting sort by cell: perm_dev[start_dev[c] ..
 * start_dev[c+1]) lists the markers of cell c in ascending index, and
 * start_dev has (xnumx-1)*(ynumy-1)+1 entries.  All pointers are device
 * pointers; the work is queued on cuda_stream (a cudaStream_t, NULL for the
 * default stream) and the call returns without waiting for it.
 *
 * For callers that cannot let the library allocate: a host program whose
 * device memory is all handed out by its own pool, or one that cannot afford
 * the device-wide synchronisation that cudaMalloc/cudaFree bring, and that
 * needs markers ordered by cell without building a whole context (which
 * allocates some 40 per-marker arrays).  This call allocates no device or
 * host memory.  Its only scratch is a fixed array in the library's device
 * memory, 16 MiB + 4 KiB per device, that holds per-cell counters, so the
 * grid may have at most V2C_STATIC_SORT_MAX_CELLS cells: larger grids return
 * V2C_ERR_CAPACITY (with a message on stderr) before anything runs.  The
 * counters must be zero before they are used; each call zeroes them on its
 * own stream, so the caller zeroes nothing and the outputs need no initial
 * value.  The first call on a device looks up the scratch address (set-up,
 * done once per device with that device current); a caller that captures
 * streams makes that first call before it begins capturing.  There is one
 * scratch per device: calls that overlap on the same device (different
 * streams or host threads without ordering between them) race on it and give
 * wrong results, so order them.  Cost: each cell's segment is put in index
 * order by one warp, in registers up to 32 markers and by a bitonic network
 * in global memory above that, O(L log^2 L) for L markers in the cell; a
 * grid with markers piled into a few cells (for example all of them outside
 * the grid, clamped into a corner cell) is sorted far more slowly than one
 * with a few tens of markers per cell.  A CUDA error left pending by earlier
 * work makes the call return V2C_ERR_CUDA before it queues anything, leaving
 * that error in place. */
/* 4 Mi cells: a 4001 x 1001 line grid (4 000 000 cells) fits */
#define V2C_STATIC_SORT_MAX_CELLS 4194304
int v2c_sort_cells_static(const double *gx_dev, long xnumx, const double *gy_dev,
                          long ynumy, const double *x_dev, const double *y_dev, long n,
                          int32_t *cell_dev, int32_t *perm_dev, int32_t *start_dev,
                          void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* V2C_H */
