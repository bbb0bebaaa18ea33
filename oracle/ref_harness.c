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
 *   interpolate_basic2center, recompute_stress_strainrate,
 *   interpolate_center2basic, copyarrays (stage bits 7, 9, 8, 10),
 *   compute_after_solve, nodes2markers, moveandrotatemarkers, calc_timestep
 * and writes the arrays back; with stage bit 12 it also runs save_model,
 * which writes the restart file state.prn into the working directory, and
 * with bit 13 preparematrix, whose CSR arrays go to stokes.bin there.
 * Stdout (the reference's progress prints) is discarded.
 *
 * Case file (native endianness), written by oracle/bindings.py:
 *   char magic[8] = "V2CCASE1"
 *   int64 xnumx, ynumy, n, bondnum, nthreads, stages, nsteps, warmup
 *   v2c_params
 *   double gx[xnumx], gy[ynumy], rt[V2C_RT_N][V2C_MAXTMR]
 *   double node[V2C_NF_N][nodenum], mark[V2C_MF_N][n]; int8 markt[n]
 *   int64 bondm[nodenum*4], bondn[bondnum*3]; double bondv[bondnum*4]
 *   double ts[6]; optional: int64 ndts, double dts[ndts] (per-step dt),
 *   double heatdif (stage bit 11: solve_temperature, new temperatures in tk2)
 *   double stokes[6] (stage bit 13: preparematrix's mukoef, dt and GXKOEF,
 *   GYKOEF, timebond, drunkensailor)
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
#include "momentum_continuity_iterate.c"
#include "temperature_iterate.c"
#include "plastic.c"
#include "recalc_marker_properties.c"
#include "load_save.c"

#include "../include/v2c.h"
#include "../velo2cycles_gb300/bind/v2c_bind_map.h"

#define node_array v2c_bind_node_array
#define marker_array v2c_bind_marker_array
#define rock_row v2c_bind_rock_row

#include "ref_case.h"

/* the reference's calc_timestep and the globals it leaves behind */
static void ref_timestep(ref_case *C, int oldornew) {
  v2c_timestep_info *o = &C->info;
  o->dt_f = calc_timestep(oldornew);
  o->maxvel = maxvel;
  o->maxVx = NAN; /* a local of calc_timestep */
  o->dtnvp = dtnvp; o->dtd = dtd; o->dtphi = dtphi; o->dtL = dtL;
  o->nr_0 = nr_0; o->nr_1 = nr_1;
  o->max_sigin_0 = max_sigin_0; o->min_sigin_0 = min_sigin_0;
  o->sum_sigin_0 = sum_sigin_0; o->sum2_sigin_0 = sum2_sigin_0;
  o->max_visc_0 = max_visc_0; o->min_visc_0 = min_visc_0;
  o->sum_visc_0 = sum_visc_0; o->sum2_visc_0 = sum2_visc_0;
  o->max_sigin_1 = max_sigin_1; o->min_sigin_1 = min_sigin_1;
  o->sum_sigin_1 = sum_sigin_1; o->sum2_sigin_1 = sum2_sigin_1;
  o->max_visc_1 = max_visc_1; o->min_visc_1 = min_visc_1;
  o->sum_visc_1 = sum_visc_1; o->sum2_visc_1 = sum2_visc_1;
  o->sigin_P1 = sigin_P1; o->sigin_P2 = sigin_P2;
  o->visco_P1 = visco_P1; o->visco_P2 = visco_P2;
}

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: v2c_ref case.bin result.bin\n"); return 2; }
  ref_case C;
  int rc = ref_load_case(argv[1], &C);
  if (rc) return rc;
  int nthreads = C.nthreads, stages = C.stages & 0xffff, nsteps = C.nsteps, warmup = C.warmup;
  /* stage bits 16-19: number of Picard passes of compute_before_solve /
   * compute_after_solve (0: one pass at rk = 0 with the other stages) */
  const int npass = (C.stages >> 16) & 0xf;
  omp_set_num_threads(nthreads > 0 ? nthreads : 1);
  if (!freopen("/dev/null", "w", stdout)) return 5;

  double secs[8] = {0};
  double deltas = 0;
  for (int step = 0; step < warmup + nsteps; step++) {
    double t0;
    int timed = step >= warmup;
    /* a per-step time step sequence: the step runs with dts[step] and
     * timesum advances after it, as in the reference's main loop */
    if (step < C.ndts) timestep = C.dts[step];
#define STAGE(bit, idx, call)                               \
  if (stages & (1 << bit)) {                                \
    t0 = omp_get_wtime();                                   \
    call;                                                   \
    if (timed) secs[idx] += omp_get_wtime() - t0;           \
  }
    STAGE(0, 0, marker2nodes());
    STAGE(1, 1, interpolate_center2basic_old(timestep));
    if (npass > 0) {
      /* Picard passes rk = 0 .. npass-1 of the node routines (the order of
       * momentum_continuity_iterate.c:67-91 without the Stokes solve): each
       * pass's compute_after_solve leaves the slip rate the next pass's
       * compute_before_solve takes (calc_RSF.c:58-86) */
      for (int rk = 0; rk < npass; rk++) {
        STAGE(2, 2, compute_before_solve(timestep, rk));
        STAGE(3, 3, deltas = compute_after_solve(timestep, rk));
      }
    } else {
    STAGE(2, 2, compute_before_solve(timestep, 0));
    STAGE(7, 7, interpolate_basic2center());
    STAGE(9, 7, recompute_stress_strainrate(timestep, 0));
    STAGE(8, 7, interpolate_center2basic(timestep));
    STAGE(3, 3, deltas = compute_after_solve(timestep, 0));
    }
    STAGE(10, 7, copyarrays(0));
    if (stages & (1 << 11)) {
      /* solve_temperature (temperature_iterate.c:2-412) with the solver
       * stubbed: the solution vector x holds the new temperatures (the case
       * passes them in tk2), so after the call tk holds them and tk2 the old
       * ones, and the marker part runs as in the reference */
      for (long m = 0; m < C.nn; m++) x[m] = tk2[m];
      heatdif = C.heatdif;
      maxtkstep = 1e30;  /* one thermal substep */
      t0 = omp_get_wtime();
      solve_temperature(0);
      if (timed) secs[7] += omp_get_wtime() - t0;
    }
    STAGE(4, 4, nodes2markers());
    STAGE(5, 5, moveandrotatemarkers());
    if (stages & (1 << 6)) {
      /* calc_timestep (calc_RSF.c:352): its controls are globals */
      maxtmstep = C.ts[0]; dtfactor = C.ts[1]; tcnvp = C.ts[2]; tcd = C.ts[3];
      tcphih = C.ts[4];
      t0 = omp_get_wtime();
      ref_timestep(&C, (int)C.ts[5]);
      if (timed) secs[6] += omp_get_wtime() - t0;
    }
#undef STAGE
    if (step < C.ndts) timesum += timestep;
  }

  if (stages & (1 << 13)) {
    /* preparematrix (momentum_continuity_addmatrix_checkerror.c:22-38) of
     * the state after the steps; the CSR arrays gausmat4_add leaves for
     * Pardiso go to stokes.bin in the working directory:
     * int64 rows, nnz; int32 ia[rows+1], ja[nnz]; double a[nnz], b[rows] */
    GXKOEF = C.stokes[2]; GYKOEF = C.stokes[3]; timebond = C.stokes[4];
    drunkensailor = (int)C.stokes[5];
    pos0cur = 0;
    const double t0s = omp_get_wtime();
    preparematrix(C.stokes[0], C.stokes[1], 0);
    const double ts = omp_get_wtime() - t0s;
    FILE *o = fopen("stokes.bin", "wb");
    if (!o) return 6;
    int64_t hdr[2] = {nodenum3, pos0cur};
    wr(hdr, sizeof(int64_t), 2, o);
    wr(ia, sizeof(int), nodenum3 + 1, o);
    wr(ja, sizeof(int), pos0cur, o);
    wr(a, sizeof(double), pos0cur, o);
    wr(b, sizeof(double), nodenum3, o);
    wr(&ts, sizeof(double), 1, o);
    fclose(o);
  }
  if (stages & (1 << 12)) {
    /* save_model (load_save.c:353-527) of the state after the steps, into
     * the working directory as state.prn (it also writes file.t3c and
     * file_hdf5.t3c there); the cycle number is the step count */
    rocknum = V2C_MAXTMR;
    strcpy(fl1out, "state.prn");
    save_model(0, warmup + nsteps, 0);
  }

  return ref_write_result(argv[2], &C, secs, deltas);
}
