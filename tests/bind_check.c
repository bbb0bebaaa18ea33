/*
 * Test program for velo2cycles_gb300/bind/v2c_bind.c (built and run by
 * tests/test_gpu_bind.py): loads a case file into the reference's globals,
 * runs one MIC step with the reference's own routines (interpolate_basic2center
 * and interpolate_center2basic between the node updates, as the Picard loop
 * calls them), writes the result,
 * restores the initial globals, runs the same step through the binding
 * (GPU) and writes that result.  With two more paths it also assembles the
 * Stokes matrix after interpolate_basic2center (preparematrix, its scalars
 * from the case's stokes trailer) on both sides and writes the CSR arrays
 * (int64 rows, nnz; int32 ia, ja; double a, b).
 *   bind_check <case.bin> <ref_result.bin> <bind_result.bin> [ref.csr bind.csr]
 * Compiled against the reference sources staged by oracle/build_ref.sh.
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

#include "v2c.h"
#include "v2c_bind_map.h"
#include "v2c_bind.c"

#define node_array v2c_bind_node_array
#define marker_array v2c_bind_marker_array
#define rock_row v2c_bind_rock_row
#include "../oracle/ref_case.h"

static double *save_arrays(long nn, long n) {
  double *s = (double *)malloc(sizeof(double) * (V2C_NF_N * nn + V2C_MF_N * (n + 1)) + n + 1);
  double *p = s;
  for (int k = 0; k < V2C_NF_N; k++, p += nn)
    if (node_array(k)) memcpy(p, node_array(k), sizeof(double) * nn);
  for (int k = 0; k < V2C_MF_N; k++, p += n + 1)
    if (marker_array(k)) memcpy(p, marker_array(k), sizeof(double) * (n + 1));
  memcpy(p, markt, n + 1);
  return s;
}

static void restore_arrays(const double *s, long nn, long n) {
  const double *p = s;
  for (int k = 0; k < V2C_NF_N; k++, p += nn)
    if (node_array(k)) memcpy(node_array(k), p, sizeof(double) * nn);
  for (int k = 0; k < V2C_MF_N; k++, p += n + 1)
    if (marker_array(k)) memcpy(marker_array(k), p, sizeof(double) * (n + 1));
  memcpy(markt, p, n + 1);
}

static int write_csr(const char *path) {
  FILE *o = fopen(path, "wb");
  if (!o) return 2;
  int64_t hdr[2] = {nodenum3, pos0cur};
  wr(hdr, sizeof(int64_t), 2, o);
  wr(ia, sizeof(int), nodenum3 + 1, o);
  wr(ja, sizeof(int), pos0cur, o);
  wr(a, sizeof(double), pos0cur, o);
  wr(b, sizeof(double), nodenum3, o);
  fclose(o);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 4) { fprintf(stderr, "usage: bind_check case ref_out bind_out\n"); return 2; }
  ref_case C;
  int rc = ref_load_case(argv[1], &C);
  if (rc) return rc;
  omp_set_num_threads(1);
  double *init = save_arrays(C.nn, C.n);
  double secs[8] = {0};
  FILE *keep = stdout;
  if (!freopen("/dev/null", "w", stdout)) return 5;

  const int csr = argc >= 6;
  GXKOEF = C.stokes[2]; GYKOEF = C.stokes[3]; timebond = C.stokes[4];
  drunkensailor = (int)C.stokes[5];
  marker2nodes();
  interpolate_center2basic_old(timestep);
  compute_before_solve(timestep, 0);
  interpolate_basic2center();
  if (csr) {
    pos0cur = 0;
    preparematrix(C.stokes[0], C.stokes[1], 0);
    if (write_csr(argv[4])) return 2;
  }
  interpolate_center2basic(timestep);
  double d_ref = compute_after_solve(timestep, 0);
  nodes2markers();
  moveandrotatemarkers();
  rc = ref_write_result(argv[2], &C, secs, d_ref);
  if (rc) return rc;

  restore_arrays(init, C.nn, C.n);
  errcheck = 0;
  v2c_bind_marker2nodes();
  v2c_bind_interpolate_center2basic_old(timestep);
  v2c_bind_compute_before_solve(timestep, 0);
  v2c_bind_interpolate_basic2center();
  if (csr) {
    pos0cur = 0;
    v2c_bind_preparematrix(C.stokes[0], C.stokes[1], 0);
    if (write_csr(argv[5])) return 2;
  }
  v2c_bind_interpolate_center2basic(timestep);
  double d_bind = v2c_bind_compute_after_solve(timestep, 0);
  v2c_bind_nodes2markers();
  v2c_bind_moveandrotatemarkers();
  v2c_bind_markers_to_host();
  v2c_bind_close();
  (void)keep;
  if (errcheck != 0) { fprintf(stderr, "binding reported an error\n"); return 6; }
  return ref_write_result(argv[3], &C, secs, d_bind);
}
