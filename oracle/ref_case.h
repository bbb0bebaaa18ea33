/*
 * ref_case.h -- loads a case file into the reference's global arrays and
 * writes its result file (formats: ref_harness.c).  TEST INFRASTRUCTURE
 * ONLY; included after the reference sources, the C-ABI header and
 * velo2cycles_gb300/bind/v2c_bind_map.h.
 */
#ifndef V2C_REF_CASE_H
#define V2C_REF_CASE_H

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

typedef struct {
  long xn, yn, n, nb, nn;
  int nthreads, stages, nsteps, warmup;
  double *scratch;
  double ts[6];            /* maxtmstep, dtfactor, tcnvp, tcd, tcphih, oldornew */
  long ndts;               /* per-step time steps (optional trailer), 0 if none */
  double *dts;
  double heatdif;          /* solve_temperature's subgrid diffusion (optional trailer) */
  double stokes[6];        /* preparematrix (stage bit 13, optional trailer): mukoef, dt,
                              GXKOEF, GYKOEF, timebond, drunkensailor */
  v2c_timestep_info info;  /* calc_timestep results (stage bit 6) */
  long ts_rc;              /* 0, or 1 when chi == 0 stopped it */
} ref_case;

/* returns 0, or the process exit code on failure */
static int ref_load_case(const char *path, ref_case *C) {
  FILE *f = fopen(path, "rb");
  if (!f) { perror(path); return 2; }
  char magic[8];
  rd(magic, 1, 8, f);
  if (memcmp(magic, "V2CCASE1", 8)) { fprintf(stderr, "bad case file\n"); return 2; }
  int64_t hdr[8];
  rd(hdr, sizeof(int64_t), 8, f);
  long xn = hdr[0], yn = hdr[1], n = hdr[2], nb = hdr[3];
  long nn = xn * yn;
  C->xn = xn; C->yn = yn; C->n = n; C->nb = nb; C->nn = nn;
  C->nthreads = (int)hdr[4]; C->stages = (int)hdr[5]; C->nsteps = (int)hdr[6];
  C->warmup = (int)hdr[7];
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
  /* a move can at most double the markers (one spawn per immobile one) */
  double *scratch = (double *)malloc(sizeof(double) * ((2 * n > nn ? 2 * n : nn) + 1));
  C->scratch = scratch;
  /* fields the reference has no array for are read into scratch */
  for (int k = 0; k < V2C_NF_N; k++) rd(node_array(k) ? node_array(k) : scratch, sizeof(double), nn, f);
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
  rd(C->ts, sizeof(double), 6, f);
  /* optional trailer: int64 ndts, double dts[ndts] */
  C->ndts = 0;
  C->dts = NULL;
  int64_t nd = 0;
  if (fread(&nd, sizeof(int64_t), 1, f) == 1 && nd > 0) {
    C->dts = (double *)malloc(sizeof(double) * nd);
    rd(C->dts, sizeof(double), nd, f);
    C->ndts = nd;
  }
  C->heatdif = 0;
  if (fread(&C->heatdif, sizeof(double), 1, f) != 1) C->heatdif = 0;
  memset(C->stokes, 0, sizeof(C->stokes));
  if (fread(C->stokes, sizeof(double), 6, f) != 6) memset(C->stokes, 0, sizeof(C->stokes));
  memset(&C->info, 0, sizeof(C->info));
  C->ts_rc = 0;
  fclose(f);
  marknum = n;
  return 0;
}

/* returns 0, or the process exit code on failure */
static int ref_write_result(const char *path, const ref_case *C, const double *secs,
                            double deltas) {
  long nn = C->nn;
  double *scratch = C->scratch;
  FILE *o = fopen(path, "wb");
  if (!o) { perror(path); return 2; }
  if (C->stages & (1 << 14)) {
    /* timing only: the seconds and the deltas, no arrays */
    wr("V2CSEC01", 1, 8, o);
    wr(secs, sizeof(double), 8, o);
    wr(&deltas, sizeof(double), 1, o);
    fclose(o);
    return 0;
  }
  wr("V2CRES01", 1, 8, o);
  int64_t nout = marknum;
  wr(&nout, sizeof(int64_t), 1, o);
  for (int k = 0; k < V2C_NF_N; k++) {
    if (node_array(k)) wr(node_array(k), sizeof(double), nn, o);
    else {
      memset(scratch, 0, sizeof(double) * nn);
      wr(scratch, sizeof(double), nn, o);
    }
  }
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
  wr(&C->ts_rc, sizeof(long), 1, o);
  wr(&C->info, sizeof(C->info), 1, o);
  fclose(o);
  return 0;
}

#endif
