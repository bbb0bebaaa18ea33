// v2c_prn.cu -- the reference's binary restart format (.prn): load_model /
// save_model (load_save.c:164-527) with the RSF extras of input_RSF.c:94-132.
//
// Host code only.  Layout (native byte order, the sizes of int / long /
// float / double as one byte each first):
//   long xnumx, ynumy, mnumx, mnumy, marknum; double xsize, ysize, pinit,
//   pkf[4], timestep, timesum, GXKOEF, GYKOEF; int rocknum; long bondnum;
//   int cycle;
//   int markim[rocknum]; 27 rows of double[rocknum]: n0 n1 s0 s1 nu dh dv ss
//   mm gg ll a0 a1 b0 b1 e0 e1 f0 f1 ro bb aa cp kt kf kp ht;
//   per node: 19 doubles (sxxee sxx exxee exx sxyee sxy exyee exy sppee pr
//   phie phis_it mvxe vx mvye vy pes pee RK_sliprs_final), 4 longs (bondm of
//   vx, vy, p, T), 2 doubles (RK_sliprs_final, RK_phidts_final);
//   double gx[xnumx], gy[ynumy];
//   for bond 1 .. bondnum-1: 4 doubles bondv, 3 longs bondn;
//   double timesave[5];
//   per marker: 14 doubles (x y k e xx v xy p exx exy d w vx vy), 1 byte type,
//   5 doubles (phi L L0 C C0).
#include <stdio.h>
#include <string.h>

#include "../../include/v2c.h"

namespace {

// file order of the node doubles and the marker doubles
const int kNode19[19] = {V2C_NF_SXXEE, V2C_NF_SXX,   V2C_NF_EXXEE,  V2C_NF_EXX,
                         V2C_NF_SXYEE, V2C_NF_SXY,   V2C_NF_EXYEE,  V2C_NF_EXY,
                         V2C_NF_SPPEE, V2C_NF_PR,    V2C_NF_PHIE,   V2C_NF_PHIS_IT,
                         V2C_NF_MVXE,  V2C_NF_VX,    V2C_NF_MVYE,   V2C_NF_VY,
                         V2C_NF_PES,   V2C_NF_PEE,   V2C_NF_RK_SLIPRS_FINAL};
const int kNodeExtra[2] = {V2C_NF_RK_SLIPRS_FINAL, V2C_NF_RK_PHIDTS_FINAL};
const int kMark14[14] = {V2C_MF_X,   V2C_MF_Y, V2C_MF_K,   V2C_MF_E,   V2C_MF_XX,
                         V2C_MF_V,   V2C_MF_XY, V2C_MF_P,  V2C_MF_EXX, V2C_MF_EXY,
                         V2C_MF_D,   V2C_MF_W, V2C_MF_VX,  V2C_MF_VY};
const int kMarkExtra[5] = {V2C_MF_PHI, V2C_MF_L, V2C_MF_L0, V2C_MF_C, V2C_MF_C0};
// rock rows in file order: a table row, or -1 - k for the k-th extra row
const int kRock[27] = {V2C_RT_N0, V2C_RT_N1, -1, -2, V2C_RT_NU, V2C_RT_DH, V2C_RT_DV,
                       V2C_RT_SS, V2C_RT_MM, V2C_RT_GG, -3, -4, -5, -6, -7, -8, -9, -10,
                       -11, V2C_RT_RO, V2C_RT_BB, V2C_RT_AA, V2C_RT_CP, V2C_RT_KT,
                       V2C_RT_KF, V2C_RT_KP, V2C_RT_HT};

struct File {
  FILE *f;
  bool ok = true;
  bool rd(void *p, size_t sz, size_t n) {
    if (ok && n && fread(p, sz, n, f) != n) ok = false;
    return ok;
  }
  bool wr(const void *p, size_t sz, size_t n) {
    if (ok && n && fwrite(p, sz, n, f) != n) ok = false;
    return ok;
  }
};

int header(File &F, v2c_prn_info *h, bool write) {
  char sz[4] = {(char)sizeof(int), (char)sizeof(long), (char)sizeof(float), (char)sizeof(double)};
  if (write) {
    F.wr(sz, 1, 4);
  } else {
    char got[4];
    if (!F.rd(got, 1, 4)) return V2C_ERR_ARG;
    if (memcmp(got, sz, 4)) return V2C_ERR_UNSUPPORTED;
  }
  long *L[5] = {&h->xnumx, &h->ynumy, &h->mnumx, &h->mnumy, &h->marknum};
  double *D[11] = {&h->xsize, &h->ysize, &h->pinit, h->pkf, h->pkf + 1, h->pkf + 2, h->pkf + 3,
                   &h->timestep, &h->timesum, &h->gxkoef, &h->gykoef};
  for (long *p : L) write ? F.wr(p, sizeof(long), 1) : F.rd(p, sizeof(long), 1);
  for (int k = 0; k < 11; k++) write ? F.wr(D[k], sizeof(double), 1) : F.rd(D[k], sizeof(double), 1);
  if (write) {
    F.wr(&h->rocknum, sizeof(int), 1);
    F.wr(&h->bondnum, sizeof(long), 1);
    F.wr(&h->cycle, sizeof(int), 1);
  } else {
    F.rd(&h->rocknum, sizeof(int), 1);
    F.rd(&h->bondnum, sizeof(long), 1);
    F.rd(&h->cycle, sizeof(int), 1);
  }
  if (!F.ok) return V2C_ERR_ARG;
  if (h->xnumx < 2 || h->ynumy < 2 || h->marknum < 0 || h->bondnum < 0 || h->rocknum < 0 ||
      h->rocknum > V2C_MAXTMR)
    return V2C_ERR_UNSUPPORTED;
  return V2C_OK;
}

// the body after the header: read (write == false) into or write from the
// caller's arrays; a NULL field pointer skips (reads) or writes zeros
int body(File &F, v2c_prn_info *h, bool write, double *rt, double *rock_extra, double *const *node,
         long *bondm, double *gx, double *gy, double *bondv, long *bondn, double *const *mark,
         signed char *markt) {
  const long xn = h->xnumx, yn = h->ynumy, nn = xn * yn, nm = h->marknum, nb = h->bondnum;
  const int nr = h->rocknum;
  auto io_d = [&](double *p) {
    double z = 0;
    if (write) F.wr(p ? p : &z, sizeof(double), 1);
    else F.rd(p ? p : &z, sizeof(double), 1);
  };
  auto io_l = [&](long *p) {
    long z = 0;
    if (write) F.wr(p ? p : &z, sizeof(long), 1);
    else F.rd(p ? p : &z, sizeof(long), 1);
  };
  // rock types: markim (int) then the 27 double rows
  for (int t = 0; t < nr; t++) {
    int im = rt ? (int)rt[(long)V2C_RT_IM * V2C_MAXTMR + t] : 0;
    if (write) F.wr(&im, sizeof(int), 1);
    else if (F.rd(&im, sizeof(int), 1) && rt) rt[(long)V2C_RT_IM * V2C_MAXTMR + t] = im;
  }
  for (int r = 0; r < 27; r++)
    for (int t = 0; t < nr; t++) {
      double *p = nullptr;
      if (kRock[r] >= 0) p = rt ? rt + (long)kRock[r] * V2C_MAXTMR + t : nullptr;
      else p = rock_extra ? rock_extra + (long)(-1 - kRock[r]) * V2C_MAXTMR + t : nullptr;
      io_d(p);
    }
  // nodes
  for (long m = 0; m < nn && F.ok; m++) {
    for (int k : kNode19) io_d(node && node[k] ? node[k] + m : nullptr);
    io_l(bondm ? bondm + m * 3 + 0 : nullptr);
    io_l(bondm ? bondm + m * 3 + 1 : nullptr);
    io_l(bondm ? bondm + m * 3 + 2 : nullptr);
    io_l(bondm ? bondm + 3 * nn + m : nullptr);
    for (int k : kNodeExtra) io_d(node && node[k] ? node[k] + m : nullptr);
  }
  for (long i = 0; i < xn; i++) io_d(gx ? gx + i : nullptr);
  for (long j = 0; j < yn; j++) io_d(gy ? gy + j : nullptr);
  for (long b = 1; b < nb && F.ok; b++) {
    for (int k = 0; k < 4; k++) io_d(bondv ? bondv + b * 4 + k : nullptr);
    for (int k = 0; k < 3; k++) io_l(bondn ? bondn + b * 3 + k : nullptr);
  }
  for (int k = 0; k < 5; k++) io_d(h->timesave + k);
  // markers
  for (long i = 0; i < nm && F.ok; i++) {
    for (int k : kMark14) io_d(mark && mark[k] ? mark[k] + i : nullptr);
    signed char t = markt ? markt[i] : 0;
    if (write) F.wr(&t, 1, 1);
    else if (F.rd(&t, 1, 1) && markt) markt[i] = t;
    for (int k : kMarkExtra) io_d(mark && mark[k] ? mark[k] + i : nullptr);
  }
  return F.ok ? V2C_OK : V2C_ERR_ARG;
}

}  // namespace

extern "C" int v2c_prn_read_info(const char *path, v2c_prn_info *info) {
  if (!path || !info) return V2C_ERR_ARG;
  memset(info, 0, sizeof(*info));
  File F{fopen(path, "rb")};
  if (!F.f) return V2C_ERR_ARG;
  const int rc = header(F, info, false);
  fclose(F.f);
  return rc;
}

extern "C" int v2c_prn_read(const char *path, v2c_prn_info *info, double *rt, double *rock_extra,
                            double *const *node, long *bondm, double *gx, double *gy,
                            double *bondv, long *bondn, double *const *mark,
                            signed char *markt) {
  if (!path || !info) return V2C_ERR_ARG;
  File F{fopen(path, "rb")};
  if (!F.f) return V2C_ERR_ARG;
  v2c_prn_info h;
  memset(&h, 0, sizeof(h));
  int rc = header(F, &h, false);
  if (!rc && (h.xnumx != info->xnumx || h.ynumy != info->ynumy || h.marknum != info->marknum ||
              h.bondnum != info->bondnum || h.rocknum != info->rocknum))
    rc = V2C_ERR_CAPACITY;  // the arrays were sized for another file
  if (!rc) rc = body(F, &h, false, rt, rock_extra, node, bondm, gx, gy, bondv, bondn, mark, markt);
  if (!rc) {
    char extra;
    if (fread(&extra, 1, 1, F.f) == 1) rc = V2C_ERR_UNSUPPORTED;  // trailing bytes: other extras
  }
  if (!rc) *info = h;
  fclose(F.f);
  return rc;
}

extern "C" int v2c_prn_write(const char *path, const v2c_prn_info *info, const double *rt,
                             const double *rock_extra, const double *const *node,
                             const long *bondm, const double *gx, const double *gy,
                             const double *bondv, const long *bondn, const double *const *mark,
                             const signed char *markt) {
  if (!path || !info) return V2C_ERR_ARG;
  File F{fopen(path, "wb")};
  if (!F.f) return V2C_ERR_ARG;
  v2c_prn_info h = *info;
  int rc = header(F, &h, true);
  if (!rc)
    rc = body(F, &h, true, const_cast<double *>(rt), const_cast<double *>(rock_extra),
              const_cast<double *const *>(node), const_cast<long *>(bondm),
              const_cast<double *>(gx), const_cast<double *>(gy), const_cast<double *>(bondv),
              const_cast<long *>(bondn), const_cast<double *const *>(mark),
              const_cast<signed char *>(markt));
  if (fclose(F.f) != 0 && !rc) rc = V2C_ERR_ARG;
  return rc;
}
