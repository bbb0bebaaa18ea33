// v2c_stokes.cu -- the Stokes matrix of the staggered grid on the device:
// preparematrix (momentum_continuity_addmatrix_checkerror.c:22-213) with its
// equation builders and gausmat4_add's CSR layout (gausevps.c:137-214).
//
// One thread per equation (3 per node: pressure/continuity, vx, vy).  The
// thread builds the equation's term list in the reference's order (the
// same columns, coefficients and right-hand side), then forms the CSR row:
// columns in increasing order, the terms of one column summed in list order
// starting from zero, zero terms and zero sums left out.  Two passes: the
// first counts each row's coefficients (and writes the right-hand side), a
// scan turns counts into row starts, the second writes columns and values;
// when the caller gives room for the coefficients the first pass also keeps
// each row (at most 24 entries) and the second only moves it.
//
// FP64 throughout, in the reference's evaluation order, and this file is
// compiled without multiply-add contraction, so a coefficient is the
// correctly rounded result of the same operations the reference performs.
#include "v2c_kernels.h"

namespace v2c {

namespace {

// terms of one equation: continuity 5, Stokes 3 + 4 x 4 + 5 drunken sailor
constexpr int MAXT = STOKES_ROW_MAX;

enum { ERR_OUTSIDE = 1, ERR_BOUNDARY = 2 };

struct Eq {
  double c;  // right-hand side
  int n;
  long col[MAXT];
  double w[MAXT];
  __device__ __forceinline__ void add(long k, double v) {
    if (n < MAXT) {
      col[n] = k;
      w[n] = v;
    }
    n++;
  }
};

struct Ctx {
  const StokesArgs &a;
  long yn, xn, nn;
  __device__ double N(int f, long m) const { return (double)a.N.f(f)[m]; }
  __device__ double gx(long i) const { return a.g.gx[i]; }
  __device__ double gy(long j) const { return a.g.gy[j]; }
};

// nueffcalc (momentum_continuity_addmatrix_checkerror.c:380-393)
__device__ __forceinline__ double nueff_of(const StokesArgs &a, double nvp, double gge,
                                           double &Z) {
  Z = gge * a.dt / (gge * a.dt + nvp);
  double nueff = Z * nvp;
  if (nueff < a.nubeg) nueff = a.nubeg;
  return nueff;
}

// sxxcalc_prepare (:395-443): the normal-stress terms of node (m1, m2)
// scaled by yv
__device__ void sxx_terms(const Ctx &C, Eq &E, long m1, long m2, double yv) {
  const long yn = C.yn;
  const long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  const double se = C.N(V2C_NF_SXXE, v3);
  double Z;
  const double nueff = nueff_of(C.a, C.N(V2C_NF_ND, v3), C.N(V2C_NF_GD, v3), Z);
  const double dx = C.gx(m1) - C.gx(m1 - 1), dy = C.gy(m2) - C.gy(m2 - 1);
  E.add(v0 * 3 + 1, -yv * nueff / dx);
  E.add(v2 * 3 + 1, +yv * nueff / dx);
  E.add(v0 * 3 + 2, +yv * nueff / dy);
  E.add(v1 * 3 + 2, -yv * nueff / dy);
  E.c -= (1.0 - Z) * yv * se;
}

// sxycalc_prepare (:483-525): the shear-stress terms of node (m1, m2)
__device__ void sxy_terms(const Ctx &C, Eq &E, long m1, long m2, double yv) {
  const long yn = C.yn;
  const long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  const double se = C.N(V2C_NF_SXYE, v3);
  double Z;
  const double nueff = nueff_of(C.a, C.N(V2C_NF_NU, v3), C.N(V2C_NF_GG, v3), Z);
  const double ddy = C.gy(m2 + 1) - C.gy(m2 - 1), ddx = C.gx(m1 + 1) - C.gx(m1 - 1);
  E.add(v2 * 3 + 1, -yv * 2.0 * nueff / ddy);
  E.add(v3 * 3 + 1, +yv * 2.0 * nueff / ddy);
  E.add(v1 * 3 + 2, -yv * 2.0 * nueff / ddx);
  E.add(v3 * 3 + 2, +yv * 2.0 * nueff / ddx);
  E.c -= (1.0 - Z) * yv * se;
}

// contadd (:932-998): div v of the cell whose pressure node is (m1, m2)
__device__ void cont_eq(const Ctx &C, Eq &E, long m1, long m2) {
  const StokesArgs &a = C.a;
  const long yn = C.yn;
  const long v0 = (m1 - 1) * yn + (m2 - 1), v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  E.n = 0;
  E.c = a.compressible ? C.N(V2C_NF_SPPE, v3) / C.N(V2C_NF_BM, v3) / a.timestep : 0.0;
  const double dx = C.gx(m1) - C.gx(m1 - 1), dy = C.gy(m2) - C.gy(m2 - 1);
  E.add(v0 * 3 + 1, -1.0 / dx);
  E.add(v2 * 3 + 1, +1.0 / dx);
  E.add(v0 * 3 + 2, -1.0 / dy);
  E.add(v1 * 3 + 2, +1.0 / dy);
  if (a.compressible) E.add(v3 * 3 + 0, 1.0 / C.N(V2C_NF_BM, v3) / a.timestep);
}

// bondadd (:192-211): the boundary equation of unknown r
__device__ void bond_eq(const Ctx &C, Eq &E, long r, int &bad) {
  const StokesArgs &a = C.a;
  const long B = a.bondm[r];
  E.n = 0;
  E.c = a.bondv[B * 4 + 0];
  E.add(r, 1.0);
  for (int k = 0; k < 3; k++) {
    const long bn = a.bondn[B * 3 + k];
    if (bn) {
      if (bn - 1 < 0 || bn - 1 >= 3 * C.nn) bad |= ERR_BOUNDARY;
      E.add(bn - 1, -a.bondv[B * 4 + k + 1]);
    }
  }
}

// xstoksadd (:642-731): x momentum at vx node (m1, m2)
__device__ void xstokes_eq(const Ctx &C, Eq &E, long m1, long m2) {
  const StokesArgs &a = C.a;
  const long yn = C.yn;
  const long v0 = m1 * yn + m2, v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  const double xkf = (C.gx(m1 + 1) - C.gx(m1 - 1)) / 2.0, ykf = C.gy(m2 + 1) - C.gy(m2);
  const double mrx = C.N(V2C_NF_MRX, v0);
  E.n = 0;
  E.c = (-a.gxkoef - a.inertyn * C.N(V2C_NF_MVX, v0) / a.dt) * mrx;
  E.add(v1 * 3 + 0, +1.0 / xkf);
  E.add(v3 * 3 + 0, -1.0 / xkf);
  E.add(v0 * 3 + 1, -a.inertyn * mrx / a.dt);
  sxx_terms(C, E, m1, m2 + 1, -1.0 / xkf);
  sxx_terms(C, E, m1 + 1, m2 + 1, 1.0 / xkf);
  sxy_terms(C, E, m1, m2, -1.0 / ykf);
  sxy_terms(C, E, m1, m2 + 1, 1.0 / ykf);
  if (a.drunkensailor == 1) {
    const double dt = a.dt, G = a.gxkoef;
    const double ro0 = C.N(V2C_NF_RO, v0), ro1 = C.N(V2C_NF_RO, v1);
    const double ro2 = C.N(V2C_NF_RO, v2), ro3 = C.N(V2C_NF_RO, v3);
    const double rol0 = C.N(V2C_NF_RO, v0 - yn), rol1 = C.N(V2C_NF_RO, v1 - yn);
    const double dxx = C.gx(m1 + 1) - C.gx(m1 - 1), dyy = C.gy(m2 + 1) - C.gy(m2);
    const double fl = C.gx(m1) - C.gx(m1 - 1), fr = C.gx(m1 + 1) - C.gx(m1);
    E.add(v0 * 3 + 1, -dt / 2.0 * G * (ro2 + ro3 - rol0 - rol1) / dxx / 2.0);
    const double wl = -dt / 2.0 * G * fl / dxx / 2.0 * (ro1 - ro0) / dyy;
    E.add(v0 * 3 + 2, wl);
    E.add(v1 * 3 + 2, wl);
    const double wr = -dt / 2.0 * G * fr / dxx / 2.0 * (ro1 - ro0) / dyy;
    E.add((v0 - yn) * 3 + 2, wr);
    E.add((v1 - yn) * 3 + 2, wr);
  }
}

// ystoksadd (:794-877): y momentum at vy node (m1, m2)
__device__ void ystokes_eq(const Ctx &C, Eq &E, long m1, long m2) {
  const StokesArgs &a = C.a;
  const long yn = C.yn;
  const long v0 = m1 * yn + m2, v1 = v0 + 1, v2 = v0 + yn, v3 = v2 + 1;
  const double xkf = C.gx(m1 + 1) - C.gx(m1), ykf = (C.gy(m2 + 1) - C.gy(m2 - 1)) / 2.0;
  const double mry = C.N(V2C_NF_MRY, v0);
  E.n = 0;
  E.c = (-a.gykoef - a.inertyn * C.N(V2C_NF_MVY, v0) / a.dt) * mry;
  E.add(v2 * 3 + 0, +1.0 / ykf);
  E.add(v3 * 3 + 0, -1.0 / ykf);
  E.add(v0 * 3 + 2, -a.inertyn * mry / a.dt);
  sxx_terms(C, E, m1 + 1, m2, 1.0 / ykf);
  sxx_terms(C, E, m1 + 1, m2 + 1, -1.0 / ykf);
  sxy_terms(C, E, m1, m2, -1.0 / xkf);
  sxy_terms(C, E, m1 + 1, m2, 1.0 / xkf);
  if (a.drunkensailor == 1) {
    const double dt = a.dt, G = a.gykoef;
    const double ro0 = C.N(V2C_NF_RO, v0), ro1 = C.N(V2C_NF_RO, v1);
    const double ro2 = C.N(V2C_NF_RO, v2), ro3 = C.N(V2C_NF_RO, v3);
    const double rob0 = C.N(V2C_NF_RO, v0 - 1), rob2 = C.N(V2C_NF_RO, v2 - 1);
    const double dyy = C.gy(m2 + 1) - C.gy(m2 - 1), dxx = C.gx(m1 + 1) - C.gx(m1);
    const double fu = C.gy(m2) - C.gy(m2 - 1), fd = C.gy(m2 + 1) - C.gy(m2);
    E.add(v0 * 3 + 2, -dt / 2.0 * G * (ro1 + ro3 - rob0 - rob2) / dyy / 2.0);
    const double wu = -dt / 2.0 * G * fu / dyy / 2.0 * (ro2 - ro0) / dxx;
    E.add(v0 * 3 + 1, wu);
    E.add(v2 * 3 + 1, wu);
    const double wd = -dt / 2.0 * G * fd / dyy / 2.0 * (ro2 - ro0) / dxx;
    E.add((v0 - 1) * 3 + 1, wd);
    E.add((v2 - 1) * 3 + 1, wd);
  }
}

// a vx or vy boundary given as a continuity equation (addvx :92-108,
// addvy :150-166): the cell of the referenced pressure; the reference
// checks that the pressure unknown k below the referenced one (k = 2 for
// vx, 3 for vy) has a boundary equation
__device__ bool cont_boundary(const Ctx &C, Eq &E, long r, long m1, long m2, int k, int &bad) {
  const StokesArgs &a = C.a;
  const long B = a.bondm[r];
  const long ref = a.bondn[B * 3 + 0];
  const long d = (ref - 1 - r) / 3;  // C division: truncates toward zero
  long dm1 = 0, dm2 = 0;
  if (d >= C.yn) dm1 = 1;
  if (d == 1 || d > C.yn) dm2 = 1;
  const long chk = ref - k;
  if (d < 0 || d > C.yn + 1 || !(m1 + dm1) || !(m2 + dm2) || chk < 0 || chk >= 4 * C.nn ||
      !a.bondm[chk]) {
    bad |= ERR_BOUNDARY;
    return false;
  }
  if (m1 + dm1 > C.xn - 1 || m2 + dm2 > C.yn - 1) {
    bad |= ERR_OUTSIDE;
    return false;
  }
  cont_eq(C, E, m1 + dm1, m2 + dm2);
  return true;
}

// the equation of unknown r as preparematrix builds it; returns false (and
// an empty equation) where the reference stops or would leave the grid
__device__ bool build_eq(const Ctx &C, long r, Eq &E, int &bad) {
  const StokesArgs &a = C.a;
  const long m3 = r / 3, kind = r - m3 * 3;
  const long m2 = m3 % C.yn, m1 = m3 / C.yn;
  const long xn = C.xn, yn = C.yn;
  E.n = 0;
  E.c = 0.0;
  bool scaled = true;
  if (kind == 0) {  // addcont (:40-71)
    if (m1 && m2) {
      if (!a.bondm[r] || a.compressible == 1) cont_eq(C, E, m1, m2);
      else bond_eq(C, E, r, bad);
    } else {
      E.c = 0.0;
      E.add(r, 1.0);
    }
  } else if (kind == 1) {  // addvx (:73-129)
    if (m2 < yn - 1) {
      if (!a.bondm[r] ||
          (a.timesum > a.timebond && m1 > 2 && m2 > 2 && m1 < xn - 4 && m2 < yn - 3)) {
        if (m1 < 1 || m1 > xn - 2 || m2 < 1 || m2 > yn - 3) {
          bad |= ERR_OUTSIDE;
          E.n = 0;
          return false;
        }
        xstokes_eq(C, E, m1, m2);
        scaled = false;
      } else if (a.bondv[a.bondm[r] * 4 + 1] > 1e+30) {
        if (!cont_boundary(C, E, r, m1, m2, 2, bad)) {
          E.n = 0;
          return false;
        }
      } else {
        bond_eq(C, E, r, bad);
      }
    } else {
      E.add(r, 1.0);
    }
  } else {  // addvy (:131-190)
    if (m1 < xn - 1) {
      if (!a.bondm[r]) {
        if (m1 < 1 || m1 > xn - 3 || m2 < 1 || m2 > yn - 2) {
          bad |= ERR_OUTSIDE;
          E.n = 0;
          return false;
        }
        ystokes_eq(C, E, m1, m2);
        scaled = false;
      } else if (a.bondv[a.bondm[r] * 4 + 1] > 1e+30) {
        if (!cont_boundary(C, E, r, m1, m2, 3, bad)) {
          E.n = 0;
          return false;
        }
      } else {
        bond_eq(C, E, r, bad);
      }
    } else {
      E.add(r, 1.0);
    }
  }
  if (E.n > MAXT) {
    bad |= ERR_BOUNDARY;
    E.n = 0;
    return false;
  }
  // ghost rows carry the scale on their one coefficient (wi = mukoef);
  // boundary and continuity rows are scaled term by term, right side too
  if (scaled) {
    E.c *= a.mukoef;
    for (int i = 0; i < E.n; i++) E.w[i] *= a.mukoef;
  }
  return true;
}

// gausmat4_add's row: sort the nonzero terms by column (stable, so the
// terms of one column keep their order) and sum each column from zero
__device__ int form_row(Eq &E) {
  int m = 0;
  for (int i = 0; i < E.n; i++)
    if (E.w[i] != 0.0) {
      E.col[m] = E.col[i];
      E.w[m] = E.w[i];
      m++;
    }
  for (int i = 1; i < m; i++) {
    const long k = E.col[i];
    const double v = E.w[i];
    int j = i - 1;
    while (j >= 0 && E.col[j] > k) {
      E.col[j + 1] = E.col[j];
      E.w[j + 1] = E.w[j];
      j--;
    }
    E.col[j + 1] = k;
    E.w[j + 1] = v;
  }
  int out = 0;
  for (int i = 0; i < m;) {
    double s = 0.0;
    const long k = E.col[i];
    for (; i < m && E.col[i] == k; i++) s += E.w[i];
    if (s != 0.0) {
      E.col[out] = k;
      E.w[out] = s;
      out++;
    }
  }
  return out;
}

__global__ void k_stokes_count(StokesArgs a) {
  const long rows = 3 * a.g.nn;
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const Ctx C{a, a.g.yn, a.g.xn, a.g.nn};
  Eq E;
  int bad = 0;
  build_eq(C, r, E, bad);
  const int n = form_row(E);
  a.cnt[r] = n;
  if (a.b) a.b[r] = E.c;
  if (a.ell_col) {
    for (int i = 0; i < n; i++) {
      a.ell_col[r * MAXT + i] = (int32_t)(E.col[i] + 1);
      a.ell_val[r * MAXT + i] = E.w[i];
    }
  }
  if (bad) atomicOr(a.err, bad);
}

// the rows the count pass kept, moved to their CSR positions
__global__ void k_stokes_move(StokesArgs a) {
  const long rows = 3 * a.g.nn;
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const long s = a.cnt[r], n = a.cnt[r + 1] - s;
  for (int i = 0; i < n; i++) {
    a.ja[s + i] = a.ell_col[r * MAXT + i];
    a.a[s + i] = a.ell_val[r * MAXT + i];
  }
}

__global__ void k_stokes_fill(StokesArgs a) {
  const long rows = 3 * a.g.nn;
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const Ctx C{a, a.g.yn, a.g.xn, a.g.nn};
  Eq E;
  int bad = 0;
  build_eq(C, r, E, bad);
  const int n = form_row(E);
  const long s = a.cnt[r];
  for (int i = 0; i < n; i++) {
    a.ja[s + i] = (int32_t)(E.col[i] + 1);
    a.a[s + i] = E.w[i];
  }
}

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_stokes_count(const StokesArgs &a, cudaStream_t st) {
  const long rows = 3 * a.g.nn;
  if (rows > 0) k_stokes_count<<<nblk(rows, 128), 128, 0, st>>>(a);
}

void launch_stokes_fill(const StokesArgs &a, cudaStream_t st) {
  const long rows = 3 * a.g.nn;
  if (rows <= 0) return;
  if (a.ell_col) k_stokes_move<<<nblk(rows, 256), 256, 0, st>>>(a);
  else k_stokes_fill<<<nblk(rows, 128), 128, 0, st>>>(a);
}

}  // namespace v2c
