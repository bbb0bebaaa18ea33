// v2c_m2n.cu -- marker2nodes (interpolation.c:55-926) as a deterministic
// segmented reduction over cell-sorted markers.
//
// Tiling.  A CTA owns node rows [j0, j0+TY) and node columns [i0, i0+TX).
// It sweeps cell columns ci = i0-1 .. i0+TX-1.  For each column it stages the
// column's markers of cell rows j0-1 .. j0+TY-1 (one contiguous run of the
// sorted order) in shared memory, evaluating every marker's properties once.
// Then thread (role, jl) accumulates, for node row j = j0+jl, the
// contributions of cells (ci, j-1) and (ci, j), which are all the cells of
// that column that reach node (ci, j) and (ci+1, j) under the
// interpolationmod=2 stencil (interpolation.c:539-628):
//   * basic node (ci, j) gets the left-half quadrants of those two cells,
//     basic node (ci+1, j) the right-half ones -> kept in a register carry
//     and completed when column ci+1 adds its left halves;
//   * vx node (ci, j) gets cell (ci, j) if u < 0.5, vx node (ci+1, j) if
//     u > 0.5 (carry);
//   * vy node (ci, j) gets cell (ci, j-1) if v > 0.5 and cell (ci, j) if
//     v < 0.5;
//   * the centre node (ci+1, j+1) gets cell (ci, j) only.
// The per-marker physics ran before, in marker order (v2c_phys.cu); staging
// only reads the marker fields and those results.
// Each node is summed by exactly one thread, in sorted-marker order, with
// FP32 two-sum compensation; the node tail (normalisation, antidiffusion
// correction, interpolation.c:714-824) runs in the same thread on the
// compensated sums, rounding each result once to FP32.
// No float atomics; the result does not depend on scheduling.
//
// Roles (one warp each per 32 node rows): 0 basic-node stress/state group,
// 1 basic-node thermal group, 2 centre node, 3 vx and vy nodes.
#include <math.h>

#include "v2c_ff.cuh"
#include "v2c_kernels.h"
#include "v2c_internal.cuh"

namespace v2c {

namespace {

constexpr int TY = 32;
constexpr int NTH = 4 * TY;
constexpr int CHUNK = 384;

enum {
  P_U = 0, P_V, P_NU, P_NUG, P_E, P_SXY, P_EXY, P_COH, P_PHI, P_RO, P_ET, P_HT,
  P_CP, P_KT, P_TK, P_SXX, P_EXX, P_P, P_VX, P_VY, P_N
};

// A chunk's markers are staged at their sorted position plus the local row
// of their cell (one free slot after each cell): the threads of consecutive
// node rows read consecutive cells in lockstep, and with the cells' runs
// at a spacing of count + 1 rather than count (16 or 20 markers per cell
// in a fresh uniform seeding) their shared-memory reads fall in different
// banks instead of a few.
constexpr int SKEW = TY + 1;
struct Smem {
  float p[P_N][CHUNK + SKEW];
  uint8_t act[CHUNK + SKEW];
};

// 4-byte asynchronous copy global -> shared (no register holds the value)
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Stage the chunk [cs, ce) of column ci's sorted markers, PER per thread,
// all of a thread's markers at once: the sort indices, then the cells and
// types, then every field by asynchronous copies straight into the
// marker's slot (three rounds of memory latency per chunk rather than
// three per marker, and no register holds a field).  Once a thread's own
// copies have landed, the payload formed from them: strictly inside the
// model (interpolation.c:219), the viscosity over the shear modulus, the
// dencalcomp adiabatic term and the rock-table constants.  The per-marker
// physics (viscosity, conductivity, density, state update) was done by the
// marker physics kernel.
constexpr int PER = CHUNK / NTH;
static_assert(PER * NTH == CHUNK, "chunk = whole staging rounds");
__device__ __forceinline__ void stage_chunk(const M2NArgs &a, Smem &sm, int cs, int ce, int ci,
                                            int jlo, int tid) {
  const Grid &g = a.g;
  int idx[PER], q[PER], t[PER];
#pragma unroll
  for (int j = 0; j < PER; j++) {
    const int s = cs + tid + j * NTH;
    idx[j] = s < ce ? __ldg(a.perm + s) : -1;
  }
#pragma unroll
  for (int j = 0; j < PER; j++) {
    q[j] = -1;
    if (idx[j] < 0) continue;
    // slot: the position in the chunk plus the skew of the cell's run (Smem)
    q[j] = tid + j * NTH + a.m.cell_in[idx[j]] - ci * g.ncy - jlo;
    t[j] = a.m.type[idx[j]];
  }
#pragma unroll
  for (int j = 0; j < PER; j++) {
    if (q[j] < 0) continue;
    const int i = idx[j], kk = q[j];
    cp_async4(&sm.p[P_U][kk], a.m.u_in + i);
    cp_async4(&sm.p[P_V][kk], a.m.v_in + i);
    cp_async4(&sm.p[P_NU][kk], a.m.mnu + i);
    cp_async4(&sm.p[P_E][kk], a.m.e + i);
    cp_async4(&sm.p[P_SXY][kk], a.m.sxy + i);
    cp_async4(&sm.p[P_EXY][kk], a.m.exy + i);
    cp_async4(&sm.p[P_COH][kk], a.m.coh + i);
    cp_async4(&sm.p[P_PHI][kk], a.m.phi + i);
    if (a.S.p.densimod) cp_async4(&sm.p[P_RO][kk], a.m.mro + i);
    cp_async4(&sm.p[P_KT][kk], a.m.mkt + i);
    cp_async4(&sm.p[P_TK][kk], a.m.tk + i);
    cp_async4(&sm.p[P_SXX][kk], a.m.sxx + i);
    cp_async4(&sm.p[P_EXX][kk], a.m.exx + i);
    cp_async4(&sm.p[P_P][kk], a.m.p + i);
    cp_async4(&sm.p[P_VX][kk], a.m.vx + i);
    cp_async4(&sm.p[P_VY][kk], a.m.vy + i);
  }
  cp_async_wait_all();
#pragma unroll
  for (int j = 0; j < PER; j++) {
    if (q[j] < 0) continue;
    const int k = q[j], tt = t[j];
    const int iy = jlo + k - (tid + j * NTH);
    const float u = sm.p[P_U][k], v = sm.p[P_V][k];
    bool act = true;
    if (ci == 0 || ci == g.ncx - 1) {
      double x = g.gx[ci] + (double)u * (g.gx[ci + 1] - g.gx[ci]);
      act = act && x > 0 && x < g.xsize;
    }
    if (iy == 0 || iy == g.ncy - 1) {
      double y = g.gy[iy] + (double)v * (g.gy[iy + 1] - g.gy[iy]);
      act = act && y > 0 && y < g.ysize;
    }
    sm.act[k] = act;
    const float bb = a.R(RK_BB, tt), T = sm.p[P_TK][k];
    sm.p[P_NUG][k] = sm.p[P_NU][k] * a.R(RK_INV_GG, tt);
    if (!a.S.p.densimod) sm.p[P_RO][k] = a.R(RK_RO, tt);
    sm.p[P_ET][k] = __fdividef(bb, 1.f - bb * (T - 298.15f));  // dencalcomp adiabatic term
    sm.p[P_HT][k] = a.R(RK_HT, tt);
    sm.p[P_CP][k] = a.R(RK_CP, tt);
  }
}

// calc_frictionpara_nodes (calc_RSF.c:298-350), FP64; out of line, taken
// only for nodes within 1 m of the frictional band (see node_friction)
__device__ __noinline__ void friction_node(const v2c_params &p, double x, double y, double &mu,
                                           double &a, double &b, double &L, double &V0) {
  double d = y - (p.fault_y + p.fault_slope * x);
  double radius = d >= 0 ? d : -d;
  if (radius <= p.fault_hw) {
    if (x > p.end_updip && x < p.start_downdip) {
      a = p.a_vw; b = p.b_vw; L = p.L_vw; V0 = p.V0_vw;
    } else if (x >= p.start_updip && x <= p.end_updip && p.half_range > 0) {
      double f = (x - (p.start_updip)) / (2 * p.half_range);
      a = p.a_vs + f * (p.a_vw - p.a_vs); b = p.b_vs + f * (p.b_vw - p.b_vs);
      L = p.L_vs + f * (p.L_vw - p.L_vs); V0 = p.V0_vs + f * (p.V0_vw - p.V0_vs);
    } else if (x >= p.start_downdip && x < p.end_downdip && p.half_range > 0) {
      double f = (x - (p.start_downdip)) / (2 * p.half_range);
      a = p.a_vw - f * (p.a_vw - p.a_vs); b = p.b_vw - f * (p.b_vw - p.b_vs);
      L = p.L_vw - f * (p.L_vw - p.L_vs); V0 = p.V0_vw - f * (p.V0_vw - p.V0_vs);
    } else {
      a = p.a_vs; b = p.b_vs; L = p.L_vs; V0 = p.V0_vs;
    }
    mu = 0.2;
  } else {
    mu = 0.6; a = p.a_hr; b = p.b_hr; L = p.L_hr; V0 = p.V0_hr;
  }
}

// Friction parameters of node (ci, j): outside the band (the FP32 distance
// clears the half-width by more than 1 m, far above its rounding) they are
// the constants of the far field; near the band the FP64 rule decides.
__device__ __forceinline__ void node_friction(const M2NArgs &a, int ci, int j, float &mu,
                                              float &fa, float &fb, float &fL, float &fV0) {
  const v2c_params &p = a.S.p;
  const Scal &S = a.S;
  const float xf = __ldg(a.gxf + ci), yf = __ldg(a.gyf + j);
  const float rad = fabsf(yf - (S.fault_y_f + S.fault_slope_f * xf));
  if (rad > S.fault_hw1_f) {
    mu = 0.6f; fa = S.a_hr_f; fb = S.b_hr_f; fL = S.L_hr_f; fV0 = S.V0_hr_f;
    return;
  }
  double dmu, da, db, dL, dV0;
  friction_node(p, a.g.gx[ci], a.g.gy[j], dmu, da, db, dL, dV0);
  mu = (float)dmu; fa = (float)da; fb = (float)db; fL = (float)dL; fV0 = (float)dV0;
}

// role 0 / role 1 accumulation into a named register array
#define ADD_BASIC_A(A, q, w)                                          \
  do {                                                                \
    A[0].add(sm.p[P_NU][q] * (w)); A[1].add(sm.p[P_NUG][q] * (w));    \
    A[2].add(sm.p[P_E][q] * (w)); A[3].add(sm.p[P_SXY][q] * (w));     \
    A[4].add(sm.p[P_EXY][q] * (w)); A[5].add(sm.p[P_COH][q] * (w));   \
    A[6].add(sm.p[P_PHI][q] * (w)); A[7].add(w);                      \
  } while (0)
#define ADD_BASIC_B(A, q, w)                                          \
  do {                                                                \
    A[0].add(sm.p[P_RO][q] * (w)); A[1].add(sm.p[P_ET][q] * (w));     \
    A[2].add(sm.p[P_HT][q] * (w)); A[3].add(sm.p[P_CP][q] * (w));     \
    A[4].add(sm.p[P_KT][q] * (w)); A[5].add(sm.p[P_TK][q] * (w));     \
    A[6].add(w);                                                      \
  } while (0)

// A compensated sum as a float pair.
__device__ __forceinline__ ff acc_ff(const Acc &a) {
  ff r;
  r.hi = two_sum(a.s, a.c, r.lo);
  return r;
}
// num / den of two compensated sums, rounded once
__device__ __forceinline__ float ratio(const Acc &num, const ff &den) {
  return ff_round(ff_div_fast(acc_ff(num), den));
}
// the antidiffusion form cur + (n - prev) (interpolation.c:730-736, 758-763,
// 784-806) from the float-pair node average n: cur and prev are consecutive
// states of one field that agree in their leading digits, so cur - prev is
// formed exactly and the sum is rounded once.
__device__ __forceinline__ float antid_rn(const ff &n, float cur, float prev) {
  return ff_round(ff_add(n, ff_diff(cur, prev)));
}

// The node tail of marker2nodes (interpolation.c:714-824) for node row j
// of column ci, from the compensated sums of one role: 0 basic node (ci, j)
// stress/state group (cur[0..7]: nu, nu/G, e, sxy, exy, C, phi, w), 1 its
// thermal group (cur[0..6]: ro, et, ht, cp, kt, tk, w), 2 the centre node
// (ci+1, j+1) of cell (ci, j) (cur[0..5]: nu, nu/G, sxx, exx, p, w) and the
// centre fields of (ci, j) when no cell feeds it, 3 vx node (ci, j)
// (cur[0..2]: vx*ro, ro, w) and vy node (ci, j) (vy3[0..2]).  The averages
// are float-pair quotients of the float-pair sums, rounded once to FP32.
__device__ __forceinline__ void node_tail(const M2NArgs &a, int role, int ci, int j,
                                          const Acc (&cur)[8], const Acc (&vy3)[3]) {
  const Grid &g = a.g;
  const int ncy = g.ncy;
  const long m3 = (long)ci * g.yn + j;
  const Nodes &N = a.N;
  const int antid = a.S.antid;
  if (role == 0) {
    const ff ssf = acc_ff(cur[7]);
    const float ss = ff_round(ssf);
    const bool interior = ci >= 1 && j >= 1 && ci < g.xn - 1 && j < g.yn - 1;
    if (ss != 0.f && interior) {
      const ff phin = ff_div_fast(acc_ff(cur[6]), ssf), sxyen = ff_div_fast(acc_ff(cur[3]), ssf);
      const ff exyen = ff_div_fast(acc_ff(cur[4]), ssf), pen = ff_div_fast(acc_ff(cur[2]), ssf);
      float phis, sxye, exye, pe;
      if (antid) {
        phis = antid_rn(phin, N.f(V2C_NF_PHIS_IT)[m3], N.f(V2C_NF_PHIE)[m3]);
        sxye = antid_rn(sxyen, N.f(V2C_NF_SXY)[m3], N.f(V2C_NF_SXYEE)[m3]);
        exye = antid_rn(exyen, N.f(V2C_NF_EXY)[m3], N.f(V2C_NF_EXYEE)[m3]);
        pe = antid_rn(pen, N.f(V2C_NF_PES)[m3], N.f(V2C_NF_PEE)[m3]);
      } else {
        phis = ff_round(phin); sxye = ff_round(sxyen); exye = ff_round(exyen); pe = ff_round(pen);
      }
      if (pe < 0.f) pe = 0.f;
      N.f(V2C_NF_PHIN)[m3] = ff_round(phin);
      N.f(V2C_NF_SXYEN)[m3] = ff_round(sxyen);
      N.f(V2C_NF_EXYEN)[m3] = ff_round(exyen);
      N.f(V2C_NF_PEN)[m3] = ff_round(pen);
      N.f(V2C_NF_PHIS)[m3] = phis;
      N.f(V2C_NF_SXYE)[m3] = sxye;
      N.f(V2C_NF_EXYE)[m3] = exye;
      N.f(V2C_NF_PE)[m3] = pe;
      N.f(V2C_NF_COHESION)[m3] = ratio(cur[5], ssf);
      N.f(V2C_NF_NU_M2C)[m3] = ratio(cur[0], ssf);
      // nu_m2c / (sum nu/G w / sum w) = sum nu w / sum nu/G w
      N.f(V2C_NF_GG)[m3] = ratio(cur[0], acc_ff(cur[1]));
    } else {
      N.f(V2C_NF_PHIN)[m3] = 0; N.f(V2C_NF_SXYEN)[m3] = 0; N.f(V2C_NF_EXYEN)[m3] = 0;
      N.f(V2C_NF_PHIS)[m3] = 0; N.f(V2C_NF_SXYE)[m3] = 0; N.f(V2C_NF_EXYE)[m3] = 0;
      N.f(V2C_NF_COHESION)[m3] = 0; N.f(V2C_NF_GG)[m3] = 0;
    }
  } else if (role == 1) {
    const ff ssf = acc_ff(cur[6]);
    const float ss = ff_round(ssf);
    const bool interior = ci >= 1 && j >= 1 && ci < g.xn - 1 && j < g.yn - 1;
    float mu = 0.f, fa = 0.f, fb = 0.f, fL = 0.f, fV0 = 0.f;
    if (ss != 0.f && interior) node_friction(a, ci, j, mu, fa, fb, fL, fV0);
    N.f(V2C_NF_MUS_S)[m3] = mu; N.f(V2C_NF_AS)[m3] = fa; N.f(V2C_NF_BS)[m3] = fb;
    N.f(V2C_NF_LS)[m3] = fL; N.f(V2C_NF_V0S)[m3] = fV0;
    if (ss != 0.f) {
      N.f(V2C_NF_RO)[m3] = ratio(cur[0], ssf); N.f(V2C_NF_ET)[m3] = ratio(cur[1], ssf);
      N.f(V2C_NF_HT)[m3] = ratio(cur[2], ssf); N.f(V2C_NF_CP)[m3] = ratio(cur[3], ssf);
      N.f(V2C_NF_KT)[m3] = ratio(cur[4], ssf); N.f(V2C_NF_TK)[m3] = ratio(cur[5], ssf);
    } else {
      N.f(V2C_NF_RO)[m3] = 0; N.f(V2C_NF_ET)[m3] = 0; N.f(V2C_NF_HT)[m3] = 0;
      N.f(V2C_NF_CP)[m3] = 0; N.f(V2C_NF_KT)[m3] = 0; N.f(V2C_NF_TK)[m3] = 0;
    }
    // arrays the reference zeroes at the start (interpolation.c:58-153)
    // and that marker2nodes itself does not fill
    static const int zl[] = {V2C_NF_NU, V2C_NF_ND, V2C_NF_WTPHISUM, V2C_NF_WTSXXSUM,
                             V2C_NF_WTVXSUM, V2C_NF_WTVYSUM, V2C_NF_PHISUM, V2C_NF_SXYSUM,
                             V2C_NF_EXYSUM, V2C_NF_ESUM, V2C_NF_SXXSUM, V2C_NF_EXXSUM,
                             V2C_NF_VXSUM, V2C_NF_VYSUM, V2C_NF_PSUM, V2C_NF_MRX0,
                             V2C_NF_MRY0};
#pragma unroll
    for (int q = 0; q < (int)(sizeof(zl) / sizeof(zl[0])); q++) N.f(zl[q])[m3] = 0;
  } else if (role == 2) {
    // centre node (ci+1, j+1) from cell (ci, j)
    if (ci < g.ncx && j < ncy) {
      const long mc = (long)(ci + 1) * g.yn + (j + 1);
      const ff s1f = acc_ff(cur[5]);
      const float s1 = ff_round(s1f);
      if (s1 != 0.f) {
        const ff sxxen = ff_div_fast(acc_ff(cur[2]), s1f), sppen = ff_div_fast(acc_ff(cur[4]), s1f);
        const ff exxen = ff_div_fast(acc_ff(cur[3]), s1f);
        float sxxe, sppe, exxe;
        if (antid) {
          sxxe = antid_rn(sxxen, N.f(V2C_NF_SXX)[mc], N.f(V2C_NF_SXXEE)[mc]);
          sppe = antid_rn(sppen, N.f(V2C_NF_PR)[mc], N.f(V2C_NF_SPPEE)[mc]);
          exxe = antid_rn(exxen, N.f(V2C_NF_EXX)[mc], N.f(V2C_NF_EXXEE)[mc]);
        } else {
          sxxe = ff_round(sxxen); sppe = ff_round(sppen); exxe = ff_round(exxen);
        }
        if (a.S.sppe_nstress) sppe = a.S.nstress_f;
        N.f(V2C_NF_SXXEN)[mc] = ff_round(sxxen); N.f(V2C_NF_SPPEN)[mc] = ff_round(sppen);
        N.f(V2C_NF_EXXEN)[mc] = ff_round(exxen); N.f(V2C_NF_SXXE)[mc] = sxxe;
        N.f(V2C_NF_SPPE)[mc] = sppe; N.f(V2C_NF_EXXE)[mc] = exxe;
        N.f(V2C_NF_ND_M2C)[mc] = ratio(cur[0], s1f);
        N.f(V2C_NF_GD)[mc] = ratio(cur[0], acc_ff(cur[1]));
        N.f(V2C_NF_BM)[mc] = 50e9f;
        N.f(V2C_NF_DRO)[mc] = 0; N.f(V2C_NF_DRP)[mc] = 0;
      } else {
        N.f(V2C_NF_SXXEN)[mc] = 0; N.f(V2C_NF_SPPEN)[mc] = 0; N.f(V2C_NF_EXXEN)[mc] = 0;
        N.f(V2C_NF_SXXE)[mc] = 0; N.f(V2C_NF_SPPE)[mc] = 0; N.f(V2C_NF_EXXE)[mc] = 0;
        N.f(V2C_NF_GD)[mc] = 0; N.f(V2C_NF_BM)[mc] = 0;
        N.f(V2C_NF_DRO)[mc] = 0; N.f(V2C_NF_DRP)[mc] = 0;
      }
    }
    // centre fields of nodes no cell feeds (first column / first row)
    if (ci == 0 || j == 0) {
      N.f(V2C_NF_SXXEN)[m3] = 0; N.f(V2C_NF_SPPEN)[m3] = 0; N.f(V2C_NF_EXXEN)[m3] = 0;
      N.f(V2C_NF_SXXE)[m3] = 0; N.f(V2C_NF_SPPE)[m3] = 0; N.f(V2C_NF_EXXE)[m3] = 0;
      N.f(V2C_NF_GD)[m3] = 0; N.f(V2C_NF_BM)[m3] = 0;
      N.f(V2C_NF_DRO)[m3] = 0; N.f(V2C_NF_DRP)[m3] = 0;
    }
  } else {
    const ff wxf = acc_ff(cur[2]);
    if (ff_round(wxf) != 0.f) {
      const ff mrx0 = acc_ff(cur[1]);
      const ff mvxn = ff_div_fast(acc_ff(cur[0]), mrx0);
      N.f(V2C_NF_MVXN)[m3] = ff_round(mvxn);
      // the boundary correction (vxvy_boundarycorrection) leaves the vx
      // ghost row at zero; only the 13-node stencil gives it weight
      N.f(V2C_NF_MVX)[m3] = j == g.yn - 1 ? 0.f
                            : antid ? antid_rn(mvxn, N.f(V2C_NF_VX)[m3], N.f(V2C_NF_MVXE)[m3])
                                    : ff_round(mvxn);
      N.f(V2C_NF_MRX)[m3] = ff_round(ff_div_fast(mrx0, wxf));
    } else {
      N.f(V2C_NF_MVX)[m3] = 0; N.f(V2C_NF_MRX)[m3] = 0;
    }
    const ff wyf = acc_ff(vy3[2]);
    if (ff_round(wyf) != 0.f) {
      const ff mry0 = acc_ff(vy3[1]);
      const ff mvyn = ff_div_fast(acc_ff(vy3[0]), mry0);
      N.f(V2C_NF_MVYN)[m3] = ff_round(mvyn);
      N.f(V2C_NF_MVY)[m3] = ci == g.xn - 1 ? 0.f  // the vy ghost column, likewise
                            : antid ? antid_rn(mvyn, N.f(V2C_NF_VY)[m3], N.f(V2C_NF_MVYE)[m3])
                                    : ff_round(mvyn);
      N.f(V2C_NF_MRY)[m3] = ff_round(ff_div_fast(mry0, wyf));
    } else {
      N.f(V2C_NF_MVY)[m3] = 0; N.f(V2C_NF_MRY)[m3] = 0;
    }
  }
}

// MINB resident CTAs per SM: 6 (80 registers, no spills); the skewed
// staging area (33.8 KB) leaves room for 6 CTAs, and at 7 (72 registers)
// the spills cost more than the extra CTA gave before the skew (C4 window:
// 0.73 against 0.65 ms)
template <int MINB>
__global__ void __launch_bounds__(NTH, MINB) k_m2n(M2NArgs a) {
  __shared__ Smem sm;
  const Grid &g = a.g;
  const int tid = threadIdx.x, role = tid / TY, jl = tid % TY;
  const int i0 = blockIdx.x * a.TX, j0 = blockIdx.y * TY;
  const int j = j0 + jl;
  const bool jvalid = j < g.yn;
  const int ncy = g.ncy;
  const int ci_end = min(i0 + a.TX, g.xn);

  // role 0: nu, nu/G, e, sxy, exy, C, phi, w      role 1: ro, et, ht, cp, kt, tk, w
  // role 2: nu, nu/G, sxx, exx, p, w (centre)     role 3: vx*ro, ro, w (vx) + vy*ro, ro, w (vy)
  Acc cur[8], car[8], vy3[3];
#pragma unroll
  for (int q = 0; q < 8; q++) { cur[q].zero(); car[q].zero(); }
#pragma unroll
  for (int q = 0; q < 3; q++) vy3[q].zero();

  for (int ci = max(i0 - 1, 0); ci < ci_end; ++ci) {
#pragma unroll
    for (int q = 0; q < 8; q++) { cur[q] = car[q]; car[q].zero(); }
#pragma unroll
    for (int q = 0; q < 3; q++) vy3[q].zero();
    if (role == 2) {
#pragma unroll
      for (int q = 0; q < 8; q++) cur[q].zero();
    }

    if (ci < g.ncx) {
      const int jlo = max(j0 - 1, 0), jhi = min(j0 + TY - 1, ncy - 1);
      const long cb = (long)ci * ncy;
      const int seg_b = __ldg(a.start + cb + jlo), seg_e = __ldg(a.start + cb + jhi + 1);
      // quarter class starts of cell (ci, j-1) (lower) and (ci, j) (upper)
      int4 ql = make_int4(0, 0, 0, 0), qu = make_int4(0, 0, 0, 0);
      int lo_e = 0, up_e = 0;
      float s1lo = 0.f, s1up = 0.f;
      const float iwx = 1.f / __ldg(g.wx + ci);
      if (jvalid && j - 1 >= 0 && j - 1 <= ncy - 1) {
        ql = __ldg(a.qstart + cb + j - 1);
        lo_e = __ldg(a.start + cb + j);
        s1lo = iwx / __ldg(g.wy + j - 1);
      }
      if (jvalid && j <= ncy - 1) {
        qu = __ldg(a.qstart + cb + j);
        up_e = __ldg(a.start + cb + j + 1);
        s1up = iwx / __ldg(g.wy + j);
      }
      const int rlo = j - 1 - jlo, rup = j - jlo;  // skews of cells (ci, j-1), (ci, j)
      for (int cs = seg_b; cs < seg_e; cs += CHUNK) {
        const int ce = min(cs + CHUNK, seg_e);
        __syncthreads();
        stage_chunk(a, sm, cs, ce, ci, jlo, tid);
        __syncthreads();
// the staged markers of sorted positions [b, e) (one quarter class run)
#define CLASS_RUN(b, e, r) \
  for (int s = max((b), cs), s_e = min((e), ce), q = s - cs + (r); s < s_e; ++s, ++q) \
    if (sm.act[q])
        if (role <= 1) {
          // cell (ci, j-1), bottom halves (v > 1/2): class 2 left, class 3 right
          CLASS_RUN(ql.z, ql.w, rlo) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            if (u < 0.5f) {
              const float w = s1lo * (1.f - 2.f * u) * (2.f * v - 1.f);
              if (role == 0) ADD_BASIC_A(cur, q, w); else ADD_BASIC_B(cur, q, w);
            }
          }
          CLASS_RUN(ql.w, lo_e, rlo) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float w = s1lo * (2.f * u - 1.f) * (2.f * v - 1.f);
            if (role == 0) ADD_BASIC_A(car, q, w); else ADD_BASIC_B(car, q, w);
          }
          // cell (ci, j), top halves (v < 1/2): class 0 left, class 1 right
          CLASS_RUN(qu.x, qu.y, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            if (u < 0.5f && v < 0.5f) {
              const float w = s1up * (1.f - 2.f * u) * (1.f - 2.f * v);
              if (role == 0) ADD_BASIC_A(cur, q, w); else ADD_BASIC_B(cur, q, w);
            }
          }
          CLASS_RUN(qu.y, qu.z, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            if (v < 0.5f) {
              const float w = s1up * (2.f * u - 1.f) * (1.f - 2.f * v);
              if (role == 0) ADD_BASIC_A(car, q, w); else ADD_BASIC_B(car, q, w);
            }
          }
        } else if (role == 2) {
          // the whole cell (ci, j) to its centre node
          CLASS_RUN(qu.x, up_e, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float w = s1up * tent(u) * tent(v);
            cur[0].add(sm.p[P_NU][q] * w); cur[1].add(sm.p[P_NUG][q] * w);
            cur[2].add(sm.p[P_SXX][q] * w); cur[3].add(sm.p[P_EXX][q] * w);
            cur[4].add(sm.p[P_P][q] * w); cur[5].add(w);
          }
        } else {
          // vy node (ci, j) from the bottom halves of cell (ci, j-1)
          CLASS_RUN(ql.z, lo_e, rlo) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float w = s1lo * (1.f - fabsf(u - 0.5f)) * v;
            const float ro = sm.p[P_RO][q];
            vy3[0].add(sm.p[P_VY][q] * ro * w); vy3[1].add(ro * w); vy3[2].add(w);
          }
          // cell (ci, j): vx node (ci, j) from u < 1/2 (classes 0, 2), vx node
          // (ci+1, j) from u > 1/2 (classes 1, 3), vy node (ci, j) from v < 1/2
          // (classes 0, 1)
          CLASS_RUN(qu.x, qu.y, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float ro = sm.p[P_RO][q];
            if (u < 0.5f) {
              const float w = s1up * (1.f - u) * (1.f - fabsf(v - 0.5f));
              cur[0].add(sm.p[P_VX][q] * ro * w); cur[1].add(ro * w); cur[2].add(w);
            }
            if (v < 0.5f) {
              const float w = s1up * (1.f - fabsf(u - 0.5f)) * (1.f - v);
              vy3[0].add(sm.p[P_VY][q] * ro * w); vy3[1].add(ro * w); vy3[2].add(w);
            }
          }
          CLASS_RUN(qu.y, qu.z, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float ro = sm.p[P_RO][q];
            const float wx = s1up * u * (1.f - fabsf(v - 0.5f));
            car[0].add(sm.p[P_VX][q] * ro * wx); car[1].add(ro * wx); car[2].add(wx);
            if (v < 0.5f) {
              const float w = s1up * (1.f - fabsf(u - 0.5f)) * (1.f - v);
              vy3[0].add(sm.p[P_VY][q] * ro * w); vy3[1].add(ro * w); vy3[2].add(w);
            }
          }
          CLASS_RUN(qu.z, qu.w, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            if (u < 0.5f) {
              const float ro = sm.p[P_RO][q];
              const float w = s1up * (1.f - u) * (1.f - fabsf(v - 0.5f));
              cur[0].add(sm.p[P_VX][q] * ro * w); cur[1].add(ro * w); cur[2].add(w);
            }
          }
          CLASS_RUN(qu.w, up_e, rup) {
            const float u = sm.p[P_U][q], v = sm.p[P_V][q];
            const float ro = sm.p[P_RO][q];
            const float w = s1up * u * (1.f - fabsf(v - 0.5f));
            car[0].add(sm.p[P_VX][q] * ro * w); car[1].add(ro * w); car[2].add(w);
          }
        }
#undef CLASS_RUN
      }
    }

    // ------------------------------------------------------ node tail
    if (ci < i0 || !jvalid) continue;
    node_tail(a, role, ci, j, cur, vy3);
  }
}

// ------------------------------------------------ interpolationmod 1
// The 13-node stencil (interpolation.c:258-538) as a gather: one thread per
// node and role sums, in sorted-marker order cell by cell, the markers of
// the cells whose stencil reaches the node, with that stencil's weight
// (bilinear on basic nodes; the staggered vx, vy and centre stencils with
// their half-cell conditions), then runs the same node tail as the tile
// sweep.  A marker in cell (cx, cy) at offsets (u, v) reaches
//   basic (cx + a, cy + b), a, b in {0, 1}:  (a ? u : 1-u) (b ? v : 1-v)
//   vx (cx + a, cy + b), b in {-1, 0, 1}:    (a ? u : 1-u) times 1-|v-1/2|
//       (b = 0), v-1/2 if v > 1/2 (b = 1), 1/2-v if v < 1/2 (b = -1)
//   vy likewise with the axes exchanged (a in {-1, 0, 1}, b in {0, 1})
//   centre (cx + a, cy + b), a, b in {0, 1, 2}: the product of the axis
//       factors 1/2-u if u < 1/2 (a = 0), 1-|u-1/2| (a = 1), u-1/2 if
//       u > 1/2 (a = 2), and the same in v.
// Contributions the reference sends past the last node row (its node
// index wraps into the next column's first row, a centre node that is
// never normalised) have no effect and are not formed.
struct Mk {
  int idx, t;
  float u, v;
};

__device__ __forceinline__ bool marker_active(const Grid &g, int cx, int cy, float u, float v) {
  bool act = true;
  if (cx == 0 || cx == g.ncx - 1) {
    double x = g.gx[cx] + (double)u * (g.gx[cx + 1] - g.gx[cx]);
    act = act && x > 0 && x < g.xsize;
  }
  if (cy == 0 || cy == g.ncy - 1) {
    double y = g.gy[cy] + (double)v * (g.gy[cy + 1] - g.gy[cy]);
    act = act && y > 0 && y < g.ysize;
  }
  return act;
}

// axis factor of a staggered (half-cell) stencil: k = 0 below the cell's
// middle, 1 across it, 2 above it; 0 where the stencil does not reach
__device__ __forceinline__ float half_factor(int k, float f) {
  if (k == 0) return f < 0.5f ? 1.f - f - 0.5f : 0.f;
  if (k == 1) return 1.f - fabsf(f - 0.5f);
  return f > 0.5f ? f - 0.5f : 0.f;
}

template <int ROLE>
__global__ void __launch_bounds__(128) k_m2n_mode1(M2NArgs a) {
  const Grid &g = a.g;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= g.nn) return;
  const int ix = (int)(t / g.yn), iy = (int)(t - (long)ix * g.yn);
  const int ncy = g.ncy;
  Acc cur[8], vy3[3];
#pragma unroll
  for (int q = 0; q < 8; q++) cur[q].zero();
#pragma unroll
  for (int q = 0; q < 3; q++) vy3[q].zero();
  // cells that can reach this node: dx, dy offsets of the cell from the node
  const int dx0 = ROLE == 2 ? -2 : -1, dx1 = ROLE == 3 ? 1 : 0;
  const int dy0 = ROLE == 2 ? -2 : -1, dy1 = ROLE == 3 ? 1 : 0;
  for (int dx = dx0; dx <= dx1; dx++) {
    const int cx = ix + dx;
    if (cx < 0 || cx >= g.ncx) continue;
    const float iwx = 1.f / __ldg(g.wx + cx);
    for (int dy = dy0; dy <= dy1; dy++) {
      const int cy = iy + dy;
      if (cy < 0 || cy >= ncy) continue;
      // stencil position of the node relative to the cell: a = -dx, b = -dy
      const int ax = -dx, by = -dy;
      if (ROLE == 3 && ax < 0 && by < 0) continue;  // (1, 1): no stencil reaches
      const float s1 = iwx / __ldg(g.wy + cy);
      const long c = (long)cx * ncy + cy;
      // quarter classes (2 (v > 1/2) + (u > 1/2)) that can have weight:
      // a half-cell factor k = 0 needs the lower half, k = 2 the upper
      constexpr int UX[3] = {0x5, 0xf, 0xa}, VY[3] = {0x3, 0xf, 0xc};
      int mask = 0xf;
      if (ROLE == 2) mask = UX[ax] & VY[by];
      if (ROLE == 3) mask = (ax >= 0 ? VY[by + 1] : 0) | (by >= 0 ? UX[ax + 1] : 0);
      const int4 qs = __ldg(a.qstart + c);
      const int qb[5] = {qs.x, qs.y, qs.z, qs.w, __ldg(a.start + c + 1)};
      for (int q = 0; q < 4; q++) {
        if (!((mask >> q) & 1)) continue;
      for (int s = qb[q]; s < qb[q + 1]; s++) {
        const int idx = __ldg(a.perm + s);
        const float u = a.m.u_in[idx], v = a.m.v_in[idx];
        if (!marker_active(g, cx, cy, u, v)) continue;
        const int tt = a.m.type[idx];
        if (ROLE == 0 || ROLE == 1) {
          const float w = s1 * (ax ? u : 1.f - u) * (by ? v : 1.f - v);
          if (ROLE == 0) {
            const float mnu = a.m.mnu[idx];
            cur[0].add(mnu * w); cur[1].add(mnu * a.R(RK_INV_GG, tt) * w);
            cur[2].add(a.m.e[idx] * w); cur[3].add(a.m.sxy[idx] * w);
            cur[4].add(a.m.exy[idx] * w); cur[5].add(a.m.coh[idx] * w);
            cur[6].add(a.m.phi[idx] * w); cur[7].add(w);
          } else {
            const float T = a.m.tk[idx], bb = a.R(RK_BB, tt);
            const float ro = a.S.p.densimod ? a.m.mro[idx] : a.R(RK_RO, tt);
            cur[0].add(ro * w);
            cur[1].add(__fdividef(bb, 1.f - bb * (T - 298.15f)) * w);
            cur[2].add(a.R(RK_HT, tt) * w); cur[3].add(a.R(RK_CP, tt) * w);
            cur[4].add(a.m.mkt[idx] * w); cur[5].add(T * w); cur[6].add(w);
          }
        } else if (ROLE == 2) {
          const float w = s1 * half_factor(ax, u) * half_factor(by, v);
          if (w != 0.f) {
            const float mnu = a.m.mnu[idx];
            cur[0].add(mnu * w); cur[1].add(mnu * a.R(RK_INV_GG, tt) * w);
            cur[2].add(a.m.sxx[idx] * w); cur[3].add(a.m.exx[idx] * w);
            cur[4].add(a.m.p[idx] * w); cur[5].add(w);
          }
        } else {
          const float ro = a.S.p.densimod ? a.m.mro[idx] : a.R(RK_RO, tt);
          // vx node: x bilinear (ax in {0, 1}), y staggered (by + 1 in {0, 1, 2})
          if (ax >= 0) {
            const float w = s1 * (ax ? u : 1.f - u) * half_factor(by + 1, v);
            if (w != 0.f) {
              cur[0].add(a.m.vx[idx] * ro * w); cur[1].add(ro * w); cur[2].add(w);
            }
          }
          // vy node: x staggered (ax + 1), y bilinear (by in {0, 1})
          if (by >= 0) {
            const float w = s1 * half_factor(ax + 1, u) * (by ? v : 1.f - v);
            if (w != 0.f) {
              vy3[0].add(a.m.vy[idx] * ro * w); vy3[1].add(ro * w); vy3[2].add(w);
            }
          }
        }
      }
      }
    }
  }
  if (ROLE != 2) {
    node_tail(a, ROLE, ix, iy, cur, vy3);
  } else if (ix >= 1 && iy >= 1) {
    node_tail(a, 2, ix - 1, iy - 1, cur, vy3);  // writes centre node (ix, iy)
  } else {
    // a centre node no cell has (first column or row)
    const Nodes &N = a.N;
    const long m3 = t;
    N.f(V2C_NF_SXXEN)[m3] = 0; N.f(V2C_NF_SPPEN)[m3] = 0; N.f(V2C_NF_EXXEN)[m3] = 0;
    N.f(V2C_NF_SXXE)[m3] = 0; N.f(V2C_NF_SPPE)[m3] = 0; N.f(V2C_NF_EXXE)[m3] = 0;
    N.f(V2C_NF_GD)[m3] = 0; N.f(V2C_NF_BM)[m3] = 0;
    N.f(V2C_NF_DRO)[m3] = 0; N.f(V2C_NF_DRP)[m3] = 0;
  }
}

__global__ void k_sticky(float *st, const uint32_t *key, long nn) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < nn) {
    uint32_t k = key[i];
    st[i] = k ? (float)(k & 3u) : 0.f;
  }
}

// ghost copy of the state when it diffuses, interpolation.c:827-859
__global__ void k_dphis(Grid g, float *phis) {
  long m3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (m3 >= g.nn) return;
  const int yn = g.yn, xn = g.xn;
  int m22 = (int)(m3 % yn), m11 = (int)(m3 / yn);
  float v;
  if (m11 == 0 && m22 >= 1 && m22 <= yn - 2) v = phis[m3 + yn];
  else if (m11 == xn - 1 && m22 >= 1 && m22 <= yn - 2) v = phis[m3 - yn];
  else if (m22 == 0 && m11 >= 1 && m11 <= xn - 2) v = phis[m3 + 1];
  else if (m22 == yn - 1 && m11 > 0 && m11 <= xn - 2) v = phis[m3 - 1];
  else if ((m11 == 0 || m11 == xn - 1) && (m22 == 0 || m22 == yn - 1)) v = 0.f;
  else return;
  // boundary values only read interior ones: no read-after-write hazard
  phis[m3] = v;
}

}  // namespace

void launch_m2n(const M2NArgs &a, cudaStream_t st) {
  if (a.S.p.interpolationmod == 1) {
    const unsigned nb = (unsigned)((a.g.nn + 127) / 128);
    k_m2n_mode1<0><<<nb, 128, 0, st>>>(a);
    k_m2n_mode1<1><<<nb, 128, 0, st>>>(a);
    k_m2n_mode1<2><<<nb, 128, 0, st>>>(a);
    k_m2n_mode1<3><<<nb, 128, 0, st>>>(a);
    return;
  }
  dim3 grid((a.g.xn + a.TX - 1) / a.TX, (a.g.yn + TY - 1) / TY);
  k_m2n<6><<<grid, NTH, 0, st>>>(a);
}

void launch_sticky(const Nodes &N, const uint32_t *key, long nn, cudaStream_t st) {
  k_sticky<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(N.f(V2C_NF_STICKY01), key, nn);
}

void launch_dphis(const Grid &g, const Nodes &N, cudaStream_t st) {
  k_dphis<<<(unsigned)((g.nn + 255) / 256), 256, 0, st>>>(g, N.f(V2C_NF_PHIS));
}

}  // namespace v2c
