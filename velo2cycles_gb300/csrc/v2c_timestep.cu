// v2c_timestep.cu -- the adaptive time step calc_timestep (calc_RSF.c:
// 352-572) over the device node fields.
//
// Per interior node: the visco-plastic Maxwell limit tcnvp*eta_vp/G, the
// displacement limit tcd/max(|vx|/dx, |vy|/dy), and with RSFmode 1 the
// Lapusta et al. (2000) slip-length limit lambda*L/V and the state limit
// tcphih/(V0/L e^-phi); the maximum slip rate; the stress and viscosity
// statistics over sticky01 == 1 / == 2 nodes.  Per-node arithmetic in FP32
// (the node fields are FP32), sums in FP64.
//
// Two sequential rules of the reference are kept by folding in node order:
// a node with b <= 0 resets the state and slip-length limits to maxtmstep
// (calc_RSF.c:497-501), so those minima run over the nodes after the last
// such node; and lambda carries over from the previous node where chi is
// NaN (no branch of calc_RSF.c:466-481 taken).  Each warp owns a contiguous
// node range and walks it in 32-node slices; segment states combine with
//   (A then B): reset = A.reset | B.reset, all = min(A.all, B.all),
//               after = B.reset ? B.after : min(A.after, B.all),
// which is associative, so the warp ranges fold in order in a tree.  The
// lambda carry crosses slices but not warp ranges: a NaN-chi node at the
// start of a range takes 1/5 (MINV(NaN, 1/5) in the reference's order).
// chi == 0 (where the reference stops) sets an error flag.
#include <math.h>

#include "v2c_kernels.h"

namespace v2c {

namespace {

enum {
  TS_DTNVP = 0, TS_DTD, TS_MAXVX, TS_MAXVEL,
  TS_PHI_ALL, TS_L_ALL, TS_PHI_AFTER, TS_L_AFTER, TS_RESET,
  TS_NR0, TS_MAXS0, TS_MINS0, TS_SUMS0, TS_SUM2S0, TS_MAXV0, TS_MINV0, TS_SUMV0, TS_SUM2V0,
  TS_NR1, TS_MAXS1, TS_MINS1, TS_SUMS1, TS_SUM2S1, TS_MAXV1, TS_MINV1, TS_SUMV1, TS_SUM2V1,
  TS_N
};
// extra output slots after the folded partial
enum { TS_P1S = TS_N, TS_P2S, TS_P1V, TS_P2V, TS_CHI0, TS_OUT_N };

constexpr int TW = 8;  // warps per block of the node pass

__device__ __forceinline__ int ts_kind(int k) {  // 0 min, 1 max, 2 sum, 3 ordered
  switch (k) {
    case TS_DTNVP: case TS_DTD: case TS_MINS0: case TS_MINV0: case TS_MINS1: case TS_MINV1:
      return 0;
    case TS_MAXVX: case TS_MAXVEL: case TS_MAXS0: case TS_MAXV0: case TS_MAXS1: case TS_MAXV1:
      return 1;
    case TS_PHI_ALL: case TS_L_ALL: case TS_PHI_AFTER: case TS_L_AFTER: case TS_RESET:
      return 3;
    default:
      return 2;
  }
}

__device__ __forceinline__ void ts_init(double *s) {
  for (int k = 0; k < TS_N; k++) s[k] = 0.0;
  s[TS_DTNVP] = s[TS_DTD] = s[TS_PHI_ALL] = s[TS_L_ALL] = s[TS_PHI_AFTER] = s[TS_L_AFTER] = 1e30;
  s[TS_MINS0] = s[TS_MINV0] = s[TS_MINS1] = s[TS_MINV1] = 1e30;
}

// a := a then b (b follows a in node order)
__device__ __forceinline__ void ts_combine(double *a, const double *b) {
  for (int k = 0; k < TS_N; k++) {
    const int kind = ts_kind(k);
    if (kind == 0) a[k] = b[k] <= a[k] ? b[k] : a[k];
    else if (kind == 1) a[k] = b[k] >= a[k] ? b[k] : a[k];
    else if (kind == 2) a[k] += b[k];
  }
  const bool br = b[TS_RESET] != 0.0;
  a[TS_PHI_AFTER] = br ? b[TS_PHI_AFTER] : (b[TS_PHI_ALL] <= a[TS_PHI_AFTER] ? b[TS_PHI_ALL] : a[TS_PHI_AFTER]);
  a[TS_L_AFTER] = br ? b[TS_L_AFTER] : (b[TS_L_ALL] <= a[TS_L_AFTER] ? b[TS_L_ALL] : a[TS_L_AFTER]);
  a[TS_PHI_ALL] = b[TS_PHI_ALL] <= a[TS_PHI_ALL] ? b[TS_PHI_ALL] : a[TS_PHI_ALL];
  a[TS_L_ALL] = b[TS_L_ALL] <= a[TS_L_ALL] ? b[TS_L_ALL] : a[TS_L_ALL];
  a[TS_RESET] = (a[TS_RESET] != 0.0 || br) ? 1.0 : 0.0;
}

struct TsArgs {
  Grid g;
  Nodes N;
  Scal S;
  v2c_timestep_ctl c;
  int oldornew;
  long per_warp;   // nodes per warp range (a multiple of 32)
  double *part;    // [warps][TS_N]
  double *out;     // [TS_OUT_N]
};

// node pass: one warp per contiguous range
__global__ void __launch_bounds__(TW * 32) k_ts_nodes(TsArgs a) {
  const Grid &g = a.g;
  const Nodes &N = a.N;
  const v2c_params &P = a.S.p;
  const int lane = threadIdx.x & 31;
  const long warp = (long)blockIdx.x * TW + (threadIdx.x >> 5);
  const long lo = warp * a.per_warp, hi = min(lo + a.per_warp, g.nn);
  const long yn = g.yn;
  double s[TS_N];
  ts_init(s);
  float lam_carry = __int_as_float(0x7fc00000);  // NaN: none yet
  for (long b0 = lo; b0 < hi; b0 += 32) {
    const long m3 = b0 + lane;
    const long m2 = m3 % yn, m1 = (m3 - m2) / yn;
    const bool interior = m3 < hi && m1 >= 1 && m2 >= 1 && m1 < g.xn - 1 && m2 < yn - 1;
    double d[TS_N];
    ts_init(d);
    bool rsf_node = false, chi_ok = false, reset = false, has_phi = false;
    float lam_raw = 0.f, LoV = 0.f, dtphi = 0.f;
    if (interior) {
      const float dx = __ldg(g.wx + m1), dy = __ldg(g.wy + m2);
      const float faultwidth = 2.f * 0.5f * (dx + dy);
      const float nu_m2c = N.f(V2C_NF_NU_M2C)[m3], gg = N.f(V2C_NF_GG)[m3];
      float NUVP;
      if (a.oldornew == 0) {
        if (nu_m2c > 1.00e+26f) {
          const float sx = N.f(V2C_NF_SXXES)[m3], sy = N.f(V2C_NF_SXYE)[m3];
          const float sg = sqrtf(sx * sx + sy * sy);
          const float V = N.f(V2C_NF_RK_SLIPRS_FINAL)[m3];
          NUVP = (sg > 0.f && V > 0.f) ? nu_m2c * sg / (2.f * nu_m2c * V / faultwidth + sg) : nu_m2c;
        } else {
          NUVP = 5.00e+26f;
        }
      } else {
        NUVP = (nu_m2c > 1.00e+26f) ? N.f(V2C_NF_NU)[m3] : 5.00e+26f;
      }
      d[TS_DTNVP] = (float)a.c.tcnvp * NUVP / gg;
      const float VXn = a.oldornew == 1 ? N.f(V2C_NF_VX)[m3] : N.f(V2C_NF_MVX)[m3];
      const float VYn = a.oldornew == 1 ? N.f(V2C_NF_VY)[m3] : N.f(V2C_NF_MVY)[m3];
      if (VXn != 0.f && VYn != 0.f) {
        const float ax = fabsf(VXn), ay = fabsf(VYn);
        d[TS_MAXVX] = ax >= ay ? ax : ay;
        const float rx = fabsf(VXn / dx), ry = fabsf(VYn / dy);
        d[TS_DTD] = (float)a.c.tcd * 1.f / (rx >= ry ? rx : ry);
      }
      if (P.RSFmode == 1) {
        rsf_node = true;
        float nps = 0.f;
        if (P.pmode == 0) nps = (float)P.nstress;
        else if (P.pmode == 1) nps = a.oldornew == 0 ? N.f(V2C_NF_SPPES)[m3] : N.f(V2C_NF_PRS)[m3];
        const float bm = N.f(V2C_NF_BM)[m3];
        const float as = N.f(V2C_NF_AS)[m3], bs = N.f(V2C_NF_BS)[m3], Ls = N.f(V2C_NF_LS)[m3];
        const float v = (3.f * bm - 2.f * gg) / (2.f * (3.f * bm + gg));
        const float k = 2.f / 3.14f * (gg / (1.f - v)) / (float)P.xstpx;
        const float q = k * Ls / (as * nps);
        const float h = q - (bs - as) / as;
        const float chi = 0.25f * h * h - q;
        if (chi > 0.f) { lam_raw = as * nps / (k * Ls - (bs - as) * nps); chi_ok = true; }
        else if (chi < 0.f) { lam_raw = 1.f - (bs - as) * nps / (k * Ls); chi_ok = true; }
        else if (chi == 0.f) a.out[TS_CHI0] = 1.0;
        reset = !(bs > 0.f);
        if (!reset) {
          const float Vf = N.f(V2C_NF_RK_SLIPRS_FINAL)[m3], Vs = N.f(V2C_NF_RK_SLIPRS_SOLVED)[m3];
          if (a.oldornew == 0 && Vf > 0.f) {
            dtphi = (float)a.c.tcphih * 1.f / (N.f(V2C_NF_V0S)[m3] / Ls * expf(-N.f(V2C_NF_PHIS)[m3]));
            LoV = Ls / Vf;
            has_phi = true;
          } else if (a.oldornew == 1 && Vs > 0.f) {
            dtphi = (float)a.c.tcphih * 1.f / (N.f(V2C_NF_V0S)[m3] / Ls * expf(-N.f(V2C_NF_PHIS_IT)[m3]));
            LoV = Ls / Vs;
            has_phi = true;
          }
        }
      }
      const float sx = N.f(V2C_NF_SXXS)[m3], sy = N.f(V2C_NF_SXY)[m3];
      const double sg = sqrtf(sx * sx + sy * sy), nv = N.f(V2C_NF_NU)[m3];
      const float st = N.f(V2C_NF_STICKY01)[m3];
      if (st == 2.f) {
        const double l = log10(nv);
        d[TS_NR1] = 1; d[TS_MAXS1] = d[TS_MINS1] = d[TS_SUMS1] = sg; d[TS_SUM2S1] = sg * sg;
        d[TS_MAXV1] = d[TS_MINV1] = nv; d[TS_SUMV1] = l; d[TS_SUM2V1] = l * l;
      }
      if (st == 1.f) {
        const double l = log10(nv);
        d[TS_NR0] = 1; d[TS_MAXS0] = d[TS_MINS0] = d[TS_SUMS0] = sg; d[TS_SUM2S0] = sg * sg;
        d[TS_MAXV0] = d[TS_MINV0] = nv; d[TS_SUMV0] = l; d[TS_SUM2V0] = l * l;
        if (m1 == 50 && m2 == 50) { a.out[TS_P1S] = sg; a.out[TS_P1V] = nv; }
        if (m1 == 500 && m2 == 50) { a.out[TS_P2S] = sg; a.out[TS_P2V] = nv; }
      }
      const float V = a.oldornew == 0 ? N.f(V2C_NF_RK_SLIPRS_FINAL)[m3] : N.f(V2C_NF_RK_SLIPRS_SOLVED)[m3];
      if (V > 0.f) d[TS_MAXVEL] = V;
    }
    // lambda: the node's own, or that of the last earlier node with a
    // defined chi (within the slice, else carried from earlier slices)
    const unsigned okm = __ballot_sync(V2C_FULL, rsf_node && chi_ok);
    const unsigned below = okm & ((lane == 31) ? 0xffffffffu : ((2u << lane) - 1u));
    const int src = below ? 31 - __clz(below) : -1;
    const float lam_from = __shfl_sync(V2C_FULL, lam_raw, src < 0 ? 0 : src);
    const float lam = src >= 0 ? lam_from : lam_carry;
    if (okm) lam_carry = __shfl_sync(V2C_FULL, lam_raw, 31 - __clz(okm));
    if (rsf_node) {
      if (reset) {
        d[TS_RESET] = 1.0;
      } else if (has_phi) {
        const float lamc = lam <= 0.2f ? lam : 0.2f;  // MINV(lambda, 1/5)
        const double dl = lamc * LoV;
        d[TS_PHI_ALL] = d[TS_PHI_AFTER] = dtphi;
        d[TS_L_ALL] = d[TS_L_AFTER] = dl;
      }
    }
    // fold the slice in lane order (adjacent pairs, lower lane first)
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      double e[TS_N];
#pragma unroll
      for (int k = 0; k < TS_N; k++) e[k] = __shfl_down_sync(V2C_FULL, d[k], o);
      if ((lane & (2 * o - 1)) == 0 && lane + o < 32) ts_combine(d, e);
    }
    if (lane == 0) ts_combine(s, d);
  }
  if (lane == 0) {
    double *p = a.part + warp * TS_N;
    for (int k = 0; k < TS_N; k++) p[k] = s[k];
  }
}

// fold the warp partials in order: pairs (2i, 2i+1) at each level
__global__ void k_ts_fold(double *part, long nw, double *out) {
  for (long step = 1; step < nw; step <<= 1) {
    for (long i = threadIdx.x; 2 * i * step + step < nw; i += blockDim.x) {
      double *A = part + (2 * i * step) * TS_N;
      const double *B = part + (2 * i * step + step) * TS_N;
      ts_combine(A, B);
    }
    __syncthreads();
  }
  if (threadIdx.x < TS_N) out[threadIdx.x] = part[threadIdx.x];
}

}  // namespace

int calc_timestep_device(const Grid &g, const Nodes &N, const Scal &S, const v2c_timestep_ctl &c,
                         int oldornew, double *scratch, long scratch_doubles,
                         v2c_timestep_info *info, cudaStream_t st) {
  const long warps_max = 152 * 4 * TW;
  long per_warp = (g.nn + warps_max - 1) / warps_max;
  per_warp = (per_warp + 31) / 32 * 32;
  const long warps = (g.nn + per_warp - 1) / per_warp;
  if ((warps + 1) * TS_N + TS_OUT_N > scratch_doubles) return V2C_ERR_CAPACITY;
  TsArgs a;
  a.g = g; a.N = N; a.S = S; a.c = c; a.oldornew = oldornew; a.per_warp = per_warp;
  a.out = scratch;
  a.part = scratch + TS_OUT_N;
  if (cudaMemsetAsync(a.out, 0, sizeof(double) * TS_OUT_N, st) != cudaSuccess) return V2C_ERR_CUDA;
  const long blocks = (warps + TW - 1) / TW;
  // warps past the node range write empty partials
  k_ts_nodes<<<(unsigned)blocks, TW * 32, 0, st>>>(a);
  k_ts_fold<<<1, 512, 0, st>>>(a.part, blocks * TW, a.out);
  double h[TS_OUT_N];
  if (cudaMemcpyAsync(h, a.out, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return V2C_ERR_CUDA;
  if (h[TS_CHI0] != 0.0) return V2C_ERR_TIMESTEP;
  const double dtphi = h[TS_RESET] != 0.0 ? (h[TS_PHI_AFTER] <= c.maxtmstep ? h[TS_PHI_AFTER] : c.maxtmstep)
                                          : h[TS_PHI_ALL];
  const double dtL = h[TS_RESET] != 0.0 ? (h[TS_L_AFTER] <= c.maxtmstep ? h[TS_L_AFTER] : c.maxtmstep)
                                        : h[TS_L_ALL];
  auto minv = [](double x, double y) { return x <= y ? x : y; };
  info->dt_f = c.dtfactor * minv(c.maxtmstep, minv(dtphi, minv(minv(dtL, h[TS_DTNVP]), h[TS_DTD])));
  info->maxvel = h[TS_MAXVEL];
  info->maxVx = h[TS_MAXVX];
  info->dtnvp = h[TS_DTNVP]; info->dtd = h[TS_DTD]; info->dtphi = dtphi; info->dtL = dtL;
  info->nr_0 = (long)h[TS_NR0]; info->nr_1 = (long)h[TS_NR1];
  info->max_sigin_0 = h[TS_MAXS0]; info->min_sigin_0 = h[TS_MINS0];
  info->sum_sigin_0 = h[TS_SUMS0]; info->sum2_sigin_0 = h[TS_SUM2S0];
  info->max_visc_0 = h[TS_MAXV0]; info->min_visc_0 = h[TS_MINV0];
  info->sum_visc_0 = h[TS_SUMV0]; info->sum2_visc_0 = h[TS_SUM2V0];
  info->max_sigin_1 = h[TS_MAXS1]; info->min_sigin_1 = h[TS_MINS1];
  info->sum_sigin_1 = h[TS_SUMS1]; info->sum2_sigin_1 = h[TS_SUM2S1];
  info->max_visc_1 = h[TS_MAXV1]; info->min_visc_1 = h[TS_MINV1];
  info->sum_visc_1 = h[TS_SUMV1]; info->sum2_visc_1 = h[TS_SUM2V1];
  info->sigin_P1 = h[TS_P1S]; info->sigin_P2 = h[TS_P2S];
  info->visco_P1 = h[TS_P1V]; info->visco_P2 = h[TS_P2V];
  return V2C_OK;
}

}  // namespace v2c
