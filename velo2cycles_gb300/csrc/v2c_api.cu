// v2c_api.cu -- the C ABI (include/v2c.h): context life cycle, transfers,
// and the step entry points that replace the reference's global-array
// routines.
#include <math.h>
#include <cmath>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "v2c_kernels.h"
#include "v2c_newton.h"

using namespace v2c;

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      ctx->last_error = V2C_ERR_CUDA;                              \
      ctx->cuda_msg = cudaGetErrorString(e_);                      \
      return V2C_ERR_CUDA;                                         \
    }                                                              \
  } while (0)

struct v2c_ctx {
  v2c_params p;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long cap = 0, n = 0;
  int xn = 0, yn = 0, ncx = 0, ncy = 0;
  long nn = 0, ncell = 0;
  // grid
  double *d_gx = nullptr, *d_gy = nullptr;
  float *d_wx = nullptr, *d_wy = nullptr, *d_gxf = nullptr, *d_gyf = nullptr;
  std::vector<double> h_gx, h_gy;
  bool have_grid = false, have_rock = false;
  // rock table
  float *d_rock = nullptr;
  std::vector<double> h_rt;
  // nodes
  float *d_node = nullptr;
  double *d_node64 = nullptr;  // boundary staging, one FP64 node field
  double *d_nstage = nullptr;  // boundary staging of several node fields
  int nstage_cap = 0;          // fields d_nstage holds
  uint32_t *d_sticky = nullptr;
  float4 *d_quad = nullptr;                  // move: velocity forms per cell quarter
  float *d_tol = nullptr;                    // temperature update: node scratch
  float *d_bs = nullptr;                     // interpolationmod 1 back-scatter payload
  unsigned *d_list_n = nullptr;              // count of listed Newton problems
  double *d_ts = nullptr;                    // calc_timestep scratch
  // markers
  Markers m{};
  void *marker_mem[32] = {};
  int n_marker_mem = 0;
  bool have_markers = false;
  // m.mnu / m.mkt hold the properties of the current marker slots (set by
  // marker2nodes, cleared when markers are uploaded or moved)
  bool props_valid = false;
  // asynchronous node-field downloads: their own staging area, copied on a
  // transfer stream after the conversion on the context stream
  cudaStream_t xfer = nullptr;
  cudaEvent_t ev_conv = nullptr, ev_copy = nullptr;
  double *d_astage = nullptr;
  int astage_fields = 0;
  bool dl_pending = false;
  // sort
  SortBufs sb{};
  bool sorted = false;
  // staging
  double *d_stage64 = nullptr, *d_stage64b = nullptr;
  // bonds
  std::vector<long> h_bondm, h_bondn;
  std::vector<double> h_bondv;
  long bondnum = 0;
  bool have_bonds = false;
  int bc_built_compressible = -1, bc_built_tempmod = -1;
  bool dsxx_valid = false;  // DSXX holds sxx - sxxe of the current node fields
  // FP64 node velocities (vx, then vy) for the strain rates, kept from the
  // uploads; valid per component while it matches the FP32 field
  double *d_vel64 = nullptr;
  bool vel64_ok[2] = {false, false};
  // FP64 copies of the uploaded node temperatures TK and TK2 (the marker
  // temperature update reads them); TK's is stale once marker2nodes writes TK
  double *d_tk64 = nullptr;
  bool tk64_ok[2] = {false, false};
  // immobile markers (type >= 100): their count, and the compaction
  // scratch, allocated the first time markers with such a type arrive
  long n_immobile = 0;
  ImmBufs imm{};
  void *imm_mem = nullptr;
  int bc_n = 0;
  void *bc_mem = nullptr;
  BcRows bc{};
  float *d_bc_scratch = nullptr;
  // status
  unsigned long long *d_stat = nullptr;
  double *d_red = nullptr;
  long red_cap = 0;
  int last_error = 0;
  long launches = 0;  // device kernels launched (instrumentation)
  const char *cuda_msg = "";
  // per-marker Newton / network
  NewtonState nw{};
  // instrumentation: event pairs per launch group, resolved on demand
  bool prof = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[V2C_PROF_N];
  double prof_ms[V2C_PROF_N] = {};
  long prof_n[V2C_PROF_N] = {};
  std::vector<cudaEvent_t> ev_pool;
  // seismic-cycle workload: per-regime velocity fields, accumulated slip,
  // captured step graphs
  float *d_cyc_v[2] = {nullptr, nullptr};  // [regime]: vx then vy, 2 nn floats
  double *d_cyc_v64[2] = {nullptr, nullptr};  // the same in FP64
  double *d_slip = nullptr;                 // accumulated slip per node
  double *d_mslip = nullptr;                // accumulated slip per marker (array order)
  struct CycleGraph {
    int regime;
    double dt;
    const void *pos;      // position buffer holding the current positions
    v2c_params p;         // all parameters, timesum zeroed
    int flags;            // the timesum classes the kernels see
    cudaGraphExec_t exec;
    long launches;        // kernels in one replay
  };
  std::vector<CycleGraph> graphs;
};

namespace {
cudaEvent_t ev_get(v2c_ctx *c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
// RAII bracket of one launch group
struct Prof {
  v2c_ctx *c;
  int g;
  cudaEvent_t a = nullptr;
  Prof(v2c_ctx *ctx, int group) : c(ctx), g(group) {
    if (c->prof) {
      a = ev_get(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~Prof() {
    if (c->prof) {
      cudaEvent_t b = ev_get(c);
      cudaEventRecord(b, c->stream);
      c->prof_ev[g].push_back({a, b});
    }
  }
};
void prof_resolve(v2c_ctx *c) {
  cudaStreamSynchronize(c->stream);
  for (int g = 0; g < V2C_PROF_N; g++) {
    for (auto &pr : c->prof_ev[g]) {
      float ms = 0;
      cudaEventElapsedTime(&ms, pr.first, pr.second);
      c->prof_ms[g] += ms;
      c->prof_n[g] += 1;
      c->ev_pool.push_back(pr.first);
      c->ev_pool.push_back(pr.second);
    }
    c->prof_ev[g].clear();
  }
}
}  // namespace

namespace {

template <class T>
cudaError_t dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}

Grid make_grid(const v2c_ctx *c) {
  Grid g;
  g.gx = c->d_gx; g.gy = c->d_gy; g.wx = c->d_wx; g.wy = c->d_wy;
  g.xn = c->xn; g.yn = c->yn; g.ncx = c->ncx; g.ncy = c->ncy; g.nn = c->nn;
  g.xsize = c->p.xsize; g.ysize = c->p.ysize;
  return g;
}

Scal make_scal(const v2c_params &p, const std::vector<double> &rt) {
  Scal s;
  s.p = p;
  s.antid = (p.timesum > 0 && p.antidiffinter == 1);
  s.phi_reset0 = (p.timesum == p.timestep);
  s.sticky_cap = (p.stickymod == 1 && p.timesum > 4e7);
  s.dt = (float)p.timestep;
  double gg2 = rt.empty() ? 0.0 : rt[V2C_RT_GG * V2C_MAXTMR + 2];
  s.sticky_nu = (float)(gg2 * p.timestep / 100);
  s.ln_nubeg = (float)log(p.nubeg);
  s.ln_nuend = (float)log(p.nuend);
  s.fault_y_f = (float)p.fault_y;
  s.fault_slope_f = (float)p.fault_slope;
  s.fault_hw1_f = (float)p.fault_hw + 1.0f;
  s.a_hr_f = (float)p.a_hr; s.b_hr_f = (float)p.b_hr;
  s.L_hr_f = (float)p.L_hr; s.V0_hr_f = (float)p.V0_hr;
  s.tdeep_f = (float)p.tdeep;
  s.zdeep_f = (float)p.zdeep;
  s.zdeep_lo_f = s.zdeep_f - 1.f - 1e-6f * fabsf(s.zdeep_f);
  s.eps2_f = (float)p.eps2;
  s.nstress_f = (float)p.nstress;
  s.nubeg_f = (float)p.nubeg;
  s.nuend_f = (float)p.nuend;
  s.faultwidth_f = (float)p.faultwidth;
  auto split = [](double d, float &hi, float &lo) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  };
  split(p.timestep, s.dt_hi, s.dt_lo);
  split(p.faultwidth, s.W_hi, s.W_lo);
  split(p.nstress, s.sn_hi, s.sn_lo);
  if (p.timestep > 0) {
    split(log(p.timestep), s.lndt_hi, s.lndt_lo);
  } else {
    s.lndt_hi = -INFINITY;
    s.lndt_lo = 0.f;
  }
  s.eps2_lo = (float)(p.eps2 - (double)s.eps2_f);
  s.tdeep_lo = (float)(p.tdeep - (double)s.tdeep_f);
  s.sppe_nstress = (p.timesum == 0 && p.reloadfromDP == 0 && p.compressiblemode == 1);
  s.timesum_pos = p.timesum > 0;
  s.timesum_zero = p.timesum == 0;
  return s;
}

Nodes make_nodes(const v2c_ctx *c) { return Nodes{c->d_node, c->nn}; }

int fail(v2c_ctx *ctx, int code) {
  if (ctx) ctx->last_error = code;
  return code;
}

int check_params(const v2c_params *p) {
  if (p->xnumx < 4 || p->ynumy < 4) return V2C_ERR_ARG;
  if (p->interpolationmod != 1 && p->interpolationmod != 2) return V2C_ERR_UNSUPPORTED;
  if (p->rkmod < 0 || p->rkmod > 3) return V2C_ERR_UNSUPPORTED;
  if (p->newton_guess < V2C_GUESS_PLAIN || p->newton_guess > V2C_GUESS_OFF) return V2C_ERR_ARG;
  if (p->newton_precision != V2C_NEWTON_SPLIT && p->newton_precision != V2C_NEWTON_FP64)
    return V2C_ERR_ARG;
  if (p->xnumx * p->ynumy > (long)INT32_MAX / 4) return V2C_ERR_CAPACITY;
  return V2C_OK;
}

// Column strip of the sweeps: the widest up to max_tx that still gives 1.5
// waves of 7 resident CTAs on each of the 152 SMs (a strip of tx columns
// restages one halo column).  The scatter takes strips of at most 16
// columns, the gather 32: at C4 (126 x 32 strips of 32 columns) the
// scatter's 4.4 waves at 6 CTAs left SMs idle in the last one, and 16
// columns (8.8 waves, 3 % more halo work) ran 5.17 -> 5.01 ms, while the
// gather ran 4.80 -> 4.86 ms with them.
int pick_tx(const v2c_ctx *c, int max_tx) {
  long rows = (c->yn + 31) / 32;
  int tx = max_tx;
  while (tx > 4 && rows * ((c->xn + tx - 1) / tx) < 152 * 7 * 3 / 2) tx /= 2;
  return tx;
}

}  // namespace

// ================================================================ life cycle
extern "C" int v2c_create(const v2c_params *p, long max_markers, void *cuda_stream,
                          v2c_ctx **out) {
  if (!p || !out || max_markers < 0) return V2C_ERR_ARG;
  if (max_markers >= SORT_MAX_MARKERS) return V2C_ERR_CAPACITY;
  int rc = check_params(p);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return V2C_ERR_CUDA;
  v2c_ctx *ctx = new v2c_ctx();
  ctx->p = *p;
  ctx->cap = max_markers;
  ctx->xn = (int)p->xnumx; ctx->yn = (int)p->ynumy;
  ctx->ncx = ctx->xn - 1; ctx->ncy = ctx->yn - 1;
  ctx->nn = (long)ctx->xn * ctx->yn;
  ctx->ncell = (long)ctx->ncx * ctx->ncy;
  if (cuda_stream) {
    ctx->stream = (cudaStream_t)cuda_stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return V2C_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
#define AL(ptr, cnt)                                                      \
  if (dalloc(&(ptr), (cnt)) != cudaSuccess) { v2c_destroy(ctx); return V2C_ERR_CUDA; }
  AL(ctx->d_gx, ctx->xn); AL(ctx->d_gy, ctx->yn);
  AL(ctx->d_wx, ctx->ncx); AL(ctx->d_wy, ctx->ncy);
  AL(ctx->d_gxf, ctx->xn); AL(ctx->d_gyf, ctx->yn);
  AL(ctx->d_rock, (size_t)RK_N * V2C_MAXTMR);
  AL(ctx->d_node, (size_t)V2C_NF_N * ctx->nn);
  AL(ctx->d_node64, ctx->nn);
  AL(ctx->d_sticky, ctx->nn);
  AL(ctx->d_quad, (size_t)ctx->ncell * QUAD_FLOAT4);
  AL(ctx->d_tol, ctx->nn);
  if (p->interpolationmod == 1) AL(ctx->d_bs, (size_t)BS_N * (ctx->cap > 0 ? ctx->cap : 1));
  AL(ctx->d_list_n, 1);
  AL(ctx->d_ts, TIMESTEP_SCRATCH);
  AL(ctx->d_stat, ST_N);
  ctx->red_cap = 2 + 2 * ((ctx->nn + 255) / 256);
  AL(ctx->d_red, ctx->red_cap);
  cudaMemsetAsync(ctx->d_node, 0, sizeof(float) * V2C_NF_N * ctx->nn, ctx->stream);
  cudaMemsetAsync(ctx->d_stat, 0, sizeof(unsigned long long) * ST_N, ctx->stream);
  // markers
  long cap = max_markers;
  Markers &m = ctx->m;
  void **mm = ctx->marker_mem;
  int k = 0;
#define AM(field, T)                                                     \
  if (dalloc(&(m.field), cap) != cudaSuccess) { v2c_destroy(ctx); return V2C_ERR_CUDA; } \
  mm[k++] = (void *)m.field; ctx->n_marker_mem = k;
  AM(cell_in, int32_t) AM(cell_out, int32_t) AM(u_in, float) AM(u_out, float)
  AM(v_in, float) AM(v_out, float) AM(id, int32_t) AM(type, int8_t) AM(flags, uint8_t)
  AM(tk, float) AM(tk_lo, float) AM(mv, float) AM(mv_lo, float) AM(e, float) AM(p, float) AM(sxx, float) AM(sxy, float) AM(exx, float)
  AM(exy, float) AM(vx, float) AM(vy, float) AM(phi, float) AM(coh, float) AM(slipv, float)
  AM(mnu, float) AM(mkt, float) AM(mro, float)
#undef AM
  ctx->n_marker_mem = k;
  // sort
  AL(ctx->sb.counts, ctx->ncell); AL(ctx->sb.start, ctx->ncell + 1);
  AL(ctx->sb.qstart, ctx->ncell + 1);
  AL(ctx->sb.slot, cap); AL(ctx->sb.tmp, cap); AL(ctx->sb.perm, cap);
  ctx->sb.blocksum_cap = (ctx->ncell + 4095) / 4096 + 1;
  AL(ctx->sb.blocksum, ctx->sb.blocksum_cap);
  AL(ctx->d_stage64, cap); AL(ctx->d_stage64b, cap);
#undef AL
  if (newton_init(ctx->nw, cap) != cudaSuccess) { v2c_destroy(ctx); return V2C_ERR_CUDA; }
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { v2c_destroy(ctx); return V2C_ERR_CUDA; }
  *out = ctx;
  return V2C_OK;
}

extern "C" int v2c_destroy(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->xfer) {
    cudaStreamSynchronize(ctx->xfer);
    cudaStreamDestroy(ctx->xfer);
  }
  if (ctx->ev_conv) cudaEventDestroy(ctx->ev_conv);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->d_astage) cudaFree(ctx->d_astage);
  for (auto &gr : ctx->graphs) cudaGraphExecDestroy(gr.exec);
  ctx->graphs.clear();
  for (float *v : ctx->d_cyc_v)
    if (v) cudaFree(v);
  for (double *v : ctx->d_cyc_v64)
    if (v) cudaFree(v);
  if (ctx->d_vel64) cudaFree(ctx->d_vel64);
  if (ctx->d_tk64) cudaFree(ctx->d_tk64);
  if (ctx->imm_mem) cudaFree(ctx->imm_mem);
  if (ctx->d_bs) cudaFree(ctx->d_bs);
  if (ctx->d_slip) cudaFree(ctx->d_slip);
  if (ctx->d_mslip) cudaFree(ctx->d_mslip);
  void *ptrs[] = {ctx->d_gx, ctx->d_gy, ctx->d_wx, ctx->d_wy, ctx->d_gxf, ctx->d_gyf,
                  ctx->d_rock, ctx->d_node, ctx->d_node64, ctx->d_sticky, ctx->d_quad, ctx->d_tol, ctx->d_list_n, ctx->d_ts,
                  ctx->d_stat, ctx->d_red, ctx->d_nstage,
                  ctx->sb.counts, ctx->sb.start, ctx->sb.qstart, ctx->sb.slot, ctx->sb.tmp, ctx->sb.perm,
                  ctx->sb.blocksum, ctx->d_stage64, ctx->d_stage64b, ctx->bc_mem,
                  ctx->d_bc_scratch};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  for (int i = 0; i < ctx->n_marker_mem; i++)
    if (ctx->marker_mem[i]) cudaFree(ctx->marker_mem[i]);
  newton_free(ctx->nw);
  prof_resolve(ctx);
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return V2C_OK;
}

extern "C" int v2c_set_params(v2c_ctx *ctx, const v2c_params *p) {
  if (!ctx || !p) return V2C_ERR_ARG;
  if (p->xnumx != ctx->p.xnumx || p->ynumy != ctx->p.ynumy) return fail(ctx, V2C_ERR_ARG);
  int rc = check_params(p);
  if (rc) return fail(ctx, rc);
  ctx->p = *p;
  // the full-stencil back-scatter's payload, allocated here so that no
  // step (or captured step) allocates
  if (p->interpolationmod == 1 && !ctx->d_bs)
    CK(cudaMalloc(&ctx->d_bs, sizeof(float) * BS_N * (ctx->cap > 0 ? ctx->cap : 1)));
  return V2C_OK;
}

extern "C" int v2c_set_grid(v2c_ctx *ctx, const double *gx, const double *gy) {
  if (!ctx || !gx || !gy) return V2C_ERR_ARG;
  for (int i = 0; i + 1 < ctx->xn; i++)
    if (!(gx[i + 1] > gx[i])) return fail(ctx, V2C_ERR_ARG);
  for (int i = 0; i + 1 < ctx->yn; i++)
    if (!(gy[i + 1] > gy[i])) return fail(ctx, V2C_ERR_ARG);
  if (gx[ctx->xn - 1] != ctx->p.xsize || gy[ctx->yn - 1] != ctx->p.ysize)
    return fail(ctx, V2C_ERR_ARG);
  ctx->h_gx.assign(gx, gx + ctx->xn);
  ctx->h_gy.assign(gy, gy + ctx->yn);
  std::vector<float> wx(ctx->ncx), wy(ctx->ncy), gxf(ctx->xn), gyf(ctx->yn);
  for (int i = 0; i < ctx->ncx; i++) wx[i] = (float)(gx[i + 1] - gx[i]);
  for (int i = 0; i < ctx->ncy; i++) wy[i] = (float)(gy[i + 1] - gy[i]);
  for (int i = 0; i < ctx->xn; i++) gxf[i] = (float)gx[i];
  for (int i = 0; i < ctx->yn; i++) gyf[i] = (float)gy[i];
  CK(cudaMemcpy(ctx->d_gx, gx, sizeof(double) * ctx->xn, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_gy, gy, sizeof(double) * ctx->yn, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_wx, wx.data(), sizeof(float) * ctx->ncx, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_wy, wy.data(), sizeof(float) * ctx->ncy, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_gxf, gxf.data(), sizeof(float) * ctx->xn, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_gyf, gyf.data(), sizeof(float) * ctx->yn, cudaMemcpyHostToDevice));
  ctx->have_grid = true;
  return V2C_OK;
}

extern "C" int v2c_set_rock_table(v2c_ctx *ctx, const double *rt) {
  if (!ctx || !rt) return V2C_ERR_ARG;
  ctx->h_rt.assign(rt, rt + V2C_RT_N * V2C_MAXTMR);
  std::vector<float> f((size_t)RK_N * V2C_MAXTMR, 0.f);
  auto R = [&](int r, int t) { return rt[r * V2C_MAXTMR + t]; };
  auto F = [&](int k, int t) -> float & { return f[(size_t)k * V2C_MAXTMR + t]; };
  for (int t = 0; t < V2C_MAXTMR; t++) {
    double nu = R(V2C_RT_NU, t), dh = R(V2C_RT_DH, t), dv = R(V2C_RT_DV, t);
    double ss = R(V2C_RT_SS, t), mm = R(V2C_RT_MM, t), gg = R(V2C_RT_GG, t);
    F(RK_GG, t) = (float)gg;
    F(RK_INV_GG, t) = (float)(1.0 / gg);  // inf for G = 0, as nu/G is in the reference
    F(RK_NU, t) = (float)nu;
    F(RK_LNNU, t) = nu > 0 ? (float)log(nu) : 0.f;
    F(RK_DH, t) = (float)dh; F(RK_DV, t) = (float)dv;
    F(RK_LNSS, t) = ss > 0 ? (float)log(ss) : 0.f;
    F(RK_MM, t) = (float)mm;
    F(RK_RO, t) = (float)R(V2C_RT_RO, t); F(RK_BB, t) = (float)R(V2C_RT_BB, t);
    F(RK_AA, t) = (float)R(V2C_RT_AA, t); F(RK_CP, t) = (float)R(V2C_RT_CP, t);
    F(RK_KT, t) = (float)R(V2C_RT_KT, t); F(RK_HT, t) = (float)R(V2C_RT_HT, t);
    F(RK_KF, t) = (float)R(V2C_RT_KF, t); F(RK_KP, t) = (float)R(V2C_RT_KP, t);
    F(RK_N0, t) = (float)R(V2C_RT_N0, t); F(RK_N1, t) = (float)R(V2C_RT_N1, t);
    F(RK_IM, t) = (float)R(V2C_RT_IM, t);
    // float pairs of the Arrhenius exponent's constants
    auto pair = [&](int khi, int klo, double d) {
      F(khi, t) = (float)d;
      F(klo, t) = std::isfinite(d) ? (float)(d - (double)(float)d) : 0.f;
    };
    pair(RK_DH, RK_DH_LO, dh);
    pair(RK_DV, RK_DV_LO, dv);
    // diffusion-creep viscosity 0.5 k1 e1, k1 = nu / ss^(mm-1)
    // (density_ductilevisc_calc.c:116-127), as ln(0.5 k1) + (E+PV)/RT
    const double lnk = (nu > 0 && ss > 0) ? log(0.5) + log(nu) - (mm - 1.0) * log(ss) : 0.0;
    pair(RK_LNK, RK_LNK_LO, lnk);
    pair(RK_LNG, RK_LNG_LO, gg > 0 ? log(gg) : -INFINITY);
    pair(RK_SS, RK_SS_LO, ss);
    pair(RK_EM, RK_EM_LO, mm != 0 ? (mm - 1.0) / mm : 0.0);
    pair(RK_MM1, RK_MM1_LO, mm - 1.0);
    pair(RK_LNSS, RK_LNSS_LO, ss > 0 ? log(ss) : 0.0);
    int kind;
    // branch selection of ductilevisc (density_ductilevisc_calc.c:44-66)
    if (t == 1) kind = VISC_STICKY;
    else if (dh == 0 && dv == 0 && (ss == 0 || mm == 1.0)) kind = VISC_NEWTON;
    else if (nu > 0 && (dh != 0 || dv != 0) && ss != 0 && mm != 1.0) kind = VISC_POWER;
    else kind = VISC_UNDEF;
    F(RK_KIND, t) = (float)kind;
  }
  CK(cudaMemcpy(ctx->d_rock, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
  ctx->have_rock = true;
  return V2C_OK;
}

extern "C" int v2c_set_bonds(v2c_ctx *ctx, const long *bondm, const long *bondn,
                             const double *bondv, long bondnum) {
  if (!ctx || !bondm || bondnum < 0 || (bondnum > 0 && (!bondn || !bondv))) return V2C_ERR_ARG;
  ctx->h_bondm.assign(bondm, bondm + ctx->nn * 4);
  ctx->h_bondn.assign(bondn, bondn + bondnum * 3);
  ctx->h_bondv.assign(bondv, bondv + bondnum * 4);
  ctx->bondnum = bondnum;
  for (long i = 0; i < ctx->nn * 4; i++)
    if (bondm[i] < 0 || bondm[i] >= bondnum) return fail(ctx, V2C_ERR_ARG);
  ctx->have_bonds = true;
  ctx->bc_built_compressible = -1;
  return V2C_OK;
}

// ------------------------------------------------ boundary rows (host side)
namespace {

struct Resolved {
  double c;
  std::vector<std::pair<long, double>> terms;  // (row, coef), identity rows
};

struct BcBlock {
  int field;
  std::vector<char> present;
  std::vector<long> bond;
  int kind;  // 0 vx, 1 vy, 2 P, 3 T
};

long decode(int kind, long bn, long nn) {
  switch (kind) {
    case 0: return ((bn - 1) - 1) / 3;
    case 1: return ((bn - 1) - 2) / 3;
    case 2: return (bn - 1) / 3;
    default: return bn - 1 - nn * 3;
  }
}

// resolve a boundary row into constant + identity-row terms, references in
// increasing row order as the frontal elimination folds them in
bool resolve(const v2c_ctx *ctx, const BcBlock &B, long r, std::map<long, Resolved> &memo,
             std::vector<char> &busy, Resolved &out) {
  auto it = memo.find(r);
  if (it != memo.end()) { out = it->second; return true; }
  if (busy[r]) return false;
  busy[r] = 1;
  long b = B.bond[r];
  Resolved res;
  res.c = ctx->h_bondv[b * 4 + 0];
  std::vector<std::pair<long, double>> refs;
  for (int k = 0; k < 3; k++) {
    long bn = ctx->h_bondn[b * 3 + k];
    if (bn) refs.push_back({decode(B.kind, bn, ctx->nn), ctx->h_bondv[b * 4 + k + 1]});
  }
  std::sort(refs.begin(), refs.end(),
            [](const std::pair<long, double> &a, const std::pair<long, double> &b2) { return a.first < b2.first; });
  for (auto &rf : refs) {
    long q = rf.first;
    if (q < 0 || q >= ctx->nn || !B.present[q]) continue;  // absent rows solve to 0
    if (!B.bond[q]) {
      res.terms.push_back({q, rf.second});
    } else {
      Resolved sub;
      if (!resolve(ctx, B, q, memo, busy, sub)) return false;
      res.c = res.c - sub.c * (-rf.second);
      for (auto &t : sub.terms) res.terms.push_back({t.first, t.second * rf.second});
    }
  }
  busy[r] = 0;
  memo[r] = res;
  out = res;
  return true;
}

int build_bc(v2c_ctx *ctx) {
  const int cm = ctx->p.compressiblemode == 1, tm = ctx->p.tempmod != 0;
  if (ctx->bc_built_compressible == cm && ctx->bc_built_tempmod == tm) return V2C_OK;
  std::vector<int> fld, nref, rfield;
  std::vector<long> node, rnode;
  std::vector<float> cst, rcoef;
  const long nn = ctx->nn;
  const int xn = ctx->xn, yn = ctx->yn;
  for (int kind = 0; kind < 4; kind++) {
    if (kind == 3 && !tm) continue;
    BcBlock B;
    B.kind = kind;
    B.field = kind == 0 ? V2C_NF_MVX : kind == 1 ? V2C_NF_MVY : kind == 2 ? V2C_NF_SPPE : V2C_NF_TK;
    B.present.assign(nn, 0);
    B.bond.assign(nn, 0);
    for (int m1 = 0; m1 < xn; m1++)
      for (int m2 = 0; m2 < yn; m2++) {
        long m3 = (long)m1 * yn + m2;
        if (kind == 0 && m2 < yn - 1) { B.present[m3] = 1; B.bond[m3] = ctx->h_bondm[m3 * 3 + 1]; }
        if (kind == 1 && m1 < xn - 1) { B.present[m3] = 1; B.bond[m3] = ctx->h_bondm[m3 * 3 + 2]; }
        if (kind == 2 && m1 && m2) { B.present[m3] = 1; B.bond[m3] = cm ? 0 : ctx->h_bondm[m3 * 3]; }
        if (kind == 3) { B.present[m3] = 1; B.bond[m3] = ctx->h_bondm[3 * nn + m3]; }
      }
    std::map<long, Resolved> memo;
    std::vector<char> busy(nn, 0);
    for (long r = 0; r < nn; r++) {
      if (!B.present[r] || !B.bond[r]) continue;
      Resolved res;
      if (!resolve(ctx, B, r, memo, busy, res)) return V2C_ERR_UNSUPPORTED;
      if ((int)res.terms.size() > V2C_BC_MAXREF) return V2C_ERR_UNSUPPORTED;
      fld.push_back(B.field);
      node.push_back(r);
      cst.push_back((float)res.c);
      nref.push_back((int)res.terms.size());
      for (int k = 0; k < V2C_BC_MAXREF; k++) {
        bool h = k < (int)res.terms.size();
        rfield.push_back(B.field);
        rnode.push_back(h ? res.terms[k].first : 0);
        rcoef.push_back(h ? (float)res.terms[k].second : 0.f);
      }
    }
  }
  int n = (int)fld.size();
  if (ctx->bc_mem) { cudaFree(ctx->bc_mem); ctx->bc_mem = nullptr; }
  if (ctx->d_bc_scratch) { cudaFree(ctx->d_bc_scratch); ctx->d_bc_scratch = nullptr; }
  ctx->bc_n = n;
  ctx->bc = BcRows{};
  ctx->bc.n = n;
  if (n == 0) { ctx->bc_built_compressible = cm; ctx->bc_built_tempmod = tm; return V2C_OK; }
  size_t M = V2C_BC_MAXREF;
  size_t bytes = n * (sizeof(int) + sizeof(long) + sizeof(float) + sizeof(int)) +
                 n * M * (sizeof(int) + sizeof(long) + sizeof(float)) + 64;
  char *mem;
  if (cudaMalloc((void **)&mem, bytes) != cudaSuccess) return V2C_ERR_CUDA;
  if (cudaMalloc((void **)&ctx->d_bc_scratch, sizeof(float) * n) != cudaSuccess) return V2C_ERR_CUDA;
  ctx->bc_mem = mem;
  size_t off = 0;
  auto put = [&](const void *src, size_t sz) {
    off = (off + 7) & ~size_t(7);
    void *dst = mem + off;
    cudaMemcpy(dst, src, sz, cudaMemcpyHostToDevice);
    off += sz;
    return dst;
  };
  ctx->bc.field = (const int *)put(fld.data(), n * sizeof(int));
  ctx->bc.node = (const long *)put(node.data(), n * sizeof(long));
  ctx->bc.c = (const float *)put(cst.data(), n * sizeof(float));
  ctx->bc.nref = (const int *)put(nref.data(), n * sizeof(int));
  ctx->bc.rfield = (const int *)put(rfield.data(), n * M * sizeof(int));
  ctx->bc.rnode = (const long *)put(rnode.data(), n * M * sizeof(long));
  ctx->bc.rcoef = (const float *)put(rcoef.data(), n * M * sizeof(float));
  ctx->bc_built_compressible = cm;
  ctx->bc_built_tempmod = tm;
  return V2C_OK;
}

}  // namespace

// ============================================================ marker arrays
// the compaction scratch of immobile markers, one allocation for the
// context's capacity (ImmBufs in v2c_kernels.h)
static int alloc_immobile(v2c_ctx *ctx) {
  const long cap = ctx->cap > 0 ? ctx->cap : 1;
  const long nb = scan_blocks(cap) + 1;
  const size_t words = (size_t)cap * 7 + 2 * (size_t)(cap + 1) + (size_t)nb + 2;
  void *mem = nullptr;
  if (cudaMalloc(&mem, sizeof(int32_t) * words) != cudaSuccess) return V2C_ERR_CUDA;
  int32_t *w = static_cast<int32_t *>(mem);
  ImmBufs &b = ctx->imm;
  b.spawn = w; w += cap;
  b.out = w; w += cap;
  b.sp_cell = w; w += cap;
  b.sp_u = reinterpret_cast<float *>(w); w += cap;
  b.sp_v = reinterpret_cast<float *>(w); w += cap;
  b.src = w; w += cap;
  b.inv = w; w += cap;
  b.spawn_rank = w; w += cap + 1;
  b.out_rank = w; w += cap + 1;
  b.blocksum = w; w += nb;
  b.totals = w;
  ctx->imm_mem = mem;
  return V2C_OK;
}

extern "C" int v2c_upload_markers(v2c_ctx *ctx, const double *const *fields,
                                  const signed char *markt, long n) {
  if (!ctx || !fields || !markt || n < 0) return V2C_ERR_ARG;
  if (!fields[V2C_MF_X] || !fields[V2C_MF_Y]) return fail(ctx, V2C_ERR_ARG);
  if (n > ctx->cap) return fail(ctx, V2C_ERR_CAPACITY);
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  long n_imm = 0;
  for (long i = 0; i < n; i++) {
    if (markt[i] < 0) return fail(ctx, V2C_ERR_UNSUPPORTED);
    n_imm += markt[i] >= 100;
  }
  if (n_imm > 0 && !ctx->imm_mem) {
    int rc = alloc_immobile(ctx);
    if (rc) return fail(ctx, rc);
  }
  ctx->n_immobile = n_imm;
  cudaStream_t st = ctx->stream;
  Markers &m = ctx->m;
  Grid g = make_grid(ctx);
  ctx->n = n;
  CK(cudaMemcpyAsync(ctx->d_stage64, fields[V2C_MF_X], sizeof(double) * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_stage64b, fields[V2C_MF_Y], sizeof(double) * n, cudaMemcpyHostToDevice, st));
  launch_assign(g, ctx->d_stage64, ctx->d_stage64b, n, m, ctx->d_stat, st);
  CK(cudaMemcpyAsync(m.type, markt, n, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(m.flags, 0, n, st));
  // the temperature and markv as float pairs, the other fields in FP32
  struct F { int id; float *dst; float *lo; } ff[] = {
      {V2C_MF_K, m.tk, m.tk_lo}, {V2C_MF_V, m.mv, m.mv_lo}, {V2C_MF_E, m.e, nullptr},
      {V2C_MF_P, m.p, nullptr},
      {V2C_MF_XX, m.sxx, nullptr}, {V2C_MF_XY, m.sxy, nullptr}, {V2C_MF_EXX, m.exx, nullptr},
      {V2C_MF_EXY, m.exy, nullptr}, {V2C_MF_VX, m.vx, nullptr}, {V2C_MF_VY, m.vy, nullptr},
      {V2C_MF_PHI, m.phi, nullptr}, {V2C_MF_C, m.coh, nullptr}, {V2C_MF_SLIPV, m.slipv, nullptr}};
  for (auto &f : ff) {
    if (fields[f.id]) {
      CK(cudaMemcpyAsync(ctx->d_stage64, fields[f.id], sizeof(double) * n, cudaMemcpyHostToDevice, st));
      if (f.lo) launch_f64_to_pair(ctx->d_stage64, f.dst, f.lo, n, st);
      else launch_f64_to_f32(ctx->d_stage64, f.dst, n, st);
    } else {
      CK(cudaMemsetAsync(f.dst, 0, sizeof(float) * n, st));
      if (f.lo) CK(cudaMemsetAsync(f.lo, 0, sizeof(float) * n, st));
    }
  }
  CK(cudaMemsetAsync(m.mnu, 0, sizeof(float) * n, st));
  CK(cudaMemsetAsync(m.mkt, 0, sizeof(float) * n, st));
  CK(cudaMemsetAsync(m.mro, 0, sizeof(float) * n, st));
  // sort once and store the markers physically in cell order
  launch_sort(m.cell_in, m.u_in, m.v_in, n, ctx->ncell, ctx->sb, ctx->d_stat, st);
  const int32_t *perm = ctx->sb.perm;
  float *tmpf = (float *)ctx->d_stage64;
  int32_t *tmpi = (int32_t *)ctx->d_stage64;
  float *fl[] = {m.u_in, m.v_in, m.tk, m.tk_lo, m.mv, m.mv_lo, m.e, m.p, m.sxx, m.sxy, m.exx,
                 m.exy, m.vx, m.vy, m.phi, m.coh, m.slipv};
  for (float *f : fl) {
    launch_gather_f32(f, perm, tmpf, n, st);
    CK(cudaMemcpyAsync(f, tmpf, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  }
  int32_t *il[] = {m.cell_in, m.id};
  for (int32_t *f : il) {
    launch_gather_i32(f, perm, tmpi, n, st);
    CK(cudaMemcpyAsync(f, tmpi, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
  }
  launch_gather_i8(m.type, perm, (int8_t *)tmpi, n, st);
  CK(cudaMemcpyAsync(m.type, tmpi, n, cudaMemcpyDeviceToDevice, st));
  // the physical order is now sorted: sort again to get the identity perm
  launch_sort(m.cell_in, m.u_in, m.v_in, n, ctx->ncell, ctx->sb, ctx->d_stat, st);
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  ctx->have_markers = true;
  ctx->sorted = true;
  ctx->props_valid = false;
  return V2C_OK;
}

extern "C" int v2c_download_markers(v2c_ctx *ctx, double *const *fields, signed char *markt,
                                    long n) {
  if (!ctx || !fields || n != ctx->n) return V2C_ERR_ARG;
  if (!ctx->have_markers) return fail(ctx, V2C_ERR_STATE);
  cudaStream_t st = ctx->stream;
  Markers &m = ctx->m;
  Grid g = make_grid(ctx);
  if (fields[V2C_MF_X] || fields[V2C_MF_Y]) {
    launch_positions(g, m, n, ctx->d_stage64, ctx->d_stage64b, st);
    if (fields[V2C_MF_X])
      CK(cudaMemcpyAsync(fields[V2C_MF_X], ctx->d_stage64, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (fields[V2C_MF_Y])
      CK(cudaMemcpyAsync(fields[V2C_MF_Y], ctx->d_stage64b, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  struct F { int id; const float *src; const float *lo; } ff[] = {
      {V2C_MF_K, m.tk, m.tk_lo}, {V2C_MF_V, m.mv, m.mv_lo}, {V2C_MF_E, m.e, nullptr},
      {V2C_MF_P, m.p, nullptr},
      {V2C_MF_XX, m.sxx, nullptr}, {V2C_MF_XY, m.sxy, nullptr}, {V2C_MF_EXX, m.exx, nullptr},
      {V2C_MF_EXY, m.exy, nullptr}, {V2C_MF_VX, m.vx, nullptr}, {V2C_MF_VY, m.vy, nullptr},
      {V2C_MF_PHI, m.phi, nullptr}, {V2C_MF_C, m.coh, nullptr}, {V2C_MF_SLIPV, m.slipv, nullptr}};
  for (auto &f : ff) {
    if (!fields[f.id]) continue;
    if (f.lo) launch_unpermute_pair(f.src, f.lo, m.id, ctx->d_stage64, n, st);
    else launch_unpermute_f32(f.src, m.id, ctx->d_stage64, n, st);
    CK(cudaMemcpyAsync(fields[f.id], ctx->d_stage64, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  if (markt) {
    launch_unpermute_i8(m.type, m.id, (int8_t *)ctx->d_stage64, n, st);
    CK(cudaMemcpyAsync(markt, ctx->d_stage64, n, cudaMemcpyDeviceToHost, st));
  }
  if (fields[V2C_MF_D] || fields[V2C_MF_W]) {
    std::vector<uint8_t> fl(n);
    launch_unpermute_u8(m.flags, m.id, (uint8_t *)ctx->d_stage64b, n, st);
    CK(cudaMemcpyAsync(fl.data(), ctx->d_stage64b, n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (long i = 0; i < n; i++) {
      if ((fl[i] & (MFLAG_RESET | MFLAG_DNEG)) && fields[V2C_MF_D]) fields[V2C_MF_D][i] = -1.0;
      if ((fl[i] & MFLAG_RESET) && fields[V2C_MF_W]) fields[V2C_MF_W][i] = -1.0;
    }
  }
  CK(cudaStreamSynchronize(st));
  return V2C_OK;
}

extern "C" int v2c_download_marker_properties(v2c_ctx *ctx, double *mnu, double *mkt, long n) {
  if (!ctx || n != ctx->n) return V2C_ERR_ARG;
  if (!ctx->have_markers || !ctx->props_valid) return fail(ctx, V2C_ERR_STATE);
  cudaStream_t st = ctx->stream;
  const float *src[2] = {ctx->m.mnu, ctx->m.mkt};
  double *dst[2] = {mnu, mkt};
  for (int k = 0; k < 2; k++) {
    if (!dst[k]) continue;
    launch_unpermute_f32(src[k], ctx->m.id, ctx->d_stage64, n, st);
    CK(cudaMemcpyAsync(dst[k], ctx->d_stage64, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  return V2C_OK;
}

extern "C" int v2c_download_cells(v2c_ctx *ctx, int32_t *cell, long n) {
  if (!ctx || !cell || n != ctx->n) return V2C_ERR_ARG;
  launch_unpermute_i32(ctx->m.cell_in, ctx->m.id, (int32_t *)ctx->d_stage64, n, ctx->stream);
  CK(cudaMemcpyAsync(cell, ctx->d_stage64, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return V2C_OK;
}

// ============================================================== node arrays
// node fields live in FP32 on the device; they are converted on the way in
// and out (the conversion kernels run on the context stream)
// keep the FP64 copy of an uploaded velocity or temperature field (staged
// at dev64)
static int keep_node64(v2c_ctx *ctx, int field, const double *dev64) {
  if (field == V2C_NF_TK || field == V2C_NF_TK2) {
    const int k = field == V2C_NF_TK ? 0 : 1;
    if (!ctx->d_tk64) CK(cudaMalloc(&ctx->d_tk64, sizeof(double) * 2 * ctx->nn));
    CK(cudaMemcpyAsync(ctx->d_tk64 + k * ctx->nn, dev64, sizeof(double) * ctx->nn,
                       cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->tk64_ok[k] = true;
    return V2C_OK;
  }
  if (field != V2C_NF_VX && field != V2C_NF_VY) return V2C_OK;
  const int k = field == V2C_NF_VX ? 0 : 1;
  if (!ctx->d_vel64) CK(cudaMalloc(&ctx->d_vel64, sizeof(double) * 2 * ctx->nn));
  CK(cudaMemcpyAsync(ctx->d_vel64 + k * ctx->nn, dev64, sizeof(double) * ctx->nn,
                     cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->vel64_ok[k] = true;
  return V2C_OK;
}

extern "C" int v2c_upload_node_field(v2c_ctx *ctx, int field, const double *src) {
  if (!ctx || !src || field < 0 || field >= V2C_NF_N) return V2C_ERR_ARG;
  ctx->dsxx_valid = false;
  CK(cudaMemcpyAsync(ctx->d_node64, src, sizeof(double) * ctx->nn, cudaMemcpyHostToDevice,
                     ctx->stream));
  if (int rc = keep_node64(ctx, field, ctx->d_node64)) return fail(ctx, rc);
  launch_node_to_f32(ctx->d_node64, ctx->d_node + (long)field * ctx->nn, ctx->nn, ctx->stream);
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_download_node_field(v2c_ctx *ctx, int field, double *dst) {
  if (!ctx || !dst || field < 0 || field >= V2C_NF_N) return V2C_ERR_ARG;
  launch_node_to_f64(ctx->d_node + (long)field * ctx->nn, ctx->d_node64, ctx->nn, ctx->stream);
  ctx->launches += 1;
  CK(cudaMemcpyAsync(dst, ctx->d_node64, sizeof(double) * ctx->nn, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return V2C_OK;
}

static int node_field_list_ok(int count, const int *fields, const void *const *ptrs) {
  if (count < 0 || count > V2C_NF_N || (count > 0 && (!fields || !ptrs))) return 0;
  for (int k = 0; k < count; k++)
    if (fields[k] < 0 || fields[k] >= V2C_NF_N || !ptrs[k]) return 0;
  return 1;
}

static int grow_node_stage(v2c_ctx *ctx, int count) {
  if (count <= ctx->nstage_cap) return V2C_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_nstage) cudaFree(ctx->d_nstage);
  ctx->d_nstage = nullptr;
  ctx->nstage_cap = 0;
  CK(cudaMalloc(&ctx->d_nstage, sizeof(double) * ctx->nn * count));
  ctx->nstage_cap = count;
  return V2C_OK;
}

extern "C" int v2c_upload_node_fields(v2c_ctx *ctx, int count, const int *fields,
                                      const double *const *src) {
  if (!ctx) return V2C_ERR_ARG;
  if (!node_field_list_ok(count, fields, (const void *const *)src)) return fail(ctx, V2C_ERR_ARG);
  if (count == 0) return V2C_OK;
  ctx->dsxx_valid = false;
  int rc = grow_node_stage(ctx, count);
  if (rc) return fail(ctx, rc);
  for (int k = 0; k < count; k++)
    CK(cudaMemcpyAsync(ctx->d_nstage + (long)k * ctx->nn, src[k], sizeof(double) * ctx->nn,
                       cudaMemcpyHostToDevice, ctx->stream));
  launch_fields_to_f32(ctx->d_nstage, ctx->nn, fields, count, ctx->d_node, ctx->stream);
  ctx->launches += 1;
  for (int k = 0; k < count; k++)
    if (int rc2 = keep_node64(ctx, fields[k], ctx->d_nstage + (long)k * ctx->nn)) return fail(ctx, rc2);
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_download_node_fields_async(v2c_ctx *ctx, int count, const int *fields,
                                              double *const *dst) {
  if (!ctx) return V2C_ERR_ARG;
  if (!node_field_list_ok(count, fields, (const void *const *)dst)) return fail(ctx, V2C_ERR_ARG);
  if (count == 0) return V2C_OK;
  cudaStream_t st = ctx->stream;
  if (!ctx->xfer) {
    CK(cudaStreamCreateWithFlags(&ctx->xfer, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->ev_conv, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming));
  }
  if (count > ctx->astage_fields) {
    // a larger staging area: the earlier copies out of the old one first
    CK(cudaStreamSynchronize(ctx->xfer));
    CK(cudaStreamSynchronize(st));
    if (ctx->d_astage) CK(cudaFree(ctx->d_astage));
    ctx->d_astage = nullptr;
    CK(cudaMalloc(&ctx->d_astage, sizeof(double) * ctx->nn * count));
    ctx->astage_fields = count;
  }
  // the staging area is reused: the conversion waits for the copies of the
  // previous asynchronous download
  if (ctx->dl_pending) CK(cudaStreamWaitEvent(st, ctx->ev_copy, 0));
  launch_fields_to_f64(ctx->d_node, ctx->nn, fields, count, ctx->d_astage, st);
  ctx->launches += 1;
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev_conv, st));
  CK(cudaStreamWaitEvent(ctx->xfer, ctx->ev_conv, 0));
  for (int k = 0; k < count; k++)
    CK(cudaMemcpyAsync(dst[k], ctx->d_astage + (long)k * ctx->nn, sizeof(double) * ctx->nn,
                       cudaMemcpyDeviceToHost, ctx->xfer));
  CK(cudaEventRecord(ctx->ev_copy, ctx->xfer));
  ctx->dl_pending = true;
  return V2C_OK;
}

extern "C" int v2c_wait_downloads(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  if (ctx->dl_pending) {
    CK(cudaEventSynchronize(ctx->ev_copy));
    ctx->dl_pending = false;
  }
  return V2C_OK;
}

extern "C" int v2c_download_node_fields(v2c_ctx *ctx, int count, const int *fields,
                                        double *const *dst) {
  if (!ctx) return V2C_ERR_ARG;
  if (!node_field_list_ok(count, fields, (const void *const *)dst)) return fail(ctx, V2C_ERR_ARG);
  if (count == 0) return V2C_OK;
  int rc = grow_node_stage(ctx, count);
  if (rc) return fail(ctx, rc);
  launch_fields_to_f64(ctx->d_node, ctx->nn, fields, count, ctx->d_nstage, ctx->stream);
  ctx->launches += 1;
  CK(cudaGetLastError());
  for (int k = 0; k < count; k++)
    CK(cudaMemcpyAsync(dst[k], ctx->d_nstage + (long)k * ctx->nn, sizeof(double) * ctx->nn,
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return V2C_OK;
}

// ============================================================ the MIC step
static int ready(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  if (!ctx->have_grid || !ctx->have_rock || !ctx->have_markers) return fail(ctx, V2C_ERR_STATE);
  return V2C_OK;
}

static void swap_positions(v2c_ctx *ctx) {
  std::swap(ctx->m.cell_in, ctx->m.cell_out);
  std::swap(ctx->m.u_in, ctx->m.u_out);
  std::swap(ctx->m.v_in, ctx->m.v_out);
}

extern "C" int v2c_marker2nodes(v2c_ctx *ctx) {
  int rc = ready(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->stream;
  if (!ctx->sorted) {
    Prof pr(ctx, V2C_PROF_SORT);
    launch_sort(ctx->m.cell_in, ctx->m.u_in, ctx->m.v_in, ctx->n, ctx->ncell, ctx->sb,
                ctx->d_stat, st);
    ctx->launches += ctx->n > 0 ? 6 : 3;
    ctx->sorted = true;
  }
  if (ctx->have_bonds) {
    rc = build_bc(ctx);
    if (rc) return fail(ctx, rc);
  }
  M2NArgs a;
  a.g = make_grid(ctx);
  a.N = make_nodes(ctx);
  a.m = ctx->m;
  a.R = Rock{ctx->d_rock};
  a.S = make_scal(ctx->p, ctx->h_rt);
  a.perm = ctx->sb.perm;
  a.start = ctx->sb.start;
  a.qstart = ctx->sb.qstart;
  a.sticky_key = ctx->d_sticky;
  a.stat = ctx->d_stat;
  a.gxf = ctx->d_gxf;
  a.gyf = ctx->d_gyf;
  a.TX = pick_tx(ctx, 16);
  a.n = ctx->n;
  CK(cudaMemsetAsync(ctx->d_sticky, 0, sizeof(uint32_t) * ctx->nn, st));
  ctx->dsxx_valid = false;  // the scatter writes sxxe
  ctx->tk64_ok[0] = false;  // and the node temperature
  {
    PhysArgs ph;
    ph.g = a.g; ph.N = a.N; ph.m = a.m; ph.R = a.R; ph.S = a.S; ph.n = ctx->n;
    ph.sticky_key = ctx->d_sticky; ph.stat = ctx->d_stat; ph.gxf = ctx->d_gxf; ph.gyf = ctx->d_gyf;
    ph.mlp = ctx->nw.have_mlp ? ctx->nw.d_mlp : nullptr;
    // the problem list borrows the sort's slot buffer, which holds nothing
    // between sorts (capacity: one entry per marker)
    ph.list = ctx->sb.slot;
    ph.list_n = ctx->d_list_n;
    ph.guess = reinterpret_cast<float *>(ctx->sb.tmp);  // likewise free between sorts
    Prof pr(ctx, ctx->p.newton_guess == V2C_GUESS_OFF ? V2C_PROF_PHYS : V2C_PROF_NEWTON);
    launch_phys(ph, st);
    ctx->launches += ctx->p.newton_guess == V2C_GUESS_OFF ? 1 : (ph.mlp && ctx->p.newton_guess == V2C_GUESS_LEARNED ? 3 : 2);
  }
  {
    Prof pr(ctx, V2C_PROF_M2N);
    launch_m2n(a, st);
    ctx->launches += ctx->p.interpolationmod == 1 ? 4 : 1;
  }
  ctx->props_valid = true;
  {
    Prof pr(ctx, V2C_PROF_M2N_TAIL);
    launch_sticky(a.N, ctx->d_sticky, ctx->nn, st);
    ctx->launches += 1;
    if (ctx->p.Dphis > 0) { launch_dphis(a.g, a.N, st); ctx->launches += 1; }
    if (ctx->have_bonds && ctx->bc.n > 0) { launch_bc(ctx->bc, a.N, ctx->d_bc_scratch, st); ctx->launches += 2; }
  }
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_collect_newton_states(v2c_ctx *ctx, long stride, double *states_dev,
                                         long cap, long *n_out) {
  int rc = ready(ctx);
  if (rc) return rc;
  if (stride < 1 || cap < 0 || (cap > 0 && !states_dev) || !n_out) return V2C_ERR_ARG;
  PhysArgs ph;
  ph.g = make_grid(ctx); ph.N = make_nodes(ctx); ph.m = ctx->m; ph.R = Rock{ctx->d_rock};
  ph.S = make_scal(ctx->p, ctx->h_rt); ph.n = ctx->n;
  ph.sticky_key = ctx->d_sticky; ph.stat = ctx->d_stat; ph.gxf = ctx->d_gxf; ph.gyf = ctx->d_gyf;
  ph.mlp = nullptr;
  ph.xs = states_dev; ph.xs_stride = stride; ph.xs_cap = cap;
  const long slots = (ctx->n + stride - 1) / stride;
  *n_out = slots < cap ? slots : cap;
  if (*n_out > 0) {
    launch_phys(ph, ctx->stream);
    ctx->launches += 1;
  }
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_center2basic_old(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  {
    Prof pr(ctx, V2C_PROF_C2B);
    launch_c2b_old(make_grid(ctx), make_nodes(ctx), ctx->stream);
  }
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_interpolate_basic2center(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  {
    Prof pr(ctx, V2C_PROF_B2C);
    launch_b2c(make_grid(ctx), make_nodes(ctx), ctx->d_stat, ctx->stream);
  }
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_interpolate_center2basic(v2c_ctx *ctx, double dt) {
  if (!ctx) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  {
    Prof pr(ctx, V2C_PROF_B2C);
    launch_c2b(make_grid(ctx), make_nodes(ctx), dt, ctx->dsxx_valid ? 1 : 0, ctx->stream);
  }
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_recompute_stress_strainrate(v2c_ctx *ctx, double dt) {
  if (!ctx) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  {
    Prof pr(ctx, V2C_PROF_B2C);
    const bool v64 = ctx->d_vel64 && ctx->vel64_ok[0] && ctx->vel64_ok[1];
    launch_recompute(make_grid(ctx), make_nodes(ctx), make_scal(ctx->p, ctx->h_rt), dt,
                     v64 ? ctx->d_vel64 : nullptr, v64 ? ctx->d_vel64 + ctx->nn : nullptr,
                     ctx->stream);
  }
  ctx->dsxx_valid = true;
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_copyarrays(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  launch_copyarrays(make_grid(ctx), make_nodes(ctx), ctx->stream);
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_compute_before_solve(v2c_ctx *ctx, double dt, int rk) {
  if (!ctx) return V2C_ERR_ARG;
  {
    Prof pr(ctx, V2C_PROF_BEFORE);
    launch_before_solve(make_grid(ctx), make_nodes(ctx), make_scal(ctx->p, ctx->h_rt), dt, rk,
                        ctx->d_stat, ctx->stream);
  }
  ctx->launches += 1;
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_compute_after_solve(v2c_ctx *ctx, double dt, int rk, double *deltas) {
  if (!ctx) return V2C_ERR_ARG;
  {
    Prof pr(ctx, V2C_PROF_AFTER);
    launch_after_solve(make_grid(ctx), make_nodes(ctx), make_scal(ctx->p, ctx->h_rt), dt, rk,
                       ctx->d_red, ctx->stream);
  }
  ctx->launches += 2;
  CK(cudaGetLastError());
  if (deltas) {
    double h[2];
    CK(cudaMemcpyAsync(h, ctx->d_red, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *deltas = h[1] > 0 ? sqrt(h[0] / h[1]) : 0.0;
  }
  return V2C_OK;
}

static int n2m_move(v2c_ctx *ctx, int do_n2m, int do_move) {
  int rc = ready(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->stream;
  if (!ctx->sorted) {
    Prof pr(ctx, V2C_PROF_SORT);
    launch_sort(ctx->m.cell_in, ctx->m.u_in, ctx->m.v_in, ctx->n, ctx->ncell, ctx->sb,
                ctx->d_stat, st);
    ctx->launches += ctx->n > 0 ? 6 : 3;
    ctx->sorted = true;
  }
  N2MArgs a;
  a.g = make_grid(ctx);
  a.N = make_nodes(ctx);
  a.m = ctx->m;
  a.R = Rock{ctx->d_rock};
  a.S = make_scal(ctx->p, ctx->h_rt);
  a.perm = ctx->sb.perm;
  a.start = ctx->sb.start;
  a.qstart = ctx->sb.qstart;
  a.stat = ctx->d_stat;
  a.gyf = ctx->d_gyf;
  a.quad = ctx->d_quad;
  a.n = ctx->n;
  a.TX = pick_tx(ctx, 32);
  a.do_n2m = 1;
  if (do_n2m && ctx->p.interpolationmod == 1 && ctx->p.antidiffinter == 1) {
    // the full-stencil back-scatter: one payload record per marker
    if (!ctx->d_bs) return fail(ctx, V2C_ERR_STATE);
    a.bs = ctx->d_bs;
  }
  if (do_n2m) {
    Prof pr(ctx, V2C_PROF_N2M);
    launch_n2m(a, st);
    ctx->launches += a.bs ? 3 : 1;
  }
  if (do_move) {
    ctx->props_valid = false;
    const bool imm = ctx->n_immobile > 0 && ctx->n > 0;
    if (imm) {
      CK(cudaMemsetAsync(ctx->imm.spawn, 0, sizeof(int32_t) * ctx->n, st));
      CK(cudaMemsetAsync(ctx->imm.out, 0, sizeof(int32_t) * ctx->n, st));
      a.imm = ctx->imm;
      a.has_imm = 1;
    }
    {
      Prof pr(ctx, V2C_PROF_MOVE);
      launch_move(a, st);
      ctx->launches += ctx->n > 0 ? 2 : 1;
    }
    CK(cudaGetLastError());
    if (imm) {
      // spawned markers appended, out-of-model slots refilled (one stream
      // synchronisation for the new marker count)
      long added = 0;
      rc = launch_immobile_compact(ctx->m, ctx->n, ctx->cap, ctx->imm, &added, st);
      if (rc) return fail(ctx, rc);
      ctx->n += added;
      ctx->launches += 8;
    }
    swap_positions(ctx);
    // next step's order: counting sort of the new cells
    Prof pr(ctx, V2C_PROF_SORT);
    launch_sort(ctx->m.cell_in, ctx->m.u_in, ctx->m.v_in, ctx->n, ctx->ncell, ctx->sb,
                ctx->d_stat, st);
    ctx->launches += ctx->n > 0 ? 6 : 3;
  }
  CK(cudaGetLastError());
  return V2C_OK;
}

extern "C" int v2c_nodes2markers(v2c_ctx *ctx) { return n2m_move(ctx, 1, 0); }
extern "C" int v2c_moveandrotatemarkers(v2c_ctx *ctx) { return n2m_move(ctx, 0, 1); }
extern "C" int v2c_nodes2markers_move(v2c_ctx *ctx) { return n2m_move(ctx, 1, 1); }

extern "C" int v2c_calc_timestep(v2c_ctx *ctx, int oldornew, const v2c_timestep_ctl *ctl,
                                 v2c_timestep_info *info) {
  if (!ctx || !ctl || !info || (oldornew != 0 && oldornew != 1)) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  memset(info, 0, sizeof(*info));
  int rc;
  {
    Prof pr(ctx, V2C_PROF_TIMESTEP);
    rc = calc_timestep_device(make_grid(ctx), make_nodes(ctx), make_scal(ctx->p, ctx->h_rt), *ctl,
                              oldornew, ctx->d_ts, TIMESTEP_SCRATCH, info, ctx->stream);
  }
  ctx->launches += 2;
  if (rc) return fail(ctx, rc);
  return V2C_OK;
}

extern "C" int v2c_synchronize(v2c_ctx *ctx) {
  if (!ctx) return V2C_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->dl_pending) {
    CK(cudaEventSynchronize(ctx->ev_copy));
    ctx->dl_pending = false;
  }
  CK(cudaGetLastError());
  return V2C_OK;
}

// ================================================== marker temperature
extern "C" int v2c_marker_temperature(v2c_ctx *ctx, double heatdif) {
  int rc = ready(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->stream;
  if (!ctx->sorted) {
    launch_sort(ctx->m.cell_in, ctx->m.u_in, ctx->m.v_in, ctx->n, ctx->ncell, ctx->sb,
                ctx->d_stat, st);
    ctx->launches += ctx->n > 0 ? 6 : 3;
    ctx->sorted = true;
  }
  TempArgs a;
  a.g = make_grid(ctx);
  a.N = make_nodes(ctx);
  a.m = ctx->m;
  a.perm = ctx->sb.perm;
  a.start = ctx->sb.start;
  a.n = ctx->n;
  a.ncell = ctx->ncell;
  a.heatdif = (float)heatdif;
  a.dt = (float)ctx->p.timestep;
  a.tdeep = (float)ctx->p.tdeep;
  a.tdeep64 = ctx->p.tdeep;
  if (ctx->d_tk64 && ctx->tk64_ok[0] && ctx->tk64_ok[1]) {
    a.tk64 = ctx->d_tk64;
    a.tk2_64 = ctx->d_tk64 + ctx->nn;
  }
  // the sort's slot buffers hold nothing between sorts (one entry per marker)
  a.dtk1 = reinterpret_cast<float *>(ctx->sb.tmp);
  a.wt = reinterpret_cast<float *>(ctx->sb.slot);
  a.tol = ctx->d_tol;
  {
    Prof pr(ctx, V2C_PROF_TEMP);
    launch_temperature(a, st);
  }
  ctx->launches += ctx->n > 0 ? (heatdif != 0 ? 3 : 1) : 0;
  CK(cudaGetLastError());
  return V2C_OK;
}

// ====================================================== Stokes assembly
namespace {
// device memory of one call, freed on every return path
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(long n) {
    return cudaMalloc(&p, sizeof(T) * (size_t)(n > 0 ? n : 1));
  }
  template <class T>
  T *get() const {
    return static_cast<T *>(p);
  }
};
}  // namespace

extern "C" int v2c_stokes_assemble(v2c_ctx *ctx, const v2c_stokes_ctl *ctl, long cap, int *ia,
                                   int *ja, double *a, double *b, long *nnz) {
  if (!ctx || !ctl || !nnz || cap < 0 || (ja == nullptr) != (a == nullptr)) return V2C_ERR_ARG;
  if (!ctx->have_grid || !ctx->have_bonds) return fail(ctx, V2C_ERR_STATE);
  const long rows = 3 * ctx->nn;
  if (rows + 1 > 0x7fffffffL) return fail(ctx, V2C_ERR_CAPACITY);
  cudaStream_t st = ctx->stream;
  const long nb = ctx->bondnum;
  DevBuf bm, bn, bv, cnt, rhs, bsum, err, dja, da, ecol, evalb;
  CK(bm.alloc<long>(ctx->nn * 4));
  CK(bn.alloc<long>(nb * 3));
  CK(bv.alloc<double>(nb * 4));
  CK(cnt.alloc<int32_t>(rows + 1));
  CK(rhs.alloc<double>(rows));
  CK(bsum.alloc<int32_t>(scan_blocks(rows)));
  CK(err.alloc<int>(1));
  CK(cudaMemcpyAsync(bm.p, ctx->h_bondm.data(), sizeof(long) * ctx->nn * 4,
                     cudaMemcpyHostToDevice, st));
  if (nb > 0) {
    CK(cudaMemcpyAsync(bn.p, ctx->h_bondn.data(), sizeof(long) * nb * 3, cudaMemcpyHostToDevice,
                       st));
    CK(cudaMemcpyAsync(bv.p, ctx->h_bondv.data(), sizeof(double) * nb * 4,
                       cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  StokesArgs s;
  s.g = make_grid(ctx);
  s.N = make_nodes(ctx);
  s.bondm = bm.get<long>();
  s.bondn = bn.get<long>();
  s.bondv = bv.get<double>();
  s.bondnum = nb;
  s.mukoef = ctl->mukoef;
  s.dt = ctl->dt;
  s.gxkoef = ctl->gxkoef;
  s.gykoef = ctl->gykoef;
  s.timebond = ctl->timebond;
  s.drunkensailor = ctl->drunkensailor;
  s.timesum = ctx->p.timesum;
  s.timestep = ctx->p.timestep;
  s.nubeg = ctx->p.nubeg;
  s.inertyn = ctx->p.inertyn;
  s.compressible = ctx->p.compressiblemode;
  s.cnt = cnt.get<int32_t>();
  s.b = rhs.get<double>();
  s.ja = nullptr;
  s.a = nullptr;
  s.ell_col = nullptr;
  s.ell_val = nullptr;
  if (ja) {
    // the caller has room for the coefficients: the count pass keeps the
    // rows, so the FP64 work is done once
    CK(ecol.alloc<int32_t>(rows * STOKES_ROW_MAX));
    CK(evalb.alloc<double>(rows * STOKES_ROW_MAX));
    s.ell_col = ecol.get<int32_t>();
    s.ell_val = evalb.get<double>();
  }
  s.err = err.get<int>();
  int h_err = 0;
  int32_t total = 0;
  {
    Prof pr(ctx, V2C_PROF_STOKES);
    launch_stokes_count(s, st);
    launch_scan(s.cnt, rows, s.cnt, bsum.get<int32_t>(), st);
    ctx->launches += 4;
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&total, s.cnt + rows, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err) return fail(ctx, V2C_ERR_UNSUPPORTED);
  if (total < 0) return fail(ctx, V2C_ERR_CAPACITY);  // more than 2^31 - 1 coefficients
  *nnz = total;
  if (ia) {
    CK(cudaMemcpyAsync(ia, s.cnt, sizeof(int32_t) * (rows + 1), cudaMemcpyDeviceToHost, st));
  }
  if (b) CK(cudaMemcpyAsync(b, s.b, sizeof(double) * rows, cudaMemcpyDeviceToHost, st));
  if (ja) {
    if (cap < total) {
      CK(cudaStreamSynchronize(st));
      return fail(ctx, V2C_ERR_CAPACITY);
    }
    CK(dja.alloc<int32_t>(total));
    CK(da.alloc<double>(total));
    s.ja = dja.get<int32_t>();
    s.a = da.get<double>();
    {
      Prof pr(ctx, V2C_PROF_STOKES);
      launch_stokes_fill(s, st);
      ctx->launches += 1;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ja, s.ja, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(a, s.a, sizeof(double) * total, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  // row starts are 1-based, as gausmat4_add leaves them for Pardiso
  if (ia)
    for (long r = 0; r <= rows; r++) ia[r] += 1;
  return V2C_OK;
}

// ======================================================= seismic cycle
extern "C" int v2c_cycle_set_velocity(v2c_ctx *ctx, int regime, const double *vx,
                                      const double *vy) {
  if (!ctx || regime < 0 || regime > 1 || !vx || !vy) return V2C_ERR_ARG;
  if (!ctx->have_grid) return fail(ctx, V2C_ERR_STATE);
  const long nn = ctx->nn;
  if (!ctx->d_cyc_v[regime]) CK(cudaMalloc(&ctx->d_cyc_v[regime], sizeof(float) * 2 * nn));
  if (!ctx->d_cyc_v64[regime]) CK(cudaMalloc(&ctx->d_cyc_v64[regime], sizeof(double) * 2 * nn));
  if (!ctx->d_vel64) CK(cudaMalloc(&ctx->d_vel64, sizeof(double) * 2 * nn));
  if (!ctx->d_slip) CK(cudaMalloc(&ctx->d_slip, sizeof(double) * nn));
  if (!ctx->d_mslip && ctx->cap > 0) CK(cudaMalloc(&ctx->d_mslip, sizeof(double) * ctx->cap));
  cudaStream_t st = ctx->stream;
  const double *src[2] = {vx, vy};
  for (int k = 0; k < 2; k++) {
    CK(cudaMemcpyAsync(ctx->d_cyc_v64[regime] + k * nn, src[k], sizeof(double) * nn,
                       cudaMemcpyHostToDevice, st));
    launch_node_to_f32(ctx->d_cyc_v64[regime] + k * nn, ctx->d_cyc_v[regime] + k * nn, nn, st);
  }
  if (regime == 0) {
    CK(cudaMemsetAsync(ctx->d_slip, 0, sizeof(double) * nn, st));
    if (ctx->d_mslip) CK(cudaMemsetAsync(ctx->d_mslip, 0, sizeof(double) * ctx->cap, st));
  }
  CK(cudaStreamSynchronize(st));
  return V2C_OK;
}

// the launches of one cycle step (no host synchronisation: capturable)
static int cycle_enqueue(v2c_ctx *ctx, int regime, double dt) {
  cudaStream_t st = ctx->stream;
  const long nn = ctx->nn;
  CK(cudaMemcpyAsync(ctx->d_node + (long)V2C_NF_VX * nn, ctx->d_cyc_v[regime],
                     sizeof(float) * nn, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_node + (long)V2C_NF_VY * nn, ctx->d_cyc_v[regime] + nn,
                     sizeof(float) * nn, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_vel64, ctx->d_cyc_v64[regime], sizeof(double) * 2 * nn,
                     cudaMemcpyDeviceToDevice, st));
  ctx->vel64_ok[0] = ctx->vel64_ok[1] = true;
  int rc;
  if ((rc = v2c_marker2nodes(ctx))) return rc;
  if ((rc = v2c_center2basic_old(ctx))) return rc;
  if ((rc = v2c_compute_before_solve(ctx, dt, 0))) return rc;
  if ((rc = v2c_interpolate_basic2center(ctx))) return rc;
  if ((rc = v2c_recompute_stress_strainrate(ctx, dt))) return rc;
  if ((rc = v2c_interpolate_center2basic(ctx, dt))) return rc;
  if ((rc = v2c_compute_after_solve(ctx, dt, 0, nullptr))) return rc;
  if ((rc = v2c_copyarrays(ctx))) return rc;
  launch_slip_acc(make_grid(ctx), make_nodes(ctx), dt, ctx->d_slip, st);
  ctx->launches += 1;
  if (ctx->p.newton_guess != V2C_GUESS_OFF && ctx->n > 0) {
    launch_marker_slip_acc(ctx->m.slipv, ctx->n, dt, ctx->d_mslip, st);
    ctx->launches += 1;
  }
  return n2m_move(ctx, 1, 1);
}

static int cycle_flags(const v2c_ctx *ctx) {
  const Scal s = make_scal(ctx->p, ctx->h_rt);
  return s.antid | s.phi_reset0 << 1 | s.sticky_cap << 2 | s.sppe_nstress << 3 |
         s.timesum_pos << 4 | s.timesum_zero << 5;
}

extern "C" int v2c_cycle_step(v2c_ctx *ctx, int regime, double dt, int use_graph) {
  int rc = ready(ctx);
  if (rc) return rc;
  if (regime < 0 || regime > 1 || !(dt > 0)) return fail(ctx, V2C_ERR_ARG);
  if (!ctx->d_cyc_v[regime] || !ctx->d_slip) return fail(ctx, V2C_ERR_STATE);
  ctx->p.timestep = dt;
  ctx->props_valid = false;  // the step moves the markers
  cudaStream_t st = ctx->stream;
  // immobile markers change the marker count inside the step (a host
  // synchronisation), which a captured graph cannot hold: run eagerly
  if (!use_graph || ctx->n_immobile > 0) {
    rc = cycle_enqueue(ctx, regime, dt);
    if (rc) return rc;
    ctx->p.timesum += dt;
    return V2C_OK;
  }
  // work the capture must not contain: the first sort and the boundary rows
  if (!ctx->sorted) {
    launch_sort(ctx->m.cell_in, ctx->m.u_in, ctx->m.v_in, ctx->n, ctx->ncell, ctx->sb,
                ctx->d_stat, st);
    ctx->sorted = true;
  }
  if (ctx->have_bonds && (rc = build_bc(ctx))) return fail(ctx, rc);
  v2c_params pk = ctx->p;
  pk.timesum = 0;
  const int flags = cycle_flags(ctx);
  const void *pos = ctx->m.cell_in;
  for (auto &gr : ctx->graphs) {
    if (gr.regime == regime && gr.dt == dt && gr.pos == pos && gr.flags == flags &&
        !memcmp(&gr.p, &pk, sizeof(pk))) {
      CK(cudaGraphLaunch(gr.exec, st));
      // the host side of the step the graph replays
      swap_positions(ctx);
      ctx->sorted = true;
      ctx->launches += gr.launches;
      ctx->p.timesum += dt;
      return V2C_OK;
    }
  }
  // capture: the enqueue does the step's host bookkeeping (position swap)
  // as it records, so afterwards the host state is the one after the step
  const Markers saved = ctx->m;
  const long l0 = ctx->launches;
  const bool prof = ctx->prof;
  ctx->prof = false;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  rc = cycle_enqueue(ctx, regime, dt);
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  ctx->prof = prof;
  cudaGraphExec_t exec = nullptr;
  if (!rc && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
    exec = nullptr;
  if (graph) cudaGraphDestroy(graph);
  if (rc || ce != cudaSuccess || !exec) {
    ctx->m = saved;  // nothing ran
    ctx->launches = l0;
    cudaGetLastError();
    return fail(ctx, rc ? rc : V2C_ERR_CUDA);
  }
  if (ctx->graphs.size() >= 8) {
    cudaGraphExecDestroy(ctx->graphs.front().exec);
    ctx->graphs.erase(ctx->graphs.begin());
  }
  ctx->graphs.push_back({regime, dt, pos, pk, flags, exec, ctx->launches - l0});
  CK(cudaGraphLaunch(exec, st));
  ctx->p.timesum += dt;
  return V2C_OK;
}

extern "C" int v2c_cycle_marker_slip(v2c_ctx *ctx, double *out, long n) {
  if (!ctx || !out || n != ctx->n) return V2C_ERR_ARG;
  if (!ctx->d_mslip) return fail(ctx, V2C_ERR_STATE);
  launch_unpermute_f64(ctx->d_mslip, ctx->m.id, ctx->d_stage64, n, ctx->stream);
  CK(cudaMemcpyAsync(out, ctx->d_stage64, sizeof(double) * n, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return V2C_OK;
}

extern "C" int v2c_cycle_slip(v2c_ctx *ctx, double *out) {
  if (!ctx || !out) return V2C_ERR_ARG;
  if (!ctx->d_slip) return fail(ctx, V2C_ERR_STATE);
  CK(cudaMemcpyAsync(out, ctx->d_slip, sizeof(double) * ctx->nn, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return V2C_OK;
}

extern "C" int v2c_get_status(v2c_ctx *ctx, v2c_status *out) {
  if (!ctx || !out) return V2C_ERR_ARG;
  unsigned long long h[ST_N];
  CK(cudaMemcpyAsync(h, ctx->d_stat, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  memset(out, 0, sizeof(*out));
  out->n_markers = ctx->n;
  out->n_out_of_grid = (long)h[ST_OUT_OF_GRID];
  out->n_far_moves = (long)h[ST_FAR_MOVES];
  out->n_nan = (long)h[ST_NAN];
  out->newton_iters = (long)h[ST_NEWTON_ITERS];
  out->newton_fallbacks = (long)h[ST_NEWTON_FALLBACK];
  out->newton_nonconv = (long)h[ST_NEWTON_NONCONV];
  double r;
  unsigned long long bits = h[ST_NEWTON_MAXRES_BITS];
  memcpy(&r, &bits, sizeof(r));
  out->newton_max_res = r;
  out->max_cell_count = (long)h[ST_MAX_CELL];
  out->kernel_launches = ctx->launches;
  out->last_error = ctx->last_error;
  return V2C_OK;
}

// ----------------------------------------------------- internal accessors
// used by the per-marker Newton launcher (v2c_newton.cu)
v2c::NewtonState *v2c_ctx_newton(v2c_ctx *ctx) { return &ctx->nw; }
cudaStream_t v2c_ctx_stream(v2c_ctx *ctx) { return ctx->stream; }
unsigned long long *v2c_ctx_stat(v2c_ctx *ctx) { return ctx->d_stat; }
const v2c_params *v2c_ctx_params(v2c_ctx *ctx) { return &ctx->p; }

extern "C" int v2c_set_profiling(v2c_ctx *ctx, int on) {
  if (!ctx) return V2C_ERR_ARG;
  prof_resolve(ctx);
  for (int g = 0; g < V2C_PROF_N; g++) { ctx->prof_ms[g] = 0; ctx->prof_n[g] = 0; }
  ctx->prof = on != 0;
  return V2C_OK;
}

extern "C" int v2c_get_profile(v2c_ctx *ctx, int group, double *ms, long *launches) {
  if (!ctx || group < 0 || group >= V2C_PROF_N) return V2C_ERR_ARG;
  prof_resolve(ctx);
  if (ms) *ms = ctx->prof_ms[group];
  if (launches) *launches = ctx->prof_n[group];
  return V2C_OK;
}

// lets the Newton launcher bracket its own launches
void v2c_ctx_prof_begin(v2c_ctx *ctx, int group, cudaEvent_t *a) {
  *a = nullptr;
  if (ctx->prof) { *a = ev_get(ctx); cudaEventRecord(*a, ctx->stream); }
}
void v2c_ctx_prof_end(v2c_ctx *ctx, int group, cudaEvent_t a) {
  if (ctx->prof && a) {
    cudaEvent_t b = ev_get(ctx);
    cudaEventRecord(b, ctx->stream);
    ctx->prof_ev[group].push_back({a, b});
  }
}
void v2c_ctx_count_launches(v2c_ctx *ctx, long k) { ctx->launches += k; }
