// v2c_n2m.cu -- nodes2markers (interpolation.c:929-1490) and
// moveandrotatemarkers (moveandrotatemarkers.c:1-178).
//
// nodes2markers: same tiling as the marker2nodes sweep (see v2c_m2n.cu).
// Staging a marker gathers the 19 node fields of interpolate_mechanical from
// the four staggered stencils in cell-local FP32 coordinates and keeps the
// quantities the antidiffusion correction scatters back (PHIS, SXY, EXY, ES
// to basic nodes, PR, SXX, EXX to the centre node, VX*MRO, VY*MRO and MRO to
// vx/vy nodes); the tile that owns the marker applies the marker update.
// The back-scatter sums are formed per node by one thread each, in sorted
// marker order with two-sum compensation, exactly as in marker2nodes.
//
// moveandrotatemarkers: one thread per marker, Euler or RK4 through four
// allinteri evaluations (interpolation.c:1688-1758) from per-quarter
// bilinear forms, stress rotation; new positions go to the second position
// buffer.
#include <math.h>

#include "v2c_kernels.h"
#include "v2c_rheology.cuh"

namespace v2c {

namespace {

constexpr int TY = 32;
constexpr int NTH = 4 * TY;
constexpr int CHUNK = 384;

enum { Q_U = 0, Q_V, Q_PHIS, Q_SXY, Q_EXY, Q_ES, Q_PR, Q_SXX, Q_EXX, Q_VX, Q_VY, Q_MRO, Q_N };

struct Smem {
  float q[Q_N][CHUNK];
};

struct Pos {
  int ix, iy;
  float X, Y;  // metres from gx[ix], gy[iy]
};

// put a position back in the cell that contains it; FP64 search if it
// crossed more than four cells
__device__ __forceinline__ void settle(const Grid &g, Pos &p, unsigned long long *stat) {
  int ix0 = p.ix, iy0 = p.iy;
  float X0 = p.X, Y0 = p.Y;
  if (!relocate(g.wx, g.ncx, p.ix, p.X, 4)) {
    double x = g.gx[ix0] + (double)X0;
    p.ix = nsearch64(g.gx, g.xn, x);
    p.X = (float)(x - g.gx[p.ix]);
    atomicAdd(stat + ST_FAR_MOVES, 1ull);
  }
  if (!relocate(g.wy, g.ncy, p.iy, p.Y, 4)) {
    double y = g.gy[iy0] + (double)Y0;
    p.iy = nsearch64(g.gy, g.yn, y);
    p.Y = (float)(y - g.gy[p.iy]);
    atomicAdd(stat + ST_FAR_MOVES, 1ull);
  }
}

// allinteri (interpolation.c:1688-1758) inside one quarter of a cell is a
// bilinear function of the position: each stencil it reads (basic nodes for
// the spin, pressure nodes for the velocities averaged in pairs, vx and vy
// nodes for the staggered velocities) keeps its nodes across the quarter,
// its weights are affine in X and Y, and the blend weight xrat is constant
// there.  k_vel_quads writes, per quarter and per quantity (VX, VY, ESP),
// the coefficients of f = c0 + c1 dX + c2 dY + c3 dX dY, with dX, dY in
// metres from the quarter's lower corner; vel_at evaluates them.  Quarter
// qx = 1 holds X >= wx/2 (allinteri: xrat and the vy stencil switch at
// X < wx/2, the pressure stencil at X > wx/2, where it is continuous).

// affine weight w = (X - A) / B of one stencil axis at the quarter's corner
// X0: w = e0 + s (X - X0)
struct Lin {
  float e0, s;
};
__device__ __forceinline__ Lin lin_w(float X0, float A, float B) {
  return Lin{__fdividef(X0 - A, B), __fdividef(1.f, B)};
}

// bilinear interpolation of f over nodes m3, m3+1, m3+yn, m3+yn+1 as
// c0 + c1 dX + c2 dY + c3 dX dY
__device__ __forceinline__ float4 bil_form(const float *f, long m3, long yn, Lin ex, Lin ny) {
  const float f0 = __ldg(f + m3), f1 = __ldg(f + m3 + 1), f2 = __ldg(f + m3 + yn),
              f3 = __ldg(f + m3 + yn + 1);
  const float d20 = f2 - f0, d10 = f1 - f0, D = (f3 - f2) - d10;
  float4 c;
  c.x = f0 + ex.e0 * d20 + ny.e0 * (d10 + ex.e0 * D);
  c.y = (d20 + ny.e0 * D) * ex.s;
  c.z = (d10 + ex.e0 * D) * ny.s;
  c.w = D * ex.s * ny.s;
  return c;
}

// the pair sums of allinteri (interpolation.c:1730-1745) at pressure node
// m (m has ix >= 1 and iy >= 1 on every pressure stencil)
__device__ __forceinline__ float4 bil_form_pairs(const float *v, long o1, long o2, long m3,
                                                 long yn, Lin ex, Lin ny) {
  auto P = [&](long m) { return 0.5f * (__ldg(v + m - o1) + __ldg(v + m - o2)); };
  const float f0 = P(m3), f1 = P(m3 + 1), f2 = P(m3 + yn), f3 = P(m3 + yn + 1);
  const float d20 = f2 - f0, d10 = f1 - f0, D = (f3 - f2) - d10;
  float4 c;
  c.x = f0 + ex.e0 * d20 + ny.e0 * (d10 + ex.e0 * D);
  c.y = (d20 + ny.e0 * D) * ex.s;
  c.z = (d10 + ex.e0 * D) * ny.s;
  c.w = D * ex.s * ny.s;
  return c;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ float4 blend(float4 p, float4 s, float xrat) {
  const float r = 1.f - xrat;
  return make_float4(p.x * r + s.x * xrat, p.y * r + s.y * xrat, p.z * r + s.z * xrat,
                     p.w * r + s.w * xrat);
}

// one thread per cell quarter t = 4 cell + 2 qy + qx; stencils as in
// stencil_basic / stencil_centre / stencil_vx / stencil_vy
__global__ void k_vel_quads(Grid g, Nodes N, float4 *Q) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)g.ncx * g.ncy * 4) return;
  const long c = t >> 2;
  const int qx = (int)(t & 1), qy = (int)((t >> 1) & 1);
  const int ix = (int)(c / g.ncy), iy = (int)(c - (long)ix * g.ncy);
  const Axis ax = make_axis(g.wx, g.ncx, ix, 0.f), ay = make_axis(g.wy, g.ncy, iy, 0.f);
  const float X0 = qx ? 0.5f * ax.w : 0.f, Y0 = qy ? 0.5f * ay.w : 0.f;
  const long yn = g.yn;
  // spin at basic nodes
  int mx = clampi(ix, 1, g.xn - 3), my = clampi(iy, 1, g.yn - 3);
  int kx = mx - ix, ky = my - iy;
  const float4 cE = bil_form(N.f(V2C_NF_ESP), (long)mx * yn + my, yn,
                             lin_w(X0, ax.G(kx), ax.G(kx + 1) - ax.G(kx)),
                             lin_w(Y0, ay.G(ky), ay.G(ky + 1) - ay.G(ky)));
  // velocities averaged to pressure nodes
  mx = clampi(ix + qx, 1, g.xn - 2); my = clampi(iy + qy, 1, g.yn - 2);
  kx = mx - ix; ky = my - iy;
  Lin ex = lin_w(X0, (ax.G(kx - 1) + ax.G(kx)) * 0.5f, (ax.G(kx + 1) - ax.G(kx - 1)) * 0.5f);
  Lin ny = lin_w(Y0, (ay.G(ky - 1) + ay.G(ky)) * 0.5f, (ay.G(ky + 1) - ay.G(ky - 1)) * 0.5f);
  const long mc = (long)mx * yn + my;
  const float4 cPX = bil_form_pairs(N.f(V2C_NF_VX), 1, yn + 1, mc, yn, ex, ny);
  const float4 cPY = bil_form_pairs(N.f(V2C_NF_VY), yn, yn + 1, mc, yn, ex, ny);
  // vx nodes
  mx = clampi(ix, 0, g.xn - 2); my = clampi(iy - (qy ? 0 : 1), 0, g.yn - 3);
  kx = mx - ix; ky = my - iy;
  const float4 cVX = bil_form(N.f(V2C_NF_VX), (long)mx * yn + my, yn,
                              lin_w(X0, ax.G(kx), ax.G(kx + 1) - ax.G(kx)),
                              lin_w(Y0, (ay.G(ky) + ay.G(ky + 1)) * 0.5f,
                                    (ay.G(ky + 2) - ay.G(ky)) * 0.5f));
  // vy nodes
  mx = clampi(ix - (qx ? 0 : 1), 0, g.xn - 3); my = clampi(iy, 0, g.yn - 2);
  kx = mx - ix; ky = my - iy;
  const float4 cVY = bil_form(N.f(V2C_NF_VY), (long)mx * yn + my, yn,
                              lin_w(X0, (ax.G(kx) + ax.G(kx + 1)) * 0.5f,
                                    (ax.G(kx + 2) - ax.G(kx)) * 0.5f),
                              lin_w(Y0, ay.G(ky), ay.G(ky + 1) - ay.G(ky)));
  // staggered weight: 2/3, or 1 in the outer half of a boundary cell
  float xrat = 2.f / 3.f;
  if ((ix == 0 && !qx) || (ix == g.ncx - 1 && qx) || (iy == 0 && !qy) ||
      (iy == g.ncy - 1 && qy))
    xrat = 1.f;
  float4 *o = Q + t * 3;
  o[0] = blend(cPX, cVX, xrat);
  o[1] = blend(cPY, cVY, xrat);
  o[2] = cE;
}

// allinteri at a cell-local position: velocity and spin from the quarter's
// forms (positions outside the model are clamped onto its boundary first)
__device__ __forceinline__ void vel_at(const Grid &g, const float4 *Q, Pos p, float &VX,
                                       float &VY, float &ESP) {
  const float wx = __ldg(g.wx + p.ix), wy = __ldg(g.wy + p.iy);
  if (p.ix == 0 && p.X < 0.f) p.X = 0.f;
  if (p.ix == g.ncx - 1 && p.X > wx) p.X = wx;
  if (p.iy == 0 && p.Y < 0.f) p.Y = 0.f;
  if (p.iy == g.ncy - 1 && p.Y > wy) p.Y = wy;
  const float hx = 0.5f * wx, hy = 0.5f * wy;
  const int qx = p.X >= hx, qy = p.Y >= hy;
  const float dX = qx ? p.X - hx : p.X, dY = qy ? p.Y - hy : p.Y;
  const float4 *c = Q + (((long)p.ix * g.ncy + p.iy) * 4 + qy * 2 + qx) * 3;
  const float4 a = __ldg(c), b = __ldg(c + 1), e = __ldg(c + 2);
  VX = fmaf(dY, fmaf(a.w, dX, a.z), fmaf(a.y, dX, a.x));
  VY = fmaf(dY, fmaf(b.w, dX, b.z), fmaf(b.y, dX, b.x));
  ESP = fmaf(dY, fmaf(e.w, dX, e.z), fmaf(e.y, dX, e.x));
}

// basic-node back-scatter into a named register array
#define ADD_BS(A, q, w)                                                 \
  do {                                                                  \
    A[0].add(sm.q[Q_PHIS][q] * (w)); A[1].add(sm.q[Q_SXY][q] * (w));    \
    A[2].add(sm.q[Q_EXY][q] * (w)); A[3].add(sm.q[Q_ES][q] * (w));      \
    A[4].add(w);                                                        \
  } while (0)

// Marker values without antidiffusion (interpolation.c:985-1011), in a
// kernel instance of their own (PLAIN) so that the common antidiffusion
// path keeps its registers: the previous node fields interpolated (change = false: a marker's first
// values), or the change of the node fields since then (change = true),
// interpolated as one field of node differences -- the same bilinear form,
// so the same value in exact arithmetic, but the FP32 node differences of
// two states that agree in their leading digits are exact where the
// separate interpolations would each round at the size of the field.
struct Plain {
  float phi, exx, exy, sxx, sxy, p, vx, vy, e;
};
__device__ __forceinline__ void plain_values(const Grid &g, const Nodes &N, Axis ax, Axis ay,
                                                 float uc, float vc, bool change, Plain &o) {
  const long yn = g.yn;
  float e, n;
  long m3 = stencil_basic(g, ax, ay, e, n);
  if (change) {
    o.exy = bil_diff(N.f(V2C_NF_EXY), N.f(V2C_NF_EXYE), m3, yn, e, n);
    o.sxy = bil_diff(N.f(V2C_NF_SXY), N.f(V2C_NF_SXYE), m3, yn, e, n);
    o.e = bil_diff(N.f(V2C_NF_PES), N.f(V2C_NF_PE), m3, yn, e, n);
    o.phi = bil_diff(N.f(V2C_NF_PHIS_IT), N.f(V2C_NF_PHIS), m3, yn, e, n);
  } else {
    o.exy = bil(N.f(V2C_NF_EXYE), m3, yn, e, n);
    o.sxy = bil(N.f(V2C_NF_SXYE), m3, yn, e, n);
    o.e = bil(N.f(V2C_NF_PE), m3, yn, e, n);
    o.phi = bil(N.f(V2C_NF_PHIS), m3, yn, e, n);
  }
  m3 = stencil_centre(g, ax, ay, uc > 0.5f, vc > 0.5f, e, n);
  if (change) {
    o.exx = bil_diff(N.f(V2C_NF_EXX), N.f(V2C_NF_EXXE), m3, yn, e, n);
    o.sxx = bil_diff(N.f(V2C_NF_SXX), N.f(V2C_NF_SXXE), m3, yn, e, n);
    o.p = bil_diff(N.f(V2C_NF_PR), N.f(V2C_NF_SPPE), m3, yn, e, n);
  } else {
    o.exx = bil(N.f(V2C_NF_EXXE), m3, yn, e, n);
    o.sxx = bil(N.f(V2C_NF_SXXE), m3, yn, e, n);
    o.p = bil(N.f(V2C_NF_SPPE), m3, yn, e, n);
  }
  m3 = stencil_vx(g, ax, ay, vc < 0.5f, g.xn - 2, e, n);
  o.vx = change ? bil_diff(N.f(V2C_NF_VX), N.f(V2C_NF_MVX), m3, yn, e, n)
                : bil(N.f(V2C_NF_MVX), m3, yn, e, n);
  m3 = stencil_vy(g, ax, ay, uc < 0.5f, g.yn - 2, e, n);
  o.vy = change ? bil_diff(N.f(V2C_NF_VY), N.f(V2C_NF_MVY), m3, yn, e, n)
                : bil(N.f(V2C_NF_MVY), m3, yn, e, n);
}

template <bool BS, bool PLAIN>
__global__ void __launch_bounds__(NTH, 7) k_n2m(N2MArgs a) {
  __shared__ Smem sm;
  const Grid &g = a.g;
  const Nodes &N = a.N;
  const int tid = threadIdx.x, role = tid / TY, jl = tid % TY;
  const int i0 = blockIdx.x * a.TX, j0 = blockIdx.y * TY;
  const int j = j0 + jl;
  const bool jvalid = j < g.yn;
  const int ncy = g.ncy;
  const int ci_end = min(i0 + a.TX, g.xn);
  const v2c_params &P = a.S.p;
  // interpolationmod 1 back-scatters through a.bs and the gather kernels
  const int backscatter = a.do_n2m && !PLAIN && !BS;
  const long yn = g.yn;

  // role 0: PHIS, SXY, EXY, ES, w (basic)   role 1: PR, SXX, EXX, w (centre)
  // role 2: VX*MRO, MRO, w (vx)             role 3: VY*MRO, MRO, w (vy)
  Acc cur[5], car[5];
#pragma unroll
  for (int q = 0; q < 5; q++) { cur[q].zero(); car[q].zero(); }

  for (int ci = max(i0 - 1, 0); ci < ci_end; ++ci) {
#pragma unroll
    for (int q = 0; q < 5; q++) { cur[q] = car[q]; car[q].zero(); }
    if (role == 1 || role == 3) {
#pragma unroll
      for (int q = 0; q < 5; q++) cur[q].zero();
    }
    if (ci < g.ncx) {
      const int jlo = max(j0 - 1, 0), jhi = min(j0 + TY - 1, ncy - 1);
      const long cb = (long)ci * ncy;
      const int seg_b = __ldg(a.start + cb + jlo), seg_e = __ldg(a.start + cb + jhi + 1);

      const bool owned_col = ci >= i0;
      for (int cs = seg_b; cs < seg_e; cs += CHUNK) {
        const int ce = min(cs + CHUNK, seg_e);
        if (backscatter) __syncthreads();
        // the chunk's sort indices of this thread, read together (three
        // markers per thread: one round of latency rather than three)
        static_assert(CHUNK == 3 * NTH, "three staging rounds per chunk");
        int pidx[3];
#pragma unroll
        for (int jj = 0; jj < 3; jj++)
          pidx[jj] = tid + jj * NTH < ce - cs ? __ldg(a.perm + cs + tid + jj * NTH) : 0;
#pragma unroll 1
        for (int jj = 0; jj < 3; jj++) {
          const int k = tid + jj * NTH;
          if (k >= ce - cs) break;
          // ---------------------------------------------- stage marker
          const int idx = jj == 0 ? pidx[0] : (jj == 1 ? pidx[1] : pidx[2]);
          const int c = a.m.cell_in[idx];
          const int ix = c / ncy, iy = c - ix * ncy;
          const float u = a.m.u_in[idx], v = a.m.v_in[idx];
          const int t = a.m.type[idx];
          const bool owned = owned_col && iy >= j0 && iy < j0 + TY;
          if (!owned && !backscatter) continue;
          // interpolate_mechanical clamps the point into the model first
          float uc = u, vc = v;
          if (ix == 0 && uc < 0.f) uc = 0.f;
          if (ix == g.ncx - 1 && uc > 1.f) uc = 1.f;
          if (iy == 0 && vc < 0.f) vc = 0.f;
          if (iy == g.ncy - 1 && vc > 1.f) vc = 1.f;
          const float wxc = __ldg(g.wx + ix), wyc = __ldg(g.wy + iy);
          const Axis ax = make_axis(g.wx, g.ncx, ix, uc * wxc);
          const Axis ay = make_axis(g.wy, g.ncy, iy, vc * wyc);
          float eb, nb, ec, ncc, e, n;
          const long mb = stencil_basic(g, ax, ay, eb, nb);
          const float EXY = bil(N.f(V2C_NF_EXY), mb, yn, eb, nb);
          const float SXY = bil(N.f(V2C_NF_SXY), mb, yn, eb, nb);
          const float ES = bil(N.f(V2C_NF_PES), mb, yn, eb, nb);
          const float PHIS = bil(N.f(V2C_NF_PHIS_IT), mb, yn, eb, nb);
          const long mc = stencil_centre(g, ax, ay, uc > 0.5f, vc > 0.5f, ec, ncc);
          const float EXX = bil(N.f(V2C_NF_EXX), mc, yn, ec, ncc);
          const float SXX = bil(N.f(V2C_NF_SXX), mc, yn, ec, ncc);
          const float PR = bil(N.f(V2C_NF_PR), mc, yn, ec, ncc);
          long m3 = stencil_vx(g, ax, ay, vc < 0.5f, g.xn - 2, e, n);
          const float VX = bil(N.f(V2C_NF_VX), m3, yn, e, n);
          m3 = stencil_vy(g, ax, ay, uc < 0.5f, g.yn - 2, e, n);
          const float VY = bil(N.f(V2C_NF_VY), m3, yn, e, n);
          if (backscatter) {
            sm.q[Q_U][k] = uc; sm.q[Q_V][k] = vc;
            sm.q[Q_PHIS][k] = PHIS; sm.q[Q_SXY][k] = SXY; sm.q[Q_EXY][k] = EXY;
            sm.q[Q_ES][k] = ES; sm.q[Q_PR][k] = PR; sm.q[Q_SXX][k] = SXX;
            sm.q[Q_EXX][k] = EXX; sm.q[Q_VX][k] = VX; sm.q[Q_VY][k] = VY;
            sm.q[Q_MRO][k] = a.R(RK_RO, t);
          }
          if (!owned) continue;
          if (BS) {
            const long s = cs + k, n = a.n;
            a.bs[BS_U * n + s] = uc; a.bs[BS_V * n + s] = vc;
            a.bs[BS_PHIS * n + s] = PHIS; a.bs[BS_SXY * n + s] = SXY;
            a.bs[BS_EXY * n + s] = EXY; a.bs[BS_ES * n + s] = ES;
            a.bs[BS_PR * n + s] = PR; a.bs[BS_SXX * n + s] = SXX;
            a.bs[BS_EXX * n + s] = EXX;
          }
          // ------------------------------------- marker update (:943-1011)
          const bool in_strict = (ix > 0 || u > 0.f) && (ix < g.ncx - 1 || u < 1.f) &&
                                 (iy > 0 || v > 0.f) && (iy < g.ncy - 1 || v < 1.f);
          const bool in_grid = (ix > 0 || u >= 0.f) && (ix < g.ncx - 1 || u <= 1.f) &&
                               (iy > 0 || v >= 0.f) && (iy < g.ncy - 1 || v <= 1.f);
          float tk = a.m.tk[idx];
          // the marker's own values are read only without antidiffusion,
          // where it keeps them plus the change of the node fields; with
          // it, an updated marker takes all nine from the nodes
          float phi = 0.f, mexx = 0.f, mexy = 0.f, msxx = 0.f, msxy = 0.f, mp = 0.f;
          float mvx = 0.f, mvy = 0.f, me = 0.f;
          if (PLAIN) {
            phi = a.m.phi[idx]; mexx = a.m.exx[idx]; mexy = a.m.exy[idx];
            msxx = a.m.sxx[idx]; msxy = a.m.sxy[idx]; mp = a.m.p[idx];
            mvx = a.m.vx[idx]; mvy = a.m.vy[idx]; me = a.m.e[idx];
          }
          bool changed = false, tk_set = false;
          if (a.do_n2m) {
            if (in_strict && t < 50 && tk <= 0.f) {
              if (!PLAIN) {
                msxx = SXX; msxy = SXY; mp = PR; mexx = EXX; mexy = EXY;
                mvx = VX; mvy = VY; phi = PHIS; me = ES;
              } else {
                Plain o;
                plain_values(g, N, ax, ay, uc, vc, false, o);
                msxx = o.sxx; msxy = o.sxy; mp = o.p; mexx = o.exx; mexy = o.exy;
                mvx = o.vx; mvy = o.vy; phi = o.phi; me = o.e;
              }
              if (!P.tempmod) {
                tk = a.S.eps2_f;
                tk_set = true;
              }
              changed = true;
            }
            if (in_grid && t < 50 && tk > 0.f) {
              if (!PLAIN) {
                phi = PHIS; mexx = EXX; mexy = EXY; msxx = SXX; msxy = SXY;
                mp = PR; mvx = VX; mvy = VY; me = ES;
              } else {
                Plain o;
                plain_values(g, N, ax, ay, uc, vc, true, o);
                phi += o.phi; mexx += o.exx; mexy += o.exy;
                msxx += o.sxx; msxy += o.sxy; mp += o.p;
                mvx += o.vx; mvy += o.vy; me += o.e;
              }
              changed = true;
            }
          }

          if (changed) {
            a.m.phi[idx] = phi; a.m.exx[idx] = mexx; a.m.exy[idx] = mexy;
            a.m.sxx[idx] = msxx; a.m.sxy[idx] = msxy; a.m.p[idx] = mp;
            a.m.vx[idx] = mvx; a.m.vy[idx] = mvy; a.m.e[idx] = me;
            a.m.tk[idx] = tk;
            if (tk_set) a.m.tk_lo[idx] = a.S.eps2_lo;
          }
        }
        if (!backscatter) continue;
        __syncthreads();
        if (!jvalid) continue;
        // quarter class starts of cell (ci, j-1) (lower) and (ci, j) (upper),
        // read here rather than held through the staging
        int4 ql = make_int4(0, 0, 0, 0), qu = make_int4(0, 0, 0, 0);
        int lo_e = 0, up_e = 0;
        float s1lo = 0.f, s1up = 0.f;
        const float iwx = 1.f / __ldg(g.wx + ci);
        if (j - 1 >= 0 && j - 1 <= ncy - 1) {
          ql = __ldg(a.qstart + cb + j - 1); lo_e = __ldg(a.start + cb + j);
          s1lo = iwx / __ldg(g.wy + j - 1);
        }
        if (j <= ncy - 1) {
          qu = __ldg(a.qstart + cb + j); up_e = __ldg(a.start + cb + j + 1);
          s1up = iwx / __ldg(g.wy + j);
        }
        // ---------------------------------------------- back-scatter
        // over the quarter class runs of cell (ci, j-1) and (ci, j); the
        // conditions inside hold for the whole run except at exact halves
#define CLASS_RUN(b, e) \
  for (int s = max((b), cs), s_e = min((e), ce), q = s - cs; s < s_e; ++s, q = s - cs)
        if (role == 0) {
          CLASS_RUN(ql.z, ql.w) {  // cell (ci, j-1), v > 1/2, u <= 1/2
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (u < 0.5f) {
              const float w = s1lo * (1.f - 2.f * u) * (2.f * v - 1.f);
              ADD_BS(cur, q, w);
            }
          }
          CLASS_RUN(ql.w, lo_e) {  // cell (ci, j-1), v > 1/2, u > 1/2
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            const float w = s1lo * (2.f * u - 1.f) * (2.f * v - 1.f);
            ADD_BS(car, q, w);
          }
          CLASS_RUN(qu.x, qu.y) {  // cell (ci, j), v <= 1/2, u <= 1/2
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (u < 0.5f && v < 0.5f) {
              const float w = s1up * (1.f - 2.f * u) * (1.f - 2.f * v);
              ADD_BS(cur, q, w);
            }
          }
          CLASS_RUN(qu.y, qu.z) {  // cell (ci, j), v <= 1/2, u > 1/2
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (v < 0.5f) {
              const float w = s1up * (2.f * u - 1.f) * (1.f - 2.f * v);
              ADD_BS(car, q, w);
            }
          }
        } else if (role == 1) {
          CLASS_RUN(qu.x, up_e) {  // the whole cell (ci, j) to its centre node
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            const float w = s1up * tent(u) * tent(v);
            cur[0].add(sm.q[Q_PR][q] * w); cur[1].add(sm.q[Q_SXX][q] * w);
            cur[2].add(sm.q[Q_EXX][q] * w); cur[3].add(w);
          }
        } else if (role == 2) {
          // vx node (ci, j) from u < 1/2 (classes 0, 2), (ci+1, j) from u > 1/2
          CLASS_RUN(qu.x, qu.y) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (u < 0.5f) {
              const float mro = sm.q[Q_MRO][q];
              const float w = s1up * (1.f - u) * (1.f - fabsf(v - 0.5f));
              cur[0].add(sm.q[Q_VX][q] * mro * w); cur[1].add(mro * w); cur[2].add(w);
            }
          }
          CLASS_RUN(qu.y, qu.z) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            const float mro = sm.q[Q_MRO][q];
            const float w = s1up * u * (1.f - fabsf(v - 0.5f));
            car[0].add(sm.q[Q_VX][q] * mro * w); car[1].add(mro * w); car[2].add(w);
          }
          CLASS_RUN(qu.z, qu.w) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (u < 0.5f) {
              const float mro = sm.q[Q_MRO][q];
              const float w = s1up * (1.f - u) * (1.f - fabsf(v - 0.5f));
              cur[0].add(sm.q[Q_VX][q] * mro * w); cur[1].add(mro * w); cur[2].add(w);
            }
          }
          CLASS_RUN(qu.w, up_e) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            const float mro = sm.q[Q_MRO][q];
            const float w = s1up * u * (1.f - fabsf(v - 0.5f));
            car[0].add(sm.q[Q_VX][q] * mro * w); car[1].add(mro * w); car[2].add(w);
          }
        } else {
          // vy node (ci, j) from v > 1/2 of cell (ci, j-1) (classes 2, 3) and
          // v < 1/2 of cell (ci, j) (classes 0, 1)
          CLASS_RUN(ql.z, lo_e) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            const float mro = sm.q[Q_MRO][q];
            const float w = s1lo * (1.f - fabsf(u - 0.5f)) * v;
            cur[0].add(sm.q[Q_VY][q] * mro * w); cur[1].add(mro * w); cur[2].add(w);
          }
          CLASS_RUN(qu.x, qu.z) {
            const float u = sm.q[Q_U][q], v = sm.q[Q_V][q];
            if (v < 0.5f) {
              const float mro = sm.q[Q_MRO][q];
              const float w = s1up * (1.f - fabsf(u - 0.5f)) * (1.f - v);
              cur[0].add(sm.q[Q_VY][q] * mro * w); cur[1].add(mro * w); cur[2].add(w);
            }
          }
        }
#undef CLASS_RUN
      }
    }

    // ----------------------------------------------- sums and normalisation
    if (!backscatter || ci < i0 || !jvalid) continue;
    const long m3 = (long)ci * yn + j;
    if (role == 0) {
      const float w = cur[4].value();
      const float ph = cur[0].value(), sy = cur[1].value(), ey = cur[2].value(), es = cur[3].value();
      N.f(V2C_NF_PHISUM)[m3] = ph; N.f(V2C_NF_SXYSUM)[m3] = sy;
      N.f(V2C_NF_EXYSUM)[m3] = ey; N.f(V2C_NF_ESUM)[m3] = es; N.f(V2C_NF_WTPHISUM)[m3] = w;
      if (w != 0.f && ci >= 1 && j >= 1 && ci < g.xn - 1 && j < g.yn - 1) {
        N.f(V2C_NF_PHIE)[m3] = __fdividef(ph, w); N.f(V2C_NF_SXYEE)[m3] = __fdividef(sy, w);
        N.f(V2C_NF_EXYEE)[m3] = __fdividef(ey, w); N.f(V2C_NF_PEE)[m3] = __fdividef(es, w);
      }
    } else if (role == 1) {
      if (ci < g.ncx && j < ncy) {
        const long mc = (long)(ci + 1) * yn + (j + 1);
        const float w = cur[3].value();
        const float ps = cur[0].value(), sx = cur[1].value(), ex = cur[2].value();
        N.f(V2C_NF_PSUM)[mc] = ps; N.f(V2C_NF_SXXSUM)[mc] = sx;
        N.f(V2C_NF_EXXSUM)[mc] = ex; N.f(V2C_NF_WTSXXSUM)[mc] = w;
        if (w != 0.f) {
          N.f(V2C_NF_SPPEE)[mc] = __fdividef(ps, w); N.f(V2C_NF_SXXEE)[mc] = __fdividef(sx, w);
          N.f(V2C_NF_EXXEE)[mc] = __fdividef(ex, w);
        }
      }
      if (ci == 0 || j == 0) {
        N.f(V2C_NF_PSUM)[m3] = 0; N.f(V2C_NF_SXXSUM)[m3] = 0;
        N.f(V2C_NF_EXXSUM)[m3] = 0; N.f(V2C_NF_WTSXXSUM)[m3] = 0;
      }
    } else if (role == 2) {
      const float w = cur[2].value(), vs = cur[0].value(), mr = cur[1].value();
      N.f(V2C_NF_VXSUM)[m3] = vs; N.f(V2C_NF_MRX0)[m3] = mr; N.f(V2C_NF_WTVXSUM)[m3] = w;
      if (w != 0.f) N.f(V2C_NF_MVXE)[m3] = __fdividef(vs, mr);
    } else {
      const float w = cur[2].value(), vs = cur[0].value(), mr = cur[1].value();
      N.f(V2C_NF_VYSUM)[m3] = vs; N.f(V2C_NF_MRY0)[m3] = mr; N.f(V2C_NF_WTVYSUM)[m3] = w;
      if (w != 0.f) N.f(V2C_NF_MVYE)[m3] = __fdividef(vs, mr);
    }
  }
}

// ------------------------------------------------ interpolationmod 1
// The back-scatter of interpolate_mechanical (interpolation.c:1104-1158 and
// 1249-1358) with the full stencils, as a gather: one thread per node sums,
// cell by cell in sorted order, the payload the tile sweep left per marker
// — bilinear weights on basic nodes, the staggered centre stencil on
// pressure nodes (no vx/vy back-scatter in this mode) — and normalises as
// the tail of nodes2markers does (interpolation.c:1014-1046).  The centre
// stencil's contributions past the last node row land, as in the
// reference, in the next column's first row (a ghost node whose sums are
// kept but never normalised).
__device__ __forceinline__ float bs_half(int k, float f) {
  if (k == 0) return f < 0.5f ? 1.f - f - 0.5f : 0.f;
  if (k == 1) return 1.f - fabsf(f - 0.5f);
  return f > 0.5f ? f - 0.5f : 0.f;
}

template <int ROLE>
__global__ void __launch_bounds__(128) k_n2m_bs_mode1(N2MArgs a) {
  const Grid &g = a.g;
  const Nodes &N = a.N;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= g.nn) return;
  const int ix = (int)(t / g.yn), iy = (int)(t - (long)ix * g.yn);
  const int ncy = g.ncy;
  const long n = a.n;
  const float *bs = a.bs;
  Acc sum[5];
#pragma unroll
  for (int q = 0; q < 5; q++) sum[q].zero();
  auto cell_sum = [&](int cx, int cy, int ax, int by) {
    if (cx < 0 || cx >= g.ncx || cy < 0 || cy >= ncy) return;
    const float s1 = (1.f / __ldg(g.wx + cx)) / __ldg(g.wy + cy);
    const long c = (long)cx * ncy + cy;
    const int sb = __ldg(a.start + c), se = __ldg(a.start + c + 1);
    for (int s = sb; s < se; s++) {
      const float u = bs[BS_U * n + s], v = bs[BS_V * n + s];
      if (ROLE == 0) {
        const float w = s1 * (ax ? u : 1.f - u) * (by ? v : 1.f - v);
        sum[0].add(bs[BS_PHIS * n + s] * w); sum[1].add(bs[BS_SXY * n + s] * w);
        sum[2].add(bs[BS_EXY * n + s] * w); sum[3].add(bs[BS_ES * n + s] * w);
        sum[4].add(w);
      } else {
        const float w = s1 * bs_half(ax, u) * bs_half(by, v);
        if (w != 0.f) {
          sum[0].add(bs[BS_PR * n + s] * w); sum[1].add(bs[BS_SXX * n + s] * w);
          sum[2].add(bs[BS_EXX * n + s] * w); sum[3].add(w);
        }
      }
    }
  };
  if (ROLE == 0) {
    for (int ax = 1; ax >= 0; ax--)
      for (int by = 1; by >= 0; by--) cell_sum(ix - ax, iy - by, ax, by);
    const float w = sum[4].value();
    const float ph = sum[0].value(), sy = sum[1].value(), ey = sum[2].value(), es = sum[3].value();
    N.f(V2C_NF_PHISUM)[t] = ph; N.f(V2C_NF_SXYSUM)[t] = sy;
    N.f(V2C_NF_EXYSUM)[t] = ey; N.f(V2C_NF_ESUM)[t] = es; N.f(V2C_NF_WTPHISUM)[t] = w;
    if (w != 0.f && ix >= 1 && iy >= 1 && ix < g.xn - 1 && iy < g.yn - 1) {
      N.f(V2C_NF_PHIE)[t] = __fdividef(ph, w); N.f(V2C_NF_SXYEE)[t] = __fdividef(sy, w);
      N.f(V2C_NF_EXYEE)[t] = __fdividef(ey, w); N.f(V2C_NF_PEE)[t] = __fdividef(es, w);
    }
  } else {
    for (int ax = 2; ax >= 0; ax--)
      for (int by = 2; by >= 0; by--) cell_sum(ix - ax, iy - by, ax, by);
    // the first row also gets what the last cell row sends past the end of
    // the previous columns
    if (iy == 0)
      for (int ax = 2; ax >= 0; ax--) cell_sum(ix - 1 - ax, ncy - 1, ax, 2);
    const float w = sum[3].value();
    const float ps = sum[0].value(), sx = sum[1].value(), ex = sum[2].value();
    N.f(V2C_NF_PSUM)[t] = ps; N.f(V2C_NF_SXXSUM)[t] = sx;
    N.f(V2C_NF_EXXSUM)[t] = ex; N.f(V2C_NF_WTSXXSUM)[t] = w;
    if (w != 0.f && ix >= 1 && iy >= 1) {
      N.f(V2C_NF_SPPEE)[t] = __fdividef(ps, w); N.f(V2C_NF_SXXEE)[t] = __fdividef(sx, w);
      N.f(V2C_NF_EXXEE)[t] = __fdividef(ex, w);
    }
  }
}

// ----------------------------------------------------------- the move
// moveandrotatemarkers (moveandrotatemarkers.c:1-178), one thread per
// marker in cell order: Euler or RK4 through allinteri, stress rotation,
// markers from depth, out-of-grid reset.  New positions go to the second
// position buffer.
__global__ void __launch_bounds__(256) k_move(N2MArgs a) {
  const Grid &g = a.g;
  const v2c_params &P = a.S.p;
  const int ncy = g.ncy;
  const float dt = a.S.dt;
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < a.n;
       s += (long)gridDim.x * blockDim.x) {
    const int idx = __ldg(a.perm + s);
    const int c = a.m.cell_in[idx];
    const int ix = c / ncy, iy = c - ix * ncy;
    const float u = a.m.u_in[idx], v = a.m.v_in[idx];
    const int t = a.m.type[idx];
    const bool in_grid = (ix > 0 || u >= 0.f) && (ix < g.ncx - 1 || u <= 1.f) &&
                         (iy > 0 || v >= 0.f) && (iy < g.ncy - 1 || v <= 1.f);
    int nix = ix, niy = iy;
    float nu_ = u, nv_ = v;
    if (!a.R(RK_IM, t) && (in_grid || P.outgrid != 1)) {
      const float wxc = __ldg(g.wx + ix), wyc = __ldg(g.wy + iy);
      const Pos p0{ix, iy, u * wxc, v * wyc};
      float vx0, vy0, sp0, vx1, vy1, sp1;
      vel_at(g, a.quad, p0, vx1, vy1, sp1);
      if (P.markmod == 1) {
        vx0 = vx1; vy0 = vy1; sp0 = sp1;
      } else {
        float vx2, vy2, sp2, vx3, vy3, sp3, vx4, vy4, sp4;
        Pos p = p0;
        p.X += vx1 * dt / 2.f; p.Y += vy1 * dt / 2.f;
        settle(g, p, a.stat);
        vel_at(g, a.quad, p, vx2, vy2, sp2);
        p = p0;
        p.X += vx2 * dt / 2.f; p.Y += vy2 * dt / 2.f;
        settle(g, p, a.stat);
        vel_at(g, a.quad, p, vx3, vy3, sp3);
        p = p0;
        p.X += vx3 * dt; p.Y += vy3 * dt;
        settle(g, p, a.stat);
        vel_at(g, a.quad, p, vx4, vy4, sp4);
        vx0 = (vx1 + 2.f * vx2 + 2.f * vx3 + vx4) / 6.f;
        vy0 = (vy1 + 2.f * vy2 + 2.f * vy3 + vy4) / 6.f;
        sp0 = (P.markmod == 2) ? (sp1 + 2.f * sp2 + 2.f * sp3 + sp4) / 6.f : sp1;
      }
      if (P.outgrid == 2) {
        if ((ix == 0 && u < 0.f) || (ix == g.ncx - 1 && u > 1.f)) vy0 = 0.f;
        if ((iy == 0 && v < 0.f) || (iy == g.ncy - 1 && v > 1.f)) vx0 = 0.f;
      }
      // new position: in offset space while the marker stays in its cell
      // (one FP32 rounding of u), else walked in metres
      nu_ = u + dt * vx0 / wxc;
      nv_ = v + dt * vy0 / wyc;
      const bool interior_x = ix > 0 && ix < g.ncx - 1, interior_y = iy > 0 && iy < g.ncy - 1;
      if (!(nu_ >= 0.f && nu_ < 1.f && (interior_x || (u >= 0.f && u <= 1.f)))) {
        Pos p{ix, 0, nu_ * wxc, 0.f};
        settle(g, p, a.stat);
        nix = p.ix;
        const float nwx = __ldg(g.wx + nix);
        nu_ = p.X / nwx;
        if (p.X < nwx && nu_ >= 1.f) nu_ = nextafterf(1.f, 0.f);
        if (p.X < 0.5f * nwx && nu_ >= 0.5f) nu_ = nextafterf(0.5f, 0.f);
        if (p.X > 0.5f * nwx && nu_ <= 0.5f) nu_ = nextafterf(0.5f, 1.f);
        if (p.X > nwx && nu_ <= 1.f) nu_ = nextafterf(1.f, 2.f);
      }
      if (!(nv_ >= 0.f && nv_ < 1.f && (interior_y || (v >= 0.f && v <= 1.f)))) {
        Pos p{0, iy, 0.f, nv_ * wyc};
        settle(g, p, a.stat);
        niy = p.iy;
        const float nwy = __ldg(g.wy + niy);
        nv_ = p.Y / nwy;
        if (p.Y < nwy && nv_ >= 1.f) nv_ = nextafterf(1.f, 0.f);
        if (p.Y < 0.5f * nwy && nv_ >= 0.5f) nv_ = nextafterf(0.5f, 0.f);
        if (p.Y > 0.5f * nwy && nv_ <= 0.5f) nv_ = nextafterf(0.5f, 1.f);
        if (p.Y > nwy && nv_ <= 1.f) nv_ = nextafterf(1.f, 2.f);
      }
      if (t >= 100) {
        // immobile marker (moveandrotatemarkers.c:88-135): inside the model
        // it spawns a mobile marker there and goes back to its anchor
        // (markk, markv), as it does when it strays more than ystpy from it
        const bool inside = (nix > 0 || nu_ >= 0.f) && (nix < g.ncx - 1 || nu_ <= 1.f) &&
                            (niy > 0 || nv_ >= 0.f) && (niy < g.ncy - 1 || nv_ <= 1.f);
        const double ax = (double)a.m.tk[idx] + (double)a.m.tk_lo[idx];
        const double ay = (double)a.m.mv[idx] + (double)a.m.mv_lo[idx];
        double x = g.gx[nix] + (double)nu_ * (g.gx[nix + 1] - g.gx[nix]);
        double y = g.gy[niy] + (double)nv_ * (g.gy[niy + 1] - g.gy[niy]);
        if (inside && a.has_imm) {
          const int id = a.m.id[idx];
          a.imm.spawn[id] = 1;
          a.imm.sp_cell[id] = nix * ncy + niy;
          a.imm.sp_u[id] = nu_;
          a.imm.sp_v[id] = nv_;
          x = ax;
          y = ay;
        }
        const double dx = x - ax, dy = y - ay;
        if (x == ax && y == ay || sqrt(dx * dx + dy * dy) > P.ystpy) {
          nix = nsearch64(g.gx, g.xn, ax);
          niy = nsearch64(g.gy, g.yn, ay);
          nu_ = offset32((ax - g.gx[nix]) / (g.gx[nix + 1] - g.gx[nix]));
          nv_ = offset32((ay - g.gy[niy]) / (g.gy[niy + 1] - g.gy[niy]));
        }
      } else {
      // stress rotation, moveandrotatemarkers.c:58-76
      float msxx = a.m.sxx[idx], msxy = a.m.sxy[idx];
      sp0 *= dt;
      if (P.stoksmod == 1) {
        float sn, cs;
        sincosf(sp0, &sn, &cs);
        const float s2 = 2.f * sn * cs, c2 = cs * cs - sn * sn;  // sin, cos of 2 sp0
        const float r1 = msxx * cs * cs - msxx * sn * sn + msxy * s2;
        const float r3 = 0.5f * (-msxx - msxx) * s2 + msxy * c2;
        msxx = r1; msxy = r3;
      } else if (P.stoksmod == 2) {
        const float r1 = msxx + msxy * 2.f * sp0;
        const float r3 = msxy + 0.5f * (-msxx - msxx) * 2.f * sp0;
        msxx = r1; msxy = r3;
      }
      a.m.sxx[idx] = msxx;
      a.m.sxy[idx] = msxy;
      // markers coming from depth, out-of-grid reset (:79-87); the FP64
      // position only when the FP32 one is within 1 m of zdeep
      // (the temperature pair's high word decides tk < tdeep; the two can
      // differ only for a temperature within half an FP32 ulp of tdeep, where
      // resetting or not leaves the same temperature to that half ulp)
      float tk = a.m.tk[idx], tk_lo = 0.f;
      bool reset = false;
      if (vy0 < 0.f && tk < a.S.tdeep_f &&
          __ldg(a.gyf + niy) + nv_ * __ldg(g.wy + niy) > a.S.zdeep_lo_f) {
        const double ynew = g.gy[niy] + (double)nv_ * (g.gy[niy + 1] - g.gy[niy]);
        if (ynew > P.zdeep) {
          tk = a.S.tdeep_f;
          tk_lo = a.S.tdeep_lo;
          reset = true;
        }
      }
      const bool out = (nix == 0 && nu_ < 0.f) || (nix == g.ncx - 1 && nu_ > 1.f) ||
                       (niy == 0 && nv_ < 0.f) || (niy == g.ncy - 1 && nv_ > 1.f);
      if (out) {
        tk = 0.f;
        tk_lo = 0.f;
        reset = true;
        a.m.e[idx] = 0.f;
        a.m.flags[idx] |= MFLAG_RESET;
        atomicAdd(a.stat + ST_OUT_OF_GRID, 1ull);
      }
      if (reset) {
        a.m.tk[idx] = tk;
        a.m.tk_lo[idx] = tk_lo;
      }
      }
    }
    // mobile markers outside the model after the move: the slots that
    // markers spawned by immobile ones refill (moveandrotatemarkers.c:141-171)
    if (a.has_imm && t < 100 &&
        !((nix > 0 || nu_ >= 0.f) && (nix < g.ncx - 1 || nu_ <= 1.f) &&
          (niy > 0 || nv_ >= 0.f) && (niy < g.ncy - 1 || nv_ <= 1.f)))
      a.imm.out[a.m.id[idx]] = 1;
    a.m.cell_out[idx] = nix * ncy + niy;
    a.m.u_out[idx] = nu_;
    a.m.v_out[idx] = nv_;
  }
}

}  // namespace

void launch_n2m(const N2MArgs &a, cudaStream_t st) {
  dim3 grid((a.g.xn + a.TX - 1) / a.TX, (a.g.yn + TY - 1) / TY);
  if (!a.bs) {
    // PLAIN: the markers take the node fields without antidiffusion
    if (a.S.p.antidiffinter == 1) k_n2m<false, false><<<grid, NTH, 0, st>>>(a);
    else k_n2m<false, true><<<grid, NTH, 0, st>>>(a);
  } else {
    k_n2m<true, false><<<grid, NTH, 0, st>>>(a);
    const unsigned nb = (unsigned)((a.g.nn + 127) / 128);
    k_n2m_bs_mode1<0><<<nb, 128, 0, st>>>(a);
    k_n2m_bs_mode1<1><<<nb, 128, 0, st>>>(a);
  }
}

void launch_move(const N2MArgs &a, cudaStream_t st) {
  const long quarters = (long)a.g.ncx * a.g.ncy * 4;
  k_vel_quads<<<(unsigned)((quarters + 255) / 256), 256, 0, st>>>(a.g, a.N, a.quad);
  if (a.n <= 0) return;
  long blocks = (a.n + 255) / 256;
  if (blocks > 152 * 8 * 4) blocks = 152 * 8 * 4;
  k_move<<<(unsigned)blocks, 256, 0, st>>>(a);
}

}  // namespace v2c
