// v2c_phys.cu -- per-marker physics of marker2nodes, in marker array order.
//
// For every marker strictly inside the model (interpolation.c:219): pressure
// at the marker (allinterpomp, interpolation.c:1923), density, thermal
// conductivity and ductile viscosity with the creep Newton
// (recalc_marker_properties.c, density_ductilevisc_calc.c), the RSF state
// update of calc_frictionpara (calc_RSF.c:224-295); for every marker the
// sticky-air flag candidate (interpolation.c:866-916).  Results go to
// per-marker arrays (mnu, mkt, mro) the scatter sweep reads.
//
// Then, unless disabled, the per-marker visco-elasto-plastic + RSF Newton
// (v2c_rsf.cuh) from the plain start (previous slip rate) or the network's
// proposal (v2c_mlp.cuh, evaluated by each warp on the tensor cores), with a
// fallback to the plain start when the proposal does not converge.
#include <math.h>

#include "v2c_kernels.h"
#include "v2c_mlp.cuh"
#include "v2c_rheology.cuh"
#include "v2c_rsf.cuh"

namespace v2c {

namespace {

constexpr int PT = 128;  // 4 warps

__device__ __forceinline__ void warp_add(unsigned long long *p, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(V2C_FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(p, v);
}
// largest value over the warp, one atomic per warp (non-negative doubles
// order like their bit patterns)
__device__ __forceinline__ void warp_max_bits(unsigned long long *p, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_down_sync(V2C_FULL, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0 && v) atomicMax(p, v);
}

// One instantiation per path, so each kernel carries only its own code:
// MODE = PHYS_OFF (no Newton), PHYS_SPLIT, PHYS_FP64, PHYS_COLLECT; LEARNED =
// the network's start (split and FP64 only).
enum { PHYS_OFF = 0, PHYS_SPLIT, PHYS_FP64, PHYS_COLLECT };

template <int MODE, bool LEARNED>
__global__ void __launch_bounds__(PT, 5) k_phys(PhysArgs a) {
  __shared__ MlpSmem S;
  const Grid &g = a.g;
  const int guess = MODE == PHYS_OFF ? V2C_GUESS_OFF : V2C_GUESS_PLAIN;
  const bool collect = MODE == PHYS_COLLECT;
  const bool learned = LEARNED;
  if (learned) {
    mlp_load_smem(S, a.mlp);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (PT / 32);
  const long n = a.n;
  const v2c_params &P = a.S.p;
  const bool fp64 = MODE == PHYS_FP64;
  // FP64 scalars of the Newton as float pairs, once per thread
  const ff dt_ff = ff_from_double(P.timestep), W_ff = ff_from_double(P.faultwidth),
           sn_ff = ff_from_double(P.nstress);
  for (long base = ((long)blockIdx.x * (PT / 32) + wl) * 32; base < n; base += nwarps * 32) {
    const long i = base + lane;
    const bool valid = i < n;
    bool act = false, solve = false;
    float mnu = 0.f, sigin = 0.f;
    int t = 0;
    Fric fr{0.f, 0.f, 1.f, 1.f, 0.f};
    float phi = 0.f;
    if (valid) {
      const int c = a.m.cell_in[i];
      const int ix = c / g.ncy, iy = c - ix * g.ncy;
      const float u = a.m.u_in[i], v = a.m.v_in[i];
      t = a.m.type[i];
      // sticky-air flag candidates: every marker, last in reference order wins
      if ((t == 1 || t == 2) && !collect) {
        long m3 = (long)ix * g.yn + iy + 1, q = -1;
        if (u < 0.5f && v < 0.5f) q = m3;
        else if (u < 0.5f && v > 0.5f) q = m3 + 1;
        else if (u > 0.5f && v < 0.5f) q = m3 + g.yn;
        else if (u > 0.5f && v > 0.5f) q = m3 + g.yn + 1;
        if (q >= 0 && q < g.nn)
          atomicMax(a.sticky_key + q, ((uint32_t)a.m.id[i] << 2) | (uint32_t)t);
      }
      act = true;
      if (ix == 0 || ix == g.ncx - 1) {
        double x = g.gx[ix] + (double)u * (g.gx[ix + 1] - g.gx[ix]);
        act = act && x > 0 && x < g.xsize;
      }
      if (iy == 0 || iy == g.ncy - 1) {
        double y = g.gy[iy] + (double)v * (g.gy[iy + 1] - g.gy[iy]);
        act = act && y > 0 && y < g.ysize;
      }
      if (act) {
        const Axis ax = make_axis(g.wx, g.ncx, ix, u * __ldg(g.wx + ix));
        const Axis ay = make_axis(g.wy, g.ncy, iy, v * __ldg(g.wy + iy));
        float e, nn;
        const long m3 = stencil_centre(g, ax, ay, u > 0.5f, v > 0.5f, e, nn);
        const float mpb = 1e-5f * bil(a.N.f(V2C_NF_PR), m3, g.yn, e, nn);
        const float T = a.m.tk[i];
        float mro, mbb;
        density32(a.R, P.densimod, t, T, mpb, mro, mbb);
        const float mkt = conductivity32(a.R, t, T, mpb);
        const float sxx = a.m.sxx[i], sxy = a.m.sxy[i];
        sigin = sqrtf(sxx * sxx + sxy * sxy);
        mnu = ductile_visc32(a.R, a.S, t, sigin, T, mpb);
        // calc_frictionpara: FP32 position away from the band, FP64 near it
        phi = a.m.phi[i];
        const float xf = __ldg(a.gxf + ix) + ax.X, yf = __ldg(a.gyf + iy) + ay.X;
        const float rad = fabsf(yf - ((float)P.fault_y + (float)P.fault_slope * xf));
        if (t > 0 && rad > (float)P.fault_hw + 1.0f) {
          phi = 50.f;
          fr.a = (float)P.a_hr; fr.b = (float)P.b_hr; fr.L = (float)P.L_hr;
          fr.V0 = (float)P.V0_hr; fr.mu0 = 0.6f;
        } else {
          const double x = g.gx[ix] + (double)u * (g.gx[ix + 1] - g.gx[ix]);
          const double y = g.gy[iy] + (double)v * (g.gy[iy + 1] - g.gy[iy]);
          phi = friction_marker(P, a.S.phi_reset0, x, y, t, phi, fr);
        }
        if (!collect) {
          if (phi != a.m.phi[i]) a.m.phi[i] = phi;
          a.m.mnu[i] = mnu;
          a.m.mkt[i] = mkt;
          if (P.densimod != 0) a.m.mro[i] = mro;
          if (!(mnu > 0.f)) atomicAdd(a.stat + ST_NAN, 1ull);
        }
        solve = (guess != V2C_GUESS_OFF || collect) && t > 0 && mnu > 0.f;
      }
    }
    if (guess == V2C_GUESS_OFF && !collect) continue;

    // ------------------------------------------- per-marker RSF Newton
    RsfIn in;
    float u_plain = 0.f;
    if (solve) {
      const float exx = a.m.exx[i], exy = a.m.exy[i];
      in.a = ff_f(fr.a); in.b = ff_f(fr.b); in.L = ff_f(fr.L); in.V0 = ff_f(fr.V0);
      in.mu0 = ff_f(fr.mu0);
      in.sn = (P.pmode == 0) ? sn_ff : ff_f(a.m.p[i]);
      in.dt = dt_ff; in.W = W_ff;
      in.phio = ff_f(phi);
      in.tau_old = ff_f(sigin);
      in.edot = ff_f(sqrtf(exx * exx + exy * exy));
      in.eta = ff_f(mnu);
      in.G = ff_f(a.R(RK_GG, t));
      const float vold = a.m.slipv[i];
      u_plain = (vold > 0.f) ? __logf(vold) : -30.f;
    }
    if (collect) {
      if (valid && i % a.xs_stride == 0 && i / a.xs_stride < a.xs_cap) {
        const long c = a.xs_cap, k = i / a.xs_stride;
        double *x = a.xs + k;
        if (solve) {
          x[V2C_RS_VOLD * c] = (double)a.m.slipv[i];
          x[V2C_RS_PHIOLD * c] = ff_to_double(in.phio);
          x[V2C_RS_A * c] = ff_to_double(in.a);
          x[V2C_RS_B * c] = ff_to_double(in.b);
          x[V2C_RS_L * c] = ff_to_double(in.L);
          x[V2C_RS_V0 * c] = ff_to_double(in.V0);
          x[V2C_RS_MU0 * c] = ff_to_double(in.mu0);
          x[V2C_RS_SN * c] = ff_to_double(in.sn);
          x[V2C_RS_DT * c] = ff_to_double(in.dt);
          x[V2C_RS_TAUOLD * c] = ff_to_double(in.tau_old);
          x[V2C_RS_EDOT * c] = ff_to_double(in.edot);
          x[V2C_RS_ETA * c] = ff_to_double(in.eta);
          x[V2C_RS_G * c] = ff_to_double(in.G);
        } else {
          x[V2C_RS_A * c] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: no problem
        }
      }
      continue;
    }
    // split form: markers whose load is certainly below the floor's yield
    // are done with one FP32 evaluation, and a warp with no other marker
    // skips the network
    bool at_floor = false;
    float A_floor = 0.f;
    if (solve && !fp64) at_floor = rsf_floor_certain(rsf32_of(in), A_floor);
    float u0 = u_plain;
    if (learned && __any_sync(V2C_FULL, solve && !at_floor)) {
      float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (solve && !at_floor) rsf_features(in, f);
#pragma unroll
      for (int k = 0; k < 8; k++) S.xin[wl][lane][k] = f[k];
      __syncwarp();
      mlp_warp_forward(S, wl);
      u0 = S.yout[wl][lane][0];
      __syncwarp();
    }
    unsigned long long it = 0, fb = 0, nc = 0, resbits = 0;
    if (solve) {
      RsfResult r = at_floor ? rsf_floor_result(in, A_floor)
                  : fp64     ? rsf_solve64(in, (double)u0, P.newton_rtol, P.newton_maxit)
                             : rsf_solve_split(in, rsf32_of(in), u0, P.newton_rtol, P.newton_maxit);
      it = r.it32 + r.itff + r.it64;
      if (!r.ok && learned) {
        RsfResult r2 = fp64 ? rsf_solve64(in, (double)u_plain, P.newton_rtol, P.newton_maxit)
                            : rsf_solve_split(in, rsf32_of(in), u_plain, P.newton_rtol, P.newton_maxit);
        it += r2.it32 + r2.itff + r2.it64;
        fb = 1;
        r = r2;
      }
      if (!r.ok) nc = 1;
      a.m.slipv[i] = r.Vf;
      if (r.res > 0) resbits = (unsigned long long)__double_as_longlong(r.res);
    }
    warp_max_bits(a.stat + ST_NEWTON_MAXRES_BITS, resbits);
    warp_add(a.stat + ST_NEWTON_ITERS, it);
    warp_add(a.stat + ST_NEWTON_FALLBACK, fb);
    warp_add(a.stat + ST_NEWTON_NONCONV, nc);
  }
}

}  // namespace

void launch_phys(const PhysArgs &a, cudaStream_t st) {
  if (a.n <= 0) return;
  long warps = (a.n + 31) / 32;
  long blocks = (warps + PT / 32 - 1) / (PT / 32);
  if (blocks > 152 * 16) blocks = 152 * 16;
  const v2c_params &p = a.S.p;
  const bool learned = p.newton_guess == V2C_GUESS_LEARNED && a.mlp != nullptr;
  const bool fp64 = p.newton_precision == V2C_NEWTON_FP64;
  const unsigned nb = (unsigned)blocks;
  if (a.xs) k_phys<PHYS_COLLECT, false><<<nb, PT, 0, st>>>(a);
  else if (p.newton_guess == V2C_GUESS_OFF) k_phys<PHYS_OFF, false><<<nb, PT, 0, st>>>(a);
  else if (fp64 && learned) k_phys<PHYS_FP64, true><<<nb, PT, 0, st>>>(a);
  else if (fp64) k_phys<PHYS_FP64, false><<<nb, PT, 0, st>>>(a);
  else if (learned) k_phys<PHYS_SPLIT, true><<<nb, PT, 0, st>>>(a);
  else k_phys<PHYS_SPLIT, false><<<nb, PT, 0, st>>>(a);
}

}  // namespace v2c
