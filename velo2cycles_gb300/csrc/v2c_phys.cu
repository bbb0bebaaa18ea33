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

// One instantiation per path: MODE = PHYS_OFF (no Newton), PHYS_SPLIT,
// PHYS_FP64 (the Newton problems go to the list), PHYS_COLLECT.
enum { PHYS_OFF = 0, PHYS_SPLIT, PHYS_FP64, PHYS_COLLECT };

// Friction parameters of a marker (calc_frictionpara, calc_RSF.c:224-295)
// and its new state: FP32 position away from the band, FP64 near it.
__device__ __forceinline__ float marker_friction(const PhysArgs &a, int ix, int iy, float u,
                                                 float v, float Xc, float Yc, int t, float phi,
                                                 Fric &fr) {
  const Grid &g = a.g;
  const v2c_params &P = a.S.p;
  const Scal &S = a.S;
  const float xf = __ldg(a.gxf + ix) + Xc, yf = __ldg(a.gyf + iy) + Yc;
  const float rad = fabsf(yf - (S.fault_y_f + S.fault_slope_f * xf));
  if (t > 0 && rad > S.fault_hw1_f) {
    fr.a = S.a_hr_f; fr.b = S.b_hr_f; fr.L = S.L_hr_f; fr.V0 = S.V0_hr_f; fr.mu0 = 0.6f;
    return 50.f;
  }
  const double x = g.gx[ix] + (double)u * (g.gx[ix + 1] - g.gx[ix]);
  const double y = g.gy[iy] + (double)v * (g.gy[iy + 1] - g.gy[iy]);
  return friction_marker(P, a.S.phi_reset0, x, y, t, phi, fr);
}

// the per-marker Newton problem of marker i, after the physics pass wrote
// its viscosity and state
__device__ __forceinline__ void marker_problem(const PhysArgs &a, long i, const ff &dt_ff,
                                               const ff &W_ff, const ff &sn_ff, RsfIn &in,
                                               float &uplain) {
  const Grid &g = a.g;
  const v2c_params &P = a.S.p;
  const int c = a.m.cell_in[i];
  const int ix = c / g.ncy, iy = c - ix * g.ncy;
  const float u = a.m.u_in[i], v = a.m.v_in[i];
  const int t = a.m.type[i];
  Fric fr{0.f, 0.f, 1.f, 1.f, 0.f};
  const float phi = a.m.phi[i];
  (void)marker_friction(a, ix, iy, u, v, u * __ldg(g.wx + ix), v * __ldg(g.wy + iy), t, phi,
                        fr);
  const float sxx = a.m.sxx[i], sxy = a.m.sxy[i], exx = a.m.exx[i], exy = a.m.exy[i];
  in.a = ff_f(fr.a); in.b = ff_f(fr.b); in.L = ff_f(fr.L); in.V0 = ff_f(fr.V0);
  in.mu0 = ff_f(fr.mu0);
  in.sn = (P.pmode == 0) ? sn_ff : ff_f(a.m.p[i]);
  in.dt = dt_ff; in.W = W_ff;
  in.phio = ff_f(phi);
  in.tau_old = ff_f(sqrtf(sxx * sxx + sxy * sxy));
  in.edot = ff_f(sqrtf(exx * exx + exy * exy));
  in.eta = ff_f(a.m.mnu[i]);
  in.G = ff_f(a.R(RK_GG, t));
  const float vold = a.m.slipv[i];
  uplain = (vold > 0.f) ? __logf(vold) : -30.f;
}

template <int MODE>
__global__ void __launch_bounds__(PT, 5) k_phys(PhysArgs a) {
  const Grid &g = a.g;
  const bool collect = MODE == PHYS_COLLECT;
  const bool newton = MODE == PHYS_SPLIT || MODE == PHYS_FP64;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (PT / 32);
  const long n = a.n;
  const v2c_params &P = a.S.p;
  const ff dt_ff{a.S.dt_hi, a.S.dt_lo}, W_ff{a.S.W_hi, a.S.W_lo}, sn_ff{a.S.sn_hi, a.S.sn_lo};
  unsigned long long it = 0;
  for (long base = ((long)blockIdx.x * (PT / 32) + wl) * 32; base < n; base += nwarps * 32) {
    const long i = base + lane;
    const bool valid = i < n;
    bool solve = false;
    float mnu = 0.f, sigin = 0.f, phi = 0.f;
    int t = 0;
    Fric fr{0.f, 0.f, 1.f, 1.f, 0.f};
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
      bool act = true;
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
        // pressure in bar, 1e-5 P, as a float pair
        const ff mpb_ff = ff_mul(bil_ff(a.N.f(V2C_NF_PR), m3, g.yn, e, nn),
                                 ff{9.99999975e-06f, 2.52621247e-13f});
        const float mpb = mpb_ff.hi;
        const float T = a.m.tk[i];
        float mro, mbb;
        density32(a.R, P.densimod, t, T, mpb, mro, mbb);
        const float mkt = conductivity32(a.R, t, T, mpb);
        const float sxx = a.m.sxx[i], sxy = a.m.sxy[i];
        sigin = sqrtf(sxx * sxx + sxy * sxy);
        const ff sig2 = ff_add(ff_mul(ff_f(sxx), ff_f(sxx)), ff_mul(ff_f(sxy), ff_f(sxy)));
        mnu = ductile_visc32(a.R, a.S, t, sig2, T, a.m.tk_lo[i], mpb_ff);
        const float phi0 = a.m.phi[i];
        phi = marker_friction(a, ix, iy, u, v, ax.X, ay.X, t, phi0, fr);
        if (!collect) {
          if (phi != phi0) a.m.phi[i] = phi;
          a.m.mnu[i] = mnu;
          a.m.mkt[i] = mkt;
          if (P.densimod != 0) a.m.mro[i] = mro;
          if (!(mnu > 0.f)) atomicAdd(a.stat + ST_NAN, 1ull);
        }
        solve = (newton || collect) && t > 0 && mnu > 0.f;
      }
    }
    if (!newton && !collect) continue;
    if (collect) {
      if (valid && i % a.xs_stride == 0 && i / a.xs_stride < a.xs_cap) {
        const long c = a.xs_cap, k = i / a.xs_stride;
        double *x = a.xs + k;
        if (solve) {
          const float exx = a.m.exx[i], exy = a.m.exy[i];
          x[V2C_RS_VOLD * c] = (double)a.m.slipv[i];
          x[V2C_RS_PHIOLD * c] = (double)phi;
          x[V2C_RS_A * c] = (double)fr.a;
          x[V2C_RS_B * c] = (double)fr.b;
          x[V2C_RS_L * c] = (double)fr.L;
          x[V2C_RS_V0 * c] = (double)fr.V0;
          x[V2C_RS_MU0 * c] = (double)fr.mu0;
          x[V2C_RS_SN * c] = (P.pmode == 0) ? P.nstress : (double)a.m.p[i];
          x[V2C_RS_DT * c] = P.timestep;
          x[V2C_RS_TAUOLD * c] = (double)sigin;
          x[V2C_RS_EDOT * c] = (double)sqrtf(exx * exx + exy * exy);
          x[V2C_RS_ETA * c] = (double)mnu;
          x[V2C_RS_G * c] = (double)a.R(RK_GG, t);
        } else {
          x[V2C_RS_A * c] = __longlong_as_double(0x7ff8000000000000ll);  // NaN: no problem
        }
      }
      continue;
    }
    // split form: a load certainly below the floor's yield is done with one
    // FP32 evaluation; every other problem goes to the list
    bool need = solve;
    if (solve && MODE == PHYS_SPLIT) {
      const float exx = a.m.exx[i], exy = a.m.exy[i];
      RsfIn in;
      in.a = ff_f(fr.a); in.b = ff_f(fr.b); in.L = ff_f(fr.L); in.V0 = ff_f(fr.V0);
      in.mu0 = ff_f(fr.mu0); in.sn = (P.pmode == 0) ? sn_ff : ff_f(a.m.p[i]);
      in.dt = dt_ff; in.W = W_ff; in.phio = ff_f(phi); in.tau_old = ff_f(sigin);
      in.edot = ff_f(sqrtf(exx * exx + exy * exy)); in.eta = ff_f(mnu);
      in.G = ff_f(a.R(RK_GG, t));
      float A_floor;
      if (rsf_floor_certain(rsf32_of(in), A_floor)) {
        a.m.slipv[i] = 1e-40f;
        it += 1;
        need = false;
      }
    }
    const unsigned bal = __ballot_sync(V2C_FULL, need);
    unsigned slot0 = 0;
    if (lane == 0 && bal) slot0 = atomicAdd(a.list_n, (unsigned)__popc(bal));
    slot0 = __shfl_sync(V2C_FULL, slot0, 0);
    if (need) a.list[slot0 + __popc(bal & ((1u << lane) - 1))] = (int32_t)i;
  }
  if (newton) warp_add(a.stat + ST_NEWTON_ITERS, it);
}

// The learned start of every listed problem, 32 per warp: the plain start
// (the previous slip rate) where its FP32 residual ratio is already below
// RSF_NET_MIN_RES, else the better of it and the network's proposal
// (evaluated by the warp on the BF16 tensor cores only when one of its
// problems needs it), written to guess[e]; a kernel of its own so the
// Newton kernel keeps the occupancy of the plain start.
__global__ void __launch_bounds__(PT, 4) k_guess(PhysArgs a, float *guess) {
  __shared__ MlpSmem S;
  mlp_load_smem(S, a.mlp);
  __syncthreads();
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (PT / 32);
  const long cnt = *a.list_n;
  const ff dt_ff{a.S.dt_hi, a.S.dt_lo}, W_ff{a.S.W_hi, a.S.W_lo}, sn_ff{a.S.sn_hi, a.S.sn_lo};
  for (long base = ((long)blockIdx.x * (PT / 32) + wl) * 32; base < cnt; base += nwarps * 32) {
    const long e = base + lane;
    const bool valid = e < cnt;
    RsfIn in;
    float uplain = 0.f, rp = 0.f, up = 0.f;
    bool need = false;
    if (valid) {
      marker_problem(a, a.list[e], dt_ff, W_ff, sn_ff, in, uplain);
      rp = rsf_start_residual(rsf32_of(in), uplain, up);
      need = !(rp <= RSF_NET_MIN_RES);
    }
    float u0 = uplain;
    if (__any_sync(V2C_FULL, need)) {
      float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (need) rsf_features(in, f);
#pragma unroll
      for (int k = 0; k < 8; k++) S.xin[wl][lane][k] = f[k];
      __syncwarp();
      mlp_warp_forward(S, wl);
      float un;
      if (need && rsf_start_residual(rsf32_of(in), S.yout[wl][lane][0], un) < rp) u0 = un;
      __syncwarp();
    }
    if (valid) guess[e] = u0;
  }
}

// The listed Newton problems, 32 per warp, densely: the split or FP64 solve
// from the plain start or (LEARNED) the network's guess[e], restarting from
// the plain start when that does not converge.  The list order comes from
// integer atomics; each problem's result depends only on its own inputs.
template <bool FP64, bool LEARNED>
__global__ void __launch_bounds__(PT, 5) k_newton(PhysArgs a, const float *guess) {
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * (PT / 32);
  const long cnt = *a.list_n;
  const v2c_params &P = a.S.p;
  const ff dt_ff{a.S.dt_hi, a.S.dt_lo}, W_ff{a.S.W_hi, a.S.W_lo}, sn_ff{a.S.sn_hi, a.S.sn_lo};
  unsigned long long it = 0, fb = 0, nc = 0, resbits = 0;
  for (long base = ((long)blockIdx.x * (PT / 32) + wl) * 32; base < cnt; base += nwarps * 32) {
    const long e = base + lane;
    if (e >= cnt) continue;
    const long i = a.list[e];
    RsfIn in;
    float uplain;
    marker_problem(a, i, dt_ff, W_ff, sn_ff, in, uplain);
    const float u0 = LEARNED ? guess[e] : uplain;
    RsfResult r = FP64 ? rsf_solve64(in, (double)u0, P.newton_rtol, P.newton_maxit)
                       : rsf_solve_split(in, rsf32_of(in), u0, P.newton_rtol, P.newton_maxit);
    it += r.it32 + r.itff + r.it64;
    if (!r.ok && LEARNED && u0 != uplain) {
      RsfResult r2 = FP64 ? rsf_solve64(in, (double)uplain, P.newton_rtol, P.newton_maxit)
                          : rsf_solve_split(in, rsf32_of(in), uplain, P.newton_rtol, P.newton_maxit);
      it += r2.it32 + r2.itff + r2.it64;
      fb += 1;
      r = r2;
    }
    if (!r.ok) nc += 1;
    a.m.slipv[i] = r.Vf;
    if (r.res > 0) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(r.res);
      if (b > resbits) resbits = b;
    }
  }
  warp_max_bits(a.stat + ST_NEWTON_MAXRES_BITS, resbits);
  warp_add(a.stat + ST_NEWTON_ITERS, it);
  warp_add(a.stat + ST_NEWTON_FALLBACK, fb);
  warp_add(a.stat + ST_NEWTON_NONCONV, nc);
}

// resident blocks of a kernel on the whole GPU (grid-stride launches)
template <class K>
unsigned resident_grid(K kernel, int threads) {
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  return (unsigned)((per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 152));
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
  if (a.xs) {
    k_phys<PHYS_COLLECT><<<nb, PT, 0, st>>>(a);
    return;
  }
  if (p.newton_guess == V2C_GUESS_OFF) {
    k_phys<PHYS_OFF><<<nb, PT, 0, st>>>(a);
    return;
  }
  cudaMemsetAsync(a.list_n, 0, sizeof(unsigned), st);
  if (fp64) k_phys<PHYS_FP64><<<nb, PT, 0, st>>>(a);
  else k_phys<PHYS_SPLIT><<<nb, PT, 0, st>>>(a);
  if (learned) k_guess<<<resident_grid(k_guess, PT), PT, 0, st>>>(a, a.guess);
  if (fp64 && learned)
    k_newton<true, true><<<resident_grid(k_newton<true, true>, PT), PT, 0, st>>>(a, a.guess);
  else if (fp64)
    k_newton<true, false><<<resident_grid(k_newton<true, false>, PT), PT, 0, st>>>(a, a.guess);
  else if (learned)
    k_newton<false, true><<<resident_grid(k_newton<false, true>, PT), PT, 0, st>>>(a, a.guess);
  else
    k_newton<false, false><<<resident_grid(k_newton<false, false>, PT), PT, 0, st>>>(a, a.guess);
}

}  // namespace v2c
