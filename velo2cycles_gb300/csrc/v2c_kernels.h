// v2c_kernels.h -- host-side launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>

#include "v2c_internal.cuh"

namespace v2c {

struct SortBufs {
  int32_t *counts;   // [ncell]
  int32_t *start;    // [ncell+1]
  int4 *qstart;      // [ncell+1]: start of each quarter class of a cell (see launch_sort)
  int32_t *slot;     // [cap]
  int32_t *tmp;      // [cap]
  int32_t *perm;     // [cap]
  int32_t *blocksum; // scan scratch
  long blocksum_cap;
};

// Sort markers by cell, within a cell by quarter class
// q = 2 (v > 1/2) + (u > 1/2), within a class by array index: perm, start
// and qstart (x, y, z, w = first sorted position of class 0, 1, 2, 3 of
// the cell; qstart[ncell].x = n).  Array indices must be below 2^30.
constexpr long SORT_MAX_MARKERS = 1L << 30;
void launch_sort(const int32_t *cell, const float *u, const float *v, long n, long ncell,
                 SortBufs &b, unsigned long long *stat, cudaStream_t st);

// exclusive scan of in[0, m) into out[0, m], total in out[m]; blocksum
// holds scan_blocks(m) entries
long scan_blocks(long m);
void launch_scan(const int32_t *in, long m, int32_t *out, int32_t *blocksum, cudaStream_t st);

// preparematrix + gausmat4_add (v2c_stokes.cu): two passes over the
// 3 nodenum equations, counting then filling
struct StokesArgs {
  Grid g;
  Nodes N;
  const long *bondm;   // [nodenum * 4]
  const long *bondn;   // [bondnum * 3]
  const double *bondv; // [bondnum * 4]
  long bondnum;
  double mukoef, dt, gxkoef, gykoef, timebond, timesum, timestep, nubeg;
  int drunkensailor, inertyn, compressible;
  int32_t *cnt;        // [3 nodenum + 1]: coefficients per row, then row starts
  int32_t *ja;         // [nnz] (fill pass)
  double *a;           // [nnz] (fill pass)
  // rows kept by the count pass (STOKES_ROW_MAX entries per row), so that
  // the fill pass only moves them; null: the fill pass rebuilds each row
  int32_t *ell_col;
  double *ell_val;
  double *b;           // [3 nodenum]
  int *err;            // set where the reference stops or a row leaves the grid
};
constexpr int STOKES_ROW_MAX = 24;
void launch_stokes_count(const StokesArgs &a, cudaStream_t st);
void launch_stokes_fill(const StokesArgs &a, cudaStream_t st);

// marker2nodes sweep (scatter + node tail) and its follow-ups
struct M2NArgs {
  Grid g;
  Nodes N;
  Markers m;
  Rock R;
  Scal S;
  const int32_t *perm;
  const int32_t *start;
  const int4 *qstart;
  uint32_t *sticky_key;
  unsigned long long *stat;
  const float *gxf, *gyf;  // FP32 line positions (coarse band test)
  int TX;
  long n = 0;  // markers (chooses the sweep's occupancy)
};
void launch_m2n(const M2NArgs &a, cudaStream_t st);

// per-marker physics (+ optional RSF Newton), marker array order
struct PhysArgs {
  Grid g;
  Nodes N;
  Markers m;
  Rock R;
  Scal S;
  long n;
  uint32_t *sticky_key;
  unsigned long long *stat;
  const float *gxf, *gyf;
  const float *mlp;  // packed network (device) or null
  // collection mode (v2c_collect_newton_states): when xs is set the kernel
  // writes the Newton state of every xs_stride-th marker to
  // xs[V2C_RS_N][xs_cap] and changes nothing else
  double *xs = nullptr;
  long xs_stride = 1, xs_cap = 0;
  // the Newton problems the physics pass leaves for the Newton kernel:
  // marker indices (capacity n) and their count (device)
  int32_t *list = nullptr;
  unsigned *list_n = nullptr;
  float *guess = nullptr;  // the network's start per listed problem (capacity n)
};
void launch_phys(const PhysArgs &a, cudaStream_t st);
void launch_sticky(const Nodes &N, const uint32_t *key, long nn, cudaStream_t st);
void launch_dphis(const Grid &g, const Nodes &N, cudaStream_t st);

// boundary corrections: flattened rows x[row] = c + sum coef*value[ref]
struct BcRows {
  int n;            // rows
  const int *field; // node field written
  const long *node; // node written
  const float *c;   // constant
  const int *nref;  // number of references (<= V2C_BC_MAXREF)
  const int *rfield;// [n*MAXREF] field of the referenced value
  const long *rnode;// [n*MAXREF]
  const float *rcoef;
};
#define V2C_BC_MAXREF 8
void launch_bc(const BcRows &rows, const Nodes &N, float *scratch, cudaStream_t st);
void launch_node_to_f32(const double *src, float *dst, long n, cudaStream_t st);
void launch_node_to_f64(const float *src, double *dst, long n, cudaStream_t st);
// count node fields (ids in fields[], count <= V2C_NF_N) to / from a staging
// area of count x nn doubles in list order
void launch_fields_to_f64(const float *base, long nn, const int *fields, int count, double *stage,
                          cudaStream_t st);
void launch_fields_to_f32(const double *stage, long nn, const int *fields, int count, float *base,
                          cudaStream_t st);

void launch_c2b_old(const Grid &g, const Nodes &N, cudaStream_t st);
void launch_c2b(const Grid &g, const Nodes &N, double dt, int use_dsxx, cudaStream_t st);
void launch_b2c(const Grid &g, const Nodes &N, unsigned long long *stat, cudaStream_t st);
// vx64, vy64: FP64 node velocities for the strain rates (nullptr: the FP32 fields)
void launch_recompute(const Grid &g, const Nodes &N, const Scal &S, double dt, const double *vx64,
                      const double *vy64, cudaStream_t st);
void launch_copyarrays(const Grid &g, const Nodes &N, cudaStream_t st);
// accumulated slip of every marker: acc[i] += dt * slipv[i]
void launch_marker_slip_acc(const float *slipv, long n, double dt, double *acc, cudaStream_t st);
void launch_unpermute_f64(const double *src, const int32_t *id, double *out, long n, cudaStream_t st);
void launch_slip_acc(const Grid &g, const Nodes &N, double dt, double *acc, cudaStream_t st);
void launch_before_solve(const Grid &g, const Nodes &N, const Scal &S, double dt, int rk,
                         unsigned long long *stat, cudaStream_t st);
void launch_after_solve(const Grid &g, const Nodes &N, const Scal &S, double dt, int rk,
                        double *red, cudaStream_t st);

// Immobile markers (moveandrotatemarkers.c:88-171): what the move kernel
// records per reference marker number, and the scratch of the compaction
// that appends the spawned markers and refills out-of-model slots.
struct ImmBufs {
  int32_t *spawn;          // [cap] 1: the immobile marker spawned (by id)
  int32_t *out;            // [cap] 1: the mobile marker ends outside the model (by id)
  int32_t *spawn_rank;     // [cap + 1] exclusive scan of spawn, total last
  int32_t *out_rank;       // [cap + 1] exclusive scan of out, total last
  int32_t *sp_cell;        // [cap] spawn position (by id)
  float *sp_u, *sp_v;
  int32_t *src;            // [cap] id of the immobile marker of each spawn rank
  int32_t *inv;            // [cap] array index of each id
  int32_t *blocksum;       // scan scratch (scan_blocks(cap) entries)
  int32_t *totals;         // [2] A (spawned), O (out of model)
};
// After launch_move: ranks, refills and appends; returns through *added the
// markers appended after the last one (the caller checks it against the
// capacity first through `cap`; V2C_ERR_CAPACITY leaves nothing changed).
// Synchronises the stream once (the new marker count).
int launch_immobile_compact(const Markers &m, long n, long cap, ImmBufs &b, long *added,
                            cudaStream_t st);

// nodes2markers + move sweep
struct N2MArgs {
  Grid g;
  Nodes N;
  Markers m;
  Rock R;
  Scal S;
  const int32_t *perm;
  const int32_t *start;
  const int4 *qstart;
  unsigned long long *stat;
  const float *gyf;  // FP32 line positions (coarse depth test)
  float4 *quad;      // allinteri's bilinear forms per cell quarter [ncell * QUAD_FLOAT4]
  long n;            // markers
  int TX;
  int do_n2m;
  // interpolationmod 1: the tile sweep writes each marker's back-scatter
  // payload (BS_N fields, SoA by sorted position) here and per-node gather
  // kernels sum it; null for interpolationmod 2
  float *bs = nullptr;
  // the move records spawns and out-of-model markers here when the markers
  // include immobile ones (has_imm; device pointers, passed by value)
  ImmBufs imm{};
  int has_imm = 0;
};
enum { BS_U = 0, BS_V, BS_PHIS, BS_SXY, BS_EXY, BS_ES, BS_PR, BS_SXX, BS_EXX, BS_N };
// float4 coefficient sets per cell: 4 quarters x (VX, VY, ESP)
constexpr int QUAD_FLOAT4 = 12;
// nodes2markers: gather, marker update, back-scatter (cell-column tiles)
void launch_n2m(const N2MArgs &a, cudaStream_t st);
// moveandrotatemarkers: one thread per marker, new positions to *_out
void launch_move(const N2MArgs &a, cudaStream_t st);

// the marker part of solve_temperature (v2c_temp.cu)
struct TempArgs {
  Grid g;
  Nodes N;
  Markers m;
  const int32_t *perm;
  const int32_t *start;
  long n, ncell;
  float heatdif, dt, tdeep;
  double tdeep64;
  // FP64 copies of the node temperatures TK (solved) and TK2 (before), as
  // uploaded; null: the FP32 node fields are used
  const double *tk64 = nullptr, *tk2_64 = nullptr;
  float *dtk1, *wt;  // per sorted position (scratch)
  float *tol;        // per node (scratch)
};
void launch_temperature(const TempArgs &a, cudaStream_t st);

// calc_timestep over the device node fields (synchronises the stream);
// scratch: TIMESTEP_SCRATCH doubles
constexpr long TIMESTEP_SCRATCH = (152 * 4 * 8 + 1) * 32 + 64;
int calc_timestep_device(const Grid &g, const Nodes &N, const Scal &S, const v2c_timestep_ctl &c,
                         int oldornew, double *scratch, long scratch_doubles,
                         v2c_timestep_info *info, cudaStream_t st);

// upload / download helpers
void launch_assign(const Grid &g, const double *x, const double *y, long n, Markers m,
                   unsigned long long *stat, cudaStream_t st);
void launch_f64_to_f32(const double *src, float *dst, long n, cudaStream_t st);
// FP64 values as float pairs hi + lo, and back (out[id[i]] = hi[i] + lo[i])
void launch_f64_to_pair(const double *src, float *hi, float *lo, long n, cudaStream_t st);
void launch_unpermute_pair(const float *hi, const float *lo, const int32_t *id, double *out,
                           long n, cudaStream_t st);
void launch_gather_f32(const float *src, const int32_t *perm, float *dst, long n, cudaStream_t st);
void launch_gather_i32(const int32_t *src, const int32_t *perm, int32_t *dst, long n, cudaStream_t st);
void launch_gather_i8(const int8_t *src, const int32_t *perm, int8_t *dst, long n, cudaStream_t st);
void launch_gather_u8(const uint8_t *src, const int32_t *perm, uint8_t *dst, long n, cudaStream_t st);
// out[id[i]] = (double)src[i]
void launch_unpermute_f32(const float *src, const int32_t *id, double *out, long n, cudaStream_t st);
void launch_unpermute_i32(const int32_t *src, const int32_t *id, int32_t *out, long n, cudaStream_t st);
void launch_unpermute_u8(const uint8_t *src, const int32_t *id, uint8_t *out, long n, cudaStream_t st);
void launch_unpermute_i8(const int8_t *src, const int32_t *id, int8_t *out, long n, cudaStream_t st);
// FP64 positions in reference numbering
void launch_positions(const Grid &g, const Markers &m, long n, double *x, double *y,
                      cudaStream_t st);

}  // namespace v2c
