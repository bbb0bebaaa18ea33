/*
 * v2c_bind.h -- the reference program's MIC routines on the GPU, working on
 * the reference's own global arrays (src/headevps.c, src/input_RSF.c).
 *
 * The reference compiles all of its sources into one translation unit
 * (src/i2evps.c:12-30).  v2c_bind.c is added to that unit after headevps.c
 * and input_RSF.c, and the call sites in src/i2evps.c:89-113 and
 * src/momentum_continuity_iterate.c:69,89 switch to the functions below
 * (same arguments and return values as the routines they replace):
 *
 *   marker2nodes()                       -> v2c_bind_marker2nodes()
 *   interpolate_center2basic_old(dt)     -> v2c_bind_interpolate_center2basic_old(dt)
 *   compute_before_solve(dt, rk)         -> v2c_bind_compute_before_solve(dt, rk)
 *   compute_after_solve(dt, rk)          -> v2c_bind_compute_after_solve(dt, rk)
 *   nodes2markers()                      -> v2c_bind_nodes2markers()
 *   moveandrotatemarkers()               -> v2c_bind_moveandrotatemarkers()
 *   calc_timestep(oldornew)              -> v2c_bind_calc_timestep(oldornew)
 *                                           (momentum_continuity_iterate.c:44,92)
 *   interpolate_basic2center()           -> v2c_bind_interpolate_basic2center()
 *   preparematrix(mukoef, dt, rk)        -> v2c_bind_preparematrix(mukoef, dt, rk)
 *   interpolate_center2basic(dt)         -> v2c_bind_interpolate_center2basic(dt)
 *                                           (momentum_continuity_iterate.c:71,87)
 *
 * Data movement.  The host arrays stay the truth for everything the host
 * solvers read and write.  Every call uploads the node arrays and brings
 * back the node arrays the routine writes; node values written by the GPU
 * carry FP32 precision.  The markers live on the GPU between calls: they
 * are uploaded on the first call and after v2c_bind_markers_changed(), and
 * the host marker arrays (positions, T, strain, pressure, stresses, strain
 * rates, velocities, state, cohesion) are refreshed only by
 * v2c_bind_markers_to_host() when v2c_bind_sync_markers is 0 (the default):
 * call it before save_model, postproc or any other host code that reads
 * marker arrays.  With v2c_bind_sync_markers = 1 they are refreshed after
 * every call that changes them, a full marker download per call.  The
 * per-marker friction
 * parameters the reference stores (mark_a, mark_b, mark_L, mark_L0,
 * mark_V0, markC0, fric_static) are recomputed from position on the GPU and
 * are not written back.
 *
 * Errors: a failing call prints one line and sets the reference's errcheck
 * flag, as the reference does for its own numerical errors.
 */
#ifndef V2C_BIND_H
#define V2C_BIND_H

extern int v2c_bind_sync_markers;

void v2c_bind_marker2nodes(void);
double v2c_bind_interpolate_center2basic_old(double dt);
void v2c_bind_compute_before_solve(double dt, int rk);
void v2c_bind_preparematrix(double mukoef, double dt, int rk);
double v2c_bind_compute_after_solve(double dt, int rk);
double v2c_bind_nodes2markers(void);
void v2c_bind_moveandrotatemarkers(void);
double v2c_bind_calc_timestep(int oldornew);
double v2c_bind_interpolate_basic2center(void);
double v2c_bind_interpolate_center2basic(double dt);
/* the marker part of solve_temperature; the thermal solve stays on the host
 * (temperature_iterate.c:2-179), followed by this call in place of its
 * lines 181-412 */
void v2c_bind_marker_temperature(void);

/* the host changed marker arrays (temperature solve, loading a file) */
void v2c_bind_markers_changed(void);
/* the host changed gx/gy, the rock table or the boundary equations */
void v2c_bind_model_changed(void);
/* copy the device markers into the host arrays */
void v2c_bind_markers_to_host(void);
/* release the GPU context */
void v2c_bind_close(void);

#endif
