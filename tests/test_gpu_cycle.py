"""Seismic-cycle step sequence (v2c_cycle_step) on the GPU: captured CUDA
graphs replay the eager step bit for bit, the reference form (no per-marker
Newton) tracks the FP64 oracle through an event, and the learned split form
tracks the plain FP64 form.
"""
import numpy as np
import pytest

import oracle
from velo2cycles_gb300 import abi, cycle, mic, newton, synth

from .parity import nxsearch_np, rel_err

pytestmark = pytest.mark.gpu

SCHED = cycle.Schedule(n_inter=4, slip_budget=0.004, v_pulse=1.0, width=1500.0)


class OracleStepper:
    """The cycle step on the oracle restatement (FP64), same call order."""

    def __init__(self, case, fields):
        self.r = oracle.Restatement(case.copy())
        self.fields = fields
        self.timesum = float(case.params["timesum"])
        self.slip = np.zeros(case.nodenum)
        yn = case.gy.size
        m = np.arange(case.nodenum)
        self.inner = ((m // yn >= 1) & (m % yn >= 1) & (m // yn < case.gx.size - 1) &
                      (m % yn < yn - 1))

    def cycle_step(self, regime, dt):
        r = self.r
        r.nodes[abi.NF_VX][:] = self.fields[regime][0]
        r.nodes[abi.NF_VY][:] = self.fields[regime][1]
        r.set_params(timestep=dt, timesum=self.timesum)
        r.marker2nodes()
        r.center2basic_old()
        r.compute_before_solve(dt, 0)
        r.basic2center()
        r.recompute_stress(dt)
        r.center2basic(dt)
        r.compute_after_solve(dt, 0)
        r.copyarrays()
        self.slip[self.inner] += dt * r.nodes[abi.NF_RK_SLIPRS_FINAL][self.inner]
        r.nodes2markers()
        r.move()
        self.timesum += dt
        r.set_params(timesum=self.timesum)

    def calc_timestep(self, oldornew):
        return self.r.calc_timestep(oldornew)[1]


def _gpu(case, fields, **params):
    c = case.copy()
    c.params.update(params)
    m = mic.from_case(c)
    for k in (0, 1):
        m.cycle_set_velocity(k, *fields[k])
    return m


class _G:
    def __init__(self, m, graph):
        self.m, self.graph = m, graph

    def cycle_step(self, regime, dt):
        self.m.cycle_step(regime, dt, use_graph=self.graph)

    def calc_timestep(self, oldornew):
        return self.m.calc_timestep(oldornew)


@pytest.fixture(scope="module")
def case(built_lib, oracle_built):
    return synth.make_case("small", seed=21)


def test_graph_replay_matches_eager(case):
    fields = cycle.pulse_fields(case, SCHED)
    ma, mb = _gpu(case, fields), _gpu(case, fields)
    rec = cycle.run(_G(ma, True), SCHED, 16)
    assert 1 in rec.regime and min(rec.dt) == SCHED.dt_co and max(rec.dt) == SCHED.dt_inter
    cycle.run(_G(mb, False), SCHED, 16, forced=list(zip(rec.regime, rec.dt)))
    f = [abi.NF_SXY, abi.NF_SXX, abi.NF_PHIS, abi.NF_RK_SLIPRS_FINAL, abi.NF_NU, abi.NF_EXXPL]
    na, nb = ma.download_nodes(f), mb.download_nodes(f)
    for k in f:
        assert np.array_equal(na[k], nb[k], equal_nan=True), abi.node_field_names()[k]
    mk = [abi.MF_X, abi.MF_Y, abi.MF_XX, abi.MF_XY, abi.MF_PHI]
    ka, kb = ma.download_markers(mk), mb.download_markers(mk)
    for k in mk:
        assert np.array_equal(ka[k], kb[k]), abi.marker_field_names()[k]
    assert np.array_equal(ma.cycle_slip(), mb.cycle_slip())
    sa, sb = ma.status(), mb.status()
    assert sa["kernel_launches"] > 0 and sa["n_nan"] == sb["n_nan"]
    ma.close(); mb.close()


def test_reference_form_tracks_oracle(case):
    """Per-marker Newton off (the reference's own algorithm): after an
    interseismic stretch, an event and the relaxation steps, the GPU state
    stays within FP32 drift of the FP64 oracle."""
    fields = cycle.pulse_fields(case, SCHED)
    m = _gpu(case, fields, newton_guess=abi.GUESS_OFF)
    ref = OracleStepper(case, fields)
    rec_ref = cycle.run(ref, SCHED, 12)
    rec = cycle.run(_G(m, True), SCHED, 12, forced=list(zip(rec_ref.regime, rec_ref.dt)))
    assert 1 in rec_ref.regime
    # the GPU's own regime decisions would have been the same
    drv = cycle.Driver(SCHED)
    own = [(0, SCHED.dt_inter)] + [drv.next(v) for v in rec.maxvel[:-1]]
    assert own == list(zip(rec_ref.regime, rec_ref.dt))
    slip = m.cycle_slip()
    e_slip = rel_err(slip[ref.inner], ref.slip[ref.inner])
    nodes = m.download_nodes([abi.NF_SXY, abi.NF_PHIS])
    e_sxy = rel_err(nodes[abi.NF_SXY], ref.r.nodes[abi.NF_SXY])
    e_phi = rel_err(nodes[abi.NF_PHIS], ref.r.nodes[abi.NF_PHIS])
    mk = m.download_markers([abi.MF_X, abi.MF_XY])
    wx = np.diff(case.gx)[nxsearch_np(case.gx, ref.r.marks[abi.MF_X])]
    e_x = (np.abs(mk[abi.MF_X] - ref.r.marks[abi.MF_X]) / wx).max()
    e_mxy = rel_err(mk[abi.MF_XY], ref.r.marks[abi.MF_XY])
    print(f"drift vs oracle after {len(rec.dt)} steps: slip {e_slip:.2e} sxy {e_sxy:.2e} "
          f"phis {e_phi:.2e} x {e_x:.2e} cells, marker sxy {e_mxy:.2e}")
    assert e_slip <= 1e-4 and e_sxy <= 1e-4 and e_phi <= 1e-4
    assert e_x <= 1e-5 and e_mxy <= 1e-4
    m.close()


def test_learned_split_tracks_plain_fp64(case):
    """The learned-start split-precision form against the plain FP64 form on
    the same regime sequence: the Newton converges to the same residual, so
    accumulated slip and stresses agree to FP32 drift."""
    fields = cycle.pulse_fields(case, SCHED)
    mp = _gpu(case, fields, newton_guess=abi.GUESS_PLAIN, newton_precision=abi.NEWTON_FP64)
    rec = cycle.run(_G(mp, True), SCHED, 12)
    ml = _gpu(case, fields, newton_guess=abi.GUESS_LEARNED, newton_precision=abi.NEWTON_SPLIT)
    newton.load(ml, newton.random_params(5))  # any start: the Newton judges it
    cycle.run(_G(ml, True), SCHED, 12, forced=list(zip(rec.regime, rec.dt)))
    sp, sl = mp.cycle_slip(), ml.cycle_slip()
    assert rel_err(sl, sp) <= 1e-4
    a, b = mp.download_nodes([abi.NF_SXY]), ml.download_nodes([abi.NF_SXY])
    assert rel_err(b[abi.NF_SXY], a[abi.NF_SXY]) <= 1e-4
    st = ml.status()
    assert st["newton_nonconv"] == 0 and st["newton_max_res"] <= 1e-10
    mp.close(); ml.close()
