"""Parity of the CUDA MIC step with the oracle restatement (GPU).

Same seeded state on both sides; the GPU stores marker fields in FP32 and
positions as cell + FP32 offset, the oracle runs FP64 on the original
inputs.  Tolerances (relative to each field's magnitude):
  * cell indices: bit-exact against nxsearch/nysearch on the FP64 positions;
  * node fields: 1e-6, viscosity-derived fields 1e-5 (see parity.VISCOUS);
  * marker fields: 1e-6; positions after the move: 3e-7 cell widths
    (the FP32 offset resolves 2^-24 = 6e-8 of a cell).
"""
import numpy as np
import pytest

import oracle
from velo2cycles_gb300 import abi, mic, synth

from .parity import (B2C_C2B_OUT, C2B_OUT, COPY_OUT, M2N_OUT, RECOMPUTE_OUT, rel_err,
                     temperature_case, MOVE_MARK, N2M_MARK, N2M_OUT, RSF_OUT, VISCOUS,
                     node_errors, marker_errors, nxsearch_np)

pytestmark = pytest.mark.gpu

TOL = 1e-6
TOL_VISC = 1e-5


def _tol(name):
    f = {v: k for k, v in abi.node_field_names().items()}.get(name)
    return TOL_VISC if f in VISCOUS else TOL


def _check_nodes(errs):
    bad = {k: v for k, v in errs.items() if not v <= _tol(k)}
    assert not bad, f"node fields over tolerance: {bad}"


@pytest.fixture(scope="module", params=["tiny", "small", "dense", "mode1"])
def case(request, built_lib, oracle_built):
    if request.param == "mode1":
        # interpolationmod 1: the 13-node stencil (per-node gather kernels)
        return synth.make_case("small", seed=7, interpolationmod=1)
    if request.param == "dense":
        # 48 markers per cell: a column strip of a tile holds about 1000
        # markers, so the tile kernels stage it in several chunks
        return synth.make_case("small", seed=7, n_markers=3 * 50 * 20 * 16)
    return synth.make_case(request.param, seed=7)


def test_cell_assignment_bit_exact(case):
    m = mic.from_case(case)
    cells = m.download_cells()
    ix = nxsearch_np(case.gx, case.marks[abi.MF_X])
    iy = nxsearch_np(case.gy, case.marks[abi.MF_Y])
    assert np.array_equal(cells, (ix * (case.gy.size - 1) + iy).astype(np.int32))
    m.close()


def test_marker2nodes(case):
    m = mic.from_case(case)
    m.marker2nodes()
    got = m.download_nodes(M2N_OUT)
    ref = oracle.Restatement(case.copy())
    ref.marker2nodes()
    _check_nodes(node_errors(got, ref.nodes, M2N_OUT))
    st = m.status()
    assert st["n_nan"] == 0
    m.close()


def test_center2basic_and_node_rsf(case):
    m = mic.from_case(case)
    ref = oracle.Restatement(case.copy())
    m.marker2nodes(); ref.marker2nodes()
    m.interpolate_center2basic_old(); ref.center2basic_old()
    dt = case.params["timestep"]
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    d_gpu = m.compute_after_solve(dt, 0)
    d_ref = ref.compute_after_solve(dt, 0)
    got = m.download_nodes(C2B_OUT + RSF_OUT)
    _check_nodes(node_errors(got, ref.nodes, C2B_OUT + RSF_OUT))
    assert abs(d_gpu - d_ref) <= 1e-5 * max(abs(d_ref), 1.0)
    m.close()


def test_basic2center_center2basic(case):
    """The Picard loop's node interpolations after marker2nodes and
    compute_before_solve, on the GPU's own node fields."""
    dt = case.params["timestep"]
    m = mic.from_case(case)
    ref = oracle.Restatement(case.copy())
    m.marker2nodes(); ref.marker2nodes()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.interpolate_basic2center(); ref.basic2center()
    m.interpolate_center2basic(dt); ref.center2basic(dt)
    _check_nodes(node_errors(m.download_nodes(B2C_C2B_OUT), ref.nodes, B2C_C2B_OUT))
    m.close()


def test_picard_pass_node_routines(case):
    """One Picard pass of node routines in the reference's order with the
    stress recompute from the given velocities and the final-rate copy."""
    dt = case.params["timestep"]
    m = mic.from_case(case)
    ref = oracle.Restatement(case.copy())
    m.marker2nodes(); ref.marker2nodes()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.interpolate_basic2center(); ref.basic2center()
    m.recompute_stress_strainrate(dt); ref.recompute_stress(dt)
    _check_nodes(node_errors(m.download_nodes(RECOMPUTE_OUT), ref.nodes, RECOMPUTE_OUT))
    m.interpolate_center2basic(dt); ref.center2basic(dt)
    m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
    m.copyarrays(); ref.copyarrays()
    _check_nodes(node_errors(m.download_nodes(COPY_OUT + RSF_OUT), ref.nodes, COPY_OUT + RSF_OUT))
    m.close()


@pytest.mark.parametrize("heatdif", [1.0, 0.0])
def test_marker_temperature(heatdif, built_lib, oracle_built):
    """The marker part of solve_temperature: fluid markers, newly arrived
    markers, subgrid diffusion and the per-cell antidiffusion."""
    c, told, tnew = temperature_case(15)
    c.nodes[abi.NF_TK], c.nodes[abi.NF_TK2] = tnew, told
    m = mic.from_case(c)
    ref = oracle.Restatement(c.copy())
    m.marker_temperature(heatdif)
    ref.marker_temperature(heatdif)
    got = m.download_markers([abi.MF_K])[abi.MF_K]
    assert not np.array_equal(ref.marks[abi.MF_K], c.marks[abi.MF_K])
    assert rel_err(got, ref.marks[abi.MF_K]) <= TOL
    m.close()


def test_nodes2markers(case):
    m = mic.from_case(case)
    ref = oracle.Restatement(case.copy())
    m.nodes2markers()
    ref.nodes2markers()
    got = m.download_nodes(N2M_OUT)
    _check_nodes(node_errors(got, ref.nodes, N2M_OUT))
    mk = m.download_markers(N2M_MARK)
    errs = marker_errors(mk, ref.marks, N2M_MARK)
    bad = {k: v for k, v in errs.items() if not v <= TOL}
    assert not bad, f"marker fields over tolerance: {bad}"
    m.close()


@pytest.mark.parametrize("markmod", [1, 2])
def test_move(case, markmod):
    c = case.copy()
    c.params["markmod"] = markmod
    m = mic.from_case(c)
    ref = oracle.Restatement(c.copy())
    m.moveandrotatemarkers()
    ref.move()
    mk = m.download_markers(MOVE_MARK)
    # a few units of the FP32 offset resolution, 2^-24 cell widths
    wx = np.diff(c.gx)[nxsearch_np(c.gx, ref.marks[abi.MF_X])]
    wy = np.diff(c.gy)[nxsearch_np(c.gy, ref.marks[abi.MF_Y])]
    ex = np.abs(mk[abi.MF_X] - ref.marks[abi.MF_X]) / wx
    ey = np.abs(mk[abi.MF_Y] - ref.marks[abi.MF_Y]) / wy
    assert ex.max() <= 3e-7 and ey.max() <= 3e-7, (ex.max(), ey.max())
    errs = marker_errors(mk, ref.marks, [abi.MF_XX, abi.MF_XY, abi.MF_K, abi.MF_E])
    bad = {k: v for k, v in errs.items() if not v <= TOL}
    assert not bad, bad
    # the cell of every moved marker is nxsearch of its FP64 position
    cells = m.download_cells()
    ix = nxsearch_np(c.gx, mk[abi.MF_X])
    iy = nxsearch_np(c.gy, mk[abi.MF_Y])
    assert np.array_equal(cells, (ix * (c.gy.size - 1) + iy).astype(np.int32))
    m.close()


def test_full_step_deterministic(case):
    outs = []
    for _ in range(2):
        m = mic.from_case(case)
        m.step()
        m.step()
        outs.append((m.download_nodes([abi.NF_NU_M2C, abi.NF_PHIE, abi.NF_MVX]),
                     m.download_markers([abi.MF_X, abi.MF_XX])))
        m.close()
    for f in outs[0][0]:
        assert np.array_equal(outs[0][0][f], outs[1][0][f])
    for f in (abi.MF_X, abi.MF_XX):
        assert np.array_equal(outs[0][1][f], outs[1][1][f])


VARIANTS = [dict(stoksmod=2, markmod=2), dict(antidiffinter=0), dict(Dphis=1.0),
            dict(densimod=1, timesum=1e9), dict(pmode=1, timesum=1e8), dict(timesum=0.0),
            dict(tempmod=0), dict(power_law_RSF=1), dict(RSFmode=0), dict(markmod=0)]


@pytest.mark.parametrize("variant", VARIANTS, ids=lambda v: ",".join(f"{k}={x}" for k, x in v.items()))
def test_flag_variants_full_step(variant, built_lib, oracle_built):
    """The whole step under the reference's other flag settings."""
    c = synth.make_case("small", seed=13, **variant)
    m = mic.from_case(c)
    ref = oracle.Restatement(c.copy())
    dt = c.params["timestep"]
    m.marker2nodes(); ref.marker2nodes()
    _check_nodes(node_errors(m.download_nodes(M2N_OUT), ref.nodes, M2N_OUT))
    m.interpolate_center2basic_old(); ref.center2basic_old()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
    _check_nodes(node_errors(m.download_nodes(C2B_OUT + RSF_OUT), ref.nodes, C2B_OUT + RSF_OUT))
    m.nodes2markers(); ref.nodes2markers()
    _check_nodes(node_errors(m.download_nodes(N2M_OUT), ref.nodes, N2M_OUT))
    m.moveandrotatemarkers(); ref.move()
    mk = m.download_markers(N2M_MARK + MOVE_MARK)
    fields = [f for f in N2M_MARK if f not in (abi.MF_X, abi.MF_Y)]
    errs = marker_errors(mk, ref.marks, fields)
    bad = {k: v for k, v in errs.items() if not v <= TOL}
    assert not bad, bad
    wx = np.diff(c.gx)[nxsearch_np(c.gx, ref.marks[abi.MF_X])]
    assert (np.abs(mk[abi.MF_X] - ref.marks[abi.MF_X]) / wx).max() <= 3e-7
    m.close()


def test_interpolation_mode_checked(built_lib):
    from velo2cycles_gb300._lib import V2CError
    c = synth.make_case("tiny", seed=1, interpolationmod=3)
    with pytest.raises(V2CError) as e:
        mic.from_case(c)
    assert e.value.code == abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("oldornew", [0, 1])
@pytest.mark.parametrize("variant", [{}, dict(pmode=1), dict(RSFmode=0)])
def test_calc_timestep(oldornew, variant, built_lib, oracle_built):
    """calc_timestep on the device node fields against the oracle: the time
    step and its limits to 1e-5 (FP32 node fields), counts exactly."""
    c = synth.make_case("small", seed=21, **variant)
    ctl = dict(maxtmstep=3e9, tcd=2e-3)
    m = mic.from_case(c)
    got = m.calc_timestep(oldornew, **ctl)
    m.close()
    rc, ref = oracle.Restatement(c.copy()).calc_timestep(oldornew, **ctl)
    assert rc == 0
    for k in ("nr_0", "nr_1"):
        assert got[k] == ref[k], k
    for k in ("dt_f", "maxvel", "maxVx", "dtnvp", "dtd", "dtphi", "dtL", "max_sigin_0",
              "min_sigin_0", "max_sigin_1", "min_sigin_1", "max_visc_0", "min_visc_0",
              "max_visc_1", "min_visc_1", "sum_sigin_0", "sum_sigin_1", "sum_visc_0",
              "sum_visc_1", "sum2_sigin_0", "sum2_visc_1"):
        assert abs(got[k] - ref[k]) <= 1e-5 * max(abs(ref[k]), 1e-30), (k, got[k], ref[k])
