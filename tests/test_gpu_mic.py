"""Parity of the CUDA MIC step with the oracle restatement (GPU).

The GPU runs on the seeded state; the oracle runs in FP64 on the same state
as the device holds it after upload (parity.device_view: FP32 marker and
node fields, the temperature as a float pair, positions as cell + FP32
offset), so the comparison measures the device's arithmetic.  Tolerances,
per entry (parity.rel_err: relative; for fields that cross zero with the
field's RMS as a floor; slip rates through the relative error of ln V):
  * cell indices: bit-exact against nxsearch/nysearch on the FP64 positions;
  * node and marker fields: 1e-6 (marker fields that nodes2markers
    interpolates, against the magnitude of the node values they come from:
    parity.n2m_floors);
  * positions after the move: 3e-7 cell widths (the FP32 offset resolves
    2^-24 = 6e-8 of a cell).
What FP32 storage adds on top (oracle against oracle) is bounded in
test_storage_error.py.
"""
import numpy as np
import pytest

from velo2cycles_gb300 import abi, mic, synth

from .parity import (B2C_C2B_OUT, C2B_OUT, COPY_OUT, M2N_OUT, RECOMPUTE_OUT, immobile_case,
                     marker_err, n2m_floors, rotated_floors,
                     temperature_case, MOVE_MARK, N2M_MARK, N2M_OUT, RSF_OUT, device_view,
                     node_errors, marker_errors, nxsearch_np, oracle_for, over)

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _check_nodes(errs):
    bad = over(errs, TOL)
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
    ref = oracle_for(case)
    ref.marker2nodes()
    _check_nodes(node_errors(got, ref.nodes, M2N_OUT))
    st = m.status()
    assert st["n_nan"] == 0
    m.close()


def test_marker_properties(case):
    """Per-marker viscosity and conductivity of marker2nodes
    (recalc_marker_properties.c) against the oracle's, entry by entry: the
    viscosities span 1e17-1e26 Pa s, and the node averages that carry them
    would hide a marker far below its node's largest."""
    m = mic.from_case(case)
    m.marker2nodes()
    nu, kt = m.download_marker_properties()
    m.close()
    nu_r, kt_r, _ = oracle_for(case).marker_properties()
    inside = nu_r > 0
    assert np.array_equal(nu > 0, inside)
    assert np.abs(nu[inside] / nu_r[inside] - 1).max() <= TOL
    assert np.abs(kt[inside] / kt_r[inside] - 1).max() <= TOL


def test_center2basic_and_node_rsf(case):
    m = mic.from_case(case)
    ref = oracle_for(case)
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
    ref = oracle_for(case)
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
    ref = oracle_for(case)
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


@pytest.mark.parametrize("n_imm,n_out", [(40, 25), (10, 30), (30, 0)])
def test_immobile_markers(n_imm, n_out, built_lib, oracle_built):
    """Immobile markers (type >= 100, anchored at markk/markv): the move
    appends the markers they spawn in reference order, sends them back to
    their anchors and refills out-of-model slots from the last appended
    marker back (moveandrotatemarkers.c:88-171; the oracle is pinned against
    the reference in test_oracle_pin.py::test_immobile_markers_bit_exact_vs_
    reference).  Then marker2nodes runs over the new marker set."""
    c = immobile_case(5, n_imm=n_imm, n_out=n_out)
    m = mic.from_case(c, max_markers=2 * c.n)
    ref = oracle_for(c, cap=2 * c.n)
    m.moveandrotatemarkers()
    assert ref.move() == 0
    assert m.n == ref.n == c.n + max(0, n_imm - n_out)
    fields = [abi.MF_X, abi.MF_Y, abi.MF_K, abi.MF_V, abi.MF_E, abi.MF_XX, abi.MF_XY, abi.MF_P,
              abi.MF_EXX, abi.MF_EXY, abi.MF_D]
    mk = m.download_markers(fields)
    assert np.array_equal(mk["markt"], ref.markt)
    for k, g in ((abi.MF_X, c.gx), (abi.MF_Y, c.gy)):
        w = np.diff(g)[nxsearch_np(g, ref.marks[k])]
        assert (np.abs(mk[k] - ref.marks[k]) / w).max() <= 3e-7, k
    errs = marker_errors(mk, ref.marks, [abi.MF_K, abi.MF_V, abi.MF_E, abi.MF_XX, abi.MF_XY,
                                         abi.MF_P, abi.MF_EXX, abi.MF_EXY])
    bad = over(errs, TOL)
    assert not bad, bad
    assert np.array_equal(mk[abi.MF_D] == -1.0, ref.marks[abi.MF_D] == -1.0)
    cells = m.download_cells()
    ix, iy = nxsearch_np(c.gx, mk[abi.MF_X]), nxsearch_np(c.gy, mk[abi.MF_Y])
    assert np.array_equal(cells, (ix * (c.gy.size - 1) + iy).astype(np.int32))
    # the next step's scatter over the grown marker set.  The immobile
    # markers' markk is their x anchor (~1e5), which marker2nodes sums as a
    # temperature (interpolation.c:229) beside temperatures of ~1e3: its FP32
    # terms carry ~1e-7 of 1e5, so the node temperature is held to 1e-5
    m.marker2nodes(); ref.marker2nodes()
    errs = node_errors(m.download_nodes(M2N_OUT), ref.nodes, M2N_OUT)
    bad = over({k: v for k, v in errs.items() if k != "tk"}, TOL)
    assert errs["tk"] <= 1e-5, errs["tk"]
    assert not bad, bad
    m.close()


@pytest.mark.parametrize("rkmod", [0, 1, 2, 3])
@pytest.mark.parametrize("variant", [{}, dict(RSFmode=0), dict(timesum=0.0)],
                         ids=["rsf", "RSFmode=0", "timesum=0"])
def test_picard_passes(rkmod, variant, built_lib, oracle_built):
    """Passes rk = 0..3 of compute_before_solve + compute_after_solve under
    each rkmod, each pass feeding the next its solved rates (the oracle's
    sequence is pinned bit-exact against the reference in
    test_oracle_pin.py::test_picard_passes_bit_exact_vs_reference)."""
    from .test_oracle_pin import picard_case
    c = picard_case("small", 31, rkmod, **variant)
    dt = c.params["timestep"]
    m = mic.from_case(c)
    ref = oracle_for(c)
    m.marker2nodes(); ref.marker2nodes()
    for rk in range(4):
        m.compute_before_solve(dt, rk); ref.compute_before_solve(dt, rk)
        _check_nodes(node_errors(m.download_nodes(RSF_OUT), ref.nodes, RSF_OUT))
        d_gpu = m.compute_after_solve(dt, rk)
        d_ref = ref.compute_after_solve(dt, rk)
        _check_nodes(node_errors(m.download_nodes(RSF_OUT), ref.nodes, RSF_OUT))
        assert abs(d_gpu - d_ref) <= 1e-5 * max(abs(d_ref), 1.0), (rk, d_gpu, d_ref)
    m.close()


@pytest.mark.parametrize("heatdif", [1.0, 0.0])
def test_marker_temperature(heatdif, built_lib, oracle_built):
    """The marker part of solve_temperature: fluid markers, newly arrived
    markers, subgrid diffusion and the per-cell antidiffusion."""
    c, told, tnew = temperature_case(15)
    c.nodes[abi.NF_TK], c.nodes[abi.NF_TK2] = tnew, told
    m = mic.from_case(c)
    ref = oracle_for(c)
    m.marker_temperature(heatdif)
    ref.marker_temperature(heatdif)
    got = m.download_markers([abi.MF_K])[abi.MF_K]
    assert not np.array_equal(ref.marks[abi.MF_K], c.marks[abi.MF_K])
    # the update runs in FP64 on the float-pair temperature, from the FP64
    # copies of the uploaded node temperatures (the subgrid diffusion change
    # itself in FP32: a few 1e-8 of the temperature)
    assert marker_err(abi.MF_K, got, ref.marks[abi.MF_K]) <= 1e-7
    m.close()


def test_nodes2markers(case):
    m = mic.from_case(case)
    ref = oracle_for(case)
    fl = n2m_floors(ref)
    m.nodes2markers()
    ref.nodes2markers()
    got = m.download_nodes(N2M_OUT)
    _check_nodes(node_errors(got, ref.nodes, N2M_OUT))
    mk = m.download_markers(N2M_MARK)
    errs = marker_errors(mk, ref.marks, N2M_MARK, fl)
    bad = over(errs, TOL)
    assert not bad, f"marker fields over tolerance: {bad}"
    m.close()


@pytest.mark.parametrize("markmod", [1, 2])
def test_move(case, markmod):
    c = case.copy()
    c.params["markmod"] = markmod
    m = mic.from_case(c)
    ref = oracle_for(c)
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
    bad = over(errs, TOL)
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
    ref = oracle_for(c)
    dt = c.params["timestep"]
    m.marker2nodes(); ref.marker2nodes()
    _check_nodes(node_errors(m.download_nodes(M2N_OUT), ref.nodes, M2N_OUT))
    m.interpolate_center2basic_old(); ref.center2basic_old()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
    _check_nodes(node_errors(m.download_nodes(C2B_OUT + RSF_OUT), ref.nodes, C2B_OUT + RSF_OUT))
    fl = n2m_floors(ref)
    m.nodes2markers(); ref.nodes2markers()
    _check_nodes(node_errors(m.download_nodes(N2M_OUT), ref.nodes, N2M_OUT))
    m.moveandrotatemarkers(); ref.move()
    mk = m.download_markers(N2M_MARK + MOVE_MARK)
    fields = [f for f in N2M_MARK if f not in (abi.MF_X, abi.MF_Y)]
    errs = marker_errors(mk, ref.marks, fields, rotated_floors(fl))
    bad = over(errs, TOL)
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
    rc, ref = oracle_for(c).calc_timestep(oldornew, **ctl)
    assert rc == 0
    for k in ("nr_0", "nr_1"):
        assert got[k] == ref[k], k
    for k in ("dt_f", "maxvel", "maxVx", "dtnvp", "dtd", "dtphi", "dtL", "max_sigin_0",
              "min_sigin_0", "max_sigin_1", "min_sigin_1", "max_visc_0", "min_visc_0",
              "max_visc_1", "min_visc_1", "sum_sigin_0", "sum_sigin_1", "sum_visc_0",
              "sum_visc_1", "sum2_sigin_0", "sum2_visc_1"):
        assert abs(got[k] - ref[k]) <= 1e-5 * max(abs(ref[k]), 1e-30), (k, got[k], ref[k])
