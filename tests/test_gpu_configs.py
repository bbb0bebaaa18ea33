"""Parity at the full sizes of the benchmark configurations (GPU).

One complete MIC step -- marker2nodes, interpolate_center2basic_old,
compute_before_solve, compute_after_solve, nodes2markers and
moveandrotatemarkers -- on
  * C1: uniform 301 x 101 grid over 600 x 200 km, 4 x 4 markers per cell
    (480 000), layered crust and mantle with power-law rocks and a slab;
  * C2: the 1001 x 401 grid refined to 100 m in a 20 km fault zone,
    16 markers per cell (6.4 M), the C2 marker-field distributions;
against the FP64 oracle on the state as the device holds it
(parity.device_view), every node and marker field the stages write,
per entry (parity.rel_err) at 1e-6 -- marker fields against the
magnitude of the node values they are interpolated from (parity.n2m_floors)
-- ; cells bit-exact before and after the
move; positions within 3e-7 cell widths.
"""
import numpy as np
import pytest

from velo2cycles_gb300 import abi, mic, synth

from .parity import (C2B_OUT, M2N_OUT, MOVE_MARK, N2M_MARK, N2M_OUT, RSF_OUT, marker_errors,
                     n2m_floors, node_errors, nxsearch_np, oracle_for, over, rotated_floors)

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module", params=["c1", "c2"])
def config(request, built_lib, oracle_built):
    c = synth.make_case(request.param, seed=7)
    return request.param, c


def _check(got, ref, fields, errors):
    errs = errors(got, ref, fields)
    return over(errs, TOL), max(errs.values())


def test_full_step_per_stage(config):
    name, c = config
    dt = c.params["timestep"]
    m = mic.from_case(c)
    ref = oracle_for(c, nthreads=8)
    cells = m.download_cells()
    ix, iy = nxsearch_np(c.gx, c.marks[abi.MF_X]), nxsearch_np(c.gy, c.marks[abi.MF_Y])
    assert np.array_equal(cells, (ix * (c.gy.size - 1) + iy).astype(np.int32))
    report = {}
    m.marker2nodes(); ref.marker2nodes()
    got = m.download_nodes(M2N_OUT)
    # where the viscosity differs most (printed with -s)
    a, b = got[abi.NF_ND_M2C], ref.nodes[abi.NF_ND_M2C]
    w = int(np.nanargmax(np.abs(a / b - 1)))
    print(name, "worst nd_m2c node", w, divmod(w, c.gy.size), a[w], b[w])
    bad, report["marker2nodes"] = _check(got, ref.nodes, M2N_OUT, node_errors)
    assert not bad, (name, "marker2nodes", bad)
    m.interpolate_center2basic_old(); ref.center2basic_old()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
    f = C2B_OUT + RSF_OUT
    bad, report["node RSF"] = _check(m.download_nodes(f), ref.nodes, f, node_errors)
    assert not bad, (name, "center2basic_old + node RSF", bad)
    # marker fields against the magnitude of the node values they are
    # interpolated from (parity.n2m_floors)
    fl = n2m_floors(ref)
    m.nodes2markers(); ref.nodes2markers()
    bad, report["nodes2markers"] = _check(m.download_nodes(N2M_OUT), ref.nodes, N2M_OUT,
                                          node_errors)
    assert not bad, (name, "nodes2markers nodes", bad)
    bad, report["markers"] = _check(m.download_markers(N2M_MARK), ref.marks, N2M_MARK,
                                    lambda a, b, f: marker_errors(a, b, f, fl))
    assert not bad, (name, "nodes2markers markers", bad)
    m.moveandrotatemarkers(); ref.move()
    mk = m.download_markers(MOVE_MARK)
    fields = [k for k in MOVE_MARK if k not in (abi.MF_X, abi.MF_Y)]
    rfl = rotated_floors(fl)
    bad, report["move"] = _check(mk, ref.marks, fields, lambda a, b, f: marker_errors(a, b, f, rfl))
    assert not bad, (name, "move", bad)
    for k, g in ((abi.MF_X, c.gx), (abi.MF_Y, c.gy)):
        w = np.diff(g)[nxsearch_np(g, ref.marks[k])]
        assert (np.abs(mk[k] - ref.marks[k]) / w).max() <= 3e-7, (name, k)
    cells = m.download_cells()
    ix, iy = nxsearch_np(c.gx, mk[abi.MF_X]), nxsearch_np(c.gy, mk[abi.MF_Y])
    assert np.array_equal(cells, (ix * (c.gy.size - 1) + iy).astype(np.int32))
    print(name, {k: f"{v:.2e}" for k, v in report.items()})
    m.close()
