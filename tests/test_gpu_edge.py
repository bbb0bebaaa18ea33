"""Edge cases of the MIC step on the GPU (against the oracle where there is
something to compare): no markers, markers only outside the model, empty
cells among full ones, one crowded cell, capacity and argument errors, and
a multi-step run whose drift against the FP64 oracle stays bounded.
"""
import numpy as np
import pytest

import oracle
from velo2cycles_gb300 import abi, mic, synth
from velo2cycles_gb300._lib import V2CError

from .parity import M2N_OUT, N2M_OUT, node_errors, marker_errors, nxsearch_np, oracle_for, over

pytestmark = pytest.mark.gpu


def _subset(c, keep):
    """Copy of case c holding only the markers selected by keep."""
    c = c.copy()
    for k in range(abi.MF_N):
        c.marks[k] = c.marks[k][keep].copy()
    c.markt = c.markt[keep].copy()
    return c


def _check(m, ref, fields):
    errs = node_errors(m.download_nodes(fields), ref.nodes, fields)
    bad = over(errs, 1e-6)
    assert not bad, bad


def test_no_markers(built_lib, oracle_built):
    """No markers: the nodes keep what marker2nodes gives an empty model,
    and the zero viscosities make compute_before_solve flag its error on
    both sides (plastic.c:2-56 checks nu <= 0 at every interior node)."""
    c = _subset(synth.make_case("tiny", seed=1), np.zeros(0, dtype=np.int64))
    m = mic.from_case(c, max_markers=16)
    ref = oracle_for(c)
    dt = c.params["timestep"]
    m.marker2nodes(); ref.marker2nodes()
    _check(m, ref, M2N_OUT)
    m.interpolate_center2basic_old(); ref.center2basic_old()
    m.compute_before_solve(dt, 0)
    rc = ref.compute_before_solve(dt, 0)
    st = m.status()
    assert st["n_markers"] == 0
    assert rc == abi.ERR_NAN and st["n_nan"] > 0
    m.nodes2markers(); m.moveandrotatemarkers()
    assert m.status()["n_markers"] == 0
    m.close()


def test_empty_cells_and_crowded_cell(built_lib, oracle_built):
    c = synth.make_case("small", seed=2)
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    # empty a band of cells, crowd one cell with 400 markers
    keep = ~((x > c.gx[10]) & (x < c.gx[14]))
    c = _subset(c, keep)
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    x[:400] = 0.5 * (c.gx[20] + c.gx[21]) + np.linspace(-1, 1, 400)
    y[:400] = 0.5 * (c.gy[8] + c.gy[9])
    m = mic.from_case(c)
    ref = oracle_for(c)
    m.marker2nodes(); ref.marker2nodes()
    _check(m, ref, M2N_OUT)
    m.nodes2markers(); ref.nodes2markers()
    _check(m, ref, N2M_OUT)
    assert m.status()["max_cell_count"] >= 400
    m.close()


def test_all_markers_outside(built_lib, oracle_built):
    c = synth.make_case("tiny", seed=3)
    c.marks[abi.MF_X][:] = -10.0
    m = mic.from_case(c)
    ref = oracle_for(c)
    m.marker2nodes(); ref.marker2nodes()
    _check(m, ref, M2N_OUT)
    m.close()


def test_capacity_and_argument_errors(built_lib):
    c = synth.make_case("tiny", seed=4)
    m = mic.MarkerInCell(c.params, 10)
    m.set_grid(c.gx, c.gy)
    m.set_rock_table(c.rt)
    with pytest.raises(V2CError) as e:
        m.upload_markers(c.marks, c.markt)
    assert e.value.code == abi.ERR_CAPACITY
    with pytest.raises(V2CError) as e:
        m.marker2nodes()  # no markers uploaded yet
    assert e.value.code == abi.ERR_STATE
    bad = dict(c.params, newton_precision=7)
    with pytest.raises(V2CError) as e:
        m.set_params(**bad)
    assert e.value.code == abi.ERR_ARG
    m.close()


def test_multi_step_drift(built_lib, oracle_built):
    """Six full steps with a changing dt on both sides: the GPU state stays
    within ten times the one-step tolerance of the FP64 oracle."""
    c = synth.make_case("small", seed=5)
    m = mic.from_case(c)
    ref = oracle_for(c)
    dts = 10.0 ** np.random.default_rng(0).uniform(6, 9, 6)
    for dt in dts:
        m.set_params(timestep=float(dt))
        ref.set_params(timestep=float(dt))
        m.marker2nodes(); ref.marker2nodes()
        m.interpolate_center2basic_old(); ref.center2basic_old()
        m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
        m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
        m.nodes2markers(); ref.nodes2markers()
        m.moveandrotatemarkers(); ref.move()
    mk = m.download_markers([abi.MF_X, abi.MF_Y, abi.MF_XX, abi.MF_XY, abi.MF_P, abi.MF_E])
    wx = np.diff(c.gx)[nxsearch_np(c.gx, ref.marks[abi.MF_X])]
    assert (np.abs(mk[abi.MF_X] - ref.marks[abi.MF_X]) / wx).max() <= 3e-6
    wy = np.diff(c.gy)[nxsearch_np(c.gy, ref.marks[abi.MF_Y])]
    assert (np.abs(mk[abi.MF_Y] - ref.marks[abi.MF_Y]) / wy).max() <= 3e-6
    errs = marker_errors(mk, ref.marks, [abi.MF_XX, abi.MF_XY, abi.MF_P, abi.MF_E])
    assert all(v <= 1e-5 for v in errs.values()), errs
    m.close()


def test_batched_node_fields(built_lib):
    """v2c_upload_node_fields / v2c_download_node_fields give the same
    arrays as the one-field calls, in any field order, and reject bad ids."""
    c = synth.make_case("tiny", seed=6)
    m = mic.from_case(c)
    fields = [abi.NF_VY, abi.NF_SXX, abi.NF_VX, abi.NF_PRS]
    rng = np.random.default_rng(1)
    vals = {f: rng.normal(size=c.nodenum) * 10.0 ** rng.integers(-9, 9) for f in fields}
    m.upload_nodes(vals)
    got = m.download_nodes(fields)
    for f in fields:
        one = m.download_node(f)
        assert np.array_equal(got[f], one)
        assert np.array_equal(one, vals[f].astype(np.float32).astype(np.float64))
    # more fields than before grows the staging area
    allf = m.download_nodes()
    assert len(allf) == abi.NF_N and np.array_equal(allf[abi.NF_VX], got[abi.NF_VX])
    with pytest.raises(V2CError) as e:
        m.download_nodes([abi.NF_N])
    assert e.value.code == abi.ERR_ARG
    m.close()


def test_async_node_download(built_lib):
    """v2c_download_node_fields_async: a snapshot of the fields as the calls
    before it leave them, copied while the node kernels after it run (they
    write other fields), equal to the synchronous download; a second
    asynchronous download reuses the staging area after the first."""
    c = synth.make_case("small", seed=8)
    m = mic.from_case(c)
    dt = c.params["timestep"]
    m.marker2nodes()
    fields = [abi.NF_NU_M2C, abi.NF_ND_M2C, abi.NF_GG, abi.NF_SXXE, abi.NF_SPPE, abi.NF_TK]
    want = m.download_nodes(fields)
    got = {f: np.full(c.nodenum, np.nan) for f in fields}
    m.download_nodes_async(got)
    m.interpolate_center2basic_old()
    m.compute_before_solve(dt, 0)
    # a second download of fields the node kernels just wrote
    f2 = [abi.NF_NU, abi.NF_SYIELDS]
    got2 = {f: np.full(c.nodenum, np.nan) for f in f2}
    m.download_nodes_async(got2)
    m.compute_after_solve(dt, 0)
    m.wait_downloads()
    for f in fields:
        assert np.array_equal(got[f], want[f]), f
    want2 = m.download_nodes(f2)
    for f in f2:
        assert np.array_equal(got2[f], want2[f]), f
    m.close()


def test_pinned_node_transfers(built_lib):
    """Node fields to and from pinned host buffers (direct asynchronous
    copies, as the end-to-end bench uses) equal the same transfers through
    pageable buffers (staged by the driver): upload, synchronous and
    asynchronous download, with an odd node count and a single field."""
    torch = pytest.importorskip("torch")
    c = synth.make_case("small", seed=9)
    m = mic.from_case(c)
    m.marker2nodes()

    def pinned(a=None):
        t = torch.empty(c.nodenum, dtype=torch.float64, pin_memory=True)
        if a is not None:
            t.copy_(torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)))
        return t.numpy()

    fields = [abi.NF_NU_M2C, abi.NF_GG, abi.NF_SXXE, abi.NF_MVX, abi.NF_TK]
    want = m.download_nodes(fields)  # pageable
    got = {f: pinned() for f in fields}
    m.download_nodes(fields, into=got)
    for f in fields:
        assert np.array_equal(got[f], want[f]), f
    one = {abi.NF_RO: pinned()}
    m.download_nodes([abi.NF_RO], into=one)
    assert np.array_equal(one[abi.NF_RO], m.download_nodes([abi.NF_RO])[abi.NF_RO])
    got_a = {f: pinned() for f in fields}
    got_a[fields[0]][:] = np.nan
    m.download_nodes_async(got_a)
    m.interpolate_center2basic_old()
    m.wait_downloads()
    for f in fields:
        assert np.array_equal(got_a[f], want[f]), f
    # upload from pinned buffers, then read back through the pageable path
    rng = np.random.default_rng(3)
    up = {abi.NF_VX: rng.normal(size=c.nodenum), abi.NF_PR: rng.normal(size=c.nodenum) * 1e8,
          abi.NF_SXY: rng.normal(size=c.nodenum) * 1e6}
    m.upload_nodes(up)
    m.synchronize()
    ref = m.download_nodes(list(up))
    m.upload_nodes({f: np.zeros(c.nodenum) for f in up})
    m.upload_nodes({f: pinned(v) for f, v in up.items()})
    m.synchronize()
    back = m.download_nodes(list(up))
    for f in up:
        assert np.array_equal(back[f], ref[f]), f
    m.close()
