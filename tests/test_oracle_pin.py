"""Pinning the oracle restatement to the reference (CPU).

The reference has no tests or stored answers, so the restatement
(oracle/v2c_oracle.c) is pinned against the reference's own routines:
  * compiled from its sources here (oracle/build_ref.sh -> oracle/_ref),
    on seeded states and flag variants, all six stages of the MIC step,
    bit-exact in FP64 (both built with -ffp-contract=off);
  * the committed fixtures tests/golden/ref_micro.npz (reference outputs
    made by tests/golden/make_golden.py), also bit-exact, which works where
    the reference sources are absent.
"""
import json
import os

import numpy as np
import pytest

import oracle
from oracle import bindings as B
from velo2cycles_gb300 import abi, synth

from .parity import immobile_case, stokes_case, temperature_case

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_micro.npz")


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build()


def _compare(r, nodes_ref, marks_ref):
    bad = [abi.node_field_names()[k] for k in range(abi.NF_N)
           if not np.array_equal(r.nodes[k], nodes_ref[k], equal_nan=True)]
    bad += ["marker " + abi.marker_field_names()[k] for k in range(abi.MF_N)
            if k != abi.MF_SLIPV and not np.array_equal(r.marks[k], marks_ref[k], equal_nan=True)]
    return bad


@pytest.mark.parametrize("name", ["default", "variant"])
def test_restatement_matches_golden(name):
    z = np.load(GOLDEN)
    p = synth.default_params()
    p.update(json.loads(str(z[f"{name}/params"])))
    nodes = {k: z[f"{name}/nodes_in"][k].copy() for k in range(abi.NF_N)}
    marks = {k: z[f"{name}/marks_in"][k].copy() for k in range(abi.MF_N)}
    c = synth.Case(name, p, z[f"{name}/gx"], z[f"{name}/gy"], z[f"{name}/rt"], nodes, marks,
                   z[f"{name}/markt"].copy(), z[f"{name}/bondm"], z[f"{name}/bondn"],
                   z[f"{name}/bondv"])
    r = oracle.Restatement(c, phantom=True)
    assert r.step() == 0
    bad = _compare(r, z[f"{name}/nodes_out"], z[f"{name}/marks_out"])
    assert not bad, bad


# the checkers are (re)built at collection, so that the reference routines
# exist wherever their sources are staged
B.build()
needs_ref = pytest.mark.skipif(not B.reference_available(),
                               reason="reference routines not built")


@needs_ref
@pytest.mark.parametrize("variant", [
    {}, dict(interpolationmod=1), dict(markmod=1), dict(markmod=0, stoksmod=2),
    dict(antidiffinter=0), dict(timesum=0.0), dict(tempmod=0), dict(Dphis=1.0), dict(pmode=1),
    dict(timesum=1e8, timestep=1e8), dict(densimod=1, timesum=1e9), dict(power_law_RSF=1),
    dict(RSFmode=0)])
def test_restatement_bit_exact_vs_reference(variant):
    c = synth.make_case("small", 5, **variant)
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    # markers outside the model, on grid lines and on cell midlines
    x[:5] = -1.0
    x[5:10] = c.gx[-1] + 3.0
    y[10:15] = c.gy[3]
    x[15:20] = c.gx[7]
    x[20:25] = 0.5 * (c.gx[4] + c.gx[5])
    c.markt[30:40] = 1  # sticky-air type
    c.rt[:, 1] = c.rt[:, 2]
    ref = B.run_reference(c, nthreads=1)
    r = oracle.Restatement(c.copy(), phantom=True)
    r.step()
    bad = _compare(r, ref["nodes"], ref["marks"])
    assert not bad, bad


@needs_ref
def test_restatement_bit_exact_nonuniform_grid():
    c = synth.make_case("c2", 2, n_markers=200000)
    ref = B.run_reference(c, nthreads=1)
    r = oracle.Restatement(c.copy(), phantom=True)
    r.step()
    assert not _compare(r, ref["nodes"], ref["marks"])


@needs_ref
@pytest.mark.parametrize("name,seed", [("small", 8), ("c2", 3)])
def test_basic2center_center2basic_bit_exact_vs_reference(name, seed):
    """interpolate_basic2center and interpolate_center2basic
    (interpolation.c:1600-1685) after marker2nodes and compute_before_solve,
    as the Picard loop calls them, on a uniform and the non-uniform C2 grid."""
    kw = dict(n_markers=100000) if name == "c2" else {}
    c = synth.make_case(name, seed, **kw)
    stages = (1 << B.STAGE_M2N) | (1 << B.STAGE_BEFORE) | B.B2C_STAGE | B.C2B_FULL_STAGE
    ref = B.run_reference(c, stages=stages, nthreads=1)
    r = oracle.Restatement(c.copy(), phantom=True)
    dt = c.params["timestep"]
    r.marker2nodes()
    r.compute_before_solve(dt, 0)
    assert r.basic2center() == 0
    assert r.center2basic(dt) == 0
    assert not _compare(r, ref["nodes"], ref["marks"])
    nd = r.nodes[abi.NF_ND]
    assert np.isfinite(nd).sum() > 0.9 * nd.size


@needs_ref
@pytest.mark.parametrize("name,seed", [("small", 9), ("c2", 4)])
def test_picard_node_sequence_bit_exact_vs_reference(name, seed):
    """The node routines of one Picard pass in the reference's order
    (momentum_continuity_iterate.c:69-92) with the Stokes solve replaced by
    the given velocities: compute_before_solve, interpolate_basic2center,
    recompute_stress_strainrate, interpolate_center2basic,
    compute_after_solve, copyarrays."""
    kw = dict(n_markers=100000) if name == "c2" else {}
    c = synth.make_case(name, seed, **kw)
    stages = ((1 << B.STAGE_M2N) | (1 << B.STAGE_BEFORE) | B.B2C_STAGE | B.RECOMPUTE_STAGE |
              B.C2B_FULL_STAGE | (1 << B.STAGE_AFTER) | B.COPY_STAGE)
    ref = B.run_reference(c, stages=stages, nthreads=1)
    r = oracle.Restatement(c.copy(), phantom=True)
    dt = c.params["timestep"]
    r.marker2nodes()
    r.compute_before_solve(dt, 0)
    r.basic2center()
    assert r.recompute_stress(dt) == 0
    r.center2basic(dt)
    r.compute_after_solve(dt, 0)
    assert r.copyarrays() == 0
    assert not _compare(r, ref["nodes"], ref["marks"])
    yn = c.gy.size
    m = np.arange(c.nodenum)
    inner = (m // yn >= 1) & (m % yn >= 1) & (m // yn < c.gx.size - 1) & (m % yn < yn - 1)
    assert np.array_equal(r.nodes[abi.NF_RK_SLIPRS_FINAL][inner],
                          r.nodes[abi.NF_RK_SLIPRS_SOLVED][inner], equal_nan=True)


def picard_case(name, seed, rkmod, **kw):
    """A case whose solved slip and state rates differ from the final ones,
    so that every pass's choice between them shows in the results."""
    c = synth.make_case(name, seed, rkmod=rkmod, **kw)
    rng = np.random.default_rng(seed)
    for f in (abi.NF_RK_SLIPRS_SOLVED, abi.NF_RK_PHIDTS_SOLVED):
        base = c.nodes[abi.NF_RK_SLIPRS_FINAL if f == abi.NF_RK_SLIPRS_SOLVED
                       else abi.NF_RK_PHIDTS_FINAL]
        c.nodes[f] = base * rng.uniform(0.3, 3.0, base.size)
    return c


@needs_ref
@pytest.mark.parametrize("rkmod", [0, 1, 2, 3])
@pytest.mark.parametrize("variant", [{}, dict(RSFmode=0), dict(timesum=0.0)],
                         ids=["rsf", "RSFmode=0", "timesum=0"])
def test_picard_passes_bit_exact_vs_reference(rkmod, variant):
    """Four passes rk = 0..3 of compute_before_solve + compute_after_solve
    under each rkmod (calc_RSF.c:46-86: rk 0 takes the final slip rate,
    later passes the solved one, except rk 3 under rkmod 1 and 2, which
    takes none), each pass feeding the next its solved rates."""
    c = picard_case("small", 31, rkmod, **variant)
    stages = (1 << B.STAGE_M2N) | (1 << B.STAGE_BEFORE) | (1 << B.STAGE_AFTER)
    ref = B.run_reference(c, stages=stages | B.picard_passes(4), nthreads=1)
    r = oracle.Restatement(c.copy(), phantom=True)
    dt = c.params["timestep"]
    r.marker2nodes()
    for rk in range(4):
        r.compute_before_solve(dt, rk)
        d = r.compute_after_solve(dt, rk)
    assert not _compare(r, ref["nodes"], ref["marks"])
    assert d == ref["deltas"]


@needs_ref
@pytest.mark.parametrize("n_imm,n_out", [(40, 25), (10, 30), (30, 0)])
def test_immobile_markers_bit_exact_vs_reference(n_imm, n_out):
    """moveandrotatemarkers with immobile markers: spawned markers appended in
    index order, anchors kept, out-of-model markers refilled from the last
    appended one back, the new marker count.  Against the reference built
    for one thread (v2c_ref_serial; see the next test for the OpenMP build)."""
    c = immobile_case(5, n_imm=n_imm, n_out=n_out)
    ref = B.run_reference(c, stages=1 << B.STAGE_MOVE, nthreads=1, serial=True)
    r = oracle.Restatement(c.copy(), cap=2 * c.n)
    assert r.move() == 0
    assert r.n == ref["n"] == c.n + max(0, n_imm - n_out)
    assert np.array_equal(r.markt, ref["markt"])
    assert not _compare(r, ref["nodes"], ref["marks"])


@needs_ref
def test_openmp_build_appends_from_zero():
    """The reference's OpenMP build appends the spawned markers through the
    reduction variable marknum1 (moveandrotatemarkers.c:5), whose private
    copy starts from 0: the spawned markers overwrite markers 0, 1, ...
    rather than landing after the last one.  The restatement (and the GPU)
    follow the routine as written for one thread."""
    c = immobile_case(5, n_imm=12, n_out=0)
    ref = B.run_reference(c, stages=1 << B.STAGE_MOVE, nthreads=1)
    imm = np.flatnonzero(c.markt >= 100)
    assert ref["n"] == c.n + imm.size
    # the first markers now hold the spawned types, the appended slots
    # nothing the move wrote
    assert np.array_equal(ref["markt"][:imm.size], c.markt[imm] - 100)
    assert np.all(ref["marks"][abi.MF_X][c.n:] == 0)


@needs_ref
def test_multi_step_dt_sequence_bit_exact_vs_reference():
    """Three full steps with a different dt each (the harness's per-step dt
    trailer; timesum advances after each step as in the reference's main
    loop), restatement against the compiled reference."""
    c = synth.make_case("small", 12)
    dts = [1e9, 3e-2, 2e7]
    ref = B.run_reference(c, nthreads=1, nsteps=3, dts=dts)
    r = oracle.Restatement(c.copy(), phantom=True)
    ts = float(c.params["timesum"])
    for dt in dts:
        r.set_params(timestep=dt, timesum=ts)
        r.step()
        ts += dt
    assert not _compare(r, ref["nodes"], ref["marks"])


@needs_ref
@pytest.mark.parametrize("heatdif", [1.0, 0.0])
def test_marker_temperature_bit_exact_vs_reference(heatdif):
    """The marker part of solve_temperature (temperature_iterate.c:181-412):
    the reference's own routine, with its thermal solve stubbed to return
    the given new temperatures, against the restatement."""
    c, told, tnew = temperature_case(14)
    cr = c.copy()
    cr.nodes[abi.NF_TK], cr.nodes[abi.NF_TK2] = told, tnew  # harness convention
    ref = B.run_reference(cr, stages=B.TEMPERATURE_STAGE, heatdif=heatdif)
    co = c.copy()
    co.nodes[abi.NF_TK], co.nodes[abi.NF_TK2] = tnew, told
    r = oracle.Restatement(co, phantom=True)
    assert r.marker_temperature(heatdif) == 0
    assert np.array_equal(ref["nodes"][abi.NF_TK], tnew)
    assert not _compare(r, ref["nodes"], ref["marks"])
    assert not np.array_equal(r.marks[abi.MF_K], c.marks[abi.MF_K])


@needs_ref
@pytest.mark.parametrize("variant", ["default", "no_sailor", "inertia", "compressible",
                                     "cont_bond"])
def test_stokes_assembly_bit_exact_vs_reference(variant):
    """preparematrix + gausmat4_add (momentum_continuity_addmatrix_checkerror.c
    :22-213, gausevps.c:137-214): the reference's own assembly of the CSR
    arrays against the restatement, on node fields from the MIC step."""
    c, ctl = stokes_case(5, variant=variant)
    ref = B.run_reference(c, stages=B.STOKES_STAGE, stokes=ctl)["stokes"]
    rc, ours = oracle.Restatement(c.copy()).stokes_assemble(**ctl)
    assert rc == 0
    for k in ("ia", "ja", "a", "b"):
        assert np.array_equal(ours[k], ref[k], equal_nan=k in ("a", "b")), k
    assert ref["ja"].size > 10 * c.nodenum


def test_stokes_assembly_matches_golden():
    """The reference's preparematrix on the micro case (committed fixture)
    against the restatement, after the same marker2nodes,
    compute_before_solve and basic2center."""
    z = np.load(GOLDEN)
    p = synth.default_params()
    p.update(json.loads(str(z["default/params"])))
    nodes = {k: z["default/nodes_in"][k].copy() for k in range(abi.NF_N)}
    marks = {k: z["default/marks_in"][k].copy() for k in range(abi.MF_N)}
    c = synth.Case("default", p, z["default/gx"], z["default/gy"], z["default/rt"], nodes, marks,
                   z["default/markt"].copy(), z["default/bondm"], z["default/bondn"],
                   z["default/bondv"])
    ctl = json.loads(str(z["stokes/ctl"]))
    r = oracle.Restatement(c)
    r.marker2nodes()
    r.compute_before_solve(ctl["dt"], 0)
    r.basic2center()
    rc, ours = r.stokes_assemble(**ctl)
    assert rc == 0
    for k in ("ia", "ja", "a", "b"):
        assert np.array_equal(ours[k], z[f"stokes/{k}"], equal_nan=k in ("a", "b")), k


def test_stokes_assembly_open_edge_is_refused():
    """A Stokes row on the model's edge would index past the grid in the
    reference; the restatement refuses it."""
    c, ctl = stokes_case(5, variant="open_edge")
    rc, _ = oracle.Restatement(c.copy()).stokes_assemble(**ctl)
    assert rc == abi.ERR_UNSUPPORTED


def test_nxsearch_ties_and_clamps():
    g = np.array([0.0, 1.0, 2.0, 4.0, 8.0])
    assert B.nxsearch(g, 2.0) == 2          # on a line: ties go left of the upper limit
    assert B.nxsearch(g, -5.0) == 0         # below the grid
    assert B.nxsearch(g, 8.0) == 3          # last line clamps to n-2
    assert B.nxsearch(g, 100.0) == 3
    assert B.nxsearch(g, 3.999) == 2


@needs_ref
@pytest.mark.parametrize("oldornew", [0, 1])
@pytest.mark.parametrize("variant", [{}, dict(pmode=1), dict(RSFmode=0)])
def test_calc_timestep_bit_exact_vs_reference(oldornew, variant):
    """calc_timestep (calc_RSF.c:352-572) alone on seeded node fields: every
    output the reference leaves in its globals, bit for bit."""
    c = synth.make_case("small", 6, **variant)
    ctl = dict(maxtmstep=3e9, tcd=2e-3)
    ref = B.run_reference(c, stages=B.TIMESTEP_STAGE, timestep=ctl, oldornew=oldornew)
    assert ref["timestep_rc"] == 0
    rc, info = oracle.Restatement(c.copy()).calc_timestep(oldornew, **ctl)
    assert rc == 0
    bad = {k: (info[k], ref["timestep"][k]) for k in info
           if k != "maxVx" and info[k] != ref["timestep"][k]}
    assert not bad, bad
    assert 0 < info["dt_f"] <= 3e9 or variant.get("pmode") == 1


def test_calc_timestep_resets_and_golden():
    """A node with b <= 0 resets the state and slip-length limits
    (calc_RSF.c:497-501): only nodes after the last reset count."""
    c = synth.make_case("tiny", 2)
    yn = c.gy.size
    bs = c.nodes[abi.NF_BS]
    m_reset = 5 * yn + 5
    bs[m_reset] = 0.0
    r = oracle.Restatement(c.copy())
    rc, info = r.calc_timestep(0, maxtmstep=1e12)
    # recompute the state limit over interior nodes after the reset
    N = c.nodes
    m = np.arange(c.nodenum)
    m2, m1 = m % yn, m // yn
    inter = (m1 >= 1) & (m2 >= 1) & (m1 < c.gx.size - 1) & (m2 < yn - 1)
    after = inter & (m > m_reset) & (N[abi.NF_BS] > 0) & (N[abi.NF_RK_SLIPRS_FINAL] > 0)
    phisc = N[abi.NF_V0S][after] / N[abi.NF_LS][after] * np.exp(-N[abi.NF_PHIS][after])
    assert info["dtphi"] == min(1e12, (0.2 / phisc).min())


@needs_ref
def test_reference_arm_builds_time_only():
    """The timed reference builds (FP contraction allowed; the full-size
    one with the arrays of the whole C4 configuration, where it built):
    a timing-only run returns the per-stage seconds and no arrays, and the
    full-size build computes what the window build computes."""
    c = synth.make_case("small", 4)
    t = B.run_reference(c, stages=B.ALL_STAGES | B.TIMING_ONLY, nthreads=2, nsteps=1, fast=True)
    assert set(t) == {"seconds", "deltas"} and t["seconds"].shape == (8,)
    assert np.all(t["seconds"][:6] >= 0) and t["seconds"][:6].sum() > 0
    if not os.path.exists(B.reference_path(full=True)):
        pytest.skip("no full-size reference build here")
    a = B.run_reference(c, nthreads=2, fast=True)
    b = B.run_reference(c, nthreads=2, fast=True, full=True)
    assert all(np.array_equal(a["nodes"][k], b["nodes"][k], equal_nan=True) for k in a["nodes"])
    assert all(np.array_equal(a["marks"][k], b["marks"][k], equal_nan=True) for k in a["marks"])
