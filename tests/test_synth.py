"""Seeded generators (CPU)."""
import numpy as np

from velo2cycles_gb300 import abi, newton, synth


def test_deterministic_and_shaped():
    a = synth.make_case("tiny", seed=3)
    b = synth.make_case("tiny", seed=3)
    assert np.array_equal(a.marks[abi.MF_X], b.marks[abi.MF_X])
    assert a.n == (a.gx.size - 1) * (a.gy.size - 1) * 16
    assert all(v.shape == (a.nodenum,) for v in a.nodes.values())
    assert (np.diff(a.gx) > 0).all() and a.gx[-1] == a.params["xsize"]


def test_markers_inside_their_subcells():
    c = synth.make_case("small", seed=1)
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    assert (x >= 0).all() and (x <= c.gx[-1]).all() and (y >= 0).all() and (y <= c.gy[-1]).all()
    counts = np.bincount(np.searchsorted(c.gx, x, "right") - 1)
    assert counts.min() == counts.max() == 4 * (c.gy.size - 1) * 4


def test_refined_grid_and_window():
    gx, gy, _, _ = synth.grid_for("c2")
    assert gx.size == 1001 and gy.size == 401
    assert abs(np.diff(gx).min() - 100.0) < 1e-6 and abs(np.diff(gy).min() - 100.0) < 1e-6
    w = synth.make_case("c4", seed=1, window=(1200, 0, 21, 11))
    assert w.gx[0] == 0 and np.allclose(np.diff(w.gx), 500.0)


def test_power_law_rocks_present():
    c = synth.make_case("small", seed=2)
    kinds = set(np.unique(c.markt))
    assert {3, 4, 5} & kinds and c.rt[abi.RT_MM, 3] != 1.0


def test_rsf_states_distributions():
    S = newton.rsf_states(20000, seed=1)
    amb = S[abi.RS_A] - S[abi.RS_B]
    assert amb.min() >= -0.01 and amb.max() <= 0.015 and np.all(S[abi.RS_B] == 0.015)
    assert 1e-15 <= S[abi.RS_VOLD].min() and S[abi.RS_VOLD].max() <= 10
    assert 5e6 <= S[abi.RS_SN].min() and S[abi.RS_SN].max() <= 100e6
    assert 1e-3 <= S[abi.RS_DT].min() and S[abi.RS_DT].max() <= 1e10
