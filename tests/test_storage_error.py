"""What FP32 storage alone costs, measured by the oracle against itself (CPU).

The device holds marker fields in FP32, the temperature as a float pair,
positions as cell + FP32 offset and node fields in FP32.  The FP64 oracle
run on that rounded state (parity.device_view) against the same oracle on
the original state gives, per output field, the error that storage alone
causes, with no GPU involved.  The GPU parity tests bound the device's own
arithmetic against the rounded state at 1e-6 per entry, so the device's
error against the original FP64 state is at most the sum of the two.

Bounds, per entry (parity.rel_err):
  * 1e-6 for every field but those in STORAGE_LIMITED;
  * 1e-5 for STORAGE_LIMITED: the node viscosity, through the FP32 node
    pressure in the Arrhenius exponent ((E + PV)/RT with PV up to a fifth of
    E, so a 6e-8 rounding of P moves the viscosity by up to ~6e-7 per
    marker), and the state rate V0/L e^-phi - V/L, a difference of two
    terms that carries the slip rate's exponential sensitivity to the node
    stresses.
Measured on these cases: at most 1.3e-6 (nu_m2c).
"""
import numpy as np
import pytest

import oracle
from velo2cycles_gb300 import abi, synth

from .parity import (C2B_OUT, M2N_OUT, MOVE_MARK, N2M_MARK, N2M_OUT, RSF_OUT, marker_err,
                     node_err, oracle_for, tolerance)

STORAGE_LIMITED_NODE = {abi.NF_NU_M2C, abi.NF_RK_PHIDTS_SOLVED}
STORAGE_LIMITED_MARK = set()


def _run(r, case):
    dt = case.params["timestep"]
    out = {}
    r.marker2nodes()
    out.update({("n", f): np.array(r.nodes[f]) for f in M2N_OUT})
    # every node field after marker2nodes (the antidiffusion inputs the
    # metric's floors come from)
    out["inputs"] = {f: np.array(r.nodes[f]) for f in range(abi.NF_N)}
    r.center2basic_old()
    r.compute_before_solve(dt, 0)
    r.compute_after_solve(dt, 0)
    out.update({("n", f): np.array(r.nodes[f]) for f in C2B_OUT + RSF_OUT})
    r.nodes2markers()
    out.update({("n", f): np.array(r.nodes[f]) for f in N2M_OUT})
    out.update({("m", f): np.array(r.marks[f]) for f in N2M_MARK})
    r.move()
    out.update({("m", f): np.array(r.marks[f]) for f in MOVE_MARK
                if f not in (abi.MF_X, abi.MF_Y)})
    return out


@pytest.mark.parametrize("name", ["tiny", "small", "mode1"])
def test_storage_error_bounded(name, oracle_built):
    kw = dict(interpolationmod=1) if name == "mode1" else {}
    c = synth.make_case("small" if name == "mode1" else name, seed=7, **kw)
    exact = _run(oracle.Restatement(c.copy()), c)
    stored = _run(oracle_for(c), c)
    nn, mn = abi.node_field_names(), abi.marker_field_names()
    bad = {}
    for key, ref in exact.items():
        if key == "inputs":
            continue
        kind, f = key
        if kind == "n":
            e = node_err(f, stored[(kind, f)], ref, exact["inputs"])
            tol = tolerance(nn[f], 1e-5 if f in STORAGE_LIMITED_NODE else 1e-6)
            label = nn[f]
        else:
            e = marker_err(f, stored[(kind, f)], ref)
            tol = tolerance(mn[f], 1e-5 if f in STORAGE_LIMITED_MARK else 1e-6)
            label = "marker " + mn[f]
        if not e <= tol:
            bad[label] = e
    assert not bad, bad


def test_device_view_keeps_cells_and_is_idempotent(oracle_built):
    """Rounding to the device's storage keeps every marker in its cell and
    rounds the rounded state to itself (so the device, uploading it again,
    holds the same values)."""
    from .parity import device_view, nxsearch_np
    c = synth.make_case("small", seed=3)
    d = device_view(c)
    for k, g in ((abi.MF_X, c.gx), (abi.MF_Y, c.gy)):
        assert np.array_equal(nxsearch_np(g, c.marks[k]), nxsearch_np(g, d.marks[k]))
    dd = device_view(d)
    for k in range(abi.MF_N):
        assert np.array_equal(dd.marks[k], d.marks[k]), abi.marker_field_names()[k]
    for f in range(abi.NF_N):
        assert np.array_equal(dd.nodes[f], d.nodes[f]), abi.node_field_names()[f]
