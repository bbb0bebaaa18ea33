"""Shared helpers of the parity tests: run a stage on the GPU and on the
oracle restatement from the same seeded state and measure per-field error.

Error metric per field: max |gpu - oracle| over entries, divided by the
field's scale max |oracle| (relative to the field's magnitude, since many
fields cross zero).
"""
from __future__ import annotations

import numpy as np

from velo2cycles_gb300 import abi

# fields written by each stage, compared after it
M2N_OUT = [abi.NF_PHIN, abi.NF_SXYEN, abi.NF_EXYEN, abi.NF_PEN, abi.NF_PHIS, abi.NF_SXYE,
           abi.NF_EXYE, abi.NF_PE, abi.NF_MUS_S, abi.NF_AS, abi.NF_BS, abi.NF_LS, abi.NF_V0S,
           abi.NF_COHESION, abi.NF_NU_M2C, abi.NF_GG, abi.NF_SXXEN, abi.NF_SPPEN, abi.NF_EXXEN,
           abi.NF_SXXE, abi.NF_SPPE, abi.NF_EXXE, abi.NF_ND_M2C, abi.NF_GD, abi.NF_BM,
           abi.NF_DRO, abi.NF_DRP, abi.NF_MVXN, abi.NF_MVX, abi.NF_MRX, abi.NF_MVYN, abi.NF_MVY,
           abi.NF_MRY, abi.NF_RO, abi.NF_ET, abi.NF_HT, abi.NF_KT, abi.NF_CP, abi.NF_TK,
           abi.NF_STICKY01, abi.NF_NU, abi.NF_ND, abi.NF_MRX0, abi.NF_MRY0]
C2B_OUT = [abi.NF_EXXES, abi.NF_SXXES, abi.NF_SPPES]
# interpolate_basic2center, interpolate_center2basic (interpolation.c:1600-1685);
# nd, exxpl and exxel carry the viscosity fields' error
B2C_C2B_OUT = [abi.NF_ND, abi.NF_EXXS, abi.NF_EXXPL, abi.NF_SXXS, abi.NF_PRS, abi.NF_EXXEL]
# recompute_stress_strainrate, copyarrays (momentum_continuity_iterate.c:214-281)
RECOMPUTE_OUT = [abi.NF_EXX, abi.NF_SXX, abi.NF_EXY, abi.NF_ESP, abi.NF_SXY]
COPY_OUT = [abi.NF_SLIPRS, abi.NF_RK_SLIPRS_FINAL, abi.NF_RK_PHIDTS_FINAL]
RSF_OUT = [abi.NF_PES, abi.NF_PHIS_IT, abi.NF_SYIELDS, abi.NF_NUVP_IT, abi.NF_SLIPRS, abi.NF_NU,
           abi.NF_RK_SLIPRS_SOLVED, abi.NF_RK_PHIDTS_SOLVED, abi.NF_RK_DELTAS]
N2M_OUT = [abi.NF_PHISUM, abi.NF_WTPHISUM, abi.NF_SXYSUM, abi.NF_EXYSUM, abi.NF_ESUM,
           abi.NF_PSUM, abi.NF_SXXSUM, abi.NF_EXXSUM, abi.NF_WTSXXSUM, abi.NF_VXSUM,
           abi.NF_VYSUM, abi.NF_WTVXSUM, abi.NF_WTVYSUM, abi.NF_MRX0, abi.NF_MRY0,
           abi.NF_PHIE, abi.NF_SXYEE, abi.NF_EXYEE, abi.NF_PEE, abi.NF_SPPEE, abi.NF_SXXEE,
           abi.NF_EXXEE, abi.NF_MVXE, abi.NF_MVYE]
N2M_MARK = [abi.MF_PHI, abi.MF_EXX, abi.MF_EXY, abi.MF_XX, abi.MF_XY, abi.MF_P, abi.MF_VX,
            abi.MF_VY, abi.MF_E, abi.MF_K]
MOVE_MARK = [abi.MF_X, abi.MF_Y, abi.MF_XX, abi.MF_XY, abi.MF_K, abi.MF_E]

# Viscosity-derived node fields carry the FP32 Arrhenius factor
# exp((E+PV)/RT) of the power-law rocks; an FP32 temperature perturbs its
# exponent by ~6e-8 relative, i.e. ~2e-6 relative on exp(40).
# The state rate RK_phidts_solved = V0/L e^-phi - V/L (calc_RSF.c:202) is a
# difference of two terms that carries the same error through the slip rate
# inverted from those viscosities; nd (harmonic mean of nu) and exxpl, exxel
# (through gd and nd_m2c, interpolation.c:1620-1632) carry it too.
VISCOUS = {abi.NF_NU_M2C, abi.NF_GG, abi.NF_ND_M2C, abi.NF_GD, abi.NF_NUVP_IT, abi.NF_NU,
           abi.NF_RK_PHIDTS_SOLVED, abi.NF_ND, abi.NF_EXXPL, abi.NF_EXXEL}


def temperature_case(seed, name="small"):
    """(case, old node T, new node T) for the marker temperature update: a
    smooth change of the node temperatures, newly arrived rock markers
    (T = 0) and fluid markers (type 50)."""
    from velo2cycles_gb300 import synth
    c = synth.make_case(name, seed)
    yn = c.gy.size
    m = np.arange(c.nodenum)
    told = c.nodes[abi.NF_TK].copy()
    tnew = told + 5.0 * np.sin(0.3 * (m // yn)) * np.cos(0.2 * (m % yn))
    c.marks[abi.MF_K][50:60] = 0.0
    c.markt[100:110] = 50
    return c, told, tnew


def stokes_case(seed, name="tiny", variant="default"):
    """(case, ctl) for the Stokes assembly: node fields of the oracle's
    marker2nodes, compute_before_solve and basic2center, rounded to FP32
    (what the device holds) and kept as FP64, so that the device, the
    restatement and the reference all see the same values.  Variants:
    'no_sailor' (drunkensailor 0), 'inertia' (inertyn 1), 'compressible'
    (compressiblemode 1), 'cont_bond' (the vx boundary of node (0, 0) given
    as the continuity equation of cell (1, 1), addvx's bondv > 1e30 form),
    'open_edge' (a left-edge vx node without a boundary equation: the
    reference would read past the grid)."""
    import oracle
    from velo2cycles_gb300 import synth
    kw = {"inertia": dict(inertyn=1), "compressible": dict(compressiblemode=1)}.get(variant, {})
    c = synth.make_case(name, seed, **kw)
    dt = float(c.params["timestep"])
    r = oracle.Restatement(c.copy())
    r.marker2nodes()
    r.compute_before_solve(dt, 0)
    r.basic2center()
    for f in range(abi.NF_N):
        c.nodes[f] = np.asarray(r.nodes[f], dtype=np.float32).astype(np.float64)
    c.bondn, c.bondv = c.bondn.copy(), c.bondv.copy()
    yn = c.gy.size
    if variant == "cont_bond":
        b = int(c.bondm[1])
        c.bondn[b * 3 + 0] = 3 * yn + 5   # the vx unknown of node (1, 1), 1-based
        c.bondv[b * 4 + 1] = 2e30
    if variant == "open_edge":
        c.bondm = c.bondm.copy()
        c.bondm[(0 * yn + 3) * 3 + 1] = 0
    from velo2cycles_gb300 import abi as _abi
    ctl = dict(_abi.STOKES_DEFAULTS, mukoef=dt * 30e5, dt=dt)
    if variant == "no_sailor":
        ctl["drunkensailor"] = 0
    return c, ctl


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fin = np.isfinite(b)
    if not np.array_equal(np.isfinite(a), fin):
        return float("inf")
    if not fin.any():
        return 0.0
    scale = np.abs(b[fin]).max()
    if scale == 0:
        return float(np.abs(a[fin]).max())
    return float(np.abs(a[fin] - b[fin]).max() / scale)


def node_errors(got: dict, ref: dict, fields) -> dict:
    names = abi.node_field_names()
    return {names[f]: rel_err(got[f], ref[f]) for f in fields}


def marker_errors(got: dict, ref: dict, fields) -> dict:
    names = abi.marker_field_names()
    return {names[f]: rel_err(got[f], ref[f]) for f in fields}


def nxsearch_np(g: np.ndarray, x: np.ndarray) -> np.ndarray:
    """nxsearch (interpolation.c:1536-1554) vectorised: the largest l with
    g[l] <= x, clamped to [0, n-2]; equal to the bisection for increasing g."""
    i = np.searchsorted(g, x, side="right") - 1
    return np.clip(i, 0, g.size - 2)
