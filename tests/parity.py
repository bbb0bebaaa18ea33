"""Shared helpers of the parity tests: run a stage on the GPU and on the
oracle restatement from the same seeded state and measure per-field error.

Two oracles per case:
  * `device_view(case)` -- the state exactly as the device holds it after
    upload: marker fields rounded to FP32, the temperature and markv (the
    y anchor of immobile markers) to float pairs,
    each position to its cell plus the device's FP32 in-cell offset, node
    fields to FP32 (except VX, VY, TK, TK2, of which the device also keeps
    the uploaded FP64 values).  The GPU against the oracle on this state is
    the arithmetic error of the device path: asserted per entry.
  * the original FP64 state.  The oracle on the device view against the
    oracle on the original is the error that FP32 storage alone causes
    (no GPU involved): `storage_errors`, bounded per field in STORAGE_BOUND.
    The GPU against the original oracle is at most the sum of the two.

Error metric, per field (rel_err):
  * fields whose entries are positive magnitudes (viscosity, density,
    temperature, conductivity, weights, friction parameters, ...): max over
    entries of |got - ref| / |ref|, every entry relative whatever decade it
    sits in;
  * fields whose entries cross zero or are differences of nearly equal
    terms (SIGNED_NODE, SIGNED_MARK: stresses, strain rates, velocities,
    pressures, state, their node sums): the same with a floor, max |got -
    ref| / max(|ref|, floor): an entry smaller than the floor is a
    cancellation of terms of that size, and is held to an absolute error
    relative to it.  The floor is the field's RMS, or for the antidiffusion
    outputs (FLOOR_FROM: a node value plus the change of a node average,
    interpolation.c:730-736, 758-763, 784-806) the RMS of the largest node
    field they are formed from;
  * slip rates (LOG_NODE, LOG_MARK), which span thirty decades and depend
    exponentially on the node state and stresses (V = 2 V0 sinh(tau/(a
    sigma)) e^-(mu0 + b phi)/a, calc_RSF.c:191, with b/a up to ~3 and
    arguments of a few hundred): max |ln got - ln ref|, i.e. the relative
    error of V, held to TOL_LOG = 2e-5, about b/a times the FP32 rounding
    (4e-6) of a state phi of ~50.  Below 1e-30 m/s both are taken as 1e-30
    (FP32 holds the path's 1e-40 floor only as a subnormal);
  * the state rates V0/L e^-phi - V/L (RATE_NODE), which carry V/L with the
    slip rate's error: the signed metric against TOL_LOG.
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

# node fields whose entries cross zero (see the module docstring)
SIGNED_NODE = {
    abi.NF_PHIN, abi.NF_SXYEN, abi.NF_EXYEN, abi.NF_PEN, abi.NF_PHIS, abi.NF_SXYE, abi.NF_EXYE,
    abi.NF_PE, abi.NF_SXXEN, abi.NF_SPPEN, abi.NF_EXXEN, abi.NF_SXXE, abi.NF_SPPE, abi.NF_EXXE,
    abi.NF_MVXN, abi.NF_MVX, abi.NF_MVYN, abi.NF_MVY, abi.NF_DRO, abi.NF_DRP,
    abi.NF_EXXES, abi.NF_SXXES, abi.NF_SPPES, abi.NF_PES, abi.NF_PHIS_IT,
    abi.NF_RK_PHIDTS_SOLVED, abi.NF_RK_PHIDTS_FINAL, abi.NF_RK_DELTAS,
    abi.NF_EXXS, abi.NF_EXXPL, abi.NF_SXXS, abi.NF_PRS, abi.NF_EXXEL,
    abi.NF_EXX, abi.NF_SXX, abi.NF_EXY, abi.NF_ESP, abi.NF_SXY, abi.NF_VX, abi.NF_VY, abi.NF_PR,
    abi.NF_PHISUM, abi.NF_SXYSUM, abi.NF_EXYSUM, abi.NF_ESUM, abi.NF_PSUM, abi.NF_SXXSUM,
    abi.NF_EXXSUM, abi.NF_VXSUM, abi.NF_VYSUM, abi.NF_PHIE, abi.NF_SXYEE, abi.NF_EXYEE,
    abi.NF_PEE, abi.NF_SPPEE, abi.NF_SXXEE, abi.NF_EXXEE, abi.NF_MVXE, abi.NF_MVYE}
SIGNED_MARK = {abi.MF_PHI, abi.MF_EXX, abi.MF_EXY, abi.MF_XX, abi.MF_XY, abi.MF_P, abi.MF_VX,
               abi.MF_VY, abi.MF_E}
LOG_NODE = {abi.NF_SLIPRS, abi.NF_RK_SLIPRS_SOLVED, abi.NF_RK_SLIPRS_FINAL}
LOG_MARK = {abi.MF_SLIPV}
RATE_NODE = {abi.NF_RK_PHIDTS_SOLVED, abi.NF_RK_PHIDTS_FINAL}
LOG_FLOOR = 1e-30
TOL_LOG = 2e-5
FLOOR_FRAC = 1.0
# antidiffusion outputs and the node fields they are formed from
FLOOR_FROM = {
    abi.NF_PHIS: (abi.NF_PHIS_IT, abi.NF_PHIE), abi.NF_SXYE: (abi.NF_SXY, abi.NF_SXYEE),
    abi.NF_EXYE: (abi.NF_EXY, abi.NF_EXYEE), abi.NF_PE: (abi.NF_PES, abi.NF_PEE),
    abi.NF_SXXE: (abi.NF_SXX, abi.NF_SXXEE), abi.NF_SPPE: (abi.NF_PR, abi.NF_SPPEE),
    abi.NF_EXXE: (abi.NF_EXX, abi.NF_EXXEE), abi.NF_MVX: (abi.NF_VX, abi.NF_MVXE),
    abi.NF_MVY: (abi.NF_VY, abi.NF_MVYE)}


def _rms(a) -> float:
    a = np.asarray(a, dtype=np.float64)
    a = a[np.isfinite(a)]
    return float(np.sqrt(np.mean(a * a))) if a.size else 0.0
# fields the device keeps in FP64 beside their FP32 copy (strain rates from
# velocity differences; the marker temperature update)
NODE_FP64 = {abi.NF_VX, abi.NF_VY, abi.NF_TK, abi.NF_TK2}


def offset32(u: np.ndarray) -> np.ndarray:
    """The device's FP32 in-cell offset of FP64 offsets u (offset32 in
    csrc/v2c_internal.cuh): the nearest float, moved back to the side of 0,
    1/2 and 1 that u is on."""
    u = np.asarray(u, dtype=np.float64)
    f = u.astype(np.float32)
    half, one, zero = np.float32(0.5), np.float32(1.0), np.float32(0.0)
    f = np.where((u < 0.5) & (f >= half), np.nextafter(half, zero), f)
    f = np.where((u > 0.5) & (f <= half), np.nextafter(half, one), f)
    f = np.where((u < 1.0) & (f >= one), np.nextafter(one, zero), f)
    f = np.where((u > 1.0) & (f <= one), np.nextafter(one, np.float32(2.0)), f)
    f = np.where((u > 0.0) & (f <= zero), np.float32(1e-30), f)
    f = np.where((u < 0.0) & (f >= zero), np.float32(-1e-30), f)
    return f.astype(np.float32)


def device_view(case):
    """Copy of case holding what the device stores after upload (module
    docstring)."""
    d = case.copy()
    for k in range(abi.MF_N):
        if k in (abi.MF_X, abi.MF_Y):
            continue
        a = np.asarray(d.marks[k], dtype=np.float64)
        if k in (abi.MF_K, abi.MF_V):  # float pairs on the device
            hi = a.astype(np.float32).astype(np.float64)
            d.marks[k] = hi + (a - hi).astype(np.float32).astype(np.float64)
        else:
            d.marks[k] = a.astype(np.float32).astype(np.float64)
    for k, g in ((abi.MF_X, d.gx), (abi.MF_Y, d.gy)):
        x = np.asarray(d.marks[k], dtype=np.float64)
        i = nxsearch_np(g, x)
        w = g[i + 1] - g[i]
        d.marks[k] = g[i] + offset32((x - g[i]) / w).astype(np.float64) * w
    for f in range(abi.NF_N):
        if f not in NODE_FP64:
            d.nodes[f] = np.asarray(d.nodes[f], dtype=np.float64).astype(np.float32).astype(np.float64)
    return d


def _round_markers(marks: dict, gx, gy, n: int) -> None:
    """Round marker arrays (in place, first n) to what the device stores."""
    for k, a in marks.items():
        v = a[:n]
        if k in (abi.MF_X, abi.MF_Y):
            g = gx if k == abi.MF_X else gy
            i = nxsearch_np(g, v)
            w = g[i + 1] - g[i]
            v[:] = g[i] + offset32((v - g[i]) / w).astype(np.float64) * w
        elif k in (abi.MF_K, abi.MF_V):
            hi = v.astype(np.float32).astype(np.float64)
            v[:] = hi + (v - hi).astype(np.float32).astype(np.float64)
        else:
            v[:] = v.astype(np.float32).astype(np.float64)


def oracle_for(case, **kw):
    """The oracle restatement on the state the device holds, rounded again
    to the device's storage after every stage (DeviceOracle)."""
    return DeviceOracle(device_view(case), **kw)


class DeviceOracle:
    """oracle.Restatement whose node and marker arrays are rounded to the
    device's storage (device_view) after every stage, so that a chain of
    stages on both sides compares the device's arithmetic stage by stage:
    node fields to FP32 except VX, VY and TK2 (the device keeps the uploaded
    FP64 values; TK too until marker2nodes writes it), marker fields to FP32,
    the temperature and markv to float pairs, positions to cell + FP32
    offset."""

    STAGES = ("marker2nodes", "center2basic_old", "basic2center", "center2basic",
              "recompute_stress", "copyarrays", "compute_before_solve", "compute_after_solve",
              "nodes2markers", "move", "marker_temperature", "step")

    def __init__(self, case, **kw):
        import oracle
        self._r = oracle.Restatement(case, **kw)
        self._tk64 = True

    def __getattr__(self, name):
        attr = getattr(self._r, name)
        if name not in DeviceOracle.STAGES:
            return attr

        def stage(*args, **kw):
            out = attr(*args, **kw)
            if name in ("marker2nodes", "step"):
                self._tk64 = False
            self._round()
            return out
        return stage

    def _round(self):
        r = self._r
        keep = {abi.NF_VX, abi.NF_VY, abi.NF_TK2} | ({abi.NF_TK} if self._tk64 else set())
        for f, a in r.nodes.items():
            if f not in keep:
                a[:] = a.astype(np.float32).astype(np.float64)
        _round_markers(r._marks, r.gx, r.gy, r.n)


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


def immobile_case(seed, name="small", n_imm=40, n_out=25, **kw):
    """A case with immobile markers (type 100 + t, anchored at their own
    position: markk holds the anchor x, markv the anchor y), some of them
    far from their anchor, and mobile markers outside the model that the
    markers they spawn refill (moveandrotatemarkers.c:88-171).  The rock
    table rows 100 + t repeat rows t."""
    from velo2cycles_gb300 import synth
    c = synth.make_case(name, seed, **kw)
    rng = np.random.default_rng(seed)
    idx = rng.choice(c.n, n_imm + n_out, replace=False)
    imm, out = idx[:n_imm], idx[n_imm:]
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    c.marks[abi.MF_K][imm] = x[imm]
    c.marks[abi.MF_V][imm] = y[imm]
    # a few start away from their anchor (moved back when more than ystpy)
    far = imm[: n_imm // 4]
    c.marks[abi.MF_V][far] = y[far] - 3.0 * c.params["ystpy"]
    c.markt[imm] = (100 + c.markt[imm]).astype(np.int8)
    x[out] = np.where(rng.random(n_out) < 0.5, -1.0 - rng.random(n_out) * 100.0,
                      c.gx[-1] + 1.0 + rng.random(n_out) * 100.0)
    for t in range(1, 28):
        c.rt[:, 100 + t] = c.rt[:, t]
    return c


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


def rel_err(a: np.ndarray, b: np.ndarray, signed: bool = True, log: bool = False,
            abs_floor=0.0) -> float:
    """Largest per-entry error of a against the reference b (module
    docstring): max |a - b| / max(|b|, floor), floor = max(abs_floor,
    FLOOR_FRAC * RMS(b)) for a signed field, abs_floor otherwise (a scalar,
    or an array of per-entry floors); for a log field the relative error of
    the logarithm.  Entries where the floor and b are both zero must match
    exactly; NaN/inf must sit at the same entries."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fin = np.isfinite(b)
    if not np.array_equal(np.isfinite(a), fin):
        return float("inf")
    if not fin.any():
        return 0.0
    aa, bb = a[fin], b[fin]
    if np.ndim(abs_floor):
        abs_floor = np.asarray(abs_floor, dtype=np.float64)[fin]
    if log:
        if (aa < 0).any() or (bb < 0).any():
            return float("inf")
        la = np.log(np.maximum(aa, LOG_FLOOR))
        lb = np.log(np.maximum(bb, LOG_FLOOR))
        return float(np.abs(la - lb).max())
    floor = abs_floor
    if signed:
        floor = np.maximum(floor, FLOOR_FRAC * float(np.sqrt(np.mean(bb * bb))))
    den = np.maximum(np.abs(bb), floor)
    d = np.abs(aa - bb)
    zero = den == 0
    if np.any(d[zero] != 0):
        return float("inf")
    if zero.all():
        return 0.0
    return float((d[~zero] / den[~zero]).max())


def node_err(f: int, a, b, ref: dict | None = None) -> float:
    """rel_err of node field f; ref (the reference's node fields) supplies
    the antidiffusion inputs of FLOOR_FROM."""
    floor = 0.0
    if ref is not None and f in FLOOR_FROM:
        floor = max(_rms(ref[k]) for k in FLOOR_FROM[f])
    return rel_err(a, b, f in SIGNED_NODE or f in RATE_NODE, f in LOG_NODE, floor)


def marker_err(f: int, a, b, floor=0.0) -> float:
    return rel_err(a, b, f in SIGNED_MARK, f in LOG_MARK, floor)


# node fields each marker field takes in nodes2markers (interpolation.c:
# 943-1011): the current field, and the previous one that the marker's change
# is measured from without antidiffusion
N2M_SOURCES = {
    abi.MF_XX: (abi.NF_SXX, abi.NF_SXXE), abi.MF_XY: (abi.NF_SXY, abi.NF_SXYE),
    abi.MF_EXX: (abi.NF_EXX, abi.NF_EXXE), abi.MF_EXY: (abi.NF_EXY, abi.NF_EXYE),
    abi.MF_P: (abi.NF_PR, abi.NF_SPPE), abi.MF_VX: (abi.NF_VX, abi.NF_MVX),
    abi.MF_VY: (abi.NF_VY, abi.NF_MVY), abi.MF_PHI: (abi.NF_PHIS_IT, abi.NF_PHIS),
    abi.MF_E: (abi.NF_PES, abi.NF_PE)}


def n2m_floors(ref) -> dict:
    """Per-marker floors of the marker fields nodes2markers writes, taken on
    the state it starts from (call before the oracle's nodes2markers): the
    largest magnitude among the node values of the 4 x 4 block of node lines
    around the marker's cell (every stencil of interpolate_mechanical lies
    in it) in the node fields the marker field is interpolated from.  The
    interpolation is a weighted sum of those FP32 node values; where they
    differ in sign or by orders of magnitude (a shear band two cells wide
    beside a quiet far field) its FP32 evaluation -- weights, products,
    sums -- is exact only to a few 1e-8 of them, not of the result, and
    that is the scale its error is measured against."""
    x, y = ref.marks[abi.MF_X], ref.marks[abi.MF_Y]
    gx, gy = ref.gx, ref.gy
    xn, yn = gx.size, gy.size
    ix, iy = nxsearch_np(gx, x), nxsearch_np(gy, y)
    idx = [np.clip(ix + dx, 0, xn - 1) * yn + np.clip(iy + dy, 0, yn - 1)
           for dx in range(-1, 3) for dy in range(-1, 3)]
    out = {}
    for f, srcs in N2M_SOURCES.items():
        m = np.zeros(x.size)
        for k in srcs:
            a = np.abs(np.asarray(ref.nodes[k], dtype=np.float64))
            for q in idx:
                m = np.maximum(m, a[q])
        out[f] = m
    return out


def rotated_floors(fl: dict) -> dict:
    """The floors after the move's stress rotation, which mixes xx and xy."""
    out = dict(fl)
    out[abi.MF_XX] = out[abi.MF_XY] = np.maximum(fl[abi.MF_XX], fl[abi.MF_XY])
    return out


def node_errors(got: dict, ref: dict, fields) -> dict:
    names = abi.node_field_names()
    return {names[f]: node_err(f, got[f], ref[f], ref) for f in fields}


_NODE_IDS = {v: k for k, v in abi.node_field_names().items()}
_MARK_IDS = {v: k for k, v in abi.marker_field_names().items()}


def tolerance(name: str, tol: float = 1e-6) -> float:
    """The tolerance of a field named as node_errors / marker_errors name
    it: tol, or TOL_LOG for slip and state rates."""
    f = _NODE_IDS.get(name)
    if f is not None and (f in LOG_NODE or f in RATE_NODE):
        return TOL_LOG
    if name in _MARK_IDS and _MARK_IDS[name] in LOG_MARK:
        return TOL_LOG
    return tol


def over(errs: dict, tol: float = 1e-6) -> dict:
    """the entries of errs above their field's tolerance"""
    return {k: v for k, v in errs.items() if not v <= tolerance(k, tol)}


def marker_errors(got: dict, ref: dict, fields, floors: dict | None = None) -> dict:
    """per-field rel_err of marker fields; floors: per-marker floors
    (n2m_floors) of the fields that have them"""
    names = abi.marker_field_names()
    fl = floors or {}
    return {names[f]: marker_err(f, got[f], ref[f], fl.get(f, 0.0)) for f in fields}


def nxsearch_np(g: np.ndarray, x: np.ndarray) -> np.ndarray:
    """nxsearch (interpolation.c:1536-1554) vectorised: the largest l with
    g[l] <= x, clamped to [0, n-2]; equal to the bisection for increasing g."""
    i = np.searchsorted(g, x, side="right") - 1
    return np.clip(i, 0, g.size - 2)
