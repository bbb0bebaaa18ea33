"""Host-side mirror of the reference's MIC interface over the C ABI.

The reference (src/i2evps.c:82-132) calls, per time step,

    marker2nodes(); interpolate_center2basic_old(timestep);
    solve_momentum_continuity(...)   # host: compute_before_solve /
                                     # compute_after_solve around Pardiso
    nodes2markers(); moveandrotatemarkers();

on global arrays.  ``MarkerInCell`` exposes the same calls on one GPU
context; arrays cross the boundary as FP64 numpy arrays in the reference
layout (node index m1*ynumy+m2, markers in reference numbering).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi
from ._lib import call, lib

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class MarkerInCell:
    """One GPU context holding grid, rock table, boundary equations, marker
    and node arrays.  Mirrors the reference routines' names and order."""

    def __init__(self, params: dict, max_markers: int, stream: int | None = None):
        self.params = dict(params)
        self._p = abi.Params.from_dict(self.params)
        h = ctypes.c_void_p()
        call("v2c_create", ctypes.byref(self._p), int(max_markers),
             ctypes.c_void_p(stream) if stream else None, ctypes.byref(h))
        self.h = h
        self.nn = int(self.params["xnumx"] * self.params["ynumy"])
        self.n = 0

    # ------------------------------------------------------------ set-up
    def close(self):
        if self.h:
            call("v2c_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, **kw):
        self.params.update(kw)
        self._p = abi.Params.from_dict(self.params)
        call("v2c_set_params", self.h, ctypes.byref(self._p))

    def set_grid(self, gx: np.ndarray, gy: np.ndarray):
        self._gx = np.ascontiguousarray(gx, dtype=np.float64)
        self._gy = np.ascontiguousarray(gy, dtype=np.float64)
        call("v2c_set_grid", self.h, _ptr(self._gx), _ptr(self._gy))

    def set_rock_table(self, rt: np.ndarray):
        rt = np.ascontiguousarray(rt, dtype=np.float64)
        call("v2c_set_rock_table", self.h, _ptr(rt))

    def set_bonds(self, bondm, bondn, bondv):
        bm = np.ascontiguousarray(bondm, dtype=np.int64)
        bn = np.ascontiguousarray(bondn, dtype=np.int64)
        bv = np.ascontiguousarray(bondv, dtype=np.float64)
        lp = ctypes.POINTER(ctypes.c_long)
        call("v2c_set_bonds", self.h, bm.ctypes.data_as(lp), bn.ctypes.data_as(lp), _ptr(bv),
             bv.size // 4)

    # ----------------------------------------------------------- markers
    def upload_markers(self, marks: dict, markt: np.ndarray):
        n = int(markt.shape[0])
        keep = {}
        arr = (_dp * abi.MF_N)()
        for f in range(abi.MF_N):
            if f in marks and marks[f] is not None:
                a = np.ascontiguousarray(marks[f], dtype=np.float64)
                assert a.shape[0] == n
                keep[f] = a
                arr[f] = _ptr(a)
        t = np.ascontiguousarray(markt, dtype=np.int8)
        call("v2c_upload_markers", self.h, arr, t.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)), n)
        self.n = n
        # immobile markers (type >= 100) append markers in the move
        self._immobile = bool((t >= 100).any())

    def _refresh_n(self):
        if getattr(self, "_immobile", False):
            self.n = int(self.status()["n_markers"])

    def download_markers(self, fields=None, into: dict | None = None):
        """FP64 marker arrays in reference numbering.  markd/markw given in
        `into` are updated in place (set to -1 for markers reset after
        leaving the grid)."""
        fields = list(range(abi.MF_N)) if fields is None else list(fields)
        device_fields = {abi.MF_X, abi.MF_Y, abi.MF_K, abi.MF_V, abi.MF_E, abi.MF_P, abi.MF_XX,
                         abi.MF_XY, abi.MF_EXX, abi.MF_EXY, abi.MF_VX, abi.MF_VY, abi.MF_PHI,
                         abi.MF_C, abi.MF_SLIPV}
        out = {} if into is None else into
        arr = (_dp * abi.MF_N)()
        for f in fields:
            if f in device_fields or f in (abi.MF_D, abi.MF_W):
                if f not in out:
                    out[f] = np.zeros(self.n) if f not in (abi.MF_D, abi.MF_W) else np.zeros(self.n)
                out[f] = np.ascontiguousarray(out[f], dtype=np.float64)
                arr[f] = _ptr(out[f])
        t = np.zeros(self.n, dtype=np.int8)
        call("v2c_download_markers", self.h, arr, t.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)),
             self.n)
        out["markt"] = t
        return out

    def download_cells(self) -> np.ndarray:
        c = np.zeros(self.n, dtype=np.int32)
        call("v2c_download_cells", self.h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), self.n)
        return c

    def download_marker_properties(self) -> tuple[np.ndarray, np.ndarray]:
        """(viscosity, conductivity) of every marker as the last
        marker2nodes evaluated them, in reference numbering (0 for markers
        outside the model)."""
        nu, kt = np.zeros(self.n), np.zeros(self.n)
        call("v2c_download_marker_properties", self.h, _ptr(nu), _ptr(kt), self.n)
        return nu, kt

    # -------------------------------------------------------------- nodes
    def upload_node(self, field: int, values: np.ndarray):
        a = np.ascontiguousarray(values, dtype=np.float64)
        assert a.size == self.nn
        call("v2c_upload_node_field", self.h, int(field), _ptr(a))

    def download_node(self, field: int) -> np.ndarray:
        a = np.zeros(self.nn)
        call("v2c_download_node_field", self.h, int(field), _ptr(a))
        return a

    def upload_nodes(self, nodes: dict):
        """Several node fields in one call (one conversion kernel, one copy
        each); the arrays must stay unchanged until the stream synchronises."""
        arrs = {int(f): np.ascontiguousarray(v, dtype=np.float64) for f, v in nodes.items()}
        for a in arrs.values():
            assert a.size == self.nn
        self._keep_up = arrs  # the copies from pinned memory run later
        fl = (ctypes.c_int * len(arrs))(*arrs.keys())
        pp = (ctypes.POINTER(ctypes.c_double) * len(arrs))(*[_ptr(a) for a in arrs.values()])
        call("v2c_upload_node_fields", self.h, len(arrs), fl, pp)

    def download_nodes(self, fields=None, into: dict | None = None) -> dict:
        fields = list(range(abi.NF_N) if fields is None else fields)
        out = into if into is not None else {}
        for f in fields:
            if f not in out:
                out[f] = np.zeros(self.nn)
        fl = (ctypes.c_int * len(fields))(*fields)
        pp = (ctypes.POINTER(ctypes.c_double) * len(fields))(*[_ptr(out[f]) for f in fields])
        call("v2c_download_node_fields", self.h, len(fields), fl, pp)
        return {f: out[f] for f in fields}

    def download_nodes_async(self, arrays: dict):
        """Start downloading node fields into arrays (field id -> nodenum
        doubles, ideally pinned): a snapshot of the fields as the calls
        enqueued so far leave them, copied while later calls run; read them
        after wait_downloads()."""
        fields = list(arrays)
        for f in fields:
            a = arrays[f]
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.nn
        fl = (ctypes.c_int * len(fields))(*fields)
        pp = (ctypes.POINTER(ctypes.c_double) * len(fields))(*[_ptr(arrays[f]) for f in fields])
        self._async_keep = (arrays, fl, pp)
        call("v2c_download_node_fields_async", self.h, len(fields), fl, pp)

    def wait_downloads(self):
        call("v2c_wait_downloads", self.h)
        self._async_keep = None

    # ----------------------------------------------------- the MIC calls
    def marker2nodes(self):
        call("v2c_marker2nodes", self.h)

    def interpolate_center2basic_old(self):
        call("v2c_center2basic_old", self.h)

    def interpolate_basic2center(self):
        """interpolate_basic2center (interpolation.c:1639): nd at the pressure
        nodes, harmonic mean of nu."""
        call("v2c_interpolate_basic2center", self.h)

    def interpolate_center2basic(self, dt: float):
        """interpolate_center2basic (interpolation.c:1600): exxs, exxpl, sxxs,
        prs, exxel on the basic nodes."""
        call("v2c_interpolate_center2basic", self.h, float(dt))

    def recompute_stress_strainrate(self, dt: float):
        """recompute_stress_strainrate (momentum_continuity_iterate.c:214):
        node strain rates and visco-elastic stresses from vx, vy."""
        call("v2c_recompute_stress_strainrate", self.h, float(dt))

    def marker_temperature(self, heatdif: float = 1.0):
        """The marker part of solve_temperature (temperature_iterate.c:181):
        node TK holds the solved temperature, TK2 the previous one."""
        call("v2c_marker_temperature", self.h, float(heatdif))

    def copyarrays(self):
        """copyarrays (momentum_continuity_iterate.c:265)."""
        call("v2c_copyarrays", self.h)

    def stokes_assemble(self, mukoef: float, dt: float, **ctl) -> dict:
        """preparematrix (momentum_continuity_addmatrix_checkerror.c:22) on
        the device's node fields: the CSR arrays gausmat4_add builds for
        Pardiso (ia, ja 1-based; a; right-hand side b).  ctl: gxkoef, gykoef,
        timebond, drunkensailor (abi.STOKES_DEFAULTS otherwise)."""
        c = abi.StokesCtl(**dict(abi.STOKES_DEFAULTS, mukoef=mukoef, dt=dt, **ctl))
        P = ctypes.POINTER
        nnz = ctypes.c_long(0)
        call("v2c_stokes_assemble", self.h, ctypes.byref(c), 0, None, None, None, None,
             ctypes.byref(nnz))
        rows = 3 * self.nn
        ia = np.zeros(rows + 1, dtype=np.int32)
        ja = np.zeros(max(nnz.value, 1), dtype=np.int32)
        a = np.zeros(max(nnz.value, 1))
        b = np.zeros(rows)
        call("v2c_stokes_assemble", self.h, ctypes.byref(c), nnz.value,
             ia.ctypes.data_as(P(ctypes.c_int)), ja.ctypes.data_as(P(ctypes.c_int)),
             a.ctypes.data_as(P(ctypes.c_double)), b.ctypes.data_as(P(ctypes.c_double)),
             ctypes.byref(nnz))
        return dict(ia=ia, ja=ja[:nnz.value], a=a[:nnz.value], b=b)

    def cycle_set_velocity(self, regime: int, vx: np.ndarray, vy: np.ndarray):
        """Velocity field of a seismic-cycle regime (0 interseismic, 1
        coseismic); regime 0 also zeroes the accumulated slip."""
        a = np.ascontiguousarray(vx, dtype=np.float64)
        b = np.ascontiguousarray(vy, dtype=np.float64)
        assert a.size == self.nn and b.size == self.nn
        call("v2c_cycle_set_velocity", self.h, int(regime), _ptr(a), _ptr(b))

    def cycle_step(self, regime: int, dt: float, use_graph: bool = True):
        """One seismic-cycle step (see v2c_cycle_step); timesum advances."""
        call("v2c_cycle_step", self.h, int(regime), float(dt), int(bool(use_graph)))
        self._refresh_n()
        self.params["timestep"] = float(dt)
        self.params["timesum"] = float(self.params["timesum"]) + float(dt)

    def cycle_slip(self) -> np.ndarray:
        a = np.zeros(self.nn)
        call("v2c_cycle_slip", self.h, _ptr(a))
        return a

    def cycle_marker_slip(self) -> np.ndarray:
        a = np.zeros(self.n)
        call("v2c_cycle_marker_slip", self.h, _ptr(a), int(self.n))
        return a

    def compute_before_solve(self, dt: float, rk: int = 0):
        call("v2c_compute_before_solve", self.h, float(dt), int(rk))

    def compute_after_solve(self, dt: float, rk: int = 0) -> float:
        d = ctypes.c_double()
        call("v2c_compute_after_solve", self.h, float(dt), int(rk), ctypes.byref(d))
        return d.value

    def nodes2markers(self):
        call("v2c_nodes2markers", self.h)

    def moveandrotatemarkers(self):
        call("v2c_moveandrotatemarkers", self.h)
        self._refresh_n()

    def nodes2markers_move(self):
        call("v2c_nodes2markers_move", self.h)
        self._refresh_n()

    def synchronize(self):
        call("v2c_synchronize", self.h)

    def calc_timestep(self, oldornew: int = 0, **ctl) -> dict:
        """calc_timestep (calc_RSF.c:352): dt_f, the maximum slip rate, the
        individual limits and the sticky-air statistics.  ctl overrides
        abi.TIMESTEP_DEFAULTS (maxtmstep, dtfactor, tcnvp, tcd, tcphih)."""
        c = abi.TimestepCtl(**dict(abi.TIMESTEP_DEFAULTS, **ctl))
        info = abi.TimestepInfo()
        call("v2c_calc_timestep", self.h, int(oldornew), ctypes.byref(c), ctypes.byref(info))
        return info.to_dict()

    def status(self) -> dict:
        s = abi.Status()
        call("v2c_get_status", self.h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in abi.Status._fields_}

    def set_profiling(self, on: bool = True):
        call("v2c_set_profiling", self.h, int(bool(on)))

    def profile(self) -> dict:
        """Summed device milliseconds and launch counts per kernel group."""
        out = {}
        names = {v: k[5:].lower() for k, v in vars(abi).items() if k.startswith("PROF_") and k != "PROF_N"}
        for g in range(abi.PROF_N):
            ms, n = ctypes.c_double(), ctypes.c_long()
            call("v2c_get_profile", self.h, g, ctypes.byref(ms), ctypes.byref(n))
            out[names[g]] = (ms.value, n.value)
        return out

    def step(self, fused: bool = True):
        """One MIC step with the solver outputs already on the device."""
        dt = self.params["timestep"]
        self.marker2nodes()
        self.interpolate_center2basic_old()
        self.compute_before_solve(dt, 0)
        self.compute_after_solve(dt, 0)
        if fused:
            self.nodes2markers_move()
        else:
            self.nodes2markers()
            self.moveandrotatemarkers()


def from_case(case, max_markers: int | None = None) -> MarkerInCell:
    """Context loaded with a synth.Case (grid, rocks, bonds, markers, nodes)."""
    mic = MarkerInCell(case.params, max_markers or case.n)
    mic.set_grid(case.gx, case.gy)
    mic.set_rock_table(case.rt)
    mic.set_bonds(case.bondm, case.bondn, case.bondv)
    mic.upload_markers(case.marks, case.markt)
    mic.upload_nodes(case.nodes)
    return mic
