"""The reference's binary restart files (.prn, load_save.c:164-527 with the
RSF extras of input_RSF.c:94-132) through the C ABI (v2c_prn_*): a model
state saved by the reference can drive the GPU step (and the oracle), and a
state can be written back for the reference to load.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi, synth
from ._lib import call

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


def read_info(path: str) -> abi.PrnInfo:
    info = abi.PrnInfo()
    call("v2c_prn_read_info", str(path).encode(), ctypes.byref(info))
    return info


def read(path: str) -> dict:
    """Every array of the file: info, rt (rock table rows of the path),
    rock_extra, nodes {NF id: array} (the node fields the file holds), bondm,
    gx, gy, bondv, bondn, marks {MF id: array}, markt."""
    info = read_info(path)
    xn, yn, n, nb = info.xnumx, info.ynumy, info.marknum, info.bondnum
    nn = xn * yn
    rt = np.zeros(abi.RT_N * abi.MAXTMR)
    extra = np.zeros(abi.PRN_ROCK_EXTRA * abi.MAXTMR)
    node_ids = (abi.NF_SXXEE, abi.NF_SXX, abi.NF_EXXEE, abi.NF_EXX, abi.NF_SXYEE, abi.NF_SXY,
                abi.NF_EXYEE, abi.NF_EXY, abi.NF_SPPEE, abi.NF_PR, abi.NF_PHIE, abi.NF_PHIS_IT,
                abi.NF_MVXE, abi.NF_VX, abi.NF_MVYE, abi.NF_VY, abi.NF_PES, abi.NF_PEE,
                abi.NF_RK_SLIPRS_FINAL, abi.NF_RK_PHIDTS_FINAL)
    nodes = {f: np.zeros(nn) for f in node_ids}
    mark_ids = (abi.MF_X, abi.MF_Y, abi.MF_K, abi.MF_E, abi.MF_XX, abi.MF_V, abi.MF_XY, abi.MF_P,
                abi.MF_EXX, abi.MF_EXY, abi.MF_D, abi.MF_W, abi.MF_VX, abi.MF_VY, abi.MF_PHI,
                abi.MF_L, abi.MF_L0, abi.MF_C, abi.MF_C0)
    marks = {f: np.zeros(n) for f in mark_ids}
    bondm = np.zeros(4 * nn, dtype=np.int64)
    gx, gy = np.zeros(xn), np.zeros(yn)
    bondv, bondn = np.zeros(4 * max(nb, 1)), np.zeros(3 * max(nb, 1), dtype=np.int64)
    markt = np.zeros(n, dtype=np.int8)
    na = (_dp * abi.NF_N)(*[_ptr(nodes[f]) if f in nodes else None for f in range(abi.NF_N)])
    ma = (_dp * abi.MF_N)(*[_ptr(marks[f]) if f in marks else None for f in range(abi.MF_N)])
    call("v2c_prn_read", str(path).encode(), ctypes.byref(info), _ptr(rt), _ptr(extra), na,
         _ptr(bondm, _lp), _ptr(gx), _ptr(gy), _ptr(bondv), _ptr(bondn, _lp), ma,
         markt.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)))
    return dict(info=info, rt=rt.reshape(abi.RT_N, abi.MAXTMR),
                rock_extra=extra.reshape(abi.PRN_ROCK_EXTRA, abi.MAXTMR), nodes=nodes,
                bondm=bondm, gx=gx, gy=gy, bondv=bondv, bondn=bondn, marks=marks, markt=markt)


def write(path: str, case, info: abi.PrnInfo | None = None, rock_extra=None) -> None:
    """Write a synth.Case (grid, rock table, node fields, boundary equations,
    markers) as a restart file; header values the case does not hold come
    from `info` (or are zero)."""
    p = case.params
    h = abi.PrnInfo() if info is None else info
    h.xnumx, h.ynumy, h.marknum, h.bondnum = case.gx.size, case.gy.size, case.n, case.bondnum
    h.xsize, h.ysize = float(p["xsize"]), float(p["ysize"])
    h.timestep, h.timesum = float(p["timestep"]), float(p["timesum"])
    h.rocknum = abi.MAXTMR if info is None else h.rocknum
    rt = np.ascontiguousarray(case.rt, dtype=np.float64).ravel()
    ex = None if rock_extra is None else np.ascontiguousarray(rock_extra, dtype=np.float64).ravel()
    nodes = {f: np.ascontiguousarray(v, dtype=np.float64) for f, v in case.nodes.items()}
    marks = {f: np.ascontiguousarray(v, dtype=np.float64) for f, v in case.marks.items()}
    na = (_dp * abi.NF_N)(*[_ptr(nodes[f]) if f in nodes else None for f in range(abi.NF_N)])
    ma = (_dp * abi.MF_N)(*[_ptr(marks[f]) if f in marks else None for f in range(abi.MF_N)])
    bondm = np.ascontiguousarray(case.bondm, dtype=np.int64)
    bondn = np.ascontiguousarray(case.bondn, dtype=np.int64)
    bondv = np.ascontiguousarray(case.bondv, dtype=np.float64)
    gx = np.ascontiguousarray(case.gx, dtype=np.float64)
    gy = np.ascontiguousarray(case.gy, dtype=np.float64)
    markt = np.ascontiguousarray(case.markt, dtype=np.int8)
    call("v2c_prn_write", str(path).encode(), ctypes.byref(h), _ptr(rt), _ptr(ex), na,
         _ptr(bondm, _lp), _ptr(gx), _ptr(gy), _ptr(bondv), _ptr(bondn, _lp), ma,
         markt.ctypes.data_as(ctypes.POINTER(ctypes.c_byte)))


def to_case(d: dict, base=None, name: str = "prn") -> synth.Case:
    """A synth.Case from a read() result: the file's grid, rocks, boundary
    equations, markers and node fields; parameters from `base` (a params
    dict, synth.default_params() when None) with the file's sizes, timestep
    and timesum.  Node fields the file does not hold are zero (the MIC step
    recomputes them)."""
    info = d["info"]
    xn, yn = info.xnumx, info.ynumy
    p = dict(synth.default_params() if base is None else base)
    p.update(xnumx=xn, ynumy=yn, xsize=info.xsize, ysize=info.ysize,
             xstpx=info.xsize / (xn - 1), ystpy=info.ysize / (yn - 1),
             timestep=info.timestep, timesum=info.timesum)
    nn = xn * yn
    nodes = {f: np.zeros(nn) for f in range(abi.NF_N)}
    nodes.update({f: v.copy() for f, v in d["nodes"].items()})
    marks = {f: np.zeros(info.marknum) for f in range(abi.MF_N)}
    marks.update({f: v.copy() for f, v in d["marks"].items()})
    nb = info.bondnum
    return synth.Case(name, p, d["gx"].copy(), d["gy"].copy(), d["rt"].copy(), nodes, marks,
                      d["markt"].copy(), d["bondm"].copy(), d["bondn"][:3 * nb].copy(),
                      d["bondv"][:4 * nb].copy())
