"""Constants and the parameter struct of the C ABI, read from include/v2c.h.

The header is the single source of truth: the enumerations (field ids,
rock-table rows, status codes) and the ``v2c_params`` layout are parsed from
it at import time, so Python never carries a second copy.
"""
from __future__ import annotations

import ctypes
import os
import re

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "v2c.h")


def _strip_comments(s: str) -> str:
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


with open(HEADER) as _f:
    _SRC = _strip_comments(_f.read())

_CONST: dict[str, int] = {}
for _m in re.finditer(r"#define\s+(V2C_\w+)\s+([0-9 ()*+\-]+?)\s*$", _SRC, flags=re.M):
    _CONST[_m.group(1)] = int(eval(_m.group(2), {}, {}))
for _body in re.findall(r"enum\s*\{(.*?)\}\s*;", _SRC, flags=re.S):
    _val = -1
    for _item in _body.split(","):
        _item = _item.strip()
        if not _item:
            continue
        if "=" in _item:
            _name, _expr = (t.strip() for t in _item.split("=", 1))
            _val = int(eval(_expr, {}, dict(_CONST)))
        else:
            _name, _val = _item, _val + 1
        _CONST[_name] = _val

for _k, _v in _CONST.items():
    globals()[_k[4:] if _k.startswith("V2C_") else _k] = _v

_CT = {"long": ctypes.c_long, "double": ctypes.c_double, "int": ctypes.c_int}


def _struct_fields(name: str) -> list:
    """(field, ctype) list of `typedef struct name { ... } name;`"""
    m = re.search(r"typedef\s+struct\s+" + name + r"\s*\{(.*?)\}\s*" + name + r"\s*;", _SRC,
                  flags=re.S)
    out = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, names = decl.split(None, 1)
        for nm in names.split(","):
            nm = nm.strip()
            a = re.match(r"(\w+)\[(\d+)\]$", nm)
            out.append((a.group(1), _CT[typ] * int(a.group(2))) if a else (nm, _CT[typ]))
    return out


# v2c_params
_FIELDS = _struct_fields("v2c_params")


class Params(ctypes.Structure):
    _fields_ = _FIELDS

    @classmethod
    def from_dict(cls, d: dict) -> "Params":
        p = cls()
        for name, _ in _FIELDS:
            if name in d:
                setattr(p, name, d[name])
        return p

    def to_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in _FIELDS}


PARAM_NAMES = [n for n, _ in _FIELDS]


class Status(ctypes.Structure):
    _fields_ = [
        ("n_markers", ctypes.c_long), ("n_out_of_grid", ctypes.c_long),
        ("n_far_moves", ctypes.c_long), ("n_nan", ctypes.c_long),
        ("newton_iters", ctypes.c_long), ("newton_fallbacks", ctypes.c_long),
        ("newton_nonconv", ctypes.c_long), ("newton_max_res", ctypes.c_double),
        ("max_cell_count", ctypes.c_long), ("kernel_launches", ctypes.c_long),
        ("last_error", ctypes.c_int),
    ]


def node_field_names() -> dict[int, str]:
    return {v: k[7:].lower() for k, v in _CONST.items() if k.startswith("V2C_NF_") and k != "V2C_NF_N"}


def marker_field_names() -> dict[int, str]:
    return {v: k[7:].lower() for k, v in _CONST.items() if k.startswith("V2C_MF_") and k != "V2C_MF_N"}


def declared_functions() -> list[str]:
    """Names of every function declared in include/*.h."""
    inc = os.path.dirname(HEADER)
    names = []
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            with open(os.path.join(inc, fn)) as f:
                src = _strip_comments(f.read())
            names += re.findall(r"^\s*(?:int|double|void|long)\s+\**\s*(\w+)\s*\(", src, flags=re.M)
    return names


class TimestepCtl(ctypes.Structure):
    _fields_ = _struct_fields("v2c_timestep_ctl")


class TimestepInfo(ctypes.Structure):
    _fields_ = _struct_fields("v2c_timestep_info")

    def to_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class StokesCtl(ctypes.Structure):
    """v2c_stokes_ctl: the scalars of preparematrix that are not parameters."""
    _fields_ = _struct_fields("v2c_stokes_ctl")


# the reference's values: drunkensailor = 1 (headevps.c:288); mukoef = dt*30e5
# (momentum_continuity_iterate.c:64) is set per call
STOKES_DEFAULTS = dict(gxkoef=0.0, gykoef=9.81, timebond=0.0, drunkensailor=1)


class PrnInfo(ctypes.Structure):
    """v2c_prn_info: the header of a restart file."""
    _fields_ = _struct_fields("v2c_prn_info")


# reference defaults (input_RSF.c:17-20); maxtmstep comes from the model file
TIMESTEP_DEFAULTS = dict(maxtmstep=1e10, dtfactor=1.0, tcnvp=0.2, tcd=1e-3, tcphih=0.2)
