"""ctypes binding of libv2c.so (the CUDA implementation behind include/v2c.h).

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libv2c.so")
_LIB = None

P = ctypes.POINTER
c_dp = P(ctypes.c_double)
c_fp = P(ctypes.c_float)
c_ctx = ctypes.c_void_p


class V2CError(RuntimeError):
    def __init__(self, fn: str, code: int):
        names = {v: k for k, v in vars(abi).items() if k.startswith("ERR_") or k == "OK"}
        super().__init__(f"{fn} failed: {names.get(code, code)} ({code})")
        self.code = code


_SIGS = {
    "v2c_create": [P(abi.Params), ctypes.c_long, ctypes.c_void_p, P(ctypes.c_void_p)],
    "v2c_destroy": [c_ctx],
    "v2c_set_params": [c_ctx, P(abi.Params)],
    "v2c_set_grid": [c_ctx, c_dp, c_dp],
    "v2c_set_rock_table": [c_ctx, c_dp],
    "v2c_set_bonds": [c_ctx, P(ctypes.c_long), P(ctypes.c_long), c_dp, ctypes.c_long],
    "v2c_upload_markers": [c_ctx, P(c_dp), P(ctypes.c_byte), ctypes.c_long],
    "v2c_download_markers": [c_ctx, P(c_dp), P(ctypes.c_byte), ctypes.c_long],
    "v2c_download_cells": [c_ctx, P(ctypes.c_int32), ctypes.c_long],
    "v2c_download_marker_properties": [c_ctx, c_dp, c_dp, ctypes.c_long],
    "v2c_upload_node_field": [c_ctx, ctypes.c_int, c_dp],
    "v2c_download_node_field": [c_ctx, ctypes.c_int, c_dp],
    "v2c_interpolate_basic2center": [c_ctx],
    "v2c_interpolate_center2basic": [c_ctx, ctypes.c_double],
    "v2c_recompute_stress_strainrate": [c_ctx, ctypes.c_double],
    "v2c_copyarrays": [c_ctx],
    "v2c_marker_temperature": [c_ctx, ctypes.c_double],
    "v2c_stokes_assemble": [c_ctx, P(abi.StokesCtl), ctypes.c_long, P(ctypes.c_int),
                            P(ctypes.c_int), c_dp, c_dp, P(ctypes.c_long)],
    "v2c_prn_read_info": [ctypes.c_char_p, P(abi.PrnInfo)],
    "v2c_prn_read": [ctypes.c_char_p, P(abi.PrnInfo), c_dp, c_dp, P(c_dp), P(ctypes.c_long),
                     c_dp, c_dp, c_dp, P(ctypes.c_long), P(c_dp), P(ctypes.c_byte)],
    "v2c_prn_write": [ctypes.c_char_p, P(abi.PrnInfo), c_dp, c_dp, P(c_dp), P(ctypes.c_long),
                      c_dp, c_dp, c_dp, P(ctypes.c_long), P(c_dp), P(ctypes.c_byte)],
    "v2c_cycle_set_velocity": [c_ctx, ctypes.c_int, c_dp, c_dp],
    "v2c_cycle_step": [c_ctx, ctypes.c_int, ctypes.c_double, ctypes.c_int],
    "v2c_cycle_slip": [c_ctx, c_dp],
    "v2c_cycle_marker_slip": [c_ctx, c_dp, ctypes.c_long],
    "v2c_upload_node_fields": [c_ctx, ctypes.c_int, P(ctypes.c_int), P(c_dp)],
    "v2c_download_node_fields": [c_ctx, ctypes.c_int, P(ctypes.c_int), P(c_dp)],
    "v2c_download_node_fields_async": [c_ctx, ctypes.c_int, P(ctypes.c_int), P(c_dp)],
    "v2c_wait_downloads": [c_ctx],
    "v2c_marker2nodes": [c_ctx],
    "v2c_center2basic_old": [c_ctx],
    "v2c_compute_before_solve": [c_ctx, ctypes.c_double, ctypes.c_int],
    "v2c_compute_after_solve": [c_ctx, ctypes.c_double, ctypes.c_int, c_dp],
    "v2c_nodes2markers": [c_ctx],
    "v2c_moveandrotatemarkers": [c_ctx],
    "v2c_nodes2markers_move": [c_ctx],
    "v2c_synchronize": [c_ctx],
    "v2c_get_status": [c_ctx, P(abi.Status)],
    "v2c_set_profiling": [c_ctx, ctypes.c_int],
    "v2c_get_profile": [c_ctx, ctypes.c_int, c_dp, P(ctypes.c_long)],
    "v2c_rsf_newton": [c_ctx, ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_void_p,
                       ctypes.c_void_p],
    "v2c_collect_newton_states": [c_ctx, ctypes.c_long, ctypes.c_void_p, ctypes.c_long,
                                  P(ctypes.c_long)],
    "v2c_mlp_load": [c_ctx, c_fp],
    "v2c_mlp_save": [c_ctx, c_fp],
    "v2c_mlp_train": [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_int,
                      ctypes.c_int, ctypes.c_float, ctypes.c_uint64, c_fp],
    "v2c_mlp_grad": [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, c_fp, c_fp],
    "v2c_mlp_infer": [c_ctx, ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p],
    "v2c_calc_timestep": [c_ctx, ctypes.c_int, P(abi.TimestepCtl), P(abi.TimestepInfo)],
    "v2c_sort_cells_static": [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p, ctypes.c_long,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
}


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run velo2cycles_gb300.build.build() "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _LIB = L
    return _LIB


def call(name: str, *args) -> None:
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise V2CError(name, rc)
