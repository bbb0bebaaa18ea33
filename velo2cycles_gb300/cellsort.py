"""Allocation-free cell assignment + stable counting sort by cell
(v2c_sort_cells_static of include/v2c.h; no counterpart in the reference).

The library call allocates nothing: its scratch is a fixed per-device array
of V2C_STATIC_SORT_MAX_CELLS counters, and it orders each cell's segment of
the caller's output in place.  Calls that overlap on one device race on that
scratch.  This wrapper takes caller-owned torch device tensors (plumbing
only) and queues the work on the current torch stream.
"""
from __future__ import annotations

import ctypes

from . import abi
from ._lib import call

MAX_CELLS = abi.STATIC_SORT_MAX_CELLS


def sort_cells_static(gx, gy, x, y, cell, perm, start) -> None:
    """gx[xnumx], gy[ynumy], x[n], y[n]: float64 device tensors;
    cell[n], perm[n], start[(xnumx-1)*(ynumy-1)+1]: int32 device tensors
    (written).  Raises V2CError(V2C_ERR_CAPACITY) for grids of more than
    MAX_CELLS cells."""
    import torch
    n = x.numel()
    ncell = (gx.numel() - 1) * (gy.numel() - 1)
    tensors = ((gx, torch.float64, None), (gy, torch.float64, None), (x, torch.float64, n),
               (y, torch.float64, n), (cell, torch.int32, n), (perm, torch.int32, n),
               (start, torch.int32, ncell + 1))
    for t, dt, k in tensors:
        # the kernels run on one device and take its pointers only: a host
        # tensor or one on another device would hand them foreign addresses
        if not t.is_cuda or t.device != x.device:
            raise ValueError("sort_cells_static: every tensor must be on the CUDA device of x")
        if t.dtype != dt or not t.is_contiguous() or (k is not None and t.numel() != k):
            raise ValueError("sort_cells_static: bad tensor dtype, layout or size")
    # the library looks up its scratch on the current device and launches
    # there: make that the tensors' device, with its current stream
    with torch.cuda.device(x.device):
        stream = torch.cuda.current_stream(x.device).cuda_stream
        call("v2c_sort_cells_static", ctypes.c_void_p(gx.data_ptr()), gx.numel(),
             ctypes.c_void_p(gy.data_ptr()), gy.numel(), ctypes.c_void_p(x.data_ptr()),
             ctypes.c_void_p(y.data_ptr()), n, ctypes.c_void_p(cell.data_ptr()),
             ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(start.data_ptr()),
             ctypes.c_void_p(stream))
