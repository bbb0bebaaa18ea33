"""The allocation-free cell sort v2c_sort_cells_static (collected last).

Checked against the context path on the same markers: the cells of
v2c_download_cells (bit-exact) and the context's stable counting sort by
cell (cells in order, markers of a cell in ascending index; the largest cell
count against the context's max_cell_count).  Integer results, so the
tolerance is zero.  Two calls in a row on different marker sets check that
the fixed scratch carries nothing from one call to the next.
"""
import numpy as np
import pytest

from velo2cycles_gb300 import abi, cellsort, mic, synth
from velo2cycles_gb300._lib import V2CError


def test_oversize_grid_rejected_before_any_device_work(built_lib):
    from velo2cycles_gb300._lib import lib
    xn = 5001
    yn = abi.STATIC_SORT_MAX_CELLS // (xn - 1) + 2
    assert (xn - 1) * (yn - 1) > abi.STATIC_SORT_MAX_CELLS
    rc = lib().v2c_sort_cells_static(None, xn, None, yn, None, None, 0, None, None, None, None)
    assert rc == abi.ERR_CAPACITY
    assert lib().v2c_sort_cells_static(None, 4001, None, 1001, None, None, 0, None, None, None,
                                       None) == abi.ERR_ARG  # fits; fails only on the pointers


def test_huge_line_counts_rejected_without_overflow(built_lib):
    """Line counts whose cell product would overflow 64 bits, or whose
    factors exceed an int, are refused as over capacity before any product
    is formed."""
    from velo2cycles_gb300._lib import lib
    big = 1 << 40
    assert lib().v2c_sort_cells_static(None, big, None, big, None, None, 0, None, None, None,
                                       None) == abi.ERR_CAPACITY
    assert lib().v2c_sort_cells_static(None, 3, None, (1 << 62), None, None, 0, None, None, None,
                                       None) == abi.ERR_CAPACITY


def test_wrapper_rejects_host_tensors(built_lib):
    """Host (CPU) tensors never reach the library: the kernels would be
    handed host addresses."""
    torch = pytest.importorskip("torch")
    g = torch.linspace(0, 1, 5, dtype=torch.float64)
    x = torch.zeros(3, dtype=torch.float64)
    i3 = torch.zeros(3, dtype=torch.int32)
    start = torch.zeros(17, dtype=torch.int32)
    with pytest.raises(ValueError, match="CUDA device"):
        cellsort.sort_cells_static(g, g, x, x, i3, i3.clone(), start)


def _expected(case):
    """cells, start, perm and max cell count from the context path."""
    m = mic.from_case(case)
    cells = m.download_cells()
    mx = m.status()["max_cell_count"]
    m.close()
    ncell = (case.gx.size - 1) * (case.gy.size - 1)
    start = np.zeros(ncell + 1, np.int64)
    start[1:] = np.cumsum(np.bincount(cells, minlength=ncell))
    return cells, start.astype(np.int32), np.argsort(cells, kind="stable").astype(np.int32), mx


def _static(case):
    import torch
    dev = torch.device("cuda:0")
    f64 = dict(dtype=torch.float64, device=dev)
    gx, gy = torch.tensor(case.gx, **f64), torch.tensor(case.gy, **f64)
    x = torch.tensor(case.marks[abi.MF_X], **f64)
    y = torch.tensor(case.marks[abi.MF_Y], **f64)
    n, ncell = x.numel(), (gx.numel() - 1) * (gy.numel() - 1)
    # outputs start as garbage on purpose: the call needs no initial value
    cell = torch.full((n,), -7, dtype=torch.int32, device=dev)
    perm = torch.full((n,), -7, dtype=torch.int32, device=dev)
    start = torch.full((ncell + 1,), -7, dtype=torch.int32, device=dev)
    cellsort.sort_cells_static(gx, gy, x, y, cell, perm, start)
    torch.cuda.synchronize()
    return cell.cpu().numpy(), start.cpu().numpy(), perm.cpu().numpy()


def _case(name, seed, crowd):
    c = synth.make_case(name, seed=seed)
    x, y = c.marks[abi.MF_X], c.marks[abi.MF_Y]
    x[:7], x[7:14] = -3.0, c.gx[-1] + 5.0          # outside the grid (clamped cells)
    y[20:30] = c.gy[2]                               # on grid lines: ties go left
    x[40:50] = c.gx[9]
    # crowd one cell so it holds more than 32 markers (the in-place
    # network path of the ordering, not only the register path)
    x[100:100 + crowd] = 0.5 * (c.gx[3] + c.gx[4])
    y[100:100 + crowd] = 0.5 * (c.gy[5] + c.gy[6])
    return c


@pytest.mark.gpu
def test_two_calls_in_a_row_match_the_context_path(built_lib):
    cases = [_case("small", 11, 300), _case("tiny", 12, 45)]
    exp = [_expected(c) for c in cases]
    got = [_static(c) for c in cases]                 # two calls back to back
    for (cells, start, perm, mx), (gc, gs, gp) in zip(exp, got):
        assert np.array_equal(gc, cells)
        assert np.array_equal(gs, start)
        assert np.array_equal(gp, perm)
        assert int(np.diff(gs).max()) == mx
    assert int(np.diff(got[0][1]).max()) > 32 and int(np.diff(got[1][1]).max()) > 32
    # the same input again after a different one gives the same answer
    again = _static(cases[0])
    assert all(np.array_equal(a, b) for a, b in zip(again, got[0]))


@pytest.mark.gpu
def test_oversize_grid_raises_through_the_wrapper(built_lib):
    import torch
    dev = torch.device("cuda:0")
    gx = torch.linspace(0, 1, 5001, dtype=torch.float64, device=dev)
    gy = torch.linspace(0, 1, 1001, dtype=torch.float64, device=dev)
    x = torch.zeros(4, dtype=torch.float64, device=dev)
    i4 = torch.zeros(4, dtype=torch.int32, device=dev)
    start = torch.zeros(5000 * 1000 + 1, dtype=torch.int32, device=dev)
    with pytest.raises(V2CError) as e:
        cellsort.sort_cells_static(gx, gy, x, x, i4, i4.clone(), start)
    assert e.value.code == abi.ERR_CAPACITY
