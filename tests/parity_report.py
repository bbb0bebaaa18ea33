"""Per-field parity report of one full MIC step on the GPU against the oracle
(the numbers of the precision table).

    python tests/parity_report.py [c1|c2|...] [seed] > report.json

For each stage -- marker2nodes, interpolate_center2basic_old +
compute_before_solve + compute_after_solve, nodes2markers,
moveandrotatemarkers -- every field the stage writes, with the per-entry
error of parity.rel_err (relative; for fields that cross zero, against the
field's RMS or, for marker fields the gather interpolates, the magnitude of
the node values they come from; slip rates through ln V), measured against
the FP64 oracle on the state the device holds, plus the per-marker
viscosity and conductivity of marker2nodes.  Needs a GPU.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from tests.parity import (C2B_OUT, M2N_OUT, MOVE_MARK, N2M_MARK, N2M_OUT, RSF_OUT,  # noqa: E402
                          marker_errors, n2m_floors, node_errors, nxsearch_np, oracle_for,
                          rotated_floors)
from velo2cycles_gb300 import abi, mic, synth  # noqa: E402


def report(name: str, seed: int = 7) -> dict:
    c = synth.make_case(name, seed=seed)
    dt = c.params["timestep"]
    m = mic.from_case(c)
    ref = oracle_for(c, nthreads=os.cpu_count() or 1)
    out = {"case": name, "markers": c.n, "nodes": c.nodenum}
    cells = m.download_cells()
    ix, iy = nxsearch_np(c.gx, c.marks[abi.MF_X]), nxsearch_np(c.gy, c.marks[abi.MF_Y])
    out["cells_bit_exact"] = bool(np.array_equal(cells, (ix * (c.gy.size - 1) + iy)
                                                 .astype(np.int32)))
    m.marker2nodes(); ref.marker2nodes()
    nu, kt = m.download_marker_properties()
    nu_r, kt_r, _ = ref.marker_properties()
    ins = nu_r > 0
    out["marker_properties"] = {"viscosity": float(np.abs(nu[ins] / nu_r[ins] - 1).max()),
                                "conductivity": float(np.abs(kt[ins] / kt_r[ins] - 1).max())}
    out["marker2nodes"] = node_errors(m.download_nodes(M2N_OUT), ref.nodes, M2N_OUT)
    m.interpolate_center2basic_old(); ref.center2basic_old()
    m.compute_before_solve(dt, 0); ref.compute_before_solve(dt, 0)
    m.compute_after_solve(dt, 0); ref.compute_after_solve(dt, 0)
    f = C2B_OUT + RSF_OUT
    out["node_rsf"] = node_errors(m.download_nodes(f), ref.nodes, f)
    fl = n2m_floors(ref)
    m.nodes2markers(); ref.nodes2markers()
    out["nodes2markers_nodes"] = node_errors(m.download_nodes(N2M_OUT), ref.nodes, N2M_OUT)
    out["nodes2markers_markers"] = marker_errors(m.download_markers(N2M_MARK), ref.marks,
                                                 N2M_MARK, fl)
    m.moveandrotatemarkers(); ref.move()
    mk = m.download_markers(MOVE_MARK)
    fields = [k for k in MOVE_MARK if k not in (abi.MF_X, abi.MF_Y)]
    out["move_markers"] = marker_errors(mk, ref.marks, fields, rotated_floors(fl))
    pos = {}
    for k, g, nm in ((abi.MF_X, c.gx, "x"), (abi.MF_Y, c.gy, "y")):
        w = np.diff(g)[nxsearch_np(g, ref.marks[k])]
        pos[nm] = float((np.abs(mk[k] - ref.marks[k]) / w).max())
    out["move_positions_cell_widths"] = pos
    m.close()
    return out


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "c1"
    seed = int(sys.argv[2]) if len(sys.argv) > 2 else 7
    print(json.dumps(report(name, seed), indent=1))
