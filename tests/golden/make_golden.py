"""Generate tests/golden/ref_micro.npz: inputs and outputs of the reference's
own routines (compiled from its sources by oracle/build_ref.sh) on two micro
cases, for pinning the oracle restatement where the reference is absent,
the restart file (.prn) the reference's save_model wrote after the step
on the first case, and the Stokes matrix its preparematrix assembled on
that case.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import bindings as B  # noqa: E402
from velo2cycles_gb300 import abi, synth  # noqa: E402

CASES = {
    "default": dict(),
    "variant": dict(interpolationmod=1, markmod=1, stoksmod=2, antidiffinter=0, Dphis=1.0),
}


def micro(seed, **kw):
    # an 8 x 7 window of the tiny grid keeps the file small
    return synth.make_case("tiny", seed=seed, window=(4, 2, 8, 7), **kw)


def main():
    B.build()
    assert B.reference_available(), "reference sources are needed to make the fixtures"
    out = {}
    for name, kw in CASES.items():
        c = micro(7, **kw)
        res = B.run_reference(c, stages=B.ALL_STAGES | B.SAVE_STAGE, nthreads=1)
        out[f"{name}/params"] = np.array(json.dumps(c.params, sort_keys=True))
        out[f"{name}/gx"], out[f"{name}/gy"], out[f"{name}/rt"] = c.gx, c.gy, c.rt
        out[f"{name}/nodes_in"] = np.stack([c.nodes[k] for k in range(abi.NF_N)])
        out[f"{name}/marks_in"] = np.stack([c.marks[k] for k in range(abi.MF_N)])
        out[f"{name}/markt"] = c.markt
        out[f"{name}/bondm"], out[f"{name}/bondn"], out[f"{name}/bondv"] = c.bondm, c.bondn, c.bondv
        out[f"{name}/nodes_out"] = np.stack([res["nodes"][k] for k in range(abi.NF_N)])
        out[f"{name}/marks_out"] = np.stack([res["marks"][k] for k in range(abi.MF_N)])
        if name == "default":
            out[f"{name}/prn"] = np.frombuffer(res["prn"], dtype=np.uint8)
    # the Stokes matrix the reference's preparematrix assembles on the first
    # case after marker2nodes, compute_before_solve and basic2center
    c = micro(7)
    dt = float(c.params["timestep"])
    ctl = dict(abi.STOKES_DEFAULTS, mukoef=dt * 30e5, dt=dt)
    res = B.run_reference(c, stages=(1 << 0) | (1 << 2) | (1 << 7) | B.STOKES_STAGE,
                          nthreads=1, stokes=ctl)["stokes"]
    out["stokes/ctl"] = np.array(json.dumps(ctl, sort_keys=True))
    for k in ("ia", "ja", "a", "b"):
        out[f"stokes/{k}"] = res[k]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_micro.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
