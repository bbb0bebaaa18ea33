"""The reference-side binding (velo2cycles_gb300/bind/v2c_bind.c) against the
reference itself (GPU).

tests/bind_check.c is compiled with the reference sources staged by
oracle/build_ref.sh and the binding, and runs one MIC step twice from the
same globals: with the reference's own routines and through the binding.
Both runs start from the state as the device holds it (parity.device_view),
so the comparison measures the device's arithmetic; tolerances are those of
the parity tests (1e-6 per entry, parity.rel_err; positions 3e-7 of a
cell).  The reference
processes one marker past the end (m3 <= marknum, interpolation.c:1053),
which adds to the raw back-scatter sums at node 0; node 0 is left out of
those sums.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from oracle import bindings as B
from velo2cycles_gb300 import abi, build, synth

from .parity import (B2C_C2B_OUT, C2B_OUT, M2N_OUT, N2M_OUT, RSF_OUT, device_view,
                     marker_err, node_err, nxsearch_np, rel_err, tolerance)

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "oracle", "_ref", "src")
RAW_SUMS = {abi.NF_PHISUM, abi.NF_WTPHISUM, abi.NF_SXYSUM, abi.NF_EXYSUM, abi.NF_ESUM,
            abi.NF_PSUM, abi.NF_SXXSUM, abi.NF_EXXSUM, abi.NF_WTSXXSUM, abi.NF_VXSUM,
            abi.NF_VYSUM, abi.NF_WTVXSUM, abi.NF_WTVYSUM, abi.NF_MRX0, abi.NF_MRY0}


@pytest.fixture(scope="module")
def bind_check(tmp_path_factory, built_lib):
    if not os.path.exists(os.path.join(SRC, "headevps.c")):
        pytest.skip("reference sources not staged (oracle/build_ref.sh)")
    d = tmp_path_factory.mktemp("bind")
    exe = str(d / "bind_check")
    libdir = os.path.dirname(build.LIB)
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-fopenmp", "-fcommon", "-w", "-ffp-contract=off",
                    *(["-mcmodel=medium"] if os.uname().machine == "x86_64" else []),
                    "-I", SRC, "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "velo2cycles_gb300", "bind"),
                    "-o", exe, os.path.join(ROOT, "tests", "bind_check.c"),
                    "-L", libdir, "-lv2c", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    return exe, d


def test_binding_step_matches_reference(bind_check):
    exe, d = bind_check
    c = device_view(synth.make_case("small", seed=17))
    case, r_ref, r_bind = str(d / "case.bin"), str(d / "ref.bin"), str(d / "bind.bin")
    csr_ref, csr_bind = str(d / "ref.csr"), str(d / "bind.csr")
    dt = float(c.params["timestep"])
    B.write_case(case, c, stokes=dict(abi.STOKES_DEFAULTS, mukoef=dt * 30e5, dt=dt))
    subprocess.run([exe, case, r_ref, r_bind, csr_ref, csr_bind], check=True, timeout=600)
    # preparematrix through the binding: the same sparsity, coefficients
    # within the FP32 storage of the device's node fields
    sr, sb = B.read_csr(csr_ref), B.read_csr(csr_bind)
    assert np.array_equal(sb["ia"], sr["ia"]) and np.array_equal(sb["ja"], sr["ja"])
    row = np.repeat(np.arange(sr["ia"].size - 1), np.diff(sr["ia"]))
    scale = np.zeros(sr["ia"].size - 1)
    np.maximum.at(scale, row, np.abs(sr["a"]))
    assert (np.abs(sb["a"] - sr["a"]) <= 1e-6 * scale[row]).all()  # per row
    assert rel_err(sb["b"], sr["b"]) <= 1e-6
    ref = B.read_result(r_ref, c.nodenum)
    got = B.read_result(r_bind, c.nodenum)
    names = abi.node_field_names()
    bad = {}
    for f in M2N_OUT + C2B_OUT + B2C_C2B_OUT + RSF_OUT + N2M_OUT:
        a, b = got["nodes"][f].copy(), ref["nodes"][f].copy()
        if f in RAW_SUMS:
            a[0] = b[0] = 0.0
        e = node_err(f, a, b, ref["nodes"])
        if not e <= tolerance(names[f]):
            bad[names[f]] = e
    assert not bad, bad
    mnames = abi.marker_field_names()
    for f in (abi.MF_K, abi.MF_E, abi.MF_P, abi.MF_XX, abi.MF_XY, abi.MF_EXX, abi.MF_EXY,
              abi.MF_VX, abi.MF_VY, abi.MF_PHI):
        e = marker_err(f, got["marks"][f], ref["marks"][f])
        assert e <= 1e-6, (mnames[f], e)
    wx = np.diff(c.gx)[nxsearch_np(c.gx, ref["marks"][abi.MF_X])]
    assert (np.abs(got["marks"][abi.MF_X] - ref["marks"][abi.MF_X]) / wx).max() <= 3e-7
    assert abs(got["deltas"] - ref["deltas"]) <= 1e-5 * max(abs(ref["deltas"]), 1.0)
