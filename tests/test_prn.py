"""The restart file (.prn) reader and writer (velo2cycles_gb300.prn over
v2c_prn_*), pinned against the reference's own save_model
(load_save.c:353-527 with input_RSF.c:106-132):

  * the committed fixture tests/golden/ref_micro.npz holds the file the
    reference wrote after one step of the micro case; the reader must return
    the reference's state after that step bit for bit, and the writer,
    given that state, must reproduce the file byte for byte;
  * where the reference routines are built, the same on a freshly written
    file of the tiny case;
  * a reference-written state drives the GPU step (GPU test).
"""
import json
import os

import numpy as np
import pytest

from oracle import bindings as B
from velo2cycles_gb300 import abi, prn, synth
from velo2cycles_gb300._lib import V2CError

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_micro.npz")

# the marker and node fields a restart file holds
MARK_FIELDS = (abi.MF_X, abi.MF_Y, abi.MF_K, abi.MF_E, abi.MF_XX, abi.MF_V, abi.MF_XY, abi.MF_P,
               abi.MF_EXX, abi.MF_EXY, abi.MF_D, abi.MF_W, abi.MF_VX, abi.MF_VY, abi.MF_PHI,
               abi.MF_L, abi.MF_L0, abi.MF_C, abi.MF_C0)
NODE_FIELDS = (abi.NF_SXXEE, abi.NF_SXX, abi.NF_EXXEE, abi.NF_EXX, abi.NF_SXYEE, abi.NF_SXY,
               abi.NF_EXYEE, abi.NF_EXY, abi.NF_SPPEE, abi.NF_PR, abi.NF_PHIE, abi.NF_PHIS_IT,
               abi.NF_MVXE, abi.NF_VX, abi.NF_MVYE, abi.NF_VY, abi.NF_PES, abi.NF_PEE,
               abi.NF_RK_SLIPRS_FINAL, abi.NF_RK_PHIDTS_FINAL)
RT_ROWS = (abi.RT_IM, abi.RT_N0, abi.RT_N1, abi.RT_NU, abi.RT_DH, abi.RT_DV, abi.RT_SS, abi.RT_MM,
           abi.RT_GG, abi.RT_RO, abi.RT_BB, abi.RT_AA, abi.RT_CP, abi.RT_KT, abi.RT_KF, abi.RT_KP,
           abi.RT_HT)

needs_ref = pytest.mark.skipif(not B.reference_available(),
                               reason="reference routines not built")


def _golden_case(z, out=True):
    """The micro case of the fixture, with the state after the step when
    `out` (what the reference saved)."""
    params = json.loads(str(z["default/params"]))
    nodes = z["default/nodes_out" if out else "default/nodes_in"]
    marks = z["default/marks_out" if out else "default/marks_in"]
    return synth.Case("golden", params, z["default/gx"], z["default/gy"], z["default/rt"],
                      {k: nodes[k].copy() for k in range(abi.NF_N)},
                      {k: marks[k].copy() for k in range(abi.MF_N)}, z["default/markt"].copy(),
                      z["default/bondm"], z["default/bondn"], z["default/bondv"])


def _check_read(got, case, cycle):
    info = got["info"]
    assert (info.xnumx, info.ynumy, info.marknum) == (case.gx.size, case.gy.size, case.n)
    assert info.bondnum == case.bondnum and info.cycle == cycle
    assert info.rocknum == abi.MAXTMR
    for f in MARK_FIELDS:
        assert np.array_equal(got["marks"][f], case.marks[f]), abi.marker_field_names()[f]
    for f in NODE_FIELDS:
        assert np.array_equal(got["nodes"][f], case.nodes[f]), abi.node_field_names()[f]
    assert np.array_equal(got["markt"], case.markt)
    assert np.array_equal(got["bondm"], case.bondm)
    nb = case.bondnum
    # bond equation 0 is the reference's "no equation" row and is not saved
    assert np.array_equal(got["bondn"][3:3 * nb], case.bondn[3:3 * nb])
    assert np.array_equal(got["bondv"][4:4 * nb], case.bondv[4:4 * nb])
    assert np.array_equal(got["gx"], case.gx) and np.array_equal(got["gy"], case.gy)
    for r in RT_ROWS:
        assert np.array_equal(got["rt"][r], case.rt[r]), r


def _write_bytes(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(bytes(data))
    return str(p)


def test_golden_restart_read_and_write(tmp_path, built_lib):
    z = np.load(GOLDEN)
    ref_bytes = z["default/prn"].tobytes()
    case = _golden_case(z)
    got = prn.read(_write_bytes(tmp_path, "ref.prn", ref_bytes))
    _check_read(got, case, cycle=1)
    out = str(tmp_path / "ours.prn")
    prn.write(out, case, info=got["info"], rock_extra=got["rock_extra"])
    assert open(out, "rb").read() == ref_bytes


def test_roundtrip_synthetic(tmp_path, built_lib):
    c = synth.make_case("tiny", seed=11)
    c.marks[abi.MF_PHI][:] = np.linspace(-1, 1, c.n)
    c.nodes[abi.NF_RK_PHIDTS_FINAL][:] = np.arange(c.nodenum) * 0.5
    p = str(tmp_path / "a.prn")
    prn.write(p, c)
    got = prn.read(p)
    _check_read(got, c, cycle=0)
    # a state read back drives the same case
    back = prn.to_case(got, base=c.params)
    for f in MARK_FIELDS:
        assert np.array_equal(back.marks[f], c.marks[f])
    assert back.params["xstpx"] == c.params["xsize"] / (c.gx.size - 1)


def test_header_checks(tmp_path, built_lib):
    c = synth.make_case("tiny", seed=3)
    p = str(tmp_path / "a.prn")
    prn.write(p, c)
    data = open(p, "rb").read()
    # another int/long/float/double size
    bad = bytearray(data)
    bad[1] = 4
    with pytest.raises(V2CError) as e:
        prn.read_info(_write_bytes(tmp_path, "sz.prn", bad))
    assert e.value.code == abi.ERR_UNSUPPORTED
    # truncated body
    with pytest.raises(V2CError) as e:
        prn.read(_write_bytes(tmp_path, "short.prn", data[:-7]))
    assert e.value.code == abi.ERR_ARG
    # trailing bytes: a file with other per-marker or per-node extras
    with pytest.raises(V2CError) as e:
        prn.read(_write_bytes(tmp_path, "long.prn", data + b"\0" * 8))
    assert e.value.code == abi.ERR_UNSUPPORTED
    # a missing file
    with pytest.raises(V2CError) as e:
        prn.read_info(str(tmp_path / "missing.prn"))
    assert e.value.code == abi.ERR_ARG


@needs_ref
def test_reference_written_file(tmp_path, built_lib):
    """The reference's save_model on the tiny case (no step: the state as
    loaded) against the reader and the writer."""
    c = synth.make_case("tiny", seed=5)
    ref_bytes = B.run_reference(c, stages=B.SAVE_STAGE)["prn"]
    got = prn.read(_write_bytes(tmp_path, "ref.prn", ref_bytes))
    _check_read(got, c, cycle=1)
    out = str(tmp_path / "ours.prn")
    prn.write(out, c, info=got["info"], rock_extra=got["rock_extra"])
    assert open(out, "rb").read() == ref_bytes


@pytest.mark.gpu
def test_reference_restart_drives_gpu_step(tmp_path, built_lib, oracle_built):
    """The state the reference saved after its step, loaded from the file,
    runs the GPU marker2nodes + nodes2markers pass like the oracle does on
    the same state (tolerances of the MIC parity tests)."""
    from velo2cycles_gb300 import mic
    from .parity import M2N_OUT, node_errors, oracle_for, over

    z = np.load(GOLDEN)
    got = prn.read(_write_bytes(tmp_path, "ref.prn", z["default/prn"].tobytes()))
    base = json.loads(str(z["default/params"]))
    case = prn.to_case(got, base=base)
    # node fields the step reads but the file does not hold (temperature,
    # properties) come from the state after the step
    nodes_out = z["default/nodes_out"]
    for f in range(abi.NF_N):
        if f not in NODE_FIELDS:
            case.nodes[f] = nodes_out[f].copy()
    m = mic.from_case(case)
    m.marker2nodes()
    out = m.download_nodes(M2N_OUT)
    ref = oracle_for(case)
    ref.marker2nodes()
    bad = over(node_errors(out, ref.nodes, M2N_OUT))
    assert not bad, bad
    m.close()
