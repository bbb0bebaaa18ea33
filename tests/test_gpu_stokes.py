"""The Stokes matrix assembly on the device (v2c_stokes_assemble) against
the restatement (GPU): preparematrix + gausmat4_add
(momentum_continuity_addmatrix_checkerror.c:22-213, gausevps.c:137-214) on
the same node values — the device's FP32 node fields, given to the
restatement as FP64 — must give the same CSR arrays bit for bit (FP64 in
the reference's order, no multiply-add contraction on either side)."""
import ctypes

import numpy as np
import pytest

import oracle
from velo2cycles_gb300 import abi, mic
from velo2cycles_gb300._lib import V2CError, call

from .parity import stokes_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tiny", "small"])
@pytest.mark.parametrize("variant", ["default", "no_sailor", "inertia", "compressible",
                                     "cont_bond"])
def test_stokes_assembly_bit_exact(name, variant, built_lib, oracle_built):
    c, ctl = stokes_case(5, name=name, variant=variant)
    m = mic.from_case(c)
    got = m.stokes_assemble(**ctl)
    rc, ref = oracle.Restatement(c.copy()).stokes_assemble(**ctl)
    assert rc == 0
    for k in ("ia", "ja", "a", "b"):
        assert np.array_equal(got[k], ref[k], equal_nan=k in ("a", "b")), k
    m.close()


def test_stokes_assembly_count_capacity_and_refusal(built_lib, oracle_built):
    c, ctl = stokes_case(5)
    m = mic.from_case(c)
    sc = abi.StokesCtl(**ctl)
    nnz = ctypes.c_long(0)
    call("v2c_stokes_assemble", m.h, ctypes.byref(sc), 0, None, None, None, None,
         ctypes.byref(nnz))
    rc, ref = oracle.Restatement(c.copy()).stokes_assemble(**ctl)
    assert nnz.value == ref["ja"].size
    # too small a capacity: refused, with the needed count
    P = ctypes.POINTER
    ja = np.zeros(nnz.value, dtype=np.int32)
    a = np.zeros(nnz.value)
    with pytest.raises(V2CError) as e:
        call("v2c_stokes_assemble", m.h, ctypes.byref(sc), nnz.value - 1, None,
             ja.ctypes.data_as(P(ctypes.c_int)), a.ctypes.data_as(P(ctypes.c_double)), None,
             ctypes.byref(nnz))
    assert e.value.code == abi.ERR_CAPACITY
    assert nnz.value == ref["ja"].size
    m.close()
    # an edge node without a boundary equation: refused like the restatement
    c2, ctl2 = stokes_case(5, variant="open_edge")
    m2 = mic.from_case(c2)
    with pytest.raises(V2CError) as e:
        m2.stokes_assemble(**ctl2)
    assert e.value.code == abi.ERR_UNSUPPORTED
    m2.close()
