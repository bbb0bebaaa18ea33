"""The C-ABI library (CPU checks; no device calls)."""
import ctypes
import os
import subprocess
import tempfile

import pytest

from velo2cycles_gb300 import abi


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in abi.declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(abi.declared_functions()) >= 25


def test_params_and_status_layout_match_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "v2c.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(v2c_params), offsetof(v2c_params, newton_guess),
         sizeof(v2c_status), offsetof(v2c_status, last_error));
  return 0;
}
'''
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    with tempfile.TemporaryDirectory() as d:
        c, exe = os.path.join(d, "t.c"), os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", inc, "-o", exe, c], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sz, off, ssz, soff = map(int, out)
    assert sz == ctypes.sizeof(abi.Params)
    assert off == abi.Params.newton_guess.offset
    assert ssz == ctypes.sizeof(abi.Status)
    assert soff == abi.Status.last_error.offset


def test_enums_parsed():
    assert abi.NF_TK2 == abi.NF_N - 1 and abi.NF_EXXS == abi.NF_PRS + 1
    assert abi.MF_SLIPV == abi.MF_N - 1
    assert abi.MLP_NPARAM == 64 * 8 + 64 + 64 * 64 + 64 + 2 * 64 + 2 + 20
    assert abi.ERR_NOCONV == 6


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from velo2cycles_gb300 import _lib
    monkeypatch.setattr(_lib, "_LIB", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()
