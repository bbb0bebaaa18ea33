"""Float-float arithmetic of the split Newton (v2c_ff.cuh) against FP64.

Builds tests/ff_check.cu with nvcc for sm_103a and compares exp, log, div
and sqrt of float-float inputs (exact copies of doubles to 48 bits) with
numpy's FP64 results over the ranges the Newton uses.  Bound: 1e-13
relative for exp/log/div/sqrt (float-float carries ~48 bits; the FP64
reference contributes 1.1e-16).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from velo2cycles_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ff_check(tmp_path_factory):
    d = tmp_path_factory.mktemp("ff")
    exe = str(d / "ff_check")
    subprocess.run([build.nvcc(), "-O3", "-std=c++17", build.ARCH, "-o", exe,
                    os.path.join(HERE, "ff_check.cu")], check=True)
    return exe, d


def _run(ff_check, x, y):
    exe, d = ff_check
    fin, fout = str(d / "in.bin"), str(d / "out.bin")
    with open(fin, "wb") as f:
        np.array([x.size], np.int64).tofile(f)
        x.astype(np.float64).tofile(f)
        y.astype(np.float64).tofile(f)
    subprocess.run([exe, fin, fout], check=True)
    o = np.fromfile(fout, np.float32).reshape(4, x.size, 2).astype(np.float64)
    return o[..., 0] + o[..., 1]


def _ff(v):
    """the float-float value of a double: hi + lo as the device forms it"""
    hi = v.astype(np.float32).astype(np.float64)
    lo = (v - hi).astype(np.float32).astype(np.float64)
    return hi + lo


def test_ff_functions(ff_check):
    rng = np.random.default_rng(0)
    n = 200000
    # exp over [-60, 87]; log and sqrt over magnitudes e^-80 .. e^80; quotients
    # of magnitudes e^-40 .. e^40 by divisors that keep them within e^+-40
    xe = np.concatenate([rng.uniform(-60, 87, n // 2), rng.uniform(-1, 1, n // 2)])
    xm = np.exp(rng.uniform(-80, 80, n)) * rng.choice([-1, 1], n)
    xd = np.exp(rng.uniform(-40, 40, n)) * rng.choice([-1, 1], n)
    yd = xd * np.exp(rng.uniform(-40, 40, n)) * rng.choice([-1, 1], n)
    ex, _, _, _ = _run(ff_check, xe, np.ones(n))
    _, lg, _, sq = _run(ff_check, xm, np.ones(n))
    _, _, dv, _ = _run(ff_check, xd, yd)
    xef, xdf, ydf = _ff(xe), _ff(xd), _ff(yd)
    axf = _ff(np.abs(xm))
    err = {
        "exp": np.abs(ex / np.exp(xef) - 1).max(),
        # log crosses zero at 1: error relative to max(|log|, 1)
        "log": (np.abs(lg - np.log(axf)) / np.maximum(np.abs(np.log(axf)), 1.0)).max(),
        "div": np.abs(dv / (xdf / ydf) - 1).max(),
        "sqrt": np.abs(sq / np.sqrt(axf) - 1).max(),
    }
    bad = {k: v for k, v in err.items() if not v < 1e-13}
    assert not bad, err
