"""ctypes / subprocess front-ends of the two CPU checkers (test infrastructure)."""
from __future__ import annotations

import ctypes
import os
import resource
import shutil
import subprocess
import tempfile

import numpy as np

from velo2cycles_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def restatement_path() -> str:
    return os.path.join(OUT, "liboracle.so")


def reference_path(serial: bool = False, fast: bool = False, full: bool = False) -> str:
    """The reference routines built with OpenMP (v2c_ref), with the OpenMP
    pragmas ignored (v2c_ref_serial), or with OpenMP and floating-point
    contraction allowed (v2c_ref_fast: the timed baseline; v2c_ref_full: the
    same with the arrays of the full C4 configuration)."""
    if full:
        return os.path.join(OUT, "v2c_ref_full")
    if fast:
        return os.path.join(OUT, "v2c_ref_fast")
    return os.path.join(OUT, "v2c_ref_serial" if serial else "v2c_ref")


def _stale() -> bool:
    outs = [restatement_path(), reference_path()]
    if not all(os.path.exists(o) for o in outs):
        return True
    t = min(os.path.getmtime(o) for o in outs)
    deps = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".c", ".h", ".sh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "v2c.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> None:
    """Compile both checkers with oracle/build_ref.sh (seconds); again when
    a source or the C-ABI header is newer than the builds."""
    if force or _stale():
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)


def reference_available() -> bool:
    return os.path.exists(reference_path())


# ------------------------------------------------------------ restatement

class _State(ctypes.Structure):
    _fields_ = [
        ("p", abi.Params),
        ("gx", ctypes.POINTER(ctypes.c_double)),
        ("gy", ctypes.POINTER(ctypes.c_double)),
        ("rt", ctypes.POINTER(ctypes.c_double)),
        ("N", ctypes.POINTER(ctypes.c_double) * abi.NF_N),
        ("M", ctypes.POINTER(ctypes.c_double) * abi.MF_N),
        ("t", ctypes.POINTER(ctypes.c_byte)),
        ("n", ctypes.c_long),
        ("bondm", ctypes.POINTER(ctypes.c_long)),
        ("bondn", ctypes.POINTER(ctypes.c_long)),
        ("bondv", ctypes.POINTER(ctypes.c_double)),
        ("bondnum", ctypes.c_long),
        ("nthreads", ctypes.c_int),
        ("phantom", ctypes.c_int),
        ("cap", ctypes.c_long),
    ]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(restatement_path()):
            build()
        lib = ctypes.CDLL(restatement_path())
        P = ctypes.POINTER
        lib.v2c_oracle_nxsearch.restype = ctypes.c_long
        lib.v2c_oracle_nxsearch.argtypes = [P(ctypes.c_double), ctypes.c_long, ctypes.c_double]
        for fn in ("v2c_oracle_marker2nodes", "v2c_oracle_center2basic_old",
                   "v2c_oracle_nodes2markers", "v2c_oracle_move"):
            getattr(lib, fn).restype = ctypes.c_int
            getattr(lib, fn).argtypes = [P(_State)]
        lib.v2c_oracle_basic2center.restype = ctypes.c_int
        lib.v2c_oracle_basic2center.argtypes = [P(_State)]
        lib.v2c_oracle_recompute_stress.restype = ctypes.c_int
        lib.v2c_oracle_recompute_stress.argtypes = [P(_State), ctypes.c_double]
        lib.v2c_oracle_marker_temperature.restype = ctypes.c_int
        lib.v2c_oracle_marker_temperature.argtypes = [P(_State), ctypes.c_double]
        lib.v2c_oracle_stokes_assemble.restype = ctypes.c_int
        lib.v2c_oracle_stokes_assemble.argtypes = [
            P(_State), P(abi.StokesCtl), ctypes.c_long, P(ctypes.c_int), P(ctypes.c_int),
            P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_long)]
        lib.v2c_oracle_marker_properties.restype = ctypes.c_int
        lib.v2c_oracle_marker_properties.argtypes = [P(_State), P(ctypes.c_double),
                                                     P(ctypes.c_double), P(ctypes.c_double)]
        lib.v2c_oracle_copyarrays.restype = ctypes.c_int
        lib.v2c_oracle_copyarrays.argtypes = [P(_State)]
        lib.v2c_oracle_center2basic.restype = ctypes.c_int
        lib.v2c_oracle_center2basic.argtypes = [P(_State), ctypes.c_double]
        lib.v2c_oracle_compute_before_solve.restype = ctypes.c_int
        lib.v2c_oracle_compute_before_solve.argtypes = [P(_State), ctypes.c_double, ctypes.c_int]
        lib.v2c_oracle_calc_timestep.restype = ctypes.c_int
        lib.v2c_oracle_calc_timestep.argtypes = [P(_State), ctypes.c_int, P(abi.TimestepCtl),
                                                 P(abi.TimestepInfo)]
        lib.v2c_oracle_compute_after_solve.restype = ctypes.c_double
        lib.v2c_oracle_compute_after_solve.argtypes = [P(_State), ctypes.c_double, ctypes.c_int]
        lib.v2c_oracle_rsf_newton.restype = ctypes.c_long
        lib.v2c_oracle_rsf_newton.argtypes = [P(ctypes.c_double), ctypes.c_long, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, P(ctypes.c_double),
                                              P(ctypes.c_double), P(ctypes.c_int)]
        lib.v2c_oracle_rsf_features.restype = None
        lib.v2c_oracle_rsf_features.argtypes = [P(ctypes.c_double), ctypes.c_long, ctypes.c_long,
                                                P(ctypes.c_double)]
        lib.v2c_oracle_rsf_residual.restype = ctypes.c_double
        lib.v2c_oracle_rsf_residual.argtypes = [P(ctypes.c_double), ctypes.c_double, ctypes.c_double,
                                                P(ctypes.c_double), P(ctypes.c_double),
                                                P(ctypes.c_double), P(ctypes.c_double)]
        lib.v2c_oracle_mlp_loss_grad.restype = ctypes.c_double
        lib.v2c_oracle_mlp_loss_grad.argtypes = [P(ctypes.c_float), P(ctypes.c_double),
                                                 P(ctypes.c_double), ctypes.c_long, P(ctypes.c_double)]
        lib.v2c_oracle_mlp_forward.restype = None
        lib.v2c_oracle_mlp_forward.argtypes = [P(ctypes.c_float), P(ctypes.c_double), ctypes.c_long,
                                               P(ctypes.c_double)]
        _LIB = lib
    return _LIB


class Restatement:
    """Runs the C restatement on a copy of a synth.Case (arrays updated in place)."""

    def __init__(self, case, nthreads: int = 1, phantom: bool = False, cap: int = 0):
        """cap: room for markers beyond case.n (immobile markers append
        markers in the move); marks/markt show the current markers."""
        self.case = case
        self.lib = _lib()
        c = case
        self._keep = []
        cap = max(int(cap), c.n)
        self.nodes = {f: np.ascontiguousarray(c.nodes[f], dtype=np.float64) for f in range(abi.NF_N)}
        self._marks = {f: np.zeros(max(cap, 1)) for f in range(abi.MF_N)}
        self._markt = np.zeros(max(cap, 1), dtype=np.int8)
        for f in range(abi.MF_N):
            self._marks[f][:c.n] = c.marks[f]
        self._markt[:c.n] = c.markt
        self.gx = np.ascontiguousarray(c.gx, dtype=np.float64)
        self.gy = np.ascontiguousarray(c.gy, dtype=np.float64)
        self.rt = np.ascontiguousarray(c.rt, dtype=np.float64)
        self.bondm = np.ascontiguousarray(c.bondm, dtype=np.int64)
        self.bondn = np.ascontiguousarray(c.bondn, dtype=np.int64)
        self.bondv = np.ascontiguousarray(c.bondv, dtype=np.float64)
        st = _State()
        st.p = abi.Params.from_dict(c.params)
        st.gx, st.gy, st.rt = _dp(self.gx), _dp(self.gy), _dp(self.rt)
        for f in range(abi.NF_N):
            st.N[f] = _dp(self.nodes[f])
        for f in range(abi.MF_N):
            st.M[f] = _dp(self._marks[f])
        st.t = self._markt.ctypes.data_as(ctypes.POINTER(ctypes.c_byte))
        st.n = c.n
        st.cap = cap
        st.bondm = self.bondm.ctypes.data_as(ctypes.POINTER(ctypes.c_long))
        st.bondn = self.bondn.ctypes.data_as(ctypes.POINTER(ctypes.c_long))
        st.bondv = _dp(self.bondv)
        st.bondnum = c.bondnum
        st.nthreads = nthreads
        st.phantom = int(phantom)
        self.st = st

    @property
    def n(self) -> int:
        return int(self.st.n)

    @property
    def marks(self) -> dict:
        return {f: a[:self.st.n] for f, a in self._marks.items()}

    @property
    def markt(self) -> np.ndarray:
        return self._markt[:self.st.n]

    def set_params(self, **kw):
        d = self.st.p.to_dict()
        d.update(kw)
        self.st.p = abi.Params.from_dict(d)

    def marker2nodes(self):
        return self.lib.v2c_oracle_marker2nodes(ctypes.byref(self.st))

    def marker_properties(self):
        """(viscosity, conductivity, pressure in bar) of every current
        marker as marker2nodes evaluates them; 0 outside the model."""
        n = self.n
        nu, kt, pb = np.zeros(n), np.zeros(n), np.zeros(n)
        self.lib.v2c_oracle_marker_properties(ctypes.byref(self.st), _dp(nu), _dp(kt), _dp(pb))
        return nu, kt, pb

    def center2basic_old(self):
        return self.lib.v2c_oracle_center2basic_old(ctypes.byref(self.st))

    def basic2center(self):
        return self.lib.v2c_oracle_basic2center(ctypes.byref(self.st))

    def center2basic(self, dt):
        return self.lib.v2c_oracle_center2basic(ctypes.byref(self.st), dt)

    def recompute_stress(self, dt):
        return self.lib.v2c_oracle_recompute_stress(ctypes.byref(self.st), dt)

    def marker_temperature(self, heatdif):
        return self.lib.v2c_oracle_marker_temperature(ctypes.byref(self.st), heatdif)

    def copyarrays(self):
        return self.lib.v2c_oracle_copyarrays(ctypes.byref(self.st))

    def stokes_assemble(self, **ctl):
        """preparematrix + gausmat4_add on the current node fields: (rc, dict
        of ia, ja, a, b as the reference leaves them)."""
        c = abi.StokesCtl(**ctl)
        rows = 3 * self.case.nodenum
        nnz = ctypes.c_long(0)
        P = ctypes.POINTER
        rc = self.lib.v2c_oracle_stokes_assemble(ctypes.byref(self.st), ctypes.byref(c), 0, None,
                                                 None, None, None, ctypes.byref(nnz))
        if rc:
            return rc, None
        ia = np.zeros(rows + 1, dtype=np.int32)
        ja = np.zeros(max(nnz.value, 1), dtype=np.int32)
        a = np.zeros(max(nnz.value, 1))
        b = np.zeros(rows)
        rc = self.lib.v2c_oracle_stokes_assemble(
            ctypes.byref(self.st), ctypes.byref(c), nnz.value, ia.ctypes.data_as(P(ctypes.c_int)),
            ja.ctypes.data_as(P(ctypes.c_int)), a.ctypes.data_as(P(ctypes.c_double)),
            b.ctypes.data_as(P(ctypes.c_double)), ctypes.byref(nnz))
        return rc, dict(ia=ia, ja=ja[:nnz.value], a=a[:nnz.value], b=b)

    def compute_before_solve(self, dt, rk=0):
        return self.lib.v2c_oracle_compute_before_solve(ctypes.byref(self.st), dt, rk)

    def compute_after_solve(self, dt, rk=0):
        return self.lib.v2c_oracle_compute_after_solve(ctypes.byref(self.st), dt, rk)

    def calc_timestep(self, oldornew=0, **ctl):
        """(status, info dict) of calc_timestep (calc_RSF.c:352-572)."""
        c = abi.TimestepCtl(**dict(abi.TIMESTEP_DEFAULTS, **ctl))
        info = abi.TimestepInfo()
        rc = self.lib.v2c_oracle_calc_timestep(ctypes.byref(self.st), oldornew, ctypes.byref(c),
                                               ctypes.byref(info))
        return rc, info.to_dict()

    def nodes2markers(self):
        return self.lib.v2c_oracle_nodes2markers(ctypes.byref(self.st))

    def move(self):
        return self.lib.v2c_oracle_move(ctypes.byref(self.st))

    def step(self):
        """One MIC step with the solver outputs held fixed."""
        dt = self.st.p.timestep
        rc = self.marker2nodes()
        rc |= self.center2basic_old()
        rc |= self.compute_before_solve(dt, 0)
        self.compute_after_solve(dt, 0)
        rc |= self.nodes2markers()
        rc |= self.move()
        return rc


def nxsearch(g: np.ndarray, x: float) -> int:
    g = np.ascontiguousarray(g, dtype=np.float64)
    return int(_lib().v2c_oracle_nxsearch(_dp(g), g.size, float(x)))


def rsf_newton(states: np.ndarray, W=400.0, rtol=1e-10, maxit=200, guess_logV=None):
    """states: float64[V2C_RS_N, n] -> (out[V2C_RO_N, n], iters[n], nonconv)"""
    states = np.ascontiguousarray(states, dtype=np.float64)
    n = states.shape[1]
    out = np.zeros((abi.RO_N, n))
    it = np.zeros(n, dtype=np.int32)
    g = None if guess_logV is None else np.ascontiguousarray(guess_logV, dtype=np.float64)
    nc = _lib().v2c_oracle_rsf_newton(_dp(states), n, W, rtol, maxit,
                                      _dp(g) if g is not None else None, _dp(out),
                                      it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return out, it, nc


def rsf_residual(states: np.ndarray, V: np.ndarray, W=400.0) -> np.ndarray:
    """FP64 relative residual |F|/(F+T*) of the per-marker problem at the
    given slip rates (oracle rsf_eval)."""
    S = np.ascontiguousarray(states, dtype=np.float64)
    n = S.shape[1]
    out = np.empty(n)
    L = _lib()
    scale = ctypes.c_double()
    for i in range(n):
        st = np.ascontiguousarray(S[:, i])
        F = L.v2c_oracle_rsf_residual(_dp(st), W, float(V[i]), None, None, None,
                                      ctypes.byref(scale))
        out[i] = abs(F) / scale.value
    return out


def rsf_features(states: np.ndarray) -> np.ndarray:
    states = np.ascontiguousarray(states, dtype=np.float64)
    n = states.shape[1]
    X = np.zeros((n, 8))
    lib = _lib()
    buf = np.zeros(8)
    for i in range(n):
        lib.v2c_oracle_rsf_features(_dp(states), n, i, _dp(buf))
        X[i] = buf
    return X


def mlp_loss_grad(params: np.ndarray, X: np.ndarray, Y: np.ndarray, want_grad=True):
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float64)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    ng = abi.MLP_NPARAM - 20
    g = np.zeros(ng) if want_grad else None
    loss = _lib().v2c_oracle_mlp_loss_grad(params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           _dp(X), _dp(Y), X.shape[0], _dp(g) if want_grad else None)
    return loss, g


def mlp_forward(params: np.ndarray, X: np.ndarray) -> np.ndarray:
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float64)
    Y = np.zeros((X.shape[0], 2))
    _lib().v2c_oracle_mlp_forward(params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                  _dp(X), X.shape[0], _dp(Y))
    return Y


# -------------------------------------------------------------- reference

STAGE_M2N, STAGE_C2B, STAGE_BEFORE, STAGE_AFTER, STAGE_N2M, STAGE_MOVE = range(6)
ALL_STAGES = 0b111111
TIMESTEP_STAGE = 1 << 6
# interpolate_basic2center after compute_before_solve, interpolate_center2basic
# before compute_after_solve (the Picard loop's order)
B2C_STAGE, C2B_FULL_STAGE = 1 << 7, 1 << 8
# recompute_stress_strainrate between them, copyarrays after compute_after_solve
RECOMPUTE_STAGE, COPY_STAGE = 1 << 9, 1 << 10
# solve_temperature with the thermal solve replaced by the node field TK2
# (the new temperatures); afterwards TK holds them and TK2 the old ones
TEMPERATURE_STAGE = 1 << 11
# save_model (load_save.c:353) after the steps: the result holds the bytes
# of the restart file the reference wrote ("prn")
SAVE_STAGE = 1 << 12
# preparematrix (momentum_continuity_addmatrix_checkerror.c:22) after the
# steps: the result holds the CSR arrays gausmat4_add built ("stokes": ia,
# ja, a, b); needs the stokes= argument (v2c_stokes_ctl values)
STOKES_STAGE = 1 << 13
# timing only: the result holds the per-stage seconds and the deltas, no
# arrays (a full C4 state is ~16 GB each way)
TIMING_ONLY = 1 << 14
STOKES_KEYS = ("mukoef", "dt", "gxkoef", "gykoef", "timebond", "drunkensailor")


def picard_passes(npass: int) -> int:
    """Stage bits asking for npass Picard passes (rk = 0 .. npass-1) of
    compute_before_solve + compute_after_solve after marker2nodes and
    interpolate_center2basic_old (with STAGE_BEFORE and STAGE_AFTER)."""
    assert 0 < npass < 16
    return npass << 16


def write_case(path: str, case, stages=ALL_STAGES, nthreads=1, nsteps=1, warmup=0,
               timestep=None, oldornew=0, dts=None, heatdif=None, stokes=None) -> None:
    """timestep: v2c_timestep_ctl values as a dict (abi.TIMESTEP_DEFAULTS when
    None); oldornew: the argument of calc_timestep (stage bit 6); dts: a
    time step per step (timesum advances after each)."""
    c = case
    nn = c.nodenum
    with open(path, "wb") as f:
        f.write(b"V2CCASE1")
        np.array([c.params["xnumx"], c.params["ynumy"], c.n, c.bondnum, nthreads, stages,
                  nsteps, warmup], dtype=np.int64).tofile(f)
        f.write(bytes(abi.Params.from_dict(c.params)))
        np.ascontiguousarray(c.gx, dtype=np.float64).tofile(f)
        np.ascontiguousarray(c.gy, dtype=np.float64).tofile(f)
        np.ascontiguousarray(c.rt, dtype=np.float64).tofile(f)
        for k in range(abi.NF_N):
            np.ascontiguousarray(c.nodes[k], dtype=np.float64).reshape(nn).tofile(f)
        for k in range(abi.MF_N):
            np.ascontiguousarray(c.marks[k], dtype=np.float64).tofile(f)
        np.ascontiguousarray(c.markt, dtype=np.int8).tofile(f)
        np.ascontiguousarray(c.bondm, dtype=np.int64).tofile(f)
        np.ascontiguousarray(c.bondn, dtype=np.int64).tofile(f)
        np.ascontiguousarray(c.bondv, dtype=np.float64).tofile(f)
        ts = dict(abi.TIMESTEP_DEFAULTS, **(timestep or {}))
        np.array([ts["maxtmstep"], ts["dtfactor"], ts["tcnvp"], ts["tcd"], ts["tcphih"],
                  float(oldornew)], dtype=np.float64).tofile(f)
        if dts is not None or heatdif is not None or stokes is not None:
            d = [] if dts is None else dts
            np.array([len(d)], dtype=np.int64).tofile(f)
            np.ascontiguousarray(d, dtype=np.float64).tofile(f)
        if heatdif is not None or stokes is not None:
            np.array([heatdif or 0.0], dtype=np.float64).tofile(f)
        if stokes is not None:
            np.array([float(stokes[k]) for k in STOKES_KEYS], dtype=np.float64).tofile(f)


def read_csr(path: str) -> dict:
    """The CSR arrays the harness writes: int64 rows, nnz; int32 ia[rows+1],
    ja[nnz]; double a[nnz], b[rows]; then (harness only) the seconds the
    reference's preparematrix took."""
    with open(path, "rb") as f:
        rows, nnz = (int(v) for v in np.fromfile(f, dtype=np.int64, count=2))
        out = dict(ia=np.fromfile(f, dtype=np.int32, count=rows + 1),
                   ja=np.fromfile(f, dtype=np.int32, count=nnz),
                   a=np.fromfile(f, dtype=np.float64, count=nnz),
                   b=np.fromfile(f, dtype=np.float64, count=rows))
        t = np.fromfile(f, dtype=np.float64, count=1)
        out["seconds"] = float(t[0]) if t.size else None
        return out


def read_result(path: str, nodenum: int):
    with open(path, "rb") as f:
        magic = f.read(8)
        if magic == b"V2CSEC01":
            secs = np.fromfile(f, dtype=np.float64, count=8)
            deltas = float(np.fromfile(f, dtype=np.float64, count=1)[0])
            return dict(seconds=secs, deltas=deltas)
        assert magic == b"V2CRES01"
        n = int(np.fromfile(f, dtype=np.int64, count=1)[0])
        nodes = {k: np.fromfile(f, dtype=np.float64, count=nodenum) for k in range(abi.NF_N)}
        marks = {k: np.fromfile(f, dtype=np.float64, count=n) for k in range(abi.MF_N)}
        markt = np.fromfile(f, dtype=np.int8, count=n)
        secs = np.fromfile(f, dtype=np.float64, count=8)
        deltas = float(np.fromfile(f, dtype=np.float64, count=1)[0])
        ts_rc = int(np.fromfile(f, dtype=np.int64, count=1)[0])
        info = abi.TimestepInfo.from_buffer_copy(f.read(ctypes.sizeof(abi.TimestepInfo)))
    return dict(nodes=nodes, marks=marks, markt=markt, seconds=secs, deltas=deltas, n=n,
                timestep_rc=ts_rc, timestep=info.to_dict())


def big_stack():
    """A 1 GB main-thread stack for the reference process: its boundary
    corrections keep two node arrays on the stack (vxvy_boundarycorrection,
    momentum_continuity_addmatrix_checkerror.c:1009), 64 MB at C4, beyond
    the usual 8 MB limit."""
    lim = 1 << 30
    soft, hard = resource.getrlimit(resource.RLIMIT_STACK)
    if hard != resource.RLIM_INFINITY:
        lim = min(lim, hard)
    if soft == resource.RLIM_INFINITY or soft < lim:
        resource.setrlimit(resource.RLIMIT_STACK, (lim, hard))


def scratch_dir(case):
    """Where the case file goes: memory-backed /dev/shm when it holds the
    case with room to spare, else the default temporary directory."""
    need = 8 * (case.nodenum * abi.NF_N + case.n * (abi.MF_N + 1)) * 1.5
    try:
        if shutil.disk_usage("/dev/shm").free > need:
            return "/dev/shm"
    except OSError:
        pass
    return None


def run_reference(case, stages=ALL_STAGES, nthreads=1, nsteps=1, warmup=0, timeout=3600,
                  timestep=None, oldornew=0, dts=None, heatdif=None, stokes=None,
                  serial=False, fast=False, full=False):
    """Run the reference routines on `case`; returns the arrays after the
    stages plus per-stage seconds summed over the timed steps.  serial: the
    build with the OpenMP pragmas ignored; fast: the build with
    floating-point contraction (timing only); full: that build with the
    arrays of the full C4 configuration (stages & TIMING_ONLY for a
    seconds-only result)."""
    if not reference_available():
        build()
    if not reference_available():
        raise RuntimeError("reference oracle not built (reference sources unavailable)")
    if full and not os.path.exists(reference_path(full=True)):
        raise RuntimeError("full-size reference build unavailable")
    with tempfile.TemporaryDirectory(dir=scratch_dir(case)) as d:
        cp, rp = os.path.join(d, "case.bin"), os.path.join(d, "res.bin")
        write_case(cp, case, stages, nthreads, nsteps, warmup, timestep, oldornew, dts, heatdif,
                   stokes)
        env = dict(os.environ, OMP_NUM_THREADS=str(max(1, nthreads)))
        exe = reference_path(serial, fast, full)
        if fast and not os.path.exists(exe):
            exe = reference_path(serial)
        r = subprocess.run([exe, cp, rp], env=env, capture_output=True,
                           timeout=timeout, cwd=d, preexec_fn=big_stack)
        if r.returncode != 0:
            raise RuntimeError(f"v2c_ref failed ({r.returncode}): {r.stderr.decode()[-2000:]}")
        res = read_result(rp, case.nodenum)
        if stages & SAVE_STAGE:
            with open(os.path.join(d, "state.prn"), "rb") as f:
                res["prn"] = f.read()
        if stages & STOKES_STAGE:
            res["stokes"] = read_csr(os.path.join(d, "stokes.bin"))
        return res
