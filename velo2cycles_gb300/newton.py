"""Per-marker visco-elasto-plastic + rate-and-state Newton and its learned
start, over the C ABI (no counterpart in the reference; see include/v2c.h).

``rsf_states`` draws seeded states with the distributions of the
per-marker Newton benchmark: a-b ~ U[-0.01, 0.015] with b = 0.015, L log-U
[1e-3, 1e-1] m, previous slip rate log-U[1e-15, 10] m/s, effective normal
stress U[5, 100] MPa, dt log-U[1e-3, 1e10] s; the rest (V0, mu0, state,
stress, strain rate, viscosity, shear modulus) are chosen here and stated in
the code.  Device buffers are torch tensors (plumbing only).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi
from ._lib import call


def rsf_states(n: int, seed: int = 0) -> np.ndarray:
    """float64[V2C_RS_N, n] column-major state block."""
    rng = np.random.default_rng(seed)
    S = np.zeros((abi.RS_N, n))
    b = np.full(n, 0.015)
    a = b + rng.uniform(-0.01, 0.015, n)
    L = 10.0 ** rng.uniform(-3, -1, n)
    V = 10.0 ** rng.uniform(-15, 1, n)
    sn = rng.uniform(5e6, 100e6, n)
    dt = 10.0 ** rng.uniform(-3, 10, n)
    V0 = 10.0 ** rng.uniform(-9, -6, n)
    mu0 = np.full(n, 0.6)
    # state near steady state at the previous slip rate
    phi = np.log(V0 / V) + rng.normal(0.0, 1.0, n)
    # stress near the steady-state friction at that slip rate
    w = np.log(V / (2 * V0)) + (mu0 + b * phi) / a
    tau = sn * a * np.where(w > 20, w + np.log(2.0), np.arcsinh(np.exp(np.minimum(w, 20)))) * \
        rng.uniform(0.8, 1.2, n)
    S[abi.RS_VOLD], S[abi.RS_PHIOLD], S[abi.RS_A], S[abi.RS_B] = V, phi, a, b
    S[abi.RS_L], S[abi.RS_V0], S[abi.RS_MU0], S[abi.RS_SN], S[abi.RS_DT] = L, V0, mu0, sn, dt
    S[abi.RS_TAUOLD] = tau
    S[abi.RS_EDOT] = 10.0 ** rng.uniform(-18, -10, n)
    S[abi.RS_ETA] = 10.0 ** rng.uniform(18, 25, n)
    S[abi.RS_G] = np.full(n, 3.0e10)
    return S


def _dev(a: np.ndarray, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype or a.dtype)).cuda()
    return t


def _torch_done(t) -> None:
    """Wait for the torch work queued on t's device (the fills of output
    buffers, the kernels that made the inputs): the library runs on its
    context's stream, which nothing orders after torch's."""
    import torch
    torch.cuda.current_stream(t.device).synchronize()


def solve(mic, states, guess: int = abi.GUESS_PLAIN, on_device: bool = False):
    """Solve every state; returns (out[V2C_RO_N, n], iterations[n]) as numpy
    (or torch device tensors when on_device).  Negative iteration counts
    mark states that did not reach the tolerance."""
    import torch
    S = states if isinstance(states, torch.Tensor) else _dev(np.asarray(states), np.float64)
    n = S.shape[1]
    out = torch.zeros((abi.RO_N, n), dtype=torch.float64, device=S.device)
    it = torch.zeros(n, dtype=torch.int32, device=S.device)
    _torch_done(S)
    call("v2c_rsf_newton", mic.h, ctypes.c_void_p(S.data_ptr()), n, int(guess),
         ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(it.data_ptr()))
    mic.synchronize()
    if on_device:
        return out, it
    return out.cpu().numpy(), it.cpu().numpy()


def collect_states(mic, stride: int = 1, cap: int | None = None):
    """Newton states of every stride-th marker of the running model as a
    float64 device tensor [V2C_RS_N, k] (markers without a problem
    dropped)."""
    import torch
    n = mic.n
    cap = cap if cap is not None else (n + stride - 1) // stride
    X = torch.empty((abi.RS_N, cap), dtype=torch.float64, device="cuda")
    _torch_done(X)
    got = ctypes.c_long()
    call("v2c_collect_newton_states", mic.h, int(stride), ctypes.c_void_p(X.data_ptr()), int(cap),
         ctypes.byref(got))
    mic.synchronize()
    X = X[:, :got.value]
    keep = ~torch.isnan(X[abi.RS_A])
    return X[:, keep].contiguous()


def train(mic, states, targets, epochs: int = 4, batch: int = 4096, lr: float = 3e-3,
          seed: int = 0) -> float:
    """Train the start-proposal network on the GPU; targets[2, n] =
    (slip rate, state) of converged plain-Newton solutions."""
    import torch
    S = states if isinstance(states, torch.Tensor) else _dev(np.asarray(states), np.float64)
    T = targets if isinstance(targets, torch.Tensor) else _dev(np.asarray(targets), np.float64)
    loss = ctypes.c_float()
    _torch_done(S)
    call("v2c_mlp_train", mic.h, ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(T.data_ptr()),
         S.shape[1], int(epochs), int(batch), float(lr), int(seed), ctypes.byref(loss))
    return loss.value


def grad(mic, states, targets):
    """(gradient[V2C_MLP_NPARAM-20], loss) at the loaded parameters."""
    S = _dev(np.asarray(states), np.float64)
    T = _dev(np.asarray(targets), np.float64)
    g = np.zeros(abi.MLP_NPARAM - 20, dtype=np.float32)
    loss = ctypes.c_float()
    _torch_done(S)
    call("v2c_mlp_grad", mic.h, ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(T.data_ptr()),
         S.shape[1], g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss))
    return g, loss.value


def infer(mic, states) -> np.ndarray:
    """Network outputs [2, n] = (log V, phi) at the loaded parameters."""
    import torch
    S = _dev(np.asarray(states), np.float64)
    out = torch.zeros((2, S.shape[1]), dtype=torch.float32, device=S.device)
    _torch_done(S)
    call("v2c_mlp_infer", mic.h, ctypes.c_void_p(S.data_ptr()), S.shape[1],
         ctypes.c_void_p(out.data_ptr()))
    mic.synchronize()
    return out.cpu().numpy()


def load(mic, params: np.ndarray):
    p = np.ascontiguousarray(params, dtype=np.float32)
    assert p.size == abi.MLP_NPARAM
    call("v2c_mlp_load", mic.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))


def save(mic) -> np.ndarray:
    p = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
    call("v2c_mlp_save", mic.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return p


def random_params(seed: int = 0, X: np.ndarray | None = None, Y: np.ndarray | None = None):
    """Packed parameters with Xavier-uniform weights and normalisation taken
    from sample features X[n,8] / targets Y[n,2] when given."""
    rng = np.random.default_rng(seed)
    p = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
    o = 0

    def put(k, lim):
        nonlocal o
        p[o:o + k] = rng.uniform(-lim, lim, k)
        o += k

    put(64 * 8, np.sqrt(6 / 72)); put(64, 0.1); put(64 * 64, np.sqrt(6 / 128)); put(64, 0.1)
    put(2 * 64, np.sqrt(6 / 66)); put(2, 0.1)
    p[o:o + 8] = X.mean(0) if X is not None else 0.0
    p[o + 8:o + 16] = X.std(0) + 1e-6 if X is not None else 1.0
    p[o + 16:o + 18] = Y.mean(0) if Y is not None else 0.0
    p[o + 18:o + 20] = Y.std(0) + 1e-6 if Y is not None else 1.0
    return p
