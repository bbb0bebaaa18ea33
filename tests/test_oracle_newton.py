"""The oracle's per-marker Newton and network reference (CPU)."""
import numpy as np

from oracle import bindings as B
from velo2cycles_gb300 import abi, newton


def test_newton_converges_on_benchmark_states():
    S = newton.rsf_states(50000, seed=3)
    out, it, nc = B.rsf_newton(S, rtol=1e-10, maxit=200)
    assert nc == 0 and (it >= 0).all()
    assert out[abi.RO_RES].max() <= 1e-10
    floored = out[abi.RO_V] == 1e-40
    # a floored state really has the load below the floor's yield
    Sf = S[:, floored][:, :50]
    for i in range(Sf.shape[1]):
        F = B._lib().v2c_oracle_rsf_residual(B._dp(np.ascontiguousarray(Sf[:, i])), 400.0, 1e-40,
                                               None, None, None, None)
        assert F >= 0


def test_solution_independent_of_start():
    S = newton.rsf_states(5000, seed=4)
    a, _, _ = B.rsf_newton(S)
    g = np.log(np.maximum(a[abi.RO_V], 1e-40)) + np.random.default_rng(0).normal(0, 3, 5000)
    b, _, _ = B.rsf_newton(S, guess_logV=g)
    assert np.quantile(np.abs(a[abi.RO_V] / b[abi.RO_V] - 1), 0.999) < 1e-8


def test_mlp_gradient_finite_difference():
    S = newton.rsf_states(64, seed=5)
    out, _, _ = B.rsf_newton(S)
    X = B.rsf_features(S)
    Y = np.stack([np.log(out[abi.RO_V]), out[abi.RO_PHI]], 1)
    P = newton.random_params(1, X, Y).astype(np.float32)
    loss, g = B.mlp_loss_grad(P, X, Y)
    rng = np.random.default_rng(0)
    for k in rng.choice(g.size, 12, replace=False):
        h = 1e-3
        Pp, Pm = P.copy(), P.copy()
        Pp[k] += h
        Pm[k] -= h
        fd = (B.mlp_loss_grad(Pp, X, Y, False)[0] - B.mlp_loss_grad(Pm, X, Y, False)[0]) / (
            float(Pp[k]) - float(Pm[k]))
        assert abs(fd - g[k]) <= 2e-3 * max(1.0, abs(g[k])) + 1e-6, (k, fd, g[k])
