"""Per-marker VEP+RSF Newton and its learned start (GPU).

* both GPU forms -- split (FP32 iterations, float-float finish) and FP64 --
  reach the 1e-10 relative residual on every state, recomputed in FP64 by
  the oracle at the returned slip rate, and find the oracle's root (FP64
  CPU Newton, oracle/v2c_oracle.c), slip rates within 1e-8 relative; the
  FP64 form takes the oracle's iteration path;
* the backward pass of the network (BF16 tensor cores, FP32 accumulate)
  matches the FP64 CPU gradient of the same loss: cosine > 0.999, relative
  norm error < 3e-2 (BF16 operands carry 8 bits of mantissa);
* inference matches the FP64 CPU forward to 3e-2 in log slip rate;
* trained on plain-Newton solutions, the network's start needs fewer
  iterations than the plain start on held-out states, with the same
  residual, and in the FP64 form takes less device time, its own pass
  included.
"""
import numpy as np
import pytest

from oracle import bindings as B
from velo2cycles_gb300 import abi, mic, newton, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_lib, oracle_built):
    c = synth.make_case("tiny", seed=3)
    m = mic.from_case(c)
    yield m
    m.close()


def _targets(out):
    return np.stack([out[abi.RO_V], out[abi.RO_PHI]])


def test_plain_newton_matches_oracle(ctx):
    S = newton.rsf_states(20000, seed=11)
    out, it = newton.solve(ctx, S, abi.GUESS_PLAIN)
    assert (it >= 0).all(), "non-converged states"
    assert out[abi.RO_RES].max() <= 1e-10
    ref, rit, nc = B.rsf_newton(S, rtol=1e-10, maxit=200)
    assert nc == 0
    rel = np.abs(out[abi.RO_V] / ref[abi.RO_V] - 1)
    assert np.quantile(rel, 0.999) < 1e-8, np.quantile(rel, 0.999)
    st = ctx.status()
    assert st["newton_nonconv"] == 0


@pytest.mark.parametrize("precision", [abi.NEWTON_SPLIT, abi.NEWTON_FP64])
def test_forms_reach_the_oracle_root(ctx, precision):
    S = newton.rsf_states(20000, seed=31)
    ref, rit, nc = B.rsf_newton(S, rtol=1e-10, maxit=200)
    assert nc == 0
    ctx.set_params(newton_precision=precision)
    try:
        out, it = newton.solve(ctx, S, abi.GUESS_PLAIN)
    finally:
        ctx.set_params(newton_precision=abi.NEWTON_SPLIT)
    assert (it >= 0).all(), "non-converged states"
    assert out[abi.RO_RES].max() <= 1e-10
    V = out[abi.RO_V]
    live = V > 1e-40
    # the converged residual recomputed in FP64 at the returned slip rate
    res = B.rsf_residual(S[:, live], V[live])
    assert res.max() <= 1e-10, res.max()
    rel = np.abs(V / ref[abi.RO_V] - 1)
    assert np.quantile(rel, 0.999) < 1e-8, np.quantile(rel, 0.999)
    tau_rel = np.abs(out[abi.RO_TAU] / ref[abi.RO_TAU] - 1)
    assert np.quantile(tau_rel[live], 0.999) < 1e-8
    if precision == abi.NEWTON_FP64:
        # same safeguarded Newton, same start: the same number of steps
        assert np.mean(it == rit) > 0.99


def test_mlp_gradient_matches_oracle(ctx):
    S = newton.rsf_states(4096, seed=5)
    ref, _, _ = B.rsf_newton(S, rtol=1e-10, maxit=200)
    T = _targets(ref)
    X = B.rsf_features(S)
    Y = np.stack([np.log(T[0]), T[1]], 1)
    P = newton.random_params(3, X, Y)
    newton.load(ctx, P)
    g, loss = newton.grad(ctx, S, T)
    loss_ref, g_ref = B.mlp_loss_grad(P, X, Y)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    err = float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))
    assert cos > 0.999 and err < 3e-2, (cos, err)
    assert abs(loss - loss_ref) <= 2e-2 * loss_ref


def test_training_gain(ctx):
    train = newton.rsf_states(200000, seed=21)
    test = newton.rsf_states(20000, seed=22)
    out, _ = newton.solve(ctx, train, abi.GUESS_PLAIN)
    loss = newton.train(ctx, train, _targets(out), epochs=6, batch=4096, lr=3e-3, seed=1)
    assert np.isfinite(loss)
    P = newton.save(ctx)
    # inference parity with the FP64 forward of the same parameters
    X = B.rsf_features(test[:, :2000])
    yref = B.mlp_forward(P, X)
    y = newton.infer(ctx, test[:, :2000])
    assert np.abs(y[0] - yref[:, 0]).max() < 3e-2 * max(1.0, np.abs(yref[:, 0]).max() / 10)
    st0 = ctx.status()
    po, pit = newton.solve(ctx, test, abi.GUESS_PLAIN)
    st1 = ctx.status()
    lo, lit = newton.solve(ctx, test, abi.GUESS_LEARNED)
    st2 = ctx.status()
    assert po[abi.RO_RES].max() <= 1e-10 and lo[abi.RO_RES].max() <= 1e-10
    assert (pit >= 0).all() and (lit >= 0).all()
    plain_it = st1["newton_iters"] - st0["newton_iters"]
    learned_it = st2["newton_iters"] - st1["newton_iters"]
    assert learned_it < plain_it, (learned_it, plain_it)
    # both reach the same root
    rel = np.abs(lo[abi.RO_V] / po[abi.RO_V] - 1)
    assert np.quantile(rel, 0.999) < 1e-8
    # and the time: in the FP64 form, whose iterations are the expensive
    # ones, the network's start (its own pass included) takes less device
    # time than the plain start on 1 M held-out states (CUDA events around
    # the library's kernels)
    import torch
    big = torch.from_numpy(newton.rsf_states(1_000_000, seed=23)).cuda()
    ms = {}
    ctx.set_params(newton_precision=abi.NEWTON_FP64)
    try:
        for g in (abi.GUESS_PLAIN, abi.GUESS_LEARNED):
            newton.solve(ctx, big, g, on_device=True)  # warm-up
            ctx.set_profiling(True)
            for _ in range(3):
                newton.solve(ctx, big, g, on_device=True)
            ms[g] = ctx.profile()["newton"][0] / 3
            ctx.set_profiling(False)
    finally:
        ctx.set_params(newton_precision=abi.NEWTON_SPLIT)
    assert ms[abi.GUESS_LEARNED] < 0.95 * ms[abi.GUESS_PLAIN], ms


def test_mic_step_runs_newton(ctx):
    c = synth.make_case("small", seed=4)
    m = mic.from_case(c)
    m.set_params(newton_guess=abi.GUESS_PLAIN)
    m.step()
    st = m.status()
    assert st["newton_iters"] > 0 and st["newton_nonconv"] == 0
    assert st["newton_max_res"] <= 1e-10
    v = m.download_markers([abi.MF_SLIPV])[abi.MF_SLIPV]
    assert np.isfinite(v).all() and (v > 0).all()
    m.close()


def test_collected_states_are_the_step_problems(ctx):
    """v2c_collect_newton_states hands out exactly the problems the step
    solves: solving them gives the slip rates the step writes."""
    c = synth.make_case("small", seed=9)
    c.marks[abi.MF_SLIPV][:] = -1.0  # plain start falls back to the same fixed value
    m = mic.from_case(c)
    S = newton.collect_states(m)
    assert S.shape[0] == abi.RS_N and S.shape[1] > 0
    out, it = newton.solve(m, S, abi.GUESS_PLAIN)
    assert (it >= 0).all() and out[abi.RO_RES].max() <= 1e-10
    before = m.download_markers([abi.MF_PHI, abi.MF_XX])
    m.set_params(newton_guess=abi.GUESS_PLAIN)
    m.marker2nodes()
    v = m.download_markers([abi.MF_SLIPV])[abi.MF_SLIPV]
    solved = v > 0
    assert solved.sum() == S.shape[1]
    # the same problems: the same slip rates up to the freedom the 1e-10
    # residual leaves (the two kernels may round their FP32 iterates
    # differently)
    a_, b_ = np.sort(v[solved]), np.sort(out[abi.RO_V].astype(np.float32).astype(np.float64))
    rel = np.abs(a_ - b_) / b_
    assert np.quantile(rel, 0.999) < 1e-6 and rel.max() < 1e-3, (np.quantile(rel, 0.999), rel.max())
    m.close()
    # collection changed nothing
    m2 = mic.from_case(c)
    newton.collect_states(m2, stride=3)
    after = m2.download_markers([abi.MF_PHI, abi.MF_XX])
    assert all(np.array_equal(before[k], after[k]) for k in before)
    m2.close()
