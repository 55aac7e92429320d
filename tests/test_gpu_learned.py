"""Learned warm start: the MLP's own BF16 kernels against the FP64 oracle, and what
the trained network gains over starting the gathering solve without it.

Bars: CUDA-core engine forward within 1e-4 relative of the FP64 oracle on the same
BF16 weights, every layer's gradient within 1e-3 relative (FP32 vs FP64
accumulation); tensor-core engine within 1e-3 / 5e-3 (relative L2) of the oracle with its BF16
activation roundings (relative L2 1e-3 / 5e-3); training reduces the loss; on a held-out scene the learned guess starts the solve closer to the solution than the
emission-only start and needs no more refinement steps to reach 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(P, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 1, (P, 32)).astype(np.float32), rng.normal(0, 1, (P, 3)).astype(np.float32)


def test_mlp_forward_and_gradients_match_oracle(lib):
    """CUDA-core engine (FP32 activations)."""
    from oracle import mlp_oracle

    m = lib.MLP(seed=7)
    m.set_tensor_cores(False)
    p = m.params()
    X, T = _data(257, 1)
    Y = m.predict(X)
    ref = mlp_oracle.forward(p, X)[-1]
    assert np.max(np.abs(Y - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))
    g, loss = m.gradients(X, T)
    gref, lref = mlp_oracle.gradients(p, X, T)
    assert abs(loss - lref) <= 1e-5 * lref
    at = 0
    for l in range(5):
        o, i = mlp_oracle.DIMS[l + 1], mlp_oracle.DIMS[l]
        for size in (o * i, o):
            a, b = g[at:at + size], gref[at:at + size]
            assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b) + 1e-12, (l, size)
            at += size
    m.close()


@pytest.mark.parametrize("P", [257, 4096, 5000])
def test_mlp_tensor_core_engine_matches_oracle(lib, P):
    """tcgen05 engine against the FP64 oracle with the same BF16 roundings of activations and
    output gradients: forward within 1e-3 relative L2, each gradient within 5e-3 relative L2,
    loss within 1e-3 (an FP32 sum and an FP64 sum can round to neighbouring BF16 values now and
    then, which moves a few outputs by about a BF16 step: the bars are norms, not maxima).
    P = 257 and 5000 leave partial row tiles and a partial 64-row K block; a call after a
    larger batch checks that no stale rows reach the sums."""
    from oracle import mlp_oracle

    m = lib.MLP(seed=7)
    p = m.params()
    if P == 257:
        m.gradients(*_data(6000, 9))  # a larger batch first
    X, T = _data(P, 1)
    Y = m.predict(X)
    ref = mlp_oracle.forward(p, X, bf16_acts=True)[-1]
    assert np.linalg.norm(Y - ref) <= 1e-3 * np.linalg.norm(ref)
    g, loss = m.gradients(X, T)
    gref, lref = mlp_oracle.gradients(p, X, T, bf16_acts=True)
    assert abs(loss - lref) <= 1e-3 * lref
    at = 0
    for l in range(5):
        o, i = mlp_oracle.DIMS[l + 1], mlp_oracle.DIMS[l]
        for size in (o * i, o):
            a, b = g[at:at + size], gref[at:at + size]
            assert np.linalg.norm(a - b) <= 5e-3 * np.linalg.norm(b) + 1e-12, (l, size)
            at += size
    m.close()


def test_mlp_training_reduces_loss(lib):
    rng = np.random.default_rng(2)
    X = rng.normal(0, 1, (6000, 32)).astype(np.float32)
    T = np.stack([np.sin(X[:, 0]) + X[:, 1] * X[:, 2], np.maximum(X[:, 3], 0), 0.5 * X[:, 4] ** 2], 1).astype(np.float32)
    m = lib.MLP(seed=3)
    _, l0 = m.gradients(X, T)
    loss, ms = m.train(X, T, epochs=60, batch=1024, lr=2e-3)
    _, l1 = m.gradients(X, T)
    assert l1 < 0.1 * l0 and ms > 0
    m.close()


def test_warm_start_gain_on_held_out_scene(lib):
    from radiosity_gb300 import learned, scenes

    X, T = learned.training_set(6, seed=11, patches=(1200, 2500), W=64, tol=1e-6)
    m = lib.MLP(seed=5)
    m.train(X, T, epochs=150, batch=2048, lr=2e-3)
    sc = scenes.cornell_variant(2000, seed=987654)
    with learned.capture(sc, W=64) as s:
        E = learned.emission_block(sc)
        d = learned.direct_light(s, E)
        guess = learned.warm_start(m, sc, d)
        _, st_e = s.gather(E, tol=1e-4, max_outer=80, sweeps=4)
        _, st_l = s.gather(E, guess=guess, tol=1e-4, max_outer=80, sweeps=4)
    assert st_l.residual <= 1e-4 and st_e.residual <= 1e-4
    assert st_l.initial_residual < 0.5 * st_e.initial_residual
    assert st_l.outer <= st_e.outer
    m.close()
