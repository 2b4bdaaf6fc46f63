"""The learned selector: device forward/backward against the numpy
restatement, training, and exactness of learned selection."""
import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from oracle import mlp_oracle, oracle

pytestmark = pytest.mark.gpu


def rand_params(seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(tc.TC_MLP_PARAM_COUNT) * 0.2).astype(np.float32)


@pytest.mark.parametrize("rows", [1, 7, 32, 33, 300])
def test_gradients_match_cpu(engine, rows):
    rng = np.random.default_rng(rows)
    w = rand_params(rows)
    X = rng.random((rows, tc.TC_MLP_FEATURES), dtype=np.float32)
    T = rng.standard_normal((rows, tc.TC_NUM_ARMS)).astype(np.float32)
    loss, grad = engine.selector_grad(w, X, T)
    ref_loss, ref_grad = mlp_oracle.loss_and_grad(w, X, T)
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
    np.testing.assert_allclose(grad, ref_grad, rtol=2e-3, atol=2e-5)


def test_numpy_oracle_gradient_is_right():
    rng = np.random.default_rng(0)
    w = rand_params(1).astype(np.float64)
    X = rng.random((5, tc.TC_MLP_FEATURES))
    T = rng.standard_normal((5, tc.TC_NUM_ARMS))
    _, g = mlp_oracle.loss_and_grad(w, X, T)
    for p in rng.choice(len(w), 40, replace=False):
        e = np.zeros_like(w)
        e[p] = 1e-6
        num = (mlp_oracle.loss_and_grad(w + e, X, T)[0] - mlp_oracle.loss_and_grad(w - e, X, T)[0]) / 2e-6
        assert abs(num - g[p]) < 1e-6 + 1e-4 * abs(g[p])


def test_predict_matches_bf16_forward(engine):
    rng = np.random.default_rng(2)
    w = rand_params(3)
    engine.set_selector_weights(w)
    X = rng.random((100, tc.TC_MLP_FEATURES), dtype=np.float32)
    pred = engine.selector_predict(X)
    import torch
    wb = torch.from_numpy(w).to(torch.bfloat16).to(torch.float32).numpy().astype(np.float64)
    ref, _ = mlp_oracle.forward(wb, X.astype(np.float64))
    np.testing.assert_allclose(pred, ref, rtol=1e-3, atol=1e-3)
    assert np.array_equal(engine.get_selector_weights(), w)


def test_training_fits_synthetic_costs(engine):
    rng = np.random.default_rng(4)
    X = rng.random((4000, tc.TC_MLP_FEATURES), dtype=np.float32)
    # arm k is cheap when feature k is large: a learnable rule
    costs = (2.0 ** (10 + 4 * (1 - X[:, :tc.TC_NUM_ARMS]))).astype(np.float32)
    loss = engine.train_selector(X, costs, epochs=40, lr=3e-3, seed=1)
    pred = engine.selector_predict(X)
    acc = np.mean(pred.argmin(1) == costs.argmin(1))
    y = mlp_oracle.targets(costs)
    assert loss < 0.25 * np.mean(0.5 * y ** 2)
    assert acc > 0.8


def test_learned_selection_is_exact(engine):
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=15, edge_factor=16, seed=21))
    rowptr, colidx = oracle.csr_from_edges(n, s, d)
    feats, costs = engine.tile_profile(rowptr, colidx)
    assert feats.shape[0] == costs.shape[0] > 0 and np.all(costs > 0)
    engine.train_selector(feats, costs, epochs=30, lr=3e-3, seed=2)
    ref, ref_pe, _, _ = oracle.triangles(rowptr, colidx, per_edge=True)
    total, pe, st = engine.count(rowptr, colidx, selector="learned", edge_counts=True)
    assert total == ref and np.array_equal(pe, ref_pe)
    assert sum(st["tiles_per_arm"].values()) == st["tiles"]


def test_shipped_selector_gains_over_fixed_rule(engine):
    """What the trained network gains: on a held-out R-MAT graph (a seed and
    the default (0.57, 0.19, 0.19) parameters that training never saw), the
    shipped weights pick arms whose summed per-tile cost is closer to the
    per-tile best than the fixed thresholds' picks (the tile cost model the
    selector is trained on; timed end to end the two tie at scale 24)."""
    from pathlib import Path
    w = np.load(Path(tc.__file__).resolve().parent / "data" / "selector_mlp.npz")["params"].astype(np.float32)
    try:
        old = engine.get_selector_weights()
    except tc.TCError:  # nothing loaded yet
        old = None
    engine.set_selector_weights(w)
    engine.set_selector_margin(0.0)  # the network's own picks, before the switching margin
    try:
        n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=18, edge_factor=16, seed=99))
        rowptr, colidx = oracle.csr_from_edges(n, s, d)
        feats, costs = engine.tile_profile(rowptr, colidx)
        best = costs.min(axis=1).sum()
        rows = np.arange(len(costs))
        learned = engine.plan_arms(rowptr, colidx, selector="learned")
        fixed = engine.plan_arms(rowptr, colidx, selector="fixed")
        regret_learned = costs[rows, learned].sum() / best
        regret_fixed = costs[rows, fixed].sum() / best
        assert regret_learned < regret_fixed, (regret_learned, regret_fixed)
        assert regret_learned < 1.05
    finally:
        if old is not None:
            engine.set_selector_weights(old)


def test_learned_selection_falls_back_to_the_fixed_rule(engine):
    """The learned selection keeps the fixed rule's PULL decision on every
    tile, and with a margin no predicted gain reaches it picks the fixed
    rule's arm everywhere (the fixed rule is the fallback)."""
    assert engine.load_shipped_selector()
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=18, edge_factor=16, seed=98))
    rowptr, colidx = oracle.csr_from_edges(n, s, d)
    pull = tc.ARM_NAMES.index("pull")
    fixed = engine.plan_arms(rowptr, colidx, selector="fixed")
    try:
        engine.set_selector_margin(0.0)
        learned = engine.plan_arms(rowptr, colidx, selector="learned")
        assert np.array_equal(learned == pull, fixed == pull)
        engine.set_selector_margin(64.0)
        assert np.array_equal(engine.plan_arms(rowptr, colidx, selector="learned"), fixed)
        with pytest.raises(tc.TCError):
            engine.set_selector_margin(-1.0)
    finally:
        engine.load_shipped_selector()
