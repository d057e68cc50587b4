"""Per-iteration dispatch and its MLP on the GPU: forward and gradients against the CPU
oracle, training, and exactness of every variant row and of the learned rule."""
import numpy as np
import pytest

import galp_gb300
import oracle
from galp_gb300 import tools
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu

SHAPE = (tools.NFEAT, tools.NHID, tools.NVAR)


def _data(B, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.random((B, tools.NFEAT)).astype(np.float32)
    t = rng.normal(0, 1, (B, tools.NVAR)).astype(np.float32)
    m = (rng.random((B, tools.NVAR)) < 0.9).astype(np.float32)
    return x, t, m


def test_forward_matches_oracle():
    mlp = tools.MLP(seed=3)
    x, _, _ = _data(300)
    y = mlp.forward(x)
    want, _ = mlp_oracle.forward(mlp.weights(), x, *SHAPE)
    np.testing.assert_allclose(y, want, rtol=1e-4, atol=1e-4)


def test_gradient_matches_oracle():
    mlp = tools.MLP(seed=5)
    x, t, m = _data(257, seed=1)
    loss, g = mlp.loss_grad(x, t, m)
    want_loss, want_g = mlp_oracle.loss_grad(mlp.weights(), x, t, m, *SHAPE)
    assert abs(loss - want_loss) <= 1e-4 * max(1.0, abs(want_loss))
    # FP32 sums over the batch against float64: relative to the gradient's scale
    scale = np.abs(want_g).max()
    np.testing.assert_allclose(g, want_g, rtol=1e-3, atol=1e-4 * scale)


def test_training_reduces_loss():
    rng = np.random.default_rng(2)
    x = rng.random((512, tools.NFEAT)).astype(np.float32)
    # a smooth target the network can fit
    t = np.stack([np.sin(3 * x[:, i % tools.NFEAT]) + x[:, (i + 1) % tools.NFEAT] for i in range(tools.NVAR)], 1)
    mlp = tools.MLP(seed=7)
    curve = mlp.train(x, t.astype(np.float32), steps=800, lr=3e-3)
    assert curve[-1] < 0.1 * curve[0]
    loss, _ = mlp.loss_grad(x, t.astype(np.float32))
    assert abs(loss - mlp_oracle.loss_grad(mlp.weights(), x, t, None, *SHAPE)[0]) < 1e-3


def test_variant_table():
    g = galp_gb300.generate_rmat(15, 16, seed=11)
    with galp_gb300.Propagator(g, frontier=1) as p:
        rows = tools.dispatch_table(p)
    assert len(rows) == tools.NVAR
    d = g.degrees()
    nmid = int(((d > 32) & (d <= 12288)).sum())
    for k, r in enumerate(rows):
        assert 0 <= r["pos1"] <= r["pos2"] <= nmid
        assert r["pos1"] == int(((d > 32) & (d <= r["warp_max_degree"])).sum())
        assert r["pos2"] == int(((d > 32) & (d <= r["cta256_max_degree"])).sum())
        assert r["frontier"] == (k & 1) and r["agg_mode"] == (1 if k & 8 else 2)


@pytest.mark.parametrize("narrow", [0, 1])
@pytest.mark.parametrize("row", range(16))
def test_every_variant_row_is_exact(row, narrow):
    # every row's split of the degree-sorted mid list, with and without the 64-thread CTA
    # range cut out of the 128-thread one (455 vertices of 257..512 neighbours)
    g = galp_gb300.generate_rmat(15, 16, seed=11)
    with galp_gb300.Propagator(g, frontier=1) as p:
        tools.dispatch_set(p, 2, row)
        tools.set_variant(p, cta_narrow=narrow)
        p.run(8)
        got, its, upd = p.get_labels(), p.iters_run, list(p.updates)
        _, rows = tools.dispatch_log(p)
    it, want, counts = oracle.run(g.offsets, g.neighbors, 8)
    assert its == it and upd == list(counts) and np.array_equal(got, want)
    assert all(r in (-1, row) for r in rows)


def test_learned_rule_is_exact_with_any_weights():
    g = galp_gb300.generate_lfr(20000, seed=5)
    w = tools.MLP(seed=11).weights()
    with galp_gb300.Propagator(g, frontier=1) as p:
        tools.dispatch_set(p, 1, 0, w)
        p.run(10)
        got, its = p.get_labels(), p.iters_run
        feats, rows = tools.dispatch_log(p)
    it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
    assert its == it and np.array_equal(got, want)
    assert feats.shape == (its, tools.NFEAT) and all(-1 <= r < tools.NVAR for r in rows)
    # the features the MLP saw: histogram sums to 1, changed fraction in [0, 1]
    assert abs(feats[-1, :16].sum() - 1) < 1e-4 and 0 <= feats[-1, 19] <= 1


def test_dispatch_set_validates():
    g = galp_gb300.generate_sbm([64] * 8, 8.0, 1.0, seed=1)
    with galp_gb300.Propagator(g) as p:
        with pytest.raises(RuntimeError):
            tools.dispatch_set(p, 2, 16)
        with pytest.raises(RuntimeError):
            tools.dispatch_set(p, 1, 0, np.zeros(5, np.float32))


def test_variant_defaults_and_validation():
    # the defaults this build measures with, and out-of-range knobs rejected without
    # changing the variant in force
    g = galp_gb300.generate_sbm([64] * 8, 8.0, 1.0, seed=1)
    with galp_gb300.Propagator(g) as p:
        v = tools.set_variant(p)
        assert (v.small_sort, v.cta_narrow, v.cta_stage, v.agg_mode, v.hub_part_shift, v.mid_sort) == \
            (2, 1, 0, 0, 1, 0)
        for bad in ({"small_sort": 3}, {"small_sort": -1}, {"cta_narrow": 2}, {"cta_stage": 2},
                    {"agg_mode": 3}, {"frontier_frac": 1.5}, {"hub_part_shift": 99}, {"mid_sort": 2}):
            with pytest.raises(RuntimeError):
                tools.set_variant(p, **bad)
        assert tools.set_variant(p).small_sort == 2
        p.run(5)
        it, want, counts = oracle.run(g.offsets, g.neighbors, 5)
        assert p.iters_run == it and np.array_equal(p.get_labels(), want)


def test_builtin_learned_dispatch_is_exact_and_not_slower():
    """opts.dispatch = 1 loads the network trained on this machine's timing sweeps; it
    changes only speed, and must not make a run slower than the fixed rule (2 % allowance
    for run-to-run noise of the best of three runs per iteration)."""
    g = galp_gb300.generate_rmat(19, 32, a=0.5, b=0.1667, c=0.1667, seed=9)
    times = {}
    labels = {}
    for name, kw in (("fixed", {}), ("learned", {"dispatch": 1})):
        with galp_gb300.Propagator(g, frontier=1, early_exit=0, **kw) as p:
            p.run(10)
            tools.profile(p, 1)
            tools.profile_iterations(p)
            best = None
            for _ in range(3):
                p.run(10)
                ms = tools.profile_iterations(p)
                best = ms if best is None else np.minimum(best, ms)
            times[name] = float(best.sum())
            labels[name] = p.get_labels()
    assert np.array_equal(labels["fixed"], labels["learned"])
    print(f"fixed {times['fixed']:.3f} ms, learned {times['learned']:.3f} ms, "
          f"gain {times['fixed'] / times['learned']:.3f}x")
    assert times["learned"] <= 1.02 * times["fixed"]
