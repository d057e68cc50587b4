"""The dispatcher MLP's CPU oracle checks itself: backprop against central differences."""
import numpy as np

from oracle import mlp_oracle


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nin, nhid, nout, B = 6, 9, 4, 13
    size = nin * nhid + nhid + nhid * nhid + nhid + nhid * nout + nout
    w = rng.normal(0, 0.5, size)
    x = rng.normal(0, 1, (B, nin))
    t = rng.normal(0, 1, (B, nout))
    mask = (rng.random((B, nout)) < 0.8).astype(float)
    loss, g = mlp_oracle.loss_grad(w, x, t, mask, nin, nhid, nout)
    idx = rng.choice(size, 60, replace=False)
    num = mlp_oracle.numeric_grad(w, x, t, mask, nin, nhid, nout, idx)
    assert loss > 0
    np.testing.assert_allclose(g[idx], num, rtol=1e-5, atol=1e-8)


def test_oracle_layout():
    nin, nhid, nout = 24, 64, 16
    size = nin * nhid + nhid + nhid * nhid + nhid + nhid * nout + nout
    parts = mlp_oracle.unpack(np.arange(size, dtype=float), nin, nhid, nout)
    assert [p.shape for p in parts] == [(24, 64), (64,), (64, 64), (64,), (64, 16), (16,)]
    assert parts[1][0] == nin * nhid
