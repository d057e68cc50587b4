"""CPU oracle of the dispatcher's MLP (test infrastructure only; nothing in the product
imports it).  float64 numpy restatement of the network behind include/galp_tools.h
galp_mlp_*: nin -> nhid -> nhid -> nout, ReLU after the first two layers, masked mean
squared error, parameters packed as W1[nin][nhid], b1, W2[nhid][nhid], b2, W3[nhid][nout],
b3.  The GPU's forward pass and gradients are checked against it.
"""
from __future__ import annotations

import numpy as np


def unpack(w, nin, nhid, nout):
    w = np.asarray(w, np.float64)
    o = 0
    out = []
    for shape in [(nin, nhid), (nhid,), (nhid, nhid), (nhid,), (nhid, nout), (nout,)]:
        k = int(np.prod(shape))
        out.append(w[o:o + k].reshape(shape))
        o += k
    assert o == w.size
    return out


def forward(w, x, nin, nhid, nout):
    W1, b1, W2, b2, W3, b3 = unpack(w, nin, nhid, nout)
    x = np.asarray(x, np.float64)
    h1 = np.maximum(x @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3, (x, h1, h2)


def loss_grad(w, x, t, mask, nin, nhid, nout):
    """Masked MSE (sum of mask * (y - t)^2 / sum of mask) and its gradient, packed."""
    W1, b1, W2, b2, W3, b3 = unpack(w, nin, nhid, nout)
    y, (x, h1, h2) = forward(w, x, nin, nhid, nout)
    t = np.asarray(t, np.float64)
    m = np.ones_like(t) if mask is None else np.asarray(mask, np.float64)
    cnt = max(m.sum(), 1.0)
    d = (y - t) * m
    loss = float((d * d).sum() / cnt)
    dy = 2.0 * d / cnt
    gW3 = h2.T @ dy
    gb3 = dy.sum(0)
    dh2 = (dy @ W3.T) * (h2 > 0)
    gW2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    gW1 = x.T @ dh1
    gb1 = dh1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, g


def numeric_grad(w, x, t, mask, nin, nhid, nout, idx, eps=1e-6):
    """Central differences of the loss at parameter indices idx."""
    w = np.asarray(w, np.float64).copy()
    out = []
    for i in idx:
        a = w[i]
        w[i] = a + eps
        lp, _ = loss_grad(w, x, t, mask, nin, nhid, nout)
        w[i] = a - eps
        lm, _ = loss_grad(w, x, t, mask, nin, nhid, nout)
        w[i] = a
        out.append((lp - lm) / (2 * eps))
    return np.array(out)
