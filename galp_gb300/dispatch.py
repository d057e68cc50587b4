"""Learned per-iteration dispatch: timing sweeps, training and evaluation.

Every in-core iteration runs one row of a 16-entry variant table (include/galp_tools.h
galp_dispatch_row): CTA-table inserts plain or warp-aggregated, the warp/CTA degree split
at 128 or 256, the 256/1024-thread CTA split at 1024 or 2048, and the frontier on or off.
All rows compute the same labels.  The fixed rule runs row 0 (row 1 once at most 5 % of
the labels changed, in frontier mode); the learned rule runs the row an MLP predicts to be
fastest from the iteration's features (degree histogram, changed fraction, distinct
labels per CSR entry, iteration index).

  sweep:    for each graph of a training set, run every row for all iterations and record
            per-iteration device times and features -> (X, T): T = log(time / fastest);
  train:    fit the MLP (galp_mlp_*: forward, backward and AdamW kernels on the GPU);
  export:   write the weights into csrc/dispatch_weights.inc (opts.dispatch = 1 uses them);
  evaluate: per-iteration time of the fixed and learned rules on a graph.

Usage (on a GPU machine):
  python -m galp_gb300.dispatch sweep --out sweep.npz
  python -m galp_gb300.dispatch train --data sweep.npz --out weights.npy [--inc]
  python -m galp_gb300.dispatch evaluate --weights weights.npy --rmat 20
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import Graph, Propagator, generate_lfr, generate_rmat, generate_sbm
from . import tools

NITER = 10
HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS_INC = os.path.join(HERE, "csrc", "dispatch_weights.inc")


def training_graphs(seed: int = 7):
    """Seeded training set: R-MAT of several scales, edge factors and skews, planted
    partitions and LFR-style graphs of several mixings (sizes that generate in seconds
    on the host)."""
    specs = []
    rmats = [(16, 8, 0.57), (17, 16, 0.57), (18, 16, 0.57), (18, 32, 0.45), (19, 8, 0.45), (19, 16, 0.57),
             (20, 16, 0.57), (20, 8, 0.50), (21, 4, 0.57), (17, 32, 0.65), (18, 8, 0.65), (19, 32, 0.50),
             (20, 32, 0.57), (21, 16, 0.57), (21, 8, 0.45), (22, 8, 0.57), (22, 16, 0.50), (16, 64, 0.57),
             (23, 16, 0.57), (24, 16, 0.57)]
    for scale, ef, a in rmats:
        b = c = (1 - a) / 3 if a < 0.57 else (1 - a) / 2.27
        specs.append((f"rmat{scale}-ef{ef}-a{a}", lambda s=scale, e=ef, a=a, b=b, c=c: generate_rmat(s, e, a, b, c,
                                                                                                     seed=seed)))
    for nb, bs, din, dout in [(64, 256, 16.0, 2.0), (256, 512, 12.0, 3.0), (32, 4096, 24.0, 6.0),
                              (1024, 128, 8.0, 4.0), (16, 16384, 20.0, 2.0)]:
        specs.append((f"sbm{nb}x{bs}", lambda nb=nb, bs=bs, din=din, dout=dout: generate_sbm([bs] * nb, din, dout,
                                                                                             seed=seed)))
    for n, mu in [(200_000, 0.3), (600_000, 0.3), (400_000, 0.1), (400_000, 0.5)]:
        specs.append((f"lfr{n}-mu{mu}", lambda n=n, mu=mu: generate_lfr(n, mu=mu, seed=seed)))
    return specs


def sweep_graph(g: Graph, niter: int = NITER, repeats: int = 2):
    """Per-iteration device ms of every variant row (frontier mode, no early exit):
    returns (features [iters, 24], times [iters, 16]); iteration 0 may be the shortcut
    (variant -1) and is dropped by the caller."""
    times = np.full((niter, tools.NVAR), np.inf)
    feats = None
    with Propagator(g, frontier=1, early_exit=0) as p:
        for k in range(tools.NVAR):
            tools.dispatch_set(p, 2, k)
            p.run(niter)  # warm-up
            tools.profile(p, 1)
            tools.profile_iterations(p)
            for _ in range(repeats):
                p.run(niter)
                ms = tools.profile_iterations(p)
                times[:len(ms), k] = np.minimum(times[:len(ms), k], ms)
            tools.profile(p, 0)
            f, v = tools.dispatch_log(p)
            if feats is None:
                feats = (f, v)
    f, v = feats
    keep = v >= 0
    return f[keep], times[:len(v)][keep]


def sweep(graphs=None, niter: int = NITER, verbose: bool = True):
    X, T, names = [], [], []
    for name, make in (graphs or training_graphs()):
        g = make()
        f, t = sweep_graph(g, niter)
        X.append(f)
        T.append(t)
        names += [name] * len(f)
        if verbose:
            best = t.argmin(1)
            print(f"{name}: n={g.n} m={g.m} fastest rows per iteration {best.tolist()} "
                  f"fixed/best {(t[:, 0] / t.min(1)).round(2).tolist()}", flush=True)
    return np.concatenate(X).astype(np.float32), np.concatenate(T), np.array(names)


def fixed_rows(X, frac: float = 0.05):
    """Rows the fixed rule runs (frontier mode): 1 once at most frac of the labels changed."""
    return np.where(X[:, 19] <= frac, 1, 0)


def targets(times):
    """Regression targets: log slowdown of every row against the iteration's fastest."""
    return np.log(times / times.min(1, keepdims=True)).astype(np.float32)


def train(X, T, steps: int = 1500, lr: float = 3e-3, seed: int = 1, weight_decay: float = 1e-3):
    mlp = tools.MLP(seed=seed)
    curve = mlp.train(X, targets(T), steps=steps, lr=lr, weight_decay=weight_decay)
    w = mlp.weights()
    mlp.close()
    return w, curve


def predict_rows(w, X, margin: float = 0.03):
    """Rows the learned rule runs: the predicted fastest, unless it beats the fixed rule's
    row by no more than margin (the device rule in lp_dispatch.cuh)."""
    mlp = tools.MLP()
    mlp.set_weights(w)
    y = mlp.forward(X)
    mlp.close()
    best = y.argmin(1)
    fixed = fixed_rows(X)
    idx = np.arange(len(X))
    return np.where(y[idx, fixed] - y[idx, best] > margin, best, fixed)


def export_inc(w, path: str = WEIGHTS_INC):
    """Write the trained weights as the library's built-in learned dispatcher."""
    body = ",\n".join(", ".join(f"{x:.9e}f" for x in w[i:i + 8]) for i in range(0, len(w), 8))
    with open(path, "w") as fh:
        fh.write("// Trained dispatcher weights (galp_mlp layout, 24 -> 64 -> 64 -> 16), written by\n"
                 "// galp_gb300/dispatch.py from timing sweeps on GB300.\n"
                 "#define GALP_HAVE_TRAINED_DISPATCH 1\n"
                 f"static const float kTrainedDispatch[{len(w)}] = {{\n{body}\n}};\n")


def evaluate(g: Graph, w, niter: int = NITER, repeats: int = 3, frontier: int = 1):
    """(fixed ms per iteration, learned ms per iteration, learned rows) on g."""
    out = {}
    with Propagator(g, frontier=frontier, early_exit=0) as p:
        for mode in (0, 1):
            tools.dispatch_set(p, mode, 0, w if mode == 1 else None)
            p.run(niter)
            tools.profile(p, 1)
            tools.profile_iterations(p)
            best = None
            for _ in range(repeats):
                p.run(niter)
                ms = tools.profile_iterations(p)
                best = ms if best is None else np.minimum(best, ms)
            tools.profile(p, 0)
            out[mode] = (float(best.sum()) / niter, tools.dispatch_log(p)[1])
    return out[0][0], out[1][0], out[1][1]


def report(X, T, names, w=None) -> str:
    """Markdown table: per training graph, the whole-run time of the fixed rule, of the
    best row in every iteration (the most any per-iteration choice over this variant set
    can gain) and of the learned rule (when weights are given)."""
    idx = np.arange(len(T))
    fixed = T[idx, fixed_rows(X)]
    best = T.min(1)
    learned = T[idx, predict_rows(w, X)] if w is not None else None
    lines = ["| graph | fixed ms | best-per-iteration ms | fixed / best |" + (" learned ms | fixed / learned |" if w is not None else ""),
             "|---|---:|---:|---:|" + ("---:|---:|" if w is not None else "")]
    for name in dict.fromkeys(names.tolist()):
        m = names == name
        row = f"| {name} | {fixed[m].sum():.3f} | {best[m].sum():.3f} | {fixed[m].sum() / best[m].sum():.3f} |"
        if learned is not None:
            row += f" {learned[m].sum():.3f} | {fixed[m].sum() / learned[m].sum():.3f} |"
        lines.append(row)
    tot = f"| **all** | {fixed.sum():.3f} | {best.sum():.3f} | {fixed.sum() / best.sum():.3f} |"
    if learned is not None:
        tot += f" {learned.sum():.3f} | {fixed.sum() / learned.sum():.3f} |"
    lines.append(tot)
    return "\n".join(lines)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m galp_gb300.dispatch")
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("sweep")
    s.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True)
    t.add_argument("--out", required=True)
    t.add_argument("--steps", type=int, default=1500)
    t.add_argument("--inc", action="store_true", help="also write csrc/dispatch_weights.inc")
    r = sub.add_parser("report", help="fixed vs per-iteration best vs learned on a sweep")
    r.add_argument("--data", required=True)
    r.add_argument("--weights", default=None, help="weights .npy (default: none, no learned column)")
    e = sub.add_parser("evaluate")
    e.add_argument("--weights", required=True)
    e.add_argument("--rmat", type=int, default=20)
    a = ap.parse_args(argv)
    if a.cmd == "sweep":
        X, T, names = sweep()
        np.savez(a.out, X=X, T=T, names=names)
    elif a.cmd == "train":
        d = np.load(a.data)
        w, curve = train(d["X"], d["T"], steps=a.steps)
        np.save(a.out, w)
        rows = predict_rows(w, d["X"])
        T = d["T"]
        idx = np.arange(len(T))
        print(f"loss {curve[0]:.4f} -> {curve[-1]:.4f}; training-set time: "
              f"fixed {T[idx, fixed_rows(d['X'])].sum():.2f} ms, learned {T[idx, rows].sum():.2f} ms, "
              f"best {T.min(1).sum():.2f} ms")
        if a.inc:
            export_inc(w)
    elif a.cmd == "report":
        d = np.load(a.data)
        print(report(d["X"], d["T"], d["names"], np.load(a.weights) if a.weights else None))
    else:
        w = np.load(a.weights)
        g = generate_rmat(a.rmat, 16, seed=3)
        f, l, rows = evaluate(g, w)
        print(f"rmat{a.rmat}: fixed {f:.3f} ms/iter, learned {l:.3f} ms/iter ({f / l:.2f}x), rows {rows.tolist()}")


if __name__ == "__main__":
    main()
