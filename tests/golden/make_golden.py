"""Generate the golden label vectors in tests/golden/ from the reference's own kernels.

Run where the reference tree is present (it builds oracle/_ref/ref_harness, which
compiles label_propagation/src/dpp/kernel.cuh and src/common/segmented_reduce.cuh
and executes them on the CPU through oracle/refsim/simt_shim.h):

    python tests/golden/make_golden.py

Each fixture stores the input graph (CSR) and, per iteration, the labels and the
exact number of changed labels produced by the reference kernels.  The reference
ships no tests or golden vectors of its own; these are the pinned outputs that the
oracle and the GPU path are checked against.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import galp_gb300  # noqa: E402
import oracle  # noqa: E402


def write_bin(g, path):
    src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.offsets))
    np.stack([src, g.neighbors.astype(np.int32)], 1).astype(np.int32).tofile(path)


# the reference tree: $GALP_REFERENCE, else a directory named "reference" beside the repository
_REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REFERENCE = os.environ.get("GALP_REFERENCE", os.path.join(os.path.dirname(_REPO), "reference"))


def sample_graph():
    # the reference's only checked-in input (datasets/sample.txt), read from its tree
    path = os.path.join(REFERENCE, "datasets", "sample.txt")
    edges = [tuple(map(int, line.split())) for line in open(path)]
    adj = [[] for _ in range(1 + max(max(e) for e in edges))]
    for u, v in edges:  # include/graph.h:166-188: symmetrised in file order
        adj[u].append(v)
        adj[v].append(u)
    off = np.zeros(len(adj) + 1, np.int64)
    off[1:] = np.cumsum([len(a) for a in adj])
    return galp_gb300.Graph(off, np.array([x for a in adj for x in a], np.int32))


def record(name, g, niter, policy=0, buffer_pow=0, extra=None):
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "g.bin")
        write_bin(g, path)
        labels, counts = oracle.ref_run(path, niter, policy, buffer_pow)
    out = dict(offsets=g.offsets, neighbors=g.neighbors, labels=labels, counts=counts,
               policy=np.int64(policy), buffer_pow=np.int64(buffer_pow), niter=np.int64(niter))
    if extra:
        out.update(extra)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(f"{name}: n={g.n} m={g.m} iterations={len(counts)} counts={counts.tolist()}")


def main():
    from galp_gb300.build import build

    build()
    if not oracle.ref_available():
        raise SystemExit("reference harness not built (reference tree missing)")
    record("sample.npz", sample_graph(), 6)
    record("sbm_4k.npz", galp_gb300.generate_sbm([256] * 16, 12.0, 3.0, seed=21), 10)
    record("rmat12.npz", galp_gb300.generate_rmat(12, 16, seed=5), 10)
    record("rmat12_policy2_b12.npz", galp_gb300.generate_rmat(12, 16, seed=5), 10, policy=2, buffer_pow=12)
    record("lfr_5k.npz", galp_gb300.generate_lfr(5000, seed=9), 10)
    # SBM config of the benchmark suite (n = 16,384): store labels only, with a graph digest
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "g.bin")
        write_bin(g, path)
        labels, counts = oracle.ref_run(path, 10)
    np.savez_compressed(os.path.join(HERE, "sbm_16k_labels.npz"), labels=labels[-1], counts=counts,
                        m=np.int64(g.m), nbr_sum=np.int64(g.neighbors.astype(np.int64).sum()),
                        nbr_wsum=np.int64((g.neighbors.astype(np.int64) * np.arange(g.m, dtype=np.int64)).sum()))
    print(f"sbm_16k_labels.npz: n={g.n} m={g.m} counts={counts.tolist()}")


if __name__ == "__main__":
    main()
