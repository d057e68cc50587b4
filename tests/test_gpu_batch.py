"""Batched mode: every graph of a batch gets exactly its standalone labels, iteration
count and change counts (one CUDA-graph launch for the whole batch)."""
import numpy as np
import pytest

import galp_gb300
import oracle

pytestmark = pytest.mark.gpu


def _mixed_graphs(count=40, seed=0):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(count):
        kind = i % 4
        if kind == 0:
            k = int(rng.integers(4, 40))
            n_blk = int(rng.integers(16, 400))
            graphs.append(galp_gb300.generate_sbm([n_blk] * k, 12.0, 3.0, seed=100 + i))
        elif kind == 1:
            graphs.append(galp_gb300.generate_lfr(int(rng.integers(2000, 20000)), seed=200 + i))
        elif kind == 2:
            graphs.append(galp_gb300.generate_rmat(int(rng.integers(8, 13)), 8, seed=300 + i))
        else:  # tiny: path and star with an isolated vertex
            n = int(rng.integers(2, 30))
            src = np.arange(n - 1)
            dst = src + 1
            s = np.concatenate([src, dst])
            d = np.concatenate([dst, src])
            order = np.lexsort((d, s))
            off = np.zeros(n + 2, np.int64)
            np.add.at(off, s[order] + 1, 1)
            graphs.append(galp_gb300.Graph(np.cumsum(off), d[order].astype(np.int32)))
    return graphs


def _standalone(g, niter, early_exit=1):
    with galp_gb300.Propagator(g, early_exit=early_exit) as p:
        p.run(niter)
        return p.get_labels(), p.iters_run, list(p.updates)


@pytest.mark.parametrize("early_exit", [1, 0])
def test_batch_equals_standalone_runs(early_exit):
    graphs = _mixed_graphs()
    with galp_gb300.Batch(graphs, early_exit=early_exit) as b:
        b.run(10)
        for i, g in enumerate(graphs):
            lab, its, upd = _standalone(g, 10, early_exit)
            bi, bupd = b.graph_stats(i)
            assert bi == its and bupd == upd, f"graph {i}: iterations/changes differ"
            assert np.array_equal(b.labels(i), lab), f"graph {i}: labels differ"


def test_batch_matches_the_oracle_and_graphs_exit_separately():
    graphs = _mixed_graphs(12, seed=3)
    with galp_gb300.Batch(graphs) as b:
        b.run(10)
        iters = []
        for i, g in enumerate(graphs):
            it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
            bi, bupd = b.graph_stats(i)
            assert bi == it and bupd == list(counts)
            assert np.array_equal(b.labels(i), want)
            iters.append(bi)
    assert len(set(iters)) > 1  # the early exit really is per graph


def test_repeat_runs_and_tuning_keep_labels():
    graphs = _mixed_graphs(16, seed=5)
    with galp_gb300.Batch(graphs) as b:
        b.run(10)
        first = b.all_labels()
        res = b.tune(2)
        assert res["trials"] >= 4 and res["small_blocks_per_sm"] in (8, 16, 24, 32)
        assert res["dispatch_row"] == -1 or res["dispatch_row"] in range(0, 16, 2)  # bucket shapes
        b.run(10)
        assert np.array_equal(b.all_labels(), first)
        b.run(4)  # another iteration count: a new captured graph
        for i, g in enumerate(graphs):
            lab, its, upd = _standalone(g, 4)
            assert np.array_equal(b.labels(i), lab)


def test_run_batch_one_shot():
    import ctypes
    graphs = _mixed_graphs(8, seed=7)
    L = galp_gb300.load_library()
    csrs = (galp_gb300._Csr * len(graphs))()
    keep = []
    for i, g in enumerate(graphs):
        off = np.ascontiguousarray(g.offsets, np.int64)
        nbr = np.ascontiguousarray(g.neighbors, np.int32)
        keep += [off, nbr]
        csrs[i] = galp_gb300._Csr(nbr.ctypes.data if len(nbr) else None, off.ctypes.data, g.n, g.m)
    total = sum(g.n for g in graphs)
    out = np.zeros(total, np.int32)
    stats = (galp_gb300.Stats * len(graphs))()
    opts = galp_gb300.default_opts()
    rc = L.galp_run_batch(csrs, len(graphs), ctypes.byref(opts), 10, out.ctypes.data, stats)
    assert rc == 0
    pos = 0
    for i, g in enumerate(graphs):
        lab, its, upd = _standalone(g, 10)
        assert np.array_equal(out[pos:pos + g.n], lab) and stats[i].iters_run == its
        pos += g.n


def test_edges_leaving_their_graph_are_rejected():
    a = galp_gb300.generate_sbm([32] * 4, 6.0, 1.0, seed=1)
    b = galp_gb300.generate_sbm([32] * 4, 6.0, 1.0, seed=2)
    off = np.concatenate([a.offsets[:-1], b.offsets + a.m])
    nbr = np.concatenate([a.neighbors, b.neighbors + a.n]).astype(np.int32)
    nbr[0] = a.n + 3  # an edge of graph 0 into graph 1
    v0 = np.array([0, a.n, a.n + b.n], np.int64)
    with pytest.raises(galp_gb300.GalpError) as e:
        galp_gb300.Batch(offsets=off, neighbors=nbr, graph_v0=v0)
    assert e.value.code == -5


def test_hub_vertices_are_not_supported_in_batches():
    g = galp_gb300.generate_rmat(17, 16, seed=11)  # a vertex above 12288 neighbours
    with pytest.raises(galp_gb300.GalpError) as e:
        galp_gb300.Batch([g, galp_gb300.generate_sbm([64] * 4, 6.0, 1.0, seed=1)])
    assert e.value.code == -6


def test_thread_per_vertex_small_counting_in_batches():
    # small_sort = 2 (one thread per small vertex) inside a captured batched run: every
    # graph keeps its standalone labels, iteration count and change counts
    from galp_gb300 import tools

    graphs = _mixed_graphs(12, seed=11)
    with galp_gb300.Batch(graphs) as b:
        b.run(10)
        first = b.all_labels()
        tools.set_variant(b, small_sort=2)
        b.run(10)
        assert np.array_equal(b.all_labels(), first)
        for i, g in enumerate(graphs):
            it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
            assert b.graph_stats(i) == (it, list(counts))
