"""The CPU oracle, pinned against the reference's own kernels and the golden vectors."""
import glob
import os
import tempfile

import numpy as np
import pytest

import galp_gb300
import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if "labels" not in os.path.basename(f))


@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
@pytest.mark.parametrize("literal", [True, False], ids=["literal", "closed"])
def test_oracle_matches_golden(path, literal):
    z = np.load(path)
    policy, bpow = int(z["policy"]), int(z["buffer_pow"])
    labels, counts = z["labels"], z["counts"]
    for k in range(1, len(counts) + 1):
        it, lab, cnt = oracle.run(z["offsets"], z["neighbors"], k, policy=policy, buffer_pow=bpow, literal=literal)
        assert it == k
        assert np.array_equal(lab, labels[k - 1]), f"iteration {k}"
        assert np.array_equal(cnt, counts[:k])


def test_oracle_sbm16k_golden():
    z = np.load(os.path.join(GOLDEN, "sbm_16k_labels.npz"))
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
    assert g.m == int(z["m"]) and int(g.neighbors.astype(np.int64).sum()) == int(z["nbr_sum"])
    it, lab, cnt = oracle.run(g.offsets, g.neighbors, 10)
    assert np.array_equal(cnt, z["counts"]) and np.array_equal(lab, z["labels"])


def _random_segments(rng, N, max_len):
    starts = [0]
    while True:
        ln = int(rng.integers(1, max_len + 1)) if rng.random() < 0.97 else int(rng.integers(1, 40 * max_len))
        if starts[-1] + ln >= N:
            break
        starts.append(starts[-1] + ln)
    return np.array(starts, np.int64)


@pytest.mark.parametrize("TB,ET", [(32, 3), (32, 1), (64, 2), (256, 17)])
def test_closed_form_matches_literal_reduce(TB, ET):
    """Closed-form tie rule vs literal emulation of segmented_reduce.cuh across chunk,
    tile, spine-block and level-2 boundaries (small TB/ET reach every level)."""
    rng = np.random.default_rng(TB * 100 + ET)
    EB = TB * ET
    for trial in range(6):
        # enough runs for several level-2 chunks when TB is small
        N = int(rng.integers(1, 4)) * TB * TB * EB + int(rng.integers(0, EB)) if TB <= 64 else int(
            rng.integers(1, 3)) * TB * EB + int(rng.integers(0, EB))
        w = rng.integers(1, 4, size=N).astype(np.int32)
        if trial % 2:
            w[:] = 1  # all ties
        seg = _random_segments(rng, N, max(3, EB // 3))
        lit, cf = oracle.seg_reduce_check(w, seg, TB, ET)
        assert np.array_equal(lit, cf), f"trial {trial}: {np.count_nonzero(lit != cf)} segments differ"


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built (needs the reference tree)")
@pytest.mark.parametrize("TB,ET", [(32, 3), (64, 2), (256, 17)])
def test_literal_reduce_matches_reference_kernels(TB, ET):
    """The literal restatement equals segmented_reduce<TB,ET> + spine + spine2 of the reference.

    The reference kernel needs 2*TB <= TB*ET + 1 (its Hillis-Steele double buffer lives
    in the EB+1-entry shared arrays), so ET >= 2; the reference itself uses ET = 17."""
    rng = np.random.default_rng(7 + TB + ET)
    EB = TB * ET
    for trial in range(4):
        N = (int(rng.integers(1, 3)) * TB * TB * EB if TB <= 64 else 2 * TB * EB) + int(rng.integers(1, EB))
        w = rng.integers(1, 4, size=N).astype(np.int32)
        if trial % 2:
            w[:] = 1
        seg = _random_segments(rng, N, max(3, EB // 3))
        lit, _ = oracle.seg_reduce_check(w, seg, TB, ET)
        ref = oracle.ref_segreduce(w, seg, TB, ET)
        assert np.array_equal(lit, ref.astype(np.int64)), f"trial {trial}"


def _write_bin(g, path):
    src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.offsets))
    np.stack([src, g.neighbors.astype(np.int32)], 1).astype(np.int32).tofile(path)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built (needs the reference tree)")
@pytest.mark.parametrize("policy,bpow", [(0, 0), (1, 11), (2, 13)])
def test_oracle_matches_reference_on_random_graphs(policy, bpow):
    for seed in range(3):
        g = galp_gb300.generate_rmat(11 + seed, 8, seed=100 + seed)
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "g.bin")
            _write_bin(g, path)
            ref_labels, ref_counts = oracle.ref_run(path, 10, policy, bpow)
        for k in (1, 2, len(ref_counts)):
            it, lab, cnt = oracle.run(g.offsets, g.neighbors, k, policy=policy, buffer_pow=bpow, literal=True)
            assert np.array_equal(lab, ref_labels[k - 1]) and np.array_equal(cnt, ref_counts[:k])
            it, lab, cnt = oracle.run(g.offsets, g.neighbors, k, policy=policy, buffer_pow=bpow)
            assert np.array_equal(lab, ref_labels[k - 1])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built (needs the reference tree)")
def test_oracle_matches_reference_past_one_spine_block():
    """A graph with more than 256 tiles of runs (> 1.1 M runs) exercises spine2."""
    g = galp_gb300.generate_sbm([512] * 160, 15.0, 1.0, seed=12)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "g.bin")
        _write_bin(g, path)
        ref_labels, ref_counts = oracle.ref_run(path, 2)
    assert g.m > 1_114_112
    it, lab, cnt = oracle.run(g.offsets, g.neighbors, 2, literal=True)
    assert np.array_equal(lab, ref_labels[-1]) and np.array_equal(cnt, ref_counts)
    it, lab, cnt = oracle.run(g.offsets, g.neighbors, 2)
    assert np.array_equal(lab, ref_labels[-1])


def test_batch_boundaries_follow_reference_rule():
    g = galp_gb300.generate_rmat(10, 8, seed=3)
    nb, bbs = oracle.batch_boundaries(g.offsets, 10)
    assert nb > 1 and bbs[0] == 0 and bbs[-1] == g.n
    edges = g.offsets[bbs[1:]] - g.offsets[bbs[:-1]]
    assert (edges < (1 << 10)).all()
    # a vertex with 2^b or more edges makes the reference loop forever; the oracle reports it
    nb, _ = oracle.batch_boundaries(g.offsets, 3)
    assert nb == -3


def test_degree_zero_vertices_equal_compacted_graph():
    g = galp_gb300.generate_sbm([64] * 6, 6.0, 1.0, seed=4)
    new_n = g.n + 3
    iso = np.array([0, 5, new_n - 1])
    keep = np.setdiff1d(np.arange(new_n), iso)
    deg = np.zeros(new_n, np.int64)
    deg[keep] = g.degrees()
    off = np.zeros(new_n + 1, np.int64)
    off[1:] = np.cumsum(deg)
    nbr = keep[g.neighbors].astype(np.int32)
    it2, lab2, cnt2 = oracle.run(off, nbr, 10)
    it, lab, cnt = oracle.run(g.offsets, g.neighbors, 10)
    assert np.array_equal(keep[lab], lab2[keep])
    assert (lab2[iso] == iso).all()


def test_fixed_iteration_count_runs_past_convergence():
    # early exit off: all iterations run (zero changes once converged) and the labels are
    # those of the early-exit run; the first iterations' counts agree
    g = galp_gb300.generate_sbm([64] * 8, 10.0, 0.5, seed=4)
    it_e, lab_e, cnt_e = oracle.run(g.offsets, g.neighbors, 30)
    it_f, lab_f, cnt_f = oracle.run(g.offsets, g.neighbors, 30, early_exit=False)
    assert it_e < 30 and it_f == 30 and len(cnt_f) == 30
    assert np.array_equal(lab_e, lab_f)
    assert list(cnt_f[:it_e]) == list(cnt_e)
    assert (cnt_f[it_e:] <= cnt_e[-1]).all()


@pytest.mark.parametrize("TB,ET", [(8, 3), (32, 2), (256, 17)])
@pytest.mark.parametrize("policy,bpow", [(0, 24), (1, 11), (2, 12)])
def test_parallel_oracle_equals_sequential(policy, bpow, TB, ET):
    """The multi-threaded closed form (used at the R-MAT 24/26 sizes) equals the sequential
    restatement: graphs with ties, hubs, isolated vertices (leading, inner and trailing),
    small TB/ET so that runs cross chunk, tile, spine-block and level-2 boundaries."""
    graphs = [galp_gb300.generate_rmat(12, 8, seed=31), galp_gb300.generate_sbm([128] * 12, 10.0, 2.0, seed=5)]
    g = graphs[1]
    new_n = g.n + 3
    iso = np.array([0, 7, new_n - 1])
    keep = np.setdiff1d(np.arange(new_n), iso)
    deg = np.zeros(new_n, np.int64)
    deg[keep] = g.degrees()
    off = np.zeros(new_n + 1, np.int64)
    off[1:] = np.cumsum(deg)
    graphs.append(galp_gb300.Graph(off, keep[g.neighbors].astype(np.int32)))
    for g in graphs:
        if policy and oracle.batch_boundaries(g.offsets, bpow)[0] < 0:
            continue
        it, lab, cnt = oracle.run(g.offsets, g.neighbors, 8, policy=policy, buffer_pow=bpow, early_exit=False,
                                  TB=TB, ET=ET)
        it2, lab2, cnt2 = oracle.run_par(g.offsets, g.neighbors, 8, policy=policy, buffer_pow=bpow,
                                         early_exit=False, TB=TB, ET=ET)
        assert it == it2 and np.array_equal(lab, lab2) and np.array_equal(cnt, cnt2)
        # stepping from given labels is the same update
        lab3 = np.arange(g.n, dtype=np.int32)
        for k in range(3):
            lab3, c = oracle.step_par(g.offsets, g.neighbors, lab3, policy=policy, buffer_pow=bpow, TB=TB, ET=ET)
            assert c == cnt[k]
        it4, lab4, _ = oracle.run(g.offsets, g.neighbors, 3, policy=policy, buffer_pow=bpow, early_exit=False,
                                  TB=TB, ET=ET)
        assert np.array_equal(lab3, lab4)


def test_parallel_oracle_early_exit_and_golden():
    for path in FIXTURES:
        z = np.load(path)
        policy, bpow = int(z["policy"]), int(z["buffer_pow"])
        it, lab, cnt = oracle.run_par(z["offsets"], z["neighbors"], len(z["counts"]), policy=policy,
                                      buffer_pow=bpow)
        assert np.array_equal(lab, z["labels"][it - 1]) and np.array_equal(cnt, z["counts"][:it])
    g = galp_gb300.generate_sbm([64] * 8, 10.0, 0.5, seed=4)
    assert oracle.run(g.offsets, g.neighbors, 30)[0] == oracle.run_par(g.offsets, g.neighbors, 30)[0]
