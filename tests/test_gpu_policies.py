"""GPU: out-of-core policies 1/2, golden vectors, and the CLI end to end."""
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

import galp_gb300
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("path", sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if "labels" not in f),
                         ids=os.path.basename)
def test_gpu_matches_golden(path):
    z = np.load(path)
    policy, bpow = int(z["policy"]), int(z["buffer_pow"])
    g = galp_gb300.Graph(z["offsets"], z["neighbors"])
    with galp_gb300.Propagator(g, policy=policy, buffer_pow=bpow if policy else 24) as p:
        for k in range(1, len(z["counts"]) + 1):
            p.run(k)
            assert p.iters_run == k
            assert np.array_equal(p.get_labels(), z["labels"][k - 1]), f"iteration {k}"
            assert list(p.updates) == list(z["counts"][:k])


def test_gpu_sbm16k_golden():
    z = np.load(os.path.join(GOLDEN, "sbm_16k_labels.npz"))
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
    with galp_gb300.Propagator(g) as p:
        p.run(10)
        assert np.array_equal(p.get_labels(), z["labels"])
        assert list(p.updates) == list(z["counts"])


@pytest.mark.parametrize("policy", [1, 2])
@pytest.mark.parametrize("bpow", [10, 13, 16])
def test_out_of_core_matches_oracle(policy, bpow):
    g = galp_gb300.generate_rmat(14, 16, seed=6)
    nb, _ = oracle.batch_boundaries(g.offsets, bpow)
    if nb < 0:
        pytest.skip("a vertex exceeds the batch buffer")
    with galp_gb300.Propagator(g, policy=policy, buffer_pow=bpow) as p:
        for k in (1, 2, 5, 10):
            p.run(k)
            it, want, counts = oracle.run(g.offsets, g.neighbors, k, policy=policy, buffer_pow=bpow)
            assert p.iters_run == it
            assert np.array_equal(p.get_labels(), want), f"policy {policy} b {bpow} k {k}"
            assert list(p.updates) == list(counts)


def test_out_of_core_single_batch_equals_in_core():
    g = galp_gb300.generate_lfr(20000, seed=3)
    with galp_gb300.Propagator(g, policy=0) as p0, galp_gb300.Propagator(g, policy=2, buffer_pow=24) as p2:
        p0.run(10)
        p2.run(10)
        assert np.array_equal(p0.get_labels(), p2.get_labels())


def test_out_of_core_rejects_vertex_above_buffer():
    g = galp_gb300.generate_rmat(12, 16, seed=1)
    with pytest.raises(galp_gb300.GalpError) as e:
        galp_gb300.Propagator(g, policy=2, buffer_pow=4)
    assert e.value.code == -8


def test_out_of_core_reports_bad_neighbour():
    g = galp_gb300.generate_sbm([64] * 8, 6.0, 1.0, seed=2)
    nbr = g.neighbors.copy()
    nbr[-3] = g.n + 7  # out of range, caught on the device when the batch streams in
    bad = galp_gb300.Graph(g.offsets, nbr)
    p = galp_gb300.Propagator(bad, policy=2, buffer_pow=10)
    with pytest.raises(galp_gb300.GalpError) as e:
        p.run(10)
    assert e.value.code == -5
    p.close()


def test_cli_end_to_end():
    cli = galp_gb300.lib_path("galp")
    g = galp_gb300.generate_sbm([128] * 16, 10.0, 2.0, seed=8)
    with tempfile.TemporaryDirectory() as td:
        gbin = os.path.join(td, "g.bin")
        src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.offsets))
        np.stack([src, g.neighbors], 1).astype(np.int32).tofile(gbin)
        gt = os.path.join(td, "gt.txt")
        with open(gt, "w") as f:
            for b in range(16):
                f.write(" ".join(str(v) for v in range(128 * b, 128 * (b + 1))) + "\n")
        for args, proc in ((["0", "0"], "dpp\tincore"), (["-b", "12", "0", "2"], "dpp\tasync"),
                           (["1", "0"], "lfht1\tincore")):
            r = subprocess.run([cli, *args, gbin, gt], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            assert f"Data is ready on the host ({g.n}, {g.m})" in r.stdout
            row = r.stderr.strip().split("\n")[-1].split("\t")
            assert "\t".join(row[:2]) == proc and row[2] == "g.bin"
            nmi, fm, ari = map(float, row[-3:])
            assert 0.0 <= nmi <= 1.0 + 1e-9 and 0.0 <= fm <= 1.0 + 1e-9
