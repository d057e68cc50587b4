"""Parity at benchmark-like sizes.

* LFR-style n = 1 M (the LFR configuration, methods 0 and 1): labels, iteration count and
  change counts equal the oracle after 10 iterations.
* R-MAT scale 22 (2.4 M vertices, 128 M CSR entries) and scale 24 (8.9 M vertices,
  521 M CSR entries, the R-MAT 24 configuration): labels and change counts equal the
  multi-threaded closed-form oracle after each of the ten iterations.
"""
import numpy as np
import pytest

import galp_gb300
import oracle

pytestmark = pytest.mark.gpu


def rmat_host(scale, edge_factor):
    """R-MAT graph (a,b,c,d = .57,.19,.19,.05, seed 1, symmetrised, deduplicated, isolated
    vertices removed) built on the device, returned as a host Graph."""
    import bench
    import torch

    off_d, nbr_d = bench.rmat_on_gpu(scale, edge_factor)
    g = galp_gb300.Graph(off_d.cpu().numpy(), nbr_d.cpu().numpy())
    del off_d, nbr_d
    torch.cuda.empty_cache()
    return g


def check_every_iteration(g, iterations, **opts):
    """GPU labels and change counts after each iteration in `iterations` (early exit off)
    against the multi-threaded closed-form oracle stepped from vertex IDs."""
    want = np.arange(g.n, dtype=np.int32)
    counts = []
    policy, bpow = opts.get("policy", 0), opts.get("buffer_pow", 24)
    with galp_gb300.Propagator(g, early_exit=0, **opts) as p:
        for k in range(1, max(iterations) + 1):
            want, c = oracle.step_par(g.offsets, g.neighbors, want, policy=policy, buffer_pow=bpow)
            counts.append(c)
            if k not in iterations:
                continue
            p.run(k)
            got = p.get_labels()
            assert p.iters_run == k
            assert np.array_equal(got, want), f"iteration {k}: {np.count_nonzero(got != want)} labels differ"
            assert list(p.updates) == counts, f"iteration {k}: change counts differ"


def test_rmat22_every_iteration_equals_the_oracle():
    g = rmat_host(22, 16)
    check_every_iteration(g, range(1, 11))


def test_rmat24_every_iteration_equals_the_oracle():
    # the R-MAT 24 configuration (edge factor 16): all ten iterations, from the tie-heavy
    # first ones to the converging last ones
    g = rmat_host(24, 16)
    assert g.m > 500_000_000
    check_every_iteration(g, range(1, 11))


def test_lfr_1m_ten_iterations_equal_the_oracle():
    # the LFR-style configuration at full size: n = 1,000,000, mean degree 20
    g = galp_gb300.generate_lfr(1_000_000, seed=1)
    for method in (0, 1):
        with galp_gb300.Propagator(g, method=method) as p:
            p.run(10)
            got, its, upd = p.get_labels(), p.iters_run, list(p.updates)
        it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
        assert its == it and upd == list(counts)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("narrow", [0, 1])
@pytest.mark.parametrize("stage", [0, 1])
def test_cta_staging_on_and_off_equal_the_oracle(stage, narrow):
    # CTA counting with the next vertex's neighbour IDs staged by bulk copies or read from
    # global memory, with and without the 64-thread range: the same labels, in-core and
    # out of core
    from galp_gb300 import tools

    g = galp_gb300.generate_rmat(17, 24, seed=11)
    assert ((g.degrees() > 256) & (g.degrees() <= 2048)).sum() > 100
    for opts in ({}, {"policy": 2, "buffer_pow": 18}):
        with galp_gb300.Propagator(g, early_exit=0, **opts) as p:
            tools.set_variant(p, cta_stage=stage, cta_narrow=narrow)
            want = np.arange(g.n, dtype=np.int32)
            for k in range(1, 5):
                want, _ = oracle.step_par(g.offsets, g.neighbors, want, policy=opts.get("policy", 0),
                                          buffer_pow=opts.get("buffer_pow", 24))
                p.run(k)
                assert np.array_equal(p.get_labels(), want), f"{opts} iteration {k}"


@pytest.mark.parametrize("narrow", [0, 1])
def test_narrow_cta_split_equals_the_oracle(narrow):
    # vertices of 257..512 neighbours in 64-thread CTAs (8 KB tables) or in the 128-thread
    # ones: the same labels, in-core with and without the frontier, and out of core
    from galp_gb300 import tools

    g = galp_gb300.generate_rmat(16, 24, seed=11)
    assert ((g.degrees() > 256) & (g.degrees() <= 512)).sum() > 1000
    for opts in ({}, {"frontier": 1}, {"policy": 2, "buffer_pow": 18}):
        with galp_gb300.Propagator(g, early_exit=0, **opts) as p:
            tools.set_variant(p, cta_narrow=narrow)
            want = np.arange(g.n, dtype=np.int32)
            counts = []
            for k in range(1, 6):
                want, c = oracle.step_par(g.offsets, g.neighbors, want, policy=opts.get("policy", 0),
                                          buffer_pow=opts.get("buffer_pow", 24))
                counts.append(c)
                p.run(k)
                assert np.array_equal(p.get_labels(), want), f"{opts} iteration {k}"
                assert list(p.updates) == counts
