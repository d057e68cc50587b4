"""bench.py's CPU-side pieces: the reference arm builds its R-MAT graph without the
project's libraries (torch restatement of the counter-based sampler), and the CPU baseline
times a strided vertex sample that depends on the graph only."""
import ctypes
import math

import numpy as np

import bench
import galp_gb300
import oracle


def test_torch_sampler_equals_library_sampler():
    G = galp_gb300.load_generators()
    G.galp_rmat_edge.restype = ctypes.c_uint64
    G.galp_rmat_edge.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint32]
    ta, tb, tc = (int(math.floor(x * 4294967296.0 + 0.5)) for x in (0.57, 0.76, 0.95))
    for seed, scale, e0 in ((1, 26, 0), (1, 26, (28 << 26) - 500), (7, 12, 1000), (2**63 + 5, 31, 12345)):
        got = bench.rmat_keys_torch(seed, scale, e0, e0 + 500, device="cpu").numpy().astype(np.uint64)
        want = np.array([G.galp_rmat_edge(seed, e, scale, ta, tb, tc) for e in range(e0, e0 + 500)], np.uint64)
        assert np.array_equal(got, want)


def test_reference_arm_graph_equals_generator():
    # the whole graph build (symmetrise, dedupe, drop isolated vertices, compact IDs)
    for scale, ef, seed in ((10, 16, 1), (9, 8, 5)):
        off, nbr = bench.rmat_on_gpu(scale, ef, seed=seed, sampler="torch", device="cpu")
        g = galp_gb300.generate_rmat(scale, ef, seed=seed)
        assert np.array_equal(off.numpy(), g.offsets) and np.array_equal(nbr.numpy(), g.neighbors)


def test_cpu_sample_is_strided_and_deterministic():
    g = galp_gb300.generate_rmat(12, 16, seed=2)
    stride = 7
    secs, used, edges, counts = oracle.cpu_baseline_strided(g.offsets, g.neighbors, 3, stride, 0, 2)
    deg = np.diff(g.offsets)
    assert edges == int(deg[::stride].sum()) and used == 2 and len(counts) == 3
    assert counts[0] > 0 and (counts <= len(deg[::stride])).all()
    assert bench.cpu_sample_stride(3_647_441_114) == 14 and bench.cpu_sample_stride(1000) == 1
    s = bench.cpu_sample(g, threads=2)
    assert s["stride"] == 1 and s["edges"] == g.m
