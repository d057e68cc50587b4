"""Parity at the benchmarked configuration: R-MAT scale 26, edge factor 28 (a,b,c,d =
.57,.19,.19,.05, seed 1; 37.5 M vertices and 3.65 G CSR entries after symmetrising,
deduplication and removal of isolated vertices).

This is the only graph in the suite whose run positions exceed 2^31 (about 3.5 G runs in
the first iteration), so it is the test of the 64-bit run bases, the tile and chunk
arithmetic of the positional tie-break and the scans above int32.  Labels and change
counts are compared with the multi-threaded closed-form oracle after each iteration:

* in-core (policy 0), all ten iterations of the benchmarked run;
* out-of-core policy 2 with 2^24-edge batches streamed from pinned host memory,
  iterations 1-3 (batch-local run positions, in-place batch order).
"""
import numpy as np
import pytest

from test_gpu_fullsize import check_every_iteration, rmat_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat26():
    g = rmat_host(26, 28)
    assert g.m > 3_500_000_000 and g.n > 30_000_000
    return g


def test_rmat26_in_core_every_iteration(rmat26):
    check_every_iteration(rmat26, range(1, 11))


def test_rmat26_policy2_b24_iterations_1_to_3(rmat26):
    check_every_iteration(rmat26, range(1, 4), policy=2, buffer_pow=24)
