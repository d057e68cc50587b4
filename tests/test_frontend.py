"""Front end: loaders and accuracy measures vs the reference's own host code; CLI parsing."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import galp_gb300
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _HG(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("offsets", ctypes.POINTER(ctypes.c_int64)),
                ("neighbors", ctypes.POINTER(ctypes.c_int32))]


def _host():
    L = ctypes.CDLL(galp_gb300.lib_path("libgalp_host.so"))
    L.galp_load_graph.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(_HG))]
    L.galp_load_graph.restype = ctypes.c_int
    L.galp_host_graph_free.argtypes = [ctypes.POINTER(_HG)]
    for f in ("galp_nmi", "galp_f_measure", "galp_ari"):
        getattr(L, f).argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        getattr(L, f).restype = ctypes.c_double
    return L


def load(path):
    L = _host()
    p = ctypes.POINTER(_HG)()
    rc = L.galp_load_graph(path.encode(), ctypes.byref(p))
    assert rc == 0
    g = p.contents
    off = np.ctypeslib.as_array(g.offsets, (g.n + 1,)).copy()
    nbr = np.ctypeslib.as_array(g.neighbors, (max(g.m, 1),))[: g.m].copy()
    L.galp_host_graph_free(p)
    return off, nbr


def _write_txt(path, edges):
    with open(path, "w") as f:
        for u, v in edges:
            f.write(f"{u} {v}\n")


def _random_txt_edges(rng, n, m):
    u = rng.integers(0, n - 1, m)
    v = u + 1 + rng.integers(0, n - 1 - u.max(initial=0) + 1, m) % np.maximum(1, n - 1 - u)
    v = np.minimum(v, n - 1)
    return [(int(a), int(b)) for a, b in zip(u, v) if a < b]


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built")


@needs_ref
@pytest.mark.parametrize("fmt", ["txt", "dat", "bin"])
def test_loader_matches_reference_csr(fmt):
    rng = np.random.default_rng(3)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "g." + fmt)
        if fmt == "bin":
            g = galp_gb300.generate_rmat(12, 8, seed=2)
            src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.offsets))
            np.stack([src, g.neighbors], 1).astype(np.int32).tofile(path)
        else:
            _write_txt(path, _random_txt_edges(rng, 3000, 20000))
        off, nbr = load(path)
        oo, on = os.path.join(td, "o.bin"), os.path.join(td, "n.bin")
        subprocess.run([oracle.REF_HARNESS, "csr", path, oo, on], check=True, stdout=subprocess.DEVNULL)
        assert np.array_equal(off, np.fromfile(oo, np.int64))
        assert np.array_equal(nbr, np.fromfile(on, np.int32))


@needs_ref
def test_bin_loader_renumbers_groups_like_reference():
    # sources 0, 2, 5 (1, 3, 4 absent): the reference numbers vertices by group order
    pairs = np.array([[0, 2], [0, 5], [2, 0], [5, 0], [5, 2], [2, 5]], np.int32)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "g.bin")
        pairs.tofile(path)
        off, nbr = load(path)
        oo, on = os.path.join(td, "o.bin"), os.path.join(td, "n.bin")
        subprocess.run([oracle.REF_HARNESS, "csr", path, oo, on], check=True, stdout=subprocess.DEVNULL)
        assert np.array_equal(off, np.fromfile(oo, np.int64))
        assert np.array_equal(nbr, np.fromfile(on, np.int32))


@needs_ref
def test_accuracy_matches_reference():
    L = _host()
    g = galp_gb300.generate_lfr(3000, seed=4)
    rng = np.random.default_rng(1)
    with tempfile.TemporaryDirectory() as td:
        gt = os.path.join(td, "gt.txt")
        members = {}
        for v, c in enumerate(g.community):
            members.setdefault(int(c), []).append(v)
        with open(gt, "w") as f:
            for c in sorted(members):
                f.write(" ".join(map(str, members[c])) + "\n")
        for trial in range(3):
            if trial == 0:
                labels = g.community.astype(np.int32)  # perfect
            elif trial == 1:
                it, labels, _ = oracle.run(g.offsets, g.neighbors, 10)
            else:
                labels = rng.integers(0, 50, g.n).astype(np.int32)
            lf = os.path.join(td, "l.bin")
            labels.tofile(lf)
            out = subprocess.run([oracle.REF_HARNESS, "acc", gt, lf], check=True, capture_output=True, text=True)
            ref = [float(x) for x in out.stdout.split("ACC")[1].split()]
            got = [L.galp_nmi(gt.encode(), labels.ctypes.data, g.n), L.galp_f_measure(gt.encode(), labels.ctypes.data, g.n),
                   L.galp_ari(gt.encode(), labels.ctypes.data, g.n)]
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-14), (trial, got, ref)


def test_cli_usage_and_unsupported_policies():
    cli = galp_gb300.lib_path("galp")
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage:" in r.stderr and "method policy data [test]" in r.stderr
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "s.txt")
        _write_txt(path, [(0, 1), (0, 2), (1, 2), (2, 3)])
        r = subprocess.run([cli, "0", "3", path], capture_output=True, text=True)
        assert r.returncode == 1 and "Data is ready on the host (4, 8)" in r.stdout
        assert "----------dpp\thybrid----------" in r.stdout
