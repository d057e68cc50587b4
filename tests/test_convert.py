"""galp_convert (galp_gb300/host/convert.cpp): the edge-list converters.

edgelist2bin --one-direction must write exactly the bytes of the reference's
utils/edgelist2bin.cpp (built from the reference tree into oracle/_ref/ when present);
the default output adds the reverse direction of every pair (the format the reference's
README and its .bin loader describe), and loads as a symmetric CSR with the same vertex
count.  normalize must write exactly what the reference's utils/normalize.py writes for
the edges, and one line per ground-truth community."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CONVERT = os.path.join(ROOT, "galp_gb300", "lib", "galp_convert")
REF_E2B = os.path.join(ROOT, "oracle", "_ref", "edgelist2bin")


def _snap_file(path, seed=3):
    """A SNAP-style edge list: comment lines, tab separators, IDs with gaps, both
    directions of some edges, repeated lines and self-loops."""
    rng = np.random.default_rng(seed)
    ids = np.sort(rng.choice(10_000, 300, replace=False)) * 7 + 11
    u = rng.choice(ids, 1500)
    v = rng.choice(ids, 1500)
    lines = ["# Undirected graph: synthetic", "# Nodes: 300 Edges: 1500", "# FromNodeId\tToNodeId"]
    for a, b in zip(u.tolist(), v.tolist()):
        lines.append(f"{a}\t{b}")
    lines += [f"{v[0]}\t{u[0]}", f"{u[1]}\t{v[1]}", f"{u[2]}\t{u[2]}"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return u, v


def _read_pairs(path):
    return np.fromfile(path, dtype=np.int32).reshape(-1, 2)


@pytest.mark.skipif(not os.path.exists(REF_E2B), reason="reference converter not built (needs the reference tree)")
def test_one_direction_equals_reference_converter(tmp_path):
    src = tmp_path / "g.txt"
    _snap_file(src)
    subprocess.run([REF_E2B, str(src)], cwd=tmp_path, check=True, stdout=subprocess.DEVNULL)
    ours = tmp_path / "ours.bin"
    subprocess.run([CONVERT, "edgelist2bin", str(src), str(ours), "--one-direction"], check=True)
    assert (tmp_path / "graph.bin").read_bytes() == ours.read_bytes()


def test_default_output_has_both_directions(tmp_path):
    src = tmp_path / "g.txt"
    u, v = _snap_file(src, seed=5)
    one, both = tmp_path / "one.bin", tmp_path / "both.bin"
    subprocess.run([CONVERT, "edgelist2bin", str(src), str(one), "--one-direction"], check=True)
    subprocess.run([CONVERT, "edgelist2bin", str(src), str(both)], check=True)
    p1, p2 = _read_pairs(one), _read_pairs(both)
    assert (p1[:, 0] < p1[:, 1]).all()
    rev = np.concatenate([p1, p1[:, ::-1]])
    assert np.array_equal(rev[np.lexsort((rev[:, 1], rev[:, 0]))], p2)
    ids = np.unique(np.concatenate([u, v]))
    assert p2.max() == len(ids) - 1
    # grouped by source with ascending neighbours: the .bin loader reads it as a
    # symmetric CSR over every vertex
    from test_frontend import load

    off, nbr = load(str(both))
    assert len(off) - 1 == len(ids) and len(nbr) == len(p2)
    src_ = np.repeat(np.arange(len(off) - 1), np.diff(off))
    fwd = np.sort(src_.astype(np.int64) * len(ids) + nbr)
    bwd = np.sort(nbr.astype(np.int64) * len(ids) + src_)
    assert np.array_equal(fwd, bwd)
    # --dedup removes the parallel pairs
    dd = tmp_path / "dd.bin"
    subprocess.run([CONVERT, "edgelist2bin", str(src), str(dd), "--dedup"], check=True)
    pd = _read_pairs(dd)
    assert len(np.unique(pd, axis=0)) == len(pd) and len(np.unique(p2, axis=0)) == len(pd)


def test_normalize_equals_reference_script(tmp_path):
    src = tmp_path / "edges.txt"
    _snap_file(src, seed=7)
    # normalize.py reads whitespace-separated pairs without comments
    body = [ln for ln in open(src).read().splitlines() if not ln.startswith("#")]
    (tmp_path / "plain.txt").write_text("\n".join(body) + "\n")
    script = os.path.join(os.environ.get("GALP_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference")),
                          "utils", "normalize.py")
    if not os.path.exists(script):
        pytest.skip("reference tree not present")
    subprocess.run([sys.executable, script, "plain.txt"], cwd=tmp_path, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    subprocess.run([CONVERT, "normalize", str(tmp_path / "plain.txt"), "--out", str(tmp_path / "ours.txt")],
                   check=True)
    assert (tmp_path / "normalized_plain.txt").read_text() == (tmp_path / "ours.txt").read_text()


def test_normalize_ground_truth(tmp_path):
    (tmp_path / "e.txt").write_text("10 30\n30 50\n50 10\n70 90\n")
    (tmp_path / "gt.txt").write_text("50 2\n10 1\n30 1\n90 2\n70 2\n")
    subprocess.run([CONVERT, "normalize", str(tmp_path / "e.txt"), str(tmp_path / "gt.txt")], check=True)
    assert (tmp_path / "normalized_e.txt").read_text() == "0 1\n0 2\n1 2\n3 4\n"
    assert (tmp_path / "normalized_gt.txt").read_text() == "2 3 4\n0 1\n"


def test_malformed_line_is_reported(tmp_path):
    (tmp_path / "bad.txt").write_text("1 2\n3 x\n")
    p = subprocess.run([CONVERT, "edgelist2bin", str(tmp_path / "bad.txt"), str(tmp_path / "o.bin")],
                       capture_output=True, text=True)
    assert p.returncode == 1 and "line 2" in p.stderr
