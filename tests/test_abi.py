"""The C-ABI libraries load and export what include/*.h declares (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

import galp_gb300
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(galp_[a-z0-9_]+)\s*\(", txt)))


@pytest.mark.parametrize("header,lib", [("galp.h", "libgalp.so"), ("galp_tools.h", "libgalp.so"),
                                        ("galp_gen.h", "libgalp_gen.so"), ("galp_host.h", "libgalp_host.so")])
def test_library_exports_every_declared_symbol(header, lib):
    if not os.path.exists(os.path.join(ROOT, "include", header)):
        pytest.skip(f"{header} not present")
    L = ctypes.CDLL(galp_gb300.lib_path(lib))
    names = _declared(header)
    assert names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_strerror_and_default_opts():
    L = galp_gb300.load_library()
    assert L.galp_strerror(0) == b"ok"
    assert L.galp_strerror(-5) == b"malformed graph"
    o = galp_gb300.default_opts()
    assert (o.method, o.policy, o.lfht_policy, o.buffer_pow, o.early_exit) == (0, 0, 1, 24, 1)


def test_create_rejects_bad_arguments_without_touching_the_gpu():
    L = galp_gb300.load_library()
    h = ctypes.c_void_p()
    assert L.galp_create(None, None, ctypes.byref(h)) == -1
    off = np.array([0, 1], np.int64)  # offsets[n] != m
    csr = galp_gb300._Csr(None, off.ctypes.data, 1, 0)
    assert L.galp_create(ctypes.byref(csr), None, ctypes.byref(h)) == -5


def test_device_closed_form_matches_oracle():
    """The tie-break closed form compiled into libgalp.so (host copy) vs the oracle's."""
    L = galp_gb300.load_library()
    rng = np.random.default_rng(5)
    for _ in range(3000):
        mode = rng.integers(0, 3)
        if mode == 0:
            N = int(rng.integers(1, 20000))
            a = int(rng.integers(0, N))
            d = int(rng.integers(1, min(N - a, 6000) + 1))
        elif mode == 1:
            N = int(rng.integers(1, 3_000_000))
            a = int(rng.integers(0, N))
            d = int(rng.integers(1, min(N - a, 40) + 1))
        else:
            N = int(rng.integers(1, 3_000_000))
            d = int(rng.integers(1, min(N, 20000) + 1))
            a = N - d
        b = a + d
        w = np.ones(b, np.int32)
        k = d if rng.random() < 0.3 else int(rng.integers(1, min(d, 6) + 1))
        cand = np.sort(rng.choice(d, size=k, replace=False)).astype(np.int32)
        w[a:b] = 1
        w[a + cand] = 2
        want = oracle.cf_winner(w, a, b, N) - a
        got = L.galp_debug_resolve_rank(a, d, N, int(b == N), cand.ctypes.data, k)
        assert got == want, (a, d, N, k)


def test_ctypes_mirrors_match_the_c_structs(tmp_path):
    """Every ctypes mirror of an include/*.h struct has the C struct's size and field
    offsets (a plain C compiler lays the headers out; no GPU needed)."""
    import shutil
    import subprocess

    from galp_gb300 import tools

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"galp_csr": galp_gb300._Csr, "galp_opts": galp_gb300.Opts, "galp_stats": galp_gb300.Stats,
               "galp_sched_info": tools.SchedInfo, "galp_kernel_times": tools.KernelTimes,
               "galp_kernel_stat": tools.KernelStat, "galp_variant": tools.Variant,
               "galp_dispatch_row": tools.DispatchRow, "galp_tune_result": tools.TuneResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "galp_tools.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])
