"""Build the native parts of galp-gb300 in-tree.

Products (all under galp_gb300/lib/ unless noted):
  libgalp.so       CUDA label-propagation library behind include/galp.h (sm_103a)
  libgalp_gen.so   seeded graph generators behind include/galp_gen.h
  libgalp_host.so  front end: .txt/.bin loaders and accuracy measures (include/galp_host.h)
  galp             the command-line front end (src mirrors the reference's main.cu CLI)
  galp_convert     edge-list converters (the reference's utils/edgelist2bin.cpp, normalize.py)
and the test-infrastructure oracle:
  oracle/_build/liblp_oracle.so   CPU restatement of the reference update
  oracle/_ref/ref_harness         reference kernels run on the CPU (only where the
                                  reference tree is present)

Every step is a direct nvcc/g++ invocation; the steps run in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "galp_gb300")
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
ORACLE = os.path.join(ROOT, "oracle")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_SOURCES = ["galp_capi.cu", "galp_tools.cu", "galp_noalloc.cu", "galp_mlp.cu"]
HOST_SOURCES = ["host/graph_io.cpp", "host/accuracy.cpp"]


def reference_tree() -> str:
    """The reference source tree the oracle's reference harness is built from:
    $GALP_REFERENCE, else a directory named "reference" beside the repository."""
    return os.environ.get("GALP_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return cmd, p.returncode, p.stdout


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _deps(*dirs: str) -> list[str]:
    out = []
    for d in dirs:
        for base, _, files in os.walk(d):
            if "_ref" in base or "_build" in base or "lib" == os.path.basename(base):
                continue
            out += [os.path.join(base, f) for f in files if f.endswith((".cu", ".cuh", ".h", ".inc", ".cpp", ".c"))]
    return out


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(os.path.join(ORACLE, "_build"), exist_ok=True)
    inc = os.path.join(ROOT, "include")
    jobs: list[tuple[str, list[str], list[str]]] = []

    # CUDA sources compile to objects in parallel, then link into libgalp.so (second phase)
    os.makedirs(os.path.join(LIB, "obj"), exist_ok=True)
    cuda_out = os.path.join(LIB, "libgalp.so")
    cuda_deps = _deps(CSRC, inc)
    objs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(LIB, "obj", src.replace(".cu", ".o"))
        objs.append(obj)
        jobs.append((obj, cuda_deps, [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
                                      "-o", obj, os.path.join(CSRC, src)]))
    link_jobs = [(cuda_out, objs, [NVCC, *ARCH, "-shared", "-o", cuda_out, *objs])]

    gen_out = os.path.join(LIB, "libgalp_gen.so")
    gen_src = os.path.join(PKG, "gen", "generators.cpp")
    jobs.append((gen_out, [gen_src, os.path.join(inc, "galp_gen.h")],
                 ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-o", gen_out, gen_src]))

    conv_src = os.path.join(PKG, "host", "convert.cpp")
    conv_out = os.path.join(LIB, "galp_convert")
    jobs.append((conv_out, [conv_src], ["g++", "-O2", "-std=c++17", "-o", conv_out, conv_src]))

    host_srcs = [os.path.join(PKG, s) for s in HOST_SOURCES]
    host_out = os.path.join(LIB, "libgalp_host.so")
    if all(os.path.exists(s) for s in host_srcs):
        jobs.append((host_out, host_srcs + [os.path.join(inc, "galp_host.h")],
                     ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-o", host_out, *host_srcs]))
        cli_src = os.path.join(PKG, "host", "main.cpp")
        cli_out = os.path.join(LIB, "galp")
        if os.path.exists(cli_src):
            # the CLI links libgalp.so next to it (found through $ORIGIN)
            link_jobs.append((cli_out, [cli_src, *host_srcs, os.path.join(inc, "galp.h"), cuda_out],
                              ["g++", "-O2", "-std=c++17", "-fopenmp", "-o", cli_out, cli_src, *host_srcs,
                               "-L" + LIB, "-lgalp", "-Wl,-rpath,$ORIGIN"]))

    # oracle: the sequential restatement (C) and its multi-threaded closed form (C++/OpenMP)
    # in one library
    orc_out = os.path.join(ORACLE, "_build", "liblp_oracle.so")
    orc_c = os.path.join(ORACLE, "lp_oracle.c")
    orc_o = os.path.join(ORACLE, "_build", "lp_oracle.o")
    orc_par = os.path.join(ORACLE, "lp_oracle_par.cpp")
    jobs.append((orc_o, [orc_c], ["gcc", "-O2", "-std=c99", "-fPIC", "-c", "-o", orc_o, orc_c]))
    link_jobs.append((orc_out, [orc_o, orc_par], ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                                                  "-o", orc_out, orc_par, orc_o]))
    port_src = os.path.join(ORACLE, "cpu_worker_port.cpp")
    if os.path.exists(port_src):
        port_out = os.path.join(ORACLE, "_build", "libcpu_worker_port.so")
        jobs.append((port_out, [port_src], ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-o",
                                            port_out, port_src]))

    failed = _run_jobs(jobs, force, verbose, extra_ref=True)
    if not failed:
        failed = _run_jobs(link_jobs, force, verbose, extra_ref=False)
    if failed:
        raise RuntimeError("galp_gb300 build failed: " + ", ".join(failed))


def _run_jobs(jobs, force: bool, verbose: bool, extra_ref: bool) -> list[str]:
    todo = [(o, cmd) for o, deps, cmd in jobs if force or not _newer(o, deps)]
    ref_script = os.path.join(ORACLE, "build_ref.sh")
    ref_deps = _deps(os.path.join(ORACLE, "refsim")) + [ref_script]
    ref_needed = extra_ref and os.path.isdir(reference_tree()) and (
        force or not all(_newer(os.path.join(ORACLE, "_ref", t), ref_deps) for t in ("ref_harness", "edgelist2bin")))
    with ThreadPoolExecutor(max_workers=max(1, len(todo) + 1)) as ex:
        futs = [ex.submit(_run, cmd) for _, cmd in todo]
        if ref_needed:
            futs.append(ex.submit(_run, ["bash", ref_script]))
        failed = []
        for f in futs:
            cmd, rc, out = f.result()
            if verbose or rc:
                sys.stderr.write(" ".join(cmd) + "\n" + out)
            if rc:
                failed.append(cmd[-1])
    return failed


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
