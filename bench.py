"""Benchmark: GTEPS per label-propagation iteration on one GB300 (and N replicas).

A step is one full galp run: labels reset to vertex IDs, 10 synchronous iterations of
the exact method-0 update over the whole graph (early exit off, so every step does the
same work).  GTEPS/iter = iterations x m / seconds, m = CSR entries (both directions).

  value     device-resident: CSR already in HBM; CUDA events on the launching stream
  e2e       through the C ABI with host buffers: galp_create (pinned H2D upload and
            schedule) + galp_run (10 iterations + labels D2H) + galp_destroy per step
  roofline  the dominant kernel's algorithmic bytes per launch / its event-timed duration
  cpu_baseline  the reference's CPU label update (port of CPUWorker::update_label,
            OpenMP over all host cores) on a bounded sample of the same graph

`--impl reference` times that CPU update alone, as the reference arm.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (kind, params)
    "rmat26": ("rmat", dict(scale=26, edge_factor=28)),
    "rmat24": ("rmat", dict(scale=24, edge_factor=16)),
    "rmat23": ("rmat", dict(scale=23, edge_factor=16)),
    "rmat22": ("rmat", dict(scale=22, edge_factor=16)),
    "rmat20": ("rmat", dict(scale=20, edge_factor=16)),
    "lfr1m": ("lfr", dict(n=1_000_000)),
    "sbm16k": ("sbm", dict()),
    "batch4096": ("batch", dict(count=4096)),
    "batch512": ("batch", dict(count=512)),
}
NITER = 10
L2_BYTES = 129 * 1024 * 1024


def _rank_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

_M64 = (1 << 64) - 1


def _s64(x: int) -> int:
    """An unsigned 64-bit constant as the int64 with the same bits."""
    x &= _M64
    return x - (1 << 64) if x >> 63 else x


def _shr(x, k: int):
    """Logical right shift of int64 tensors holding unsigned 64-bit values."""
    return (x >> k) & ((1 << (64 - k)) - 1)


def _splitmix64(x):
    x = x + _s64(0x9E3779B97F4A7C15)
    x = (x ^ _shr(x, 30)) * _s64(0xBF58476D1CE4E5B9)
    x = (x ^ _shr(x, 27)) * _s64(0x94D049BB133111EB)
    return x ^ _shr(x, 31)


def _splitmix64_int(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def rmat_keys_torch(seed: int, scale: int, e0: int, e1: int, a=0.57, b=0.19, c=0.19, device="cuda"):
    """Raw R-MAT edge keys (u << 32 | v) of edges [e0, e1) computed with torch only: the
    counter-based sampler of galp_gb300/csrc/rmat_rng.h restated on int64 tensors (a
    SplitMix64 finaliser of (seed, edge, level) picks the quadrant at every level; int64
    multiplication wraps exactly like uint64).  Used where the workload must be built
    without the library, e.g. for the reference arm."""
    import torch

    ta, tb, tc = (int(math.floor(x * 4294967296.0 + 0.5)) for x in (a, a + b, a + b + c))
    base0 = _s64(_splitmix64_int((seed ^ 0x52D4A7F1C3B9E605) & _M64))
    e = torch.arange(e0, e1, dtype=torch.int64, device=device)
    base = e * _s64(0x9E3779B97F4A7C15)
    base ^= base0
    del e
    u = torch.zeros_like(base)
    v = torch.zeros_like(base)
    for lvl in range(scale):
        r = _shr(_splitmix64(base + _s64(lvl * 0xD1B54A32D192ED03)), 32)
        ub = r >= tb
        vb = ((r >= ta) & (r < tb)) | (r >= tc)
        u = (u << 1) | ub.to(torch.int64)
        v = (v << 1) | vb.to(torch.int64)
    return (u << 32) | v


def rmat_on_gpu(scale: int, edge_factor: int, seed: int = 1, a=0.57, b=0.19, c=0.19, sampler: str = "library",
                device: str = "cuda"):
    """R-MAT graph built on the device: raw edges from the counter-based sampler (the
    library's kernel, or its torch restatement with sampler="torch"; both give the CPU
    generator's edges), then symmetrise, drop self-loops and duplicates, delete isolated
    vertices and compact IDs.  Returns device tensors (offsets int64[n+1], neighbors
    int32[m])."""
    import torch

    ne = edge_factor << scale
    if sampler == "torch":
        keys = torch.empty(ne, dtype=torch.int64, device=device)
        step = 1 << 27
        for e0 in range(0, ne, step):
            keys[e0:min(ne, e0 + step)] = rmat_keys_torch(seed, scale, e0, min(ne, e0 + step), a, b, c, device)
    else:
        import galp_gb300

        L = galp_gb300.load_library()
        L.galp_gen_rmat_keys_device.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.galp_gen_rmat_keys_device.restype = ctypes.c_int
        keys = torch.empty(ne, dtype=torch.int64, device="cuda")
        rc = L.galp_gen_rmat_keys_device(seed, scale, ne, a, b, c, keys.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
        assert rc == 0, rc
    u = keys >> 32
    v = keys & 0xFFFFFFFF
    del keys
    keep = u != v
    u, v = u[keep], v[keep]
    del keep
    # bucket by the source's top bits so every sort stays below 2^31 elements
    nb = 64 if scale >= 6 else 1
    shift = scale - (nb.bit_length() - 1)
    parts_src, parts_dst = [], []
    for bkt in range(nb):
        mu = (u >> shift) == bkt
        mv = (v >> shift) == bkt
        kb = torch.cat([(u[mu] << 32) | v[mu], (v[mv] << 32) | u[mv]])
        del mu, mv
        kb = torch.unique(kb)  # sorted, deduplicated
        parts_src.append((kb >> 32).to(torch.int32))
        parts_dst.append((kb & 0xFFFFFFFF).to(torch.int32))
        del kb
    del u, v
    src = torch.cat(parts_src)
    del parts_src
    dst = torch.cat(parts_dst)
    del parts_dst
    deg = torch.bincount(src, minlength=1 << scale)
    del src
    nz = deg > 0
    newid = (torch.cumsum(nz.to(torch.int64), 0) - 1).to(torch.int32)
    n = int(nz.sum().item())
    nbr = torch.empty_like(dst)
    step = 1 << 28
    for i in range(0, dst.numel(), step):
        nbr[i:i + step] = newid[dst[i:i + step].long()]
    del dst
    offsets = torch.zeros(n + 1, dtype=torch.int64, device=device)
    offsets[1:] = torch.cumsum(deg[nz], 0)
    if device != "cpu":
        torch.cuda.synchronize()
    return offsets, nbr


def sbm_batch_on_gpu(count: int, seed: int = 1, deg_in: float = 12.0, deg_out: float = 3.0):
    """`count` planted-partition graphs built on the device: graph g (seed + g) has n_g
    log-uniform in [1000, 200000] vertices in k_g ~ U{4..256} equal communities; n_g *
    deg_in / 2 intra-community pairs (a uniform vertex and a uniform member of its
    community) and n_g * deg_out / 2 uniform pairs, self-loops and duplicates dropped,
    symmetrised.  Returns device tensors of the concatenation (offsets int64[n+1],
    neighbours int32[m] with global IDs), host graph_v0 int64[count+1] and k per graph."""
    import numpy as np
    import torch

    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(1000), np.log(200000), count)).astype(np.int64)
    ks = rng.integers(4, 257, count)
    v0 = np.zeros(count + 1, np.int64)
    v0[1:] = np.cumsum(ns)
    N = int(v0[-1])
    srcs, dsts = [], []
    gen = torch.Generator(device="cuda")
    chunk = 256
    for c in range(0, count, chunk):
        pa, pb = [], []
        for g in range(c, min(c + chunk, count)):
            n, k = int(ns[g]), int(ks[g])
            gen.manual_seed(seed * 1_000_003 + g)
            csize = (n + k - 1) // k
            mi, mo = int(n * deg_in / 2), int(n * deg_out / 2)
            u = torch.randint(0, n, (mi,), device="cuda", generator=gen)
            c0 = (u // csize) * csize
            span = torch.clamp(torch.full_like(u, n) - c0, max=csize)
            v = c0 + (torch.rand(mi, device="cuda", generator=gen) * span).long().clamp_max(n - 1)
            uo = torch.randint(0, n, (mo,), device="cuda", generator=gen)
            vo = torch.randint(0, n, (mo,), device="cuda", generator=gen)
            pa.append(torch.cat([u, uo]) + int(v0[g]))
            pb.append(torch.cat([v, vo]) + int(v0[g]))
        a, b = torch.cat(pa), torch.cat(pb)
        del pa, pb
        keep = a != b
        a, b = a[keep], b[keep]
        key = torch.unique(torch.cat([a * N + b, b * N + a]))  # sorted by (src, dst), deduplicated
        del a, b, keep
        srcs.append((key // N).to(torch.int32))
        dsts.append((key % N).to(torch.int32))
        del key
    src = torch.cat(srcs)
    del srcs
    nbr = torch.cat(dsts)
    del dsts
    deg = torch.bincount(src.long(), minlength=N)
    del src
    offsets = torch.zeros(N + 1, dtype=torch.int64, device="cuda")
    offsets[1:] = torch.cumsum(deg, 0)
    torch.cuda.synchronize()
    return offsets, nbr, v0, ks


def run_batch(args, desc_count: int):
    """Batched workload: one CUDA-graph launch of 10 iterations over all graphs, against
    the same graphs run one after another through per-graph contexts."""
    import numpy as np
    import torch

    import galp_gb300
    from galp_gb300 import tools

    t0 = time.perf_counter()
    off_d, nbr_d, v0, ks = sbm_batch_on_gpu(desc_count)
    gen_s = time.perf_counter() - t0
    n, m = int(off_d.numel() - 1), int(nbr_d.numel())
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    b = galp_gb300.Batch(offsets=off_d.data_ptr(), neighbors=nbr_d.data_ptr(), graph_v0=v0, n=n, m=m)
    setup_s = time.perf_counter() - t0
    b.set_stream(stream.cuda_stream)
    tune = b.tune(NITER)
    for _ in range(args.warmup):
        b.enqueue(NITER)
    b.sync()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            b.enqueue(NITER)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    b.sync()
    its = np.array([b.graph_stats(g)[0] for g in range(desc_count)])
    e_g = (off_d[torch.from_numpy(v0[1:]).cuda()] - off_d[torch.from_numpy(v0[:-1]).cuda()]).cpu().numpy()
    edge_iters = int((e_g * its).sum())
    batch_labels = b.all_labels()

    # sequential arm: one context per graph (setup untimed), enqueue + sync timed per graph
    off_h = off_d.cpu().numpy()
    seq_s = 0.0
    mism = 0
    t_all = time.perf_counter()
    for g in range(desc_count):
        a0, a1 = int(v0[g]), int(v0[g + 1])
        e0, e1 = int(off_h[a0]), int(off_h[a1])
        loc_nbr = (nbr_d[e0:e1] - a0).contiguous()
        gg = galp_gb300.Graph(off_h[a0:a1 + 1] - e0, np.zeros(0, np.int32))
        p = _propagator_device_nbr(gg, loc_nbr, e1 - e0)
        p.set_stream(stream.cuda_stream)
        torch.cuda.synchronize()
        t = time.perf_counter()
        p.enqueue(NITER)
        p.sync()
        seq_s += time.perf_counter() - t
        if g % 64 == 0:  # spot-check labels against the batch
            if not np.array_equal(p.get_labels(), batch_labels[a0:a1]):
                mism += 1
        p.close()
        del loc_nbr
    seq_wall = time.perf_counter() - t_all
    value = edge_iters / (ms / 1e3) / 1e9
    line = {
        "metric": "GTEPS per LP iteration", "value": round(value, 3), "unit": "GTEPS", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"sbm-batch-{desc_count}", "graphs": desc_count, "n": n, "m": m,
                   "n_per_graph": "log-uniform [1000, 200000]", "communities": "U{4..256}", "deg_in": 12,
                   "deg_out": 3, "iterations_per_step": NITER, "early_exit": "per graph",
                   "edge_iterations_per_step": edge_iters, "generation_s": round(gen_s, 2),
                   "setup_s": round(setup_s, 2), "tuned_launch_shapes": tune,
                   "l2": "inputs larger than L2 (neighbours {:.1f} GB)".format(4 * m / 1e9)},
        "clocks": clk.summary(),
        "batched_vs_sequential": {"batched_s": round(ms / 1e3, 4), "sequential_s": round(seq_s, 4),
                                  "speedup": round(seq_s / (ms / 1e3), 2), "sequential_wall_s": round(seq_wall, 1),
                                  "label_spot_checks_failed": mism},
    }
    b.close()
    return line


def _propagator_device_nbr(g, nbr_dev, m):
    """Per-graph context whose neighbours come from a device tensor (galp_create copies
    with cudaMemcpyDefault)."""
    import numpy as np

    import galp_gb300

    p = galp_gb300.Propagator.__new__(galp_gb300.Propagator)
    L = galp_gb300.load_library()
    p.graph = g
    p._off = np.ascontiguousarray(g.offsets, dtype=np.int64)
    p._nbr = nbr_dev
    p._csr = galp_gb300._Csr(nbr_dev.data_ptr() if m else None, p._off.ctypes.data, len(p._off) - 1, m)
    p.opts = galp_gb300.default_opts()
    h = ctypes.c_void_p()
    galp_gb300._check(L.galp_create(ctypes.byref(p._csr), ctypes.byref(p.opts), ctypes.byref(h)), "galp_create")
    p._h = h
    p.stats = galp_gb300.Stats()
    return p


def build_workload(name: str, library: bool = True):
    """Returns (host Graph with pinned arrays, description).  library=False builds the
    graph without loading any of this project's native libraries (the reference arm):
    R-MAT through the torch restatement of the sampler, edge for edge the same graph."""
    import galp_gb300

    kind, prm = WORKLOADS[name]
    if kind == "rmat":
        import torch

        off_d, nbr_d = rmat_on_gpu(prm["scale"], prm["edge_factor"], sampler="library" if library else "torch")
        off_h = torch.empty(off_d.numel(), dtype=torch.int64, pin_memory=True)
        nbr_h = torch.empty(nbr_d.numel(), dtype=torch.int32, pin_memory=True)
        off_h.copy_(off_d)
        nbr_h.copy_(nbr_d)
        del off_d, nbr_d
        torch.cuda.empty_cache()
        g = galp_gb300.Graph(off_h.numpy(), nbr_h.numpy())
        g._pinned = (off_h, nbr_h)  # keep the pinned storage alive
        desc = dict(workload=f"rmat-scale{prm['scale']}-ef{prm['edge_factor']}", a=0.57, b=0.19, c=0.19,
                    seed=1, symmetrised=True, dedup=True, isolated_removed=True)
    elif not library:
        raise SystemExit(f"--impl reference: workload {name} is generated by the project's native generator; "
                         "use an R-MAT workload")
    elif kind == "lfr":
        g = galp_gb300.generate_lfr(prm["n"], seed=1)
        desc = dict(workload="lfr-style-n1M", tau1=2.5, mean_deg=20, max_deg=1000, tau2=1.5, cmin=20, cmax=1000,
                    mu=0.3, seed=1)
    else:
        g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
        desc = dict(workload="sbm-n16384-64x256-din16-dout2", seed=1)
    desc.update(n=int(g.n), m=int(g.m))
    return g, desc


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _loop(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._loop, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 4 + i and
                          s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload: str, group: str):
    """DRAM bytes per iteration of a kernel group from the committed ncu summary (None
    when that workload was not captured)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        v = d.get(workload, {})
        return v.get(group) if isinstance(v, dict) else None
    return None


CPU_SAMPLE_ENTRIES = 1 << 28  # CSR entries of the strided CPU sample (about 4 s per 3 sweeps on 16 cores)
CPU_SAMPLE_SWEEPS = 3


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


def cpu_sample_stride(m: int) -> int:
    """Vertex stride of the CPU sample: every stride-th vertex, about CPU_SAMPLE_ENTRIES
    CSR entries in expectation; a function of the graph only, so both arms time the same
    vertices."""
    return max(1, int(round(m / CPU_SAMPLE_ENTRIES)))


def cpu_sample(g, threads: int = 0):
    """Time the reference's CPU update (port of CPUWorker::update_label, OpenMP dynamic
    schedule over all host cores, OMP_PROC_BIND=true as the reference's experiment
    scripts set it) for CPU_SAMPLE_SWEEPS in-place sweeps (iterations 1-3, labels from
    vertex IDs) over the strided vertex sample."""
    os.environ.setdefault("OMP_PROC_BIND", "true")  # read when the port's OpenMP runtime loads
    import oracle

    stride = cpu_sample_stride(g.m)
    secs, used, edges, _ = oracle.cpu_baseline_strided(g.offsets, g.neighbors, CPU_SAMPLE_SWEEPS, stride, 0, threads)
    return dict(seconds=secs, threads=used, edges=edges, stride=stride,
                gteps=CPU_SAMPLE_SWEEPS * edges / max(secs, 1e-9) / 1e9)


def cpu_sample_desc(g, s) -> str:
    return (f"{CPU_SAMPLE_SWEEPS} in-place sweeps (iterations 1-{CPU_SAMPLE_SWEEPS}, labels from vertex IDs) of "
            f"CPUWorker::update_label (port, std::map counting, OpenMP dynamic schedule, OMP_PROC_BIND=true) "
            f"over every {s['stride']}-th vertex: {s['edges']} of {g.m} CSR entries per sweep; "
            f"host CPU: {cpu_model()}, {os.cpu_count()} cores")


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def run_reference(args, g, desc, rank, world):
    """The reference arm: the reference's CPU label update on this host's cores, on the
    same graph (built without the library) and the same strided sample every step."""
    for _ in range(args.warmup):
        cpu_sample(g)
    res = []
    for _ in range(args.steps):
        res.append(cpu_sample(g))
    v = statistics.median(r["gteps"] for r in res)
    ms = statistics.median(1e3 * r["seconds"] for r in res)
    line = {
        "metric": "GTEPS per LP iteration", "value": round(v, 4), "unit": "GTEPS", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": desc,
        "ms_per_step": round(ms, 3),
        "cpu_baseline": {"value": round(v, 4), "unit": "GTEPS", "cores": res[0]["threads"], "kind": "port",
                         "sample": cpu_sample_desc(g, res[0])},
        "e2e": {"value": round(v, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def run_gpu(args, g, desc, rank, world, dist):
    import torch

    import galp_gb300

    L = galp_gb300.load_library()
    from galp_gb300 import tools

    dev = torch.cuda.current_device()
    peak, peak_kind = measured_peaks()
    # a dedicated stream: the library launches on it and the events are recorded on it
    stream = torch.cuda.Stream()
    ooc = dict(policy=args.policy, buffer_pow=args.buffer_pow) if args.policy else {}
    # end-to-end arm through the C ABI with host buffers, first: creating and destroying
    # contexts of this size slows the later uploads on the same box (the kernels do not move)
    e2e_times = []
    h2d = d2h = 0
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q = galp_gb300.Propagator(g, early_exit=0, device=dev, **ooc)
        q.run(NITER)
        lab = q.get_labels()
        h2d, d2h = q.stats.h2d_bytes, q.stats.d2h_bytes
        q.close()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
    e2e_t = statistics.median(e2e_times) if e2e_times else float("nan")
    if dist:
        t = torch.tensor([e2e_t], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_val = world * NITER * g.m / e2e_t / 1e9 if e2e_times else None
    # device-resident arm
    p = galp_gb300.Propagator(g, early_exit=0, device=dev, **ooc)
    p.set_stream(stream.cuda_stream)
    info = tools.schedule_info(p)
    for _ in range(args.warmup):
        p.enqueue(NITER)
    p.sync()
    tools.profile(p, True)
    tools.profile_read(p)  # discard
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = tools.schedule_info(p).launches
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            p.enqueue(NITER)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    st = p.sync()
    launches_timed = tools.schedule_info(p).launches - launches0
    kt = tools.profile_read(p)
    if st.err:
        raise RuntimeError(f"device error bits {st.err}")
    t_max = ms
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    ms_per_step = t_max / args.steps
    edges_all = world * NITER * g.m * args.steps
    value = edges_all / (t_max / 1e3) / 1e9

    # roofline of the dominant kernel group, over dense iterations only: the first
    # iteration's shortcut (labels = IDs, sorted adjacency lists: one pass that gathers no
    # labels) is timed as its own group and left out of both groups' averages
    n, m, mb = info.n, info.m, info.m_big
    # algorithmic bytes: 4 B neighbour + 4 B gathered label per CSR entry, 8 B offset,
    # 4 B old + 4 B new label per vertex (8m + 16n + 8 per dense iteration)
    pipe_bytes = 8 * (m - mb) + 16 * n + 8
    big_bytes = 8 * mb
    shares = {"count_scan_resolve": kt.pipe_ms, "big_vertex_kernels": kt.big_pre_ms + kt.big_post_ms}
    dom = max(shares, key=shares.get)
    if dom == "count_scan_resolve":
        dur = kt.pipe_ms / max(kt.pipe_groups, 1)
        alg = pipe_bytes
    else:
        dur = (kt.big_pre_ms + kt.big_post_ms) / max(kt.big_pre_groups, 1)
        alg = big_bytes
    achieved = alg / (dur / 1e3) / 1e9
    traffic = ncu_traffic(desc["workload"], dom) if not args.policy else None
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                "alg_bytes_per_launch": int(alg), "avg_launch_ms": round(dur, 4),
                "launches_averaged": int(kt.pipe_groups if dom == "count_scan_resolve" else kt.big_pre_groups),
                "kernel_share": {k: round(v / max(sum(shares.values()), 1e-9), 3) for k, v in shares.items()}}
    it_ms = tools.profile_iterations(p)
    if not args.policy and len(it_ms) >= NITER:
        first_short = bool(info.flags & tools.SchedInfo.SORTED)
        dense = [float(t) for i, t in enumerate(it_ms) if t > 0 and not (first_short and i % NITER == 0)]
        if dense:
            it_dense = statistics.mean(dense)
            whole = (8 * m + 16 * n + 8) / (it_dense / 1e3) / 1e9
            roofline["whole_iteration"] = {
                "alg_bytes": int(8 * m + 16 * n + 8), "dense_iteration_ms": round(it_dense, 4),
                "achieved": round(whole, 1), "frac": round(whole / peak, 4),
                "first_iteration_ms": round(kt.first_ms / max(kt.first_groups, 1), 4) if kt.first_groups else None}
    if not args.policy:
        # the gather floor: one pass that only streams the neighbour IDs and gathers their
        # labels (random 4-byte loads, one L2 sector each) -- what any exact update pays
        g_ms = tools.probe_gather(p, 5)
        if g_ms > 0 and "whole_iteration" in roofline:
            it_d = roofline["whole_iteration"]["dense_iteration_ms"]
            roofline["gather_floor"] = {
                "ms_per_pass": round(g_ms, 4), "G_gathers_per_s": round(m / (g_ms / 1e3) / 1e9, 1),
                "hbm_GBps": round(8 * m / (g_ms / 1e3) / 1e9, 1),
                "dense_iteration_vs_floor": round(g_ms / it_d, 4)}
    if args.policy:  # out-of-core: the neighbours cross the host link every iteration
        roofline["h2d_GBps_per_iteration"] = round(4 * m / (ms_per_step / NITER / 1e3) / 1e9, 1)
    p.close()
    del p

    # out-of-core policy 2 on the same graph: 2^24-edge batches streamed from pinned host
    # memory every iteration, bounded by the host link (reported against its measured peak)
    policy2 = None
    if rank == 0 and not args.policy and not args.no_policy2:
        policy2 = run_policy2(g, dev, stream, args.buffer_pow)

    # frontier mode under the fixed rule and the learned dispatcher (same labels)
    dispatch = None
    if not args.no_dispatch and not args.policy:
        dispatch = {"frontier": True, "iterations": NITER}
        for name, kw in (("fixed", {}), ("learned", {"dispatch": 1})):
            try:
                q = galp_gb300.Propagator(g, early_exit=0, frontier=1, device=dev, **kw)
            except galp_gb300.GalpError as e:
                dispatch[name] = f"unavailable: {e}"
                continue
            q.set_stream(stream.cuda_stream)
            for _ in range(args.warmup):
                q.enqueue(NITER)
            q.sync()
            torch.cuda.synchronize()
            ev0.record(stream)
            for _ in range(args.steps):
                q.enqueue(NITER)
            ev1.record(stream)
            torch.cuda.synchronize()
            dispatch[name + "_ms_per_iter"] = round(ev0.elapsed_time(ev1) / args.steps / NITER, 4)
            dispatch[name + "_rows"] = [int(r) for r in tools.dispatch_log(q)[1]]
            q.close()
        if "fixed_ms_per_iter" in dispatch and "learned_ms_per_iter" in dispatch:
            dispatch["learned_speedup_vs_fixed"] = round(dispatch["fixed_ms_per_iter"] /
                                                         dispatch["learned_ms_per_iter"], 3)
        if "fixed_ms_per_iter" in dispatch:
            dispatch["frontier_fixed_vs_dense"] = round((ms_per_step / NITER) / dispatch["fixed_ms_per_iter"], 3)


    cpu = None
    if rank == 0 and not args.no_cpu:
        reps = [cpu_sample(g) for _ in range(3)]
        s = sorted(reps, key=lambda r: r["gteps"])[1]
        cpu = {"value": round(s["gteps"], 4), "unit": "GTEPS", "cores": s["threads"], "kind": "port",
               "sample": cpu_sample_desc(g, s) + "; median of 3"}
    cfg = dict(desc)
    cfg.update(iterations_per_step=NITER, early_exit=False, method=0, policy=args.policy,
               l2="inputs larger than L2 (neighbours {:.1f} GB vs 129 MB L2)".format(4 * g.m / 1e9),
               parallelism="replicas" if world > 1 else "single-gpu", packs=int(info.npacks),
               mid_vertices=int(info.nmid), large_vertices=int(info.nlarge), big_vertices=int(info.nbig),
               big_edges=int(info.m_big))
    if args.policy:
        cfg["buffer_pow"] = args.buffer_pow
    line = {
        "metric": "GTEPS per LP iteration", "value": round(value, 3), "unit": "GTEPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic", "config": cfg, "clocks": clk.summary(), "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_val, 3) if e2e_val else None, "unit": "GTEPS", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds_per_step": round(e2e_t, 4) if e2e_times else None},
        "dispatch": dispatch,
        "policy2": policy2,
        "gpu_launches": int(launches_timed),
        "iteration_ms": round(ms_per_step / NITER, 4),
    }
    return line


def pinned_h2d_peak(nbytes: int = 1 << 31, reps: int = 5) -> float:
    """Host-to-device copy bandwidth (GB/s) of one plain cudaMemcpyAsync of a pinned host
    buffer (torch copy_), best of reps, timed by CUDA events on its stream."""
    import torch

    src = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dst = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    st = torch.cuda.Stream()
    best = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
        e1.synchronize()
        best = max(best, nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9)
    del src, dst
    return best


def run_policy2(g, dev, stream, buffer_pow: int, steps: int = 2, warmup: int = 1):
    """Policy 2 (AsyncLP: batches of < 2^buffer_pow edges, pinned double-buffered copies
    overlapped with compute) over NITER iterations, early exit off."""
    import torch

    import galp_gb300

    peak = pinned_h2d_peak()
    t0 = time.perf_counter()
    q = galp_gb300.Propagator(g, early_exit=0, device=dev, policy=2, buffer_pow=buffer_pow)
    setup_s = time.perf_counter() - t0
    q.set_stream(stream.cuda_stream)
    for _ in range(warmup):
        q.enqueue(NITER)
        q.sync()
    torch.cuda.synchronize()
    step_ms = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q.enqueue(NITER)
        q.sync()
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    ms = sum(step_ms) / steps
    q.close()
    it_ms = ms / NITER
    link = 4 * g.m / (it_ms / 1e3) / 1e9  # every iteration streams every neighbour once
    return {"buffer_pow": buffer_pow, "steps": steps, "warmup": warmup, "ms_per_iteration": round(it_ms, 3),
            "step_ms": [round(x, 1) for x in step_ms],
            "value": round(g.m / (it_ms / 1e3) / 1e9, 3), "unit": "GTEPS",
            "setup_s": round(setup_s, 2),
            "roofline": {"bound": "host-to-device link", "achieved": round(link, 1), "unit": "GB/s",
                         "peak": round(peak, 1), "peak_kind": "measured pinned cudaMemcpyAsync H2D (2 GiB, best of 5)",
                         "frac": round(link / peak, 4), "alg_bytes_per_iteration": int(4 * g.m)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="galp", choices=["galp", "reference"])
    ap.add_argument("--workload", default=os.environ.get("GALP_BENCH_WORKLOAD", "rmat26"), choices=list(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-dispatch", action="store_true")
    ap.add_argument("--no-policy2", action="store_true", help="skip the out-of-core policy-2 sub-record")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched (4096 SBM graphs) sub-record")
    ap.add_argument("--policy", type=int, default=0, choices=[0, 1, 2],
                    help="1/2: out-of-core, neighbours streamed from pinned host memory in 2^buffer_pow chunks")
    ap.add_argument("--buffer-pow", type=int, default=24)
    ap.add_argument("--case", type=int, default=0,
                    help="profiler case: build the workload, run this many iterations once, print a summary")
    args = ap.parse_args()
    rank, world, local = _rank_env()

    if args.impl == "reference":
        if rank != 0:
            return 0
        from galp_gb300.build import build

        build()
        import torch

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        g, desc = build_workload(args.workload, library=False)
        print(json.dumps(run_reference(args, g, desc, rank, world)))
        return 0

    import torch

    dist = None
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
        dist = tdist
    torch.cuda.set_device(local)
    from galp_gb300.build import build

    if rank == 0:
        build()
    if dist:
        dist.barrier()
    if args.case:
        import galp_gb300

        g, desc = build_workload(args.workload)
        with galp_gb300.Propagator(g, early_exit=0) as p:
            p.run(args.case)
            print(json.dumps({"case": desc["workload"], "n": desc["n"], "m": desc["m"], "iterations": p.iters_run,
                              "updates": list(p.updates)[:p.iters_run]}))
        return 0
    if WORKLOADS[args.workload][0] == "batch":
        line = run_batch(args, WORKLOADS[args.workload][1]["count"])
        if rank == 0:
            print(json.dumps(line))
        return 0
    g, desc = build_workload(args.workload)
    line = run_gpu(args, g, desc, rank, world, dist)
    if rank == 0 and not args.no_batch and not args.policy and WORKLOADS[args.workload][0] == "rmat":
        # batched mode (4096 SBM graphs in one CUDA-graph launch vs per-graph launches)
        import gc

        del g
        gc.collect()
        torch.cuda.empty_cache()
        b = run_batch(argparse.Namespace(steps=3, warmup=3), WORKLOADS["batch4096"][1]["count"])
        line["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "steps", "warmup", "config",
                                              "batched_vs_sequential", "clocks")}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
