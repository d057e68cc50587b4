"""Measurement helpers over include/galp_tools.h (schedule sizes, per-kernel device times)."""
from __future__ import annotations

import ctypes

from . import load_library


class SchedInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("m_big", ctypes.c_int64), ("npacks", ctypes.c_int64),
                ("nmid", ctypes.c_int64), ("nlarge", ctypes.c_int64), ("nbig", ctypes.c_int64),
                ("table_slots", ctypes.c_int64), ("launches_per_iter", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("launches", ctypes.c_int64), ("setup_ms", ctypes.c_double * 5)]

    SORTED = 1
    SYMMETRIC = 2
    FRONTIER = 4


class KernelTimes(ctypes.Structure):
    _fields_ = [("pipe_ms", ctypes.c_double), ("pipe_groups", ctypes.c_int32), ("big_pre_groups", ctypes.c_int32),
                ("big_pre_ms", ctypes.c_double), ("big_post_ms", ctypes.c_double),
                ("big_post_groups", ctypes.c_int32), ("first_groups", ctypes.c_int32),
                ("first_ms", ctypes.c_double)]


class Variant(ctypes.Structure):
    _fields_ = [("agg_mode", ctypes.c_int32), ("frontier_frac", ctypes.c_float), ("learned_margin", ctypes.c_float),
                ("small_sort", ctypes.c_int32), ("hub_part_shift", ctypes.c_int32),
                ("cta_stage", ctypes.c_int32), ("cta_narrow", ctypes.c_int32), ("mid_sort", ctypes.c_int32)]


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("ms", ctypes.c_double), ("launches", ctypes.c_int64)]


def _lib():
    L = load_library()
    if not getattr(L, "_tools_typed", False):
        P = ctypes.c_void_p
        L.galp_schedule_info.argtypes = [P, ctypes.POINTER(SchedInfo)]
        L.galp_schedule_info.restype = ctypes.c_int
        L.galp_profile.argtypes = [P, ctypes.c_int32]
        L.galp_profile.restype = ctypes.c_int
        L.galp_profile_read.argtypes = [P, ctypes.POINTER(KernelTimes)]
        L.galp_profile_read.restype = ctypes.c_int
        L.galp_profile_kernels.argtypes = [P, ctypes.POINTER(KernelStat), ctypes.c_int32,
                                           ctypes.POINTER(ctypes.c_int32)]
        L.galp_profile_kernels.restype = ctypes.c_int
        L.galp_set_variant.argtypes = [P, ctypes.POINTER(Variant)]
        L.galp_set_variant.restype = ctypes.c_int
        L.galp_get_variant.argtypes = [P, ctypes.POINTER(Variant)]
        L.galp_get_variant.restype = ctypes.c_int
        L._tools_typed = True
    return L


def probe_gather(prop, reps: int = 5) -> float:
    """Mean ms of one pass that streams every neighbour ID and gathers its label (the
    gather floor of an iteration; include/galp_tools.h galp_probe_gather)."""
    L = _lib()
    L.galp_probe_gather.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)]
    L.galp_probe_gather.restype = ctypes.c_int
    ms = ctypes.c_float()
    rc = L.galp_probe_gather(prop._h, reps, ctypes.byref(ms))
    if rc:
        raise RuntimeError(f"galp_probe_gather: {rc}")
    return float(ms.value)


def schedule_info(prop) -> SchedInfo:
    s = SchedInfo()
    rc = _lib().galp_schedule_info(prop._h, ctypes.byref(s))
    if rc:
        raise RuntimeError(f"galp_schedule_info: {rc}")
    return s


def profile(prop, level) -> None:
    """0 = off, 1 (or True) = kernel groups, 2 = every kernel."""
    rc = _lib().galp_profile(prop._h, int(level))
    if rc:
        raise RuntimeError(f"galp_profile: {rc}")


def profile_read(prop) -> KernelTimes:
    k = KernelTimes()
    rc = _lib().galp_profile_read(prop._h, ctypes.byref(k))
    if rc:
        raise RuntimeError(f"galp_profile_read: {rc}")
    return k


def profile_kernels(prop) -> dict:
    """{kernel name: (ms, launches)} since the last read (profile level 2)."""
    cap = 64
    buf = (KernelStat * cap)()
    cnt = ctypes.c_int32()
    rc = _lib().galp_profile_kernels(prop._h, buf, cap, ctypes.byref(cnt))
    if rc:
        raise RuntimeError(f"galp_profile_kernels: {rc}")
    return {buf[i].name.decode(): (buf[i].ms, buf[i].launches) for i in range(min(cnt.value, cap))}


def set_variant(prop, **knobs) -> Variant:
    """Change kernel variant knobs (e.g. agg_mode=1); returns the variant now in force."""
    v = Variant()
    L = _lib()
    if L.galp_get_variant(prop._h, ctypes.byref(v)):
        raise RuntimeError("galp_get_variant failed")
    for k, x in knobs.items():
        setattr(v, k, x)
    rc = L.galp_set_variant(prop._h, ctypes.byref(v))
    if rc:
        raise RuntimeError(f"galp_set_variant: {rc}")
    return v


# ---------------------------------------------------------------------------
# per-iteration dispatch
# ---------------------------------------------------------------------------

NFEAT, NHID, NVAR = 24, 64, 16


class DispatchRow(ctypes.Structure):
    _fields_ = [("agg_mode", ctypes.c_int32), ("frontier", ctypes.c_int32), ("warp_max_degree", ctypes.c_int32),
                ("cta256_max_degree", ctypes.c_int32), ("pos1", ctypes.c_int32), ("pos2", ctypes.c_int32)]


def _dlib():
    L = _lib()
    if not getattr(L, "_dispatch_typed", False):
        P, F = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
        I32 = ctypes.POINTER(ctypes.c_int32)
        L.galp_dispatch_set.argtypes = [P, ctypes.c_int32, ctypes.c_int32, F, ctypes.c_int64]
        L.galp_dispatch_set.restype = ctypes.c_int
        L.galp_dispatch_log.argtypes = [P, F, I32, ctypes.c_int32, I32]
        L.galp_dispatch_log.restype = ctypes.c_int
        L.galp_dispatch_table.argtypes = [P, ctypes.POINTER(DispatchRow), ctypes.c_int32, I32]
        L.galp_dispatch_table.restype = ctypes.c_int
        L.galp_profile_iterations.argtypes = [P, F, ctypes.c_int32, I32]
        L.galp_profile_iterations.restype = ctypes.c_int
        L.galp_mlp_size.argtypes = [ctypes.c_int32] * 3
        L.galp_mlp_size.restype = ctypes.c_int64
        L.galp_mlp_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
                                      ctypes.POINTER(P)]
        L.galp_mlp_create.restype = ctypes.c_int
        L.galp_mlp_set_weights.argtypes = [P, F, ctypes.c_int64]
        L.galp_mlp_set_weights.restype = ctypes.c_int
        L.galp_mlp_get_weights.argtypes = [P, F, ctypes.c_int64]
        L.galp_mlp_get_weights.restype = ctypes.c_int
        L.galp_mlp_forward.argtypes = [P, F, ctypes.c_int32, F]
        L.galp_mlp_forward.restype = ctypes.c_int
        L.galp_mlp_loss_grad.argtypes = [P, F, F, F, ctypes.c_int32, F, F]
        L.galp_mlp_loss_grad.restype = ctypes.c_int
        L.galp_mlp_train.argtypes = [P, F, F, F, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_float, F]
        L.galp_mlp_train.restype = ctypes.c_int
        L.galp_mlp_destroy.argtypes = [P]
        L.galp_mlp_destroy.restype = None
        L._dispatch_typed = True
    return L


def _fptr(a):
    import numpy as np
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def dispatch_set(prop, mode: int, forced: int = 0, weights=None) -> None:
    """mode 0 fixed rule, 1 learned (weights float32[mlp_size] or None to keep), 2 forced variant."""
    import numpy as np
    L = _dlib()
    if weights is not None:
        w = np.ascontiguousarray(weights, np.float32)
        rc = L.galp_dispatch_set(prop._h, mode, forced, _fptr(w), w.size)
    else:
        rc = L.galp_dispatch_set(prop._h, mode, forced, None, 0)
    if rc:
        raise RuntimeError(f"galp_dispatch_set: {rc}")


def dispatch_log(prop):
    """(features float32[iters, 24], variant int32[iters]) of the last run (-1 = shortcut)."""
    import numpy as np
    L = _dlib()
    f = np.zeros((64, NFEAT), np.float32)
    v = np.zeros(64, np.int32)
    cnt = ctypes.c_int32()
    rc = L.galp_dispatch_log(prop._h, _fptr(f), v.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 64,
                             ctypes.byref(cnt))
    if rc:
        raise RuntimeError(f"galp_dispatch_log: {rc}")
    return f[:cnt.value].copy(), v[:cnt.value].copy()


def dispatch_table(prop) -> list:
    L = _dlib()
    rows = (DispatchRow * NVAR)()
    cnt = ctypes.c_int32()
    rc = L.galp_dispatch_table(prop._h, rows, NVAR, ctypes.byref(cnt))
    if rc:
        raise RuntimeError(f"galp_dispatch_table: {rc}")
    return [dict(agg_mode=r.agg_mode, frontier=r.frontier, warp_max_degree=r.warp_max_degree,
                 cta256_max_degree=r.cta256_max_degree, pos1=r.pos1, pos2=r.pos2) for r in rows[:cnt.value]]


def profile_iterations(prop):
    """Device ms of every in-core iteration since the last read (profile level >= 1)."""
    import numpy as np
    L = _dlib()
    ms = np.zeros(4096, np.float32)
    cnt = ctypes.c_int32()
    rc = L.galp_profile_iterations(prop._h, _fptr(ms), ms.size, ctypes.byref(cnt))
    if rc:
        raise RuntimeError(f"galp_profile_iterations: {rc}")
    return ms[:min(cnt.value, ms.size)].copy()


class MLP:
    """The dispatcher's network on the GPU (include/galp_tools.h galp_mlp_*)."""

    def __init__(self, nin=NFEAT, nhid=NHID, nout=NVAR, seed=1):
        self.shape = (nin, nhid, nout)
        self.L = _dlib()
        self._h = ctypes.c_void_p()
        rc = self.L.galp_mlp_create(nin, nhid, nout, seed, ctypes.byref(self._h))
        if rc:
            raise RuntimeError(f"galp_mlp_create: {rc}")
        self.size = int(self.L.galp_mlp_size(nin, nhid, nout))

    def close(self):
        if self._h:
            self.L.galp_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def weights(self):
        import numpy as np
        w = np.zeros(self.size, np.float32)
        rc = self.L.galp_mlp_get_weights(self._h, _fptr(w), self.size)
        if rc:
            raise RuntimeError(f"galp_mlp_get_weights: {rc}")
        return w

    def set_weights(self, w):
        import numpy as np
        w = np.ascontiguousarray(w, np.float32)
        rc = self.L.galp_mlp_set_weights(self._h, _fptr(w), w.size)
        if rc:
            raise RuntimeError(f"galp_mlp_set_weights: {rc}")

    def forward(self, x):
        import numpy as np
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], self.shape[2]), np.float32)
        rc = self.L.galp_mlp_forward(self._h, _fptr(x), x.shape[0], _fptr(y))
        if rc:
            raise RuntimeError(f"galp_mlp_forward: {rc}")
        return y

    def loss_grad(self, x, t, mask=None):
        import numpy as np
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, np.float32)
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.size, np.float32)
        rc = self.L.galp_mlp_loss_grad(self._h, _fptr(x), _fptr(t), None if m is None else _fptr(m), x.shape[0],
                                       _fptr(loss), _fptr(g))
        if rc:
            raise RuntimeError(f"galp_mlp_loss_grad: {rc}")
        return float(loss[0]), g

    def train(self, x, t, mask=None, steps=1000, lr=3e-3, weight_decay=1e-4):
        import numpy as np
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, np.float32)
        curve = np.zeros(max(steps, 1), np.float32)
        rc = self.L.galp_mlp_train(self._h, _fptr(x), _fptr(t), None if m is None else _fptr(m), x.shape[0], steps,
                                   lr, weight_decay, _fptr(curve))
        if rc:
            raise RuntimeError(f"galp_mlp_train: {rc}")
        return curve[:steps]


class TuneResult(ctypes.Structure):
    _fields_ = [("small_blocks_per_sm", ctypes.c_int32), ("mid_blocks_per_sm", ctypes.c_int32),
                ("resolve_blocks_per_sm", ctypes.c_int32), ("trials", ctypes.c_int32), ("best_ms", ctypes.c_float),
                ("dispatch_row", ctypes.c_int32)]


def batch_tune(batch, niter: int = 3) -> dict:
    """Launch-shape autotuner of a batched context (galp_batch_tune)."""
    L = _lib()
    L.galp_batch_tune.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(TuneResult)]
    L.galp_batch_tune.restype = ctypes.c_int
    r = TuneResult()
    rc = L.galp_batch_tune(batch._h, niter, ctypes.byref(r))
    if rc:
        raise RuntimeError(f"galp_batch_tune: {rc}")
    return dict(small_blocks_per_sm=r.small_blocks_per_sm, mid_blocks_per_sm=r.mid_blocks_per_sm,
                resolve_blocks_per_sm=r.resolve_blocks_per_sm, trials=r.trials, best_ms=r.best_ms,
                dispatch_row=r.dispatch_row)
