"""Measurement helpers over include/galp_tools.h (schedule sizes, per-kernel device times)."""
from __future__ import annotations

import ctypes

from . import load_library


class SchedInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("m_big", ctypes.c_int64), ("npacks", ctypes.c_int64),
                ("nmid", ctypes.c_int64), ("nlarge", ctypes.c_int64), ("nbig", ctypes.c_int64),
                ("table_slots", ctypes.c_int64), ("launches_per_iter", ctypes.c_int32), ("pad", ctypes.c_int32)]


class KernelTimes(ctypes.Structure):
    _fields_ = [("pipe_ms", ctypes.c_double), ("pipe_groups", ctypes.c_int32), ("big_pre_groups", ctypes.c_int32),
                ("big_pre_ms", ctypes.c_double), ("big_post_ms", ctypes.c_double),
                ("big_post_groups", ctypes.c_int32), ("pad", ctypes.c_int32)]


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
        L._tools_typed = True
    return L


def schedule_info(prop) -> SchedInfo:
    s = SchedInfo()
    rc = _lib().galp_schedule_info(prop._h, ctypes.byref(s))
    if rc:
        raise RuntimeError(f"galp_schedule_info: {rc}")
    return s


def profile(prop, enable: bool) -> None:
    rc = _lib().galp_profile(prop._h, int(enable))
    if rc:
        raise RuntimeError(f"galp_profile: {rc}")


def profile_read(prop) -> KernelTimes:
    k = KernelTimes()
    rc = _lib().galp_profile_read(prop._h, ctypes.byref(k))
    if rc:
        raise RuntimeError(f"galp_profile_read: {rc}")
    return k
