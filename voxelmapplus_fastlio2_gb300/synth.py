"""Seeded synthetic LiDAR-inertial packages (host C++ generator, csrc/synth.cpp).

A package is what the reference node hands to LIOBuilder::process: one scan
(LiDAR-frame float points with their ms time offsets) plus the IMU samples up
to the scan end.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
SYNTH_SO = os.path.join(_HERE, "_build", "libvmp_synth.so")

KIND_ROOM, KIND_URBAN, KIND_CORRIDOR = 0, 1, 2


class vmp_synth_config(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("points_per_scan", C.c_int), ("seed", C.c_ulonglong), ("scan_hz", C.c_double),
        ("imu_hz", C.c_double), ("range_sigma", C.c_double), ("max_range", C.c_double), ("min_range", C.c_double),
        ("speed", C.c_double), ("gyro_noise", C.c_double), ("acc_noise", C.c_double), ("bias_walk", C.c_double),
        ("beams", C.c_int), ("clutter_frac", C.c_double),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(SYNTH_SO):
            from . import build as _b
            _b.build_synth()
        lib = C.CDLL(SYNTH_SO)
        lib.vmp_synth_default.argtypes = [C.POINTER(vmp_synth_config), C.c_int]
        lib.vmp_synth_create.argtypes = [C.POINTER(vmp_synth_config)]
        lib.vmp_synth_create.restype = C.c_void_p
        lib.vmp_synth_destroy.argtypes = [C.c_void_p]
        lib.vmp_synth_pose.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.vmp_synth_package.argtypes = [
            C.c_void_p, C.c_int, C.POINTER(abi.vmp_point), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
            C.POINTER(abi.vmp_imu), C.c_int, C.POINTER(C.c_int)]
        lib.vmp_synth_package.restype = C.c_int
        _lib = lib
    return _lib


class Package:
    """One scan and its IMU samples, as numpy-backed ctypes arrays."""

    def __init__(self, points, n, t_start, t_end, imus, n_imu):
        self.points = points  # ctypes array of vmp_point
        self.n = n
        self.t_start = t_start
        self.t_end = t_end
        self.imus = imus
        self.n_imu = n_imu

    def scan(self):
        return abi.vmp_scan(C.cast(self.points, C.POINTER(abi.vmp_point)), self.n, self.t_start, self.t_end)

    def points_np(self):
        return np.ctypeslib.as_array(C.cast(self.points, C.POINTER(C.c_float)), shape=(self.n, 4)).copy()


class Sequence:
    """Deterministic package stream for one seeded scene (read in order)."""

    def __init__(self, kind=KIND_ROOM, seed=0x5EED0000, points_per_scan=None, **overrides):
        lib = _load()
        cfg = vmp_synth_config()
        lib.vmp_synth_default(C.byref(cfg), kind)
        cfg.seed = seed
        if points_per_scan is not None:
            cfg.points_per_scan = points_per_scan
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        self._h = lib.vmp_synth_create(C.byref(cfg))
        self._k = 0
        self._max_pts = cfg.points_per_scan + 16
        self._max_imu = 4096

    def __del__(self):
        try:
            if self._h:
                _load().vmp_synth_destroy(self._h)
        except Exception:
            pass

    def next(self):
        lib = _load()
        pts = (abi.vmp_point * self._max_pts)()
        imus = (abi.vmp_imu * self._max_imu)()
        ts, te, nimu = C.c_double(), C.c_double(), C.c_int()
        n = lib.vmp_synth_package(self._h, self._k, pts, self._max_pts, C.byref(ts), C.byref(te), imus,
                                  self._max_imu, C.byref(nimu))
        self._k += 1
        return Package(pts, n, ts.value, te.value, imus, nimu.value)

    def pose(self, t):
        R = (C.c_double * 9)()
        p = (C.c_double * 3)()
        _load().vmp_synth_pose(self._h, t, R, p)
        return np.array(R[:]).reshape(3, 3), np.array(p[:])
