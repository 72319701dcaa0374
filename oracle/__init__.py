"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes loader for the CPU restatement of the reference hot path
(oracle/oracle.cpp, built by oracle/Makefile into oracle/_build/liboracle.so).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product library never does.

Parity unpinned: the reference has no tests or golden vectors for this path
and cannot be built here (no Eigen3 / Sophus / PCL / ROS).
"""
import ctypes as C
import os
import subprocess

from voxelmapplus_fastlio2_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(_HERE, "_build", "liboracle.so")

_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(ORACLE_SO):
        build()
    lib = C.CDLL(ORACLE_SO)
    vp = C.c_void_p
    P = C.POINTER
    d = C.c_double
    lib.orc_create.argtypes = [P(abi.vmp_config)]
    lib.orc_create.restype = vp
    lib.orc_destroy.argtypes = [vp]
    lib.orc_set_threads.argtypes = [vp, C.c_int]
    lib.orc_process.argtypes = [vp, P(abi.vmp_scan), P(abi.vmp_imu), C.c_int, P(abi.vmp_result)]
    lib.orc_get_state.argtypes = [vp, P(abi.vmp_state), P(d)]
    lib.orc_set_state.argtypes = [vp, P(abi.vmp_state), P(d)]
    lib.orc_get_aux.argtypes = [vp, P(d)]
    lib.orc_set_aux.argtypes = [vp, P(d)]
    lib.orc_map_info.argtypes = [vp, P(abi.vmp_map_info)]
    lib.orc_map_export.argtypes = [vp, P(abi.vmp_voxel), C.c_longlong]
    lib.orc_map_export.restype = C.c_longlong
    lib.orc_map_keys.argtypes = [vp, P(C.c_int64), C.c_longlong]
    lib.orc_map_keys.restype = C.c_longlong
    lib.orc_residual_valid.argtypes = [vp, P(C.c_ubyte), C.c_int]
    lib.orc_map_export_points.argtypes = [vp, P(d), P(d), C.c_longlong]
    lib.orc_map_export_points.restype = C.c_longlong
    lib.orc_map_import.argtypes = [vp, P(abi.vmp_voxel), C.c_longlong, P(d), P(d), C.c_longlong]
    lib.orc_map_build.argtypes = [vp, P(d), P(d), C.c_int]
    lib.orc_map_update.argtypes = [vp, P(d), P(d), C.c_int]
    lib.orc_map_index.argtypes = [vp, P(d), C.c_int, P(C.c_int64)]
    lib.orc_residual_reduce.argtypes = [vp, P(abi.vmp_state), P(d), P(d), P(d), C.c_int, P(d), P(d),
                                        P(C.c_int), P(C.c_ubyte)]
    lib.orc_ieskf_predict.argtypes = [vp, P(d), P(d), d, P(d)]
    lib.orc_ieskf_update.argtypes = [vp, P(C.c_float), C.c_int, P(C.c_int), P(C.c_int)]
    lib.orc_undistort.argtypes = [vp, P(abi.vmp_scan), P(abi.vmp_imu), C.c_int, P(abi.vmp_point)]
    lib.orc_downsample.argtypes = [P(abi.vmp_point), C.c_int, d, P(abi.vmp_point)]
    lib.orc_livox_decode.argtypes = [P(abi.vmp_livox_point), C.c_int, C.c_int, d, d, P(abi.vmp_point), P(C.c_float)]
    lib.orc_livox_decode.restype = C.c_int
    lib.orc_set_intensity.argtypes = [vp, P(C.c_float), C.c_int]
    lib.orc_output_cloud.argtypes = [vp, C.c_int, P(abi.vmp_point), P(C.c_float), C.c_int]
    lib.orc_output_cloud.restype = C.c_int
    lib.orc_map_planes.argtypes = [vp, P(abi.vmp_plane_marker), C.c_int]
    lib.orc_map_planes.restype = C.c_int
    lib.orc_std_plane_voxels.argtypes = [P(C.c_float), C.c_int, C.c_int, d, C.c_int, d, P(abi.vmp_std_voxel),
                                         C.c_int]
    lib.orc_std_plane_voxels.restype = C.c_int
    lib.orc_fit_planes.argtypes = [P(C.c_float), P(C.c_float), P(C.c_longlong), C.c_int, C.c_longlong, C.c_int, d,
                                   P(abi.vmp_fit_rec), C.c_int]
    lib.orc_downsample.restype = C.c_int
    lib.orc_calc_body_cov.argtypes = [P(d), C.c_int, d, d, P(d), P(d)]
    lib.orc_last_cloud.argtypes = [vp, C.c_int, P(abi.vmp_point), C.c_int]
    lib.orc_last_cloud.restype = C.c_int
    lib.orc_hat_sandwich.argtypes = [P(d), P(d), C.c_int, P(d)]
    lib.orc_restatement_check.argtypes = [C.c_int, C.c_longlong, C.c_ulonglong, P(C.c_longlong), P(d)]
    lib.orc_so3_exp.argtypes = [P(d), P(d)]
    lib.orc_so3_log.argtypes = [P(d), P(d)]
    lib.orc_eig_sym3.argtypes = [P(d), P(d), P(d)]
    _lib = lib
    return lib


class Oracle:
    """lio::LIOBuilder restated on the CPU (one sensor stream)."""

    def __init__(self, cfg=None, threads=1):
        self.lib = load()
        self.cfg = cfg if cfg is not None else abi.default_config()
        self.h = self.lib.orc_create(C.byref(self.cfg))
        self.lib.orc_set_threads(self.h, threads)

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def process(self, pkg):
        res = abi.vmp_result()
        scan = pkg.scan()
        self.lib.orc_process(self.h, C.byref(scan), pkg.imus, pkg.n_imu, C.byref(res))
        return res

    def process_points(self, pts4, t_start, t_end, imus, n_imu, intensity=None):
        """process() on a (n, 4) float32 cloud (x y z t_ms), optional intensities."""
        import numpy as np
        pts4 = np.ascontiguousarray(pts4, dtype=np.float32)
        if intensity is not None:
            inten = np.ascontiguousarray(intensity, dtype=np.float32)
            self.lib.orc_set_intensity(self.h, inten.ctypes.data_as(C.POINTER(C.c_float)), len(inten))
        scan = abi.vmp_scan(pts4.ctypes.data_as(C.POINTER(abi.vmp_point)), len(pts4), t_start, t_end)
        res = abi.vmp_result()
        self.lib.orc_process(self.h, C.byref(scan), imus, n_imu, C.byref(res))
        return res

    def map_keys(self):
        """Keys of all voxels in cache order (front = most recently used)."""
        import numpy as np
        n = self.lib.orc_map_keys(self.h, None, 0)
        out = np.zeros((max(1, n), 3), dtype=np.int64)
        self.lib.orc_map_keys(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)), n)
        return out[:n]

    def residual_valid(self, n):
        """is_valid of the first n residual_info entries (the last match set)."""
        import numpy as np
        v = np.zeros(max(1, n), dtype=np.uint8)
        self.lib.orc_residual_valid(self.h, v.ctypes.data_as(C.POINTER(C.c_ubyte)), n)
        return v[:n]

    def output_cloud(self, frame):
        import numpy as np
        n = self.lib.orc_output_cloud(self.h, frame, None, None, 0)
        out = np.zeros((max(1, n), 4), dtype=np.float32)
        inten = np.zeros(max(1, n), dtype=np.float32)
        self.lib.orc_output_cloud(self.h, frame, out.ctypes.data_as(C.POINTER(abi.vmp_point)),
                                  inten.ctypes.data_as(C.POINTER(C.c_float)), n)
        return out[:n], inten[:n]


def livox_decode(livox, filter_num=1, range_min=0.5, range_max=20.0):
    """livox2pcl restated on the CPU: (points (m, 4) float32, intensity (m,))."""
    import numpy as np
    lib = load()
    livox = np.ascontiguousarray(livox, dtype=abi.livox_dtype())
    n = len(livox)
    out = np.zeros((max(1, n), 4), dtype=np.float32)
    inten = np.zeros(max(1, n), dtype=np.float32)
    m = lib.orc_livox_decode(livox.ctypes.data_as(C.POINTER(abi.vmp_livox_point)), n, filter_num, range_min,
                             range_max, out.ctypes.data_as(C.POINTER(abi.vmp_point)),
                             inten.ctypes.data_as(C.POINTER(C.c_float)))
    return out[:m], inten[:m]
