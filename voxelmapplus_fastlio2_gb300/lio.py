"""Python mirror of the voxel_plus call surface, over the C ABI of libvmp.

    LIOBuilder   lio::LIOBuilder (voxel_plus/src/map_builder/lio_builder.h:56-83)
      .process(package)             LIOBuilder::process
      .map  -> VoxelMapView         lio::VoxelMap (voxel_map.h:107-128)
      .kf   -> IESKFView            kf::IESKF (ieskf.h:76-110)

Every call runs on the GPU through libvmp.so; nothing here computes.
"""
import ctypes as C

import numpy as np

from . import abi
from ._lib import check, load


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class IESKFView:
    """kf::IESKF of one stream (state on the device)."""

    def __init__(self, owner):
        self._o = owner

    def get(self):
        x = abi.vmp_state()
        P = np.zeros(529)
        check(self._o.h, self._o.lib.vmp_get_state(self._o.h, C.byref(x), _dptr(P)))
        return x, P.reshape(23, 23)

    def x(self):
        return abi.state_to_dict(self.get()[0])

    def P(self):
        return self.get()[1]

    def set(self, x, P):
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(529)
        check(self._o.h, self._o.lib.vmp_set_state(self._o.h, C.byref(x), _dptr(P)))

    def predict(self, acc, gyro, dt, Q=None):
        acc = np.ascontiguousarray(acc, dtype=np.float64)
        gyro = np.ascontiguousarray(gyro, dtype=np.float64)
        q = None if Q is None else np.ascontiguousarray(Q, dtype=np.float64).reshape(144)
        check(self._o.h, self._o.lib.vmp_ieskf_predict(self._o.h, _dptr(acc), _dptr(gyro), float(dt),
                                                       None if q is None else _dptr(q)))

    def update(self, pts_l):
        pts = np.ascontiguousarray(pts_l, dtype=np.float32).reshape(-1, 3)
        it, eff = C.c_int(), C.c_int()
        check(self._o.h, self._o.lib.vmp_ieskf_update(self._o.h, pts.ctypes.data_as(C.POINTER(C.c_float)),
                                                      pts.shape[0], C.byref(it), C.byref(eff)))
        return it.value, eff.value


class VoxelMapView:
    """lio::VoxelMap of one stream (map on the device)."""

    def __init__(self, owner):
        self._o = owner

    def index(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        keys = np.zeros((pts.shape[0], 3), dtype=np.int64)
        check(self._o.h, self._o.lib.vmp_map_index(self._o.h, _dptr(pts), pts.shape[0],
                                                   keys.ctypes.data_as(C.POINTER(C.c_int64))))
        return keys

    def build(self, pts, cov):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        cov = np.ascontiguousarray(cov, dtype=np.float64).reshape(-1, 9)
        check(self._o.h, self._o.lib.vmp_map_build(self._o.h, _dptr(pts), _dptr(cov), pts.shape[0]))

    def update(self, pts, cov):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        cov = np.ascontiguousarray(cov, dtype=np.float64).reshape(-1, 9)
        check(self._o.h, self._o.lib.vmp_map_update(self._o.h, _dptr(pts), _dptr(cov), pts.shape[0]))

    def info(self):
        i = abi.vmp_map_info()
        check(self._o.h, self._o.lib.vmp_map_info_get(self._o.h, C.byref(i)))
        return i

    def export(self):
        """All voxels, most recently used first (vmp_voxel array)."""
        n = C.c_longlong()
        check(self._o.h, self._o.lib.vmp_map_export(self._o.h, None, 0, C.byref(n)))
        arr = (abi.vmp_voxel * max(1, n.value))()
        check(self._o.h, self._o.lib.vmp_map_export(self._o.h, arr, n.value, C.byref(n)))
        return arr, n.value

    def keys(self):
        """Keys of all voxels, most recently used first ((n, 3) int64)."""
        n = C.c_longlong()
        check(self._o.h, self._o.lib.vmp_map_keys(self._o.h, None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 3), dtype=np.int64)
        check(self._o.h, self._o.lib.vmp_map_keys(self._o.h, out.ctypes.data_as(C.POINTER(C.c_int64)), n.value,
                                                  C.byref(n)))
        return out[: n.value]

    def planes(self, max_markers=100000):
        """voxel2MarkerArray's data: the frozen planes in LRU order
        (records of abi.plane_marker_dtype())."""
        out = np.zeros(max(1, max_markers), dtype=abi.plane_marker_dtype())
        n = C.c_int()
        check(self._o.h, self._o.lib.vmp_map_planes(self._o.h, C.c_void_p(out.ctypes.data), max_markers, C.byref(n)))
        return out[: n.value]

    def export_points(self):
        n = C.c_longlong()
        check(self._o.h, self._o.lib.vmp_map_export_points(self._o.h, None, None, 0, C.byref(n)))
        pts = np.zeros((max(1, n.value), 3))
        cov = np.zeros((max(1, n.value), 9))
        check(self._o.h, self._o.lib.vmp_map_export_points(self._o.h, _dptr(pts), _dptr(cov), n.value, C.byref(n)))
        return pts[: n.value], cov[: n.value]

    def import_(self, vox, n, pts, cov, group_counter):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        cov = np.ascontiguousarray(cov, dtype=np.float64).reshape(-1, 9)
        check(self._o.h, self._o.lib.vmp_map_import(self._o.h, vox, n, _dptr(pts), _dptr(cov), group_counter))


class LIOBuilder:
    """lio::LIOBuilder for one sensor stream, executed on the GPU."""

    def __init__(self, config=None):
        self.lib = load()
        self.cfg = config if config is not None else abi.default_config()
        h = C.c_void_p()
        code = self.lib.vmp_create(C.byref(self.cfg), C.byref(h))
        if code != abi.VMP_OK:
            from ._lib import VmpError
            raise VmpError(code, "vmp_create: " + (self.lib.vmp_last_error(None) or b"").decode())
        self.h = h
        self.map = VoxelMapView(self)
        self.kf = IESKFView(self)

    @classmethod
    def view(cls, lib, handle, config):
        """A LIOBuilder over a handle owned elsewhere (a server's stream):
        the same calls, and close() leaves the handle alone."""
        obj = cls.__new__(cls)
        obj.lib = lib
        obj.cfg = config
        obj.h = handle
        obj._borrowed = True
        obj.map = VoxelMapView(obj)
        obj.kf = IESKFView(obj)
        return obj

    def close(self):
        if getattr(self, "h", None) and not getattr(self, "_borrowed", False):
            self.lib.vmp_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def process(self, pkg):
        """LIOBuilder::process on one package (scan + IMU samples)."""
        res = abi.vmp_result()
        scan = pkg.scan()
        check(self.h, self.lib.vmp_process(self.h, C.byref(scan), pkg.imus, pkg.n_imu, C.byref(res)))
        return res

    def process_device(self, d_points, n, t_start, t_end, d_imus, n_imu):
        res = abi.vmp_result()
        check(self.h, self.lib.vmp_process_device(self.h, C.c_void_p(d_points), n, t_start, t_end,
                                                  C.c_void_p(d_imus), n_imu, C.byref(res)))
        return res

    def livox_decode(self, livox, filter_num=1, range_min=0.5, range_max=20.0, copy_out=True):
        """livox2pcl on the device (src/utils.cpp:3-28).  livox: numpy array of
        abi.livox_dtype().  Returns (points (m, 4) float32: x y z t_ms,
        intensity (m,), last point's t_ms) -- with copy_out=False only the
        count and the last time are read back (the node's use); the cloud
        stays on the device for process_decoded."""
        livox = np.ascontiguousarray(livox, dtype=abi.livox_dtype())
        n = len(livox)
        out = np.empty((max(1, n), 4), dtype=np.float32) if copy_out else None
        inten = np.empty(max(1, n), dtype=np.float32) if copy_out else None
        m = C.c_int()
        last = C.c_float()
        check(self.h, self.lib.vmp_livox_decode(self.h, C.c_void_p(livox.ctypes.data), n, filter_num, range_min,
                                                range_max, C.c_void_p(out.ctypes.data) if copy_out else None,
                                                C.c_void_p(inten.ctypes.data) if copy_out else None,
                                                C.byref(m), C.byref(last)))
        if not copy_out:
            return m.value, last.value
        return out[: m.value], inten[: m.value], last.value

    def process_decoded(self, t_start, t_end, imus, n_imu):
        """process() on the cloud of the last livox_decode."""
        res = abi.vmp_result()
        check(self.h, self.lib.vmp_process_decoded(self.h, t_start, t_end, imus, n_imu, C.byref(res)))
        return res

    def output_cloud(self, frame):
        """lidarToBody (frame 0) / lidarToWorld (frame 1) of the last scan's
        undistorted cloud: (points (n, 4) float32, intensity (n,))."""
        n = C.c_int()
        check(self.h, self.lib.vmp_output_cloud(self.h, frame, None, None, 0, C.byref(n)))
        out = np.empty((max(1, n.value), 4), dtype=np.float32)
        inten = np.empty(max(1, n.value), dtype=np.float32)
        check(self.h, self.lib.vmp_output_cloud(self.h, frame, C.c_void_p(out.ctypes.data),
                                                C.c_void_p(inten.ctypes.data), n.value, C.byref(n)))
        return out[: n.value], inten[: n.value]

    def residual_reduce(self, x, P, pts_l, cov_l):
        pts = np.ascontiguousarray(pts_l, dtype=np.float64).reshape(-1, 3)
        cov = np.ascontiguousarray(cov_l, dtype=np.float64).reshape(-1, 9)
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(529)
        H = np.zeros(144)
        b = np.zeros(12)
        eff = C.c_int()
        check(self.h, self.lib.vmp_residual_reduce(self.h, C.byref(x), _dptr(P), _dptr(pts), _dptr(cov), pts.shape[0],
                                                   _dptr(H), _dptr(b), C.byref(eff)))
        return H.reshape(12, 12), b, eff.value

    def residual_valid(self, n):
        v = np.zeros(max(1, n), dtype=np.uint8)
        check(self.h, self.lib.vmp_residual_valid(self.h, v.ctypes.data_as(C.POINTER(C.c_ubyte)), n))
        return v[:n]

    def undistort(self, pkg):
        out = (abi.vmp_point * max(1, pkg.n))()
        scan = pkg.scan()
        check(self.h, self.lib.vmp_undistort(self.h, C.byref(scan), pkg.imus, pkg.n_imu, out))
        return np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), shape=(pkg.n, 4)).copy()

    def downsample(self, pts4, leaf):
        pts4 = np.ascontiguousarray(pts4, dtype=np.float32).reshape(-1, 4)
        n = pts4.shape[0]
        out = np.zeros((max(1, n), 4), dtype=np.float32)
        m = C.c_int()
        check(self.h, self.lib.vmp_downsample(self.h, pts4.ctypes.data_as(C.POINTER(abi.vmp_point)), n, float(leaf),
                                              out.ctypes.data_as(C.POINTER(abi.vmp_point)), C.byref(m)))
        return out[: m.value]

    def last_cloud(self, kind):
        n = C.c_int()
        check(self.h, self.lib.vmp_last_cloud(self.h, kind, None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 4), dtype=np.float32)
        check(self.h, self.lib.vmp_last_cloud(self.h, kind, out.ctypes.data_as(C.POINTER(abi.vmp_point)), n.value,
                                              C.byref(n)))
        return out[: n.value]

    def set_merge_mode(self, mode):
        check(self.h, self.lib.vmp_set_merge_mode(self.h, mode))

    def last_merge_rounds(self):
        return self.lib.vmp_last_merge_rounds(self.h)
