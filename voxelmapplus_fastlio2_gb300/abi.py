"""ctypes mirror of include/vmp.h (the C ABI of libvmp.so).

Field order and types follow the header exactly; ``tests/test_abi.py`` checks
the struct sizes against the compiled library.
"""
import ctypes as C

VMP_OK = 0
STATUS_NAMES = {
    0: "VMP_OK", 1: "VMP_ERR_INVALID_ARG", 2: "VMP_ERR_OUT_OF_MEMORY", 3: "VMP_ERR_ADMISSION_DENIED",
    4: "VMP_ERR_HASH_FULL", 5: "VMP_ERR_TIMEOUT", 6: "VMP_ERR_CUDA", 7: "VMP_ERR_KEY_RANGE",
    8: "VMP_ERR_STATE", 9: "VMP_ERR_CAPACITY",
}
VMP_ERR_INVALID_ARG, VMP_ERR_OUT_OF_MEMORY, VMP_ERR_ADMISSION_DENIED = 1, 2, 3
VMP_ERR_HASH_FULL, VMP_ERR_TIMEOUT, VMP_ERR_CUDA, VMP_ERR_KEY_RANGE, VMP_ERR_STATE, VMP_ERR_CAPACITY = 4, 5, 6, 7, 8, 9
IMU_INIT, MAP_INIT, LIO_MAPPING = 0, 1, 2


class vmp_config(C.Structure):
    _fields_ = [
        ("opti_max_iter", C.c_int),
        ("na", C.c_double), ("ng", C.c_double), ("nba", C.c_double), ("nbg", C.c_double),
        ("imu_init_num", C.c_int),
        ("r_il", C.c_double * 9),
        ("p_il", C.c_double * 3),
        ("gravity_align", C.c_int),
        ("estimate_ext", C.c_int),
        ("scan_resolution", C.c_double),
        ("voxel_size", C.c_double),
        ("update_size_thresh", C.c_int),
        ("max_point_thresh", C.c_int),
        ("plane_thresh", C.c_double),
        ("ranging_cov", C.c_double),
        ("angle_cov", C.c_double),
        ("merge_thresh_for_angle", C.c_double),
        ("merge_thresh_for_distance", C.c_double),
        ("map_capacity", C.c_int),
        ("ieskf_max_iter", C.c_int),
        ("ieskf_eps", C.c_double),
        ("max_scan_points", C.c_int),
        ("max_imu_per_scan", C.c_int),
        ("reserved", C.c_int * 6),
    ]


class vmp_point(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("t_ms", C.c_float)]


class vmp_imu(C.Structure):
    _fields_ = [("t", C.c_double), ("acc", C.c_double * 3), ("gyro", C.c_double * 3)]


class vmp_livox_point(C.Structure):
    """livox_ros_driver2 CustomPoint (20 bytes)."""
    _fields_ = [("offset_time", C.c_uint32), ("x", C.c_float), ("y", C.c_float), ("z", C.c_float),
                ("reflectivity", C.c_uint8), ("tag", C.c_uint8), ("line", C.c_uint8), ("pad", C.c_uint8)]


def livox_dtype():
    import numpy as np
    return np.dtype([("offset_time", "<u4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("reflectivity", "u1"),
                     ("tag", "u1"), ("line", "u1"), ("pad", "u1")])


class vmp_scan(C.Structure):
    _fields_ = [("points", C.POINTER(vmp_point)), ("n", C.c_int), ("t_start", C.c_double), ("t_end", C.c_double)]


class vmp_state(C.Structure):
    _fields_ = [
        ("pos", C.c_double * 3), ("rot", C.c_double * 9), ("rot_ext", C.c_double * 9), ("pos_ext", C.c_double * 3),
        ("vel", C.c_double * 3), ("bg", C.c_double * 3), ("ba", C.c_double * 3), ("g", C.c_double * 3),
    ]


class vmp_result(C.Structure):
    _fields_ = [
        ("lio_status", C.c_int), ("iters", C.c_int), ("effect_num", C.c_int), ("n_raw", C.c_int),
        ("n_down", C.c_int), ("flags", C.c_int), ("map_size", C.c_longlong), ("evicted", C.c_longlong),
        ("x", vmp_state), ("P", C.c_double * 529),
    ]


class vmp_map_info(C.Structure):
    _fields_ = [("size", C.c_longlong), ("capacity", C.c_longlong), ("group_counter", C.c_longlong),
                ("slab_points", C.c_longlong)]


class vmp_voxel(C.Structure):
    _fields_ = [
        ("key", C.c_int64 * 3), ("n", C.c_int32), ("newly_add_point", C.c_int32),
        ("is_init", C.c_int32), ("is_plane", C.c_int32), ("update_enable", C.c_int32), ("merged", C.c_int32),
        ("group_id", C.c_uint64), ("lru_stamp", C.c_uint64), ("n_temp", C.c_int32), ("pad", C.c_int32),
        ("mean", C.c_double * 3), ("ppt", C.c_double * 9), ("norm", C.c_double * 3), ("center", C.c_double * 3),
        ("cov", C.c_double * 36),
    ]


def default_config(**kw):
    """vmp_config with lio::LIOConfig defaults (lio_builder.h:17-42)."""
    c = vmp_config()
    c.opti_max_iter = 5
    c.na, c.ng, c.nba, c.nbg = 0.01, 0.01, 0.0001, 0.0001
    c.imu_init_num = 20
    for i in range(9):
        c.r_il[i] = 1.0 if i in (0, 4, 8) else 0.0
    c.gravity_align = 1
    c.estimate_ext = 0
    c.scan_resolution = 0.1
    c.voxel_size = 0.5
    c.update_size_thresh = 10
    c.max_point_thresh = 100
    c.plane_thresh = 0.01
    c.ranging_cov = 0.04
    c.angle_cov = 0.1
    c.merge_thresh_for_angle = 0.1
    c.merge_thresh_for_distance = 0.04
    c.map_capacity = 100000
    c.ieskf_max_iter = 5
    c.ieskf_eps = 0.001
    c.max_scan_points = 262144
    c.max_imu_per_scan = 1000
    for k, v in kw.items():
        if k in ("r_il", "p_il"):
            arr = getattr(c, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(c, k, v)
    return c


class vmp_server_config(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_longlong), ("max_streams", C.c_int), ("workers", C.c_int),
                ("queue_depth", C.c_int), ("autotune", C.c_int), ("merge_grid_divisor", C.c_int),
                ("seg_grid_blocks", C.c_int), ("reserved", C.c_int * 4)]


class vmp_server_result(C.Structure):
    _fields_ = [("cookie", C.c_longlong), ("stream_id", C.c_int), ("status", C.c_int),
                ("submit_ms", C.c_double), ("start_ms", C.c_double), ("end_ms", C.c_double),
                ("result", vmp_result)]


def state_to_dict(x):
    import numpy as np
    return {
        "pos": np.array(x.pos[:]), "rot": np.array(x.rot[:]).reshape(3, 3),
        "rot_ext": np.array(x.rot_ext[:]).reshape(3, 3), "pos_ext": np.array(x.pos_ext[:]),
        "vel": np.array(x.vel[:]), "bg": np.array(x.bg[:]), "ba": np.array(x.ba[:]), "g": np.array(x.g[:]),
    }


# ---- batched plane fitting (vmp_fit_planes)
VMP_FIT_FP64, VMP_FIT_FP32, VMP_FIT_FP32C = 0, 1, 2
FIT_MODE_NAMES = {VMP_FIT_FP64: "fp64", VMP_FIT_FP32: "fp32", VMP_FIT_FP32C: "fp32c"}
VMP_FIT_FITTED, VMP_FIT_PLANE, VMP_FIT_FLIPPED = 1, 2, 4


class vmp_fit_params(C.Structure):
    _fields_ = [("mode", C.c_int), ("update_point_thresh", C.c_int), ("plane_thresh", C.c_double)]


class vmp_fit_rec(C.Structure):
    _fields_ = [("mean", C.c_double * 3), ("cov", C.c_double * 6), ("evals", C.c_double * 3),
                ("norm", C.c_double * 3), ("plane_cov", C.c_double * 21), ("n", C.c_int), ("flags", C.c_int)]


def fit_rec_dtype():
    """numpy dtype with the layout of vmp_fit_rec (296 bytes)."""
    import numpy as np
    return np.dtype([("mean", "<f8", (3,)), ("cov", "<f8", (6,)), ("evals", "<f8", (3,)), ("norm", "<f8", (3,)),
                     ("plane_cov", "<f8", (21,)), ("n", "<i4"), ("flags", "<i4")])


class vmp_plane_marker(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("norm", C.c_double * 3), ("orientation", C.c_double * 4),
                ("trace", C.c_double), ("rgb", C.c_uint8 * 3), ("merged", C.c_uint8), ("pad", C.c_int32)]


def plane_marker_dtype():
    import numpy as np
    return np.dtype([("center", "<f8", (3,)), ("norm", "<f8", (3,)), ("orientation", "<f8", (4,)), ("trace", "<f8"),
                     ("rgb", "u1", (3,)), ("merged", "u1"), ("pad", "<i4")])


class vmp_std_voxel(C.Structure):
    _fields_ = [("key", C.c_int64 * 3), ("n", C.c_int32), ("valid", C.c_int32), ("is_plane", C.c_int32),
                ("pad", C.c_int32), ("sum", C.c_double * 3), ("ppt", C.c_double * 9), ("mean", C.c_double * 3),
                ("lamdas", C.c_double * 3), ("norms", C.c_double * 9)]


def std_voxel_dtype():
    import numpy as np
    return np.dtype([("key", "<i8", (3,)), ("n", "<i4"), ("valid", "<i4"), ("is_plane", "<i4"), ("pad", "<i4"),
                     ("sum", "<f8", (3,)), ("ppt", "<f8", (9,)), ("mean", "<f8", (3,)), ("lamdas", "<f8", (3,)),
                     ("norms", "<f8", (9,))])
