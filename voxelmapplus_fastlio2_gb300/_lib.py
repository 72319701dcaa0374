"""Loader of the in-tree CUDA library (_build/libvmp.so).

There is no CPU fallback: if the library is missing or no GPU is visible the
calls fail with an exception.
"""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvmp.so")

_lib = None


class VmpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def _declare(lib):
    P = C.POINTER
    vp = C.c_void_p
    d = C.c_double
    st = C.c_int
    sig = {
        "vmp_abi_version": ([], C.c_int),
        "vmp_config_default": ([P(abi.vmp_config)], None),
        "vmp_create": ([P(abi.vmp_config), P(vp)], st),
        "vmp_destroy": ([vp], st),
        "vmp_last_error": ([vp], C.c_char_p),
        "vmp_process": ([vp, P(abi.vmp_scan), P(abi.vmp_imu), C.c_int, P(abi.vmp_result)], st),
        "vmp_process_device": ([vp, vp, C.c_int, d, d, vp, C.c_int, P(abi.vmp_result)], st),
        "vmp_map_index": ([vp, P(d), C.c_int, P(C.c_int64)], st),
        "vmp_map_build": ([vp, P(d), P(d), C.c_int], st),
        "vmp_map_update": ([vp, P(d), P(d), C.c_int], st),
        "vmp_map_info_get": ([vp, P(abi.vmp_map_info)], st),
        "vmp_map_export": ([vp, P(abi.vmp_voxel), C.c_longlong, P(C.c_longlong)], st),
        "vmp_map_keys": ([vp, P(C.c_int64), C.c_longlong, P(C.c_longlong)], st),
        "vmp_map_import": ([vp, P(abi.vmp_voxel), C.c_longlong, P(d), P(d), C.c_longlong], st),
        "vmp_map_export_points": ([vp, P(d), P(d), C.c_longlong, P(C.c_longlong)], st),
        "vmp_residual_reduce": ([vp, P(abi.vmp_state), P(d), P(d), P(d), C.c_int, P(d), P(d), P(C.c_int)], st),
        "vmp_get_state": ([vp, P(abi.vmp_state), P(d)], st),
        "vmp_set_state": ([vp, P(abi.vmp_state), P(d)], st),
        "vmp_ieskf_predict": ([vp, P(d), P(d), d, P(d)], st),
        "vmp_ieskf_update": ([vp, P(C.c_float), C.c_int, P(C.c_int), P(C.c_int)], st),
        "vmp_undistort": ([vp, P(abi.vmp_scan), P(abi.vmp_imu), C.c_int, P(abi.vmp_point)], st),
        "vmp_downsample": ([vp, P(abi.vmp_point), C.c_int, d, P(abi.vmp_point), P(C.c_int)], st),
        "vmp_residual_valid": ([vp, P(C.c_ubyte), C.c_int], st),
        "vmp_last_cloud": ([vp, C.c_int, P(abi.vmp_point), C.c_int, P(C.c_int)], st),
        "vmp_set_merge_mode": ([vp, C.c_int], st),
        "vmp_profile_enable": ([vp, C.c_int], st),
        "vmp_profile_read": ([vp, P(d), P(C.c_longlong), P(C.c_longlong)], st),
        "vmp_cuda_stream": ([vp], vp),
        "vmp_launch_count": ([], C.c_longlong),
        "vmp_io_bytes": ([vp, P(C.c_longlong), P(C.c_longlong)], st),
        "vmp_last_merge_rounds": ([vp], C.c_int),
        "vmp_last_merge_calls": ([vp], C.c_int),
        "vmp_last_merge_profile": ([vp, P(d), C.c_int], C.c_int),
        "vmp_device_bytes": ([vp], C.c_longlong),
        "vmp_eviction_splits": ([vp], C.c_longlong),
        "vmp_set_wait_mode": ([vp, C.c_int], st),
        "vmp_set_graphs": ([vp, C.c_int], st),
        "vmp_server_config_default": ([P(abi.vmp_server_config)], None),
        "vmp_server_create": ([P(abi.vmp_server_config), P(vp)], st),
        "vmp_server_destroy": ([vp], st),
        "vmp_server_open_stream": ([vp, P(abi.vmp_config), P(C.c_int)], st),
        "vmp_server_open_stream_wait": ([vp, P(abi.vmp_config), C.c_int, P(C.c_int)], st),
        "vmp_server_close_stream": ([vp, C.c_int], st),
        "vmp_submit": ([vp, C.c_int, P(abi.vmp_scan), P(abi.vmp_imu), C.c_int, C.c_longlong], st),
        "vmp_submit_device": ([vp, C.c_int, vp, C.c_int, d, d, vp, C.c_int, C.c_longlong], st),
        "vmp_submit_livox": ([vp, C.c_int, vp, C.c_int, C.c_int, d, d, d, P(abi.vmp_imu), C.c_int, C.c_longlong], st),
        "vmp_poll": ([vp, P(abi.vmp_server_result), C.c_int, C.c_int], C.c_int),
        "vmp_server_stream": ([vp, C.c_int, P(vp)], st),
        "vmp_server_info": ([vp, P(C.c_longlong), P(C.c_int), P(C.c_int), P(C.c_int)], st),
        "vmp_server_last_error": ([vp], C.c_char_p),
        "vmp_server_tuning": ([vp, P(C.c_int), P(C.c_longlong), P(d)], st),
        "vmp_server_knob": ([vp, C.c_char_p, P(C.c_int)], st),
        "vmp_set_residual_ctas_per_sm": ([C.c_int], st),
        "vmp_test_autotune": ([C.c_int, C.c_int, C.c_int, vp, C.c_int, vp], st),
        "vmp_fit_planes": ([vp, vp, vp, C.c_int, C.c_longlong, P(abi.vmp_fit_params), vp], st),
        "vmp_fit_planes_device": ([vp, vp, vp, C.c_int, C.c_longlong, P(abi.vmp_fit_params), vp, vp], st),
        "vmp_fit_profile": ([C.c_int], st),
        "vmp_map_planes": ([vp, vp, C.c_int, P(C.c_int)], st),
        "vmp_test_division": ([vp, vp, C.c_int, vp, vp], st),
        "vmp_test_body_cov": ([vp, C.c_int, d, d, vp, vp], st),
        "vmp_test_hat_sandwich": ([vp, vp, C.c_int, vp], st),
        "vmp_test_barrier_timeout": ([C.c_int, C.c_longlong, P(C.c_int), P(d)], st),
        "vmp_std_plane_voxels": ([vp, C.c_int, C.c_int, d, C.c_int, d, vp, C.c_int, P(C.c_int)], st),
        "vmp_livox_decode": ([vp, vp, C.c_int, C.c_int, d, d, vp, vp, P(C.c_int), P(C.c_float)], st),
        "vmp_process_decoded": ([vp, d, d, P(abi.vmp_imu), C.c_int, P(abi.vmp_result)], st),
        "vmp_output_cloud": ([vp, C.c_int, vp, vp, C.c_int, P(C.c_int)], st),
        "vmp_output_cloud_device": ([vp, C.c_int, vp, vp, C.c_int, P(C.c_int)], st),
        "vmp_fit_profile_read": ([P(d), P(C.c_longlong)], st),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def load():
    """Returns the ctypes handle of libvmp.so (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def check(handle, code):
    if code != abi.VMP_OK:
        lib = load()
        msg = lib.vmp_last_error(handle) if handle else b""
        raise VmpError(code, (msg or b"").decode(errors="replace"))
