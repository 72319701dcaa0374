"""C ABI checks that need no GPU: the library loads, exports every function
include/vmp.h declares, and the ctypes mirror has the C compiler's layout."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from voxelmapplus_fastlio2_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vmp.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vmp_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("vmp_create", "vmp_destroy", "vmp_process", "vmp_map_build", "vmp_map_update",
                 "vmp_residual_reduce", "vmp_ieskf_predict", "vmp_ieskf_update", "vmp_undistort",
                 "vmp_downsample", "vmp_map_export", "vmp_map_import"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from voxelmapplus_fastlio2_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from voxelmapplus_fastlio2_gb300 import build
        build.build_all()
    lib = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.vmp_abi_version() == 2


def test_config_default_matches_lioconfig():
    from voxelmapplus_fastlio2_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libvmp.so not built")
    lib = _lib.load()
    c = abi.vmp_config()
    lib.vmp_config_default(C.byref(c))
    # lio::LIOConfig defaults (lio_builder.h:17-42)
    assert c.opti_max_iter == 5 and c.imu_init_num == 20
    assert (c.na, c.ng, c.nba, c.nbg) == (0.01, 0.01, 0.0001, 0.0001)
    assert list(c.r_il) == [1, 0, 0, 0, 1, 0, 0, 0, 1] and list(c.p_il) == [0, 0, 0]
    assert c.gravity_align == 1 and c.estimate_ext == 0
    assert (c.scan_resolution, c.voxel_size) == (0.1, 0.5)
    assert (c.update_size_thresh, c.max_point_thresh, c.plane_thresh) == (10, 100, 0.01)
    assert (c.ranging_cov, c.angle_cov) == (0.04, 0.1)
    assert (c.merge_thresh_for_angle, c.merge_thresh_for_distance) == (0.1, 0.04)
    assert c.map_capacity == 100000 and c.ieskf_max_iter == 5 and c.ieskf_eps == 0.001


def test_struct_layouts_match_c():
    structs = ["vmp_config", "vmp_point", "vmp_imu", "vmp_scan", "vmp_state", "vmp_result", "vmp_map_info",
               "vmp_voxel", "vmp_server_config", "vmp_server_result"]
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "vmp.h"\nint main(void){\n'
    for s in structs:
        src += f'printf("{s} %zu\\n", sizeof({s}));\n'
    src += 'printf("off_result_x %zu\\n", offsetof(vmp_result, x));\n'
    src += 'printf("off_voxel_mean %zu\\n", offsetof(vmp_voxel, mean));\n'
    src += 'printf("off_config_map_capacity %zu\\n", offsetof(vmp_config, map_capacity));\n'
    src += 'printf("off_sres_result %zu\\n", offsetof(vmp_server_result, result));\nreturn 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        cfile = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(cfile, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), "-o", exe, cfile])
        out = subprocess.check_output([exe], text=True)
    sizes = dict(line.split() for line in out.strip().splitlines())
    for s in structs:
        assert int(sizes[s]) == C.sizeof(getattr(abi, s)), s
    assert int(sizes["off_result_x"]) == abi.vmp_result.x.offset
    assert int(sizes["off_voxel_mean"]) == abi.vmp_voxel.mean.offset
    assert int(sizes["off_config_map_capacity"]) == abi.vmp_config.map_capacity.offset
    assert int(sizes["off_sres_result"]) == abi.vmp_server_result.result.offset


def test_no_gpu_path_fails_loudly():
    """Without a GPU, vmp_create must refuse (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from voxelmapplus_fastlio2_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libvmp.so not built")
    lib = _lib.load()
    h = C.c_void_p()
    code = lib.vmp_create(None, C.byref(h))
    assert code == 6  # VMP_ERR_CUDA
    assert not h.value
