"""The drop-in C++ builder (include/vmp_lio_builder.hpp behind the
include/vmp_node/map_builder/ headers) as the ROS node uses it.

tests/adapter_node/node_main.cpp is a LIONode-like program: it includes
"map_builder/lio_builder.h" and makes the node's calls with the node's
expressions (lio_node.cpp:44, 171-178, 185-190, 227; the map walk of
utils.cpp:154-208).  It is compiled against mock Eigen / PCL headers and mock
kf::State / lio::SyncPackage types (tests/adapter_node/mock; the image has no
Eigen, PCL or ROS) and linked with libvmp.so.

* CPU: the program compiles and links unchanged.
* GPU: driven over a seeded room sequence, its per-scan pose, 6x6 pose
  covariance, body / world clouds and plane markers match the oracle's
  LIOBuilder::process, kf.x(), kf.P(), lidarToBody / lidarToWorld and the
  frozen-plane walk of voxel2MarkerArray.
"""
import ctypes as C
import os
import struct
import subprocess

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from tests.helpers import rot_angle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NODE = os.path.join(ROOT, "tests", "adapter_node")


def _compile(out_dir):
    from voxelmapplus_fastlio2_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_all()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = os.path.join(out_dir, "node_main")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-Wall", "-Werror",
                           "-I", os.path.join(ROOT, "include", "vmp_node"), "-I", os.path.join(NODE, "mock"),
                           "-I", os.path.join(ROOT, "include"), "-o", exe, os.path.join(NODE, "node_main.cpp"),
                           "-L" + libdir, "-lvmp", "-Wl,-rpath," + libdir])
    return exe


def test_node_program_compiles_against_drop_in_headers(tmp_path):
    exe = _compile(str(tmp_path))
    assert os.path.exists(exe)


def _write_packages(path, pkgs):
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(pkgs)))
        for p in pkgs:
            f.write(struct.pack("<iidd", p.n, p.n_imu, p.t_start, p.t_end))
            f.write(p.points_np().astype(np.float32).tobytes())
            imu = np.zeros((p.n_imu, 7))
            for i in range(p.n_imu):
                m = p.imus[i]
                imu[i] = [m.t, *m.acc[:], *m.gyro[:]]
            f.write(imu.tobytes())


def _read_results(path, count):
    data = open(path, "rb").read()
    off = 0
    out = []

    def take(fmt_or_dtype, n=1):
        nonlocal off
        if isinstance(fmt_or_dtype, str):
            v = struct.unpack_from(fmt_or_dtype, data, off)
            off += struct.calcsize(fmt_or_dtype)
            return v
        a = np.frombuffer(data, dtype=fmt_or_dtype, count=n, offset=off)
        off += a.nbytes
        return a

    for _ in range(count):
        (status,) = take("<i")
        r = {"status": status}
        if status == abi.LIO_MAPPING:
            pose = take(np.float64, 12)
            r["pos"], r["rot"] = pose[:3], pose[3:]
            r["P6"] = take(np.float64, 36).reshape(6, 6)
            for name in ("body", "world"):
                (n,) = take("<i")
                r[name] = take(np.float32, 3 * n).reshape(n, 3)
            (n,) = take("<i")
            mk = np.dtype([("center", "<f8", 3), ("trace", "<f8"), ("norm", "<f8", 3), ("merged", "<i4")])
            r["markers"] = take(mk, n)
        out.append(r)
    assert off == len(data)
    return out


def _oracle_plane_walk(o):
    """The frozen planes in LRU order, as voxel2MarkerArray walks the map."""
    info = abi.vmp_map_info()
    o.lib.orc_map_info(o.h, C.byref(info))
    arr = (abi.vmp_voxel * max(1, info.size))()
    n = o.lib.orc_map_export(o.h, arr, info.size)
    v = np.frombuffer(C.string_at(arr, n * C.sizeof(abi.vmp_voxel)), dtype=np.dtype(abi.vmp_voxel), count=n)
    sel = (v["is_plane"] != 0) & (v["update_enable"] == 0)
    return v[sel]


@pytest.mark.gpu
def test_node_program_on_gpu_matches_oracle(tmp_path):
    import oracle
    exe = _compile(str(tmp_path))
    seq = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    pkgs = [seq.next() for _ in range(30)]
    pin, pout = str(tmp_path / "packages.bin"), str(tmp_path / "results.bin")
    _write_packages(pin, pkgs)
    run = subprocess.run([exe, pin, pout], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert run.returncode == 0, run.stdout
    res = _read_results(pout, len(pkgs))
    cfg = abi.default_config(scan_resolution=0.2)
    o = oracle.Oracle(cfg)
    mapping = 0
    for k, (p, r) in enumerate(zip(pkgs, res)):
        ro = o.process(p)
        assert r["status"] == ro.lio_status, k
        if ro.lio_status != abi.LIO_MAPPING:
            continue
        mapping += 1
        dp = float(np.max(np.abs(r["pos"] - np.array(ro.x.pos[:]))))
        da = rot_angle(r["rot"], ro.x.rot[:])
        assert dp <= 1e-6 and da <= 1e-6, (k, dp, da)
        Po = np.array(ro.P[:]).reshape(23, 23)[:6, :6]
        assert np.max(np.abs(r["P6"] - Po)) <= 1e-6 * np.max(np.abs(Po)), k
        body, _ = o.output_cloud(0)
        world, _ = o.output_cloud(1)
        assert np.array_equal(r["body"], body[:, :3]), k
        assert r["world"].shape == world[:, :3].shape
        assert np.max(np.abs(r["world"] - world[:, :3])) <= 1e-5 * max(1.0, float(np.max(np.abs(world)))), k
        planes = _oracle_plane_walk(o)
        mk = r["markers"]
        assert len(mk) == len(planes), k
        # centres are means of float world points, whose transform is the
        # float cast of the pose (lio_builder.cpp:155-163): equal unless that
        # cast differs in a last bit
        assert np.allclose(mk["center"], planes["center"], rtol=0, atol=1e-6), k
        assert np.array_equal(mk["merged"], planes["merged"]), k
        assert np.allclose(mk["norm"], planes["norm"], rtol=0, atol=1e-9), k
        tr = planes["cov"][:, [0, 7, 14]].sum(axis=1)
        assert np.allclose(mk["trace"], tr, rtol=1e-9, atol=0), k
    assert mapping >= 25
