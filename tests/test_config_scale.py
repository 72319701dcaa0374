"""Parity at the workload sizes of the three odometry configurations, GPU
against the CPU oracle, scan by scan, through the C ABI.

* room: 20x20x5 m room, rosette LiDAR at 20 000 rays per scan, downsampled
  at 0.25 m to about 4 000 points, 5 IEKF iterations, 62 mapping scans;
* urban block: 100x100x20 m block, 128-beam spinning LiDAR at 200 000 rays
  per scan (~173 000 returns, ~130 000 points after the 0.1 m downsample),
  4 IEKF iterations, 12 mapping scans on a map holding more than 1.2 M voxels;
* corridor: 1 km corridor, 32-beam spinning LiDAR at 100 000 rays per scan,
  0.2 m downsample, an LRU capacity of 4 500 voxels that the map reaches after
  a few scans, so that most of the 45 mapping scans evict.

Checked at every mapping scan (LIOBuilder::process, lio_builder.cpp:175-248):
the LIO status, downsampled point count, effective residual count, IEKF
iteration count and map size are identical; the voxel keys of the map are
identical in LRU order (the reference's featmap key set and its cache list,
voxel_map.h:124-125); the match set -- ResidualData::is_valid of every
downsampled point after the last iteration (lio_builder.cpp:260-274) -- is
identical; the pose is within 1e-6 m and 1e-6 rad of the oracle's (the bar
the odometry path is specified to) and P within 1e-6 relative.  At the end
the maps' integer fields (counts, flags, group ids) are identical and their
floating-point fields agree to rounding level.

The urban block at 0.5 m voxels holds about 30 000 surface voxels after a
dozen scans, far from the ~2 M voxels the workload description anticipates
(a 100x100x20 m block has only 1.6 M voxels of volume).  To run the hash and
the record pool at that scale, the map built from the first scan is extended
on both sides, through the map import entry points, with 1.2 M frozen voxels
of a plane 500 m above the block (least recently used, no point reaches
them), and the sequence continues on that 1.2 M-voxel map.
"""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from tests.helpers import rot_angle

pytestmark = pytest.mark.gpu

VOXEL_DTYPE = np.dtype(abi.vmp_voxel)
INT_FIELDS = ("key", "n", "newly_add_point", "is_init", "is_plane", "update_enable", "merged", "group_id", "n_temp")


def _oracle(cfg):
    import os
    import oracle as orc
    return orc.Oracle(cfg, threads=max(1, min(16, os.cpu_count() or 1)))


def _voxels_np(arr, n):
    return np.frombuffer(C.string_at(arr, n * VOXEL_DTYPE.itemsize), dtype=VOXEL_DTYPE, count=n)


def _oracle_export(o):
    info = abi.vmp_map_info()
    o.lib.orc_map_info(o.h, C.byref(info))
    arr = (abi.vmp_voxel * max(1, info.size))()
    n = o.lib.orc_map_export(o.h, arr, info.size)
    pts = np.zeros((max(1, info.slab_points), 3))
    cov = np.zeros((max(1, info.slab_points), 9))
    m = o.lib.orc_map_export_points(o.h, pts.ctypes.data_as(C.POINTER(C.c_double)),
                                    cov.ctypes.data_as(C.POINTER(C.c_double)), info.slab_points)
    return arr, n, info, pts[:m], cov[:m]


def _compare_final_maps(g, o):
    vg, ng = g.map.export()
    vo, no, _, _, _ = _oracle_export(o)
    assert ng == no
    a = _voxels_np(vg, ng)
    b = _voxels_np(vo, no)
    for f in INT_FIELDS:
        bad = np.flatnonzero(np.any((a[f] != b[f]).reshape(ng, -1), axis=1))
        assert bad.size == 0, f"{f} differs at {bad.size} voxels (first {a['key'][bad[0]]})"
    for f, tol in (("mean", 1e-9), ("ppt", 1e-9), ("norm", 1e-6), ("center", 1e-9), ("cov", 1e-6)):
        x, y = a[f].reshape(ng, -1), b[f].reshape(ng, -1)
        scale = np.maximum(1e-12, np.max(np.abs(y), axis=1, keepdims=True))
        err = np.max(np.abs(x - y) / scale)
        assert err <= tol, (f, err)


def _run(kind, rays, cfg, scans, extend_map=None, min_evicting=0):
    """Runs `scans` packages of one seeded sequence through the GPU library
    and the oracle (the same packages), checking every mapping scan."""
    from voxelmapplus_fastlio2_gb300 import lio
    seq = synth.Sequence(kind, points_per_scan=rays)
    g = lio.LIOBuilder(cfg)
    o = _oracle(cfg)
    worst = [0.0, 0.0, 0.0]
    mapping = evicting = 0
    try:
        for k in range(scans):
            pkg = seq.next()
            rg = g.process(pkg)
            ro = o.process(pkg)
            assert rg.lio_status == ro.lio_status, k
            if ro.lio_status == abi.LIO_MAPPING and extend_map is not None and k == 1:
                extend_map(g, o)
            if ro.lio_status != abi.LIO_MAPPING or rg.n_down == 0:
                continue
            mapping += 1
            assert (rg.n_down, rg.effect_num, rg.iters, rg.map_size) == \
                (ro.n_down, ro.effect_num, ro.iters, ro.map_size), k
            evicting += ro.evicted > 0
            kg, ko = g.map.keys(), o.map_keys()
            assert kg.shape == ko.shape and np.array_equal(kg, ko), f"scan {k}: voxel keys / LRU order differ"
            vg, vo = g.residual_valid(rg.n_down), o.residual_valid(ro.n_down)
            assert np.array_equal(vg, vo), f"scan {k}: match sets differ at {np.flatnonzero(vg != vo)[:10]}"
            dp = float(np.max(np.abs(np.array(rg.x.pos[:]) - np.array(ro.x.pos[:]))))
            da = rot_angle(rg.x.rot[:], ro.x.rot[:])
            Pg, Po = np.array(rg.P[:]), np.array(ro.P[:])
            dP = float(np.max(np.abs(Pg - Po)) / np.max(np.abs(Po)))
            assert dp <= 1e-6 and da <= 1e-6 and dP <= 1e-6, (k, dp, da, dP)
            worst = [max(worst[0], dp), max(worst[1], da), max(worst[2], dP)]
        _compare_final_maps(g, o)
    finally:
        g.close()
    assert evicting >= min_evicting, evicting
    return mapping, worst, rg


def test_room_20k_rays_62_mapping_scans():
    cfg = abi.default_config(scan_resolution=0.25, max_scan_points=20064, map_capacity=100000)
    mapping, worst, last = _run(synth.KIND_ROOM, 20000, cfg, 64)
    assert mapping >= 60
    assert 3000 <= last.n_down <= 6000  # ~4k points per scan


def _filler_voxels(n, group_base, max_points):
    """n frozen non-plane voxels on a 0.5 m grid 500 m above the block."""
    side = int(np.ceil(np.sqrt(n)))
    v = np.zeros(n, dtype=VOXEL_DTYPE)
    i = np.arange(n)
    v["key"][:, 0] = i % side - side // 2
    v["key"][:, 1] = i // side - side // 2
    v["key"][:, 2] = 1000
    v["n"] = max_points
    v["is_init"] = 1
    v["group_id"] = group_base + i
    centre = (v["key"].astype(np.float64) + 0.5) * 0.5
    v["mean"] = centre
    v["center"] = centre
    v["ppt"] = (centre[:, :, None] * centre[:, None, :]).reshape(n, 9) + np.eye(3).reshape(9) * 0.02
    return v


def test_urban_200k_rays_on_a_1m_voxel_map():
    cfg = abi.default_config(scan_resolution=0.1, map_capacity=4000000, ieskf_max_iter=4, max_scan_points=200064)
    n_fill = 1_200_000

    def extend(g, o):
        arr, n, info, pts, cov = _oracle_export(o)
        own = _voxels_np(arr, n)
        fill = _filler_voxels(n_fill, info.group_counter, cfg.max_point_thresh)
        allv = np.concatenate([own, fill])
        buf = (abi.vmp_voxel * len(allv)).from_buffer_copy(allv.tobytes())
        counter = info.group_counter + n_fill
        dp = pts.ctypes.data_as(C.POINTER(C.c_double))
        dc = cov.ctypes.data_as(C.POINTER(C.c_double))
        o.lib.orc_map_import(o.h, buf, len(allv), dp, dc, counter)
        g.map.import_(buf, len(allv), pts, cov, counter)
        assert g.map.info().size == len(allv) > 1_000_000

    mapping, worst, last = _run(synth.KIND_URBAN, 200000, cfg, 14, extend_map=extend)
    assert mapping >= 12
    assert last.map_size > 1_200_000
    assert last.n_down > 100000


def test_corridor_100k_rays_evicting():
    cfg = abi.default_config(scan_resolution=0.2, map_capacity=4500, max_scan_points=100064)
    mapping, worst, last = _run(synth.KIND_CORRIDOR, 100000, cfg, 47, min_evicting=30)
    assert mapping >= 45
    assert last.map_size == 4500
