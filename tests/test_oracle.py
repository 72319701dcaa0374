"""CPU checks of the oracle (the restated reference) -- no GPU needed.

The reference ships no tests or golden vectors for this path, so the oracle
is pinned by (a) independent numpy restatements of its building blocks,
(b) the committed golden fixtures (tests/golden, made by
tests/golden/make_golden.py) and (c) behaving as a working odometry on a
seeded synthetic sequence with ground truth.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from tests.helpers import export_oracle_map, merge_scene, plane_points

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_so3_exp_log_roundtrip(oracle_lib):
    rng = np.random.default_rng(0)
    for _ in range(200):
        w = rng.normal(0, 1.0, 3) * rng.choice([1e-12, 1e-6, 1e-2, 1.0])
        R = np.zeros(9)
        oracle_lib.orc_so3_exp(_dp(w), _dp(R))
        R = R.reshape(3, 3)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-14)
        th = np.linalg.norm(w)
        if th > 1e-8:
            k = w / th
            K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
            Rr = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
            assert np.allclose(R, Rr, atol=1e-14)
        w2 = np.zeros(3)
        oracle_lib.orc_so3_log(_dp(np.ascontiguousarray(R.reshape(9))), _dp(w2))
        if th < np.pi - 1e-3:
            assert np.allclose(w2, w, atol=1e-12, rtol=1e-10)
        else:  # log wraps to the angle in [0, pi]
            R2 = np.zeros(9)
            oracle_lib.orc_so3_exp(_dp(w2), _dp(R2))
            assert np.linalg.norm(w2) <= np.pi + 1e-12
            assert np.allclose(R2.reshape(3, 3), R, atol=1e-12)


def test_eig_sym3_matches_numpy(oracle_lib):
    rng = np.random.default_rng(1)
    for _ in range(300):
        A = rng.normal(size=(3, 3))
        A = A @ A.T * rng.choice([1e-4, 1.0, 100.0])
        ev = np.zeros(3)
        V = np.zeros(9)
        oracle_lib.orc_eig_sym3(_dp(np.ascontiguousarray(A.reshape(9))), _dp(ev), _dp(V))
        V = V.reshape(3, 3)
        evn = np.linalg.eigvalsh(A)
        assert np.allclose(ev, evn, rtol=1e-12, atol=1e-14 * np.abs(evn).max())
        assert np.allclose(A @ V, V * ev, atol=1e-12 * np.abs(evn).max())


def _calc_body_cov_numpy(p, range_inc, degree_inc):
    p = p.copy()
    if p[2] == 0:
        p[2] = 0.001
    r = np.linalg.norm(p)
    d = p / r
    s = np.sin(degree_inc * 0.017453293)
    dh = np.array([[0, -d[2], d[1]], [d[2], 0, -d[0]], [-d[1], d[0], 0]])
    b1 = np.array([1, 1, -(d[0] + d[1]) / d[2]])
    b1 /= np.linalg.norm(b1)
    b2 = np.cross(b1, d)
    b2 /= np.linalg.norm(b2)
    A = r * dh @ np.stack([b1, b2], 1)
    return p, np.outer(d, d) * range_inc ** 2 + A @ np.diag([s * s, s * s]) @ A.T


def test_calc_body_cov_matches_numpy(oracle_lib):
    rng = np.random.default_rng(2)
    P = rng.normal(0, 10, (500, 3))
    P[:5, 2] = 0.0  # commons.cpp:20-23 quirk
    out_p = np.zeros_like(P)
    cov = np.zeros((500, 9))
    oracle_lib.orc_calc_body_cov(_dp(P), 500, 0.04, 0.1, _dp(out_p), _dp(cov))
    for i in range(500):
        p, c = _calc_body_cov_numpy(P[i], 0.04, 0.1)
        assert np.array_equal(out_p[i], p)
        assert np.allclose(cov[i].reshape(3, 3), c, rtol=1e-12, atol=1e-15)


def _voxelgrid_numpy(pts, leaf):
    """pcl::VoxelGrid leaf-centroid filter restated in numpy (float32)."""
    inv = np.float32(1.0) / np.float32(leaf)
    xyz = pts[:, :3]
    mn, mx = xyz.min(0), xyz.max(0)
    d = ((mx - mn) * inv).astype(np.int64) + 1
    if d[0] * d[1] * d[2] > 2 ** 31 - 1:
        return pts.copy()
    minb = np.floor(mn * inv).astype(np.int64)
    maxb = np.floor(mx * inv).astype(np.int64)
    div = maxb - minb + 1
    ijk = (np.floor(xyz * inv) - minb.astype(np.float32)).astype(np.int64)
    idx = (ijk[:, 0] + ijk[:, 1] * div[0] + ijk[:, 2] * div[0] * div[1]).astype(np.uint32)
    order = np.argsort(idx, kind="stable")
    out = []
    s = 0
    while s < len(order):
        e = s + 1
        while e < len(order) and idx[order[e]] == idx[order[s]]:
            e += 1
        acc = np.zeros(4, dtype=np.float32)
        for k in range(s, e):
            acc = (acc + pts[order[k]]).astype(np.float32)
        out.append(acc / np.float32(e - s))
        s = e
    return np.array(out, dtype=np.float32)


def test_downsample_matches_numpy(oracle_lib):
    rng = np.random.default_rng(4)
    n = 3000
    pts = np.zeros((n, 4), dtype=np.float32)
    pts[:, :3] = rng.uniform(-3, 3, (n, 3)).astype(np.float32)
    pts[:, 3] = np.arange(n, dtype=np.float32) * 0.01
    out = (abi.vmp_point * n)()
    m = oracle_lib.orc_downsample(pts.ctypes.data_as(C.POINTER(abi.vmp_point)), n, 0.5, out)
    o = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), shape=(n, 4))[:m]
    ref = _voxelgrid_numpy(pts, 0.5)
    assert o.shape == ref.shape
    assert np.array_equal(o, ref)


def test_map_semantics_small(oracle_lib):
    """VoxelGrid state machine on a hand-made case: a single voxel receives
    points; refits at 10, 20, ...; freezes at 100; then merges run."""
    cfg = abi.default_config()
    h = oracle_lib.orc_create(C.byref(cfg))
    try:
        rng = np.random.default_rng(5)
        # plane z = 0.25 inside voxel (0,0,0)
        pts = np.c_[rng.uniform(0.01, 0.49, (130, 2)), np.full(130, 0.25)]
        cov = np.tile(np.eye(3).reshape(9) * 1e-4, (130, 1))
        oracle_lib.orc_map_update(h, _dp(pts[:9].copy()), _dp(cov[:9].copy()), 9)
        info = abi.vmp_map_info()
        oracle_lib.orc_map_info(h, C.byref(info))
        arr = (abi.vmp_voxel * 1)()
        oracle_lib.orc_map_export(h, arr, 1)
        assert arr[0].n == 9 and arr[0].is_init == 0
        oracle_lib.orc_map_update(h, _dp(pts[9:10].copy()), _dp(cov[9:10].copy()), 1)
        oracle_lib.orc_map_export(h, arr, 1)
        assert arr[0].n == 10 and arr[0].is_init == 1 and arr[0].is_plane == 1
        assert abs(abs(arr[0].norm[2]) - 1.0) < 1e-9
        oracle_lib.orc_map_update(h, _dp(pts[10:100].copy()), _dp(cov[10:100].copy()), 90)
        oracle_lib.orc_map_export(h, arr, 1)
        assert arr[0].n == 100 and arr[0].update_enable == 0 and arr[0].n_temp == 0
        oracle_lib.orc_map_update(h, _dp(pts[100:].copy()), _dp(cov[100:].copy()), 30)
        oracle_lib.orc_map_export(h, arr, 1)
        assert arr[0].n == 100  # frozen: points dropped
    finally:
        oracle_lib.orc_destroy(h)


def test_merge_scene_merges(oracle_lib):
    """The merge fixture does what the GPU merge test relies on: the first
    re-observation batch merges most voxels of the floor and the wall (one
    group per surface is not reached in one batch: merge() gives a
    neighbour the caller's group, so later callers regroup it) and every
    voxel is a plane."""
    rng = np.random.default_rng(21)
    (P, Cv), updates = merge_scene(rng)
    cfg = abi.default_config(map_capacity=200000, max_scan_points=120000)
    h = oracle_lib.orc_create(C.byref(cfg))
    try:
        oracle_lib.orc_map_build(h, _dp(P), _dp(Cv), len(P))
        vo, no, _, _, _ = export_oracle_map(oracle_lib, h)
        assert no == 768 and all(vo[i].is_plane and not vo[i].merged for i in range(no))
        P2, C2 = updates[0]
        oracle_lib.orc_map_update(h, _dp(P2), _dp(C2), len(P2))
        vo, no, _, _, _ = export_oracle_map(oracle_lib, h)
        merged = [vo[i] for i in range(no) if vo[i].merged]
        assert len(merged) > 600
        assert len(set(vo[i].group_id for i in range(no))) < no
    finally:
        oracle_lib.orc_destroy(h)


def test_oracle_tracks_ground_truth():
    import oracle
    seq = synth.Sequence(synth.KIND_ROOM, points_per_scan=6000)
    cfg = abi.default_config(scan_resolution=0.2)
    o = oracle.Oracle(cfg)
    errs = []
    p0 = None
    for k in range(40):
        pkg = seq.next()
        r = o.process(pkg)
        _, pg = seq.pose(pkg.t_end)
        if p0 is None:
            p0 = pg
        if r.lio_status == abi.LIO_MAPPING:
            errs.append(np.linalg.norm(np.array(r.x.pos[:]) - (pg - p0)))
    assert max(errs) < 0.1, max(errs)


@pytest.mark.parametrize("name", ["map_small", "scan_room"])
def test_oracle_matches_golden(oracle_lib, name):
    path = os.path.join(GOLDEN, name + ".json")
    if not os.path.exists(path):
        pytest.skip("golden fixture not generated")
    from tests.golden import make_golden
    g = json.load(open(path))
    cur = make_golden.compute(name)
    assert cur["digest"] == g["digest"], f"{name}: oracle output changed"
    for k in g["values"]:
        assert np.allclose(np.array(cur["values"][k]), np.array(g["values"][k]), rtol=1e-12, atol=1e-12), k
