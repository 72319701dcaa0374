"""The steps either side of the path: Livox CustomMsg decode (livox2pcl,
src/utils.cpp:3-28) on the device, and the published clouds (lidarToBody /
lidarToWorld, lio_builder.cpp:155-173) from the device's undistorted cloud."""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from tests.helpers import rot_angle


def random_livox(rng, n, t_ms=None):
    """Livox points with every line / tag class, ranges around the gates and
    points placed exactly on a gate."""
    a = np.zeros(n, dtype=abi.livox_dtype())
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.uniform(0.05, 30.0, n)
    p = (d * r[:, None]).astype(np.float32)
    p[:8] = np.array([[0.5, 0, 0], [0, 20.0, 0], [0, 0, -0.5], [20.0, 0, 0], [0.3, 0.4, 0], [12, 16, 0],
                      [0.49999997, 0, 0], [20.000002, 0, 0]], dtype=np.float32)
    a["x"], a["y"], a["z"] = p[:, 0], p[:, 1], p[:, 2]
    if t_ms is None:
        a["offset_time"] = np.sort(rng.integers(0, 100_000_000, n)).astype(np.uint32)
    else:
        a["offset_time"] = np.rint(np.asarray(t_ms, dtype=np.float64) * 1e6).astype(np.uint32)
    a["reflectivity"] = rng.integers(0, 256, n)
    a["tag"] = rng.choice(np.array([0x00, 0x10, 0x20, 0x30, 0x01, 0x12, 0x05, 0x16], dtype=np.uint8), n)
    a["line"] = rng.choice(np.array([0, 1, 2, 3, 4, 5], dtype=np.uint8), n, p=[0.2, 0.2, 0.2, 0.2, 0.1, 0.1])
    return a


def _numpy_livox2pcl(a, filter_num, rmin, rmax):
    keep = []
    valid_num = 0
    for i, q in enumerate(a):
        if q["line"] < 4 and ((q["tag"] & 0x30) == 0x10 or (q["tag"] & 0x30) == 0x00):
            k = valid_num
            valid_num += 1
            if k % filter_num != 0:
                continue
            x, y, z = np.float32(q["x"]), np.float32(q["y"]), np.float32(q["z"])
            sq = float(np.float32(np.float32(x * x) + np.float32(y * y)) + np.float32(z * z))
            if rmin * rmin < sq < rmax * rmax:
                keep.append(i)
    return np.array(keep, dtype=np.int64)


def test_livox_point_layout():
    assert C.sizeof(abi.vmp_livox_point) == 20 == abi.livox_dtype().itemsize
    assert abi.vmp_livox_point.reflectivity.offset == 16 and abi.vmp_livox_point.line.offset == 18


@pytest.mark.parametrize("filter_num", [1, 3])
def test_oracle_livox_decode_matches_numpy(oracle_lib, filter_num):
    import oracle
    rng = np.random.default_rng(7 + filter_num)
    a = random_livox(rng, 3000)
    pts, inten = oracle.livox_decode(a, filter_num, 0.5, 20.0)
    keep = _numpy_livox2pcl(a, filter_num, 0.5, 20.0)
    assert len(pts) == len(keep) > 0
    assert np.array_equal(pts[:, 0], a["x"][keep]) and np.array_equal(pts[:, 2], a["z"][keep])
    assert np.array_equal(pts[:, 3], a["offset_time"][keep].astype(np.float32) / np.float32(1e6))
    assert np.array_equal(inten, a["reflectivity"][keep].astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("filter_num", [1, 2, 5])
def test_livox_decode_matches_oracle(filter_num):
    import oracle
    from voxelmapplus_fastlio2_gb300 import lio
    rng = np.random.default_rng(100 + filter_num)
    a = random_livox(rng, 50000)
    g = lio.LIOBuilder(abi.default_config(max_scan_points=65536))
    pts, inten, last = g.livox_decode(a, filter_num, 0.5, 20.0)
    opts, ointen = oracle.livox_decode(a, filter_num, 0.5, 20.0)
    assert pts.tobytes() == opts.tobytes()
    assert inten.tobytes() == ointen.tobytes()
    assert last == opts[-1, 3]
    # an empty decode leaves nothing to process
    e, _, _ = g.livox_decode(a[:0], filter_num, 0.5, 20.0)
    assert len(e) == 0
    # a message whose points all fail the line test keeps none
    b = a.copy()
    b["line"] = 4
    e, _, _ = g.livox_decode(b, filter_num, 0.5, 20.0)
    assert len(e) == 0 and len(oracle.livox_decode(b, filter_num, 0.5, 20.0)[0]) == 0
    # and the next message decodes as before
    pts2, _, last2 = g.livox_decode(a, filter_num, 0.5, 20.0)
    assert pts2.tobytes() == opts.tobytes() and last2 == last
    g.close()


def _to_livox(rng, pkg):
    pts = pkg.points_np()
    a = np.zeros(pkg.n, dtype=abi.livox_dtype())
    a["x"], a["y"], a["z"] = pts[:, 0], pts[:, 1], pts[:, 2]
    a["offset_time"] = np.rint(pts[:, 3].astype(np.float64) * 1e6).astype(np.uint32)
    a["reflectivity"] = rng.integers(0, 256, pkg.n)
    a["tag"] = rng.choice(np.array([0x00, 0x10, 0x20], dtype=np.uint8), pkg.n, p=[0.6, 0.35, 0.05])
    a["line"] = rng.choice(np.array([0, 1, 2, 3, 4], dtype=np.uint8), pkg.n, p=[0.24, 0.24, 0.24, 0.24, 0.04])
    return a


@pytest.mark.gpu
def test_decoded_sequence_and_output_clouds_match_oracle():
    """Livox packages decoded on the device, processed without a re-upload,
    and the published body / world clouds: identical to the oracle's
    livox2pcl -> process -> lidarToBody / lidarToWorld, intensities carried
    through the time sort."""
    import oracle
    from voxelmapplus_fastlio2_gb300 import lio
    rng = np.random.default_rng(5)
    seq = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=16384)
    g = lio.LIOBuilder(cfg)
    o = oracle.Oracle(cfg)
    checked = 0
    for k in range(14):
        pkg = seq.next()
        a = _to_livox(rng, pkg)
        pts, inten, last = g.livox_decode(a, 1, 0.1, 100.0)
        opts, ointen = oracle.livox_decode(a, 1, 0.1, 100.0)
        assert pts.tobytes() == opts.tobytes() and inten.tobytes() == ointen.tobytes()
        rg = g.process_decoded(pkg.t_start, pkg.t_end, pkg.imus, pkg.n_imu)
        ro = o.process_points(opts, pkg.t_start, pkg.t_end, pkg.imus, pkg.n_imu, ointen)
        assert rg.lio_status == ro.lio_status and rg.n_raw == len(opts)
        if ro.lio_status != abi.LIO_MAPPING:
            continue
        assert rg.n_down == ro.n_down and rg.iters == ro.iters and rg.map_size == ro.map_size, k
        assert np.max(np.abs(np.array(rg.x.pos[:]) - np.array(ro.x.pos[:]))) < 1e-9, k
        assert rot_angle(rg.x.rot[:], ro.x.rot[:]) < 1e-9, k
        for frame in (0, 1):
            cg, ig = g.output_cloud(frame)
            co, io = o.output_cloud(frame)
            assert len(cg) == len(co) == len(opts)
            assert ig.tobytes() == io.tobytes(), (k, frame)
            if frame == 0:
                assert cg.tobytes() == co.tobytes(), k
            else:  # the state agrees to ~1e-15: its float cast may differ in the last bit
                assert np.max(np.abs(cg - co)) <= 1e-5 * max(1.0, float(np.max(np.abs(co)))), k
                assert np.array_equal(cg[:, 3], co[:, 3])
        checked += 1
    assert checked >= 10
    # a plain vmp_process scan has no intensities
    g.process(seq.next())
    _, ig = g.output_cloud(0)
    assert not np.any(ig)
    with pytest.raises(Exception):
        g.process_decoded(0.0, 0.1, seq.next().imus, 1)
    g.close()


def _oracle_planes(o, max_markers):
    out = np.zeros(max(1, max_markers), dtype=abi.plane_marker_dtype())
    n = o.lib.orc_map_planes(o.h, out.ctypes.data_as(C.POINTER(abi.vmp_plane_marker)), max_markers)
    return out[:n]


@pytest.mark.gpu
def test_map_planes_match_oracle():
    """voxel2MarkerArray's data compacted on the device: the frozen planes in
    LRU order, centre / normal bit-identical (the points are), trace and
    orientation within rounding, the jet colour within one step."""
    import oracle
    from voxelmapplus_fastlio2_gb300 import lio
    seq_g = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    seq_o = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=16384)
    g = lio.LIOBuilder(cfg)
    o = oracle.Oracle(cfg)
    for _ in range(16):
        g.process(seq_g.next())
        o.process(seq_o.next())
    for cap in (50, 100000):
        mg = g.map.planes(cap)
        mo = _oracle_planes(o, cap)
        assert len(mg) == len(mo) > 0, cap
        assert np.array_equal(mg["center"], mo["center"]) and np.array_equal(mg["norm"], mo["norm"])
        assert np.array_equal(mg["merged"], mo["merged"])
        # plane covariances carry the point covariances, which depend on the
        # filter covariance P (equal to ~1e-15, not bit for bit)
        assert np.allclose(mg["trace"], mo["trace"], rtol=1e-9, atol=0)
        assert np.max(np.abs(mg["orientation"] - mo["orientation"])) < 1e-12
        assert np.max(np.abs(mg["rgb"].astype(int) - mo["rgb"].astype(int))) <= 1
    assert len(mo) < g.map.info().size  # only the frozen planes
    g.close()
