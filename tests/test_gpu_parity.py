"""GPU parity against the CPU oracle (restated reference), through the C ABI.

Tolerances: integer / index work (voxel keys, match sets, group ids, flags,
point counts, downsampled float clouds) must be identical.  FP64 results:
the map's per-voxel arithmetic runs in the reference's order on both sides
and must be bit-identical; H / b of the residual reduction differ only by the
summation order of a parallel reduction (relative 1e-9); the pose after a
scan must agree within 1e-6 m and 1e-6 rad (the target the odometry hot path
is specified to).
"""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from tests.helpers import compare_maps, export_oracle_map, merge_scene, plane_points, rot_angle

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.fixture(scope="module")
def lio_mod():
    from voxelmapplus_fastlio2_gb300 import lio
    return lio


def test_downsample_matches_oracle(lio_mod, oracle_lib):
    rng = np.random.default_rng(7)
    g = lio_mod.LIOBuilder(abi.default_config(max_scan_points=70000))
    for trial in range(3):
        n = [1, 5000, 65000][trial]
        pts = np.zeros((n, 4), dtype=np.float32)
        pts[:, :3] = rng.uniform(-30, 30, (n, 3)).astype(np.float32)
        pts[:, 3] = np.sort(rng.uniform(0, 100, n)).astype(np.float32)
        for leaf in (0.1, 0.5):
            out_g = g.downsample(pts, leaf)
            out_o = (abi.vmp_point * n)()
            m = oracle_lib.orc_downsample(pts.ctypes.data_as(C.POINTER(abi.vmp_point)), n, leaf, out_o)
            o = np.ctypeslib.as_array(C.cast(out_o, C.POINTER(C.c_float)), shape=(n, 4))[:m]
            assert out_g.shape[0] == m
            assert np.array_equal(out_g.view(np.uint32), o.view(np.uint32))


@pytest.mark.parametrize("merge_mode", [0, 1])
def test_map_build_update_bit_exact(lio_mod, oracle_lib, merge_mode):
    rng = np.random.default_rng(11 + merge_mode)
    cfg = abi.default_config(map_capacity=200000, max_scan_points=60000)
    g = lio_mod.LIOBuilder(cfg)
    g.set_merge_mode(merge_mode)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        P, Cv = plane_points(rng, n_planes=120)
        oracle_lib.orc_map_build(o, _dp(P), _dp(Cv), len(P))
        g.map.build(P, Cv)
        for step in range(6):
            P2, C2 = plane_points(rng, n_planes=150, pts_per=(2, 90))
            oracle_lib.orc_map_update(o, _dp(P2), _dp(C2), len(P2))
            g.map.update(P2, C2)
            vo, no, info, _, _ = export_oracle_map(oracle_lib, o)
            vg, ng = g.map.export()
            problems = compare_maps(vo, no, vg, ng, exact=True)
            assert not problems, f"step {step}: " + "; ".join(problems[:8])
    finally:
        oracle_lib.orc_destroy(o)


@pytest.mark.parametrize("term_cap", [0, 300])
def test_map_update_term_buffer_overflow(lio_mod, oracle_lib, term_cap):
    """The plane-covariance terms of a batch go through a term buffer; with a
    buffer far too small most refits form their terms in the summation kernel
    instead.  Both ways the map must equal the oracle's bit for bit."""
    rng = np.random.default_rng(31)
    cfg = abi.default_config(map_capacity=200000, max_scan_points=60000)
    cfg.reserved[1] = term_cap
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        P, Cv = plane_points(rng, n_planes=80, pts_per=(40, 160), iso_frac=0.0)
        oracle_lib.orc_map_build(o, _dp(P), _dp(Cv), len(P))
        g.map.build(P, Cv)
        for step in range(4):
            P2, C2 = plane_points(rng, n_planes=120, pts_per=(20, 120), iso_frac=0.0)
            oracle_lib.orc_map_update(o, _dp(P2), _dp(C2), len(P2))
            g.map.update(P2, C2)
            vo, no, info, _, _ = export_oracle_map(oracle_lib, o)
            vg, ng = g.map.export()
            problems = compare_maps(vo, no, vg, ng, exact=True)
            assert not problems, f"step {step}: " + "; ".join(problems[:8])
    finally:
        oracle_lib.orc_destroy(o)


@pytest.mark.parametrize("merge_mode", [0, 1])
def test_map_merges_bit_exact(lio_mod, oracle_lib, merge_mode):
    """VoxelGrid::merge chains: frozen floor and wall voxels re-observed in
    random order.  The whole map (group ids, merged flags, merged planes and
    covariances included) must equal the oracle's after every batch; the
    parallel fixed point must have needed several rounds."""
    rng = np.random.default_rng(21)
    (P, Cv), updates = merge_scene(rng)
    cfg = abi.default_config(map_capacity=200000, max_scan_points=120000)
    g = lio_mod.LIOBuilder(cfg)
    g.set_merge_mode(merge_mode)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        oracle_lib.orc_map_build(o, _dp(P), _dp(Cv), len(P))
        g.map.build(P, Cv)
        for step, (P2, C2) in enumerate(updates):
            oracle_lib.orc_map_update(o, _dp(P2), _dp(C2), len(P2))
            g.map.update(P2, C2)
            rounds = g.last_merge_rounds()
            vo, no, info, _, _ = export_oracle_map(oracle_lib, o)
            vg, ng = g.map.export()
            problems = compare_maps(vo, no, vg, ng, exact=True)
            assert not problems, f"step {step}: " + "; ".join(problems[:8])
            if step == 0:
                assert sum(1 for i in range(no) if vo[i].merged) > 100
                if merge_mode == 0:
                    assert rounds >= 3, rounds
    finally:
        oracle_lib.orc_destroy(o)


def test_map_eviction_bit_exact(lio_mod, oracle_lib):
    """LRU eviction (VoxelMap::update's cache splice / pop_back,
    voxel_map.cpp:232-256) with a map capacity far below the voxels the
    batches create: evictions in most batches, batches whose evicted voxels
    are touched again later in the same batch (the reference re-creates them;
    the batch is split), LRU-queue compaction and hash rehash.  The whole map,
    LRU order included, must equal the oracle's after every batch."""
    rng = np.random.default_rng(41)
    cap = 1500
    cfg = abi.default_config(map_capacity=cap, max_scan_points=12000)
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        P0, C0 = plane_points(rng, n_planes=60, extent=30.0)
        oracle_lib.orc_map_build(o, _dp(P0), _dp(C0), len(P0))
        g.map.build(P0, C0)
        seen = set(map(tuple, np.floor(P0 / cfg.voxel_size).astype(np.int64)))
        Pp, Cp = P0, C0
        for step in range(12):
            P2, C2 = plane_points(rng, n_planes=70, pts_per=(5, 120), extent=30.0 + 4.0 * step)
            Pn, Cn = P2, C2
            if step % 3 == 2:
                # at the end of the batch: voxels of the previous batch (still
                # in the map when the batch starts, evicted by its creations,
                # then touched again) and long-evicted ones
                P2 = np.vstack([P2, Pp[:300], P0[:150]])
                C2 = np.vstack([C2, Cp[:300], C0[:150]])
            Pp, Cp = Pn, Cn
            seen |= set(map(tuple, np.floor(P2 / cfg.voxel_size).astype(np.int64)))
            oracle_lib.orc_map_update(o, _dp(P2), _dp(C2), len(P2))
            g.map.update(P2, C2)
            vo, no, info, _, _ = export_oracle_map(oracle_lib, o)
            vg, ng = g.map.export()
            assert no <= cap
            problems = compare_maps(vo, no, vg, ng, exact=True)
            assert not problems, f"step {step}: " + "; ".join(problems[:8])
            order_o = [tuple(vo[i].key) for i in range(no)]
            order_g = [tuple(vg[i].key) for i in range(ng)]
            assert order_o == order_g, f"step {step}: LRU order differs"
        assert len(seen) > 5 * cap  # most voxels were evicted along the way
        assert g.lib.vmp_eviction_splits(g.h) > 0  # the split path ran
    finally:
        oracle_lib.orc_destroy(o)


def test_process_sequence_with_eviction(lio_mod, oracle_lib):
    """LIOBuilder::process on a corridor walk with a small map capacity: the
    map stays at capacity while evicting; per-scan pose, counts and map size
    as the oracle's."""
    import oracle as orc
    seq_g = synth.Sequence(synth.KIND_CORRIDOR, points_per_scan=8000)
    seq_o = synth.Sequence(synth.KIND_CORRIDOR, points_per_scan=8000)
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=16384, map_capacity=2500)
    g = lio_mod.LIOBuilder(cfg)
    o = orc.Oracle(cfg)
    full = 0
    for k in range(40):
        rg = g.process(seq_g.next())
        ro = o.process(seq_o.next())
        assert rg.lio_status == ro.lio_status
        if ro.lio_status != abi.LIO_MAPPING or k < 2:
            continue
        assert (rg.n_down, rg.effect_num, rg.iters, rg.map_size) == (ro.n_down, ro.effect_num, ro.iters, ro.map_size), k
        assert rg.map_size <= 2500
        full += rg.map_size == 2500
        dp = np.max(np.abs(np.array(rg.x.pos[:]) - np.array(ro.x.pos[:])))
        da = rot_angle(rg.x.rot[:], ro.x.rot[:])
        assert dp < 1e-9 and da < 1e-9, (k, dp, da)
    assert full > 10


def test_map_index_matches_oracle(lio_mod, oracle_lib):
    rng = np.random.default_rng(3)
    cfg = abi.default_config()
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        P = rng.uniform(-500, 500, (20000, 3))
        P[:100] = np.round(P[:100] * 2) / 2  # exact voxel boundaries
        kg = g.map.index(P)
        ko = np.zeros_like(kg)
        oracle_lib.orc_map_index(o, _dp(P), len(P), ko.ctypes.data_as(C.POINTER(C.c_int64)))
        assert np.array_equal(kg, ko)
    finally:
        oracle_lib.orc_destroy(o)


def _seeded_state(rng):
    x = abi.vmp_state()
    ang = rng.normal(0, 0.3, 3)
    th = np.linalg.norm(ang)
    k = ang / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
    for i in range(9):
        x.rot[i] = R.reshape(9)[i]
        x.rot_ext[i] = 1.0 if i in (0, 4, 8) else 0.0
    for i in range(3):
        x.pos[i] = rng.normal(0, 0.5)
        x.vel[i] = rng.normal(0, 0.3)
        x.bg[i] = rng.normal(0, 0.01)
        x.ba[i] = rng.normal(0, 0.05)
    x.g[0], x.g[1], x.g[2] = 0.0, 0.0, -9.81
    A = rng.normal(0, 0.01, (23, 23))
    P = A @ A.T + np.eye(23) * 1e-4
    return x, P


def test_residual_reduce_matches_oracle(lio_mod, oracle_lib):
    rng = np.random.default_rng(5)
    cfg = abi.default_config(map_capacity=200000, max_scan_points=60000)
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        P, Cv = plane_points(rng, n_planes=200, noise=0.005, iso_frac=0.0)
        oracle_lib.orc_map_build(o, _dp(P), _dp(Cv), len(P))
        g.map.build(P, Cv)
        x, Pc = _seeded_state(rng)
        # LiDAR points near the map: world points pulled back through the pose
        R = np.array(x.rot[:]).reshape(3, 3)
        t = np.array(x.pos[:])
        for rep in range(3):
            sel = rng.choice(len(P), 20000)
            pw = P[sel] + rng.normal(0, 0.02, (20000, 3))
            pl = (pw - t) @ R
            pl = pl.astype(np.float32).astype(np.float64)
            cov_l = np.zeros((20000, 9))
            pl_fix = np.zeros_like(pl)
            oracle_lib.orc_calc_body_cov(_dp(pl), 20000, 0.04, 0.1, _dp(pl_fix), _dp(cov_l))
            Hg, bg, eg = g.residual_reduce(x, Pc, pl_fix, cov_l)
            Ho = np.zeros(144)
            bo = np.zeros(12)
            eo = C.c_int()
            vo = np.zeros(20000, dtype=np.uint8)
            oracle_lib.orc_residual_reduce(o, C.byref(x), _dp(Pc), _dp(pl_fix), _dp(cov_l), 20000, _dp(Ho), _dp(bo),
                                           C.byref(eo), vo.ctypes.data_as(C.POINTER(C.c_ubyte)))
            vg = g.residual_valid(20000)
            assert eg == eo.value
            assert np.array_equal(vg, vo), f"match sets differ at {np.flatnonzero(vg != vo)[:10]}"
            scale = np.max(np.abs(Ho))
            assert np.max(np.abs(Hg.reshape(144) - Ho)) <= 1e-9 * scale
            assert np.max(np.abs(bg - bo)) <= 1e-9 * max(1.0, np.max(np.abs(bo)))
    finally:
        oracle_lib.orc_destroy(o)


def test_ieskf_predict_matches_oracle(lio_mod, oracle_lib):
    """20 single IESKF::predict steps (ieskf.cpp:101-123) through
    vmp_ieskf_predict.  The step's SO3 exp calls sin / cos, whose CUDA and
    glibc results may differ in the last bit, so state and covariance are
    compared within 1e-13 (absolute for the state, relative for P), not bit
    for bit."""
    rng = np.random.default_rng(9)
    cfg = abi.default_config()
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        x, P = _seeded_state(rng)
        P = np.ascontiguousarray(P)
        g.kf.set(x, P)
        oracle_lib.orc_set_state(o, C.byref(x), _dp(P))
        Q = np.diag([0.01] * 6 + [1e-4] * 6)
        for k in range(20):
            acc = rng.normal(0, 0.3, 3) + np.array([0, 0, 9.81])
            gyro = rng.normal(0, 0.2, 3)
            dt = 0.005
            g.kf.predict(acc, gyro, dt, Q)
            oracle_lib.orc_ieskf_predict(o, _dp(acc), _dp(gyro), dt, _dp(np.ascontiguousarray(Q.reshape(144))))
        xg, Pg = g.kf.get()
        xo = abi.vmp_state()
        Po = np.zeros(529)
        oracle_lib.orc_get_state(o, C.byref(xo), _dp(Po))
        for f in ("pos", "rot", "vel", "bg", "ba", "g"):
            a = np.array(getattr(xg, f)[:])
            b = np.array(getattr(xo, f)[:])
            assert np.allclose(a, b, rtol=0, atol=1e-13), f
        assert np.max(np.abs(Pg.reshape(529) - Po)) <= 1e-13 * np.max(np.abs(Po))
    finally:
        oracle_lib.orc_destroy(o)


def test_process_sequence_room(lio_mod, oracle_lib):
    """LIOBuilder::process over a seeded room sequence: identical downsample
    sizes, valid-residual counts, iteration counts and map sizes; pose within
    1e-6 m / 1e-6 rad (the specified bar) -- and, to catch a slow divergence
    of the filter recursion long before it reaches that bar, pose within 1e-9
    and covariance within 1e-8 relative over 40 scans."""
    import oracle as orc
    seq_g = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    seq_o = synth.Sequence(synth.KIND_ROOM, points_per_scan=8000)
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=16384)
    g = lio_mod.LIOBuilder(cfg)
    o = orc.Oracle(cfg)
    for k in range(40):
        pg = seq_g.next()
        po = seq_o.next()
        rg = g.process(pg)
        ro = o.process(po)
        assert rg.lio_status == ro.lio_status
        if ro.lio_status != abi.LIO_MAPPING or k < 2:
            continue
        assert rg.n_down == ro.n_down, k
        assert rg.effect_num == ro.effect_num, k
        assert rg.iters == ro.iters, k
        assert rg.map_size == ro.map_size, k
        dp = np.max(np.abs(np.array(rg.x.pos[:]) - np.array(ro.x.pos[:])))
        da = rot_angle(rg.x.rot[:], ro.x.rot[:])
        assert dp < 1e-6 and da < 1e-6, (k, dp, da)
        assert dp < 1e-9 and da < 1e-9, (k, dp, da)
        Pg, Po = np.array(rg.P[:]), np.array(ro.P[:])
        assert np.max(np.abs(Pg - Po)) <= 1e-8 * np.max(np.abs(Po)), k


@pytest.mark.parametrize("evicting", [False, True])
def test_graph_and_direct_launches_agree(lio_mod, evicting):
    """The steady-state scan as captured graphs and as direct launches: the
    same kernels with the same grids, so the same bits -- every result, and
    the map at the end.  Urban scans (several size classes captured) with
    room to grow; corridor scans at a 2500-voxel capacity, where every scan's
    map update may evict and only the scan front runs as a graph."""
    from voxelmapplus_fastlio2_gb300 import abi as A
    out = []
    for graphs in (1, 0):
        if evicting:
            seq = synth.Sequence(synth.KIND_CORRIDOR, points_per_scan=8000)
            cfg = A.default_config(scan_resolution=0.2, max_scan_points=16384, map_capacity=2500)
        else:
            seq = synth.Sequence(synth.KIND_URBAN, points_per_scan=30000)
            cfg = A.default_config(scan_resolution=0.1, map_capacity=300000, max_scan_points=40000, ieskf_max_iter=4)
        g = lio_mod.LIOBuilder(cfg)
        g.lib.vmp_set_graphs(g.h, graphs)
        res = []
        for k in range(30 if evicting else 12):
            r = g.process(seq.next())
            res.append((r.lio_status, r.iters, r.effect_num, r.n_down, r.map_size, bytes(r.x), bytes(r.P)))
        v, n = g.map.export()
        out.append((res, C.string_at(v, n * C.sizeof(A.vmp_voxel))))
        g.close()
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]


@pytest.mark.parametrize("graphs", [1, 0])
def test_shuffled_scans_give_the_same_results(lio_mod, graphs):
    """The points of every scan in a random order instead of time order.  The
    time sort's passes then run in full (on time-ordered scans they return at
    once: the stable sort is the identity), and since the point times are
    distinct they give back the time order: every result and the final map
    equal those of the time-ordered scans, bit for bit."""
    from voxelmapplus_fastlio2_gb300 import abi as A
    seq = synth.Sequence(synth.KIND_URBAN, points_per_scan=30000)
    cfg = A.default_config(scan_resolution=0.1, map_capacity=300000, max_scan_points=40000, ieskf_max_iter=4)
    pkgs = [seq.next() for _ in range(10)]
    rng = np.random.default_rng(0x5EED)
    shuffled = []
    for p in pkgs:
        pts = p.points_np()
        assert np.all(np.diff(pts[:, 3]) > 0)  # generated in time order, distinct times
        perm = rng.permutation(p.n)
        arr = (A.vmp_point * p.n).from_buffer_copy(np.ascontiguousarray(pts[perm], dtype=np.float32).tobytes())
        shuffled.append(synth.Package(arr, p.n, p.t_start, p.t_end, p.imus, p.n_imu))
    out = []
    for run in (pkgs, shuffled):
        g = lio_mod.LIOBuilder(cfg)
        g.lib.vmp_set_graphs(g.h, graphs)
        res = []
        for q in run:
            r = g.process(q)
            res.append((r.lio_status, r.iters, r.effect_num, r.n_down, r.map_size, bytes(r.x), bytes(r.P)))
        v, n = g.map.export()
        out.append((res, C.string_at(v, n * C.sizeof(A.vmp_voxel))))
        g.close()
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]


def test_undistort_and_predict_chain_match_oracle(lio_mod, oracle_lib):
    """undistortCloud after IMU init + map init: the time-sorted compensated
    cloud and the filter state / covariance at the scan end."""
    import oracle as orc
    seq_g = synth.Sequence(synth.KIND_ROOM, points_per_scan=6000)
    seq_o = synth.Sequence(synth.KIND_ROOM, points_per_scan=6000)
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=8192)
    g = lio_mod.LIOBuilder(cfg)
    o = orc.Oracle(cfg)
    for _ in range(2):  # IMU_INIT, MAP_INIT
        g.process(seq_g.next())
        o.process(seq_o.next())
    for _ in range(3):
        pg, po = seq_g.next(), seq_o.next()
        cg = g.undistort(pg)
        out = (abi.vmp_point * po.n)()
        scan = po.scan()
        oracle_lib.orc_undistort(o.h, C.byref(scan), po.imus, po.n_imu, out)
        co = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), shape=(po.n, 4))
        assert np.array_equal(cg[:, 3], co[:, 3])  # same time order
        same = np.mean(np.all(cg.view(np.uint32) == co.view(np.uint32), axis=1))
        assert same > 0.999 and np.max(np.abs(cg - co)) < 1e-5, (same, np.max(np.abs(cg - co)))
        xg, Pg = g.kf.get()
        xo = abi.vmp_state()
        Po = np.zeros(529)
        oracle_lib.orc_get_state(o.h, C.byref(xo), _dp(Po))
        for fld in ("pos", "rot", "vel"):
            assert np.allclose(np.array(getattr(xg, fld)[:]), np.array(getattr(xo, fld)[:]), rtol=0, atol=1e-12), fld
        assert np.max(np.abs(Pg.reshape(529) - Po)) <= 1e-12 * np.max(np.abs(Po))
