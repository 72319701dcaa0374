"""Edge cases of the entry points: empty and oversized inputs, a scan of
exactly max_scan_points, voxels hit by thousands of (partly identical)
points, voxel indices outside the packed key range, an empty residual
batch."""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth
from voxelmapplus_fastlio2_gb300._lib import VmpError
from tests.helpers import compare_maps, export_oracle_map


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.fixture(scope="module")
def lio_mod():
    from voxelmapplus_fastlio2_gb300 import lio
    return lio


def _cov(rng, n):
    A = rng.normal(0, 0.02, (n, 3, 3))
    return (A @ A.transpose(0, 2, 1) + np.eye(3) * 1e-4).reshape(n, 9)


@pytest.mark.gpu
def test_process_rejects_bad_sizes(lio_mod):
    cfg = abi.default_config(max_scan_points=4096, max_imu_per_scan=64)
    g = lio_mod.LIOBuilder(cfg)
    seq = synth.Sequence(synth.KIND_ROOM, points_per_scan=3000)
    p = seq.next()
    codes = []
    for pk in (synth.Package(p.points, 0, p.t_start, p.t_end, p.imus, p.n_imu),
               synth.Package(p.points, p.n, p.t_start, p.t_end, p.imus, 0),
               synth.Package(p.points, 5000, p.t_start, p.t_end, p.imus, p.n_imu),
               synth.Package(p.points, p.n, p.t_start, p.t_end, p.imus, 65)):
        with pytest.raises(VmpError) as e:
            g.process(pk)
        codes.append(e.value.code)
    assert codes == [abi.VMP_ERR_INVALID_ARG, abi.VMP_ERR_INVALID_ARG, abi.VMP_ERR_CAPACITY, abi.VMP_ERR_CAPACITY]
    # the stream is unharmed: the same package is processed afterwards
    assert g.process(p).lio_status in (abi.IMU_INIT, abi.MAP_INIT)
    g.close()


@pytest.mark.gpu
def test_scan_of_exactly_max_points(lio_mod, oracle_lib):
    import oracle
    seq_g = synth.Sequence(synth.KIND_ROOM, points_per_scan=6000)
    seq_o = synth.Sequence(synth.KIND_ROOM, points_per_scan=6000)
    pk = [seq_g.next() for _ in range(8)]
    cfg = abi.default_config(scan_resolution=0.2, max_scan_points=max(p.n for p in pk))
    g = lio_mod.LIOBuilder(cfg)
    o = oracle.Oracle(cfg)
    for p, q in zip(pk, (seq_o.next() for _ in range(8))):
        rg, ro = g.process(p), o.process(q)
        assert rg.lio_status == ro.lio_status and rg.n_down == ro.n_down and rg.map_size == ro.map_size
    assert max(p.n for p in pk) == cfg.max_scan_points
    g.close()


@pytest.mark.gpu
def test_crowded_voxels_bit_exact(lio_mod, oracle_lib):
    """Thousands of points in a handful of voxels, many of them identical:
    long point chains (refits, freezing at max_point_thresh, merge() calls of
    frozen planes) against the oracle, bit for bit."""
    rng = np.random.default_rng(4)
    cfg = abi.default_config(map_capacity=1000, max_scan_points=20000)
    g = lio_mod.LIOBuilder(cfg)
    o = oracle_lib.orc_create(C.byref(cfg))
    try:
        base = np.array([[0.1, 0.1, 0.0], [0.6, 0.1, 0.0], [0.1, 0.6, 0.0], [3.2, 3.3, 1.1]])
        pts = []
        for c in base:
            q = c + np.c_[rng.uniform(0, 0.35, (2500, 2)), rng.normal(0, 0.003, 2500)]
            q[::7] = q[0]  # exact duplicates
            pts.append(q)
        P = np.concatenate(pts).astype(np.float32).astype(np.float64)
        P = P[rng.permutation(len(P))]
        Cv = _cov(rng, len(P))
        oracle_lib.orc_map_build(o, _dp(P[:4000]), _dp(Cv[:4000]), 4000)
        g.map.build(P[:4000], Cv[:4000])
        oracle_lib.orc_map_update(o, _dp(P[4000:]), _dp(Cv[4000:]), len(P) - 4000)
        g.map.update(P[4000:], Cv[4000:])
        vo, no, _, _, _ = export_oracle_map(oracle_lib, o)
        vg, ng = g.map.export()
        problems = compare_maps(vo, no, vg, ng, exact=True)
        assert not problems, "; ".join(problems[:8])
        assert ng <= 12
    finally:
        oracle_lib.orc_destroy(o)
        g.close()


@pytest.mark.gpu
def test_voxel_index_outside_key_range(lio_mod):
    """Points more than 2^20 voxels from the origin: the batch reports
    VMP_ERR_KEY_RANGE (those points are not inserted) and the stream keeps
    working."""
    rng = np.random.default_rng(9)
    cfg = abi.default_config(map_capacity=10000, max_scan_points=4096)
    g = lio_mod.LIOBuilder(cfg)
    P = rng.uniform(-5, 5, (1000, 3))
    P[10] = [1.0e6, 0.0, 0.0]
    P[20] = [0.0, -6.0e5, 0.0]
    with pytest.raises(VmpError) as e:
        g.map.build(P, _cov(rng, 1000))
    assert e.value.code == abi.VMP_ERR_KEY_RANGE
    g.map.update(rng.uniform(-5, 5, (500, 3)), _cov(rng, 500))
    info = g.map.info()
    assert 0 < info.size <= 10000
    g.close()


@pytest.mark.gpu
def test_residual_reduce_empty(lio_mod):
    cfg = abi.default_config(max_scan_points=1024)
    g = lio_mod.LIOBuilder(cfg)
    x = abi.vmp_state()
    for k in range(3):
        x.rot[4 * k] = 1.0
        x.rot_ext[4 * k] = 1.0
    H, b, eff = g.residual_reduce(x, np.eye(23) * 1e-3, np.zeros((0, 3)), np.zeros((0, 9)))
    assert eff == 0 and not np.any(H) and not np.any(b)
    g.close()


@pytest.mark.gpu
def test_shared_divisor_division_is_exact():
    """The kernels divide by a shared divisor through its reciprocal and
    Markstein's correction; it must equal the FP64 division bit for bit --
    random operands over wide exponent ranges, the covariance-term operands
    (differences of nearby coordinates over n (l0 - lm)), signed zeros,
    exact quotients and divisors at the range limits."""
    from voxelmapplus_fastlio2_gb300._lib import load
    rng = np.random.default_rng(17)
    n = 1 << 20
    a = rng.uniform(1, 2, n) * 2.0 ** rng.integers(-60, 60, n) * rng.choice([-1, 1], n)
    b = rng.uniform(1, 2, n) * 2.0 ** rng.integers(-60, 60, n) * rng.choice([-1, 1], n)
    m = n // 4  # the plane-covariance operands
    a[:m] = rng.normal(0, 0.2, m)
    b[:m] = rng.integers(10, 400, m) * -rng.uniform(1e-4, 2e-2, m)
    a[m:m + 8] = [0.0, -0.0, 0.0, -0.0, 3.0, -7.5, 1e-300, 6.0]
    b[m:m + 8] = [2.0, 2.0, -2.0, -2.0, 1.5, 2.5, 1e-289, 1e291]
    a[m + 8:m + 1000] = b[m + 8:m + 1000] * rng.integers(-50, 50, 992)  # exact quotients
    by_recip = np.zeros(n)
    by_div = np.zeros(n)
    dp = lambda x: C.c_void_p(x.ctypes.data)
    rc = load().vmp_test_division(dp(a), dp(b), n, dp(by_recip), dp(by_div))
    assert rc == 0
    assert np.array_equal(by_recip.view(np.uint64), by_div.view(np.uint64))


@pytest.mark.gpu
def test_body_cov_bit_exact(oracle_lib):
    """calcBodyCov on the device (normalisations through one reciprocal per
    vector with Markstein's correction, the products with the zeros of
    direction_hat and dvar left out) against the oracle's dense form
    (commons.cpp:18-45 as written), bit for bit over 1 M points, including
    points with z == 0 (fixed to 0.001 in place, as the reference) and
    exact zeros of both signs in x and y."""
    from voxelmapplus_fastlio2_gb300._lib import load
    rng = np.random.default_rng(23)
    n = 1_000_000
    pts = rng.normal(0, 8, (n, 3))
    pts[::97, 2] = 0.0
    pts[::89] = pts[::89].astype(np.float32).astype(np.float64)
    pts[::53, 0] = 0.0
    pts[::59, 1] = -0.0
    pts[::61, 2] = -0.0
    gp, gc = np.zeros((n, 3)), np.zeros((n, 9))
    op, oc = np.zeros((n, 3)), np.zeros((n, 9))
    dp = lambda x: C.c_void_p(x.ctypes.data)
    assert load().vmp_test_body_cov(dp(pts), n, 0.04, 0.1, dp(gp), dp(gc)) == 0
    oracle_lib.orc_calc_body_cov(_dp(pts), n, 0.04, 0.1, _dp(op), _dp(oc))
    assert np.array_equal(gp, op)
    assert np.array_equal(gc.view(np.uint64), oc.view(np.uint64))


@pytest.mark.gpu
def test_hat_sandwich_matches_dense_form(oracle_lib):
    """[p]x P_rr [p]x^T on the device (the products with [p]x's zero diagonal
    left out) against the oracle's dense form (lio_builder.cpp:199-202 as
    written) over 1 M inputs with exact zeros of both signs: equal values
    everywhere, bits different only where the value is zero."""
    from voxelmapplus_fastlio2_gb300._lib import load
    rng = np.random.default_rng(29)
    n = 1_000_000
    pts = rng.normal(0, 10, (n, 3))
    for k, step in enumerate((7, 11, 13)):
        pts[::step, k] = 0.0 if k % 2 else -0.0
    A = rng.normal(0, 0.02, (n, 3, 3))
    M = (A @ A.transpose(0, 2, 1) + np.eye(3) * 1e-4).reshape(n, 9)
    M[::17, 1] = M[::17, 3] = 0.0
    gout, oout = np.zeros((n, 9)), np.zeros((n, 9))
    dp = lambda x: C.c_void_p(x.ctypes.data)
    assert load().vmp_test_hat_sandwich(dp(pts), dp(M), n, dp(gout)) == 0
    oracle_lib.orc_hat_sandwich(_dp(pts), _dp(M), n, _dp(oout))
    assert np.array_equal(gout, oout)
    bits = gout.view(np.uint64) != oout.view(np.uint64)
    assert np.all(oout[bits] == 0.0)


@pytest.mark.gpu
def test_grid_barrier_wait_is_bounded():
    """The merge resolution's grid barrier gives up instead of hanging: with
    one CTA that never arrives the other's wait runs out (a status the host
    reads, no fault), the context stays usable, and with both CTAs arriving
    nothing times out."""
    from voxelmapplus_fastlio2_gb300._lib import load
    lib = load()
    to, ms = C.c_int(-1), C.c_double(0.0)
    assert lib.vmp_test_barrier_timeout(1, 100_000, C.byref(to), C.byref(ms)) == 0
    assert to.value == 1
    assert ms.value < 2000.0  # 1e5 polls with a 64 ns sleep each: milliseconds, not a hang
    to.value = -1
    assert lib.vmp_test_barrier_timeout(0, 100_000_000, C.byref(to), C.byref(ms)) == 0
    assert to.value == 0
    assert ms.value < 100.0
