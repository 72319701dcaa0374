"""Batched plane fitting (vmp_fit_planes): the oracle's per-voxel fit
(VoxelGrid::addPoint + updatePlane, voxel_map.cpp:29-40, 97-136) against an
independent numpy/LAPACK restatement, and the three GPU arithmetic modes
against the oracle."""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, fit


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def oracle_fit(lib, xyz, cov, off, upt=10, plane_thresh=0.01, threads=4):
    out = np.zeros(len(off) - 1, dtype=abi.fit_rec_dtype())
    lib.orc_fit_planes(_ptr(xyz, C.c_float), _ptr(cov, C.c_float), _ptr(off, C.c_longlong), len(off) - 1,
                       xyz.shape[1], upt, plane_thresh, out.ctypes.data_as(C.POINTER(abi.vmp_fit_rec)), threads)
    return out


def _numpy_fit(p, S, plane_thresh):
    """updatePlane in numpy: dense J cov J^T per point, LAPACK eigh."""
    n = len(p)
    mean = p.mean(axis=0)
    C_ = p.T @ p / n - np.outer(mean, mean)
    ev, E = np.linalg.eigh(C_)
    res = {"mean": mean, "C": C_, "evals": ev, "plane": ev[0] <= plane_thresh, "e0": E[:, 0]}
    if not res["plane"]:
        return res
    pn = E[:, 0]
    P = np.zeros((6, 6))
    for i in range(n):
        F = np.zeros((3, 3))
        for m in (1, 2):
            vm = E[:, m]
            F[m] = (p[i] - mean) / (n * (ev[0] - ev[m])) @ (np.outer(vm, pn) + np.outer(pn, vm))
        J = np.vstack([E @ F, np.eye(3) / n])
        P += J @ S[i] @ J.T
    res["P"] = P
    res["norm"] = -pn if -mean @ pn < 0 else pn
    return res


def test_fit_abi_layout():
    assert C.sizeof(abi.vmp_fit_rec) == 296 == abi.fit_rec_dtype().itemsize
    assert C.sizeof(abi.vmp_fit_params) == 16


def test_synth_voxels_shape():
    xyz, cov, off = fit.synth_voxels(3000, seed=3)
    n = np.diff(off)
    assert off[0] == 0 and off[-1] == xyz.shape[1] == cov.shape[1]
    assert n.min() >= 5 and n.max() <= 4000
    assert 30 < np.median(n) < 50
    assert xyz.dtype == np.float32 and cov.dtype == np.float32
    again = fit.synth_voxels(3000, seed=3)
    assert np.array_equal(again[0], xyz) and np.array_equal(again[2], off)


def test_oracle_fit_matches_numpy(oracle_lib):
    xyz, cov, off = fit.synth_voxels(400, seed=11, n_max=400)
    ref = oracle_fit(oracle_lib, xyz, cov, off)
    iu = [(i, j) for i in range(6) for j in range(i, 6)]
    planes = 0
    for v in range(len(off) - 1):
        a, b = off[v], off[v + 1]
        p = xyz[:, a:b].T.astype(np.float64)
        c6 = cov[:, a:b].T.astype(np.float64)
        S = np.stack([c6[:, [0, 1, 2]], c6[:, [1, 3, 4]], c6[:, [2, 4, 5]]], axis=1)
        r = _numpy_fit(p, S, 0.01)
        o = ref[v]
        assert o["n"] == b - a
        assert np.allclose(o["mean"], r["mean"], rtol=0, atol=1e-10)
        if b - a < 10:  # below update_point_thresh: updatePlane returns early
            assert o["flags"] == 0 and not np.any(o["cov"]) and not np.any(o["plane_cov"])
            continue
        lmax = abs(r["evals"][-1])
        Co = np.array([[o["cov"][0], o["cov"][1], o["cov"][2]], [o["cov"][1], o["cov"][3], o["cov"][4]],
                       [o["cov"][2], o["cov"][4], o["cov"][5]]])
        assert np.max(np.abs(Co - r["C"])) < 1e-8 * lmax
        assert np.max(np.abs(o["evals"] - r["evals"])) < 1e-8 * lmax
        assert bool(o["flags"] & abi.VMP_FIT_PLANE) == bool(r["plane"])
        if not r["plane"]:
            assert not np.any(o["norm"]) and not np.any(o["plane_cov"])
            continue
        planes += 1
        assert abs(abs(o["norm"] @ r["norm"]) - 1.0) < 1e-9
        assert o["norm"] @ r["norm"] > 0  # same sign after the flip rule
        # the off-diagonal block follows the sign of the unflipped normal
        un_o = o["norm"] * (-1.0 if o["flags"] & abi.VMP_FIT_FLIPPED else 1.0)
        P = r["P"].copy()
        if un_o @ r["e0"] < 0:
            P[:3, 3:] *= -1
            P[3:, :3] *= -1
        Pu = np.array([P[i, j] for i, j in iu])
        assert np.max(np.abs(o["plane_cov"] - Pu)) < 1e-6 * np.max(np.abs(Pu))
    assert planes > 300


def test_compare_identity(oracle_lib):
    xyz, cov, off = fit.synth_voxels(500, seed=5)
    ref = oracle_fit(oracle_lib, xyz, cov, off)
    m = fit.compare(ref, ref)
    assert m["fitted_differ"] == 0 and m["plane_differ"] == 0
    assert m["cov_rel"]["max"] == 0.0 and m["normal_rad"]["max"] == 0.0 and m["plane_cov_rel"]["max"] == 0.0
    assert m["planes"] > 0.8 * m["voxels"]


# ---------------------------------------------------------------- GPU
def _edge_case_set():
    """Regular voxels plus an empty voxel, one below the fitting threshold,
    a single-point voxel and a 4000-point voxel."""
    xyz, cov, off = fit.synth_voxels(3000, seed=21)
    big = fit.synth_voxels(1, seed=22, median=4000, sigma=0.0, n_min=4000)
    small = fit.synth_voxels(2, seed=23, median=5, sigma=0.0, n_min=1, n_max=7)
    counts = list(np.diff(off)) + [0] + list(np.diff(big[2])) + [7, 1]
    pts = np.concatenate([xyz, big[0], small[0][:, :8]], axis=1)
    cv = np.concatenate([cov, big[1], small[1][:, :8]], axis=1)
    o = np.zeros(len(counts) + 1, dtype=np.int64)
    np.cumsum(counts, out=o[1:])
    assert o[-1] == pts.shape[1]
    return np.ascontiguousarray(pts), np.ascontiguousarray(cv), o


@pytest.mark.gpu
def test_fit_fp64_matches_oracle(oracle_lib):
    xyz, cov, off = _edge_case_set()
    ref = oracle_fit(oracle_lib, xyz, cov, off)
    rec = fit.fit_planes(xyz, cov, off, mode=fit.FP64)
    assert np.array_equal(rec["n"], ref["n"])
    assert np.array_equal(rec["flags"], ref["flags"])  # fitted, plane and flip decisions identical
    m = fit.compare(rec, ref)
    print("fp64", m)
    # C = ppt / n - mean mean^T cancels ~1e4 m^2 against ~1e-2 m^2 at 100 m
    # from the origin, so FP64 sums taken in another order differ by
    # ~1e-12 m^2 absolute: ~1e-10 of C, ~1e-8 of the 1 cm^2 smallest
    # eigenvalue, more where a voxel's spread or eigenvalue gap is small
    assert m["mean_abs_m"]["max"] < 1e-11
    assert m["cov_rel"]["p50"] < 1e-9 and m["cov_rel"]["max"] < 1e-7
    assert m["evals_rel"]["max"] < 1e-7
    assert m["eval0_rel"]["p50"] < 1e-7
    assert m["normal_rad"]["p50"] < 1e-9 and m["normal_rad"]["max"] < 1e-6
    assert m["plane_cov_rel"]["p50"] < 1e-8 and m["plane_cov_rel"]["max"] < 1e-5
    # the appended voxels: empty, 4000 points, 7 points, 1 point
    V = len(off) - 1
    empty, big, seven, one = V - 4, V - 3, V - 2, V - 1
    assert rec[big]["n"] == 4000 and rec[big]["flags"] & abi.VMP_FIT_FITTED
    for v in (empty, seven, one):  # not fitted: mean and n only
        assert rec[v]["flags"] == 0 and not np.any(rec[v]["evals"]) and not np.any(rec[v]["plane_cov"])
    assert rec[empty]["n"] == 0 and not np.any(rec[empty]["mean"])
    assert rec[seven]["n"] == 7 and rec[one]["n"] == 1


@pytest.mark.gpu
def test_fit_fp32_modes_against_oracle(oracle_lib):
    xyz, cov, off = fit.synth_voxels(20000, seed=31)
    ref = oracle_fit(oracle_lib, xyz, cov, off)
    mc = fit.compare(fit.fit_planes(xyz, cov, off, mode=fit.FP32C), ref)
    mp = fit.compare(fit.fit_planes(xyz, cov, off, mode=fit.FP32), ref)
    print("fp32c", mc)
    print("fp32", mp)
    # compensated FP32: plane decisions and normals as FP64 up to float rounding
    assert mc["fitted_differ"] == 0
    assert mc["plane_differ"] <= 0.001 * mc["fitted"]
    assert mc["normal_rad"]["p99"] < 1e-5
    assert mc["eval0_rel"]["p50"] < 1e-3
    assert mc["plane_cov_rel"]["p99"] < 1e-3
    # plain FP32 on world coordinates loses the small eigenvalue to cancellation
    assert mp["eval0_rel"]["p50"] > 10 * mc["eval0_rel"]["p50"]


@pytest.mark.gpu
def test_fit_device_entry_matches_host_entry():
    import torch
    xyz, cov, off = fit.synth_voxels(5000, seed=41)
    host = fit.fit_planes(xyz, cov, off, mode=fit.FP32C)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_cov = torch.from_numpy(cov).cuda()
    d_off = torch.from_numpy(off).cuda()
    d_out = torch.zeros(len(off) - 1, abi.fit_rec_dtype().itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    fit.fit_planes_device(d_xyz.data_ptr(), d_cov.data_ptr(), d_off.data_ptr(), len(off) - 1, xyz.shape[1],
                          d_out.data_ptr(), mode=fit.FP32C, cuda_stream=stream)
    torch.cuda.synchronize()
    dev = d_out.cpu().numpy().view(abi.fit_rec_dtype()).reshape(-1)
    assert dev.tobytes() == host.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [fit.FP64, fit.FP32, fit.FP32C])
def test_fit_record_depends_only_on_its_voxel(mode):
    """A voxel's record is the same whatever voxels share its warp: the
    batch shifted by 13 voxels (other warp groups) gives the same bytes."""
    xyz, cov, off = fit.synth_voxels(3000, seed=43)
    full = fit.fit_planes(xyz, cov, off, mode=mode)
    s = 13
    sub_off = np.ascontiguousarray(off[s:] - off[s])
    sub_xyz = np.ascontiguousarray(xyz[:, off[s]:])
    sub_cov = np.ascontiguousarray(cov[:, off[s]:])
    part = fit.fit_planes(sub_xyz, sub_cov, sub_off, mode=mode)
    assert part.tobytes() == full[s:].tobytes()
