"""Plane voxels of a key cloud for the STD loop-closure descriptor
(STDManager::buildVoxels, std_matcher/src/std_manager/descriptor.cpp:70-122):
the oracle against numpy, the device (vmp_std_plane_voxels) against the
oracle."""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi
from tests.helpers import plane_points


def key_cloud(seed, n_planes=60, stride=8):
    rng = np.random.default_rng(seed)
    P, _ = plane_points(rng, n_planes=n_planes, pts_per=(5, 400), extent=15.0, noise=0.01, iso_frac=0.15)
    pts = np.zeros((len(P), stride), dtype=np.float32)
    pts[:, :3] = P
    if stride > 4:
        pts[:, 4] = rng.uniform(0, 255, len(P))  # intensity of pcl::PointXYZI (after x y z and padding)
    return pts


def oracle_std(lib, pts, voxel_size=1.0, min_point=10, thresh=0.01):
    n, stride = pts.shape
    out = np.zeros(max(1, n), dtype=abi.std_voxel_dtype())
    m = lib.orc_std_plane_voxels(pts.ctypes.data_as(C.POINTER(C.c_float)), stride, n, voxel_size, min_point, thresh,
                                 out.ctypes.data_as(C.POINTER(abi.vmp_std_voxel)), n)
    return out[:m]


def by_key(rec):
    order = np.lexsort((rec["key"][:, 0], rec["key"][:, 1], rec["key"][:, 2]))
    return rec[order]


def test_std_voxel_layout():
    assert C.sizeof(abi.vmp_std_voxel) == 256 == abi.std_voxel_dtype().itemsize


def test_oracle_std_voxels_match_numpy(oracle_lib):
    pts = key_cloud(1, n_planes=25)
    ref = oracle_std(oracle_lib, pts, voxel_size=1.0, min_point=10)
    keys = np.floor(pts[:, :3].astype(np.float64) / 1.0).astype(np.int64)
    groups = {}
    for i, k in enumerate(map(tuple, keys)):
        groups.setdefault(k, []).append(i)
    assert len(ref) == len(groups)
    planes = 0
    for r in ref:
        idx = groups[tuple(r["key"])]
        p = pts[idx, :3].astype(np.float64)
        s = np.zeros(3)
        for q in p:  # cloud order, as the reference accumulates
            s = s + q
        assert r["n"] == len(idx) and np.array_equal(r["sum"], s)
        if len(idx) <= 10:
            assert r["valid"] == 0 and not r["is_plane"]
            continue
        mean = s / len(idx)
        ppt = r["ppt"].reshape(3, 3)
        C_ = ppt / len(idx) - np.outer(mean, mean)
        ev, E = np.linalg.eigh(C_)
        assert np.array_equal(r["mean"], mean)
        assert bool(r["is_plane"]) == bool(ev[0] < 0.01)
        if r["is_plane"]:
            planes += 1
            assert np.max(np.abs(r["lamdas"] - ev)) < 1e-12 * max(1.0, abs(ev[-1]))
            N = r["norms"].reshape(3, 3)
            assert abs(abs(N[:, 0] @ E[:, 0]) - 1.0) < 1e-9
    assert planes > 5


@pytest.mark.gpu
@pytest.mark.parametrize("stride,voxel_size", [(8, 1.0), (4, 0.5), (3, 0.3)])
def test_std_voxels_match_oracle(oracle_lib, stride, voxel_size):
    from voxelmapplus_fastlio2_gb300 import fit
    pts = key_cloud(10 + stride, n_planes=120, stride=stride)
    g = by_key(fit.std_plane_voxels(pts, voxel_size, 10, 0.01))
    o = by_key(oracle_std(oracle_lib, pts, voxel_size, 10, 0.01))
    assert len(g) == len(o) > 50
    for f in ("key", "n", "valid", "is_plane", "sum", "ppt", "mean"):
        assert np.array_equal(g[f], o[f]), f  # the reference's sums in cloud order, bit for bit
    pl = g["is_plane"] == 1
    assert pl.sum() > 10
    scale = np.maximum(np.abs(o["lamdas"][pl]).max(axis=1), 1e-300)
    assert np.max(np.abs(g["lamdas"][pl] - o["lamdas"][pl]).max(axis=1) / scale) < 1e-12
    Ng = g["norms"][pl].reshape(-1, 3, 3)
    No = o["norms"][pl].reshape(-1, 3, 3)
    dots = np.abs(np.einsum("vij,vij->vj", Ng, No))  # columns up to sign
    assert np.max(np.abs(dots[:, 0] - 1.0)) < 1e-9
