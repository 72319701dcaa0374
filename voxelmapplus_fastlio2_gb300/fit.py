"""Batched plane fitting through libvmp: ``VoxelGrid::updatePlane``
(voxel_plus/src/map_builder/voxel_map.cpp:97-136) over all points of many
voxels at once, in the FP64, plain FP32 and compensated FP32 modes of
``vmp_fit_planes``.

Point layout (structure of arrays, float32): ``xyz`` of shape (3, n_pts),
``cov`` of shape (6, n_pts) holding xx xy xz yy yz zz of each point's 3x3
covariance, and ``offsets`` (int64, n_vox + 1): voxel v owns points
offsets[v] .. offsets[v + 1] - 1.  Results are numpy records with the layout of
``vmp_fit_rec`` (``abi.fit_rec_dtype()``).
"""
import ctypes as C

import numpy as np

from . import abi
from ._lib import VmpError, load

FP64, FP32, FP32C = abi.VMP_FIT_FP64, abi.VMP_FIT_FP32, abi.VMP_FIT_FP32C


def params(mode=FP32C, update_point_thresh=10, plane_thresh=0.01):
    return abi.vmp_fit_params(mode, update_point_thresh, plane_thresh)


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def fit_planes(xyz, cov, offsets, mode=FP32C, update_point_thresh=10, plane_thresh=0.01):
    """Host buffers in, records out (vmp_fit_planes)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    cov = np.ascontiguousarray(cov, dtype=np.float32)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    n_vox = len(offsets) - 1
    n_pts = xyz.shape[1]
    if xyz.shape != (3, n_pts) or cov.shape != (6, n_pts):
        raise ValueError("xyz must be (3, n) and cov (6, n)")
    out = np.zeros(max(n_vox, 0), dtype=abi.fit_rec_dtype())
    p = params(mode, update_point_thresh, plane_thresh)
    rc = load().vmp_fit_planes(_ptr(xyz), _ptr(cov), _ptr(offsets), n_vox, n_pts, C.byref(p), _ptr(out))
    if rc != abi.VMP_OK:
        raise VmpError(rc, "vmp_fit_planes")
    return out


def fit_planes_device(xyz_ptr, cov_ptr, offsets_ptr, n_vox, n_pts, out_ptr, mode=FP32C, update_point_thresh=10,
                      plane_thresh=0.01, cuda_stream=0):
    """Device buffers (raw addresses) in and out; only enqueues the work on
    cuda_stream (vmp_fit_planes_device)."""
    p = params(mode, update_point_thresh, plane_thresh)
    rc = load().vmp_fit_planes_device(C.c_void_p(xyz_ptr), C.c_void_p(cov_ptr), C.c_void_p(offsets_ptr), n_vox,
                                      n_pts, C.byref(p), C.c_void_p(out_ptr), C.c_void_p(cuda_stream))
    if rc != abi.VMP_OK:
        raise VmpError(rc, "vmp_fit_planes_device")


def std_plane_voxels(pts, voxel_size=1.0, voxel_min_point=10, voxel_plane_thresh=0.01):
    """STDManager::buildVoxels on the device (vmp_std_plane_voxels): pts is an
    (n, k) float32 array with x y z in the first three columns (k >= 3).
    Returns records of abi.std_voxel_dtype() in packed-key order."""
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    n, stride = pts.shape
    cnt = C.c_int()
    lib = load()
    out = np.zeros(max(1, n), dtype=abi.std_voxel_dtype())
    rc = lib.vmp_std_plane_voxels(_ptr(pts), stride, n, voxel_size, voxel_min_point, voxel_plane_thresh, _ptr(out),
                                  n, C.byref(cnt))
    if rc != abi.VMP_OK:
        raise VmpError(rc, "vmp_std_plane_voxels")
    return out[: cnt.value]


# ---------------------------------------------------------------- workload
def synth_voxels(n_vox, seed=0, median=40.0, sigma=1.0, n_min=5, n_max=4000, nonplanar=0.1, noise=0.01,
                 voxel=0.5, extent=(400, 400, 40), chunk=100_000):
    """Seeded batched-fit workload: n_vox distinct voxels of a 0.5 m grid spread
    over extent voxels (centred on the origin: about +-100 m x +-100 m x +-10 m),
    point counts lognormal (median 40, sigma 1) clipped to [5, 4000].  A planar
    voxel's points lie on a random plane through the voxel centre with normal
    noise of `noise` m; a `nonplanar` fraction are isotropic Gaussian clusters
    (sigma 0.1 m).  Point covariances are 1e-4 I + w w^T, w ~ N(0, 0.01^2 I).
    Returns xyz (3, n) float32, cov (6, n) float32, offsets (n_vox + 1) int64."""
    rng = np.random.default_rng(seed)
    ext = np.array(extent, dtype=np.int64)
    keys = np.empty((0, 3), dtype=np.int64)
    while len(keys) < n_vox:
        k = rng.integers(-ext // 2, ext // 2, size=(int(1.2 * n_vox) + 16, 3), dtype=np.int64)
        keys = np.concatenate([keys, k])
        _, first = np.unique(keys, axis=0, return_index=True)
        keys = keys[np.sort(first)]
    keys = keys[:n_vox]
    counts = np.clip(np.rint(rng.lognormal(np.log(median), sigma, n_vox)), n_min, n_max).astype(np.int64)
    offsets = np.zeros(n_vox + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    n_pts = int(offsets[-1])
    planar = rng.random(n_vox) >= nonplanar
    nrm = rng.normal(size=(n_vox, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    xyz = np.empty((3, n_pts), dtype=np.float32)
    cov = np.empty((6, n_pts), dtype=np.float32)
    for v0 in range(0, n_vox, chunk):
        v1 = min(n_vox, v0 + chunk)
        p0, p1 = int(offsets[v0]), int(offsets[v1])
        vid = np.repeat(np.arange(v0, v1), counts[v0:v1])
        centre = (keys[vid].astype(np.float64) + 0.5) * voxel
        u = centre + (rng.random((p1 - p0, 3)) - 0.5) * voxel
        nv = nrm[vid]
        onplane = u - np.sum((u - centre) * nv, axis=1, keepdims=True) * nv + rng.normal(0.0, noise, (p1 - p0, 1)) * nv
        iso = centre + rng.normal(0.0, 0.1, (p1 - p0, 3))
        q = np.where(planar[vid][:, None], onplane, iso)
        xyz[:, p0:p1] = q.T.astype(np.float32)
        w = rng.normal(0.0, 0.01, (p1 - p0, 3))
        cov[0, p0:p1] = 1e-4 + w[:, 0] * w[:, 0]
        cov[1, p0:p1] = w[:, 0] * w[:, 1]
        cov[2, p0:p1] = w[:, 0] * w[:, 2]
        cov[3, p0:p1] = 1e-4 + w[:, 1] * w[:, 1]
        cov[4, p0:p1] = w[:, 1] * w[:, 2]
        cov[5, p0:p1] = 1e-4 + w[:, 2] * w[:, 2]
    return xyz, cov, offsets


# ---------------------------------------------------------------- errors
_TOP_RIGHT = np.array([e for e, (i, j) in enumerate((i, j) for i in range(6) for j in range(i, 6))
                       if i < 3 <= j])


def _q(x):
    if len(x) == 0:
        return {"p50": 0.0, "p99": 0.0, "max": 0.0}
    return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)), "max": float(np.max(x))}


def compare(rec, ref):
    """Errors of fitted records against reference records (both vmp_fit_rec
    layouts): relative Frobenius error of C, eigenvalue errors relative to the
    largest eigenvalue, relative error of the smallest eigenvalue, normal angle
    (rad), relative error of the 6x6 plane covariance, and the decisions that
    differ.  The plane covariance's off-diagonal block carries the sign of the
    eigensolver's normal before the flip; it is compared after aligning that
    sign (the count of aligned voxels is reported)."""
    fit_g = (rec["flags"] & abi.VMP_FIT_FITTED) != 0
    fit_o = (ref["flags"] & abi.VMP_FIT_FITTED) != 0
    pl_g = (rec["flags"] & abi.VMP_FIT_PLANE) != 0
    pl_o = (ref["flags"] & abi.VMP_FIT_PLANE) != 0
    both_fit = fit_g & fit_o
    both_pl = pl_g & pl_o
    out = {"voxels": int(len(rec)), "fitted": int(both_fit.sum()), "planes": int(both_pl.sum()),
           "fitted_differ": int((fit_g != fit_o).sum()), "plane_differ": int((pl_g != pl_o)[both_fit].sum())}
    mean_err = np.max(np.abs(rec["mean"] - ref["mean"]), axis=1)
    out["mean_abs_m"] = _q(mean_err)
    C_g, C_o = rec["cov"][both_fit], ref["cov"][both_fit]
    w = np.array([1.0, 2.0, 2.0, 1.0, 2.0, 1.0])
    cn = np.sqrt(np.sum(w * (C_g - C_o) ** 2, axis=1)) / np.maximum(np.sqrt(np.sum(w * C_o ** 2, axis=1)), 1e-300)
    out["cov_rel"] = _q(cn)
    e_g, e_o = rec["evals"][both_fit], ref["evals"][both_fit]
    scale = np.maximum(np.max(np.abs(e_o), axis=1), 1e-300)
    out["evals_rel"] = _q(np.max(np.abs(e_g - e_o), axis=1) / scale)
    out["eval0_rel"] = _q(np.abs(e_g[:, 0] - e_o[:, 0]) / np.maximum(np.abs(e_o[:, 0]), 1e-300))
    n_g, n_o = rec["norm"][both_pl], ref["norm"][both_pl]
    cr = np.linalg.norm(np.cross(n_g, n_o), axis=1)
    dt = np.sum(n_g * n_o, axis=1)
    out["normal_rad"] = _q(np.arctan2(cr, np.abs(dt)))
    out["normal_sign_differ"] = int((dt < 0).sum())
    sg = np.where((rec["flags"][both_pl] & abi.VMP_FIT_FLIPPED) != 0, -1.0, 1.0)
    so = np.where((ref["flags"][both_pl] & abi.VMP_FIT_FLIPPED) != 0, -1.0, 1.0)
    align = np.sum((n_g * sg[:, None]) * (n_o * so[:, None]), axis=1) < 0
    P_g = rec["plane_cov"][both_pl].copy()
    P_o = ref["plane_cov"][both_pl]
    P_g[np.ix_(align, _TOP_RIGHT)] *= -1.0
    wp = np.array([1.0 if i == j else 2.0 for i in range(6) for j in range(i, 6)])
    pn = np.sqrt(np.sum(wp * (P_g - P_o) ** 2, axis=1)) / np.maximum(np.sqrt(np.sum(wp * P_o ** 2, axis=1)), 1e-300)
    out["plane_cov_rel"] = _q(pn)
    out["plane_cov_sign_aligned"] = int(align.sum())
    return out
