"""Shared helpers of the parity tests: seeded inputs and oracle/GPU pairs."""
import ctypes as C

import numpy as np

from voxelmapplus_fastlio2_gb300 import abi


def rot_angle(Ra, Rb):
    """Angle of Ra^T Rb, accurate for small angles (atan2 of the skew part
    against the trace, not arccos of the trace)."""
    R = np.asarray(Ra).reshape(3, 3).T @ np.asarray(Rb).reshape(3, 3)
    s = 0.5 * np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    c = (np.trace(R) - 1.0) / 2.0
    return float(np.arctan2(s, c))


def plane_points(rng, n_planes=40, pts_per=(5, 160), extent=20.0, noise=0.01, iso_frac=0.1):
    """Points on random planes (with normal noise) plus isotropic clusters, and
    per-point covariances like the map receives them (3x3, row-major)."""
    P, Cv = [], []
    for k in range(n_planes):
        c = rng.uniform(-extent, extent, 3)
        m = int(rng.integers(pts_per[0], pts_per[1]))
        if rng.random() < iso_frac:
            p = c + rng.normal(0, 0.15, (m, 3))
        else:
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            u = np.cross(nrm, [1.0, 0.0, 0.0])
            if np.linalg.norm(u) < 1e-3:
                u = np.cross(nrm, [0.0, 1.0, 0.0])
            u /= np.linalg.norm(u)
            v = np.cross(nrm, u)
            a = rng.uniform(-0.6, 0.6, (m, 2))
            p = c + a[:, :1] * u + a[:, 1:] * v + rng.normal(0, noise, (m, 1)) * nrm
        # float world points, as the reference's float transform produces
        p = p.astype(np.float32).astype(np.float64)
        for q in p:
            A = rng.normal(0, 0.02, (3, 3))
            cov = A @ A.T + np.eye(3) * 1e-4
            P.append(q)
            Cv.append(cov.reshape(9))
    P = np.array(P)
    Cv = np.array(Cv)
    perm = rng.permutation(len(P))
    return P[perm], Cv[perm]


def merge_scene(rng, per_voxel=130, update_per_voxel=6, n_updates=3, noise=0.005):
    """A floor and a wall sampled densely enough that their voxels freeze as
    planes, then sparse re-observations of both: every re-observation of a
    frozen plane voxel is a merge() call, and neighbouring voxels of one
    surface start in different groups, so the calls merge in long chains.
    Returns the build batch and the update batches (points, covariances)."""
    def cov_for(m):
        A = rng.normal(0, 0.02, (m, 3, 3))
        return (A @ A.transpose(0, 2, 1) + np.eye(3) * 1e-4).reshape(m, 9)

    def surface(count_per_voxel):
        pts = []
        for ix in range(-12, 12):
            for iy in range(-12, 12):  # floor z = -1.73
                a = rng.uniform(0, 0.5, (count_per_voxel, 2))
                z = -1.73 + rng.normal(0, noise, count_per_voxel)
                pts.append(np.c_[ix * 0.5 + a[:, 0], iy * 0.5 + a[:, 1], z])
            for iz in range(-3, 5):  # wall x = 3.21
                a = rng.uniform(0, 0.5, (count_per_voxel, 2))
                x = 3.21 + rng.normal(0, noise, count_per_voxel)
                pts.append(np.c_[x, ix * 0.5 + a[:, 0], iz * 0.5 + a[:, 1]])
        p = np.concatenate(pts).astype(np.float32).astype(np.float64)
        return p[rng.permutation(len(p))]

    P = surface(per_voxel)
    build = (P, cov_for(len(P)))
    updates = []
    for _ in range(n_updates):
        P = surface(update_per_voxel)
        updates.append((P, cov_for(len(P))))
    return build, updates


def export_oracle_map(olib, h):
    info = abi.vmp_map_info()
    olib.orc_map_info(h, C.byref(info))
    arr = (abi.vmp_voxel * max(1, info.size))()
    n = olib.orc_map_export(h, arr, info.size)
    pts = np.zeros((max(1, info.slab_points), 3))
    cov = np.zeros((max(1, info.slab_points), 9))
    m = olib.orc_map_export_points(h, pts.ctypes.data_as(C.POINTER(C.c_double)),
                                   cov.ctypes.data_as(C.POINTER(C.c_double)), info.slab_points)
    return arr, n, info, pts[:m], cov[:m]


def voxels_by_key(arr, n):
    return {tuple(arr[i].key): arr[i] for i in range(n)}


# The plane covariance's lower triangle: the oracle accumulates the dense
# J cov J^T of voxel_map.cpp:129, whose entry (i, j) below the diagonal has
# its own rounding; the device forms the upper triangle and mirrors it.  Per
# term the two differ by at most 3.7e-14 sqrt(C_ii C_jj) (measured on 1 M
# random terms, tests/test_restatements.py); summed over a voxel's refits
# (Cauchy-Schwarz over the positive semidefinite terms) and merges the bound
# stated here is 1e-12 sqrt(C_ii C_jj).
COV_LOWER_TOL = 1e-12


def plane_cov_problems(x, y, tol=COV_LOWER_TOL):
    """x: the oracle's 6x6 plane covariance (36 values, row-major), y: the
    device's.  The upper triangle (diagonal included) must be equal value for
    value, the lower within tol * sqrt(C_ii C_jj).  Returns (problem or None,
    largest normalised lower-triangle difference)."""
    X = np.asarray(x, dtype=np.float64).reshape(6, 6)
    Y = np.asarray(y, dtype=np.float64).reshape(6, 6)
    iu = np.triu_indices(6)
    if not np.array_equal(X[iu], Y[iu]):
        return f"upper triangle differs by {np.max(np.abs(X[iu] - Y[iu])):.3e}", 0.0
    il = np.tril_indices(6, -1)
    d = np.abs(X - Y)[il]
    s = np.sqrt(np.abs(np.diag(X)[il[0]] * np.diag(X)[il[1]]))
    worst = float(np.max(np.where(d > 0, d / np.maximum(s, 1e-300), 0.0))) if d.size else 0.0
    if np.any(d > tol * s):
        return f"lower triangle differs by {worst:.3e} sqrt(C_ii C_jj)", worst
    return None, worst


def compare_maps(vo, no, vg, ng, exact=True, tol=1e-9):
    """Compares two exported maps voxel by voxel; returns a list of problems.
    exact: every field equal, the plane covariance's lower triangle within
    COV_LOWER_TOL (see plane_cov_problems)."""
    problems = []
    A = voxels_by_key(vo, no)
    B = voxels_by_key(vg, ng)
    if set(A) != set(B):
        problems.append(f"key sets differ: oracle-only {len(set(A) - set(B))}, gpu-only {len(set(B) - set(A))}")
        return problems
    for k, a in A.items():
        b = B[k]
        for f in ("n", "newly_add_point", "is_init", "is_plane", "update_enable", "merged", "group_id", "n_temp"):
            if getattr(a, f) != getattr(b, f):
                problems.append(f"{k}: {f} oracle={getattr(a, f)} gpu={getattr(b, f)}")
        for f, size in (("mean", 3), ("ppt", 9), ("norm", 3), ("center", 3), ("cov", 36)):
            x = np.array(getattr(a, f)[:size])
            y = np.array(getattr(b, f)[:size])
            if exact and f == "cov":
                msg, _ = plane_cov_problems(x, y)
                if msg:
                    problems.append(f"{k}: cov {msg}")
            elif exact:
                if not np.array_equal(x, y):
                    problems.append(f"{k}: {f} differs by {np.max(np.abs(x - y)):.3e}")
            else:
                scale = max(1.0, float(np.max(np.abs(x))))
                if np.max(np.abs(x - y)) > tol * scale:
                    problems.append(f"{k}: {f} differs by {np.max(np.abs(x - y)):.3e}")
        if len(problems) > 20:
            break
    # LRU order
    ko = [tuple(vo[i].key) for i in range(no)]
    kg = [tuple(vg[i].key) for i in range(ng)]
    if ko != kg:
        problems.append("LRU order differs")
    return problems
