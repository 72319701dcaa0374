"""Generates the golden fixtures of the oracle (small, seeded).

    python tests/golden/make_golden.py        # rewrites tests/golden/*.json

Each fixture stores a SHA-256 digest over the integer outputs (voxel keys,
counts, flags, group ids, point counts) -- these must not change -- and a few
FP64 summaries compared with a 1e-12 relative tolerance.
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _map_small():
    import oracle
    from voxelmapplus_fastlio2_gb300 import abi
    from tests.helpers import export_oracle_map, plane_points
    lib = oracle.load()
    cfg = abi.default_config()
    h = lib.orc_create(C.byref(cfg))
    rng = np.random.default_rng(1234)
    P, Cv = plane_points(rng, n_planes=60)
    lib.orc_map_build(h, _dp(P), _dp(Cv), len(P))
    for _ in range(4):
        P2, C2 = plane_points(rng, n_planes=80, pts_per=(2, 90))
        lib.orc_map_update(h, _dp(P2), _dp(C2), len(P2))
    vox, n, info, pts, cov = export_oracle_map(lib, h)
    lib.orc_destroy(h)
    ints = []
    for i in range(n):
        v = vox[i]
        ints += list(v.key) + [v.n, v.newly_add_point, v.is_init, v.is_plane, v.update_enable, v.merged, v.group_id,
                               v.n_temp]
    means = np.array([vox[i].mean[:] for i in range(n)])
    norms = np.array([vox[i].norm[:] for i in range(n)])
    covs = np.array([vox[i].cov[:] for i in range(n)])
    return ints, {"mean_sum": means.sum(0).tolist(), "norm_abs_sum": np.abs(norms).sum(0).tolist(),
                  "cov_trace_sum": [float(sum(covs[:, k * 7].sum() for k in range(6)))],
                  "n_voxels": [float(n)], "slab_points": [float(info.slab_points)]}


def _scan_room():
    import oracle
    from voxelmapplus_fastlio2_gb300 import abi, synth
    seq = synth.Sequence(synth.KIND_ROOM, points_per_scan=4000)
    cfg = abi.default_config(scan_resolution=0.2)
    o = oracle.Oracle(cfg)
    ints = []
    poses = []
    for _ in range(8):
        r = o.process(seq.next())
        ints += [r.lio_status, r.n_raw, r.n_down, r.effect_num, r.iters, r.map_size]
        poses.append(list(r.x.pos[:]) + list(r.x.rot[:]))
    return ints, {"final_pose": poses[-1], "pose_sum": np.array(poses).sum(0).tolist()}


CASES = {"map_small": _map_small, "scan_room": _scan_room}


def compute(name):
    ints, values = CASES[name]()
    digest = hashlib.sha256(np.array(ints, dtype=np.int64).tobytes()).hexdigest()
    return {"digest": digest, "values": values}


def main():
    import oracle
    oracle.build()
    for name in CASES:
        out = compute(name)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(out, f, indent=1)
        print(name, out["digest"][:16])


if __name__ == "__main__":
    main()
