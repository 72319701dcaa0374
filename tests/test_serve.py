"""Serving (many streams on one GPU) through libvmp's server API.

The reference has no serving layer; these tests pin the server's contract:
each stream's results are bit-identical alone and in the mix (their work
overlaps on the device), per-stream order is kept, admission follows the HBM
budget (at once, or waiting for slots and memory to free up), and a closed
stream frees its budget.
"""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi, synth

pytestmark = pytest.mark.gpu


def _packages(kind, seed, pts, count):
    seq = synth.Sequence(kind, seed=seed, points_per_scan=pts)
    return [seq.next() for _ in range(count)]


def _cfg(kind):
    if kind == synth.KIND_URBAN:
        return abi.default_config(scan_resolution=0.1, map_capacity=300000, max_scan_points=40064, ieskf_max_iter=4)
    return abi.default_config(scan_resolution=0.2, map_capacity=100000, max_scan_points=16384)


def _key(res):
    """The bits of a result that must not depend on the other streams."""
    return (res.lio_status, res.iters, res.effect_num, res.n_raw, res.n_down, res.map_size, bytes(res.x),
            bytes(res.P))


def _run_server(streams, workers, concurrent, **server_kw):
    """streams: list of (kind, packages).  concurrent=False submits one
    stream's next package only after the previous stream's finished."""
    from voxelmapplus_fastlio2_gb300.serve import Server
    srv = Server(hbm_budget_bytes=150e9, max_streams=len(streams), workers=workers, **server_kw)
    try:
        sids = [srv.open_stream(_cfg(kind)) for kind, _ in streams]
        out = {sid: [] for sid in sids}
        if concurrent:
            total = 0
            for k in range(max(len(p) for _, p in streams)):
                for sid, (_, pk) in zip(sids, streams):
                    if k < len(pk):
                        srv.submit(sid, pk[k], cookie=k)
                        total += 1
            got = 0
            while got < total:
                for r in srv.poll(timeout_ms=1000):
                    assert r.status == abi.VMP_OK, r.status
                    out[r.stream_id].append((r.cookie, _key(r.result)))
                    got += 1
        else:
            for sid, (_, pk) in zip(sids, streams):
                for k, p in enumerate(pk):
                    srv.submit(sid, p, cookie=k)
                    rs = []
                    while not rs:
                        rs = srv.poll(timeout_ms=1000)
                    assert len(rs) == 1 and rs[0].status == abi.VMP_OK
                    out[sid].append((rs[0].cookie, _key(rs[0].result)))
        maps = {}
        for sid in sids:
            v, n = srv.stream(sid).map.export()
            maps[sid] = C.string_at(v, n * C.sizeof(abi.vmp_voxel))
        return [out[s] for s in sids], [maps[s] for s in sids]
    finally:
        srv.close()


def test_alone_equals_mix():
    """Eight streams (rooms and urban blocks, own seeds and scan sizes):
    every per-scan result and every final map is the same bits whether the
    streams run one at a time or all at once on 8 workers."""
    streams = []
    for i in range(8):
        kind = synth.KIND_ROOM if i % 2 == 0 else synth.KIND_URBAN
        pts = [3000, 20000, 8000, 40000, 12000, 30000, 5000, 25000][i]
        streams.append((kind, _packages(kind, 0x5EED0000 + 100 + i, pts, 8)))
    alone, maps_alone = _run_server(streams, workers=1, concurrent=False)
    mix, maps_mix = _run_server(streams, workers=8, concurrent=True)
    for i, (a, b) in enumerate(zip(alone, mix)):
        assert [c for c, _ in b] == list(range(len(streams[i][1])))  # per-stream order kept
        assert [k for _, k in a] == [k for _, k in b], f"stream {i} differs between alone and mix"
        assert maps_alone[i] == maps_mix[i], f"stream {i} map differs"


def test_admission_by_budget_and_release():
    from voxelmapplus_fastlio2_gb300.serve import Server
    from voxelmapplus_fastlio2_gb300._lib import VmpError
    srv = Server(hbm_budget_bytes=150e9, max_streams=8, workers=2)
    try:
        a = srv.open_stream(_cfg(synth.KIND_ROOM))
        one = srv.info()["budget_used"]
        assert one > 0
    finally:
        srv.close()
    srv = Server(hbm_budget_bytes=int(2.5 * one), max_streams=8, workers=2)
    try:
        a = srv.open_stream(_cfg(synth.KIND_ROOM))
        b = srv.open_stream(_cfg(synth.KIND_ROOM))
        with pytest.raises(VmpError) as e:
            srv.open_stream(_cfg(synth.KIND_ROOM))
        assert e.value.code == abi.VMP_ERR_ADMISSION_DENIED
        assert srv.info()["streams_open"] == 2
        srv.close_stream(a)
        c = srv.open_stream(_cfg(synth.KIND_ROOM))  # the freed budget admits a new stream
        assert srv.info()["streams_open"] == 2 and c != b
    finally:
        srv.close()


def _alone(kind, pkgs):
    """A stream's per-package results on a stream of its own."""
    from voxelmapplus_fastlio2_gb300 import lio
    g = lio.LIOBuilder(_cfg(kind))
    out = [_key(g.process(p)) for p in pkgs]
    g.close()
    return out


def test_admission_waits_for_budget_while_streams_run():
    """vmp_server_open_stream_wait: with the budget full and packages of the
    open streams in flight, a request waits (the other streams keep
    running), is admitted as soon as a stream closes, and its stream then
    runs; every stream's results equal its results alone.  A request that
    never fits is denied at once; one that outlasts its time limit times out."""
    import threading
    import time
    from voxelmapplus_fastlio2_gb300.serve import Server
    from voxelmapplus_fastlio2_gb300._lib import VmpError
    kinds = [synth.KIND_ROOM, synth.KIND_ROOM, synth.KIND_ROOM]
    pk = [_packages(k, 0x5EED0000 + 400 + i, [6000, 9000, 7000][i], 10) for i, k in enumerate(kinds)]
    ref = [_alone(k, p) for k, p in zip(kinds, pk)]
    srv = Server(hbm_budget_bytes=150e9, max_streams=4, workers=2)
    try:
        srv.open_stream(_cfg(synth.KIND_ROOM))
        one = srv.info()["budget_used"]
    finally:
        srv.close()
    srv = Server(hbm_budget_bytes=int(2.5 * one), max_streams=4, workers=2)
    try:
        a = srv.open_stream(_cfg(kinds[0]))
        b = srv.open_stream(_cfg(kinds[1]))
        for k in range(10):
            srv.submit(a, pk[0][k], cookie=k)
            srv.submit(b, pk[1][k], cookie=k)
        got = {}
        waiter = {}

        def wait_open():
            try:
                waiter["sid"] = srv.open_stream_wait(_cfg(kinds[2]), timeout_ms=120000)
            except VmpError as e:
                waiter["err"] = e.code

        th = threading.Thread(target=wait_open)
        th.start()
        time.sleep(0.3)
        assert th.is_alive() and srv.info()["streams_open"] == 2  # waiting while a and b run
        srv.close_stream(a)  # waits for a's packages, frees its budget
        th.join(timeout=60)
        assert not th.is_alive() and "sid" in waiter, waiter
        c = waiter["sid"]  # may reuse a's slot: its packages carry cookies 100..109
        for k in range(10):
            srv.submit(c, pk[2][k], cookie=100 + k)
        while sum(len(v) for v in got.values()) < 30:
            for r in srv.poll(timeout_ms=1000):
                assert r.status == abi.VMP_OK, r.status
                i = 2 if r.cookie >= 100 else (0 if r.stream_id == a else 1)
                got.setdefault(i, []).append((r.cookie % 100, _key(r.result)))
        for i in range(3):
            seq = sorted(got[i])
            assert [x for x, _ in seq] == list(range(10))
            assert [k for _, k in seq] == ref[i], f"stream {i} differs from its results alone"
        # budget full again (b and c open): a request with a short limit times out
        with pytest.raises(VmpError) as e:
            srv.open_stream_wait(_cfg(synth.KIND_ROOM), timeout_ms=200)
        assert e.value.code == abi.VMP_ERR_TIMEOUT
        assert srv.info()["streams_open"] == 2
    finally:
        srv.close()
    srv = Server(hbm_budget_bytes=int(0.5 * one), max_streams=4, workers=2)
    try:
        with pytest.raises(VmpError) as e:
            srv.open_stream_wait(_cfg(synth.KIND_ROOM), timeout_ms=-1)  # larger than the whole budget
        assert e.value.code == abi.VMP_ERR_ADMISSION_DENIED
    finally:
        srv.close()


def test_residual_register_budget_does_not_change_results():
    """The residual kernel compiled for 3 or 4 resident CTAs per SM
    (vmp_set_residual_ctas_per_sm), switched between scans (the scan graphs
    are captured again): the same results as with either setting throughout."""
    from voxelmapplus_fastlio2_gb300 import lio
    kind = synth.KIND_URBAN
    pk = _packages(kind, 0x5EED0000 + 500, 30000, 10)
    lib = lio.load()
    runs = []
    try:
        for sched in ([3] * 10, [4] * 10, [3, 3, 3, 4, 4, 3, 4, 3, 4, 4]):
            g = lio.LIOBuilder(_cfg(kind))
            res = []
            for c, p in zip(sched, pk):
                assert lib.vmp_set_residual_ctas_per_sm(c) == 0
                res.append(_key(g.process(p)))
            runs.append(res)
            g.close()
    finally:
        lib.vmp_set_residual_ctas_per_sm(4)  # the default
    assert runs[1] == runs[0] and runs[2] == runs[0]


def test_merge_launch_shape_does_not_change_results():
    """The served merge resolution runs on grids of SMs / divisor CTAs (the
    autotuner's knob): every divisor gives the same results and maps."""
    streams = []
    for i in range(4):
        kind = synth.KIND_ROOM if i % 2 == 0 else synth.KIND_URBAN
        streams.append((kind, _packages(kind, 0x5EED0000 + 200 + i, [6000, 30000, 10000, 20000][i], 7)))
    runs = [_run_server(streams, workers=4, concurrent=True, autotune=False, merge_grid_divisor=d)
            for d in (2, 16, 152)]
    for res, maps in runs[1:]:
        assert [[k for _, k in r] for r in res] == [[k for _, k in r] for r in runs[0][0]]
        assert maps == runs[0][1]


def test_seg_grid_blocks_do_not_change_results():
    """The voxel-chain kernels' working blocks (the autotuner's
    seg_grid_blocks knob, read on the device by the captured launches): one
    block, a few and all of them give the same results and maps, and the
    setting is undone when the server is destroyed."""
    from voxelmapplus_fastlio2_gb300 import _lib
    streams = []
    for i in range(4):
        kind = synth.KIND_ROOM if i % 2 == 0 else synth.KIND_URBAN
        streams.append((kind, _packages(kind, 0x5EED0000 + 300 + i, [8000, 30000, 12000, 24000][i], 7)))
    runs = [_run_server(streams, workers=4, concurrent=True, autotune=False, seg_grid_blocks=b)
            for b in (1, 152, 2432)]
    for res, maps in runs[1:]:
        assert [[k for _, k in r] for r in res] == [[k for _, k in r] for r in runs[0][0]]
        assert maps == runs[0][1]
    from voxelmapplus_fastlio2_gb300.serve import Server
    srv = Server(hbm_budget_bytes=150e9, max_streams=1, workers=1)  # one worker: no throughput mode
    try:
        v = C.c_int()
        assert _lib.load().vmp_server_knob(srv.h, b"seg_grid_blocks", C.byref(v)) == abi.VMP_OK
        assert v.value == 0  # every block works again
    finally:
        srv.close()


def test_autotuner_reports_state():
    from voxelmapplus_fastlio2_gb300.serve import Server
    srv = Server(hbm_budget_bytes=150e9, max_streams=2, workers=2)
    try:
        t = srv.tuning()
        assert t["merge_grid_divisor"] in (4, 8, 16, 32, 64) and t["windows"] == 0
        assert t["max_inflight"] == 2  # starts at the workers
        assert t["seg_grid_blocks"] == 152
    finally:
        srv.close()


def _livox(rng, pkg):
    pts = pkg.points_np()
    a = np.zeros(pkg.n, dtype=abi.livox_dtype())
    a["x"], a["y"], a["z"] = pts[:, 0], pts[:, 1], pts[:, 2]
    a["offset_time"] = np.rint(pts[:, 3].astype(np.float64) * 1e6).astype(np.uint32)
    a["reflectivity"] = rng.integers(0, 256, pkg.n)
    a["tag"] = rng.choice(np.array([0x00, 0x10, 0x20], dtype=np.uint8), pkg.n, p=[0.6, 0.35, 0.05])
    a["line"] = rng.choice(np.array([0, 1, 2, 3, 4], dtype=np.uint8), pkg.n, p=[0.24, 0.24, 0.24, 0.24, 0.04])
    return a


def test_served_livox_messages_match_direct_decode():
    """Raw Livox messages submitted to the server (decoded by the worker, end
    time from the last kept point) give the results of vmp_livox_decode +
    vmp_process_decoded on a stream of one's own, bit for bit, with four
    streams' messages in flight together."""
    from voxelmapplus_fastlio2_gb300 import lio
    from voxelmapplus_fastlio2_gb300.serve import Server
    rng = np.random.default_rng(11)
    streams = []
    for s in range(4):
        pk = _packages(synth.KIND_ROOM, 0x5EED0000 + 300 + s, 6000, 12)
        streams.append([(p, _livox(rng, p)) for p in pk])
    cfg = _cfg(synth.KIND_ROOM)
    direct = []
    for msgs in streams:
        g = lio.LIOBuilder(cfg)
        res = []
        for p, a in msgs:
            n, last = g.livox_decode(a, 2, 0.1, 100.0, copy_out=False)
            res.append(_key(g.process_decoded(p.t_start, p.t_start + float(last) / 1000.0, p.imus, p.n_imu)))
        direct.append(res)
        g.close()
    srv = Server(hbm_budget_bytes=50e9, max_streams=4, workers=4)
    try:
        sids = [srv.open_stream(cfg) for _ in streams]
        for k in range(12):
            for sid, msgs in zip(sids, streams):
                p, a = msgs[k]
                srv.submit_livox(sid, a, p.t_start, p.imus, p.n_imu, filter_num=2, range_min=0.1, range_max=100.0,
                                 cookie=k)
        got = {}
        while sum(len(v) for v in got.values()) < 12 * len(sids):
            for r in srv.poll(timeout_ms=1000):
                assert r.status == abi.VMP_OK
                got.setdefault(r.stream_id, []).append((r.cookie, _key(r.result)))
        for i, sid in enumerate(sids):
            seq = sorted(got[sid])
            assert [c for c, _ in seq] == list(range(12))
            assert [k for _, k in seq] == direct[i]
    finally:
        srv.close()
