"""The multi-GPU path of bench.py on CPU: two gloo ranks (one process each,
as torchrun launches them on a GPU node).  Each rank serves its own streams
(no collective on the data path); the job's value is all ranks' scans over
the slowest rank's time."""
import multiprocessing as mp
import os
import socket


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import argparse
    import bench
    r, ws, barrier, allmax, dist = bench.dist_setup(argparse.Namespace(), backend="gloo")
    streams = bench.serve_streams(argparse.Namespace(streams=6), r)
    barrier()
    wall = 1.5 if r == 1 else 1.0  # rank 1 is the slower one
    value = bench.aggregate_value(ws, 30, wall, allmax)
    q.put((r, ws, value, [s[3] for s in streams], [s[1] for s in streams]))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, v0, seeds0, rays0), (r1, ws1, v1, seeds1, rays1) = out
    assert (r0, r1, ws0, ws1) == (0, 1, 2, 2)
    assert v0 == v1 == 2 * 30 / 1.5          # max over ranks, same on both
    assert not set(seeds0) & set(seeds1)     # each rank its own streams
    assert rays0 != rays1
