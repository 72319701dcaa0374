"""The serving autotuner's climb (vmp_server_* with autotune on), driven by a
model throughput instead of a GPU through the vmp_test_autotune hook: the
same code the server runs at every completed package, fed completion times
spaced by 1 / rate of the launch shapes it currently applies.

Knobs: merge grid divisor (4, 8, 16, 32, 64), max_inflight, the packages
on the GPU at once (8, 16, 24, 32), and seg_grid_blocks, the working blocks
of the voxel-chain kernels (76, 152, 304: the launches' size under a server).  The climbs start
after 24 windows of 128 packages at the starting shapes, take the knobs one
after the other, and then keep the shapes for 32 windows.  No knob changes
results: the merge divisor and the voxel-chain blocks are tested on the GPU
(test_serve.py: test_merge_launch_shape_does_not_change_results,
test_seg_grid_blocks_do_not_change_results); max_inflight only decides when
a worker starts the next package."""
import ctypes as C
import os

import numpy as np
import pytest

DIV = [4, 8, 16, 32, 64]
INFL = [8, 16, 24, 32]
SEG = [76, 152, 304]
FIRST = 24  # windows at the starting shapes


def _lib():
    from voxelmapplus_fastlio2_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_all()
    return _lib.load()


def _climb(start, rate_fn, windows):
    rates = np.array([[[rate_fn(d, c, b) for b in SEG] for c in INFL] for d in DIV], dtype=np.float64).reshape(-1)
    trace = np.zeros(3 * windows, dtype=np.int32)
    code = _lib().vmp_test_autotune(start[0], start[1], start[2], C.c_void_p(rates.ctypes.data), windows,
                                    C.c_void_p(trace.ctypes.data))
    assert code == 0
    return trace.reshape(windows, 3)


def _peaked(best):
    # throughput falling off with the distance (in candidates) from the best shape
    bd, bc, bb = best
    return lambda d, c, b: (5000.0 - 400.0 * abs(DIV.index(d) - DIV.index(bd))
                            - 150.0 * abs(INFL.index(c) - INFL.index(bc))
                            - 250.0 * abs(SEG.index(b) - SEG.index(bb)))


def _settled(tr, last=40):
    """The shapes kept in the last windows (exploiting, with the next round's
    probes of the neighbours in between)."""
    vals, counts = np.unique(tr[-last:], axis=0, return_counts=True)
    return tuple(int(v) for v in vals[np.argmax(counts)])


def test_climb_moves_off_a_bad_start():
    tr = _climb((64, 8, 76), _peaked((16, 24, 304)), 140)
    assert all(tuple(t) == (64, 8, 76) for t in tr[:FIRST - 1])  # the first windows keep the starting shapes
    assert _settled(tr) == (16, 24, 304)
    # settled within the first round of climbs, then kept for the exploit windows
    assert all(tuple(t) == (16, 24, 304) for t in tr[FIRST + 15:FIRST + 45])


@pytest.mark.parametrize("best", [(4, 8, 76), (32, 32, 152), (64, 16, 304)])
def test_climb_reaches_the_best_shape(best):
    tr = _climb((16, 32, 304), _peaked(best), 140)
    assert _settled(tr) == best


def test_climb_keeps_a_good_start():
    tr = _climb((16, 32, 152), _peaked((16, 32, 152)), 140)
    # probes visit the neighbours only; the kept shape is the start
    assert set(int(d) for d in tr[:, 0]) <= {8, 16, 32}
    assert set(int(c) for c in tr[:, 1]) <= {24, 32}
    assert set(int(b) for b in tr[:, 2]) <= {76, 152, 304}
    assert _settled(tr) == (16, 32, 152)
