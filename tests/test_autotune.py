"""The serving autotuner's climb (vmp_server_* with autotune on), driven by a
model throughput instead of a GPU through the vmp_test_autotune hook: the
same code the server runs at every completed package, fed completion times
spaced by 1 / rate of the launch shapes it currently applies.

Knobs: merge grid divisor (4, 8, 16, 32, 64) and residual CTAs per SM
(3, 4).  The climbs start after 8 windows of 128 packages at the starting
shapes, take the knobs one after the other, and then keep the shapes for 32
windows.  That both knobs leave results unchanged is tested on the GPU
(test_serve.py: test_merge_launch_shape_does_not_change_results,
test_residual_register_budget_does_not_change_results)."""
import ctypes as C
import os

import numpy as np
import pytest

DIV = [4, 8, 16, 32, 64]
CTAS = [3, 4]


def _lib():
    from voxelmapplus_fastlio2_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_all()
    return _lib.load()


def _climb(start_d, start_c, rate_fn, windows):
    rates = np.array([[rate_fn(d, c) for c in CTAS] for d in DIV], dtype=np.float64).reshape(-1)
    trace = np.zeros(2 * windows, dtype=np.int32)
    code = _lib().vmp_test_autotune(start_d, start_c, C.c_void_p(rates.ctypes.data), windows,
                                    C.c_void_p(trace.ctypes.data))
    assert code == 0
    return trace.reshape(windows, 2)


def _peaked(best_d, best_c):
    # throughput falling off with the distance (in candidates) from the best shape
    return lambda d, c: 5000.0 - 400.0 * abs(DIV.index(d) - DIV.index(best_d)) - 150.0 * abs(c - best_c)


def _settled(tr, last=40):
    """The shapes kept in the last windows (exploiting, with the next round's
    probes of the neighbours in between)."""
    vals, counts = np.unique(tr[-last:], axis=0, return_counts=True)
    return tuple(int(v) for v in vals[np.argmax(counts)])


def test_climb_moves_off_a_bad_start():
    tr = _climb(64, 3, _peaked(16, 4), 80)
    assert all(tuple(t) == (64, 3) for t in tr[:7])  # the first windows keep the starting shapes
    assert _settled(tr) == (16, 4)
    # settled within the first round of climbs, then kept for the exploit windows
    assert all(tuple(t) == (16, 4) for t in tr[20:45])


@pytest.mark.parametrize("best", [(4, 3), (32, 4), (64, 4)])
def test_climb_reaches_the_best_shape(best):
    tr = _climb(16, 3, _peaked(*best), 80)
    assert _settled(tr) == best


def test_climb_keeps_a_good_start():
    tr = _climb(16, 3, _peaked(16, 3), 80)
    # probes visit the neighbours only; the kept shape is the start
    assert set(int(d) for d in tr[:, 0]) <= {8, 16, 32}
    assert _settled(tr) == (16, 3)
