"""The device's short forms of three reference products against the dense
reference-order forms, on the CPU (oracle/restatements.cpp), 1 M random
inputs each with exact zeros of both signs mixed in:

* point_crossmat * P_rr * point_crossmat^T (lio_builder.cpp:199-202, 240-243);
* calcBodyCov's (range direction_hat) N and A dvar A^T (commons.cpp:40-43);
* updatePlane's per-point J * pv.cov * J^T (voxel_map.cpp:115-129), of which
  the device forms the upper triangle.

Leaving out a product with an exact zero can only change the sign of a zero
result: every value must be equal, and bits may differ only where the value
is zero.  Which signed zero a covariance entry holds cannot reach a decision
or a non-zero output (the entries only enter sums, products and square roots
of sums, never a division or a sign test).  For the plane covariance the dense
form's lower triangle, which the device mirrors from the upper, must stay
within the bound the map tests use.
"""
import ctypes as C

import pytest

from tests.helpers import COV_LOWER_TOL

N = 1_000_000


def _check(oracle_lib, kind, seed):
    counts = (C.c_longlong * 4)()
    worst = C.c_double()
    oracle_lib.orc_restatement_check(kind, N, seed, counts, C.byref(worst))
    entries, value_mismatch, bit_mismatch, bit_mismatch_nonzero = list(counts)
    return entries, value_mismatch, bit_mismatch, bit_mismatch_nonzero, worst.value


@pytest.mark.parametrize("kind,name", [(0, "hat sandwich"), (1, "body covariance")])
def test_zero_skipping_forms_equal_dense_forms(oracle_lib, kind, name):
    entries, value_mismatch, bit_mismatch, bit_mismatch_nonzero, _ = _check(oracle_lib, kind, 1234 + kind)
    assert entries == 9 * N
    assert value_mismatch == 0, name
    assert bit_mismatch_nonzero == 0, name


def test_plane_cov_upper_triangle_equals_dense_form(oracle_lib):
    entries, value_mismatch, bit_mismatch, bit_mismatch_nonzero, worst = _check(oracle_lib, 2, 99)
    assert entries == 21 * N
    assert value_mismatch == 0
    assert bit_mismatch_nonzero == 0
    # the dense lower triangle against the mirrored upper, per term
    assert 0.0 < worst <= COV_LOWER_TOL / 10, worst
