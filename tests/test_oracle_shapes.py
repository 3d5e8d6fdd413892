"""Shape partition of unity, restating share/picongpu/unit/shape.cpp:105-207.

Uses the reference test's own 1024 positions (std::mt19937(42), uniform [0,1),
tests/golden/make_shape_positions.sh) and its tolerance: Catch::Approx(1.0)
with margin = float epsilon (shape.cpp:52-55), where Approx keeps its default
relative epsilon of 100 float epsilons, so |sum - 1| <= 100 * eps passes.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
POS = np.fromfile(os.path.join(HERE, "golden", "shape_positions_mt19937_42.f32"), np.float32)
EPS = np.finfo(np.float32).eps
TOL = max(EPS, 100 * EPS * 1.0)  # Catch::Approx(1.0).margin(eps)

# (begin, end) of ChargeAssignmentOnSupport and ChargeAssignment per shape (NGP, CIC, TSC, PQS, PCS)
ON_SUPPORT = {0: (0, 0), 1: (0, 1), 2: (-1, 1), 3: (-1, 2), 4: (-2, 2)}
FULL = {0: (0, 1), 1: (0, 2), 2: (-1, 2), 3: (-1, 3), 4: (-2, 3)}


def position_shift(pos, is_even):
    """PositionShift functor of shape.cpp:86-101."""
    v = np.float32(pos - np.float32(0.5))
    if is_even:
        s = 0 if v >= np.float32(-0.5) else -1
    else:
        s = 1 if v >= np.float32(0.0) else 0
    return np.float32(np.float32(v - np.float32(s)) + np.float32(0.5))


def test_positions_fixture():
    assert POS.shape == (1024,)
    assert POS.min() >= 0.0 and POS.max() < 1.0


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
def test_partition_of_unity_on_support(orc, shape):
    L = orc.lib()
    b, e = ON_SUPPORT[shape]
    supp = shape + 1
    for pos in POS:
        p = position_shift(pos, supp % 2 == 0)
        s = np.float32(0.0)
        for gp in range(b, e + 1):
            s = np.float32(s + np.float32(L.orc_shape_value(shape, 1, float(np.float32(gp) - p))))
        assert abs(s - 1.0) <= TOL, (shape, pos, s)


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
def test_partition_of_unity_charge_assignment(orc, shape):
    L = orc.lib()
    b, e = FULL[shape]
    for pos in POS:
        s = np.float32(0.0)
        for gp in range(b, e + 1):
            s = np.float32(s + np.float32(L.orc_shape_value(shape, 0, float(np.float32(gp) - pos))))
        assert abs(s - 1.0) <= TOL, (shape, pos, s)


@pytest.mark.parametrize("shape", [1, 2, 3, 4])
def test_shape_arrays_match_piecewise(orc, shape):
    """The cached shape arrays (ShapeSelector.hpp Cached) equal the piecewise functions (Jit)."""
    import ctypes

    L = orc.lib()
    supp = shape + 1
    b = FULL[shape][0]
    out = np.zeros(supp + 1, np.float32)
    for pos in POS[:256]:
        x = np.float32(pos - np.float32(0.5)) if supp % 2 else pos  # in-range domain of the cached array
        for oor in (0, 1):
            p = np.float32(x + np.float32(1.0)) if oor else x  # out of range: one cell above the base cell
            L.orc_shape_ca_array(shape, float(p), oor, out.ctypes.data_as(ctypes.c_void_p))
            for k in range(supp + 1):
                ref = L.orc_shape_value(shape, 0, float(np.float32(b + k) - p))
                assert abs(out[k] - ref) <= 4 * EPS, (shape, p, oor, k, out[k], ref)
            assert abs(out.sum() - 1.0) <= TOL
