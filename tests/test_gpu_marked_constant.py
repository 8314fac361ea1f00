"""Marking functions 1-10 with constant marks give exact multiples of the
unweighted pair counts, the pattern of halotools' own marked tests
(test_marked_npairs_3d.py:235-575): a regular 10^3 grid in a unit periodic box
(spacing (1 - 0.001) / 9), edges 0, 0.1, 0.2, 0.3.  The GPU sums (FP32 with
compensation, FP64 totals) must equal the multiple exactly, and the oracle."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _grid():
    g = np.linspace(0, 1 - 0.001, 10)
    xx, yy, zz = np.meshgrid(g, g, g)
    return np.vstack([xx.ravel(), yy.ravel(), zz.ravel()]).T


def _marks(a, b, n):
    return np.vstack([np.full(n, float(a)), np.full(n, float(b))]).T


# (weight function id, marks per point, multiple of the unweighted counts)
CASES = [
    (1, np.full(1000, 3.0), 9.0),
    (2, np.full(1000, 3.0), 6.0),
    (3, _marks(2, 3, 1000), 9.0),
    (3, _marks(3, 2, 1000), 4.0),
    (4, _marks(2, 3, 1000), 0.0),
    (5, _marks(2, 3, 1000), 0.0),
    (6, _marks(2, 3, 1000), 0.0),
    (7, _marks(1, -1, 1000), -1.0),
    (8, _marks(1, 3, 1000), 3.0),
    (9, _marks(1, 3, 1000), 3.0),
    (10, _marks(1, 3, 1000), 0.0),
    (10, _marks(1, -3, 1000), -3.0),
]


@pytest.mark.parametrize("wid,marks,mult", CASES)
def test_constant_marks_give_exact_multiples(gpu, wid, marks, mult):
    x = _grid()
    rb = np.array([0.0, 0.1, 0.2, 0.3])
    counts = gpu.npairs_3d(x, x, rb, period=1.0)
    got = gpu.marked_npairs_3d(x, x, rb, wid, period=1.0, weights1=marks, weights2=marks)
    assert np.array_equal(got, mult * counts.astype(np.float64)), (wid, got, counts)
    want = oracle.marked_npairs_3d(x, x, rb, wid, period=1.0, weights1=marks, weights2=marks)
    assert np.array_equal(got, want)
