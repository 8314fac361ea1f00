"""The cell grid each entry point chooses, computed on the host (no GPU).

gbp_grid_describe runs the same grid choice and stencil build as npairs_3d,
npairs_s_mu and npairs_xy_z.  The counts do not depend on the grid (every
in-range pair is visited once, whatever the cell size), so these tests pin the
performance choices: reach 4 in blocks of 2 for dense 3-D and (s, mu')
samples, plain reach-1 cells for the (rp, pi) count and the 100k-point case,
blocks for sparse samples, the plan's hints, and the reference's limit on the
search length (rectangular_mesh.py:376-417)."""
import ctypes

import numpy as np
import pytest

from halotools_gb300 import _native as N


def describe(period, search, n2, kind, reach=0, block=0, pbc=1):
    lib = N.load()
    out = (ctypes.c_int32 * 7)()
    p = np.ascontiguousarray(period, dtype=np.float64)
    s = np.ascontiguousarray(search, dtype=np.float64)
    rc = lib.gbp_grid_describe(p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), pbc,
                               s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n2, kind,
                               reach, block, out)
    return rc, dict(zip(("reach", "block", "nx", "ny", "nz", "runs", "block_reach"), out))


@pytest.mark.parametrize("kind", [0, 1])
def test_dense_counts_take_reach_4_in_blocks_of_2(kind):
    # 10M points in L = 2000 with a 50 search: 19.5 points per 25-unit cell
    rc, g = describe([2000.0] * 3, [50.0] * 3, 10_000_000, kind)
    assert rc == N.GBP_OK
    assert (g["reach"], g["block"], g["nx"], g["ny"], g["nz"]) == (4, 2, 160, 160, 160)
    assert g["block_reach"] == 2 and g["runs"] == 84


def test_projected_count_keeps_reach_1():
    # 2M points in L = 1000, rp up to 30 and pi up to 40
    rc, g = describe([1000.0] * 3, [30.0, 30.0, 40.0], 2_000_000, 2)
    assert rc == N.GBP_OK
    assert (g["reach"], g["block"], g["nx"], g["ny"], g["nz"]) == (1, 1, 33, 33, 25)
    assert g["runs"] == 14


def test_moderate_density_keeps_reach_1():
    # 100k points in L = 250 with a 20 search: 6.4 points per reach-2 cell
    rc, g = describe([250.0] * 3, [20.0] * 3, 100_000, 0)
    assert rc == N.GBP_OK
    assert (g["reach"], g["block"], g["nx"]) == (1, 1, 12)


def test_sparse_sample_takes_blocks():
    rc, g = describe([2000.0] * 3, [50.0] * 3, 10_000, 0)
    assert rc == N.GBP_OK
    assert g["reach"] == 1 and g["block"] == 4


def test_hints_override_the_choice():
    rc, g = describe([2000.0] * 3, [50.0] * 3, 10_000_000, 0, reach=2, block=1)
    assert rc == N.GBP_OK
    assert (g["reach"], g["block"], g["nx"], g["runs"]) == (2, 1, 80, 63)


def test_search_beyond_a_third_of_the_box_is_refused():
    rc, _ = describe([100.0] * 3, [40.0] * 3, 1000, 0)
    assert rc == N.GBP_ERR_RANGE
    rc, _ = describe([100.0] * 3, [10.0] * 3, 1000, 3)
    assert rc == N.GBP_ERR_INVALID
