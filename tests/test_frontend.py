"""Argument handling of the drop-in front-ends; mirrors the reference's own
error-message tests (test_npairs_3d.py:270-304, test_npairs_xy_z.py:267-341,
test_marked_npairs_3d.py:181-232).  Every case raises before any GPU work."""
import numpy as np
import pytest

import halotools_gb300 as h

rng = np.random.default_rng(3)
S = rng.uniform(0, 1, (50, 3))


def test_sensible_num_threads():
    with pytest.raises(ValueError) as err:
        h.npairs_3d(S, S, [0.1, 0.2], period=1, num_threads="Cuba Gooding Jr.")
    assert "Input ``num_threads`` argument must be an integer or the string 'max'" in str(err.value)


def test_sensible_rbins():
    with pytest.raises(ValueError) as err:
        h.npairs_3d(S, S, 0.1, period=1)
    assert "Input ``rbins`` must be a monotonically increasing 1D array with at least two entries" in str(err.value)
    with pytest.raises(ValueError):
        h.npairs_3d(S, S, [0.1, 0.3, 0.2], period=1)


def test_sensible_period():
    with pytest.raises(ValueError) as err:
        h.npairs_3d(S, S, [0.1, 0.2], period=np.inf)
    assert "Input ``period`` must be a bounded positive number in all dimensions" in str(err.value)


def test_search_longer_than_third_of_box():
    with pytest.raises(ValueError) as err:
        h.npairs_3d(S, S, [0.1, 0.4], period=1)
    assert "cannot be larger than Lbox/3" in str(err.value)


def test_rp_pi_bins_messages():
    with pytest.raises(ValueError) as err:
        h.npairs_xy_z(S, S, 0.1, [0.1, 0.2], period=1)
    assert "Input ``rp_bins`` must be a monotonically increasing 1D array" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.npairs_xy_z(S, S, [0.1, 0.2], [0.3, 0.2, 0.1], period=1)
    assert "Input ``pi_bins`` must be a monotonically increasing 1D array" in str(err.value)


def test_mu_bins_message():
    with pytest.raises(ValueError) as err:
        h.npairs_s_mu(S, S, [0.1, 0.2], [0.5, 0.2, 0.1], period=1)
    assert "Input `mu_bins` must be a monotonically increasing" in str(err.value)


def test_approx_cell_size_shape():
    with pytest.raises(ValueError) as err:
        h.npairs_3d(S, S, [0.1, 0.2], period=1, approx_cell1_size=[0.1, 0.1])
    assert "must be a length-3 sequence" in str(err.value)


@pytest.mark.parametrize("wid", list(range(1, 18)))
def test_marked_weight_shapes(wid):
    nw = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 2, 11: 2,
          12: 4, 13: 4, 14: 3, 15: 3, 16: 5, 17: 5}[wid]
    with pytest.raises(h.HalotoolsError):
        h.marked_npairs_3d(S, S, [0.1, 0.2], wid, period=1, weights1=np.ones((50, nw + 1)),
                           weights2=np.ones((50, nw + 1)))
    with pytest.raises(h.HalotoolsError):
        h.marked_npairs_3d(S, S, [0.1, 0.2], wid, period=1, weights1=np.ones(49),
                           weights2=np.ones((50, nw)))


def test_marked_bad_ids():
    with pytest.raises(h.HalotoolsError):
        h.marked_npairs_3d(S, S, [0.1, 0.2], 18, period=1)
    with pytest.raises(ValueError):
        h.marked_npairs_3d(S, S, [0.1, 0.2], 1.0, period=1)


def test_marked_xy_z_ids_and_shapes():
    # marked_npairs_xy_z.py:292-333 knows ids 1-15; the default id 0 is an error
    for wid in (0, 16, 17):
        with pytest.raises(h.HalotoolsError) as err:
            h.marked_npairs_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], period=1, weight_func_id=wid)
        assert "is not recognized" in str(err.value)
    with pytest.raises(ValueError):
        h.marked_npairs_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], period=1, weight_func_id=1.0)
    with pytest.raises(h.HalotoolsError):
        h.marked_npairs_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], period=1, weight_func_id=5,
                             weights1=np.ones((50, 3)), weights2=np.ones((50, 2)))
    with pytest.raises(ValueError) as err:
        h.marked_npairs_xy_z(S, S, [0.3, 0.2, 0.1], [0.1, 0.2], period=1, weight_func_id=1)
    assert "rp_bins" in str(err.value)


def test_weighted_s_mu_messages():
    # weighted_npairs_s_mu.py:171-187
    with pytest.raises(AssertionError) as err:
        h.weighted_npairs_s_mu(S, S, np.ones(49), np.ones(50), [0.1, 0.2], [0, 1], period=1)
    assert "``weights1`` should have shape (50, )" in str(err.value)
    with pytest.raises(AssertionError) as err:
        h.weighted_npairs_s_mu(S, S, np.ones(50), np.ones((50, 1)), [0.1, 0.2], [0, 1], period=1)
    assert "``weights2`` should have shape (50, )" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.weighted_npairs_s_mu(S, S, np.ones(50), np.ones(50), [0.1, 0.2], [0, 0.5, 0.4],
                               period=1)
    assert "Input `mu_bins` must be a monotonically increasing" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.weighted_npairs_s_mu(S, S, np.ones(50), np.ones(50), [0.3, 0.2, 0.1], [0, 1], period=1)
    assert "Input ``rbins`` must be a monotonically increasing" in str(err.value)



def test_jackknife_xy_z_messages():
    t = np.ones(50, dtype=int)
    with pytest.raises(h.HalotoolsError) as err:
        h.npairs_jackknife_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], t[:49], t, 1, period=1)
    assert "jtags1 should have same len as sample1" in str(err.value)
    with pytest.raises(h.HalotoolsError) as err:
        h.npairs_jackknife_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], t, t * 3, 2, period=1)
    assert "jtags2 must be <= N_samples" in str(err.value)
    with pytest.raises(h.HalotoolsError) as err:
        h.npairs_jackknife_xy_z(S, S, [0.1, 0.2], [0.1, 0.2], t, t, 1, period=1,
                                weights1=np.ones(49))
    assert "weights1 should have same len as sample1" in str(err.value)


def test_neighbour_messages():
    with pytest.raises(ValueError) as err:
        h.counts_in_cylinders(S, S, np.ones(3), 0.1, period=1)
    assert "``proj_search_radius`` must be a scalar or length-Npts1 array" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.counts_in_cylinders(S, S, 0.1, np.ones(3), period=1)
    assert "``cylinder_half_length`` must be a scalar or length-Npts1 array" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.counts_in_cylinders(S, S, 0.1, 0.1, period=1, condition="bogus")
    assert "'condition' must be None or a permitted descriptive string" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.spherical_isolation(S, S, 0.0, period=1)
    assert "bounded positive numbers" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.cylindrical_isolation(S, S, np.ones(3), 0.1, period=1)
    assert "must be the same length as ``sample1``" in str(err.value)
    with pytest.raises(h.HalotoolsError):
        h.conditional_spherical_isolation(S, S, 0.1, cond_func=7, period=1)
    with pytest.raises(ValueError) as err:
        h.conditional_cylindrical_isolation(S, S, 0.1, 0.1, marks1=np.ones((50, 1)),
                                            marks2=np.ones((50, 1)), cond_func=5, period=1)
    assert "there should be 2 marks per point" in str(err.value)
    with pytest.raises(ValueError) as err:
        h.spherical_isolation(S, S, 0.5, period=1)
    assert "cannot be larger than Lbox/3" in str(err.value)


def test_marked_channels_messages():
    # (N, nch) marks, 1 <= nch <= 32, the same channel count on both sides
    rb = [0.1, 0.2]
    with pytest.raises(ValueError, match="1 to 32 mark channels"):
        h.marked_npairs_3d_channels(S, S, rb, period=1, weights1=np.ones((50, 33)),
                                    weights2=np.ones((50, 33)))
    with pytest.raises(h.HalotoolsError, match="same number of channels"):
        h.marked_npairs_3d_channels(S, S, rb, period=1, weights1=np.ones((50, 2)),
                                    weights2=np.ones((50, 3)))
    with pytest.raises(h.HalotoolsError, match="must have shape"):
        h.marked_npairs_3d_channels(S, S, rb, period=1, weights1=np.ones((49, 2)))
    with pytest.raises(h.HalotoolsError, match="must have shape"):
        h.marked_npairs_3d_channels(S, S, rb, period=1, weights1=np.ones((50, 2, 1)))
    with pytest.raises(ValueError, match="monotonically increasing"):
        h.marked_npairs_3d_channels(S, S, [0.2, 0.1, 0.05], period=1)


def test_batched_weight_columns_message():
    torch = pytest.importorskip("torch")
    from halotools_gb300 import differentiable as D
    x = torch.zeros((10, 3), dtype=torch.float64)
    for W in (torch.ones((10, 33), dtype=torch.float64), torch.ones(10, dtype=torch.float64)):
        with pytest.raises(ValueError, match="1 <= M <= 32"):
            D.weighted_pair_counts_batched(W, x, [0.1, 0.2], 1.0)
    with pytest.raises(ValueError, match="Lbox/3"):
        D.weighted_pair_counts_batched(torch.ones((10, 2), dtype=torch.float64), x, [0.1, 0.5],
                                       1.0)


def _enclose_per_column(s1, s2, min_size):
    # the reference's form (mesh_helpers.py:17-64): six per-column minima and
    # maxima, both samples shifted in their input dtype
    x1, x2 = s1[:, :3], s2[:, :3]
    cols = [x1[:, 0], x2[:, 0], x1[:, 1], x2[:, 1], x1[:, 2], x2[:, 2]]
    xyzmin = np.min([np.min(c) for c in cols])
    xyzmax = np.max([np.max(c) for c in cols]) - xyzmin
    lbox = np.array([xyzmax] * 3)
    min_size = np.atleast_1d(min_size)
    lbox[lbox < min_size] = min_size[lbox < min_size]
    return x1 - xyzmin, x2 - xyzmin, lbox.astype(np.float64)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("ncol", [3, 4])
def test_enclose_in_box_matches_per_column_form(dtype, ncol):
    from halotools_gb300.pair_counters import _enclose_in_box
    g = np.random.default_rng(ncol)
    a = (g.uniform(-40, 60, (500, ncol)) * [1.0, 0.5, 2.0, 1.0][:ncol]).astype(dtype)
    b = g.uniform(-10, 90, (300, ncol)).astype(dtype)
    for s1, s2, same in ((a, b, False), (a, a, True), (b, a, False)):
        for min_size in ([1.0, 1.0, 1.0], [500.0, 1.0, 300.0]):
            got = _enclose_in_box(s1, s2, min_size, same)
            want = _enclose_per_column(s1, s2, min_size)
            for x, y in zip(got, want):
                assert x.dtype == y.dtype and np.array_equal(x, y)


def test_per_point_radii_match_broadcast_forms():
    from halotools_gb300.neighbours import _get_r_max, _per_point
    for v in (2.5, -0.0, 0.0, np.nan, np.inf):
        got, gmax = _per_point(v, 7, "m")
        want = np.zeros(7) + np.atleast_1d(v).astype("f8")[0]
        assert got.dtype == want.dtype and np.array_equal(got.view(np.int64), want.view(np.int64))
        assert np.array_equal(np.float64(gmax).view(np.int64), np.max(want).view(np.int64))
        assert _per_point(v, 0, "m")[1] == 0.0
    arr = np.linspace(1.0, 2.0, 7)
    got, gmax = _per_point(arr, 7, "m")
    assert np.array_equal(got, arr) and gmax == 2.0
    with pytest.raises(ValueError, match="m"):
        _per_point(arr, 6, "m")
    # isolation_functions_helpers.py:11-35
    assert np.array_equal(_get_r_max(5, 1.5), np.array([1.5] * 5))
    for bad in (0.0, -1.0, np.inf, np.nan):
        with pytest.raises(ValueError, match="bounded positive"):
            _get_r_max(5, bad)
        assert len(_get_r_max(0, bad)) == 0
    with pytest.raises(ValueError, match="same length"):
        _get_r_max(5, [1.0, 2.0])
    with pytest.raises(ValueError, match="bounded positive"):
        _get_r_max(2, [1.0, 0.0])


def test_jackknife_tag_checks_and_coverage_warning():
    import warnings as w
    from halotools_gb300.pair_counters import _jackknife_inputs
    t = np.arange(50) % 5 + 1  # every subsample 1..5 present
    with w.catch_warnings():
        w.simplefilter("error")
        _jackknife_inputs(S, S, t, t, 5, None, None)
        _jackknife_inputs(S, S, t.astype(float), t, 5.0, None, None)
        _jackknife_inputs(S, S, t[:, None], t[:, None], 5, None, None)  # (N, 1) tags
    for tags, n in ((np.minimum(t, 4), 5), (t, 6)):  # subsample 5, or 6, has no point
        with pytest.warns(UserWarning, match="every jackknife sample"):
            _jackknife_inputs(S, S, tags, tags, n, None, None)
    with pytest.warns(UserWarning, match="every jackknife sample"):
        _jackknife_inputs(S, S, t, t, 5.5, None, None)  # np.unique form for a fractional count
    # one array for both sides is still checked against each sample
    with pytest.raises(h.HalotoolsError, match="jtags1 must be >= 1"):
        _jackknife_inputs(S, S, t - 1, t - 1, 5, None, None)
    with pytest.raises(h.HalotoolsError, match="jtags2 should have same len as sample2"):
        _jackknife_inputs(S, S[:40], t, t, 5, None, None)
    with pytest.raises(h.HalotoolsError, match="jtags2 must be <= N_samples"):
        _jackknife_inputs(S, S, t, t + 1, 5, None, None)
