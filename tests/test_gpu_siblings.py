"""Sibling counters (npairs_projected, npairs_jackknife_3d, npairs_per_object_3d)
against halotools' own engines (golden vectors, make_sibling_golden.py)."""
import os

import numpy as np
import pytest

from tests.golden import make_sibling_golden as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_sibling_matches_reference(gpu, name):
    d = np.load(os.path.join(G.OUT, name + ".npz"))
    if str(d["sha"]) != G.input_sha():
        pytest.skip("seeded generator differs on this platform")
    fn = {"projected": "npairs_projected", "jackknife": "npairs_jackknife_3d",
          "per_object": "npairs_per_object_3d"}[name.rsplit("_", 2)[0]]
    if not hasattr(gpu, fn):
        pytest.skip(fn + " not built")
    got = G.run_case(gpu, name)
    assert got.dtype == d["out"].dtype and got.shape == d["out"].shape
    assert np.array_equal(got, d["out"])  # integer counts and half-integers are exact
