"""The driver of the reference's compiled engines (oracle/ref_driver.py), which
times halotools' own npairs_3d / npairs_xy_z engines as the benchmark's CPU
reference: its restated mesh must be the reference's mesh, its full call must
give the reference front-end's counts, and its slabs must add up to the whole
workload exactly.  CPU only; skipped where the compiled engines are absent."""
import numpy as np
import pytest

from oracle import oracle, ref_driver as R

pytestmark = pytest.mark.skipif(not R.engines_available(),
                                reason="reference engines not compiled here")


def _pts(n, L, seed):
    return np.random.default_rng(seed).uniform(0, L, (n, 3))


def test_full_call_and_slabs_match_oracle_3d():
    x = _pts(40000, 250.0, 1)
    rb = np.logspace(-1, np.log10(20), 15)
    want = oracle.npairs_3d(x, x, rb, period=250.0, num_threads=4)
    assert np.array_equal(R.full_call("3d", x, x, rb, None, 250.0, 4), want)
    sc = R.SlabCounter("3d", x, x, rb, None, 250.0, 3, 5)
    try:
        tot = sum(sc.count(k)[0] for k in range(sc.nslabs))
    finally:
        sc.close()
    assert np.array_equal(tot, want)


def test_full_call_and_slabs_match_oracle_xy_z():
    x = _pts(30000, 200.0, 2)
    y = _pts(20000, 200.0, 3)
    rp = np.logspace(-1, np.log10(25), 10)
    pi = np.linspace(0, 30, 9)
    want = oracle.npairs_xy_z(x, y, rp, pi, period=200.0, num_threads=4)
    assert np.array_equal(R.full_call("xyz", x, y, rp, pi, 200.0, 4), want)
    sc = R.SlabCounter("xyz", x, y, rp, pi, 200.0, 4, 7)
    try:
        tot = sum(sc.count(k)[0] for k in range(sc.nslabs))
    finally:
        sc.close()
    assert np.array_equal(tot, want)


def test_cell1_ranges_split_like_the_reference():
    # np.array_split of the cell ids, empty parts dropped (mesh_helpers.py:214-221)
    assert R.cell1_ranges(0, 10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert R.cell1_ranges(5, 7, 4) == [(5, 6), (6, 7)]
    assert R.cell1_ranges(0, 9, 1) == [(0, 9)]


def test_mesh_and_counts_match_the_reference_front_end():
    """Against halotools' own RectangularDoubleMesh and npairs_3d, where the
    halotools tree is available to import them."""
    try:
        from oracle import ref_loader
        ns = ref_loader.load()
        from halotools.mock_observables.pair_counters.rectangular_mesh import \
            RectangularDoubleMesh
    except Exception as exc:  # no halotools checkout here
        pytest.skip("reference front-ends not importable: %r" % (exc,))
    x = _pts(30000, 300.0, 4)
    c = (x[:, 0], x[:, 1], x[:, 2])
    for search, approx2 in (((25.0,) * 3, (25.0,) * 3), ((20.0, 20.0, 40.0), (10.0, 10.0, 20.0))):
        dm = R.DoubleMesh(c, c, search, approx2, search, (300.0,) * 3)
        rm = RectangularDoubleMesh(*c, *c, *search, *approx2, *search, 300.0, 300.0, 300.0, True)
        for m in ("mesh1", "mesh2"):
            a, b = getattr(dm, m), getattr(rm, m)
            for k in ("idx_sorted", "cell_id_indices", "num_xdivs", "num_ydivs", "num_zdivs",
                      "xcell_size", "zcell_size", "ncells"):
                assert np.array_equal(getattr(a, k), getattr(b, k)), (m, k)
    rb = np.logspace(-1, np.log10(25), 12)
    assert np.array_equal(R.full_call("3d", x, x, rb, None, 300.0, 4),
                          ns.npairs_3d(x, x, rb, period=300.0, num_threads=4))
    pi = np.linspace(0, 40, 11)
    assert np.array_equal(R.full_call("xyz", x, x, rb, pi, 300.0, 4),
                          ns.npairs_xy_z(x, x, rb, pi, period=300.0, num_threads=4))


def test_bench_reference_arm_counts_the_whole_workload():
    """bench.py --impl reference on config 1: its K slabs count the workload once
    (21,542,180 in-range ordered pairs, the reference's own count) and the line
    carries the contract's keys."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--workload", "3d100k", "--steps", "3", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "reference"
    assert line["pairs_counted"] == 21542180 and line["slabs"] == 3
    assert line["full_call"]["same_counts_as_slabs"] is True
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
