"""install_into_halotools() against halotools' own estimator modules.

halotools is not installed here; oracle/ref_loader.py loads its estimator
modules from a halotools checkout over the reference's compiled engines.  In a
fresh process: install rebinds the counter names that tpcf, rp_pi_tpcf,
s_mu_tpcf and marked_tpcf imported at load time (tpcf.py:26, rp_pi_tpcf.py:23,
s_mu_tpcf.py:25, marked_tpcf.py:17), halotools' own tpcf then calls the GPU
counter (which, with no GPU here, raises GBPairsUnavailable from inside
halotools' code), and the modules that cannot import are reported.  Skipped
where no checkout or compiled engines exist."""
import os
import subprocess
import sys

import pytest

import halotools_gb300 as h

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

SCRIPT = r"""
import sys, warnings
sys.path.insert(0, %(root)r)
warnings.simplefilter("ignore", SyntaxWarning)
import numpy as np
from oracle import ref_loader
try:
    est = ref_loader.load_estimators()
except Exception as exc:
    print("SKIP", repr(exc)); sys.exit(0)
import halotools_gb300 as h
names = {"tpcf": "npairs_3d", "rp_pi_tpcf": "npairs_xy_z", "s_mu_tpcf": "npairs_s_mu",
         "marked_tpcf": "marked_npairs_3d"}
before = {m: getattr(est[m], a) for m, a in names.items()}
assert all(f is not getattr(h, names[m]) for m, f in before.items())
# strict: the modules of the table that cannot import here are named
try:
    h.install_into_halotools()
    raise SystemExit("strict install did not report failing modules")
except ImportError as exc:
    assert "failed to import" in str(exc)
with warnings.catch_warnings(record=True):
    warnings.simplefilter("always")
    done = h.install_into_halotools(strict=False)
for m, a in names.items():
    assert getattr(est[m], a) is getattr(h, a), (m, a)
    assert "halotools.mock_observables.two_point_clustering.%%s.%%s" %% (m, a) in done
# halotools' own tpcf now reaches the GPU counter
x = np.random.default_rng(0).uniform(0, 100.0, (500, 3))
try:
    est["tpcf"].tpcf(x, np.logspace(-1, 1, 5), period=100.0)
except h.GBPairsUnavailable:
    print("ROUTED")
else:
    import torch
    print("ROUTED" if torch.cuda.is_available() else "NOT ROUTED")
"""


def test_install_rebinds_halotools_estimators():
    r = subprocess.run([sys.executable, "-c", SCRIPT % {"root": ROOT}], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    if r.stdout.startswith("SKIP"):
        pytest.skip(r.stdout.strip())
    assert "ROUTED" in r.stdout.split(), r.stdout


def test_install_without_halotools_is_a_noop():
    assert h.install_into_halotools() == []


IA_SCRIPT = r"""
import sys, warnings
sys.path.insert(0, %(root)r)
warnings.simplefilter("ignore", SyntaxWarning)
import numpy as np
from oracle import ref_loader
try:
    ia = ref_loader.load_alignments()
except Exception as exc:
    print("SKIP", repr(exc)); sys.exit(0)
import halotools_gb300 as h
rng = np.random.default_rng(0)
x = rng.uniform(0, 100.0, (300, 3))
o = rng.normal(size=(300, 3))
rb = np.logspace(-1, 1, 5)
# before: halotools' own ee_3d over its own engines
before = ia["ee_3d"].ee_3d(x, o, x, o, rb, period=100.0)
assert len(before) == len(rb) - 1
with warnings.catch_warnings(record=True):
    warnings.simplefilter("always")
    done = h.install_into_halotools(strict=False)
pre = "halotools.mock_observables.ia_correlations."
for m, names in (("ee_3d", ("marked_npairs_3d", "npairs_3d")),
                 ("ee_projected", ("marked_npairs_xy_z", "npairs_xy_z"))):
    for a in names:
        assert getattr(ia[m], a) is getattr(h, a), (m, a)
        assert pre + m + "." + a in done, (m, a)
# after: halotools' own ee_3d reaches the GPU counters
try:
    ia["ee_3d"].ee_3d(x, o, x, o, rb, period=100.0)
except h.GBPairsUnavailable:
    print("ROUTED")
else:
    import torch
    print("ROUTED" if torch.cuda.is_available() else "NOT ROUTED")
"""


def test_install_rebinds_alignment_estimators():
    # halotools' ee_3d / ee_projected bind their plain and marked counters at
    # import time (ee_3d.py:15, ee_projected.py:15)
    r = subprocess.run([sys.executable, "-c", IA_SCRIPT % {"root": ROOT}], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    if r.stdout.startswith("SKIP"):
        pytest.skip(r.stdout.strip())
    assert "ROUTED" in r.stdout.split(), r.stdout


USERS_SCRIPT = r"""
import sys, warnings
sys.path.insert(0, %(root)r)
warnings.simplefilter("ignore", SyntaxWarning)
import numpy as np
from oracle import ref_loader
try:
    mods = ref_loader.load_counter_users()
except Exception as exc:
    print("SKIP", repr(exc)); sys.exit(0)
import halotools_gb300 as h
with warnings.catch_warnings(record=True):
    warnings.simplefilter("always")
    done = h.install_into_halotools(strict=False)
want = {"angular_tpcf": ("npairs_3d",),
        "tpcf_one_two_halo_decomp": ("npairs_3d", "marked_npairs_3d"),
        "large_scale_density_spherical_volume": ("npairs_per_object_3d",),
        "large_scale_density_spherical_annulus": ("npairs_per_object_3d",),
        "underdensity_prob_func": ("npairs_per_object_3d",)}
for m, names in want.items():
    for a in names:
        assert getattr(mods[m], a) is getattr(h, a), (m, a)
        assert any(d.endswith("." + m + "." + a) for d in done), (m, a)
# halotools' own large-scale density function reaches the GPU per-object counter
x = np.random.default_rng(0).uniform(0, 100.0, (400, 3))
try:
    mods["large_scale_density_spherical_volume"].large_scale_density_spherical_volume(
        x, x, 5.0, period=100.0)
except h.GBPairsUnavailable:
    print("ROUTED")
else:
    import torch
    print("ROUTED" if torch.cuda.is_available() else "NOT ROUTED")
"""


def test_install_rebinds_other_counter_users():
    # angular_tpcf.py:15, tpcf_one_two_halo_decomp.py:24-25,
    # large_scale_density_spherical_volume.py:12, ..._annulus.py:12,
    # underdensity_prob_func.py:12 bind their counters at import time
    r = subprocess.run([sys.executable, "-c", USERS_SCRIPT % {"root": ROOT}],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    if r.stdout.startswith("SKIP"):
        pytest.skip(r.stdout.strip())
    assert "ROUTED" in r.stdout.split(), r.stdout
