"""The C-ABI library builds, loads and exports every symbol of include/gbpairs.h
(no compute call: these run without a GPU)."""
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gbpairs.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*\*?\s*(gbp_\w+)\s*\(", txt, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("gbp_npairs_3d", "gbp_npairs_xy_z", "gbp_npairs_s_mu", "gbp_marked_npairs_3d",
              "gbp_plan_create", "gbp_plan_destroy"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from halotools_gb300 import _native
    lib = _native.load()
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_binding_covers_header():
    from halotools_gb300 import _native
    assert set(declared_symbols()) <= set(_native.EXPORTED)


def test_plan_create_without_gpu_reports_no_device():
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("GPU present")
    import halotools_gb300 as h
    with pytest.raises(h.GBPairsUnavailable):
        h.Plan(0)
