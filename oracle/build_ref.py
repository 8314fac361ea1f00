"""Build recipe for the reference's own Cython pair-counting engines.

Test infrastructure only: it compiles the halotools ``.pyx`` engines where
they lie in a read-only halotools source tree, writing every generated and
compiled file under ``oracle/_ref/`` (git-ignored).  The reference flags are
kept: ``language="c++"`` and ``-Ofast`` (halotools
``mock_observables/pair_counters/cpairs/setup_package.py:22-27``).

Cython is needed, so this runs only where Cython is installed; machines
without it (or without the halotools tree) skip it and the repository's own
C restatement of the engines (``oracle/pairs_oracle.c``) is used instead.

Usage::

    python oracle/build_ref.py [--src /path/to/halotools/checkout]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_SRC = "/root/reference"

PC = os.path.join("halotools", "mock_observables", "pair_counters")
CIC = os.path.join("halotools", "mock_observables", "counts_in_cells")
ISO = os.path.join("halotools", "mock_observables", "isolation_functions")
# engines on the pair-counting path, plus the cimported marking-function modules
ENGINES = [
    (os.path.join(PC, "cpairs"), "npairs_3d_engine"),
    (os.path.join(PC, "cpairs"), "npairs_xy_z_engine"),
    (os.path.join(PC, "cpairs"), "npairs_s_mu_engine"),
    (os.path.join(PC, "cpairs"), "npairs_projected_engine"),
    (os.path.join(PC, "cpairs"), "npairs_jackknife_3d_engine"),
    (os.path.join(PC, "cpairs"), "npairs_per_object_3d_engine"),
    (os.path.join(PC, "cpairs"), "weighted_npairs_s_mu_engine"),
    (os.path.join(PC, "cpairs"), "npairs_jackknife_xy_z_engine"),
    (os.path.join(PC, "marked_cpairs"), "marking_functions"),
    (os.path.join(PC, "marked_cpairs"), "custom_marking_func"),
    (os.path.join(PC, "marked_cpairs"), "marked_npairs_3d_engine"),
    (os.path.join(PC, "marked_cpairs"), "marked_npairs_xy_z_engine"),
    # per-object neighbours: counts in cylinders and the isolation functions
    (os.path.join(CIC, "engines", "conditions"), "conditions"),
    (os.path.join(CIC, "engines"), "counts_in_cylinders_engine"),
    (os.path.join(ISO, "engines"), "isolation_criteria_marking_functions"),
    (os.path.join(ISO, "engines"), "spherical_isolation_engine"),
    (os.path.join(ISO, "engines"), "cylindrical_isolation_engine"),
    (os.path.join(ISO, "engines"), "marked_spherical_isolation_engine"),
    (os.path.join(ISO, "engines"), "marked_cylindrical_isolation_engine"),
]


def _build_one(src_root: str, subdir: str, name: str) -> str:
    import numpy as np

    pyx = os.path.join(src_root, subdir, name + ".pyx")
    outdir = os.path.join(OUT, subdir)
    os.makedirs(outdir, exist_ok=True)
    cpp = os.path.join(outdir, name + ".cpp")
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    so = os.path.join(outdir, name + ext)
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(pyx):
        return so
    subprocess.run([sys.executable, "-m", "cython", "--cplus", "-o", cpp, pyx],
                   check=True, capture_output=True)
    inc = sysconfig.get_paths()["include"]
    subprocess.run(["g++", "-Ofast", "-shared", "-fPIC", "-I", inc, "-I", np.get_include(),
                    cpp, "-o", so], check=True, capture_output=True)
    return so


def build(src_root: str = DEFAULT_SRC) -> bool:
    """Compile the reference engines into ``oracle/_ref``; False if impossible here."""
    if not os.path.isdir(os.path.join(src_root, PC)):
        return False
    try:
        import Cython  # noqa: F401
    except ImportError:
        return False
    with ThreadPoolExecutor(max_workers=len(ENGINES)) as ex:
        list(ex.map(lambda e: _build_one(src_root, *e), ENGINES))
    return True


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=DEFAULT_SRC)
    a = ap.parse_args()
    ok = build(a.src)
    print("reference engines built" if ok else "reference engines not buildable here")
