"""Build recipe for the reference's own Cython pair-counting engines.

Test infrastructure only: it compiles the halotools ``.pyx`` engines where
they lie in a read-only halotools source tree, writing every generated and
compiled file under ``oracle/_ref/`` (git-ignored).  The reference flags are
kept: ``language="c++"`` and ``-Ofast`` (halotools
``mock_observables/pair_counters/cpairs/setup_package.py:22-27``).

Generating the C++ needs Cython and the halotools tree.  Compiling the
generated C++ needs neither: ``build_generated`` compiles whatever
``oracle/_ref`` already holds for the running platform (g++, the Python and
numpy headers), which is how the engines are built on a machine that has the
generated files but no halotools checkout.  Where neither works, the
repository's own C restatement (``oracle/pairs_oracle.c``) stands in.

The halotools checkout is read from ``$HALOTOOLS_SRC``, else from
``DEFAULT_SRC``.

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
DEFAULT_SRC = os.environ.get("HALOTOOLS_SRC", "/root/reference")

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


def _compile(cpp: str, so: str) -> str:
    """g++ with the reference flags (-Ofast, C++), into a temporary name first."""
    import numpy as np

    inc = sysconfig.get_paths()["include"]
    tmp = so + ".tmp%d" % os.getpid()
    subprocess.run(["g++", "-Ofast", "-shared", "-fPIC", "-I", inc, "-I", np.get_include(),
                    cpp, "-o", tmp], check=True, capture_output=True)
    os.replace(tmp, so)
    return so


def _build_one(src_root: str, subdir: str, name: str) -> str:
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
    return _compile(cpp, so)


# the engines the CPU reference of the benchmark runs (oracle/ref_driver.py)
DRIVER_ENGINES = ("npairs_3d_engine", "npairs_xy_z_engine")


def build_generated(names=DRIVER_ENGINES) -> bool:
    """Compile the already generated C++ of the ``cpairs`` engines ``names`` for
    this platform where no up-to-date module exists; True when all are there."""
    outdir = os.path.join(OUT, PC, "cpairs")
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    todo = []
    for name in names:
        cpp = os.path.join(outdir, name + ".cpp")
        so = os.path.join(outdir, name + ext)
        if os.path.exists(so) and (not os.path.exists(cpp) or
                                   os.path.getmtime(so) >= os.path.getmtime(cpp)):
            continue
        if not os.path.exists(cpp):
            return False
        todo.append((cpp, so))
    if todo:
        try:
            with ThreadPoolExecutor(max_workers=len(todo)) as ex:
                list(ex.map(lambda t: _compile(*t), todo))
        except (subprocess.CalledProcessError, OSError):
            return False
    return True


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
