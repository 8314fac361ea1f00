"""In-tree build of the gbpairs CUDA library for sm_103a (GB300).

``python -m halotools_gb300.build`` compiles every translation unit under
``halotools_gb300/csrc`` in parallel with nvcc and links
``halotools_gb300/_lib/libgbpairs.so``.  No CMake, no torch extension
machinery: the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import glob
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUTDIR, "libgbpairs.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-fmad=true",
              "-Xptxas", "-O3"]


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _fingerprint() -> str:
    h = hashlib.sha256()
    for f in sorted(glob.glob(os.path.join(CSRC, "*")) +
                    [os.path.join(HERE, "..", "include", "gbpairs.h")]):
        with open(f, "rb") as fh:
            h.update(os.path.basename(f).encode())
            h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()[:16]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if sources changed) and return the path of libgbpairs.so."""
    os.makedirs(OUTDIR, exist_ok=True)
    stamp = os.path.join(OUTDIR, "build.stamp")
    fp = _fingerprint()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == fp:
                return LIB
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUTDIR, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", os.path.join(HERE, "..", "include"),
               "-c", src, "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(_sources()))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp%d" % os.getpid()
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
