"""Loader for the golden vectors in tests/golden (made by make_golden.py)."""
import glob
import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(prefix=""):
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = {}
    for k in d.files:
        if k.endswith("_none"):
            continue
        if k + "_none" in d.files:
            c[k] = None
        else:
            v = d[k]
            c[k] = v.item() if v.ndim == 0 else v
    if "gen" in c:
        x = np.random.default_rng(0).uniform(0, 250, (100000, 3))
        if hashlib.sha256(x.tobytes()).hexdigest() != c["sha"]:
            return None
        c["s1"] = x
    if c.get("period") is not None and np.ndim(c["period"]) == 0:
        c["period"] = float(c["period"])
    return c


def call(mod, c):
    """Run one golden case through a module with the halotools signatures."""
    s1 = c["s1"]
    s2 = s1 if c["s2"] is None else c["s2"]
    kind = c["kind"]
    if kind == "3d":
        return mod.npairs_3d(s1, s2, c["bins"], period=c["period"])
    if kind == "xyz":
        return mod.npairs_xy_z(s1, s2, c["bins"], c["bins2"], period=c["period"])
    if kind == "smu":
        return mod.npairs_s_mu(s1, s2, c["bins"], c["bins2"], period=c["period"])
    if kind == "marked":
        w1 = c["w1"]
        w2 = w1 if c["w2"] is None else c["w2"]
        return mod.marked_npairs_3d(s1, s2, c["bins"], int(c["wid"]), period=c["period"],
                                    weights1=w1, weights2=w2)
    raise ValueError(kind)
