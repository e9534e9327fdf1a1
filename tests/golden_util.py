"""Loading helpers for the golden vectors of tests/golden (made by
tests/golden/make_golden.py from the reference's own code)."""
import glob
import os

import numpy as np

from vbm3d_gb300._abi import Params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def _params(vec):
    p = Params()
    for (name, typ), v in zip(Params._fields_, vec):
        setattr(p, name, float(v) if "float" in typ.__name__ else int(v))
    return p


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["p1"] = _params(g["p1"])
    g["p2"] = _params(g["p2"])
    g["sigma"] = float(g["sigma"])
    g["color_space"] = bool(g["color_space"])
    g.setdefault("fflow", None)
    g.setdefault("bflow", None)
    return g
