"""Loading of the committed golden fixtures (tests/golden/*.npz, made from
the reference's own geometry code by tests/golden/make_golden.py)."""
import glob
import os

import numpy as np

from axgb.grids import MeshArrays

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def mesh(z, prefix):
    return MeshArrays(np.asarray(z[f"{prefix}_lonlat"]), np.asarray(z[f"{prefix}_off"]),
                      np.asarray(z[f"{prefix}_idx"]), name=prefix)


def cases(kind):
    return sorted(os.path.basename(p)[len(kind) + 1:-4] for p in glob.glob(os.path.join(GOLDEN, f"{kind}_*.npz")))


def load(kind, name=None):
    fn = f"{kind}_{name}.npz" if name else f"{kind}.npz"
    return np.load(os.path.join(GOLDEN, fn))
