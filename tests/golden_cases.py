"""Loader of the golden fixtures made by tests/golden/make_golden.py from the reference build."""
import glob
import json
import os

import numpy as np

from ooc_svo_builder_gb300 import octree

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    tree = octree.Octree(meta["s"], np.frombuffer(z["nodes"].tobytes(), dtype=octree.NODE_DTYPE),
                         np.frombuffer(z["data"].tobytes(), dtype=octree.DATA_DTYPE))
    return z["tris"], meta, tree
