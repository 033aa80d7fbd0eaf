"""Loader of the golden fixtures made from the reference build by tests/golden/make_golden.py
(small cases, whole files) and tests/golden/make_fullsize_golden.py (full-size
configurations, as digests)."""
import glob
import json
import os

import numpy as np

from ooc_svo_builder_gb300 import octree, tri

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    tree = octree.Octree(meta["s"], np.frombuffer(z["nodes"].tobytes(), dtype=octree.NODE_DTYPE),
                         np.frombuffer(z["data"].tobytes(), dtype=octree.DATA_DTYPE))
    return z["tris"], meta, tree


# Full-size configurations whose reference outputs are recorded as digests in
# golden/fullsize_reference.json by golden/make_fullsize_golden.py.
FULLSIZE = {
    # svo_builder_binary -s 256 -l 2048 on a subdivision-5 icosphere (20,480 triangles)
    "icosphere256": dict(gridsize=256, limit=2048, payload=False, color="model",
                         make=lambda: tri.icosphere_tris(5, radius=0.4, jitter=0.002, seed=1)),
    # svo_builder -s 1024 -l 2048 -c model on a 1024x1024-vertex heightfield (2,093,058 triangles)
    "heightfield1024": dict(gridsize=1024, limit=2048, payload=True, color="model",
                            make=lambda: tri.heightfield_tris(1024, seed=2, payload=True)),
    # the same with -levels: averaged payloads on every inner node
    "heightfield1024_levels": dict(gridsize=1024, limit=2048, payload=True, color="model", levels=True,
                                   make=lambda: tri.heightfield_tris(1024, seed=2, payload=True)),
}


def fullsize_reference():
    with open(os.path.join(GOLDEN, "fullsize_reference.json")) as f:
        return json.load(f)


def input_sha256(tris) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(tris).tobytes()).hexdigest()


# The first meshes of the seeded mesh streams of configurations 4 (batched builds) and 5
# (served requests); their reference digests are in golden/stream_samples_reference.json.
STREAMS = {
    "batch4096": dict(seed=4, n=64, gridsizes=(64, 128, 256, 512)),
    "serve": dict(seed=5, n=16, gridsizes=(128, 256, 512, 1024, 2048)),
}
STREAM_LIMIT_MB = 2048


def stream_sample(name):
    """[(triangles, gridsize, payload)] of the first meshes of stream `name`."""
    s = STREAMS[name]
    return tri.batch_meshes(s["n"], seed=s["seed"], gridsizes=s["gridsizes"])


def stream_samples_reference():
    with open(os.path.join(GOLDEN, "stream_samples_reference.json")) as f:
        return json.load(f)
