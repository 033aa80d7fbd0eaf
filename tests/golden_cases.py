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


# Configuration 3, recorded by make_fullsize_golden.py --large: svo_builder_binary -s 4096
# -l 2048 (64 partitions) on the seeded 20M-triangle soup; the node file is about 16 GB.
FULLSIZE_LARGE = {
    "soup4096": dict(gridsize=4096, limit=2048, payload=False, color="model",
                     make=lambda: tri.soup_tris(20_000_000, 4096, seed=3, sigma=1.0)),
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


def seeded_case(i: int):
    """Case i of a seeded mix of inputs and flags: (triangles, gridsize, memory limit,
    payload, colour mode, -levels, kind).  Kinds: random triangles inside the grid, soups,
    icospheres, triangles spilling far outside the grid, triangles much smaller than a
    voxel, and vertices on a lattice of voxel faces; gridsize 1 to 256, with 1 to 64
    partitions."""
    import random
    rng = random.Random(1000 + i)
    payload = rng.random() < 0.5
    N = rng.choice([1, 2, 4, 8, 16, 32, 64, 128, 256])
    limit = rng.choice([2048, 2, 4]) if N >= 128 else 2048
    color = rng.choice(["model", "fixed", "linear", "normal"]) if payload else "model"
    levels = rng.random() < 0.4
    kind = ["random", "soup", "ico", "outside", "tiny", "lattice"][i % 6]
    seed = rng.randrange(1 << 30)
    if kind == "random":
        t = tri.random_tris(rng.randrange(1, 1500), seed, payload, lo=-0.1, hi=1.1, max_edge=rng.choice([0.01, 0.1, 0.5]))
    elif kind == "soup":
        t = tri.soup_tris(rng.randrange(10, 2000), max(N, 8), seed=seed, sigma=1.0, n_spheres=3, payload=payload)
    elif kind == "ico":
        t = tri.icosphere_tris(rng.randrange(1, 4), radius=rng.uniform(0.1, 0.49), jitter=0.002, seed=seed,
                               payload=payload)
    elif kind == "outside":
        t = tri.random_tris(rng.randrange(1, 1000), seed, payload, lo=-1.0, hi=2.0, max_edge=0.6)
    elif kind == "tiny":
        t = tri.random_tris(rng.randrange(1, 500), seed, payload, lo=0.0, hi=1.0, max_edge=1e-5)
    else:
        g = np.arange(0, 9, dtype=np.float32) / np.float32(8)
        r = np.random.default_rng(seed)
        t = g[r.integers(0, 9, size=(rng.randrange(1, 300), 9))].astype(np.float32)
        if payload:
            t = np.concatenate([t, r.random((t.shape[0], 12), dtype=np.float32)], axis=1)
    return t, N, limit, payload, color, levels, kind


N_SEEDED = 48


def reference_undefined(gridsize, mortons):
    """Why the reference's output is undefined for a build with these set voxels (Morton
    codes), or None.

    finalizeTree (OctreeBuilder.cpp:35-37) pads with empty voxels only while the next
    Morton code is below N^3 - 1.  When the last set voxel is N^3 - 2, the last voxel is
    never added, the top groups are never completed and the root is read from an empty
    buffer; with N = 1 and no set voxel the same read happens."""
    last = int(np.max(mortons)) if len(mortons) else None
    if gridsize ** 3 >= 2 and last == gridsize ** 3 - 2:
        return "the last set voxel is N^3-2: finalizeTree leaves the tree unfinished (OctreeBuilder.cpp:35-37)"
    if gridsize == 1 and last is None:
        return "N = 1 with no set voxel: finalizeTree reads the root from an empty buffer (OctreeBuilder.cpp:35-41)"
    return None


def set_voxels(tree, payload):
    """Morton codes of a tree's set voxels."""
    return tree.data["morton"][1:] if payload else octree.leaves(tree)[0]
