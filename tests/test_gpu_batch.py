"""ooc_build_batch: many meshes of different gridsizes, modes and flags in one call.

Each mesh's octree must equal the oracle's (and so ooc_build's) on that mesh alone.
"""
import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc

import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu


def mixed_meshes(seed=5, count=24):
    rng = np.random.default_rng(seed)
    meshes, params, oracle_args = [], [], []
    for i in range(count):
        payload = bool(rng.integers(0, 2))
        N = int(rng.choice([1, 8, 32, 64, 128, 256]))
        limit = 2 if (N == 256 and rng.random() < 0.5) else 2048
        levels = bool(rng.integers(0, 2))
        color = str(rng.choice(["model", "fixed", "linear", "normal"])) if payload else "model"
        kind = rng.integers(0, 3)
        if kind == 0:
            t = tri.icosphere_tris(int(rng.integers(1, 4)), payload=payload, seed=int(rng.integers(0, 1000)))
        elif kind == 1:
            t = tri.random_tris(int(rng.integers(1, 400)), int(rng.integers(0, 1000)), payload, lo=-0.1, hi=1.1,
                                max_edge=float(rng.uniform(0.01, 0.5)))
        else:
            t = np.zeros((0, 21 if payload else 9), np.float32)
        meshes.append(t)
        params.append(make_params(N, limit, geometry_only=not payload, color=color, levels=levels))
        oracle_args.append(dict(gridsize=N, memory_limit_mb=limit, color=color, levels=levels))
    return meshes, params, oracle_args


def test_batch_matches_single_mesh_builds(builder):
    meshes, params, args = mixed_meshes()
    results = builder.build_batch(meshes, params)
    assert len(results) == len(meshes)
    for t, r, a in zip(meshes, results, args):
        nodes, data, info = pyoracle.build(t, a["gridsize"], a["memory_limit_mb"], color=a["color"],
                                           levels=a["levels"])
        d = octree.diff(r.tree, octree.Octree(a["gridsize"], nodes, data))
        assert not d, "\n".join(d)
        assert r.info["n_filled"] == info["n_filled"]
        assert r.info["n_partitions"] == info["n_partitions"]


def test_batch_split_into_sub_batches(builder):
    # many 256^3 meshes exceed no budget; the call must still give per-mesh results in order
    meshes = [tri.random_tris(300, 700 + i, i % 2 == 1, max_edge=0.2) for i in range(6)]
    params = [make_params(256, 2048 if i % 3 else 2, geometry_only=(i % 2 == 0)) for i in range(6)]
    results = builder.build_batch(meshes, params)
    for i, (t, r) in enumerate(zip(meshes, results)):
        nodes, data, _ = pyoracle.build(t, 256, 2048 if i % 3 else 2)
        assert not octree.diff(r.tree, octree.Octree(256, nodes, data))


def test_batch_device_matches_single_mesh_builds(builder):
    # octrees written straight into device memory equal the oracle's, mesh by mesh
    meshes, params, args = mixed_meshes(seed=6, count=32)
    results = builder.build_batch_device(meshes, params)
    for t, r, a in zip(meshes, results, args):
        nodes, data, info = pyoracle.build(t, a["gridsize"], a["memory_limit_mb"], color=a["color"],
                                           levels=a["levels"])
        d = octree.diff(r.tree, octree.Octree(a["gridsize"], nodes, data))
        assert not d, "\n".join(d)
        assert r.info["n_filled"] == info["n_filled"]


def test_batch_device_meshes_straddling_sub_batches(builder):
    # a small pyramid budget splits meshes across sub-batches: their early
    # stripes wait in the carry buffers until the mesh's destination exists
    meshes = [tri.random_tris(400, 900 + i, i % 2 == 1, max_edge=0.3) for i in range(5)]
    params = [make_params(256, 2, geometry_only=(i % 2 == 0), levels=(i == 3)) for i in range(5)]
    old = builder.batch_budget()
    try:
        builder.set_batch_budget(700_000)  # two 128^3 stripes (300 KB of pyramid each) per sub-batch
        results = builder.build_batch_device(meshes, params)
        host = builder.build_batch(meshes, params)
    finally:
        builder.set_batch_budget(old)
    for i, (t, r) in enumerate(zip(meshes, results)):
        nodes, data, _ = pyoracle.build(t, 256, 2, levels=(i == 3))
        assert not octree.diff(r.tree, octree.Octree(256, nodes, data))
        assert not octree.diff(host[i].tree, r.tree)


def test_every_tuning_gives_the_same_octrees(builder):
    # launch choices change speed only: extreme values against the oracle
    meshes, params, args = mixed_meshes(seed=8, count=12)
    meshes.append(tri.random_tris(60, 5, True, lo=0.0, hi=1.0, max_edge=1.2))  # many large triangles
    params.append(make_params(128, 2048, geometry_only=False))
    args.append(dict(gridsize=128, memory_limit_mb=2048, color="model", levels=False))
    old = builder.tuning()
    want = []
    for t, a in zip(meshes, args):
        nodes, data, _ = pyoracle.build(t, a["gridsize"], a["memory_limit_mb"], color=a["color"], levels=a["levels"])
        want.append(octree.Octree(a["gridsize"], nodes, data))
    try:
        for small_vol, lpl, block, cps, budget, graphs, ept, pdl, persistent in [
                (1, 1, 64, 1, 4096, 1, 1, 1, 0), (64, 64, 256, 16, 1 << 30, 0, 16, 1, 0),
                (27, 3, 128, 2, 700_000, 1, 3, 0, 0), (64, 16, 256, 4, 4 << 30, 1, 4, 0, 0),
                (64, 16, 256, 4, 4 << 30, 0, 8, 0, 0),
                # the persistent phase A: tiny sub-batches, captured; wide task lists; defaults
                (1, 1, 64, 1, 4096, 1, 1, 1, 1), (64, 64, 256, 16, 1 << 30, 0, 16, 1, 1),
                (27, 3, 128, 2, 700_000, 1, 3, 0, 1), (64, 16, 256, 4, 4 << 30, 0, 8, 1, 1)]:
            builder.set_tuning(ooc.Tuning(small_vol, lpl, block, cps, budget, graphs, ept, pdl, persistent))
            for r, w in zip(builder.build_batch_device(meshes, params), want):
                assert not octree.diff(r.tree, w)
    finally:
        builder.set_tuning(old)


def test_persistent_phase_walks_the_tasks_that_do_not_fit_its_queue():
    # Three flat triangles across a 512^2 face: 262,144 lines each, 8,192 warp tasks at
    # one line per lane, 24,576 in all, more than the 4,096 entries a fresh context's task
    # queue holds, so their chunk walks them itself.  Their boxes are two voxels deep, so
    # the oracle tests few candidates.
    rng = np.random.default_rng(12)
    tris = []
    for k in range(3):
        z = 0.1 + 0.3 * k + rng.uniform(0, 0.001, size=3)
        tris.append([0.0005, 0.0005, z[0], 0.9995, 0.0007, z[1], 0.0006, 0.9993, z[2]])
    tris = np.asarray(tris, dtype=np.float32)
    want = octree.Octree(512, *pyoracle.build(tris, 512, 2048, color="model")[:2])
    with ooc.Builder(0) as fresh:  # no tasks seen yet: the smallest queue
        fresh.set_tuning(ooc.Tuning(64, 1, 256, 4, 4 << 30, 0, 8, 1, 1))
        for _ in range(2):  # the second build has the larger queue the first one sized
            got = fresh.build_batch_device([tris], [make_params(512, 2048, geometry_only=True)])[0]
            assert not octree.diff(got.tree, want)


def test_autotune_keeps_a_valid_tuning(builder):
    meshes = [tri.soup_tris(3000, 256, seed=s, sigma=1.0, n_spheres=2, payload=bool(s % 2)) for s in range(6)]
    params = [make_params(256, 2048, geometry_only=not bool(s % 2)) for s in range(6)]
    old = builder.tuning()
    try:
        t = builder.autotune(meshes, params)
        assert 1 <= t.small_vol <= 64 and 1 <= t.lines_per_lane <= 64 and t.large_block in (64, 128, 256)
        assert builder.tuning().as_dict() == t.as_dict()
        for r, (m, p) in zip(builder.build_batch(meshes, params), zip(meshes, params)):
            assert not octree.diff(r.tree, builder.build(m, p).tree)
    finally:
        builder.set_tuning(old)
