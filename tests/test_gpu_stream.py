"""Out-of-core builds: meshes whose triangle records exceed the device triangle budget are
read again for every group of partitions and never held in device memory whole, as the
reference streams each partition from its .tripdata file (partitioner.cpp:101-149,
main.cpp:329-345).  A small budget forces the path on small meshes; every result must equal
the oracle (and so the in-core build) byte for byte."""
import os

import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc
import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu


def oracle(t, N, limit, **kw):
    nodes, data, info = pyoracle.build(t, N, limit, **kw)
    return octree.Octree(N, nodes, data), info


CASES = [
    # (name, triangles, gridsize, -l, build kwargs, budget as a fraction of the mesh's bytes)
    ("binary_P8", lambda: tri.soup_tris(30_000, 256, seed=21, sigma=1.0, n_spheres=6), 256, 2, {}, 0.7),
    ("payload_P8_levels", lambda: tri.soup_tris(20_000, 256, seed=22, sigma=1.2, n_spheres=4, payload=True), 256, 2,
     {"levels": True}, 0.6),
    ("binary_P64", lambda: tri.soup_tris(60_000, 512, seed=23, sigma=1.0, n_spheres=10), 512, 2, {}, 0.25),
    ("payload_P64_linear", lambda: tri.icosphere_tris(5, radius=0.45, jitter=0.002, seed=24, payload=True), 512, 2,
     {"color": "linear"}, 0.3),
    # triangles spilling outside the grid: the partition box filter drops some, clamps others
    ("outside_P8", lambda: tri.random_tris(5_000, 25, False, lo=-0.5, hi=1.5, max_edge=0.3), 256, 2, {}, 0.1),
]


@pytest.mark.parametrize("name,make,N,limit,kw,frac", CASES, ids=[c[0] for c in CASES])
def test_streamed_build_equals_oracle(builder, name, make, N, limit, kw, frac):
    t = make()
    want, info = oracle(t, N, limit, **kw)
    builder.set_stream_budget(int(t.nbytes * frac))
    try:
        got = builder.build(t, make_params(N, limit, geometry_only=t.shape[1] == 9, **kw))
        passes = builder.stream_passes()
        tris_per_part, filled = builder.partition_counts()
    finally:
        builder.set_stream_budget(0)
    assert passes >= 3, "not built out of core (%d passes)" % passes  # the count pass and two groups at least
    d = octree.diff(got.tree, want)
    assert not d, "\n".join(d)
    assert got.info["n_filled"] == info["n_filled"]
    assert tris_per_part == [int(v) for v in info["part_tricounts"]]
    assert sum(filled) == info["n_filled"]
    # and the in-core build of the same mesh
    assert builder.stream_passes() == passes
    incore = builder.build(t, make_params(N, limit, geometry_only=t.shape[1] == 9, **kw))
    assert builder.stream_passes() == 0
    assert not octree.diff(incore.tree, want)


def test_streamed_build_from_file(builder, tmp_path):
    """ooc_build_files reads the .tridata again for every group instead of uploading it whole."""
    t = tri.soup_tris(40_000, 512, seed=26, sigma=1.0, n_spheres=8, payload=True)
    path = tri.write_tri(str(tmp_path / "big"), t)
    want, _ = oracle(t, 512, 2, levels=True)
    builder.set_stream_budget(t.nbytes // 4)
    try:
        base, info = builder.build_files(path, make_params(512, 2, geometry_only=False, levels=True))
        passes = builder.stream_passes()
    finally:
        builder.set_stream_budget(0)
    assert passes >= 3
    assert base.endswith("big512_64")
    d = octree.diff(octree.read_octree(base), want)
    assert not d, "\n".join(d)


def test_partition_over_half_the_budget_is_refused(builder):
    t = tri.icosphere_tris(4, radius=0.3, seed=27)
    builder.set_stream_budget(t.nbytes // 8)  # one partition holds more than a sixteenth of the sphere
    try:
        with pytest.raises(ooc.OocError) as e:
            builder.build(t, make_params(256, 2))
    finally:
        builder.set_stream_budget(0)
    assert e.value.code == 6  # OOC_ERR_LIMIT
    assert "device triangle budget" in str(e.value)
    # the context still builds
    got = builder.build(t, make_params(256, 2))
    assert not octree.diff(got.tree, oracle(t, 256, 2)[0])
