"""The file formats on the path, without a GPU: .tri/.tridata written and read back
(tri_tools.h:75-127), the .octree header text (octree_io.h:74-83), the node and data
records (octree_io.h:48-66), and the structural differ and digest used by the parity tests."""
import os

import numpy as np
import pytest

import pyoracle
from ooc_svo_builder_gb300 import octree, tri


@pytest.mark.parametrize("payload", [False, True])
def test_tri_round_trip(tmp_path, payload):
    t = tri.random_tris(57, 3, payload, lo=-0.2, hi=1.3)
    path = tri.write_tri(str(tmp_path / "m"), t, bbox_min=(-0.25, 0, 0), bbox_max=(1.5, 1, 1.125))
    h, back = tri.read_tri(path)
    assert (h.n_triangles, h.geo_only, h.version) == (57, 0 if payload else 1, 1)
    assert h.bbox_min == (-0.25, 0.0, 0.0) and h.bbox_max == (1.5, 1.0, 1.125)
    assert back.dtype == np.float32 and np.array_equal(back.view(np.uint32), t.view(np.uint32))
    assert os.path.getsize(str(tmp_path / "m.tridata")) == 57 * (84 if payload else 36)


def test_tri_header_text_follows_the_reference_writer(tmp_path):
    # writeTriHeader (tri_tools.h:118-127): two spaces after "bbox"
    tri.write_tri(str(tmp_path / "m"), tri.random_tris(4, 1, False))
    assert open(str(tmp_path / "m.tri")).read() == "#tri 1\nntriangles 4\ngeo_only 1\nbbox  0 0 0 1 1 1\nEND\n"


def test_tri_header_unknown_words_skip_their_line(tmp_path):
    p = str(tmp_path / "a.tri")
    with open(p, "w") as f:
        f.write("#tri 1\nntriangles 7\nnote geo_only 1 bbox 5 5 5 6 6 6\ngeo_only 0\nbbox 0 0 0 2 2 2\nEND\n")
    h = tri.read_tri_header(p)
    assert (h.n_triangles, h.geo_only, h.bbox_max) == (7, 0, (2.0, 2.0, 2.0))
    with open(p, "w") as f:
        f.write("#tri 1\nntriangles 7\n")
    with pytest.raises(ValueError):
        tri.read_tri_header(p)
    with open(p, "w") as f:
        f.write("#triangles 1\nEND\n")
    with pytest.raises(ValueError):
        tri.read_tri_header(p)


def small_tree(payload=True, levels=False):
    t = tri.random_tris(300, 21, payload, max_edge=0.2)
    nodes, data, info = pyoracle.build(t, 32, 2048, levels=levels)
    return octree.Octree(32, nodes, data), info


def test_octree_files_round_trip(tmp_path):
    tree, info = small_tree()
    base = str(tmp_path / "m32_1")
    octree.write_octree(base, tree)
    # writeOctreeHeader (octree_io.h:74-83)
    assert open(base + ".octree").read() == "#octreeheader 1\ngridlength 32\nn_nodes %d\nn_data %d\nEND\n" % (
        info["n_nodes"], info["n_data"])
    assert os.path.getsize(base + ".octreenodes") == 24 * info["n_nodes"]
    assert os.path.getsize(base + ".octreedata") == 32 * info["n_data"]
    back = octree.read_octree(base)
    assert not octree.diff(back, tree)
    assert octree.parse_header(base + ".octree")["n_nodes"] == info["n_nodes"]


def test_read_octree_rejects_counts_that_disagree_with_the_header(tmp_path):
    tree, _ = small_tree()
    base = str(tmp_path / "m")
    octree.write_octree(base, tree)
    with open(base + ".octreenodes", "ab") as f:
        f.write(bytes(24))
    with pytest.raises(ValueError):
        octree.read_octree(base)


def test_leaves_walk_finds_every_set_voxel_in_morton_order():
    tree, info = small_tree()
    mortons, data_idx = octree.leaves(tree)
    assert mortons.size == info["n_filled"]
    assert np.all(np.diff(mortons.astype(np.int64)) > 0)
    # payload leaves point at their data records, whose Morton codes agree
    assert np.array_equal(tree.data["morton"][data_idx], mortons)


def test_diff_and_digest_see_any_change_but_not_nan_bits():
    tree, _ = small_tree(levels=True)
    nodes, data = tree.nodes.copy(), tree.data.copy()
    same = octree.Octree(32, nodes, data)
    assert not octree.diff(tree, same) and octree.digest(tree) == octree.digest(same)
    # another NaN bit pattern in a colour: equal for both
    data2 = data.copy()
    data2["color"][1, 0] = np.float32(np.nan)
    data3 = data.copy()
    data3["color"][1, 0] = np.array([0xFFC00001], dtype=np.uint32).view(np.float32)[0]
    a, b = octree.Octree(32, nodes, data2), octree.Octree(32, nodes, data3)
    assert not octree.diff(a, b) and octree.digest(a) == octree.digest(b)
    # a moved child pointer or a flipped payload bit: both see it
    nodes4 = nodes.copy()
    inner = np.nonzero((nodes4["children_offset"] != -1).any(axis=1))[0][0]
    nodes4["children_base"][inner] += 1
    c = octree.Octree(32, nodes4, data)
    assert octree.diff(tree, c) and octree.digest(tree) != octree.digest(c)
    data5 = data.copy()
    data5["normal"][1, 2] = np.nextafter(data5["normal"][1, 2], np.float32(2))
    e = octree.Octree(32, nodes, data5)
    assert octree.diff(tree, e) and octree.digest(tree) != octree.digest(e)


def test_stream_digest_equals_whole_digest(tmp_path):
    """octree.StreamDigest over pieces cut anywhere (inside records too) and file_digest
    over chunked reads give octree.digest of the whole tree, NaNs made canonical."""
    rng = np.random.default_rng(7)
    nodes = np.frombuffer(rng.integers(0, 255, 1001 * 24, dtype=np.uint8).tobytes(), octree.NODE_DTYPE)
    data = np.zeros(777, octree.DATA_DTYPE)
    data["morton"] = rng.integers(0, 1 << 40, 777)
    data["color"] = rng.random((777, 3))
    data["color"][5, 1] = np.nan
    data["normal"][9, 2] = np.float32(np.nan)
    tree = octree.Octree(64, nodes, data)
    want = octree.digest(tree)
    d = octree.StreamDigest(64)
    nb, db = nodes.tobytes(), data.tobytes()
    for i in range(0, len(nb), 1000):
        d.update(0, nb[i:i + 1000])
    for i in range(0, len(db), 999):
        d.update(1, db[i:i + 999])
    assert d.result() == want and d.nan_fields == 2
    base = str(tmp_path / "t")
    octree.write_octree(base, tree)
    assert octree.file_digest(base, chunk=4096) == want
