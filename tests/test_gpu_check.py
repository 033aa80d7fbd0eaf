"""The octree check (ooc_check_octree_device, octree_check CLI): builds are well formed, and
copies with one planted defect (changed on the host, then uploaded) are caught."""
import os
import subprocess

import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def check_tree(tree: octree.Octree, binary: bool) -> dict:
    n = torch.from_numpy(tree.nodes.view(np.uint8).copy()).cuda()
    d = torch.from_numpy(tree.data.view(np.uint8).copy()).cuda()
    r = ooc.check_octree_device(n.data_ptr(), tree.nodes.shape[0], d.data_ptr(), tree.data.shape[0],
                                tree.gridlength, binary)
    torch.cuda.synchronize()
    return r


CASES = [
    ("icosphere binary", lambda: tri.icosphere_tris(4, seed=1), 128, 2048, False),
    ("payload levels", lambda: tri.random_tris(1500, 3, True, max_edge=0.2), 64, 2048, True),
    ("payload 8 partitions", lambda: tri.random_tris(2000, 5, True, lo=-0.1, hi=1.1, max_edge=0.1), 256, 2, False),
    ("binary levels 64 partitions", lambda: tri.to_binary(tri.random_tris(800, 7, True, max_edge=0.3)), 256, 1, True),
]


@pytest.mark.parametrize("name,make,N,limit,levels", CASES, ids=[c[0] for c in CASES])
def test_builds_are_well_formed(builder, name, make, N, limit, levels):
    t = make()
    binary = t.shape[1] == 9
    r = builder.build(t, make_params(N, limit, geometry_only=binary, levels=levels))
    c = check_tree(r.tree, binary)
    assert c["errors"] == []
    assert c["n_leaves"] == r.info["n_filled"]
    assert c["max_depth"] == int(np.log2(N))
    assert c["n_leaves"] + c["n_inner"] == r.info["n_nodes"]


def test_planted_defects_are_caught(builder):
    t = tri.random_tris(1500, 11, True, max_edge=0.2)
    tree = builder.build(t, make_params(64, 2048, geometry_only=False)).tree
    assert check_tree(tree, False)["errors"] == []
    inner = np.nonzero((tree.nodes["children_offset"] >= 0).sum(1) >= 2)[0]
    leaf = np.nonzero((tree.nodes["children_offset"] < 0).all(1))[0]

    bad = octree.Octree(tree.gridlength, tree.nodes.copy(), tree.data.copy())
    i = inner[len(inner) // 2]
    ks = np.nonzero(bad.nodes["children_offset"][i] >= 0)[0]
    o = bad.nodes["children_offset"][i].copy()
    o[ks[0]], o[ks[1]] = o[ks[1]], o[ks[0]]  # two children swapped
    bad.nodes["children_offset"][i] = o
    r = check_tree(bad, False)
    assert "child group order" in r["errors"] and r["first_bad"] <= i

    bad = octree.Octree(tree.gridlength, tree.nodes.copy(), tree.data.copy())
    bad.data["morton"][bad.nodes["data"][leaf[3]]] ^= 8  # a voxel's Morton code moved
    assert "payload Morton code" in check_tree(bad, False)["errors"]

    bad = octree.Octree(tree.gridlength, tree.nodes.copy(), tree.data.copy())
    bad.nodes["data"][leaf[5]] = tree.data.shape[0] + 7  # data index past the file
    assert "data index" in check_tree(bad, False)["errors"]

    bad = octree.Octree(tree.gridlength, tree.nodes.copy(), tree.data.copy())
    bad.nodes["children_base"][inner[0]] += 1  # children pointer off by one
    assert check_tree(bad, False)["errors"] != []


def test_octree_check_cli(builder, tmp_path):
    t = tri.icosphere_tris(3, seed=2, payload=True)
    tree = builder.build(t, make_params(64, 2048, geometry_only=False)).tree
    base = str(tmp_path / "ico64_1")
    octree.write_octree(base, tree)
    exe = os.path.join(os.path.dirname(ooc.LIB_PATH), "bin", "octree_check")
    out = subprocess.run([exe, base + ".octree"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "well formed" in out.stdout
    nodes = np.fromfile(base + ".octreenodes", dtype=octree.NODE_DTYPE)
    nodes["data"][0] = 10 ** 9
    nodes.tofile(base + ".octreenodes")
    out = subprocess.run([exe, base + ".octree"], capture_output=True, text=True)
    assert out.returncode == 1 and "data index" in out.stdout
