"""Full-size configurations.  Configurations 1 and 2 against the oracle run on the same mesh
and against the reference's recorded digests; configuration 3 (20M triangles, N = 4096, 64
partitions; the oracle would take minutes) against the reference's recorded digest, through
the host-output path in one streaming pass, and through properties: the octree check
(structure, leaf count = filled voxels, depth) and the batched path against the plain one."""
import ctypes
import hashlib

import numpy as np
import pytest

import golden_cases
import ooc_svo_builder_gb300 as ooc
import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_check(builder, info, N, binary):
    nodes_ptr, data_ptr = builder.result_device()
    return ooc.check_octree_device(nodes_ptr, info["n_nodes"], data_ptr, info["n_data"], N, binary)


def test_configuration_3_full_size_is_well_formed(builder):
    # svo_builder_binary -s 4096 -l 2048: 20M triangles, 64 partitions, 651M nodes
    t = tri.soup_tris(20_000_000, 4096, seed=3, sigma=1.0)
    d = torch.from_numpy(t).cuda()
    info = builder.build_device(d.data_ptr(), t.shape[0], make_params(4096, 2048, geometry_only=True))
    assert info["n_partitions"] == 64
    c = device_check(builder, info, 4096, True)
    assert c["errors"] == []
    assert c["n_leaves"] == info["n_filled"] > 0
    assert c["max_depth"] == 12
    assert c["n_leaves"] + c["n_inner"] == info["n_nodes"]


@pytest.mark.parametrize("name", sorted(golden_cases.FULLSIZE_LARGE))
def test_configuration_3_full_size_matches_reference(builder, name):
    """svo_builder_binary -s 4096 -l 2048 on the seeded 20M-triangle soup, through ooc_build
    (pinned staging, three sub-batches, host output): the node and data files streamed
    through the sink hash to the digest the reference build recorded (about 16 GB of nodes,
    so they are hashed as they arrive, not collected)."""
    w, want = golden_cases.FULLSIZE_LARGE[name], golden_cases.fullsize_reference()[name]
    t = w["make"]()
    assert golden_cases.input_sha256(t) == want["input_sha256"], "this host's generator gives another mesh"
    dig = octree.StreamDigest(w["gridsize"])

    def sink(user, kind, ptr, n):
        dig.update(kind, (ctypes.c_char * n).from_address(ptr))
        return 0

    cb = ooc.SINK(sink)
    info = builder.build_ptr(t.ctypes.data, t.shape[0], make_params(w["gridsize"], w["limit"], geometry_only=True), cb)
    assert info["n_partitions"] == want["n_partitions"]
    assert info["n_filled"] == want["n_filled"]
    assert dig.result() == want["digest"]


def test_configuration_2_full_size_batch_equals_plain(builder):
    # svo_builder -s 1024 -c model on the 2,093,058-triangle heightfield: the batched call's
    # files hash the same as the plain call's, and the tree is well formed
    t = tri.heightfield_tris(1024, seed=2, payload=True)
    p = make_params(1024, 2048, geometry_only=False)
    plain = builder.build(t, p)
    other = tri.icosphere_tris(3, seed=5, payload=True)
    batch = builder.build_batch([other, t, other], [make_params(64, 2048, geometry_only=False), p,
                                                   make_params(64, 2048, geometry_only=False)])
    h = lambda tree: hashlib.sha256(tree.nodes.tobytes() + tree.data.tobytes()).hexdigest()
    assert h(batch[1].tree) == h(plain.tree)
    d = torch.from_numpy(t).cuda()
    info = builder.build_device(d.data_ptr(), t.shape[0], p)
    c = device_check(builder, info, 1024, False)
    assert c["errors"] == [] and c["n_leaves"] == info["n_filled"] == plain.info["n_filled"]


@pytest.mark.parametrize("name", sorted(golden_cases.FULLSIZE))
def test_full_size_matches_oracle_and_reference(builder, name):
    """Configurations 1 and 2 (also with -levels) at full size through ooc_build: equal to the oracle on the same
    mesh (bit for bit, NaNs aside), and to the reference's recorded digest when this host's
    generator gives the recorded mesh."""
    w, want = golden_cases.FULLSIZE[name], golden_cases.fullsize_reference()[name]
    t = w["make"]()
    levels = w.get("levels", False)
    got = builder.build(t, make_params(w["gridsize"], w["limit"], geometry_only=not w["payload"], color=w["color"],
                                       levels=levels))
    nodes, data, info = pyoracle.build(t, w["gridsize"], w["limit"], color=w["color"], levels=levels)
    d = octree.diff(got.tree, octree.Octree(w["gridsize"], nodes, data))
    assert not d, "\n".join(d)
    assert got.info["n_filled"] == info["n_filled"]
    if golden_cases.input_sha256(t) == want["input_sha256"]:
        assert octree.digest(got.tree) == want["digest"]


@pytest.mark.parametrize("name", sorted(golden_cases.STREAMS))
def test_stream_samples_in_one_batch_match_reference(builder, name):
    """The first meshes of the configuration-4 and -5 streams, built in one ooc_build_batch
    call: each equals the reference's recorded digest (the oracle's where the reference's
    output is undefined), or the oracle on the same mesh when this host's generator gives
    other meshes."""
    sample = golden_cases.stream_sample(name)
    rows = golden_cases.stream_samples_reference()[name]
    params = [make_params(N, golden_cases.STREAM_LIMIT_MB, geometry_only=not payload) for _, N, payload in sample]
    got = builder.build_batch([t for t, _, _ in sample], params)
    for i, ((t, N, payload), want) in enumerate(zip(sample, rows)):
        if golden_cases.input_sha256(t) == want["input_sha256"]:
            assert octree.digest(got[i].tree) == want.get("digest", want.get("oracle_digest")), i
        else:
            nodes, data, _ = pyoracle.build(t, N, golden_cases.STREAM_LIMIT_MB)
            assert not octree.diff(got[i].tree, octree.Octree(N, nodes, data)), i
