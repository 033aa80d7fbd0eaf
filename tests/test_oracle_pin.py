"""Pin the CPU oracle: against the golden fixtures made by the reference itself, and
(where the reference sources are present) against the reference build on fresh seeds."""
import os
import subprocess

import numpy as np
import pytest

import golden_cases
import pyoracle
from ooc_svo_builder_gb300 import octree, tri

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", golden_cases.names())
def test_oracle_matches_golden(name):
    tris, meta, want = golden_cases.load(name)
    nodes, data, info = pyoracle.build(tris, meta["s"], meta.get("l", 2048), color=meta.get("c", "model"),
                                       levels=meta.get("levels", False))
    got = octree.Octree(meta["s"], nodes, data)
    d = octree.diff(got, want)
    assert not d, "\n".join(d)
    assert info["n_partitions"] == meta["n_partitions"]
    assert info["n_filled"] == meta["n_filled"]
    assert octree.header_text(meta["s"], nodes.shape[0], data.shape[0]) == meta["header"]


def test_golden_set_is_present():
    assert len(golden_cases.names()) >= 15


def _reference_available(binary):
    return os.path.exists(pyoracle.ref_binary(binary))


def _run_ref(tmp_path, tris, N, limit, extra=()):
    base = str(tmp_path / "m")
    tri.write_tri(base, tris)
    exe = pyoracle.ref_binary(tris.shape[1] == 9)
    out = subprocess.run([exe, "-f", base + ".tri", "-s", str(N), "-l", str(limit), *extra], cwd=str(tmp_path),
                         stdout=subprocess.PIPE, text=True, check=True).stdout
    P = int([ln for ln in out.splitlines() if ln.startswith("Partitioning data into")][0].split()[3])
    return octree.read_octree(base + "%d_%d" % (N, P))


@pytest.mark.parametrize("seed,N,limit,payload,extra", [
    (201, 128, 2048, False, ()), (202, 256, 2, False, ()), (203, 64, 2048, True, ()),
    (204, 64, 2048, True, ("-levels",)), (205, 128, 2, True, ("-c", "linear")),
    (206, 64, 2048, True, ("-c", "normal", "-levels")), (207, 512, 2, False, ("-levels",)),
])
def test_oracle_matches_reference_build(tmp_path, seed, N, limit, payload, extra):
    if not _reference_available(not payload):
        pytest.skip("reference build not present (make -C oracle ref needs the reference sources)")
    tris = tri.random_tris(1500, seed, payload, lo=-0.1, hi=1.1, max_edge=0.2)
    want = _run_ref(tmp_path, tris, N, limit, extra)
    color = extra[extra.index("-c") + 1] if "-c" in extra else "model"
    nodes, data, _ = pyoracle.build(tris, N, limit, color=color, levels="-levels" in extra)
    d = octree.diff(octree.Octree(N, nodes, data), want)
    assert not d, "\n".join(d)


def test_reference_optimisation_levels_agree(tmp_path):
    """The reference has undefined behaviour in its uint_fast32_t& casts; -O0 and the
    recipe's -O3 -fno-strict-aliasing must give the same octree."""
    from ooc_svo_builder_gb300 import build as recipe
    if not (recipe.reference_present() and _reference_available(True)):
        pytest.skip("reference sources not present")
    recipe.build_reference("ref-O0")
    exe = os.path.join(ROOT, "oracle", "_ref", "svo_builder_binary_O0")
    tris = tri.random_tris(800, 301, False, lo=-0.1, hi=1.1, max_edge=0.2)
    a = _run_ref(tmp_path, tris, 256, 2)
    base = str(tmp_path / "m")
    subprocess.run([exe, "-f", base + ".tri", "-s", "256", "-l", "2"], cwd=str(tmp_path), stdout=subprocess.PIPE,
                   check=True)
    b = octree.read_octree(base + "256_8")
    assert not octree.diff(a, b)


@pytest.mark.parametrize("payload", [False, True])
def test_reference_partition_invariance_inside_the_grid(tmp_path, payload):
    """For triangles inside the grid the reference gives the same octree with one partition
    (-l 2048) and with eight (-l 2): its partition box filter (partitioner.cpp:54-61) keeps
    every triangle a partition's voxel test can set a voxel for."""
    if not _reference_available(not payload):
        pytest.skip("reference build not present (make -C oracle ref needs the reference sources)")
    tris = tri.random_tris(1500, 208, payload, lo=0.02, hi=0.98, max_edge=0.2)
    (tmp_path / "one").mkdir()
    (tmp_path / "eight").mkdir()
    d = octree.diff(_run_ref(tmp_path / "one", tris, 256, 2048), _run_ref(tmp_path / "eight", tris, 256, 2))
    assert not d, "\n".join(d)


def test_reference_outside_triangles_depend_on_partitions():
    """Triangles just outside the grid are where the partition count shows.  With one
    partition their clamped box (voxelizer.cpp:199-204) puts candidates on the grid's outer
    layer, and the Schwarz-Seidel test, which has no bounding-box axis of its own, passes some
    of them.  With eight partitions the box filter drops those triangles first.  Every voxel
    that only one partition count sets lies on the grid's faces.  The oracle follows the
    reference in both, which test_oracle_matches_reference_build pins; the GPU follows the
    oracle."""
    t = tri.random_tris(1500, 208, True, lo=-0.1, hi=1.1, max_edge=0.2)
    _, d1, _ = pyoracle.build(t, 256, 2048)
    _, d8, i8 = pyoracle.build(t, 256, 2)
    assert i8["n_partitions"] == 8
    one, eight = set(d1["morton"][1:].tolist()), set(d8["morton"][1:].tolist())
    assert eight <= one and one != eight
    for m in one - eight:
        xyz = [sum(((m >> (3 * i + a)) & 1) << i for i in range(21)) for a in range(3)]
        assert min(xyz) == 0 or max(xyz) == 255, xyz


@pytest.mark.parametrize("name", sorted(golden_cases.FULLSIZE))
def test_oracle_matches_reference_at_full_size(name):
    """Configurations 1 and 2 (also with -levels) at full size: the oracle's octree has the
    digest the reference build gave on the same mesh (recorded by
    tests/golden/make_fullsize_golden.py)."""
    w, want = golden_cases.FULLSIZE[name], golden_cases.fullsize_reference()[name]
    t = w["make"]()
    if golden_cases.input_sha256(t) != want["input_sha256"]:
        pytest.skip("the mesh generator gives other bytes on this host")
    nodes, data, info = pyoracle.build(t, w["gridsize"], w["limit"], color=w["color"], levels=w.get("levels", False))
    assert octree.digest(octree.Octree(w["gridsize"], nodes, data)) == want["digest"]
    assert info["n_filled"] == want["n_filled"] and info["n_partitions"] == want["n_partitions"]
    assert octree.header_text(w["gridsize"], nodes.shape[0], data.shape[0]) == want["header"]


@pytest.mark.parametrize("name", sorted(golden_cases.STREAMS))
def test_oracle_matches_reference_on_stream_samples(name):
    """The first meshes of the configuration-4 and -5 streams: the oracle gives the reference's
    digest.  Where the reference's output is undefined (its finalizeTree leaves the tree
    unfinished when the last set voxel is N^3-2), the recorded digest is the oracle's own,
    and the condition is checked to hold."""
    checked = 0
    for (t, N, payload), want in zip(golden_cases.stream_sample(name), golden_cases.stream_samples_reference()[name]):
        if golden_cases.input_sha256(t) != want["input_sha256"]:
            continue
        nodes, data, info = pyoracle.build(t, N, golden_cases.STREAM_LIMIT_MB)
        tree = octree.Octree(N, nodes, data)
        assert info["n_filled"] == want["n_filled"] and info["n_partitions"] == want["n_partitions"]
        if "reference_undefined" in want:
            assert golden_cases.reference_undefined(N, golden_cases.set_voxels(tree, payload))
            assert octree.digest(tree) == want["oracle_digest"]
        else:
            assert octree.digest(tree) == want["digest"]
        checked += 1
    if not checked:
        pytest.skip("the mesh generator gives other bytes on this host")


@pytest.mark.parametrize("i", range(golden_cases.N_SEEDED))
def test_oracle_matches_reference_on_seeded_cases(tmp_path, i):
    """A seeded mix of inputs (inside, outside and on the grid's lattice, sub-voxel, soups,
    spheres) and flags (gridsize 1 to 256, 1 to 64 partitions, every colour mode, -levels):
    the oracle's files are the reference build's, except where the reference's own output
    is undefined, and then that condition must hold."""
    t, N, limit, payload, color, levels, kind = golden_cases.seeded_case(i)
    if not _reference_available(not payload):
        pytest.skip("reference build not present (make -C oracle ref needs the reference sources)")
    extra = (("-c", color) if payload else ()) + (("-levels",) if levels else ())
    want = _run_ref(tmp_path, t, N, limit, extra)
    nodes, data, _ = pyoracle.build(t, N, limit, color=color, levels=levels)
    got = octree.Octree(N, nodes, data)
    if octree.diff(got, want):
        assert golden_cases.reference_undefined(N, golden_cases.set_voxels(got, payload)), kind
