"""GPU path against the CPU oracle on the same seeded inputs (through the C ABI).

Bar: node files byte-identical; data files identical field by field with FP32
compared by bit pattern, except that NaN equals NaN (NaN bits differ between
x86-64, AArch64 and the GPU even for the reference itself).
"""
import numpy as np
import pytest

import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu


def run_both(builder, tris, N, limit=2048, color="model", levels=False, bbox_max=(1.0, 1.0, 1.0)):
    binary = tris.shape[1] == 9
    prm = make_params(N, limit, geometry_only=binary, color=color, levels=levels, bbox_max=bbox_max)
    got = builder.build(tris, prm)
    nodes, data, info = pyoracle.build(tris, N, limit, color=color, levels=levels, bbox_max=bbox_max)
    want = octree.Octree(N, nodes, data)
    return got, want, info


def assert_same(got, want, info):
    d = octree.diff(got.tree, want)
    assert not d, "\n".join(d)
    assert got.info["n_filled"] == info["n_filled"]
    assert got.info["n_partitions"] == info["n_partitions"]
    assert got.info["n_nodes"] == want.nodes.shape[0]
    assert got.info["n_data"] == want.data.shape[0]


@pytest.mark.parametrize("N", [1, 2, 8, 64, 256])
def test_icosphere_binary(builder, N):
    t = tri.icosphere_tris(4)
    assert_same(*run_both(builder, t, N))


@pytest.mark.parametrize("N,limit", [(256, 2), (512, 2), (128, 2048)])
def test_partitions_binary(builder, N, limit):
    t = tri.random_tris(3000, 11, False, lo=-0.05, hi=1.05, max_edge=0.15)
    got, want, info = run_both(builder, t, N, limit)
    assert_same(got, want, info)


@pytest.mark.parametrize("color", ["model", "fixed", "linear", "normal"])
@pytest.mark.parametrize("levels", [False, True])
def test_payload_modes(builder, color, levels):
    t = tri.icosphere_tris(3, payload=True)
    assert_same(*run_both(builder, t, 64, color=color, levels=levels))


def test_binary_levels(builder):
    t = tri.icosphere_tris(3)
    assert_same(*run_both(builder, t, 64, levels=True))


@pytest.mark.parametrize("levels", [False, True])
def test_payload_partitions(builder, levels):
    t = tri.random_tris(2000, 5, True, lo=-0.1, hi=1.1, max_edge=0.1)
    assert_same(*run_both(builder, t, 256, limit=2, levels=levels))


def test_large_triangles(builder):
    # bounding boxes up to the whole grid: the warp-task path
    t = tri.random_tris(40, 3, True, lo=0.0, hi=1.0, max_edge=1.5)
    assert_same(*run_both(builder, t, 128))


def _large_plane_cases(seed):
    """Large triangles whose lines along the walk axis stress the run search: planes exactly
    on voxel faces and axis-aligned, nearly parallel to an axis, tiny normal components,
    collinear and zero-area triangles spanning the grid."""
    rng = np.random.default_rng(seed)
    out = []
    g = np.float32(1.0 / 64)
    for axis in range(3):  # axis-aligned planes on and between voxel faces
        for c in (0.0, 17 * g, 17.5 * g, 1.0 - g, 1.0):
            v = rng.random((3, 3), dtype=np.float32)
            v[:, axis] = c
            out.append(v.reshape(9))
    for _ in range(60):  # nearly parallel to an axis: one normal component tiny
        v = rng.random((3, 3), dtype=np.float32)
        axis = int(rng.integers(0, 3))
        v[1, axis] = v[0, axis] + np.float32(rng.choice([1e-7, 1e-5, 1e-3, -1e-6]))
        v[2, axis] = v[0, axis] + np.float32(rng.choice([0.0, 2e-7, -1e-4]))
        out.append(v.reshape(9))
    for _ in range(40):  # generic large triangles with grid-aligned vertices
        out.append((rng.integers(0, 65, size=9) * g).astype(np.float32))
    a = rng.random((20, 3), dtype=np.float32)
    b = rng.random((20, 3), dtype=np.float32)
    out.extend(np.stack([a, (a + b) * np.float32(0.5), b], 1).reshape(20, 9))  # collinear, long
    out.extend(np.stack([a, a, b], 1).reshape(20, 9))
    return np.asarray(out, dtype=np.float32)


@pytest.mark.parametrize("scale", [1.0, 1e-3, 1e4])
def test_large_plane_runs(builder, scale):
    t = _large_plane_cases(17) * np.float32(scale)
    s = float(np.float32(scale))
    assert_same(*run_both(builder, t, 64, bbox_max=(s, s, s)))
    rng = np.random.default_rng(3)
    col = rng.random((t.shape[0], 12), dtype=np.float32)
    tp = np.concatenate([t, col], 1).astype(np.float32)
    assert_same(*run_both(builder, tp, 128, limit=1, levels=True, bbox_max=(s, s, s)))


def test_overlapping_first_writer(builder):
    # many coincident triangles with different colours: the payload must come
    # from the first one in stream order (voxelizer.cpp:263)
    base = tri.random_tris(50, 9, True, max_edge=0.2)
    rng = np.random.default_rng(4)
    reps = np.repeat(base, 4, axis=0)
    reps[:, 12:21] = rng.random((reps.shape[0], 9), dtype=np.float32)
    assert_same(*run_both(builder, reps, 64, levels=True))


def test_degenerate_triangles(builder):
    rng = np.random.default_rng(8)
    a = rng.random((100, 3), dtype=np.float32)
    b = rng.random((100, 3), dtype=np.float32)
    pts = np.stack([a, a, b], 1).reshape(100, 9)             # two equal vertices
    mid = ((a + b) * np.float32(0.5)).astype(np.float32)
    line = np.stack([a, mid, b], 1).reshape(100, 9)          # collinear
    same = np.stack([a, a, a], 1).reshape(100, 9)            # a point
    t = np.concatenate([pts, line, same], 0).astype(np.float32)
    assert_same(*run_both(builder, t, 64))
    col = rng.random((300, 12), dtype=np.float32)
    tp = np.concatenate([t, col[:, :3], col[:, 3:]], 1).astype(np.float32)
    assert_same(*run_both(builder, tp, 32, levels=True))


def test_grid_aligned_vertices(builder):
    # vertices exactly on voxel faces: truncation puts max in the next cell
    g = np.arange(0, 17, dtype=np.float32) / np.float32(16)
    rng = np.random.default_rng(12)
    idx = rng.integers(0, 17, size=(500, 9))
    t = g[idx].astype(np.float32)
    assert_same(*run_both(builder, t, 16))
    assert_same(*run_both(builder, t, 64, limit=2048))


def test_empty_mesh(builder):
    t = np.zeros((0, 9), np.float32)
    assert_same(*run_both(builder, t, 32))
    tp = np.zeros((0, 21), np.float32)
    assert_same(*run_both(builder, tp, 32, levels=True))


def test_outside_grid(builder):
    # triangles partly or fully outside [0, 1]^3 are clamped to the partition
    t = tri.random_tris(1000, 21, True, lo=-0.4, hi=1.4, max_edge=0.3)
    assert_same(*run_both(builder, t, 64))
    assert_same(*run_both(builder, tri.to_binary(t), 256, limit=2))


def test_non_unit_bbox(builder):
    t = tri.random_tris(800, 31, False, lo=0.0, hi=3.0, max_edge=0.5)
    assert_same(*run_both(builder, t, 128, bbox_max=(3.0, 3.0, 3.0)))


@pytest.mark.parametrize("payload,N,limit,levels", [(False, 128, 2048, False), (True, 64, 2048, True),
                                                    (False, 256, 2, True), (True, 256, 2, False)])
def test_device_resident_build(builder, payload, N, limit, levels):
    """ooc_build_device keeps the octree on the GPU; copied back it equals the host-API result."""
    torch = pytest.importorskip("torch")
    t = tri.random_tris(1500, 77, payload, lo=-0.05, hi=1.05, max_edge=0.15)
    prm = make_params(N, limit, geometry_only=not payload, levels=levels)
    d = torch.from_numpy(t).cuda()
    for _ in range(2):  # the second call reuses every buffer
        info = builder.build_device(d.data_ptr(), t.shape[0], prm)
        dev = builder.result_tree(N, info["n_nodes"], info["n_data"])
        host = builder.build(t, prm)
        diffs = octree.diff(dev, host.tree)
        assert not diffs, "\n".join(diffs)
    nodes, data, _ = pyoracle.build(t, N, limit, levels=levels)
    assert not octree.diff(dev, octree.Octree(N, nodes, data))


def test_soup_64_partitions(builder):
    """Configuration 3 scaled down: skewed log-normal soup plus sphere-surface triangles,
    gridsize 1024 with -l 16 (64 partitions of 256^3)."""
    t = tri.soup_tris(400_000, 1024, seed=33, sigma=1.0, n_spheres=50)
    got, want, info = run_both(builder, t, 1024, limit=16)
    assert info["n_partitions"] == 64
    assert_same(got, want, info)


# Stripes of 512^3 voxels and more keep their leaf level zero between builds, mark the
# blocks the voxelization writes and scan the leaf level by groups of blocks; these cases
# put that path against the oracle.
@pytest.mark.parametrize("N,sub,payload,levels", [(512, 4, False, False), (1024, 4, False, False),
                                                  (512, 4, True, True), (1024, 5, True, False)])
def test_marked_leaf_levels(builder, N, sub, payload, levels):
    t = tri.icosphere_tris(sub, payload=payload)
    assert_same(*run_both(builder, t, N, levels=levels))


def test_marked_soup_payload(builder):
    t = tri.soup_tris(100_000, 1024, seed=41, sigma=1.0, n_spheres=20, payload=True)
    assert_same(*run_both(builder, t, 1024))


def test_marked_eight_stripes(builder):
    """Gridsize 2048 at -l 2048: eight partitions of 1024^3, one sub-batch."""
    t = tri.icosphere_tris(3, radius=0.2)
    got, want, info = run_both(builder, t, 2048)
    assert info["n_partitions"] == 8
    assert_same(got, want, info)


def test_marked_and_unmarked_in_one_batch(builder):
    meshes = [tri.soup_tris(20_000, 1024, seed=43, sigma=1.0, n_spheres=5, payload=True),
              tri.icosphere_tris(3, seed=2),
              tri.icosphere_tris(4, seed=3, payload=True),
              tri.random_tris(2000, 44, False, max_edge=0.1)]
    sizes = [1024, 64, 512, 256]
    params = [make_params(N, 2048, geometry_only=t.shape[1] == 9) for t, N in zip(meshes, sizes)]
    got = builder.build_batch(meshes, params)
    for t, N, g in zip(meshes, sizes, got):
        nodes, data, _ = pyoracle.build(t, N, 2048)
        d = octree.diff(g.tree, octree.Octree(N, nodes, data))
        assert not d, "\n".join(d)


@pytest.mark.parametrize("payload,N,T", [(True, 128, 450_000), (False, 512, 1_000_000)])
def test_upload_in_pieces(builder, payload, N, T):
    """Host meshes of more than 32 MB in one partition go up in 16 MB pieces, each
    voxelized as soon as it is on the device."""
    t = tri.soup_tris(T, N, seed=45, sigma=0.5 if N == 512 else 1.0, n_spheres=30, payload=payload)
    assert t.nbytes > 32 << 20
    assert_same(*run_both(builder, t, N))

