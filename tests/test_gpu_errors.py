"""Failures made on the host (a sink that refuses bytes, an allocation callback that fails,
invalid parameters): each call returns its status code, and the same context builds the next
mesh correctly afterwards.  No GPU fault is involved."""
import ctypes

import pytest

import pyoracle
import ooc_svo_builder_gb300 as ooc
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def still_builds(builder):
    t = tri.icosphere_tris(3, seed=4, payload=True)
    got = builder.build(t, make_params(64, 2048, geometry_only=False))
    nodes, data, _ = pyoracle.build(t, 64, 2048)
    assert not octree.diff(got.tree, octree.Octree(64, nodes, data))


def test_sink_error_aborts_and_context_recovers(builder):
    t = tri.random_tris(3000, 2, True, max_edge=0.2)
    calls = {"n": 0}

    def refuse(user, kind, ptr, n):
        calls["n"] += 1
        return 1 if calls["n"] >= 2 else 0  # the second piece is refused

    with pytest.raises(ooc.OocError) as e:
        builder.build_ptr(t.ctypes.data, t.shape[0], make_params(128, 2048, geometry_only=False), ooc.SINK(refuse))
    assert e.value.code == 5  # OOC_ERR_SINK
    assert "sink" in str(e.value)
    still_builds(builder)


def test_failing_allocation_aborts_batch_and_context_recovers(builder):
    meshes = [tri.random_tris(500, 10 + i, i % 2 == 1, max_edge=0.2) for i in range(6)]
    params = [make_params(128, 2048, geometry_only=(i % 2 == 0)) for i in range(6)]
    arr, keep = builder._mesh_array(meshes, params)
    buf = torch.empty(64 << 20, dtype=torch.uint8, device="cuda")
    used = {"off": 0, "calls": []}

    def alloc(user, mesh, nb, db, stream, pn, pd):
        used["calls"].append(mesh)
        if mesh == 3:
            return 1  # this mesh cannot get memory
        n = (nb + 255) // 256 * 256
        pn[0] = buf.data_ptr() + used["off"]
        pd[0] = buf.data_ptr() + used["off"] + n
        used["off"] += n + (db + 255) // 256 * 256
        return 0

    infos = (ooc.BuildInfo * 6)()
    cb = ooc.ALLOC(alloc)
    rc = builder.lib.ooc_build_batch_device(builder.h, arr, 6, ctypes.cast(cb, ctypes.c_void_p), None, None, infos)
    assert rc == 2  # OOC_ERR_OOM
    assert used["calls"] == [0, 1, 2, 3]  # asked in mesh order, stopped at the failure
    still_builds(builder)
    assert len(builder.build_batch_device(meshes, params)) == 6


def test_failure_after_voxelization_leaves_no_bits_behind(builder):
    """A batch whose allocation fails after its voxelization (512^3 stripes, whose leaf levels
    are kept zero between builds) must not leak set bits into the next build."""
    meshes = [tri.icosphere_tris(4, seed=5 + i, payload=True) for i in range(2)]
    params = [make_params(512, 2048, geometry_only=False) for _ in range(2)]
    arr, keep = builder._mesh_array(meshes, params)
    infos = (ooc.BuildInfo * 2)()
    cb = ooc.ALLOC(lambda user, mesh, nb, db, stream, pn, pd: 1)
    rc = builder.lib.ooc_build_batch_device(builder.h, arr, 2, ctypes.cast(cb, ctypes.c_void_p), None, None, infos)
    assert rc == 2  # OOC_ERR_OOM
    t = tri.icosphere_tris(3, seed=9, payload=True)  # a different, smaller surface in the same stripe
    got = builder.build(t, make_params(512, 2048, geometry_only=False))
    nodes, data, _ = pyoracle.build(t, 512, 2048)
    assert not octree.diff(got.tree, octree.Octree(512, nodes, data))


def test_ready_callback_error_aborts(builder):
    meshes = [tri.random_tris(300, 20 + i, False, max_edge=0.1) for i in range(3)]
    params = [make_params(64, 2048) for _ in range(3)]
    arr, keep = builder._mesh_array(meshes, params)
    buf = torch.empty(16 << 20, dtype=torch.uint8, device="cuda")
    arena = ooc.DeviceArena(buf.data_ptr(), buf.numel(), 0)
    infos = (ooc.BuildInfo * 3)()
    fn = ctypes.cast(builder.lib.ooc_arena_alloc, ctypes.c_void_p)
    ready = ooc.READY(lambda user, mesh: 1)
    # the arena allocator takes the arena as user data; the ready callback refuses the first mesh
    rc = builder.lib.ooc_build_batch_device(builder.h, arr, 3, fn, ctypes.cast(ready, ctypes.c_void_p),
                                            ctypes.byref(arena), infos)
    assert rc == 5  # OOC_ERR_SINK
    still_builds(builder)


@pytest.mark.parametrize("field,value", [("gridsize", 3), ("gridsize", 0), ("memory_limit_mb", 0),
                                         ("color_mode", 9), ("reserved", 1)])
def test_invalid_parameters(builder, field, value):
    p = make_params(64, 2048, geometry_only=False)
    setattr(p, field, value)
    t = tri.random_tris(10, 1, True)
    with pytest.raises(ooc.OocError) as e:
        builder.build(t, p)
    assert e.value.code == 1  # OOC_ERR_INVALID
    still_builds(builder)


def test_file_errors_name_the_file(builder, tmp_path):
    """ooc_build_files: a missing header and a .tridata shorter than its header's triangle
    count fail with OOC_ERR_IO and a message naming the file; no device work is left behind."""
    p = make_params(64, 2048, geometry_only=False)
    with pytest.raises(ooc.OocError) as e:
        builder.build_files(str(tmp_path / "absent.tri"), p)
    assert e.value.code == 4 and "absent.tri does not exist" in str(e.value)
    base = str(tmp_path / "short")
    tri.write_tri(base, tri.random_tris(100, 3, True))
    with open(base + ".tridata", "r+b") as f:
        f.truncate(84 * 60)
    with pytest.raises(ooc.OocError) as e:
        builder.build_files(base + ".tri", p)
    assert e.value.code == 4 and "short read of " + base + ".tridata" in str(e.value)
    still_builds(builder)
