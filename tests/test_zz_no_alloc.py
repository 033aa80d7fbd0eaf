"""ooc_voxelize_occupancy_noalloc: the occupancy pass for callers that cannot allocate GPU memory.

Such callers (code running under stream capture, engines that pre-reserve all
device memory, latency-critical loops) pass inputs and outputs; the entry point's
scratch is a fixed array inside the library.  These tests call it through the C
ABI and compare its bitfield with the voxels of the octree that the regular
entry point (ooc_build) produces for the same triangles, bit for bit, on two
calls in a row.  The file sorts last so that a run stopping at the first failure
has already run every other test.
"""
import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc
from ooc_svo_builder_gb300 import octree, tri

pytestmark = pytest.mark.gpu


def occupancy_from_octree(tree, N):
    """Morton-ordered occupancy bitfield (u32 words) of the octree's leaves."""
    words = max(1, N ** 3 // 32)
    bits = np.zeros(words, dtype=np.uint32)
    m, _ = octree.leaves(tree)
    m = m.astype(np.int64)
    np.bitwise_or.at(bits, m >> 5, (np.uint32(1) << (m & 31).astype(np.uint32)))
    return bits


def noalloc_occupancy(torch, tris, N, payload):
    prm = ooc.make_params(N, 2048, geometry_only=not payload)
    d_tris = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    words = max(1, N ** 3 // 32)
    out = torch.full((words,), -1, dtype=torch.int32, device="cuda")  # garbage the call must clear
    rc = ooc.voxelize_occupancy_noalloc(prm, d_tris.data_ptr(), tris.shape[0], out.data_ptr(), words)
    torch.cuda.synchronize()
    assert rc == ooc.OOC_OK, ooc.ERRORS.get(rc, rc)
    return out.cpu().numpy().view(np.uint32)


def regular_occupancy(tris, N, payload):
    with ooc.Builder(0) as b:
        res = b.build(tris, ooc.make_params(N, 2048, geometry_only=not payload))
    return occupancy_from_octree(res.tree, N)


def test_noalloc_matches_regular_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    cases = [
        (tri.icosphere_tris(4), 128, False),
        (tri.random_tris(3000, 41, True, lo=-0.1, hi=1.1, max_edge=0.6), 64, True),
    ]
    for tris, N, payload in cases:  # two calls in a row; the second reuses the scratch of the first
        got = noalloc_occupancy(torch, tris, N, payload)
        want = regular_occupancy(tris, N, payload)
        assert got.shape == want.shape
        assert np.array_equal(got, want), "occupancy differs in %d words" % int((got != want).sum())
        assert int(np.unpackbits(got.view(np.uint8)).sum()) > 0


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    prm = ooc.make_params(64, 2048, geometry_only=True)
    out = torch.zeros(64 ** 3 // 32, dtype=torch.int32, device="cuda")
    tris = torch.zeros((1, 9), dtype=torch.float32, device="cuda")
    rc = ooc.voxelize_occupancy_noalloc(prm, tris.data_ptr(), ooc.NOALLOC_MAX_TRIANGLES + 1, out.data_ptr(),
                                        out.numel())
    assert rc == 6  # OOC_ERR_LIMIT, before any GPU work
    big = ooc.make_params(2 * ooc.NOALLOC_MAX_GRIDSIZE, 1 << 20, geometry_only=True)
    rc = ooc.voxelize_occupancy_noalloc(big, tris.data_ptr(), 1, out.data_ptr(), out.numel())
    assert rc == 6


def test_noalloc_near_its_limits():
    """Gridsize 1024 (the largest it takes) and 1,040,000 triangles (close to its 1,048,576),
    half of them large enough for the large-triangle kernel: the sizes that fill its fixed
    scratch.  The regular build runs in payload mode so that its leaves' Morton codes come
    straight from the data records."""
    torch = pytest.importorskip("torch")
    N = ooc.NOALLOC_MAX_GRIDSIZE
    tris = tri.soup_tris(1_040_000, N, seed=43, sigma=1.0, n_spheres=50, payload=True)
    assert tris.shape[0] <= ooc.NOALLOC_MAX_TRIANGLES
    got = noalloc_occupancy(torch, tris, N, True)
    with ooc.Builder(0) as b:
        res = b.build(tris, ooc.make_params(N, 2048, geometry_only=False))
    m = res.tree.data["morton"][1:].astype(np.int64)
    want = np.zeros(N ** 3 // 32, dtype=np.uint32)
    np.bitwise_or.at(want, m >> 5, (np.uint32(1) << (m & 31).astype(np.uint32)))
    assert int(np.unpackbits(want.view(np.uint8)).sum()) == res.info["n_filled"]
    assert np.array_equal(got, want), "occupancy differs in %d words" % int((got != want).sum())
