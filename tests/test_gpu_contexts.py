"""Contexts used from several host threads at once.

The C ABI's threading contract is one host thread per context and any number of
contexts.  Each context keeps its own launch count and kernel-timing hooks, so two
contexts building at the same time on two threads neither count each other's launches
nor time them.  Both results must still equal the oracle."""
import threading

import pytest

import ooc_svo_builder_gb300 as ooc
import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu

CASES = (
    # (triangles, gridsize, memory limit MB, build kwargs): a payload sphere with -levels
    # at N = 256, and a binary soup at N = 256 split into 8 partitions (-l 2 -> P = 8)
    (lambda: tri.icosphere_tris(4, radius=0.45, jitter=0.002, seed=11, payload=True), 256, 2048, {"levels": True}),
    (lambda: tri.soup_tris(40_000, 256, seed=12, sigma=1.0, n_spheres=20), 256, 2, {}),
)


def _params(t, N, limit, kw):
    return make_params(N, limit, geometry_only=t.shape[1] == 9, **kw)


def test_two_contexts_on_two_threads():
    meshes = [(mk(), N, limit, kw) for mk, N, limit, kw in CASES]
    want = []
    for t, N, limit, kw in meshes:
        nodes, data, _ = pyoracle.build(t, N, limit, **kw)
        want.append(octree.Octree(N, nodes, data))
    with ooc.Builder(0) as a, ooc.Builder(0) as b:
        b.set_kernel_timing("*")
        builders = (a, b)
        alone = []
        for k, (t, N, limit, kw) in enumerate(meshes):
            # twice: a context's first build may launch fewer kernels (the large-triangle
            # task map is built once the context has seen many tasks)
            for _ in range(2):
                got = builders[k].build(t, _params(t, N, limit, kw))
                assert not octree.diff(got.tree, want[k])
            alone.append(builders[k].kernel_launches())
        assert alone[0] > 0 and alone[1] > 0
        timed_alone = set(b.kernel_times())
        assert timed_alone

        rounds = 6
        barrier = threading.Barrier(2)
        errors, counts, timed = [], [[], []], [[], []]

        def run(k):
            t, N, limit, kw = meshes[k]
            p = _params(t, N, limit, kw)
            try:
                for _ in range(rounds):
                    barrier.wait(timeout=60)
                    got = builders[k].build(t, p)
                    d = octree.diff(got.tree, want[k])
                    if d:
                        errors.append("context %d: %s" % (k, d[:3]))
                    counts[k].append(builders[k].kernel_launches())
                    timed[k].append(builders[k].kernel_times())
            except Exception as e:  # reported below, on the test's thread
                errors.append("context %d: %r" % (k, e))
                barrier.abort()

        threads = [threading.Thread(target=run, args=(k,)) for k in range(2)]
        for th in threads:
            th.start()
        for th in threads:
            th.join(timeout=300)
        assert not any(th.is_alive() for th in threads)
        assert not errors, errors
        # each context counted exactly its own launches, as when it ran alone
        assert counts[0] == [alone[0]] * rounds
        assert counts[1] == [alone[1]] * rounds
        # only the context with timing on timed kernels, and only its own launches
        assert all(not kt for kt in timed[0])
        for kt in timed[1]:
            assert set(kt) == timed_alone
            assert sum(n for _, n in kt.values()) == alone[1]
