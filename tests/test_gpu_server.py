"""Serving loop: requests submitted together run in shared batches, and each
result equals the oracle on that request's mesh and flags (and so the same mesh
built alone with ooc_build), also when a batch fails part-way and its unfinished
requests run again alone."""
import threading
import time

import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc
import pyoracle
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu

COLOR_NAMES = {v: k for k, v in ooc.COLOR_MODES.items()}


def oracle_tree(t, p):
    """The oracle's octree for one request."""
    nodes, data, _ = pyoracle.build(t, int(p.gridsize), int(p.memory_limit_mb), color=COLOR_NAMES[p.color_mode],
                                    levels=bool(p.generate_levels))
    return octree.Octree(int(p.gridsize), nodes, data)


def serve_all(reqs, feed_delay=0.0, stats=None, **server_kw):
    """Submit every request (from a second thread when feed_delay > 0) and poll until all
    are back: (ids, {id: polled result}); `stats` (a dict) receives the server's state
    after the last poll."""
    with ooc.Server(0, **server_kw) as srv:
        ids = [None] * len(reqs)

        def feed():
            for i, (t, p) in enumerate(reqs):
                ids[i] = srv.submit(t, p)
                if feed_delay:
                    time.sleep(feed_delay)

        th = threading.Thread(target=feed)
        th.start()
        if not feed_delay:
            th.join()
        got = {}
        deadline = time.time() + 180
        while len(got) < len(reqs) and time.time() < deadline:
            r = srv.poll(1000)
            if r is not None:
                got[r["id"]] = r
        th.join()
        if stats is not None:
            stats.update(srv.stats())
    return ids, got


def request_mix(seed=9, count=40):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        payload = bool(rng.integers(0, 2))
        N = int(rng.choice([16, 64, 128, 256, 512]))
        limit = 2 if (N >= 256 and rng.random() < 0.4) else 2048
        color = str(rng.choice(["model", "fixed", "linear", "normal"])) if payload else "model"
        levels = bool(rng.integers(0, 2))
        if rng.random() < 0.5:
            t = tri.icosphere_tris(int(rng.integers(1, 5)), radius=float(rng.uniform(0.2, 0.45)), jitter=0.002,
                                   seed=int(rng.integers(0, 1 << 30)), payload=payload)
        else:
            t = tri.soup_tris(int(rng.integers(10, 3000)), N, seed=int(rng.integers(0, 1 << 30)), sigma=1.0,
                              n_spheres=2, payload=payload)
        out.append((t, make_params(N, limit, geometry_only=not payload, color=color, levels=levels)))
    return out


@pytest.fixture(scope="module")
def mix40():
    reqs = request_mix()
    return reqs, [oracle_tree(t, p) for t, p in reqs]


@pytest.fixture(scope="module")
def mix30():
    reqs = request_mix(seed=11, count=30)
    return reqs, [oracle_tree(t, p) for t, p in reqs]


@pytest.mark.parametrize("resident", [False, True], ids=["host", "device"])
def test_results_in_the_mix_equal_oracle(builder, mix40, resident):
    reqs, want = mix40
    ids, got = serve_all(reqs, engines=2, max_batch=16, memory_budget=8 << 30, resident=resident)
    assert len(got) == len(ids)
    assert max(r["batch_size"] for r in got.values()) > 1, "no request shared a batch"
    for k, (rid, w) in enumerate(zip(ids, want)):
        r = got[rid]
        assert r["status"] == 0
        assert r["location"] == (1 if resident else 0)
        d = octree.diff(r["tree"], w)
        assert not d, "request %d: %s" % (k, "\n".join(d))
        assert r["t_submit_us"] <= r["t_start_us"] <= r["t_built_us"] <= r["t_done_us"]
    # and the same mesh built alone through ooc_build
    for k in range(0, len(reqs), 7):
        assert not octree.diff(builder.build(*reqs[k]).tree, want[k])


def test_host_results_from_a_pinned_reserve_equal_oracle(mix40):
    """Host results carved out of a 2 MiB pinned reserve: small results share it (freed
    blocks merge with their neighbours for the next ones), larger ones get blocks pinned
    on demand.  Every result still equals the oracle."""
    reqs, want = mix40
    stats = {}
    ids, got = serve_all(reqs, engines=2, max_batch=16, memory_budget=8 << 30, host_pool_mb=2, stats=stats)
    for k, (rid, w) in enumerate(zip(ids, want)):
        assert got[rid]["status"] == 0, k
        assert not octree.diff(got[rid]["tree"], w), k
    # everything polled and released: the reserve is whole again, nothing is left in flight
    assert stats["pinned_reserve_bytes"] == 2 << 20
    assert stats["pinned_reserve_free_bytes"] == 2 << 20
    assert stats["in_flight_bytes"] == 0 and stats["queued"] == 0 and stats["held"] == 0
    assert stats["pinned_on_demand_allocs"] >= 1  # the larger results


@pytest.mark.parametrize("resident", [False, True], ids=["host", "device"])
def test_arrivals_while_busy_join_later_batches(mix30, resident):
    # a submitting thread keeps adding requests while the engines are running
    reqs, want = mix30
    ids, got = serve_all(reqs, feed_delay=0.002, engines=2, max_batch=8, memory_budget=8 << 30, resident=resident)
    for k, (rid, w) in enumerate(zip(ids, want)):
        assert got[rid]["status"] == 0
        assert not octree.diff(got[rid]["tree"], w), k


@pytest.mark.parametrize("resident", [False, True], ids=["host", "device"])
def test_failed_batch_reruns_its_unfinished_requests_alone(mix40, resident):
    """The first shared batch fails at its third mesh (fault injection on the host: that
    mesh's allocation fails as if out of memory).  The batch's first two requests are
    complete already; every other one runs again alone.  All results still equal the
    oracle."""
    reqs, want = mix40
    ids, got = serve_all(reqs, engines=1, max_batch=16, memory_budget=8 << 30, resident=resident,
                         fail_batch_at_mesh=3)
    assert len(got) == len(ids)
    sizes = [got[rid]["batch_size"] for rid in ids]
    assert max(sizes) > 1 and sizes.count(1) >= 1, sizes
    for k, (rid, w) in enumerate(zip(ids, want)):
        assert got[rid]["status"] == 0, k
        assert not octree.diff(got[rid]["tree"], w), k


def test_request_larger_than_budget_is_refused():
    """Admission by computed footprint: a request whose triangles and occupancy pyramids
    alone exceed the budget completes with OOC_ERR_LIMIT without running; the request
    after it still runs."""
    t = tri.icosphere_tris(3)
    with ooc.Server(0, engines=1, max_batch=4, memory_budget=64 << 20) as srv:
        big = srv.submit(t, make_params(1024))  # a 1024^3 stripe's pyramid is ~146 MB
        small = srv.submit(t, make_params(64))
        got = {}
        deadline = time.time() + 60
        while len(got) < 2 and time.time() < deadline:
            r = srv.poll(1000)
            if r is not None:
                got[r["id"]] = r
    assert got[big]["status"] == 6  # OOC_ERR_LIMIT
    assert got[small]["status"] == 0
    assert not octree.diff(got[small]["tree"], oracle_tree(t, make_params(64)))


def test_submit_rejects_invalid_request():
    with ooc.Server(0, engines=1, max_batch=4, memory_budget=1 << 30) as srv:
        bad = make_params(100, 2048)  # not a power of two
        with pytest.raises(ooc.OocError):
            srv.submit(np.zeros((1, 9), np.float32), bad)
        assert srv.poll(10) is None
