"""Serving loop: requests submitted together run in shared batches, and each
result is byte-identical to the same mesh built alone with ooc_build."""
import threading
import time

import numpy as np
import pytest

import ooc_svo_builder_gb300 as ooc
from ooc_svo_builder_gb300 import make_params, octree, tri

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("resident", [False, True], ids=["host", "device"])
def test_results_alone_equal_results_in_the_mix(builder, resident):
    reqs = request_mix()
    alone = [builder.build(t, p).tree for t, p in reqs]
    with ooc.Server(0, engines=2, max_batch=16, memory_budget=8 << 30, resident=resident) as srv:
        ids = [srv.submit(t, p) for t, p in reqs]
        got = {}
        deadline = time.time() + 120
        while len(got) < len(ids) and time.time() < deadline:
            r = srv.poll(1000)
            if r is not None:
                got[r["id"]] = r
    assert len(got) == len(ids)
    assert max(r["batch_size"] for r in got.values()) > 1, "no request shared a batch"
    for rid, want in zip(ids, alone):
        r = got[rid]
        assert r["status"] == 0
        assert r["location"] == (1 if resident else 0)
        d = octree.diff(r["tree"], want)
        assert not d, "\n".join(d)
        assert r["t_submit_us"] <= r["t_start_us"] <= r["t_done_us"]


@pytest.mark.parametrize("resident", [False, True], ids=["host", "device"])
def test_arrivals_while_busy_join_later_batches(builder, resident):
    # a submitting thread keeps adding requests while the engines are running
    reqs = request_mix(seed=11, count=30)
    alone = [builder.build(t, p).tree for t, p in reqs]
    with ooc.Server(0, engines=2, max_batch=8, memory_budget=8 << 30, resident=resident) as srv:
        ids = [None] * len(reqs)

        def feed():
            for i, (t, p) in enumerate(reqs):
                ids[i] = srv.submit(t, p)
                time.sleep(0.002)

        th = threading.Thread(target=feed)
        th.start()
        got = {}
        deadline = time.time() + 120
        while len(got) < len(reqs) and time.time() < deadline:
            r = srv.poll(1000)
            if r is not None:
                got[r["id"]] = r
        th.join()
    for rid, want in zip(ids, alone):
        assert not octree.diff(got[rid]["tree"], want)


def test_submit_rejects_invalid_request():
    with ooc.Server(0, engines=1, max_batch=4, memory_budget=1 << 30) as srv:
        bad = make_params(100, 2048)  # not a power of two
        with pytest.raises(ooc.OocError):
            srv.submit(np.zeros((1, 9), np.float32), bad)
        assert srv.poll(10) is None
