"""Serving loop: argument checks that need no GPU (nothing here creates an engine)."""
import ctypes

import ooc_svo_builder_gb300 as ooc


def test_server_create_rejects_bad_config():
    lib = ooc.load_library()
    h = ctypes.c_void_p()
    for cfg in (ooc.ServerConfig(0, 0, 8, 0, 1 << 30),   # no engines
                ooc.ServerConfig(0, 1, 0, 0, 1 << 30),   # batches of zero requests
                ooc.ServerConfig(0, 1, 8, 0, 0),         # no memory budget
                ooc.ServerConfig(0, 1, 8, 2, 1 << 30)):  # unknown result location
        assert lib.ooc_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert lib.ooc_server_create(None, ctypes.byref(h)) == 1


def test_server_calls_reject_null():
    lib = ooc.load_library()
    r = ooc.Result()
    m = ooc.Mesh()
    rid = ctypes.c_uint64()
    assert lib.ooc_server_submit(None, ctypes.byref(m), ctypes.byref(rid)) == 1
    assert lib.ooc_server_poll(None, 0, ctypes.byref(r)) == 1
    assert lib.ooc_server_release(None, 1) == 1
    assert lib.ooc_server_read(None, 1, None, None) == 1
    st = ooc.ServerStats()
    assert lib.ooc_server_stats(None, ctypes.byref(st)) == 1
    lib.ooc_server_destroy(None)


def test_result_struct_layout():
    # ooc_result: id, status, location, nodes, nodes_bytes, data, data_bytes, info (6 x u64), 4 doubles, batch_size
    assert ctypes.sizeof(ooc.Result) == 8 + 4 + 4 + 8 * 4 + 48 + 32 + 8
    # ooc_server_config: device, engines, max_batch, result_location, memory_budget, fail_batch_at_mesh, host_pool_mb
    assert ctypes.sizeof(ooc.ServerConfig) == 32
    # ooc_server_state: nine u64 counters
    assert ctypes.sizeof(ooc.ServerStats) == 9 * 8


def test_tuning_calls_reject_null():
    lib = ooc.load_library()
    t = ooc.Tuning(64, 16, 256, 4, 1 << 30, 0, 4, 1, 0)
    assert lib.ooc_set_tuning(None, ctypes.byref(t)) == 1
    assert lib.ooc_get_tuning(None, ctypes.byref(t)) == 1
    assert lib.ooc_autotune(None, None, 0, None) == 1
    assert ctypes.sizeof(ooc.Tuning) == 40
