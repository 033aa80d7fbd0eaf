"""The C ABI library loads and exports every symbol include/ooc_svo_gpu.h declares (no GPU needed)."""
import ctypes
import os
import re

import ooc_svo_builder_gb300 as ooc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "ooc_svo_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ooc_[a-z_]+)\s*\(", text)))


def test_header_matches_binding_list():
    assert declared_symbols() == sorted(ooc.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(ooc.LIB_PATH)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_estimate_partitions_without_gpu():
    # partitioner.cpp:12-28; needs no device
    assert ooc.estimate_partitions(256, 2048) == 1
    assert ooc.estimate_partitions(256, 2) == 8
    assert ooc.estimate_partitions(1024, 2048) == 1
    assert ooc.estimate_partitions(4096, 2048) == 64
    assert ooc.estimate_partitions(512, 2) == 64


def test_context_on_missing_device_fails_cleanly():
    lib = ooc.load_library()
    h = ctypes.c_void_p()
    assert lib.ooc_ctx_create(999, ctypes.byref(h)) != 0
    assert not h.value
