"""ctypes binding of the CPU oracle (oracle/_build/libooc_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
benchmark's CPU-baseline leg as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libooc_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

NODE_DTYPE = np.dtype([("data", "<u8"), ("children_base", "<u8"), ("children_offset", "i1", (8,))])
DATA_DTYPE = np.dtype([("morton", "<u8"), ("color", "<f4", (3,)), ("normal", "<f4", (3,))])
COLOR_MODES = {"model": 0, "fixed": 1, "linear": 2, "normal": 3}


class _Params(ctypes.Structure):
    _fields_ = [("gridsize", ctypes.c_uint64), ("memory_limit_mb", ctypes.c_uint64),
                ("geometry_only", ctypes.c_int), ("color_mode", ctypes.c_int), ("generate_levels", ctypes.c_int),
                ("bbox_min", ctypes.c_float * 3), ("bbox_max", ctypes.c_float * 3)]


class _Result(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("n_nodes", ctypes.c_uint64), ("data", ctypes.c_void_p),
                ("n_data", ctypes.c_uint64), ("n_filled", ctypes.c_uint64), ("n_partitions", ctypes.c_uint64),
                ("part_tricounts", ctypes.c_void_p)]


_lib = None


def build_oracle() -> None:
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=subprocess.DEVNULL)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build_oracle()
        lib = ctypes.CDLL(LIB)
        lib.oracle_build.argtypes = [ctypes.POINTER(_Params), ctypes.c_void_p, ctypes.c_uint64,
                                     ctypes.POINTER(_Result)]
        lib.oracle_build.restype = ctypes.c_int
        lib.oracle_free.argtypes = [ctypes.POINTER(_Result)]
        lib.oracle_free.restype = None
        lib.oracle_estimate_partitions.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        lib.oracle_estimate_partitions.restype = ctypes.c_uint64
        lib.oracle_morton_encode.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        lib.oracle_morton_encode.restype = ctypes.c_uint64
        _lib = lib
    return _lib


def estimate_partitions(gridsize: int, memory_limit_mb: int) -> int:
    return int(load().oracle_estimate_partitions(gridsize, memory_limit_mb))


def morton_encode(x: int, y: int, z: int) -> int:
    return int(load().oracle_morton_encode(x, y, z))


def build(tris: np.ndarray, gridsize: int, memory_limit_mb: int = 2048, color: str = "model",
          levels: bool = False, bbox_min=(0.0, 0.0, 0.0), bbox_max=(1.0, 1.0, 1.0)):
    """Run the oracle on [T, 9] (binary) or [T, 21] (payload) triangles.

    Returns (nodes[NODE_DTYPE], data[DATA_DTYPE], info dict)."""
    tris = np.ascontiguousarray(tris, dtype=np.float32)
    lib = load()
    p = _Params()
    p.gridsize = gridsize
    p.memory_limit_mb = memory_limit_mb
    p.geometry_only = 1 if tris.shape[1] == 9 else 0
    p.color_mode = COLOR_MODES[color] if isinstance(color, str) else int(color)
    p.generate_levels = 1 if levels else 0
    for a in range(3):
        p.bbox_min[a] = bbox_min[a]
        p.bbox_max[a] = bbox_max[a]
    r = _Result()
    rc = lib.oracle_build(ctypes.byref(p), tris.ctypes.data_as(ctypes.c_void_p), tris.shape[0], ctypes.byref(r))
    if rc != 0:
        raise RuntimeError("oracle_build failed (%d)" % rc)
    try:
        nodes = np.frombuffer(ctypes.string_at(r.nodes, r.n_nodes * 24), dtype=NODE_DTYPE).copy()
        data = np.frombuffer(ctypes.string_at(r.data, r.n_data * 32), dtype=DATA_DTYPE).copy()
        counts = np.frombuffer(ctypes.string_at(r.part_tricounts, r.n_partitions * 8), dtype=np.uint64).copy()
        info = {"n_nodes": int(r.n_nodes), "n_data": int(r.n_data), "n_filled": int(r.n_filled),
                "n_partitions": int(r.n_partitions), "part_tricounts": counts}
    finally:
        lib.oracle_free(ctypes.byref(r))
    return nodes, data, info


def ref_binary(geometry_only: bool) -> str:
    """Path of the reference executable built by `make -C oracle ref` (may not exist)."""
    return os.path.join(REF_DIR, "svo_builder_binary" if geometry_only else "svo_builder")
