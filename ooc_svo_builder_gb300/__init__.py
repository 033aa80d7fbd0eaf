"""GB300-native partition -> voxelize -> SVO-build path of ooc_svo_builder.

Python binding of ``libooc_svo_gpu.so`` (C ABI in ``include/ooc_svo_gpu.h``).
The library is required: importing the binding raises if it has not been built
(``python -c "import __graft_entry__ as g; g.build()"``).  There is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass

import numpy as np

from . import octree as _octree

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libooc_svo_gpu.so")

OOC_OK = 0
ERRORS = {1: "OOC_ERR_INVALID", 2: "OOC_ERR_OOM", 3: "OOC_ERR_DEVICE", 4: "OOC_ERR_IO", 5: "OOC_ERR_SINK",
          6: "OOC_ERR_LIMIT", 7: "OOC_ERR_TIMEOUT"}
OOC_ERR_TIMEOUT = 7
OOC_STREAM_NODES, OOC_STREAM_DATA, OOC_STREAM_END = 0, 1, 2
NOALLOC_MAX_TRIANGLES = 1048576
NOALLOC_MAX_GRIDSIZE = 1024
COLOR_MODES = {"model": 0, "fixed": 1, "linear": 2, "normal": 3}
PHASES = ("partition", "voxelize", "pyramid", "octree", "copies", "build")

# Every symbol declared in include/ooc_svo_gpu.h.
EXPORTS = ("ooc_ctx_create", "ooc_ctx_destroy", "ooc_last_error", "ooc_estimate_partitions", "ooc_build",
           "ooc_build_device", "ooc_result_device", "ooc_result_copy", "ooc_set_phase_timing", "ooc_phase_times",
           "ooc_kernel_launches", "ooc_build_files", "ooc_set_kernel_timing", "ooc_kernel_time",
           "ooc_voxelize_occupancy_noalloc", "ooc_build_batch", "ooc_server_create", "ooc_server_submit",
           "ooc_server_poll", "ooc_server_release", "ooc_server_destroy", "ooc_build_batch_device",
           "ooc_arena_alloc", "ooc_set_batch_budget", "ooc_batch_budget", "ooc_server_read", "ooc_get_tuning",
           "ooc_set_tuning", "ooc_autotune", "ooc_check_octree_device", "ooc_build_from_device",
           "ooc_partition_counts", "ooc_file_times", "ooc_set_stream_budget", "ooc_stream_budget",
           "ooc_stream_passes", "ooc_server_stats")
CHECK_BITS = {1: "child group order", 2: "reference count", 4: "depth", 8: "data index", 16: "payload Morton code"}


class BuildParams(ctypes.Structure):
    _fields_ = [("gridsize", ctypes.c_uint64), ("memory_limit_mb", ctypes.c_uint64),
                ("geometry_only", ctypes.c_int32), ("color_mode", ctypes.c_int32),
                ("generate_levels", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("bbox_min", ctypes.c_float * 3), ("bbox_max", ctypes.c_float * 3)]


class BuildInfo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint64), ("n_data", ctypes.c_uint64), ("n_filled", ctypes.c_uint64),
                ("n_partitions", ctypes.c_uint64), ("n_stripes", ctypes.c_uint64), ("n_items", ctypes.c_uint64)]


SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint64)
BATCH_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p,
                              ctypes.c_uint64)


class Mesh(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_void_p), ("n_tris", ctypes.c_uint64), ("params", BuildParams)]


RESULT_HOST, RESULT_DEVICE = 0, 1


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("engines", ctypes.c_int32), ("max_batch", ctypes.c_uint32),
                ("result_location", ctypes.c_int32), ("memory_budget", ctypes.c_uint64),
                ("fail_batch_at_mesh", ctypes.c_uint32), ("host_pool_mb", ctypes.c_uint32)]


class Result(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int32), ("location", ctypes.c_int32),
                ("nodes", ctypes.c_void_p), ("nodes_bytes", ctypes.c_uint64), ("data", ctypes.c_void_p),
                ("data_bytes", ctypes.c_uint64), ("info", BuildInfo), ("t_submit_us", ctypes.c_double),
                ("t_start_us", ctypes.c_double), ("t_built_us", ctypes.c_double), ("t_done_us", ctypes.c_double),
                ("batch_size", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in (
        "queued", "in_flight_bytes", "completed_unpolled", "held", "deliveries", "pinned_reserve_bytes",
        "pinned_reserve_free_bytes", "pinned_on_demand_bytes", "pinned_on_demand_allocs")]


class Tuning(ctypes.Structure):
    _fields_ = [("small_vol", ctypes.c_uint32), ("lines_per_lane", ctypes.c_uint32), ("large_block", ctypes.c_uint32),
                ("large_ctas_per_sm", ctypes.c_uint32), ("batch_budget", ctypes.c_uint64), ("graphs", ctypes.c_uint32),
                ("light_per_thread", ctypes.c_uint32), ("pdl", ctypes.c_uint32), ("persistent", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class OctreeCheck(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint64), ("n_data", ctypes.c_uint64), ("n_leaves", ctypes.c_uint64),
                ("n_inner", ctypes.c_uint64), ("first_bad", ctypes.c_uint64), ("errors", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32)]


class DeviceArena(ctypes.Structure):
    _fields_ = [("base", ctypes.c_void_p), ("capacity", ctypes.c_uint64), ("used", ctypes.c_uint64)]


ALLOC = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p))
READY = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64)


def arena_layout(infos, n: int):
    """Offsets of each mesh's node and data files in an arena filled by ooc_arena_alloc (mesh order,
    256-byte aligned files)."""
    out, off = [], 0
    for i in range(n):
        nb, db = int(infos[i].n_nodes) * 24, int(infos[i].n_data) * 32
        out.append((off, nb, off + (nb + 255) // 256 * 256, db))
        off += (nb + 255) // 256 * 256 + (db + 255) // 256 * 256
    return out, off


class OocError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libooc_svo_gpu.so and declare its signatures; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libooc_svo_gpu.so not built at %s; run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    lib.ooc_ctx_create.argtypes = [ctypes.c_int32, P(ctypes.c_void_p)]
    lib.ooc_ctx_create.restype = ctypes.c_int
    lib.ooc_ctx_destroy.argtypes = [ctypes.c_void_p]
    lib.ooc_ctx_destroy.restype = None
    lib.ooc_last_error.argtypes = [ctypes.c_void_p]
    lib.ooc_last_error.restype = ctypes.c_char_p
    lib.ooc_estimate_partitions.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    lib.ooc_estimate_partitions.restype = ctypes.c_uint64
    lib.ooc_build.argtypes = [ctypes.c_void_p, P(BuildParams), ctypes.c_void_p, ctypes.c_uint64, SINK,
                              ctypes.c_void_p, P(BuildInfo)]
    lib.ooc_build.restype = ctypes.c_int
    lib.ooc_build_device.argtypes = [ctypes.c_void_p, P(BuildParams), ctypes.c_void_p, ctypes.c_uint64,
                                     ctypes.c_void_p, P(BuildInfo)]
    lib.ooc_build_device.restype = ctypes.c_int
    lib.ooc_result_device.argtypes = [ctypes.c_void_p, P(ctypes.c_void_p), P(ctypes.c_void_p)]
    lib.ooc_result_device.restype = ctypes.c_int
    lib.ooc_result_copy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.ooc_result_copy.restype = ctypes.c_int
    lib.ooc_set_phase_timing.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.ooc_set_phase_timing.restype = ctypes.c_int
    lib.ooc_phase_times.argtypes = [ctypes.c_void_p, P(ctypes.c_float), ctypes.c_int32]
    lib.ooc_phase_times.restype = ctypes.c_int
    lib.ooc_kernel_launches.argtypes = [ctypes.c_void_p]
    lib.ooc_kernel_launches.restype = ctypes.c_uint64
    lib.ooc_partition_counts.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, P(ctypes.c_uint64),
                                         P(ctypes.c_uint64)]
    lib.ooc_partition_counts.restype = ctypes.c_uint64
    lib.ooc_file_times.argtypes = [ctypes.c_void_p, P(ctypes.c_float), ctypes.c_int32]
    lib.ooc_file_times.restype = ctypes.c_int
    lib.ooc_set_stream_budget.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    lib.ooc_set_stream_budget.restype = ctypes.c_int
    lib.ooc_stream_budget.argtypes = [ctypes.c_void_p]
    lib.ooc_stream_budget.restype = ctypes.c_uint64
    lib.ooc_stream_passes.argtypes = [ctypes.c_void_p]
    lib.ooc_stream_passes.restype = ctypes.c_uint64
    lib.ooc_build_files.argtypes = [ctypes.c_void_p, ctypes.c_char_p, P(BuildParams), ctypes.c_char_p,
                                    ctypes.c_uint64, P(BuildInfo)]
    lib.ooc_build_files.restype = ctypes.c_int
    lib.ooc_set_kernel_timing.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.ooc_set_kernel_timing.restype = ctypes.c_int
    lib.ooc_kernel_time.argtypes = [ctypes.c_void_p, ctypes.c_int32, P(ctypes.c_char_p), P(ctypes.c_float),
                                    P(ctypes.c_uint64)]
    lib.ooc_kernel_time.restype = ctypes.c_int
    lib.ooc_build_batch.argtypes = [ctypes.c_void_p, P(Mesh), ctypes.c_uint64, BATCH_SINK, ctypes.c_void_p,
                                    P(BuildInfo)]
    lib.ooc_build_batch.restype = ctypes.c_int
    lib.ooc_build_batch_device.argtypes = [ctypes.c_void_p, P(Mesh), ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, P(BuildInfo)]
    lib.ooc_build_batch_device.restype = ctypes.c_int
    lib.ooc_arena_alloc.restype = ctypes.c_int
    lib.ooc_set_batch_budget.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    lib.ooc_set_batch_budget.restype = ctypes.c_int
    lib.ooc_batch_budget.argtypes = [ctypes.c_void_p]
    lib.ooc_batch_budget.restype = ctypes.c_uint64
    lib.ooc_get_tuning.argtypes = [ctypes.c_void_p, P(Tuning)]
    lib.ooc_get_tuning.restype = ctypes.c_int
    lib.ooc_set_tuning.argtypes = [ctypes.c_void_p, P(Tuning)]
    lib.ooc_set_tuning.restype = ctypes.c_int
    lib.ooc_autotune.argtypes = [ctypes.c_void_p, P(Mesh), ctypes.c_uint64, P(Tuning)]
    lib.ooc_autotune.restype = ctypes.c_int
    lib.ooc_build_from_device.argtypes = [ctypes.c_void_p, P(BuildParams), ctypes.c_void_p, ctypes.c_uint64, SINK,
                                          ctypes.c_void_p, P(BuildInfo)]
    lib.ooc_build_from_device.restype = ctypes.c_int
    lib.ooc_check_octree_device.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                            ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p, P(OctreeCheck)]
    lib.ooc_check_octree_device.restype = ctypes.c_int
    lib.ooc_server_create.argtypes = [P(ServerConfig), P(ctypes.c_void_p)]
    lib.ooc_server_create.restype = ctypes.c_int
    lib.ooc_server_submit.argtypes = [ctypes.c_void_p, P(Mesh), P(ctypes.c_uint64)]
    lib.ooc_server_submit.restype = ctypes.c_int
    lib.ooc_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_int32, P(Result)]
    lib.ooc_server_poll.restype = ctypes.c_int
    lib.ooc_server_read.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    lib.ooc_server_read.restype = ctypes.c_int
    lib.ooc_server_stats.argtypes = [ctypes.c_void_p, P(ServerStats)]
    lib.ooc_server_stats.restype = ctypes.c_int
    lib.ooc_server_release.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    lib.ooc_server_release.restype = ctypes.c_int
    lib.ooc_server_destroy.argtypes = [ctypes.c_void_p]
    lib.ooc_server_destroy.restype = None
    lib.ooc_voxelize_occupancy_noalloc.argtypes = [P(BuildParams), ctypes.c_void_p, ctypes.c_uint64,
                                                   ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    lib.ooc_voxelize_occupancy_noalloc.restype = ctypes.c_int
    _lib = lib
    return lib


def estimate_partitions(gridsize: int, memory_limit_mb: int) -> int:
    """estimate_partitions (partitioner.cpp:12-28), through the library."""
    return int(load_library().ooc_estimate_partitions(gridsize, memory_limit_mb))


def make_params(gridsize: int, memory_limit_mb: int = 2048, geometry_only: bool = True, color: str = "model",
                levels: bool = False, bbox_min=(0.0, 0.0, 0.0), bbox_max=(1.0, 1.0, 1.0)) -> BuildParams:
    p = BuildParams()
    p.gridsize = gridsize
    p.memory_limit_mb = memory_limit_mb
    p.geometry_only = 1 if geometry_only else 0
    p.color_mode = COLOR_MODES[color] if isinstance(color, str) else int(color)
    p.generate_levels = 1 if levels else 0
    p.reserved = 0
    for a in range(3):
        p.bbox_min[a] = float(bbox_min[a])
        p.bbox_max[a] = float(bbox_max[a])
    return p


def voxelize_occupancy_noalloc(params: BuildParams, tris_device_ptr: int, n_tris: int, occupancy_device_ptr: int,
                               occupancy_words: int, stream: int = 0) -> int:
    """Occupancy bitfield of a single-partition grid without any GPU allocation.

    For callers that may not allocate device memory where they voxelize (stream
    capture, engines that pre-reserve all memory, latency-critical loops).  The
    scratch is a fixed array inside the library; at most NOALLOC_MAX_TRIANGLES
    triangles and gridsize NOALLOC_MAX_GRIDSIZE.  Calls on one device share that
    scratch, so calls that may overlap on the GPU race.  Returns the OOC_* code;
    the work is queued on `stream` and not waited for.
    """
    return int(load_library().ooc_voxelize_occupancy_noalloc(
        ctypes.byref(params), ctypes.c_void_p(tris_device_ptr), n_tris, ctypes.c_void_p(occupancy_device_ptr),
        occupancy_words, ctypes.c_void_p(stream or None)))


def check_octree_device(nodes_ptr: int, n_nodes: int, data_ptr: int, n_data: int, gridsize: int,
                        geometry_only: bool, stream: int = 0) -> dict:
    """Structural check of an octree in device memory (ooc_check_octree_device); `errors` lists
    the violated invariants, empty for a well-formed octree."""
    lib = load_library()
    r = OctreeCheck()
    rc = lib.ooc_check_octree_device(ctypes.c_void_p(nodes_ptr), n_nodes, ctypes.c_void_p(data_ptr), n_data, gridsize,
                                     1 if geometry_only else 0, ctypes.c_void_p(stream or None), ctypes.byref(r))
    if rc != OOC_OK:
        raise OocError(rc, "ooc_check_octree_device failed")
    return {"n_leaves": int(r.n_leaves), "n_inner": int(r.n_inner), "max_depth": int(r.max_depth),
            "first_bad": int(r.first_bad), "errors": [v for b, v in CHECK_BITS.items() if r.errors & b]}


@dataclass
class BuildResult:
    tree: _octree.Octree
    info: dict


def _info_dict(info: BuildInfo) -> dict:
    return {k: int(getattr(info, k)) for k, _ in BuildInfo._fields_}


class Builder:
    """One library context on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.ooc_ctx_create(device, ctypes.byref(h))
        if rc != OOC_OK:
            raise OocError(rc, "ooc_ctx_create(%d) failed" % device)
        self.h = h

    def close(self):
        if self.h:
            self.lib.ooc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != OOC_OK:
            raise OocError(rc, self.lib.ooc_last_error(self.h).decode(errors="replace"))

    def set_phase_timing(self, on: bool = True):
        self._check(self.lib.ooc_set_phase_timing(self.h, 1 if on else 0))

    def phase_times(self) -> dict:
        arr = (ctypes.c_float * 6)()
        self._check(self.lib.ooc_phase_times(self.h, arr, 6))
        return {k: float(arr[i]) for i, k in enumerate(PHASES)}

    def kernel_launches(self) -> int:
        return int(self.lib.ooc_kernel_launches(self.h))

    def set_stream_budget(self, nbytes: int) -> None:
        """Device bytes for the triangle records of an out-of-core build (0: half the free device memory)."""
        self._check(self.lib.ooc_set_stream_budget(self.h, nbytes))

    def stream_passes(self) -> int:
        """Passes over the triangles of the last build (0: not built out of core)."""
        return int(self.lib.ooc_stream_passes(self.h))

    def file_times(self) -> dict:
        arr = (ctypes.c_float * 2)()
        self._check(self.lib.ooc_file_times(self.h, arr, 2))
        return {"read": float(arr[0]), "write": float(arr[1])}

    def partition_counts(self):
        """(triangles per partition, filled voxels per partition) of the last build's first mesh."""
        n = int(self.lib.ooc_partition_counts(self.h, 0, 0, None, None))
        tris = (ctypes.c_uint64 * max(n, 1))()
        filled = (ctypes.c_uint64 * max(n, 1))()
        self.lib.ooc_partition_counts(self.h, 0, n, tris, filled)
        return [int(v) for v in tris[:n]], [int(v) for v in filled[:n]]

    def set_kernel_timing(self, kernel):
        """Time `kernel` ("*" = all, None = off) with CUDA events in later builds."""
        self._check(self.lib.ooc_set_kernel_timing(self.h, kernel.encode() if kernel else None))

    def kernel_times(self) -> dict:
        """{kernel: (total device ms, launches)} of the last build."""
        out = {}
        i = 0
        while True:
            name = ctypes.c_char_p()
            ms = ctypes.c_float()
            n = ctypes.c_uint64()
            if self.lib.ooc_kernel_time(self.h, i, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(n)) != 0:
                break
            out[name.value.decode()] = (float(ms.value), int(n.value))
            i += 1
        return out

    def build(self, tris: np.ndarray, params: BuildParams, sink=None) -> BuildResult:
        """Host triangles in, octree bytes out (through the sink into host memory)."""
        tris = np.ascontiguousarray(tris, dtype=np.float32)
        width = 9 if params.geometry_only else 21
        if tris.ndim != 2 or tris.shape[1] != width:
            raise ValueError("triangles must be [T, %d] float32 for this mode" % width)
        parts = {0: [], 1: []}

        if sink is None:
            def _collect(user, kind, ptr, n):
                parts[kind].append(ctypes.string_at(ptr, n))
                return 0
            cb = SINK(_collect)
        else:
            cb = SINK(sink)
        info = BuildInfo()
        rc = self.lib.ooc_build(self.h, ctypes.byref(params), tris.ctypes.data_as(ctypes.c_void_p),
                                tris.shape[0], cb, None, ctypes.byref(info))
        self._check(rc)
        tree = _octree.from_bytes(int(params.gridsize), b"".join(parts[0]), b"".join(parts[1]))
        return BuildResult(tree, _info_dict(info))

    def build_batch(self, meshes, params_list) -> list:
        """Many meshes in one call; returns one BuildResult per mesh (host octree bytes)."""
        if len(meshes) != len(params_list):
            raise ValueError("one BuildParams per mesh")
        arrs = []
        arr = (Mesh * max(1, len(meshes)))()
        for i, (t, p) in enumerate(zip(meshes, params_list)):
            t = np.ascontiguousarray(t, dtype=np.float32)
            width = 9 if p.geometry_only else 21
            if t.ndim != 2 or t.shape[1] != width:
                raise ValueError("mesh %d: triangles must be [T, %d] float32" % (i, width))
            arrs.append(t)
            arr[i].tris = t.ctypes.data
            arr[i].n_tris = t.shape[0]
            arr[i].params = p
        parts = [{0: [], 1: []} for _ in meshes]

        ends = []

        def _collect(user, mesh, kind, ptr, n):
            if kind == OOC_STREAM_END:
                ends.append(mesh)
            else:
                parts[mesh][kind].append(ctypes.string_at(ptr, n))
            return 0

        cb = BATCH_SINK(_collect)
        infos = (BuildInfo * max(1, len(meshes)))()
        self._check(self.lib.ooc_build_batch(self.h, arr, len(meshes), cb, None, infos))
        if ends != list(range(len(meshes))):
            raise OocError(3, "meshes did not complete once each, in order: %r" % ends[:16])
        return [BuildResult(_octree.from_bytes(int(params_list[i].gridsize), b"".join(parts[i][0]),
                                               b"".join(parts[i][1])), _info_dict(infos[i]))
                for i in range(len(meshes))]

    def tuning(self) -> "Tuning":
        t = Tuning()
        self._check(self.lib.ooc_get_tuning(self.h, ctypes.byref(t)))
        return t

    def set_tuning(self, t: "Tuning") -> None:
        self._check(self.lib.ooc_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, meshes=None, params_list=None, mesh_array=None, n_meshes: int = 0) -> "Tuning":
        """Tune on a sample (host arrays, or a ctypes Mesh array); the context keeps the result."""
        keep = None
        if mesh_array is None:
            mesh_array, keep = self._mesh_array(meshes, params_list)
            n_meshes = len(meshes)
        t = Tuning()
        self._check(self.lib.ooc_autotune(self.h, mesh_array, n_meshes, ctypes.byref(t)))
        del keep
        return t

    def set_batch_budget(self, nbytes: int) -> None:
        self._check(self.lib.ooc_set_batch_budget(self.h, nbytes))

    def batch_budget(self) -> int:
        return int(self.lib.ooc_batch_budget(self.h))

    def build_batch_device(self, meshes, params_list, capacity: int = 1 << 30) -> list:
        """Many meshes in one call, each octree written into device memory (one arena, a torch
        buffer of `capacity` bytes); returns one BuildResult per mesh after copying the arena back."""
        import torch
        arr, keep = self._mesh_array(meshes, params_list)
        arena_buf = torch.empty(capacity, dtype=torch.uint8, device="cuda")
        arena = DeviceArena(arena_buf.data_ptr(), capacity, 0)
        infos = (BuildInfo * max(1, len(meshes)))()
        ready = []
        cb = READY(lambda user, mesh: ready.append(mesh) or 0)
        fn = ctypes.cast(self.lib.ooc_arena_alloc, ctypes.c_void_p)
        self._check(self.lib.ooc_build_batch_device(self.h, arr, len(meshes), fn, cb, ctypes.byref(arena), infos))
        if ready != list(range(len(meshes))):
            raise OocError(3, "meshes were not ready once each, in order")
        layout, used = arena_layout(infos, len(meshes))
        if used != arena.used:
            raise OocError(3, "arena layout differs from the allocator's")
        host = arena_buf[:used].cpu().numpy().tobytes()
        return [BuildResult(_octree.from_bytes(int(params_list[i].gridsize), host[no:no + nb], host[do:do + db]),
                            _info_dict(infos[i])) for i, (no, nb, do, db) in enumerate(layout)]

    def build_batch_device_ptrs(self, mesh_array, n_meshes: int, arena: "DeviceArena", infos) -> None:
        """Low-level device batch call into an arena (ooc_arena_alloc), no ready callback."""
        fn = ctypes.cast(self.lib.ooc_arena_alloc, ctypes.c_void_p)
        self._check(self.lib.ooc_build_batch_device(self.h, mesh_array, n_meshes, fn, None, ctypes.byref(arena),
                                                    infos))

    def _mesh_array(self, meshes, params_list):
        if len(meshes) != len(params_list):
            raise ValueError("one BuildParams per mesh")
        keep = []
        arr = (Mesh * max(1, len(meshes)))()
        for i, (t, p) in enumerate(zip(meshes, params_list)):
            t = np.ascontiguousarray(t, dtype=np.float32)
            width = 9 if p.geometry_only else 21
            if t.ndim != 2 or t.shape[1] != width:
                raise ValueError("mesh %d: triangles must be [T, %d] float32" % (i, width))
            keep.append(t)
            arr[i].tris = t.ctypes.data
            arr[i].n_tris = t.shape[0]
            arr[i].params = p
        return arr, keep

    def build_batch_ptrs(self, mesh_array, n_meshes: int, sink, infos) -> None:
        """Low-level batch call: a ctypes Mesh array, a BATCH_SINK and a BuildInfo array."""
        self._check(self.lib.ooc_build_batch(self.h, mesh_array, n_meshes, sink, None, infos))

    def build_ptr(self, tris_ptr: int, n_tris: int, params: BuildParams, sink) -> dict:
        """Host triangles given by address (e.g. pinned memory); `sink` is a SINK instance."""
        info = BuildInfo()
        self._check(self.lib.ooc_build(self.h, ctypes.byref(params), ctypes.c_void_p(tris_ptr), n_tris, sink,
                                       None, ctypes.byref(info)))
        return _info_dict(info)

    def build_device(self, tris_dev_ptr: int, n_tris: int, params: BuildParams, stream: int = 0) -> dict:
        """Triangles already in device memory; the octree stays on the device."""
        info = BuildInfo()
        self._check(self.lib.ooc_build_device(self.h, ctypes.byref(params), ctypes.c_void_p(tris_dev_ptr), n_tris,
                                              ctypes.c_void_p(stream or None), ctypes.byref(info)))
        return _info_dict(info)

    def result_device(self):
        n = ctypes.c_void_p()
        d = ctypes.c_void_p()
        self._check(self.lib.ooc_result_device(self.h, ctypes.byref(n), ctypes.byref(d)))
        return int(n.value or 0), int(d.value or 0)

    def result_tree(self, gridsize: int, n_nodes: int, n_data: int) -> _octree.Octree:
        """Copy the last build_device result to host memory."""
        nodes = np.empty(n_nodes, dtype=_octree.NODE_DTYPE)
        data = np.empty(n_data, dtype=_octree.DATA_DTYPE)
        self._check(self.lib.ooc_result_copy(self.h, nodes.ctypes.data_as(ctypes.c_void_p),
                                             data.ctypes.data_as(ctypes.c_void_p)))
        return _octree.Octree(gridsize, nodes, data)

    def build_files(self, tri_path: str, params: BuildParams):
        out = ctypes.create_string_buffer(4096)
        info = BuildInfo()
        self._check(self.lib.ooc_build_files(self.h, tri_path.encode(), ctypes.byref(params), out, 4096,
                                             ctypes.byref(info)))
        return out.value.decode(), _info_dict(info)


class Server:
    """The serving loop: submit meshes, poll completed octrees (see ooc_server_* in the C ABI)."""

    def __init__(self, device: int = 0, engines: int = 2, max_batch: int = 256, memory_budget: int = 120 << 30,
                 resident: bool = False, fail_batch_at_mesh: int = 0, host_pool_mb: int = 0):
        """`resident`: results stay in device memory (read with poll(copy=True) or ooc_server_read).
        `fail_batch_at_mesh`: fault injection for tests; `host_pool_mb`: pinned host memory reserved
        for host results at creation (ooc_server_config)."""
        self.lib = load_library()
        cfg = ServerConfig(device, engines, max_batch, RESULT_DEVICE if resident else RESULT_HOST, memory_budget,
                           fail_batch_at_mesh, host_pool_mb)
        h = ctypes.c_void_p()
        rc = self.lib.ooc_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != OOC_OK:
            raise OocError(rc, "ooc_server_create failed")
        self.h = h
        self._keep = {}
        # a request can complete before its submitting call returns: the id is recorded
        # under this lock, which a poller takes before looking the id up
        self._lock = threading.Lock()

    def submit(self, tris: np.ndarray, params: BuildParams) -> int:
        tris = np.ascontiguousarray(tris, dtype=np.float32)
        width = 9 if params.geometry_only else 21
        if tris.ndim != 2 or tris.shape[1] != width:
            raise ValueError("triangles must be [T, %d] float32" % width)
        m = Mesh()
        m.tris = tris.ctypes.data
        m.n_tris = tris.shape[0]
        m.params = params
        rid = ctypes.c_uint64()
        with self._lock:
            rc = self.lib.ooc_server_submit(self.h, ctypes.byref(m), ctypes.byref(rid))
            if rc != OOC_OK:
                raise OocError(rc, "ooc_server_submit failed")
            self._keep[rid.value] = (tris, int(params.gridsize))
        return rid.value

    def submit_ptr(self, tris_ptr: int, n_tris: int, params: BuildParams, gridsize: int) -> int:
        """Queue triangles given by address (e.g. pinned memory kept alive by the caller)."""
        m = Mesh()
        m.tris = tris_ptr
        m.n_tris = n_tris
        m.params = params
        rid = ctypes.c_uint64()
        with self._lock:
            rc = self.lib.ooc_server_submit(self.h, ctypes.byref(m), ctypes.byref(rid))
            if rc != OOC_OK:
                raise OocError(rc, "ooc_server_submit failed")
            self._keep[rid.value] = (None, gridsize)
        return rid.value

    def poll(self, timeout_ms: int = 100, copy: bool = True):
        """Next completed request as a dict (None on timeout); `copy` returns its octree."""
        r = Result()
        rc = self.lib.ooc_server_poll(self.h, timeout_ms, ctypes.byref(r))
        if rc == OOC_ERR_TIMEOUT:
            return None
        if rc != OOC_OK:
            raise OocError(rc, "ooc_server_poll failed")
        with self._lock:
            _, gridsize = self._keep.pop(r.id)
        out = {"id": r.id, "status": r.status, "info": _info_dict(r.info), "t_submit_us": r.t_submit_us,
               "t_start_us": r.t_start_us, "t_built_us": r.t_built_us, "t_done_us": r.t_done_us,
               "batch_size": r.batch_size,
               "bytes": r.nodes_bytes + r.data_bytes, "location": r.location}
        if copy and r.status == OOC_OK:
            nodes = np.empty(r.nodes_bytes, np.uint8)
            data = np.empty(r.data_bytes, np.uint8)
            rc = self.lib.ooc_server_read(self.h, r.id, nodes.ctypes.data, data.ctypes.data)
            if rc != OOC_OK:
                raise OocError(rc, "ooc_server_read failed")
            out["tree"] = _octree.from_bytes(gridsize, nodes.tobytes(), data.tobytes())
        self.lib.ooc_server_release(self.h, r.id)
        return out

    def stats(self) -> dict:
        """The serving loop's state (ooc_server_stats)."""
        st = ServerStats()
        rc = self.lib.ooc_server_stats(self.h, ctypes.byref(st))
        if rc != OOC_OK:
            raise OocError(rc, "ooc_server_stats failed")
        return {k: int(getattr(st, k)) for k, _ in st._fields_}

    def close(self):
        if self.h:
            self.lib.ooc_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
