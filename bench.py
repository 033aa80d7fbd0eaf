#!/usr/bin/env python
"""Benchmark of the GPU partition -> voxelize -> SVO-build path.

Workload (default): configuration 2 -- payload-mode ``svo_builder -s 1024 -l 2048
-c model`` (one partition) on a seeded 1024x1024-vertex value-noise heightfield,
2,093,058 FP32 triangles (176 MB of .tridata, larger than the 129 MB L2).
A step is one complete build: voxelization, payload, octree layout and records.

* ``value``: Mtri/s with the triangles resident in HBM (``ooc_build_device``),
  CUDA events on the build stream around exactly ``--steps`` builds.
* ``e2e``: the same metric through ``ooc_build`` (the C ABI call the CLI uses):
  host->device copy of the pinned triangles and device->host copy of the node
  and data files inside the timed region, wall clock.
* ``roofline``: the dominant kernel, timed live with CUDA events in the timed
  region; algorithmic bytes per launch from the workload.
* ``cpu_baseline``: the CPU oracle (a plain-C restatement of the reference,
  single-threaded like the reference) on the same mesh.

``--impl reference`` times the reference's CPU path (the oracle port; the
reference sources are not available on the GPU host) on the same workload.
Multi-GPU (torchrun): independent replicas, one mesh per rank, max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from ooc_svo_builder_gb300 import tri  # noqa: E402

HEIGHTFIELD_N = 1024
WORKLOADS = {
    "heightfield1024": dict(gridsize=1024, limit=2048, payload=True, color="model",
                            desc="configuration 2: payload svo_builder -s 1024 -l 2048 -c model on a 1024x1024-vertex "
                                 "value-noise heightfield (2,093,058 triangles, one partition)"),
    "icosphere256": dict(gridsize=256, limit=2048, payload=False, color="model",
                         desc="configuration 1: svo_builder_binary -s 256 -l 2048 on a subdivision-5 icosphere "
                              "(20,480 triangles)"),
    "soup4096": dict(gridsize=4096, limit=2048, payload=False, color="model",
                     desc="configuration 3: svo_builder_binary -s 4096 -l 2048 (64 partitions) on a 20M-triangle "
                          "soup: half small triangles on 200 spheres, half log-normal edges (median 4 voxels, "
                          "sigma 1.0, clipped at 512)"),
    "soup2048": dict(gridsize=2048, limit=2048, payload=False, color="model",
                     desc="profiling case of the batched stripe kernels: svo_builder_binary -s 2048 -l 2048 (8 "
                          "partitions of 1024^3, one sub-batch) on a 1M-triangle soup of the configuration-3 "
                          "distribution"),
    "soup1024": dict(gridsize=1024, limit=2048, payload=False, color="model",
                     desc="profiling case of the configuration-3 soup: svo_builder_binary -s 1024 -l 2048 (one "
                          "partition) on a 4M-triangle soup of the same distribution"),
}


def make_mesh(name: str) -> np.ndarray:
    if name == "heightfield1024":
        return tri.heightfield_tris(HEIGHTFIELD_N, seed=2, payload=True)
    if name == "icosphere256":
        return tri.icosphere_tris(5, radius=0.4, jitter=0.002, seed=1)
    if name == "soup4096":
        return tri.soup_tris(20_000_000, 4096, seed=3, sigma=1.0)
    if name == "soup1024":
        return tri.soup_tris(4_000_000, 1024, seed=3, sigma=1.0)
    if name == "soup2048":
        return tri.soup_tris(1_000_000, 2048, seed=3, sigma=1.0)
    raise SystemExit("unknown workload " + name)


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "of measured (MEASURED_PEAKS.json hbm_gbs)"}
    return {"hbm_gbs": 6800.0, "source": "of fallback (MEASURED_PEAKS.json absent: 6.8 TB/s, one earlier GB300 copy)"}


def workload_config(name: str, world: int) -> dict:
    """The `config` of a workload's bench line; both arms print the same one."""
    w = WORKLOADS[name]
    N = w["gridsize"]
    T = {"heightfield1024": 2 * (HEIGHTFIELD_N - 1) ** 2, "icosphere256": 20 * 4 ** 5, "soup4096": 20_000_000,
         "soup1024": 4_000_000, "soup2048": 1_000_000}[name]
    # estimate_partitions (partitioner.cpp:12-28) and stripes of at most 1024^3 voxels
    need, P = N ** 3 // (1 << 20), 1
    while need > w["limit"]:
        need //= 8
        P *= 8
    stripes = max(1, N ** 3 // min(N ** 3, 1 << 30))
    tri_bytes = T * (84 if w["payload"] else 36)
    return {"workload": w["desc"], "name": name, "gridsize": N, "memory_limit_mb": w["limit"], "n_triangles": T,
            "mode": "payload" if w["payload"] else "binary", "partitions": P, "stripes": stripes,
            "l2": "inputs larger than L2 (%.0f MB of triangles per step; L2 129 MB)" % (tri_bytes / 1e6)
                  if tri_bytes > 129e6 else "inputs smaller than L2 (%.0f MB of triangles per step)" % (tri_bytes / 1e6),
            "parallelism": "replicas" if world > 1 else "single GPU"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_port_time(tris, w, budget_s: float, max_runs: int, min_runs: int = 1):
    """Time the oracle port on the whole mesh; returns (seconds per build, runs)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    times = []
    t_start = time.perf_counter()
    while len(times) < max_runs and (len(times) < min_runs or time.perf_counter() - t_start < budget_s):
        t0 = time.perf_counter()
        pyoracle.build(tris, w["gridsize"], w["limit"], color=w["color"])
        times.append(time.perf_counter() - t0)
    return statistics.mean(times), len(times)


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of a workload's dominant
# kernel, from the ncu captures summarised under profiles/: (workload, kernel) -> (bytes, summary)
NCU_TRAFFIC = {
    ("heightfield1024", "vox_small_occupancy"): (179.5e6 + 34.5e6, "profiles/vox_small_heightfield1024.md"),
}


def algorithmic_bytes(kernel: str, n_tris: int, info: dict, S: int, payload: bool) -> float:
    """Minimum DRAM bytes one launch of `kernel` must move for this workload."""
    tri_bytes = 84 if payload else 36
    leaf_words = S // 32
    if kernel == "vox_small_occupancy":
        # vertices of every triangle (36 B) + its task count (8 B) + (payload) pass mask and box (16 B)
        return n_tris * (36 + 8 + (16 if payload else 0))
    if kernel in ("vox_small_winner", "vox_large_occupancy", "vox_large_winner"):
        # vertices of every triangle (36 B) + the task count per item (8 B)
        return n_tris * (36 + 8)
    if kernel == "pyramid":  # leaf level dominates: read bits, write parent bits + block counts
        return leaf_words * 4 * (1 + 1 / 8 + 1 / 8)
    if kernel == "compact":
        return leaf_words * 4 + info["n_nodes"] * 4
    if kernel == "leaf_payload":
        return info["n_filled"] * (4 + 4 + tri_bytes + 24)
    if kernel in ("top_down", "bottom_up"):
        return info["n_nodes"] * (4 + 4 + 4 + 8 + 8 + 24) + info["n_data"] * 32
    return 0.0


def small_candidates(tris: np.ndarray, gridsize: int, small_vol: int = 64) -> int:
    """Candidate voxels of the triangles the one-thread-per-triangle pass voxelizes: the sum of
    their clamped grid-box volumes (voxelizer.cpp:199-204, boxes of at most `small_vol` voxels).
    Meshes in the unit cube, so unit_div = gridsize."""
    v = tris[:, :9].reshape(-1, 3, 3).astype(np.float32)
    g = np.float32(gridsize)
    lo = np.clip((v.min(axis=1) * g).astype(np.int64), 0, gridsize - 1)
    hi = np.clip((v.max(axis=1) * g).astype(np.int64), 0, gridsize - 1)
    vol = np.prod(hi - lo + 1, axis=1)
    return int(vol[vol <= small_vol].sum())


def run_ours(args, world, rank, local):
    import torch
    import ooc_svo_builder_gb300 as ooc

    w = WORKLOADS[args.workload]
    torch.cuda.set_device(local)
    tris = make_mesh(args.workload)
    T = tris.shape[0]
    prm = ooc.make_params(w["gridsize"], w["limit"], geometry_only=not w["payload"], color=w["color"])
    d_tris = torch.from_numpy(tris).to(f"cuda:{local}")
    h_tris = torch.from_numpy(tris).pin_memory()
    stream = torch.cuda.Stream(device=local)
    b = ooc.Builder(local)
    if args.batch_budget:
        b.set_batch_budget(args.batch_budget)

    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    # warm-up (also sizes every device buffer)
    for _ in range(args.warmup):
        info = b.build_device(d_tris.data_ptr(), T, prm, stream.cuda_stream)
    torch.cuda.synchronize()
    # one profiling build: phases and every kernel (outside the timed region)
    b.set_phase_timing(True)
    b.set_kernel_timing("*")
    info = b.build_device(d_tris.data_ptr(), T, prm, stream.cuda_stream)
    phases = b.phase_times()
    kt = b.kernel_times()
    b.set_phase_timing(False)
    dominant = max(kt.items(), key=lambda kv: kv[1][0])[0] if kt else None
    b.set_kernel_timing(dominant)

    # ---- timed region: device-resident input ----
    # The clock sampler watches a window of back-to-back builds around the timed ones: untimed
    # builds for about a second before them and half a second after, so that its 200 ms samples
    # see the GPU under this load even when the timed steps take only milliseconds.
    sampler = ClockSampler(local)
    sampler.start()
    t_pre = time.perf_counter()
    while time.perf_counter() - t_pre < args.clock_window * 2 / 3:
        for _ in range(16):
            b.build_device(d_tris.data_ptr(), T, prm, stream.cuda_stream)
        torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    dom_ms, dom_n = 0.0, 0
    ev0.record(stream)
    for _ in range(args.steps):
        info = b.build_device(d_tris.data_ptr(), T, prm, stream.cuda_stream)
        launches += b.kernel_launches()
        ms, n = b.kernel_times().get(dominant, (0.0, 0))
        dom_ms += ms
        dom_n += n
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    t_post = time.perf_counter()
    b.set_kernel_timing(None)
    while time.perf_counter() - t_post < args.clock_window / 3:
        for _ in range(16):
            b.build_device(d_tris.data_ptr(), T, prm, stream.cuda_stream)
        torch.cuda.synchronize()
    clocks = sampler.stop()
    clocks["window"] = ("samples every 200 ms over %.1f s of back-to-back builds: untimed before the timed "
                        "steps, the timed steps, untimed after" % args.clock_window)
    ms_total = max_over_ranks(ev0.elapsed_time(ev1), world)
    ms_step = ms_total / args.steps
    value = world * T / (ms_step / 1e3) / 1e6
    nodes_per_s = world * info["n_nodes"] / (ms_step / 1e3)

    # ---- end to end through the C ABI: pinned host triangles in, host octree out ----
    got = {"n": 0}

    def sink(user, kind, ptr, n):
        got["n"] += n
        return 0

    cb = ooc.SINK(sink)
    for _ in range(max(1, args.warmup)):
        b.build_ptr(h_tris.data_ptr(), T, prm, cb)
    b.set_phase_timing(True)
    b.build_ptr(h_tris.data_ptr(), T, prm, cb)
    e2e_phases = b.phase_times()
    b.set_phase_timing(False)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_info = b.build_ptr(h_tris.data_ptr(), T, prm, cb)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    barrier(world)
    e2e_value = world * T / (e2e_s / args.steps) / 1e6

    # ---- file to file (ooc_build_files, what the svo_builder drop-ins run), outside the timed region ----
    files = None
    if not args.no_files:
        import shutil
        import tempfile
        tmp = tempfile.mkdtemp(prefix="ooc_bench_")
        try:
            tri_path = tri.write_tri(os.path.join(tmp, "mesh"), tris)
            b.build_files(tri_path, prm)  # warm page cache and buffers
            runs = 2
            t0 = time.perf_counter()
            for _ in range(runs):
                out_base, _ = b.build_files(tri_path, prm)
            fs = (time.perf_counter() - t0) / runs
            out_bytes = sum(os.path.getsize(out_base + ext) for ext in (".octreenodes", ".octreedata"))
            files = {"value": T / fs / 1e6, "unit": "Mtri/s", "s_per_build": fs, "output_bytes": out_bytes,
                     "note": "ooc_build_files: .tridata read to the device in 64 MB chunks through two pinned "
                             "buffers, octree files written by one thread per file; warm page cache, local disk"}
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
    stripes = e2e_info["n_stripes"]
    h2d = T * tris.shape[1] * 4
    # the stripe spans are copied back; header records and the stripe roots are written on the host
    payload = w["payload"]
    d2h = (e2e_info["n_nodes"] - stripes) * 24 + (e2e_info["n_data"] - (1 if payload else 2)) * 32 + stripes * 36

    # ---- roofline of the dominant kernel ----
    peaks = measured_peaks()
    S = min(w["gridsize"] ** 3, 1 << 30)
    alg = algorithmic_bytes(dominant, T, info, S, payload) if dominant else 0.0
    per_launch_ms = dom_ms / dom_n if dom_n else float("nan")
    launches_per_build = kt.get(dominant, (0, 1))[1] if dominant else 1
    alg_per_launch = alg / max(1, launches_per_build)
    achieved = alg_per_launch / (per_launch_ms / 1e3) / 1e9 if dom_n else None
    traffic, traffic_src = args.traffic, "--traffic" if args.traffic else None
    if traffic is None and (args.workload, dominant) in NCU_TRAFFIC:
        traffic, traffic_src = NCU_TRAFFIC[(args.workload, dominant)]
    roofline = {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": (achieved / peaks["hbm_gbs"]) if achieved else None, "traffic": traffic,
                "traffic_source": traffic_src,
                "peak_source": peaks["source"],
                "per_launch_ms": per_launch_ms, "algorithmic_bytes_per_launch": alg_per_launch}
    # The voxelization is issue-bound, not HBM-bound: its own roofline is the FP32 rate without
    # FMA (SMs x 128 lanes x the measured SM clock) against the 47 flops of the full
    # Schwarz-Seidel test per candidate voxel (voxelizer.cpp:266-287).
    if dominant == "vox_small_occupancy" and dom_n and clocks.get("sm_mhz"):
        flops = 47.0 * small_candidates(tris, w["gridsize"]) / max(1, launches_per_build)
        fp32_peak = sm_count * 128 * clocks["sm_mhz"] * 1e6 / 1e12
        fp32_achieved = flops / (per_launch_ms / 1e3) / 1e12
        roofline["fp32"] = {"bound": "fp32 issue (no FMA)", "achieved": fp32_achieved, "peak": fp32_peak,
                            "unit": "TFLOP/s", "frac": fp32_achieved / fp32_peak,
                            "flops_per_launch": flops,
                            "peak_source": "%d SMs (device attribute) x 128 FP32 lanes x measured SM clock" % sm_count}

    line = {
        "metric": "Mtri/s", "value": value, "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.workload, world),
        "svo_nodes_per_s": nodes_per_s, "n_nodes": info["n_nodes"], "n_data": info["n_data"],
        "n_filled": info["n_filled"],
        "e2e": {"value": e2e_value, "unit": "Mtri/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s / args.steps * 1e3},
        "gpu_launches": launches,
        "roofline": roofline,
        "phases_ms": phases,
        "e2e_phases_ms": e2e_phases,
        "file_to_file": files,
        "kernels_ms": {k: v[0] for k, v in sorted(kt.items(), key=lambda kv: -kv[1][0])},
        "clocks": clocks,
        "tuning": b.tuning().as_dict(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sec, runs = cpu_port_time(tris, w, budget_s=10.0, max_runs=8)
        line["cpu_baseline"] = {"value": T / sec / 1e6, "unit": "Mtri/s", "cores": 1, "kind": "port",
                                "sample": "whole %s mesh (%d triangles), %d build(s), mean; single thread like the "
                                          "reference" % (args.workload, T, runs)}
    b.close()
    return line


def run_batch(args, world, rank, local):
    """Configuration 4: the batched form against the plain per-mesh path, through the C ABI from pinned
    host triangles, with octrees delivered to host memory (ooc_build_batch vs ooc_build per mesh) and
    kept resident in HBM (ooc_build_batch_device over all meshes vs one mesh per call)."""
    import ctypes
    import torch
    import ooc_svo_builder_gb300 as ooc

    torch.cuda.set_device(local)
    meshes = tri.batch_meshes(args.n_meshes, seed=4)
    n = len(meshes)
    total_tris = sum(m[0].shape[0] for m in meshes)
    offs = [0]
    for t, _, _ in meshes:
        offs.append(offs[-1] + (t.nbytes + 255) // 256 * 256)
    pinned = torch.empty(offs[-1], dtype=torch.uint8).pin_memory()
    host = pinned.numpy()
    arr = (ooc.Mesh * n)()
    params = []
    for i, (t, N, payload) in enumerate(meshes):
        host[offs[i]:offs[i] + t.nbytes] = t.reshape(-1).view(np.uint8)
        p = ooc.make_params(N, 2048, geometry_only=not payload)
        params.append(p)
        arr[i].tris = pinned.data_ptr() + offs[i]
        arr[i].n_tris = t.shape[0]
        arr[i].params = p
    infos = (ooc.BuildInfo * n)()
    cb = ooc.BATCH_SINK(lambda user, mesh, kind, ptr, nb: 0)
    cb1 = ooc.SINK(lambda user, kind, ptr, nb: 0)
    b = ooc.Builder(local)
    # the autotuner picks the launch choices on every 16th mesh (untimed)
    sample_idx = list(range(0, n, 16))
    sample = (ooc.Mesh * len(sample_idx))()
    for q, i in enumerate(sample_idx):
        sample[q] = arr[i]
    t0 = time.perf_counter()
    tuned = b.autotune(mesh_array=sample, n_meshes=len(sample_idx))
    tune_s = time.perf_counter() - t0
    if args.persistent != "auto":  # one phase-A form held, for comparing the two
        tuned.persistent = int(args.persistent)
        b.set_tuning(tuned)
    tuning = tuned.as_dict()

    def timed(fn, warm, reps):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps

    # host output
    t_batch = timed(lambda: b.build_batch_ptrs(arr, n, cb, infos), max(1, args.warmup), args.steps)
    launches = b.kernel_launches()
    n_nodes = sum(int(infos[i].n_nodes) for i in range(n))
    out_bytes = sum(int(infos[i].n_nodes) * 24 + int(infos[i].n_data) * 32 for i in range(n))

    def plain_host():
        for i in range(n):
            b.build_ptr(arr[i].tris, arr[i].n_tris, params[i], cb1)
    for i in range(min(n, 64)):
        b.build_ptr(arr[i].tris, arr[i].n_tris, params[i], cb1)
    t_plain = timed(plain_host, 0, 1)

    # device-resident output into one HBM arena
    arena_buf = torch.empty(out_bytes + 512 * n + (64 << 20), dtype=torch.uint8, device="cuda")
    arena = ooc.DeviceArena(arena_buf.data_ptr(), arena_buf.numel(), 0)
    dinfos = (ooc.BuildInfo * n)()

    def batch_dev():
        arena.used = 0
        b.build_batch_device_ptrs(arr, n, arena, dinfos)
    t_batch_dev = timed(batch_dev, max(1, args.warmup), args.steps)
    launches_dev = b.kernel_launches()
    # one more call with CUDA-event phase and per-kernel timing (not part of the timed steps)
    b.set_phase_timing(True)
    b.set_kernel_timing("*")
    t0 = time.perf_counter()
    batch_dev()
    wall_dev = time.perf_counter() - t0
    phases_dev = b.phase_times()
    kernels_dev = {k: round(v[0], 3) for k, v in sorted(b.kernel_times().items(), key=lambda kv: -kv[1][0])}
    b.set_phase_timing(False)
    b.set_kernel_timing(None)
    one = (ooc.Mesh * 1)()

    def plain_dev():
        for i in range(n):
            one[0] = arr[i]
            arena.used = 0
            b.build_batch_device_ptrs(one, 1, arena, dinfos)
    t_plain_dev = timed(plain_dev, 0, 1)

    # parity sample: for every 64th mesh, the batch's host bytes and its arena bytes equal ooc_build's
    sample = list(range(0, n, 64))
    got = {i: {0: [], 1: []} for i in sample}

    def collect(user, mesh, kind, ptr, nb):
        if mesh in got and kind < 2:
            got[mesh][kind].append(ctypes.string_at(ptr, nb))
        return 0

    b.build_batch_ptrs(arr, n, ooc.BATCH_SINK(collect), infos)
    batch_dev()
    layout, _ = ooc.arena_layout(dinfos, n)
    identical = dev_identical = True
    for i in sample:
        want = {0: [], 1: []}

        def collect1(user, kind, ptr, nb, want=want):
            want[kind].append(ctypes.string_at(ptr, nb))
            return 0

        b.build_ptr(arr[i].tris, arr[i].n_tris, params[i], ooc.SINK(collect1))
        w = (b"".join(want[0]), b"".join(want[1]))
        identical = identical and (b"".join(got[i][0]), b"".join(got[i][1])) == w
        no, nb, do, db = layout[i]
        d = (arena_buf[no:no + nb].cpu().numpy().tobytes(), arena_buf[do:do + db].cpu().numpy().tobytes())
        dev_identical = dev_identical and d == w
    b.close()
    value = n / t_batch_dev
    return {
        "metric": "meshes/s", "value": value, "unit": "meshes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_batch_dev * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "configuration 4: %d meshes, log-uniform 64..200k triangles (icospheres and soups), "
                               "gridsize 64/128/256/512, binary or payload 50/50, one batch call per step; "
                               "value = octrees resident in HBM (ooc_build_batch_device), e2e = octrees "
                               "copied back to host memory (ooc_build_batch)" % n,
                   "name": "batch4096", "n_meshes": n, "n_triangles": total_tris,
                   "l2": "inputs larger than L2 (%.1f GB of triangles per step)" % (offs[-1] / 1e9)},
        "mtri_per_s": total_tris / t_batch_dev / 1e6, "svo_nodes_per_s": n_nodes / t_batch_dev,
        "resident": {"batched_meshes_per_s": n / t_batch_dev, "plain_meshes_per_s": n / t_plain_dev,
                     "speedup_vs_plain": t_plain_dev / t_batch_dev,
                     "timed_call": {"wall_ms": wall_dev * 1e3, "phases_ms": phases_dev, "kernels_ms": kernels_dev}},
        "host": {"batched_meshes_per_s": n / t_batch, "plain_meshes_per_s": n / t_plain,
                 "speedup_vs_plain": t_plain / t_batch},
        "tuning": dict(tuning, sample_meshes=len(sample_idx), seconds=round(tune_s, 2)),
        "parity_sample": {"meshes": len(sample), "host_identical_to_plain": identical,
                          "resident_identical_to_plain": dev_identical},
        "e2e": {"value": n / t_batch, "unit": "meshes/s", "h2d_bytes_per_step": int(sum(m[0].nbytes for m in meshes)),
                "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": launches_dev, "gpu_launches_host_output": launches,
    }


def serve_stream(srv, pool, rate: float, duration: float, seed: int, drain_s: float) -> dict:
    """Drive one Poisson arrival stream through a server; latencies from the server's own clock."""
    import threading

    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.5) + 16))
    arrivals = arrivals[arrivals < duration]
    picks = rng.integers(0, len(pool), size=len(arrivals))
    results = []
    submitted = [0]
    stop = threading.Event()

    def collect():
        while not stop.is_set() or len(results) < submitted[0]:
            r = srv.poll(50, copy=False)
            if r is not None:
                results.append(r)
            elif stop.is_set() and time.perf_counter() > t_end:
                return

    t_end = float("inf")
    th = threading.Thread(target=collect)
    th.start()
    t0 = time.perf_counter()
    for a, k in zip(arrivals, picks):
        while True:
            dt = t0 + a - time.perf_counter()
            if dt <= 0:
                break
            time.sleep(min(dt, 0.0005) if dt > 0.0002 else 0)
        ptr, n, params, N = pool[k]
        srv.submit_ptr(ptr, n, params, N)
        submitted[0] += 1
    t_end = time.perf_counter() + drain_s
    stop.set()
    th.join()
    lat = np.array([(r["t_done_us"] - r["t_submit_us"]) / 1e3 for r in results])
    built = np.array([(r["t_built_us"] - r["t_submit_us"]) / 1e3 for r in results])  # queue + build
    deliver = np.array([(r["t_done_us"] - r["t_built_us"]) / 1e3 for r in results])  # host copy back
    done = np.array([r["t_done_us"] for r in results])
    sub = np.array([r["t_submit_us"] for r in results])
    span = (done.max() - sub.min()) / 1e6 if len(results) else float("nan")
    return {"offered_req_s": rate, "requests": int(submitted[0]), "completed": len(results),
            "failed": int(sum(r["status"] != 0 for r in results)),
            "meshes_per_s": len(results) / span if len(results) else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "p99_built_ms": float(np.percentile(built, 99)) if len(lat) else None,
            "p99_deliver_ms": float(np.percentile(deliver, 99)) if len(lat) else None,
            "mean_batch": float(np.mean([r["batch_size"] for r in results])) if results else None,
            "output_gb": float(sum(r["bytes"] for r in results) / 1e9)}


def serve_burst(srv, pool, n: int, seed: int) -> dict:
    """Capacity: `n` requests submitted at once; meshes/s until the last completes."""
    rng = np.random.default_rng(seed)
    picks = rng.integers(0, len(pool), size=n)
    t0 = time.perf_counter()
    for k in picks:
        srv.submit_ptr(*pool[k])
    done = []
    while len(done) < n:
        r = srv.poll(1000, copy=False)
        if r is not None:
            done.append(r)
    wall = time.perf_counter() - t0
    lat = np.array([(r["t_done_us"] - r["t_submit_us"]) / 1e3 for r in done])
    return {"requests": n, "meshes_per_s": n / wall, "seconds": wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_batch": float(np.mean([r["batch_size"] for r in done])),
            "failed": int(sum(r["status"] != 0 for r in done))}


def serve_bounds(pool, local: int, n: int) -> dict:
    """What limits capacity, on `n` requests drawn like the burst's: one batch call over all of
    them (no serving loop), the kernel time alone (events around every kernel of that call), and
    one call per request.  Results stay in one HBM arena."""
    import torch
    import ooc_svo_builder_gb300 as ooc

    rng = np.random.default_rng(77)
    picks = rng.integers(0, len(pool), size=n)
    arr = (ooc.Mesh * n)()
    for q, k in enumerate(picks):
        ptr, nt, params, _ = pool[k]
        arr[q].tris = ptr
        arr[q].n_tris = nt
        arr[q].params = params
    infos = (ooc.BuildInfo * n)()
    out = {"requests": n}
    with ooc.Builder(local) as b:
        sink = ooc.BATCH_SINK(lambda user, mesh, kind, p, nb: 0)
        b.build_batch_ptrs(arr, n, sink, infos)  # sizes the arena
        out_bytes = sum(int(infos[i].n_nodes) * 24 + int(infos[i].n_data) * 32 for i in range(n))
        arena_buf = torch.empty(out_bytes + 512 * n + (64 << 20), dtype=torch.uint8, device="cuda")
        arena = ooc.DeviceArena(arena_buf.data_ptr(), arena_buf.numel(), 0)

        def batch():
            arena.used = 0
            b.build_batch_device_ptrs(arr, n, arena, infos)
        batch()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch()
        out["one_batch_meshes_per_s"] = n / (time.perf_counter() - t0)
        b.set_kernel_timing("*")
        batch()
        kernel_ms = sum(v[0] for v in b.kernel_times().values())
        b.set_kernel_timing(None)
        out["kernel_ms_per_request"] = kernel_ms / n
        out["kernel_bound_meshes_per_s"] = n / (kernel_ms / 1e3)
        one = (ooc.Mesh * 1)()
        t0 = time.perf_counter()
        for q in range(n):
            one[0] = arr[q]
            arena.used = 0
            b.build_batch_device_ptrs(one, 1, arena, infos)
        out["one_call_per_request_meshes_per_s"] = n / (time.perf_counter() - t0)
        del arena_buf
    return out


SERVE_ARMS = ("served_resident", "plain_resident", "served_host", "plain_host")


def serve_pool(args):
    """The request pool of configuration 5: (meshes, pinned host buffer, [(ptr, n_tris, params, N)])."""
    import torch
    import ooc_svo_builder_gb300 as ooc

    meshes = tri.batch_meshes(args.n_meshes, seed=5, gridsizes=(128, 256, 512, 1024, 2048))
    offs = [0]
    for t, _, _ in meshes:
        offs.append(offs[-1] + (t.nbytes + 255) // 256 * 256)
    pinned = torch.empty(offs[-1], dtype=torch.uint8).pin_memory()
    host = pinned.numpy()
    pool = []
    for i, (t, N, payload) in enumerate(meshes):
        host[offs[i]:offs[i] + t.nbytes] = t.reshape(-1).view(np.uint8)
        pool.append((pinned.data_ptr() + offs[i], t.shape[0], ooc.make_params(N, 2048, geometry_only=not payload), N))
    return meshes, pinned, pool


def serve_part(args, local, part):
    """One part of configuration 5, in a process of its own: an arm at every rate, a capacity
    burst of a resident arm ("burst:<arm>"), or the capacity bounds ("bounds")."""
    import torch
    import ooc_svo_builder_gb300 as ooc

    torch.cuda.set_device(local)
    meshes, pinned, pool = serve_pool(args)
    if part == "bounds":
        return serve_bounds(pool, local, args.bound_meshes)
    # served: continuous batching over engines; plain: one request at a time through the same library.
    # resident: octrees stay in HBM (released by the poller); host: copied back to host memory.
    arms = {"served_resident": dict(engines=args.engines, max_batch=256, memory_budget=120 << 30, resident=True),
            "plain_resident": dict(engines=1, max_batch=1, memory_budget=120 << 30, resident=True),
            "served_host": dict(engines=args.engines, max_batch=256, memory_budget=120 << 30,
                                host_pool_mb=args.host_pool_mb),
            "plain_host": dict(engines=1, max_batch=1, memory_budget=120 << 30, host_pool_mb=args.host_pool_mb)}
    # warm-up set: the requests with the largest grids, then a spread of the rest
    order = sorted(range(len(pool)), key=lambda i: -pool[i][3] * pool[i][1])
    warm = order[:16] + order[16::max(1, len(pool) // 64)]

    def warmed(cfg):
        srv = ooc.Server(local, **cfg)
        for i in warm:
            srv.submit_ptr(*pool[i])
        for _ in warm:
            while srv.poll(1000, copy=False) is None:
                pass
        return srv

    if part.startswith("burst:"):
        arm = part.split(":", 1)[1]
        with warmed(arms[arm]) as srv:
            out = serve_burst(srv, pool, args.burst, seed=77)
        print("serve burst %s: %s" % (arm, json.dumps(out)), file=sys.stderr, flush=True)
        return out
    out = []
    for r in (float(x) for x in args.rates.split(",")):
        # a fresh server per rate: a backlog left by an overloaded rate does not carry over
        with warmed(arms[part]) as srv:
            # an unmeasured stream at the same rate first, so the measured one sees the
            # server in its steady state (engine buffers grown, pinned result blocks pooled)
            if args.serve_warmup > 0:
                serve_stream(srv, pool, r, args.serve_warmup, seed=1005 + int(r), drain_s=args.drain)
            out.append(serve_stream(srv, pool, r, args.duration, seed=5 + int(r), drain_s=args.drain))
            st = srv.stats()
            out[-1]["server"] = {"pinned_on_demand_gb": st["pinned_on_demand_bytes"] / 1e9,
                                 "pinned_on_demand_allocs": st["pinned_on_demand_allocs"],
                                 "pinned_reserve_gb": st["pinned_reserve_bytes"] / 1e9}
        print("serve %s %.0f req/s: %s" % (part, r, json.dumps(out[-1])), file=sys.stderr, flush=True)
    return out


def run_serve(args, world, rank, local):
    """Configuration 5: Poisson request streams through the serving loop (continuous batching,
    footprint admission) and, on the same streams, through the plain path (one request at a time).
    Each arm, each capacity burst and the bounds run in a child process of their own, so no
    arm inherits the process state (device memory pool, pinned memory) an earlier one left."""
    import subprocess

    fwd = ["--workload", "serve", "--rates", args.rates, "--duration", str(args.duration), "--drain",
           str(args.drain), "--serve-warmup", str(args.serve_warmup), "--engines", str(args.engines), "--burst",
           str(args.burst), "--bound-meshes", str(args.bound_meshes), "--host-pool-mb", str(args.host_pool_mb),
           "--n-meshes", str(args.n_meshes)]

    def child(part):
        p = subprocess.run([sys.executable, os.path.abspath(__file__), *fwd, "--serve-part", part],
                           stdout=subprocess.PIPE, text=True, env=dict(os.environ, LOCAL_RANK=str(local)))
        if p.returncode != 0:
            raise RuntimeError("serve part %s failed (exit %d)" % (part, p.returncode))
        return json.loads(p.stdout.strip().splitlines()[-1])

    out = {arm: child(arm) for arm in SERVE_ARMS}
    capacity = {arm: child("burst:" + arm) for arm in ("served_resident", "plain_resident")}
    bounds = child("bounds")
    print("serve bounds: %s" % json.dumps(bounds), file=sys.stderr, flush=True)
    top = out["served_resident"][-1]
    top_host = out["served_host"][-1]
    meshes = tri.batch_meshes(args.n_meshes, seed=5, gridsizes=(128, 256, 512, 1024, 2048))

    def ratio(a, b):
        return [x["meshes_per_s"] / max(y["meshes_per_s"], 1e-9) for x, y in zip(out[a], out[b])]

    return {
        "metric": "served meshes/s", "value": top["meshes_per_s"], "unit": "meshes/s", "n_gpus": world,
        "steps": top["completed"], "warmup": 1, "ms_per_step": 1e3 / max(top["meshes_per_s"], 1e-9),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "configuration 5: Poisson arrivals at %s req/s, %.0f s each after %.0f s "
                               "unmeasured at the same rate, meshes drawn from a pool of %d configuration-4 "
                               "meshes with gridsizes 128..2048; 120 GB admission budget; pinned host "
                               "triangles in, host octree bytes out; each arm in a process of its own"
                               % (args.rates, args.duration, args.serve_warmup, len(meshes)),
                   "name": "serve", "engines": args.engines, "max_batch": 256, "host_pool_mb": args.host_pool_mb,
                   "value_arm": "served_resident: octrees resident in HBM, released by the poller"},
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
        "arms": out,
        "speedup_vs_plain_resident": ratio("served_resident", "plain_resident"),
        "capacity": dict(capacity, speedup_vs_plain=capacity["served_resident"]["meshes_per_s"] /
                         max(capacity["plain_resident"]["meshes_per_s"], 1e-9)),
        "speedup_vs_plain_host": ratio("served_host", "plain_host"),
        "bounds": bounds,
        "e2e": {"value": top_host["meshes_per_s"], "unit": "meshes/s", "p50_ms": top_host["p50_ms"],
                "p99_ms": top_host["p99_ms"], "note": "results copied back to host memory",
                "h2d_bytes_per_step": int(np.mean([t.nbytes for t, _, _ in meshes])),
                "d2h_bytes_per_step": int(top_host["output_gb"] * 1e9 / max(top_host["completed"], 1))},
    }


def _reference_worker(job):
    """One host core: `warmup` untimed builds of the workload's mesh, then `steps` timed ones after
    every worker has reached the barrier; returns the timed seconds."""
    name, warmup, steps, barrier = job
    w = WORKLOADS[name]
    tris = make_mesh(name)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    for _ in range(warmup):
        pyoracle.build(tris, w["gridsize"], w["limit"], color=w["color"])
    barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        pyoracle.build(tris, w["gridsize"], w["limit"], color=w["color"])
    return time.perf_counter() - t0


def run_reference(args, world, rank):
    """The reference's CPU path (the oracle restatement: the reference's sources are not on the GPU
    host) on all host cores.  The reference builds one mesh per process on one thread, so its
    throughput on the box is one build per core, all cores at once."""
    if rank != 0:
        return None
    import multiprocessing as mp
    w = WORKLOADS[args.workload]
    if args.workload not in ("heightfield1024", "icosphere256"):
        raise SystemExit("--impl reference times whole builds; use heightfield1024 or icosphere256")
    T = make_mesh(args.workload).shape[0]
    cores = args.ref_cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        barrier = mgr.Barrier(cores)
        with ctx.Pool(cores) as pool:
            secs = pool.map(_reference_worker, [(args.workload, args.warmup, args.steps, barrier)] * cores)
    wall = max(secs)  # the workers start together at the barrier
    value = cores * args.steps * T / wall / 1e6
    return {
        "metric": "Mtri/s", "value": value, "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": workload_config(args.workload, world),
        "cpu_baseline": {"value": value, "unit": "Mtri/s", "cores": cores, "kind": "port",
                         "sample": "whole mesh per step on every core at once (%d processes x %d steps); "
                                   "per-core build %.0f ms" % (cores, args.steps, statistics.mean(secs) / args.steps * 1e3)},
        "e2e": {"value": value, "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heightfield1024", choices=sorted(WORKLOADS) + ["batch4096", "serve"])
    ap.add_argument("--n-meshes", type=int, default=None,
                    help="meshes of the batch4096 workload (4096) or of the serve pool (512)")
    ap.add_argument("--rates", default="200,500,1000,2000", help="serve: offered request rates, req/s")
    ap.add_argument("--duration", type=float, default=5.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--drain", type=float, default=10.0, help="serve: seconds to wait for the queue to drain")
    ap.add_argument("--serve-warmup", type=float, default=3.0,
                    help="serve: seconds of unmeasured arrivals at each rate before the measured ones")
    ap.add_argument("--engines", type=int, default=2, help="serve: engines of the served arm")
    ap.add_argument("--host-pool-mb", type=int, default=8192,
                    help="serve: pinned host memory each host-result server reserves at creation, MiB")
    ap.add_argument("--burst", type=int, default=4096, help="serve: requests of the capacity burst")
    ap.add_argument("--serve-part", default=None, help=argparse.SUPPRESS)  # set by run_serve for its children
    ap.add_argument("--bound-meshes", type=int, default=512,
                    help="serve: requests of the capacity bounds (one batch call; kernels alone; one call each)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-budget", type=int, default=0,
                    help="occupancy-pyramid bytes per sub-batch (0: the library's default, 4 GiB)")
    ap.add_argument("--persistent", default="auto", choices=["auto", "0", "1"],
                    help="configuration 4: the autotuner's phase-A form, or one held (0: a launch per pass, "
                         "1: the persistent work-queue kernel)")
    ap.add_argument("--clock-window", type=float, default=1.5,
                    help="seconds of back-to-back builds the clock sampler watches around the timed steps")
    ap.add_argument("--no-files", action="store_true", help="skip the file-to-file measurement")
    ap.add_argument("--ref-cores", type=int, default=0, help="reference arm: host processes (default: all cores)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, world, rank)
    elif args.workload == "batch4096":
        args.n_meshes = args.n_meshes or 4096
        line = run_batch(args, world, rank, local)
    elif args.workload == "serve":
        args.n_meshes = args.n_meshes or 512
        if args.serve_part:  # a child of run_serve: print its part alone
            print(json.dumps(serve_part(args, local, args.serve_part)))
            return
        line = run_serve(args, world, rank, local)
    else:
        line = run_ours(args, world, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
