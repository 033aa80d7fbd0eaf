"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference svo_builder / svo_builder_binary compiled from the
reference's own sources by ``make -C oracle ref`` (output oracle/_ref/) on small
seeded inputs, and stores input triangles, flags and the three output files of
each case in ``<case>.npz``.  The fixtures pin both the CPU oracle and the GPU
path; regenerate with ``python tests/golden/make_golden.py`` (needs the
reference sources and g++).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ooc_svo_builder_gb300 import tri  # noqa: E402


def cases():
    rng = np.random.default_rng(77)
    a = rng.random((40, 3), dtype=np.float32)
    b = rng.random((40, 3), dtype=np.float32)
    degenerate = np.concatenate([np.stack([a, a, b], 1).reshape(40, 9), np.stack([a, a, a], 1).reshape(40, 9),
                                 np.stack([a, ((a + b) * np.float32(0.5)).astype(np.float32), b], 1).reshape(40, 9)])
    g = np.arange(0, 9, dtype=np.float32) / np.float32(8)
    aligned = g[rng.integers(0, 9, size=(120, 9))].astype(np.float32)
    ico_b = tri.icosphere_tris(2)
    ico_p = tri.icosphere_tris(2, payload=True)
    rnd_b = tri.random_tris(300, 101, False, lo=-0.05, hi=1.05, max_edge=0.12)
    rnd_p = tri.random_tris(300, 102, True, lo=-0.05, hi=1.05, max_edge=0.12)
    out_p = tri.random_tris(200, 103, True, lo=-0.4, hi=1.4, max_edge=0.3)
    big_p = tri.random_tris(12, 104, True, lo=0.0, hi=1.0, max_edge=1.5)
    dup = np.repeat(tri.random_tris(20, 105, True, max_edge=0.25), 3, axis=0)
    dup[:, 12:21] = rng.random((dup.shape[0], 9), dtype=np.float32)
    return [
        ("ico_binary_32", ico_b, dict(s=32)),
        ("ico_binary_32_levels", ico_b, dict(s=32, levels=True)),
        ("ico_payload_32_model", ico_p, dict(s=32)),
        ("ico_payload_32_linear_levels", ico_p, dict(s=32, c="linear", levels=True)),
        ("ico_payload_16_normal", ico_p, dict(s=16, c="normal")),
        ("ico_payload_16_fixed_levels", ico_p, dict(s=16, c="fixed", levels=True)),
        ("soup_binary_256_l2", rnd_b, dict(s=256, l=2)),
        ("soup_payload_256_l2_levels", rnd_p, dict(s=256, l=2, levels=True)),
        ("degenerate_binary_16", degenerate.astype(np.float32), dict(s=16)),
        ("aligned_binary_8_levels", aligned, dict(s=8, levels=True)),
        ("outside_payload_32", out_p, dict(s=32)),
        ("large_payload_32_levels", big_p, dict(s=32, levels=True)),
        ("duplicates_payload_16", dup, dict(s=16)),
        ("empty_binary_8", np.zeros((0, 9), np.float32), dict(s=8)),
        ("empty_payload_4_levels", np.zeros((0, 21), np.float32), dict(s=4, levels=True)),
        ("grid1_binary", ico_b, dict(s=1)),
        ("grid2_payload_levels", ico_p, dict(s=2, levels=True)),
    ]


def run_reference(tris: np.ndarray, flags: dict, workdir: str):
    binary = tris.shape[1] == 9
    exe = os.path.join(ROOT, "oracle", "_ref", "svo_builder_binary" if binary else "svo_builder")
    if not os.path.exists(exe):
        raise SystemExit("reference build missing: run `make -C oracle ref`")
    base = os.path.join(workdir, "mesh")
    tri.write_tri(base, tris)
    args = [exe, "-f", base + ".tri", "-s", str(flags["s"]), "-l", str(flags.get("l", 2048))]
    if flags.get("levels"):
        args.append("-levels")
    if "c" in flags:
        args += ["-c", flags["c"]]
    out = subprocess.run(args, cwd=workdir, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
    n_part = int([ln for ln in out.stdout.splitlines() if ln.startswith("Partitioning data into")][0].split()[3])
    filled = int([ln for ln in out.stdout.splitlines() if ln.startswith("Total amount of voxels")][0].split()[-1])
    ob = base + "%d_%d" % (flags["s"], n_part)
    header = open(ob + ".octree").read()
    nodes = np.fromfile(ob + ".octreenodes", dtype=np.uint8)
    data = np.fromfile(ob + ".octreedata", dtype=np.uint8)
    return header, nodes, data, n_part, filled


def main():
    for name, tris, flags in cases():
        with tempfile.TemporaryDirectory() as d:
            header, nodes, data, n_part, filled = run_reference(tris, flags, d)
        meta = dict(flags)
        meta.update(n_partitions=n_part, n_filled=filled, header=header)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), tris=tris, nodes=nodes, data=data,
                            meta=np.array(json.dumps(meta)))
        print("%-32s P=%-3d nodes=%-7d data=%-6d filled=%d" % (name, n_part, nodes.size // 24, data.size // 32, filled))


if __name__ == "__main__":
    main()
