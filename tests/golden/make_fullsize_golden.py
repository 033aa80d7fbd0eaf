"""Record the reference's outputs for the full-size configurations as digests.

Runs the reference svo_builder / svo_builder_binary built from the reference's own
sources by ``make -C oracle ref`` (output oracle/_ref/) on the full-size meshes of
tests/golden_cases.py FULLSIZE, and stores per configuration: the SHA-256 of the input
triangles, the octree digest (``octree.digest``: node and data files, NaNs made
canonical), the header text and the filled-voxel count, in fullsize_reference.json.
It does the same, per mesh, for the first meshes of the seeded streams of
configurations 4 and 5 (golden_cases STREAMS) into stream_samples_reference.json.
The CPU oracle is run on the same meshes and must give the same digests.  Regenerate with
``python tests/golden/make_fullsize_golden.py`` (needs the reference build).

``--large`` runs the reference once on configuration 3 (golden_cases FULLSIZE_LARGE: the
seeded 20M-triangle soup, ``svo_builder_binary -s 4096 -l 2048``, 64 partitions).  Its node
file is about 16 GB, so it is hashed from disk in chunks instead of loaded, and the oracle is
not run beside it (it would take as long again); the row goes into the same JSON file.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.dirname(HERE), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)

import golden_cases  # noqa: E402
import pyoracle  # noqa: E402
from ooc_svo_builder_gb300 import octree, tri  # noqa: E402


def run_reference(t, gridsize, limit, payload, color, levels=False):
    """The reference build on one mesh: (octree, header text, filled voxels, partitions, command)."""
    with tempfile.TemporaryDirectory() as d:
        base = os.path.join(d, "mesh")
        tri.write_tri(base, t)
        exe = pyoracle.ref_binary(not payload)
        cmd = [exe, "-f", base + ".tri", "-s", str(gridsize), "-l", str(limit)]
        if payload:
            cmd += ["-c", color]
        if levels:
            cmd.append("-levels")
        stdout = subprocess.run(cmd, cwd=d, stdout=subprocess.PIPE, text=True, check=True).stdout
        filled = int([ln for ln in stdout.splitlines() if ln.startswith("Total amount of voxels")][0].split()[-1])
        P = int([ln for ln in stdout.splitlines() if ln.startswith("Partitioning data into")][0].split()[3])
        obase = base + "%d_%d" % (gridsize, P)
        tree = octree.read_octree(obase)
        with open(obase + ".octree") as f:
            header = f.read()
    command = " ".join([os.path.basename(exe)] + cmd[1:]).replace(base, "mesh")
    return tree, header, filled, P, command


def file_digest(obase: str) -> tuple:
    """(octree.digest of the files at obase, header text, NaN data fields), reading the node
    and data files in 64 MiB chunks."""
    with open(obase + ".octree") as f:
        header = f.read()
    d = octree.StreamDigest(octree.parse_header(obase + ".octree")["gridlength"])
    for kind, ext in ((0, ".octreenodes"), (1, ".octreedata")):
        with open(obase + ext, "rb") as f:
            while True:
                b = f.read(64 << 20)
                if not b:
                    break
                d.update(kind, b)
    return d.result(), header, d.nan_fields


def large_digest(t, gridsize, limit, payload, color, workdir):
    """The reference build on a mesh too large to load its octree: the row of
    fullsize_reference.json, digests computed from the files in chunks."""
    os.makedirs(workdir, exist_ok=True)
    base = os.path.join(workdir, "mesh")
    tri.write_tri(base, t)
    exe = pyoracle.ref_binary(not payload)
    cmd = [exe, "-f", base + ".tri", "-s", str(gridsize), "-l", str(limit)]
    if payload:
        cmd += ["-c", color]
    t0 = time.time()
    stdout = subprocess.run(cmd, cwd=workdir, stdout=subprocess.PIPE, text=True, check=True).stdout
    secs = time.time() - t0
    filled = int([ln for ln in stdout.splitlines() if ln.startswith("Total amount of voxels")][0].split()[-1])
    P = int([ln for ln in stdout.splitlines() if ln.startswith("Partitioning data into")][0].split()[3])
    obase = base + "%d_%d" % (gridsize, P)
    dig, header, nan = file_digest(obase)
    for ext in (".octree", ".octreenodes", ".octreedata", ".tri", ".tridata"):
        path = (obase if ext.startswith(".octree") else base) + ext
        if os.path.exists(path):
            os.remove(path)
    command = " ".join([os.path.basename(exe)] + cmd[1:]).replace(base, "mesh")
    return {"command": command, "input_sha256": golden_cases.input_sha256(t), "n_triangles": int(t.shape[0]),
            "n_partitions": P, "n_filled": filled, "header": header, "digest": dig, "nan_data_fields": nan,
            "reference_seconds": round(secs, 1), "oracle_checked": False}


def checked_digest(name, t, gridsize, limit, payload, color, levels=False):
    """Digest of the reference's output, which the oracle must reproduce; where the reference's
    output is undefined (see reference_undefined), the reason and the oracle's digest."""
    tree, header, filled, P, command = run_reference(t, gridsize, limit, payload, color, levels)
    nodes, data, info = pyoracle.build(t, gridsize, limit, color=color, levels=levels)
    mine_tree = octree.Octree(gridsize, nodes, data)
    dig, mine = octree.digest(tree), octree.digest(mine_tree)
    assert info["n_filled"] == filled, name
    row = {"command": command, "input_sha256": golden_cases.input_sha256(t), "n_triangles": int(t.shape[0]),
           "n_partitions": P, "n_filled": filled}
    if mine != dig:
        why = golden_cases.reference_undefined(gridsize, golden_cases.set_voxels(mine_tree, payload))
        assert why, "%s: the oracle differs from the reference" % name
        row.update({"reference_undefined": why, "oracle_digest": mine})
    else:
        nan = int(sum(int(np.isnan(tree.data[f]).sum()) for f in ("color", "normal")))
        row.update({"header": header, "digest": dig, "nan_data_fields": nan})
    return row


def main_large(workdir: str) -> None:
    path = os.path.join(HERE, "fullsize_reference.json")
    for name, w in golden_cases.FULLSIZE_LARGE.items():
        t0 = time.time()
        row = large_digest(w["make"](), w["gridsize"], w["limit"], w["payload"], w["color"], workdir)
        with open(path) as f:
            out = json.load(f)
        out[name] = row
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
            f.write("\n")
        print("%s: %.1f s" % (name, time.time() - t0))


def main() -> None:
    if "--large" in sys.argv:
        main_large(sys.argv[sys.argv.index("--large") + 1] if len(sys.argv) > sys.argv.index("--large") + 1
                   else tempfile.mkdtemp())
        return
    out = {k: v for k, v in golden_cases.fullsize_reference().items() if k in golden_cases.FULLSIZE_LARGE}
    for name, w in golden_cases.FULLSIZE.items():
        t0 = time.time()
        out[name] = checked_digest(name, w["make"](), w["gridsize"], w["limit"], w["payload"], w["color"],
                                   w.get("levels", False))
        print("%s: %.1f s" % (name, time.time() - t0))
    with open(os.path.join(HERE, "fullsize_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    streams = {}
    for name in golden_cases.STREAMS:
        t0 = time.time()
        rows = []
        for i, (t, N, payload) in enumerate(golden_cases.stream_sample(name)):
            r = checked_digest("%s[%d]" % (name, i), t, N, golden_cases.STREAM_LIMIT_MB, payload, "model")
            r["gridsize"], r["payload"] = N, payload
            r.pop("header", None)
            rows.append(r)
        streams[name] = rows
        print("%s: %d meshes, %.1f s" % (name, len(rows), time.time() - t0))
    with open(os.path.join(HERE, "stream_samples_reference.json"), "w") as f:
        json.dump(streams, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
