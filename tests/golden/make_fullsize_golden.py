"""Record the reference's outputs for the full-size configurations as digests.

Runs the reference svo_builder / svo_builder_binary built from the reference's own
sources by ``make -C oracle ref`` (output oracle/_ref/) on the full-size meshes of
tests/golden_cases.py FULLSIZE, and stores per configuration: the SHA-256 of the input
triangles, the octree digest (``octree.digest``: node and data files, NaNs made
canonical), the header text and the filled-voxel count, in fullsize_reference.json.
The CPU oracle is run on the same mesh and must give the same digest.  Regenerate with
``python tests/golden/make_fullsize_golden.py`` (needs the reference build).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.dirname(HERE), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)

import golden_cases  # noqa: E402
import pyoracle  # noqa: E402
from ooc_svo_builder_gb300 import octree, tri  # noqa: E402


def main() -> None:
    out = {}
    for name, w in golden_cases.FULLSIZE.items():
        t = w["make"]()
        with tempfile.TemporaryDirectory() as d:
            base = os.path.join(d, "mesh")
            tri.write_tri(base, t)
            exe = pyoracle.ref_binary(not w["payload"])
            cmd = [exe, "-f", base + ".tri", "-s", str(w["gridsize"]), "-l", str(w["limit"])]
            if w["payload"]:
                cmd += ["-c", w["color"]]
            t0 = time.time()
            stdout = subprocess.run(cmd, cwd=d, stdout=subprocess.PIPE, text=True, check=True).stdout
            sec = time.time() - t0
            filled = int([ln for ln in stdout.splitlines() if ln.startswith("Total amount of voxels")][0].split()[-1])
            P = int([ln for ln in stdout.splitlines() if ln.startswith("Partitioning data into")][0].split()[3])
            obase = base + "%d_%d" % (w["gridsize"], P)
            tree = octree.read_octree(obase)
            with open(obase + ".octree") as f:
                header = f.read()
        nodes, data, info = pyoracle.build(t, w["gridsize"], w["limit"], color=w["color"])
        dig = octree.digest(tree)
        assert octree.digest(octree.Octree(w["gridsize"], nodes, data)) == dig, name
        assert info["n_filled"] == filled, name
        out[name] = {"command": " ".join([os.path.basename(exe)] + cmd[1:]).replace(base, "mesh"),
                     "input_sha256": golden_cases.input_sha256(t), "n_triangles": int(t.shape[0]),
                     "n_partitions": P, "n_filled": filled, "header": header, "digest": dig,
                     "nan_data_fields": int(sum(int(octree.np.isnan(tree.data[f]).sum()) for f in ("color", "normal")))}
        print("%s: reference %.1f s, %d nodes, %d data records" % (name, sec, dig["n_nodes"], dig["n_data"]))
    with open(os.path.join(HERE, "fullsize_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
