"""Command lines and input files for the CLI diagnostics checks.

The reference's executables (src/svo_builder/main.cpp:100-196 for the flags,
main.cpp:244-267 with tri_tools.h:75-115 for the .tri header, partitioner.cpp:12-28
for the partition estimate) report every bad argument or input on stdout and exit
with status 0.  A drop-in has to print the same lines.  tests/golden/make_cli_golden.py
records the reference's lines for each case below into tests/golden/cli_messages.json.

Left out on purpose: a flag that takes a value given as the last argument (``-f a.tri
-s``).  The reference reads past argv there and crashes; the GPU build reports it as
an invalid argument.
"""
from __future__ import annotations

import os

import re

import numpy as np

from ooc_svo_builder_gb300 import tri

# (executable, arguments); paths are relative to the folder make_inputs() fills
CASES = [
    ("svo_builder_binary", []),
    ("svo_builder_binary", ["-h"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-h"]),
    ("svo_builder_binary", ["-f", "x.obj"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-s", "100"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-s", "0"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-s", "-8"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-l", "1"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-l", "0"]),
    ("svo_builder_binary", ["-f", "missing.tri", "-v", "-l", "-5"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-d", "-5"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-q"]),
    ("svo_builder_binary", ["-f", "missing.tri"]),
    ("svo_builder_binary", ["-f", "missing.tri", "-c", "model"]),
    ("svo_builder", ["-f", "missing.tri", "-c", "foo"]),
    ("svo_builder", ["-f", "missing.tri", "-v", "-s", "64", "-l", "5", "-levels", "-c", "linear", "-d", "35"]),
    ("svo_builder", ["-f", "missing.tri", "-v", "-c", "fixed", "-c", "model"]),
    ("svo_builder", ["-s", "64", "-f", "geo.tri", "-s", "3"]),
    ("svo_builder", ["-f", "geo.tri", "-d", "50", "-f", "x.tri"]),
    ("svo_builder_binary", ["-f", "pay.tri"]),
    ("svo_builder", ["-f", "geo.tri"]),
    ("svo_builder_binary", ["-f", "nodata.tri"]),
    ("svo_builder", ["-f", "empty.tri"]),
    ("svo_builder", ["-f", "wrong.tri"]),
    ("svo_builder", ["-f", "noend.tri"]),
    ("svo_builder_binary", ["-f", "unknown.tri", "-v", "-s", "256", "-l", "2"]),
    ("svo_builder_binary", ["-f", "geo.tri", "-s", "512", "-l", "2"]),
    ("svo_builder", ["-f", "pay.tri", "-v", "-c", "normal", "-s", "64"]),
]


# Complete runs: every stdout line from the parameter parse to the timer block must
# match the reference's, timing values aside (full_run_lines).  Binary runs with -v
# use meshes sparse enough that no partition overflows the -d side-array: that
# verbose-only message (voxelizer.cpp:177-184) is not reproduced.
FULL_RUNS = [
    ("svo_builder_binary", ["-f", "soup.tri", "-s", "256", "-l", "2"]),
    ("svo_builder_binary", ["-f", "spheres.tri", "-s", "256", "-l", "2", "-v"]),
    ("svo_builder_binary", ["-f", "spheres.tri", "-s", "64"]),
    ("svo_builder", ["-f", "paysoup.tri", "-s", "256", "-l", "2", "-c", "linear", "-levels"]),
    ("svo_builder", ["-f", "pay.tri", "-s", "64", "-levels", "-v"]),
    ("svo_builder_binary", ["-f", "unknown.tri", "-v", "-s", "256", "-l", "2"]),
]


def case_id(exe: str, args) -> str:
    return " ".join([exe, *args])


def make_inputs(folder: str) -> None:
    """The .tri files the cases name: well-formed geometry-only and payload meshes,
    a header without its .tridata, and three malformed headers."""
    tri.write_tri(os.path.join(folder, "geo"), tri.random_tris(10, 1, False))
    tri.write_tri(os.path.join(folder, "pay"), tri.random_tris(10, 1, True))
    tri.write_tri(os.path.join(folder, "nodata"), tri.random_tris(10, 1, False))
    os.remove(os.path.join(folder, "nodata.tridata"))
    open(os.path.join(folder, "empty.tri"), "w").close()
    with open(os.path.join(folder, "wrong.tri"), "w") as f:
        f.write("#triangles 1\nEND\n")
    with open(os.path.join(folder, "noend.tri"), "w") as f:
        f.write("#tri 1\nntriangles 10\ncomment 3\n")
    open(os.path.join(folder, "noend.tridata"), "w").close()
    with open(os.path.join(folder, "unknown.tri"), "w") as f:
        f.write("#tri 1\nntriangles 0\nauthor someone else\ngeo_only 1\nbbox 0 0 0 2 2 2\nEND\n")
    open(os.path.join(folder, "unknown.tridata"), "w").close()
    # complete runs: a soup over 8 partitions, two small spheres in two octants (six
    # partitions without triangles), a payload soup
    tri.write_tri(os.path.join(folder, "soup"), tri.soup_tris(3000, 64, seed=5, sigma=1.0, n_spheres=3))
    a = tri.icosphere_tris(2, radius=0.04, jitter=0.0, seed=1)
    b = a.copy()
    a[:, :9] -= np.float32(0.25)
    b[:, [0, 3, 6]] += np.float32(0.3)
    tri.write_tri(os.path.join(folder, "spheres"), np.concatenate([a, b]))
    tri.write_tri(os.path.join(folder, "paysoup"), tri.soup_tris(2000, 64, seed=6, sigma=1.0, n_spheres=3,
                                                                 payload=True))


def diagnostics(stdout: str):
    """The lines a drop-in must reproduce: from the parameter parse up to the help
    text (whose example path and defaults differ on purpose), or up to and including
    the partition count, cut before the per-partition progress."""
    lines = stdout.splitlines()
    start = lines.index("Reading program parameters ...")
    out = []
    for ln in lines[start:]:
        if ln.startswith("Example:"):
            break
        if ln.startswith("Partitioning data into"):
            out.append(ln[:ln.index("partitions ... ") + len("partitions ... ")])
            break
        out.append(ln)
    return out


_TIME = re.compile(r"(time[\t ]*: )-?[0-9][0-9.e+-]*( m?s\.)$")


def full_run_lines(stdout: str):
    """A complete run's lines from the parameter parse on, with every timer value
    (main.cpp:219-241) replaced by <t>."""
    lines = stdout.splitlines()
    return [_TIME.sub(r"\1<t>\2", ln) for ln in lines[lines.index("Reading program parameters ..."):]]
