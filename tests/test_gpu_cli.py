"""Complete runs of the drop-in CLIs on the GPU: every stdout line from the parameter
parse to the timer block equals the reference's recorded line (main.cpp:281-398 with
partitioner.cpp:64-71, trip_tools.h:28-40 and printTimerInfo, main.cpp:219-241), timer
values aside, and the octree files equal the oracle's."""
import json
import os
import subprocess

import pytest

import cli_cases
import ooc_svo_builder_gb300 as ooc
import pyoracle
from ooc_svo_builder_gb300 import octree, tri

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cli_full_runs.json")
BIN = os.path.join(os.path.dirname(ooc.LIB_PATH), "bin")
FULL = json.load(open(GOLDEN))


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("cli_full"))
    cli_cases.make_inputs(d)
    return d


def _flag(args, name, default):
    return args[args.index(name) + 1] if name in args else default


@pytest.mark.parametrize("exe,args", cli_cases.FULL_RUNS, ids=[cli_cases.case_id(e, a) for e, a in cli_cases.FULL_RUNS])
def test_complete_run_matches_reference(inputs, exe, args):
    want = FULL[cli_cases.case_id(exe, args)]
    r = subprocess.run([os.path.join(BIN, exe), *args], cwd=inputs, stdout=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == want["status"] == 0
    got = cli_cases.full_run_lines(r.stdout)
    assert got == want["lines"], "\n".join(
        "%r != %r" % (g, w) for g, w in zip(got + [None] * len(want["lines"]), want["lines"] + [None] * len(got))
        if g != w)
    # the files it wrote equal the oracle's on the same mesh and flags
    path = os.path.join(inputs, _flag(args, "-f", None))
    N, limit = int(_flag(args, "-s", "1024")), int(_flag(args, "-l", "2048"))
    h, tris = tri.read_tri(path)
    P = ooc.estimate_partitions(N, limit)
    got_tree = octree.read_octree(os.path.join(inputs, "%s%d_%d" % (path[:-4], N, P)))
    nodes, data, _ = pyoracle.build(tris, N, limit, color=_flag(args, "-c", "model"), levels="-levels" in args,
                                    bbox_min=h.bbox_min, bbox_max=h.bbox_max)
    d = octree.diff(got_tree, octree.Octree(N, nodes, data))
    assert not d, d
