"""GPU path against the golden fixtures produced by the reference build (tests/golden/)."""
import pytest

import golden_cases
from ooc_svo_builder_gb300 import make_params, octree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_cases.names())
def test_gpu_matches_golden(builder, name):
    tris, meta, want = golden_cases.load(name)
    prm = make_params(meta["s"], meta.get("l", 2048), geometry_only=tris.shape[1] == 9,
                      color=meta.get("c", "model"), levels=meta.get("levels", False))
    got = builder.build(tris, prm)
    d = octree.diff(got.tree, want)
    assert not d, "\n".join(d)
    assert got.info["n_partitions"] == meta["n_partitions"]
    assert got.info["n_filled"] == meta["n_filled"]


@pytest.mark.parametrize("name", golden_cases.names())
def test_cli_file_to_file_matches_golden(name, tmp_path):
    # the drop-in executables, file to file: .tri/.tridata in, <base><N>_<P>.octree* out
    import os
    import subprocess

    import ooc_svo_builder_gb300 as ooc
    from ooc_svo_builder_gb300 import tri

    tris, meta, want = golden_cases.load(name)
    binary = tris.shape[1] == 9
    tri.write_tri(str(tmp_path / "mesh"), tris)
    exe = os.path.join(os.path.dirname(ooc.LIB_PATH), "bin", "svo_builder_binary" if binary else "svo_builder")
    cmd = [exe, "-f", str(tmp_path / "mesh.tri"), "-s", str(meta["s"]), "-l", str(meta.get("l", 2048))]
    if meta.get("levels"):
        cmd.append("-levels")
    if not binary and meta.get("c", "model") != "model":
        cmd += ["-c", meta["c"]]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    base = str(tmp_path / ("mesh%d_%d" % (meta["s"], meta["n_partitions"])))
    got = octree.read_octree(base)
    d = octree.diff(got, want)
    assert not d, "\n".join(d)
    with open(base + ".octree") as f:
        assert f.read() == meta["header"]  # the reference's own header text
