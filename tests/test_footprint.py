"""The serving loop admits requests by a computed footprint whose node term rests on a
per-triangle bound of the voxels a triangle can set (csrc/ooc_footprint.h).  Checked on
the host: for each of 300 seeded triangles of every size and orientation (slivers, needles,
flat and diagonal ones, triangles crossing the grid's edge), the oracle's voxel count of
that triangle alone must not exceed the bound."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ooc_svo_builder_gb300", "csrc")


def triangles(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = i % 5
        c = rng.uniform(0.05, 0.95, size=3)
        if kind == 0:    # small, any orientation
            t = c + rng.normal(0, 0.01, size=(3, 3))
        elif kind == 1:  # large
            t = c + rng.normal(0, 0.25, size=(3, 3))
        elif kind == 2:  # needle: two vertices close together
            a = c + rng.normal(0, 0.3, size=3)
            t = np.stack([c, a, a + rng.normal(0, 0.002, size=3)])
        elif kind == 3:  # flat in one axis, wide in the other two
            t = c + rng.normal(0, 0.3, size=(3, 3))
            t[:, rng.integers(0, 3)] = c[0]
        else:            # crossing the grid's faces
            t = rng.uniform(-0.3, 1.3, size=(3, 3))
        out.append(t.astype(np.float32).reshape(9))
    return np.asarray(out, dtype=np.float32)


@pytest.mark.parametrize("N", [32, 128])
def test_voxel_bound_covers_the_oracle(tmp_path, N):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "footprint_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "footprint_check.cpp"), "-o", exe],
                   check=True)
    tris = triangles(300, seed=N)
    unit_div = np.float32(1.0) / (np.float32(1.0) / np.float32(N))  # bbox [0, 1]^3, as make_params
    lines = ["%d %s" % (N, float(unit_div).hex())] + [" ".join(float(x).hex() for x in t) for t in tris]
    p = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    bounds = [float(x) for x in p.stdout.split()]
    assert len(bounds) == len(tris)
    tight = 0
    for t, bound in zip(tris, bounds):
        filled = pyoracle.build(t.reshape(1, 9), N, 2048)[2]["n_filled"]
        assert filled <= bound, (t.tolist(), filled, bound)
        tight += filled > 0.5 * bound
    assert tight > 0  # the bound is not vacuous on every case
