"""The free-block bookkeeping of the server's pinned result reserve (csrc/ooc_extents.h),
checked on the host: a randomised take/put sequence per seed (extents_check.cpp) must never
hand out overlapping or misaligned blocks, must account for every byte, and must merge the
region back into one extent once every block is returned."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ooc_svo_builder_gb300", "csrc")


def test_extents_random_sequences(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "extents_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "extents_check.cpp"), "-o", exe],
                   check=True)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert p.stdout.strip().endswith("ok")
