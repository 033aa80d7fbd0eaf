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
