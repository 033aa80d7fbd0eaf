"""A seeded mix of inputs and flags, each built on the GPU through ooc_build and compared
with the oracle on the same input.  The oracle is pinned to the reference build on the
same mix in the CPU suite."""
import pytest

import golden_cases
import pyoracle
from ooc_svo_builder_gb300 import make_params, octree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("i", range(golden_cases.N_SEEDED))
def test_seeded_cases_match_oracle(builder, i):
    """The seeded mix the oracle is pinned on against the reference build: inside, outside
    and lattice-aligned inputs, sub-voxel triangles, soups and spheres, gridsize 1 to 256,
    1 to 64 partitions, every colour mode, with and without -levels."""
    t, N, limit, payload, color, levels, kind = golden_cases.seeded_case(i)
    got = builder.build(t, make_params(N, limit, geometry_only=not payload, color=color, levels=levels))
    nodes, data, info = pyoracle.build(t, N, limit, color=color, levels=levels)
    d = octree.diff(got.tree, octree.Octree(N, nodes, data))
    assert not d, kind + "\n" + "\n".join(d)
    assert got.info["n_filled"] == info["n_filled"]
