"""The test DAG builder (tests/dagbuild.py) against the library's voxel
lookup, and the compact store and oracle on random DAGs (CPU only)."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
from dagbuild import build_dag, random_voxels, random_rays
from test_compact_layout import check_equivalent


@pytest.mark.parametrize("seed", range(6))
def test_random_dag_voxels_and_compact_store(seed):
    rng = np.random.default_rng(seed)
    edge = 1 << int(rng.integers(2, 6))
    vox = random_voxels(rng, edge)
    origin = tuple(int(x) * edge for x in rng.integers(-(1 << 20) // edge, (1 << 20) // edge, 3))
    nodes, root = build_dag(vox, origin)
    cbq.validate(nodes, root)
    for x, y, z in rng.integers(0, edge, (300, 3)):
        assert cbq.dag_voxel(nodes, root, int(x) + origin[0], int(y) + origin[1], int(z) + origin[2]) == vox[z, y, x]
    check_equivalent(nodes, root)


def test_uniform_and_empty_volumes():
    for fill in (0, 9):
        vox = np.full((8, 8, 8), fill, np.uint8)
        nodes, root = build_dag(vox, (64, -128, 8))
        cbq.validate(nodes, root)
        assert cbq.dag_voxel(nodes, root, 65, -125, 12) == fill
        check_equivalent(nodes, root)


def test_random_rays_shapes():
    rng = np.random.default_rng(1)
    o, d = random_rays(rng, (16, 32, -48), 16, 1000)
    assert o.shape == (1000, 4) and d.shape == (1000, 4)
    assert np.allclose(np.linalg.norm(d[:, :3], axis=1), 1.0, atol=1e-5)
    assert ((d[:, :3] == 0).sum(axis=1) == 2).any()  # axis-aligned rays present
