"""Native input preprocessing (greedy colouring, bend pairs) against the
Python restatement of the reference's input pipeline (xpbd_core.py:730-747,
828-859): identical arrays on grids, random meshes, non-manifold edges and
out-of-range indices.  Host-only code: runs without a GPU."""
import numpy as np
import pytest

from xpbd_gb300 import scene


@pytest.fixture(scope="module")
def prep():
    from xpbd_gb300 import build

    build.build()
    scene._PREP = None
    lib = scene._native_prep()
    assert lib is not None, "library without the preprocessing entry points"
    return lib


def _random_mesh(rng, V, T):
    tris = rng.integers(0, V, size=(T, 3)).astype(np.int32)
    return tris


@pytest.mark.parametrize("n", [2, 3, 17, 64])
def test_grid_bends_and_colours(prep, n):
    pos, tris = scene.grid_mesh(n, 1.0, 0.0)
    assert np.array_equal(scene.bend_pairs(tris), scene.bend_pairs_py(tris))
    edges, _ = scene.edge_constraints(tris, pos)
    assert np.array_equal(scene.greedy_colors(edges, len(pos)), scene.greedy_colors_py(edges, len(pos)))
    bends = scene.bend_pairs(tris)
    assert np.array_equal(scene.greedy_colors(bends, len(pos)), scene.greedy_colors_py(bends, len(pos)))


@pytest.mark.parametrize("seed", range(6))
def test_random_meshes(prep, seed):
    rng = np.random.default_rng(seed)
    V = int(rng.integers(3, 60))
    tris = _random_mesh(rng, V, int(rng.integers(1, 200)))  # degenerate and non-manifold triangles included
    assert np.array_equal(scene.bend_pairs(tris), scene.bend_pairs_py(tris))
    pairs = rng.integers(-3, V + 3, size=(int(rng.integers(1, 400)), 2)).astype(np.int32)  # out-of-range endpoints
    assert np.array_equal(scene.greedy_colors(pairs, V), scene.greedy_colors_py(pairs, V))


def test_more_than_64_colours(prep):
    # a star: every pair shares vertex 0, so pair k takes colour k
    pairs = np.stack([np.zeros(150, np.int32), np.arange(1, 151, dtype=np.int32)], axis=1)
    c = scene.greedy_colors(pairs, 151)
    assert np.array_equal(c, np.arange(150))
    assert np.array_equal(c, scene.greedy_colors_py(pairs, 151))
