"""Device preprocessing of the cloth builder (edges, bend pairs, rest
lengths, inverse masses) against the numpy restatement: the same arrays bit
for bit on a jittered grid, a fan with a high-degree vertex, a triangle soup
with repeated and degenerate triangles and unused vertices, and a whole
cloth built either way."""
import numpy as np
import pytest

from xpbd_gb300 import scene

pytestmark = pytest.mark.gpu


def _jittered_grid(n, seed):
    pos, tris = scene.grid_mesh(n, 1.0, 0.0)
    rng = np.random.default_rng(seed)
    return (pos + rng.uniform(-2e-3, 2e-3, pos.shape)).astype(np.float32), tris


def _fan(k):
    ang = np.linspace(0.0, 2.0 * np.pi, k, endpoint=False)
    pos = np.concatenate([[[0.0, 0.0, 0.0]], np.stack([np.cos(ang), np.sin(ang), 0.1 * np.sin(3 * ang)], 1)]).astype(np.float32)
    tris = np.array([[0, 1 + i, 1 + (i + 1) % k] for i in range(k)], np.int32)
    return pos, tris


def _soup(seed):
    rng = np.random.default_rng(seed)
    pos = rng.normal(0.0, 0.3, (300, 3)).astype(np.float32)
    tris = rng.integers(0, 250, (700, 3)).astype(np.int32)  # vertices 250..299 unused
    tris[::37] = tris[::37][:, [0, 0, 1]]                    # degenerate (repeated corner)
    tris = np.concatenate([tris, tris[:50], tris[:20, ::-1]])  # repeated triangles, both windings
    return pos, tris


def _same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    a, b = np.ascontiguousarray(a).reshape(-1), np.ascontiguousarray(b).reshape(-1)
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("case", ["grid", "fan", "soup"])
@pytest.mark.parametrize("density", [0.2, 1.0e-12])
def test_device_inputs_equal_numpy(case, density, gpu_lib):
    pos, tris = {"grid": lambda: _jittered_grid(48, 1), "fan": lambda: _fan(97), "soup": lambda: _soup(2)}[case]()
    hard = np.zeros(len(pos), bool)
    hard[::41] = True
    e_ref, r_ref = scene.edge_constraints(tris, pos)
    inv_ref = scene.vertex_inverse_mass(pos, tris, density, hard).astype(np.float32)
    b_ref, br_ref = scene.bend_constraints(tris, pos)
    e, r, inv, b, br = scene.cloth_inputs_device(pos, tris, density, hard)
    assert _same_bits(e, e_ref.astype(np.int32))
    assert _same_bits(r, r_ref.astype(np.float32))
    assert _same_bits(inv, inv_ref)
    assert len(b_ref) > 0
    assert _same_bits(b, b_ref.astype(np.int32))
    assert _same_bits(br, br_ref.astype(np.float32))


def test_device_built_cloth_equals_numpy_built(gpu_lib):
    pos, tris = _jittered_grid(64, 3)
    w = np.zeros(len(pos), np.float32)
    w[[0, 63, 2000]] = [1.0, 1.0, 0.5]
    a = scene.build_cloth(pos, tris, 0.2, w, tether_slack=1.05)
    b = scene.build_cloth(pos, tris, 0.2, w, tether_slack=1.05, device=True)
    for f in a.__dataclass_fields__:
        assert _same_bits(getattr(a, f), getattr(b, f)), f


def test_device_prep_rejects_bad_index(gpu_lib):
    pos, tris = _fan(8)
    tris = tris.copy()
    tris[3, 1] = 99
    with pytest.raises(RuntimeError, match="triangle index 99 outside the 9 vertices"):
        scene.cloth_inputs_device(pos, tris, 0.2, np.zeros(len(pos), bool))
