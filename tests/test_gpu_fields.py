"""Prediction extras on the GPU against the oracle: volume pressure along
the vertex normals and every force-field kind, alone and inside a batch.

Kinds whose arithmetic uses only IEEE basic operations must match bit for
bit; kinds that call powf (distance falloff powers) may differ from the
host libm in the last place, so they are held to the stated tolerance
(1e-4 x cloth extent per frame).  The noise of wind and texture fields
hashes fract(sin(x) * 43758.5453), which turns a last-place difference of
sin into an unrelated value: the GPU keeps CUDA's sinf (the reference's
device function), so those are checked for determinism and bounds, not
against the host oracle."""
import ctypes

import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import F3, NativeForceField, NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu


def _field(kind, **kw):
    f = NativeForceField()
    f.type = kind
    f.strength = kw.get("strength", 4.0)
    f.origin = F3(*kw.get("origin", (0.1, -0.2, 0.6)))
    f.direction = F3(*kw.get("direction", (0.3, 0.2, 1.0)))
    f.axis = F3(*kw.get("axis", (0.0, 0.0, 1.0)))
    f.apply_to_location = 1
    for k in ("use_min_distance", "use_max_distance", "seed", "use_radial_min", "use_radial_max", "use_2d_force",
              "use_global_coords"):
        setattr(f, k, int(kw.get(k, 0)))
    for k in ("falloff_power", "distance_min", "distance_max", "radial_min", "radial_max", "noise", "linear_drag",
              "quadratic_drag", "harmonic_damping", "flow", "size", "rest_length", "radial_falloff", "texture_nabla"):
        setattr(f, k, float(kw.get(k, 0.0)))
    return f


EXACT = {
    "wind": [_field(1, strength=6.0)],
    "force_2d_maxdist": [_field(2, use_2d_force=1, use_max_distance=1, distance_max=1.5, distance_min=0.1)],
    "vortex_flow": [_field(3, strength=3.0, flow=0.5)],
    "turbulence": [_field(4, strength=5.0, size=0.4)],
    "charge_radial": [_field(5, strength=0.5, use_radial_max=1, radial_max=2.0, radial_min=0.2)],
    "harmonic": [_field(6, strength=20.0, rest_length=0.3, harmonic_damping=0.4)],
    "lennard_jones": [_field(7, strength=0.01, rest_length=0.2)],
    "magnet_drag": [_field(8, strength=2.0), _field(9, strength=0.8, linear_drag=0.3, quadratic_drag=0.1)],
}
TOLERANT = {
    "force_falloff_power": [_field(2, use_min_distance=1, distance_min=0.2, falloff_power=2.0)],
}


def _scene():
    sc = scene.plain_grid_scene(16, 4)
    return sc


def _run(sc, fields, frames, exact, oracle_lib):
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    arr = (NativeForceField * max(len(fields), 1))(*fields)
    gpu.update_force_fields(fields)
    ora.update_force_fields(arr if fields else [])
    moved = 0.0
    for f in range(frames):
        gpu.step(sc.substeps, sc.iterations, diagnostics=False, synchronize=True)
        ora.step(sc.substeps, sc.iterations)
        pg, po = gpu.download_positions(), ora.download_positions()
        assert np.isfinite(pg).all()
        err = float(np.abs(pg - po).max())
        assert err <= 1e-4 * sc.extent, (f, err)
        if exact:
            assert np.array_equal(pg, po), (f, err)
        moved = float(np.abs(pg - sc.cloth.positions_world).max())
    return moved


@pytest.mark.parametrize("name", sorted(EXACT))
def test_force_fields_bit_exact(name, gpu_lib, oracle_lib):
    sc = _scene()
    _run(sc, EXACT[name], 4, True, oracle_lib)


@pytest.mark.parametrize("name", sorted(TOLERANT))
def test_force_fields_within_tolerance(name, gpu_lib, oracle_lib):
    sc = _scene()
    _run(sc, TOLERANT[name], 4, False, oracle_lib)


def test_fields_change_the_motion(gpu_lib, oracle_lib):
    sc = _scene()
    plain = _run(sc, [], 3, True, oracle_lib)
    pushed = _run(_scene(), [_field(2, strength=30.0)], 3, True, oracle_lib)
    assert abs(pushed - plain) > 1e-3


@pytest.mark.parametrize("strength", [0.2, 1.5])
def test_volume_pressure_bit_exact(strength, gpu_lib, oracle_lib):
    sc = scene.plain_grid_scene(16, 4)
    sc.options.use_volume_pressure = True
    sc.options.pressure_strength = strength
    _run(sc, [], 4, True, oracle_lib)


def test_pressure_and_fields_in_a_batch(gpu_lib, oracle_lib):
    """Per-cloth fields and pressure inside a batch: each cloth equals the
    oracle run alone."""
    scs = [scene.plain_grid_scene(n, 3) for n in (10, 14, 12)]
    scs[0].options.use_volume_pressure = True
    scs[0].options.pressure_strength = 0.8
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    fields = {1: [_field(3, strength=3.0)], 2: [_field(6, strength=10.0, rest_length=0.2)]}
    oras = [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    for k, fl in fields.items():
        batch.update_cloth_force_fields(k, fl)
        oras[k].update_force_fields((NativeForceField * len(fl))(*fl))
    for _ in range(3):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), k


def test_force_field_limits(gpu_lib):
    sc = _scene()
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    from xpbd_gb300.native import NativeSolverError

    with pytest.raises(NativeSolverError, match="force field count exceeds SSBL maximum"):
        gpu.update_force_fields([_field(2)] * 65)
    gpu.update_force_fields([_field(2)] * 64)
    gpu.step(10, 2)
    assert gpu.diagnostics()["force_field_count"] == 64


@pytest.mark.parametrize("field", [_field(10, strength=3.0, noise=2.0, seed=5), _field(1, strength=6.0, noise=0.5, seed=3)],
                         ids=["texture", "wind_noise"])
def test_noise_fields_deterministic_and_bounded(field, gpu_lib):
    sc = _scene()
    out = []
    for _ in range(2):
        gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
        gpu.update_force_fields([field])
        for _ in range(3):
            gpu.step(sc.substeps, sc.iterations, diagnostics=False, synchronize=True)
        out.append(gpu.download_positions().copy())
    assert np.array_equal(out[0], out[1])
    assert np.isfinite(out[0]).all()
    # the texture push is at most |strength| * sqrt(3) per unit mass: bounded drift
    assert float(np.abs(out[0] - sc.cloth.positions_world).max()) < 1.0
