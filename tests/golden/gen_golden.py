"""Generate the golden fixtures of this directory from the reference itself.

Run in a container where the reference checkout is present:

    python tests/golden/gen_golden.py /path/to/ssbl-cuda-xpbd

It imports the reference's own Python modules (xpbd_core.py for the solver
inputs, native_backend.py for the ctypes mirror of the ABI41 structs) with
minimal stand-ins for the Blender modules they import at load time, and
records:

* ``topology_grid32.npz`` -- edges, edge colours, bends, bend colours,
  inverse masses and hidden tethers of the 32 x 32 plain-XPBD grid with two
  hard-pinned corners, plus hardness-derived compliances;
* ``abi_layout.json`` -- size and field offsets of every ABI41 struct as the
  reference bridge lays them out, and the bytes of the config it builds for
  a fixed SolverOptions.

Nothing in the test suite imports the reference at run time; the tests read
these files only.
"""
from __future__ import annotations

import ctypes
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _stub_blender():
    bpy = types.ModuleType("bpy")
    bpy.types = types.SimpleNamespace(Object=object, Mesh=object, Depsgraph=object, Context=object, Scene=object)
    translations = types.SimpleNamespace(pgettext_tip=lambda s: s, pgettext_iface=lambda s: s)
    bpy.app = types.SimpleNamespace(translations=translations)
    bpy.context = types.SimpleNamespace()
    sys.modules["bpy"] = bpy
    sys.modules["bpy.app"] = bpy.app
    sys.modules["bpy.app.translations"] = translations
    sys.modules["bpy.types"] = bpy.types
    sys.modules["bmesh"] = types.ModuleType("bmesh")
    mu = types.ModuleType("mathutils")
    mu.Matrix = mu.Vector = object
    mu.kdtree = types.SimpleNamespace()
    sys.modules["mathutils"] = mu


def _import_reference(root: str):
    _stub_blender()
    spec = importlib.util.spec_from_file_location("ssbl_reference", os.path.join(root, "__init__.py"),
                                                  submodule_search_locations=[root])
    pkg = importlib.util.module_from_spec(spec)
    sys.modules["ssbl_reference"] = pkg  # package shell only; __init__ (Blender UI) is not executed
    mods = {}
    for name in ("force_fields", "xpbd_core", "native_backend"):
        s = importlib.util.spec_from_file_location(f"ssbl_reference.{name}", os.path.join(root, f"{name}.py"))
        m = importlib.util.module_from_spec(s)
        sys.modules[f"ssbl_reference.{name}"] = m
        s.loader.exec_module(m)
        mods[name] = m
    return mods


def _layout(struct) -> dict:
    return {"size": ctypes.sizeof(struct),
            "fields": [[name, getattr(struct, name).offset, getattr(struct, name).size] for name, _ in struct._fields_]}


def main(root: str) -> None:
    mods = _import_reference(root)
    xc, nb = mods["xpbd_core"], mods["native_backend"]
    sys.path.insert(0, os.path.join(REPO, "ssbl-cuda-xpbd_gb300"))
    from xpbd_gb300.scene import grid_mesh

    pos, tris = grid_mesh(32, 1.0, 0.0)
    world = np.ascontiguousarray(pos, np.float32)
    n = len(world)
    w = np.zeros(n, np.float32)
    w[(32 - 1) * 32] = 1.0
    w[n - 1] = 1.0
    hard = w >= xc.PIN_HARD_WEIGHT_THRESHOLD
    edges, edge_rest = xc.edge_constraints(tris, world)
    edges, edge_rest, edge_off = xc.color_distance_constraints(edges, edge_rest, n)
    bends, bend_rest = xc.bend_constraints(tris, world)
    bends, bend_rest, bend_off = xc.color_distance_constraints(bends, bend_rest, n)
    lra, lra_rest = xc.hidden_tether_constraints(world, hard, 1.0)
    inv = xc.vertex_inverse_mass(world, tris, 0.2, hard)
    hs = [xc.derive_hardness_settings(h) for h in (0.0, 0.4, 0.8, 1.0)]
    np.savez_compressed(
        os.path.join(HERE, "topology_grid32.npz"),
        positions=world, triangles=tris, edges=np.asarray(edges, np.int32), edge_rest=np.asarray(edge_rest, np.float32),
        edge_offsets=np.asarray(edge_off, np.int32), bends=np.asarray(bends, np.int32),
        bend_rest=np.asarray(bend_rest, np.float32), bend_offsets=np.asarray(bend_off, np.int32),
        lra=np.asarray(lra, np.int32), lra_rest=np.asarray(lra_rest, np.float32), inv_mass=np.asarray(inv, np.float32),
        hardness=np.array([[h.hardness, h.stretch_compliance, h.bend_compliance, h.hidden_tether_compliance,
                            h.hidden_tether_slack, float(h.hidden_tether_enabled)] for h in hs], np.float64),
    )

    layout = {name: _layout(getattr(nb, cls)) for name, cls in (
        ("SsblXpbdConfig", "_NativeConfig"), ("SsblXpbdDiagnostics", "_NativeDiagnostics"),
        ("SsblXpbdMesh", "_NativeMesh"), ("SsblXpbdRuntimeColliders", "_NativeRuntimeColliders"),
        ("SsblXpbdForceField", "_NativeForceField"), ("SsblXpbdFrameInputs", "_NativeFrameInputs"),
        ("SsblXpbdGlobalDynamicSceneInputs", "_NativeGlobalDynamicSceneInputs"))}
    opts = xc.SolverOptions(
        dt=1.0 / 60.0, damping=0.99, gravity=np.array([0.0, 0.0, -9.81], np.float32), stretch_compliance=1e-7,
        stretch_optimization_enabled=False, stretch_optimization_strength=0.0, bend_compliance=1e-4,
        lra_compliance=0.0, collision_margin=0.005, use_ground=True, ground_height=-1.0, use_wall=False,
        wall_origin=np.zeros(3, np.float32), wall_normal=np.array([0, 0, 1], np.float32), use_sphere=True,
        sphere_center=np.array([0.1, 0.2, 0.3], np.float32), sphere_radius=0.3, self_collision=True,
        self_collision_mode=2, cloth_thickness=0.002, self_collision_distance=0.0, self_collision_interval=1,
        max_self_collision_neighbors=64, fast_self_collision_passes=4, use_volume_pressure=False,
        volume_compliance=1e-6, pressure_strength=0.0, volume_target_scale=1.0, volume_solve_interval=1,
        self_probe_interval=1, self_surface_pair_interval=1, jitter_stabilizer_enabled=False, contact_friction=0.3,
        contact_tangent_damping=0.2, contact_compliance=0.0, static_sdf_voxel_size=0.0, static_sdf_band_voxels=4,
        static_sdf_max_resolution=64)
    cloth = xc.ClothBuildData(
        positions_world=world, inv_mass=np.asarray(inv, np.float32), triangles=tris, edges=edges,
        edge_rest_lengths=edge_rest, edge_color_offsets=edge_off, bends=bends, bend_rest_lengths=bend_rest,
        bend_color_offsets=bend_off, lra_edges=np.empty((0, 2), np.int32), lra_rest_lengths=np.empty(0, np.float32),
        lra_color_offsets=np.asarray([0], np.int32), pin_indices=np.flatnonzero(hard).astype(np.int32),
        pin_targets_world=world[hard], matrix_world_inv=np.eye(4, dtype=np.float32), rest_volume=0.0)
    cfg = nb._config_from_options(cloth, opts, np.zeros((12, 3, 3), np.float32))
    layout["config_bytes_hex"] = bytes(cfg).hex()
    layout["capability_bits"] = [nb._CAP_STRETCH_OPTIMIZATION, nb._CAP_PIN_WEIGHTS, nb._CAP_GLOBAL_DYNAMIC_SCENE]
    with open(os.path.join(HERE, "abi_layout.json"), "w") as f:
        json.dump(layout, f, indent=1)
    print("wrote", os.path.join(HERE, "topology_grid32.npz"), "and abi_layout.json")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SSBL_REFERENCE_ROOT", "")
    if not root:
        sys.exit("usage: gen_golden.py REFERENCE_CHECKOUT (or set SSBL_REFERENCE_ROOT)")
    main(root)
