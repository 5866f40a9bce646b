"""Restated input builders and ABI layout against fixtures generated from the
reference's own Python modules (tests/golden/gen_golden.py)."""
import ctypes
import json
import os
import subprocess

import numpy as np

from xpbd_gb300 import native, scene

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
ROOT = os.path.dirname(HERE)


def test_topology_matches_reference_builders():
    g = np.load(os.path.join(GOLD, "topology_grid32.npz"))
    pos, tris = scene.grid_mesh(32, 1.0, 0.0)
    assert np.array_equal(pos, g["positions"]) and np.array_equal(tris, g["triangles"])
    e, er = scene.edge_constraints(tris, pos)
    e, er, eo = scene.color_constraints(e, er, len(pos))
    assert np.array_equal(e, g["edges"]) and np.array_equal(er, g["edge_rest"]) and np.array_equal(eo, g["edge_offsets"])
    b, br = scene.bend_constraints(tris, pos)
    b, br, bo = scene.color_constraints(b, br, len(pos))
    assert np.array_equal(b, g["bends"]) and np.array_equal(br, g["bend_rest"]) and np.array_equal(bo, g["bend_offsets"])
    w = np.zeros(len(pos), np.float32)
    w[31 * 32] = 1.0
    w[-1] = 1.0
    hard = w >= 0.75
    inv = scene.vertex_inverse_mass(pos, tris, 0.2, hard).astype(np.float32)
    assert np.array_equal(inv, g["inv_mass"])
    lra, lr = scene.hidden_tethers(pos, hard, 1.0)
    assert np.array_equal(lra, g["lra"]) and np.array_equal(lr, g["lra_rest"])
    for row in g["hardness"]:
        d = scene.derive_hardness(row[0])
        assert np.isclose(d["stretch_compliance"], row[1], rtol=1e-12)
        assert np.isclose(d["bend_compliance"], row[2], rtol=1e-12)
        assert np.isclose(d["hidden_tether_compliance"], row[3], rtol=1e-12)
        assert np.isclose(d["hidden_tether_slack"], row[4], rtol=1e-12)
        assert d["hidden_tether_enabled"] == bool(row[5])
    # sizes quoted for the 32 x 32 case
    assert (len(pos), len(tris), len(e), len(b)) == (1024, 1922, 2945, 2821)


def _layout(struct):
    return [[n, getattr(struct, n).offset, getattr(struct, n).size] for n, _ in struct._fields_]


def test_ctypes_mirror_matches_reference_bridge_layout():
    gold = json.load(open(os.path.join(GOLD, "abi_layout.json")))
    pairs = {
        "SsblXpbdConfig": native.NativeConfig, "SsblXpbdDiagnostics": native.NativeDiagnostics,
        "SsblXpbdMesh": native.NativeMesh, "SsblXpbdRuntimeColliders": native.NativeRuntimeColliders,
        "SsblXpbdForceField": native.NativeForceField, "SsblXpbdFrameInputs": native.NativeFrameInputs,
    }
    for name, cls in pairs.items():
        assert ctypes.sizeof(cls) == gold[name]["size"], name
        assert _layout(cls) == gold[name]["fields"], name


def test_config_bytes_match_reference_bridge():
    gold = json.load(open(os.path.join(GOLD, "abi_layout.json")))
    g = np.load(os.path.join(GOLD, "topology_grid32.npz"))
    cloth = scene.ClothData(
        positions_world=g["positions"], inv_mass=g["inv_mass"], triangles=g["triangles"], edges=g["edges"],
        edge_rest_lengths=g["edge_rest"], edge_color_offsets=g["edge_offsets"], bends=g["bends"],
        bend_rest_lengths=g["bend_rest"], bend_color_offsets=g["bend_offsets"], lra_edges=np.empty((0, 2), np.int32),
        lra_rest_lengths=np.empty(0, np.float32), lra_color_offsets=np.asarray([0], np.int32),
        pin_indices=np.empty(0, np.int32), pin_targets_world=np.empty((0, 3), np.float32), pin_weights=np.empty(0, np.float32))
    opt = scene.SolverOptions(dt=1 / 60, damping=0.99, stretch_compliance=1e-7, bend_compliance=1e-4, collision_margin=0.005,
                              use_ground=True, ground_height=-1.0, use_sphere=True, sphere_center=(0.1, 0.2, 0.3),
                              sphere_radius=0.3, self_collision=True, self_collision_mode=2, cloth_thickness=0.002,
                              self_collision_interval=1, max_self_collision_neighbors=64, fast_self_collision_passes=4,
                              contact_friction=0.3, contact_tangent_damping=0.2, static_sdf_max_resolution=64)
    cfg = native.config_from_options(cloth, opt, np.zeros((12, 3, 3), np.float32))
    assert bytes(cfg).hex() == gold["config_bytes_hex"]


def test_c_header_layout_matches_reference_bridge(tmp_path):
    """The public header compiles to the same offsets the reference bridge uses."""
    gold = json.load(open(os.path.join(GOLD, "abi_layout.json")))
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ssbl_xpbd_cuda.h"', "int main(void){"]
    for name, spec in gold.items():
        if not isinstance(spec, dict):
            continue
        lines.append(f'printf("{name} __sizeof__ %zu\\n", sizeof({name}));')
        for f, _, _ in spec["fields"]:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for name, spec in gold.items():
        if not isinstance(spec, dict):
            continue
        assert got[(name, "__sizeof__")] == spec["size"], name
        for f, off, _ in spec["fields"]:
            assert got[(name, f)] == off, (name, f)
