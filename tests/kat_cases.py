"""Known-answer cases of the reference's native smoke test, restated.

Each case reproduces the inputs and the directional assertions of one block
of native/smoke/abi41_smoke.cpp (cited per case) and runs against any
backend with the NativeXpbdSolver method names: the GPU library or the CPU
oracle.  The reference holds no golden vectors for the step; these
inequalities and exact pin checks are its known answers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from xpbd_gb300.native import NativeConfig, NativeMesh, _fp, _ip


def _cfg(**kw) -> NativeConfig:
    c = NativeConfig()
    for k, v in kw.items():
        if k in ("gravity", "wall_origin", "wall_normal", "sphere_center"):
            setattr(c, k, (ctypes.c_float * 3)(*v))
        else:
            setattr(c, k, v)
    return c


def _mesh(**arrays):
    keep = {k: np.ascontiguousarray(v, np.int32 if k in ("edges", "bends", "lra_edges", "triangles") else np.float32)
            for k, v in arrays.items()}
    m = NativeMesh()
    for k, a in keep.items():
        setattr(m, k, _ip(a) if a.dtype == np.int32 else _fp(a))
    return m, keep


def _dist(p, a, b):
    return float(np.linalg.norm(p[a] - p[b]))


class Case:
    def __init__(self, name, cfg, mesh, keep, pins=None):
        self.name, self.cfg, self.mesh, self.keep, self.pins = name, cfg, mesh, keep, pins


def static_sdf_plane():
    """abi41_smoke.cpp:71-127: a vertex 2 cm above a plane with 8 cm margin is
    pushed up by more than 1 cm; the pinned vertex stays within 1e-5."""
    pos = np.array([[0, 0, 0.02], [0.25, 0, 0.02]], np.float32)
    plane = np.array([[-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    cfg = _cfg(vertex_count=2, static_triangle_count=2, dt=1 / 60, damping=1.0, collision_margin=0.08,
               cloth_thickness=0.02, static_sdf_voxel_size=0.04, static_sdf_band_voxels=2, static_sdf_max_resolution=48)
    m, keep = _mesh(positions=pos, inv_mass=[1.0, 0.0], static_triangles=plane)

    def run(solver):
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert out[0, 2] > pos[0, 2] + 0.01, out
        assert abs(out[1, 2] - pos[1, 2]) <= 1e-5
        return out

    return Case("static_sdf_plane", cfg, m, keep), run


def box_triangles(h):
    t = [
        [[-h, -h, -h], [-h, h, -h], [h, h, -h]], [[-h, -h, -h], [h, h, -h], [h, -h, -h]],
        [[-h, -h, h], [h, -h, h], [h, h, h]], [[-h, -h, h], [h, h, h], [-h, h, h]],
        [[-h, -h, -h], [h, -h, -h], [h, -h, h]], [[-h, -h, -h], [h, -h, h], [-h, -h, h]],
        [[-h, h, -h], [-h, h, h], [h, h, h]], [[-h, h, -h], [h, h, h], [h, h, -h]],
        [[-h, -h, -h], [-h, -h, h], [-h, h, h]], [[-h, -h, -h], [-h, h, h], [-h, h, -h]],
        [[h, -h, -h], [h, h, -h], [h, h, h]], [[h, -h, -h], [h, h, h], [h, -h, h]],
    ]
    return np.asarray(t, np.float32)


def static_sdf_box():
    """abi41_smoke.cpp:129-178: after switching the collider to a closed 1 m
    box, a vertex inside it is pushed out by more than 5 cm."""
    case, run_plane = static_sdf_plane()

    def run(solver):
        run_plane(solver)
        box_pos = np.array([[0.11, 0.07, 0.03], [0.20, 0.0, 0.0]], np.float32)
        solver.update_positions(box_pos)
        solver.update_static_triangles(box_triangles(0.5))
        solver.step(1, 2)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert np.linalg.norm(out[0] - box_pos[0]) > 0.05, out
        return out

    case.name = "static_sdf_box"
    return case, run


def self_vv():
    """abi41_smoke.cpp:227-311: two vertices 3 cm apart with a 10 cm thickness
    separate (gap grows by more than 1e-4) under fast self collision."""
    n = 600
    pos = np.zeros((n, 3), np.float32)
    pos[:, 0] = np.arange(n, dtype=np.float32)
    cfg = _cfg(vertex_count=n, dt=1 / 60, damping=1.0, gravity=(0, 0, 0), self_collision=1, self_collision_mode=1,
               cloth_thickness=0.10, collision_margin=0.0, max_self_collision_neighbors=32)
    m, keep = _mesh(positions=pos, inv_mass=np.ones(n))

    def run(solver):
        close = pos.copy()
        close[n - 1, 0] = 0.03
        g0 = _dist(close, 0, n - 1)
        solver.update_positions(close)
        solver.step(1, 6)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert _dist(out, 0, n - 1) > g0 + 1e-4
        return out

    return Case("self_vv", cfg, m, keep), run


def self_vt():
    """abi41_smoke.cpp:313-446: a vertex 3 cm above a pinned triangle is pushed
    up by more than 1e-4."""
    n = 600
    pos = np.zeros((n, 3), np.float32)
    pos[0], pos[1], pos[2] = (-1, -1, 0), (1, -1, 0), (0, 1, 0)
    inv = np.ones(n, np.float32)
    inv[:3] = 0
    for i in range(3, n):
        pos[i] = (20.0 + i, 20.0 + (i % 7) * 0.25, (i % 5) * 0.20)
    pos[n - 1] = (5, 5, 1)
    tris = [[0, 1, 2]] + [[3 + t * 3, 4 + t * 3, 5 + t * 3] for t in range(1, 64)]
    cfg = _cfg(vertex_count=n, triangle_count=64, dt=1 / 60, damping=1.0, gravity=(0, 0, 0), self_collision=1,
               self_collision_mode=1, cloth_thickness=0.10, collision_margin=0.0, max_self_collision_neighbors=32)
    m, keep = _mesh(positions=pos, inv_mass=inv, triangles=tris)

    def run(solver):
        close = pos.copy()
        close[n - 1] = (0.0, -0.2, 0.03)
        solver.update_positions(close)
        solver.step(1, 6)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert out[n - 1, 2] > 0.03 + 1e-4, out[n - 1]
        return out

    return Case("self_vt", cfg, m, keep), run


def self_ee():
    """abi41_smoke.cpp:448-597: an edge 3 cm above a pinned crossing edge is
    pushed up by more than 1e-4 (edge-edge contact)."""
    n = 600
    pos = np.zeros((n, 3), np.float32)
    for i in range(n):
        pos[i] = (200.0 + i * 3.0, 100.0 + (i % 11), 0.0)
    pos[0], pos[1], pos[2], pos[3] = (-1, 0, 0), (1, 0, 0), (5, -1, 0), (5, 1, 0)
    inv = np.ones(n, np.float32)
    inv[:2] = 0
    edges = [[0, 1], [2, 3]]
    for e in range(2, 64):
        a = 4 + (e - 2) * 2
        pos[a] = (50.0 + e * 4.0, 30.0, 0.0)
        pos[a + 1] = (51.0 + e * 4.0, 30.0, 0.0)
        edges.append([a, a + 1])
    edges = np.asarray(edges, np.int32)
    rest = np.linalg.norm(pos[edges[:, 0]] - pos[edges[:, 1]], axis=1).astype(np.float32)
    cfg = _cfg(vertex_count=n, edge_count=64, dt=1 / 60, damping=1.0, gravity=(0, 0, 0), self_collision=1,
               self_collision_mode=1, cloth_thickness=0.10, collision_margin=0.0, max_self_collision_neighbors=32)
    m, keep = _mesh(positions=pos, inv_mass=inv, edges=edges, edge_rest_lengths=rest)

    def run(solver):
        close = pos.copy()
        close[2] = (0.0, -1.0, 0.03)
        close[3] = (0.0, 1.0, 0.03)
        h0 = 0.5 * (close[2, 2] + close[3, 2])
        solver.update_positions(close)
        solver.step(1, 6)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert 0.5 * (out[2, 2] + out[3, 2]) > h0 + 1e-4
        return out

    return Case("self_ee", cfg, m, keep), run


def tether_static():
    """abi41_smoke.cpp:879-941: a tether of rest 0.5 pulls the free end of a
    2 m pair in by more than 5 mm."""
    pos = np.array([[0, 0, 0], [2, 0, 0]], np.float32)
    cfg = _cfg(vertex_count=2, lra_count=1, dt=1 / 60, damping=1.0, lra_compliance=1e-9)
    m, keep = _mesh(positions=pos, inv_mass=[0.0, 1.0], lra_edges=[[0, 1]], lra_rest_lengths=[0.5])
    pins = (np.array([0], np.int32), np.array([[0, 0, 0]], np.float32), np.array([1.0], np.float32))

    def run(solver):
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert out[1, 0] < pos[1, 0] - 0.005
        return out

    return Case("tether_static", cfg, m, keep, pins), run


def tether_animated():
    """abi41_smoke.cpp:943-1003: with the anchor pin moved, the tether still
    pulls the free end in by more than 5 mm."""
    pos = np.array([[1, 0, 0], [2, 0, 0]], np.float32)
    cfg = _cfg(vertex_count=2, lra_count=1, dt=1 / 60, damping=1.0, lra_compliance=1e-9)
    m, keep = _mesh(positions=pos, inv_mass=[0.0, 1.0], lra_edges=[[0, 1]], lra_rest_lengths=[0.25])
    pins = (np.array([0], np.int32), np.array([[1, 0, 0]], np.float32), np.array([1.0], np.float32))

    def run(solver):
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert out[1, 0] < pos[1, 0] - 0.005
        return out

    return Case("tether_animated", cfg, m, keep, pins), run


def bend_hinge():
    """abi41_smoke.cpp:1005-1087: a folded hinge's wing distance error
    decreases after one step (no colours given: all bends at once)."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    folded = rest.copy()
    folded[3, 2] = 1.0
    rd = float(np.sqrt(np.float32(2.0)))
    cfg = _cfg(vertex_count=4, bend_count=1, triangle_count=2, dt=1 / 60, damping=1.0, bend_compliance=1e-9)
    m, keep = _mesh(positions=rest, inv_mass=[0, 1, 1, 1], bends=[[0, 3]], bend_rest_lengths=[rd],
                    triangles=[[0, 1, 2], [1, 3, 2]])

    def run(solver):
        solver.update_positions(folded)
        e0 = abs(_dist(folded, 0, 3) - rd)
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert abs(_dist(out, 0, 3) - rd) < e0
        return out

    return Case("bend_hinge", cfg, m, keep), run


def pin_weights():
    """abi41_smoke.cpp:1171-1269: pin weight 1.0 holds y = 1 to 1e-5, 0.375
    pulls partly (0.2 < y < 0.95), 0.04 is ignored (equal to the free vertex to
    1e-6), and the free vertex falls."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]], np.float32)
    cfg = _cfg(vertex_count=4, dt=1 / 60, damping=1.0, gravity=(0, -9.8, 0))
    m, keep = _mesh(positions=pos, inv_mass=np.ones(4))
    pins = (np.array([0, 1, 2], np.int32), np.array([[0, 1, 0], [1, 1, 0], [2, 1, 0]], np.float32),
            np.array([1.0, 0.375, 0.04], np.float32))

    def run(solver):
        solver.step(1, 3)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert abs(out[0, 1] - 1.0) <= 1e-5
        assert 0.20 < out[1, 1] < 0.95 and out[3, 1] < -1e-5
        assert abs(out[2, 1] - out[3, 1]) <= 1e-6
        return out

    return Case("pin_weights", cfg, m, keep, pins), run


def pinned_square():
    """abi41_smoke.cpp:1273-1415: a 4-vertex square with two hard pins, ground
    at z = 0: pins exact to 1e-5 after 4 x 4, the free corner falls in y."""
    pos = np.array([[0, 0.2, 0], [1, 0.2, 0], [0, 1.2, 0], [1, 1.2, 0]], np.float32)
    edges = np.array([[0, 1], [0, 2], [1, 3], [2, 3], [0, 3], [1, 2]], np.int32)
    rest = np.linalg.norm(pos[edges[:, 0]] - pos[edges[:, 1]], axis=1).astype(np.float32)
    cfg = _cfg(vertex_count=4, edge_count=6, triangle_count=2, dt=1 / 60, damping=0.99, gravity=(0, -9.8, 0),
               stretch_compliance=1e-6, collision_margin=0.005, use_ground=1, ground_height=0.0, cloth_thickness=0.02)
    m, keep = _mesh(positions=pos, inv_mass=[0, 0, 1, 1], edges=edges, edge_rest_lengths=rest, triangles=[[0, 1, 2], [1, 3, 2]])
    pins = (np.array([0, 1], np.int32), pos[:2].copy(), np.array([1.0, 1.0], np.float32))

    def run(solver):
        solver.step(4, 4)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert np.abs(out[:2] - pos[:2]).max() <= 1e-5
        assert out[2, 1] < pos[2, 1]
        return out

    return Case("pinned_square", cfg, m, keep, pins), run


ALL = [static_sdf_plane, static_sdf_box, self_vv, self_vt, self_ee, tether_static, tether_animated, bend_hinge,
       pin_weights, pinned_square]


def _hard_stretch_case(rest, inv, start, enabled):
    """abi41_smoke.cpp:599-652: one edge of rest 1 m, soft springs, PCG on or
    off at full strength, stepped 1 x 1 from `start`."""
    cfg = _cfg(vertex_count=2, edge_count=1, dt=1 / 60, damping=1.0, gravity=(0, 0, 0), stretch_compliance=1.0e6,
               stretch_optimization_enabled=1 if enabled else 0, stretch_optimization_strength=1.0)
    m, keep = _mesh(positions=np.asarray(rest, np.float32), inv_mass=inv, edges=[[0, 1]], edge_rest_lengths=[1.0])
    start = np.asarray(start, np.float32)

    def run(solver):
        solver.update_positions(start)
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        return out

    return Case("hard_stretch", cfg, m, keep), run


def _chain_case():
    """abi41_smoke.cpp:654-742: a pinned 4-vertex chain with its end pulled
    2 m out; the PCG pass pulls the end back by more than 2 cm."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]], np.float32)
    start = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [5, 0, 0]], np.float32)
    cfg = _cfg(vertex_count=4, edge_count=3, dt=1 / 60, damping=1.0, stretch_compliance=1.0e6,
               stretch_optimization_enabled=1, stretch_optimization_strength=1.0)
    m, keep = _mesh(positions=rest, inv_mass=[0, 1, 1, 1], edges=[[0, 1], [1, 2], [2, 3]], edge_rest_lengths=[1, 1, 1])

    def run(solver):
        solver.update_positions(start)
        solver.step(1, 1)
        out = solver.download_positions().copy()
        assert np.isfinite(out).all()
        assert out[3, 0] < start[3, 0] - 0.02
        return out

    return Case("chain", cfg, m, keep), run


def hard_stretch_suite(make_solver):
    """abi41_smoke.cpp:744-876 with `make_solver(case)` building the backend:
    returns the outputs so callers can compare backends."""
    rest = [[0, 0, 0], [1, 0, 0]]
    stretched = [[0, 0, 0], [2.5, 0, 0]]
    outs = {}
    for name, args in {
        "off": (rest, [1.0, 1.0], stretched, False),
        "on": (rest, [1.0, 1.0], stretched, True),
        "pinned": (rest, [0.0, 1.0], stretched, True),
        "both_pinned": ([[0, 0, 0], [2.5, 0, 0]], [0.0, 0.0], [[0, 0, 0], [2.5, 0, 0]], True),
        "zero": (rest, [1.0, 1.0], [[0, 0, 0], [0, 0, 0]], True),
    }.items():
        case, run = _hard_stretch_case(*args)
        outs[name] = run(make_solver(case))
    off_d = float(np.linalg.norm(outs["off"][1] - outs["off"][0]))
    on_d = float(np.linalg.norm(outs["on"][1] - outs["on"][0]))
    assert on_d < off_d - 0.05, (off_d, on_d)
    assert abs(outs["pinned"][0, 0]) <= 1e-5 and outs["pinned"][1, 0] < 2.5 - 0.05
    assert abs(float(np.linalg.norm(outs["both_pinned"][1] - outs["both_pinned"][0])) - 2.5) <= 1e-4
    case, run = _chain_case()
    outs["chain"] = run(make_solver(case))
    return outs
