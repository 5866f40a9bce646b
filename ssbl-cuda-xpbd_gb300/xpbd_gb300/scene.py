"""Synthetic cloth scenes and the solver inputs built from them.

The constraint builders restate the reference's input pipeline
(xpbd_core.py, devin22ldh-afk/ssbl-cuda-xpbd) without Blender:

* ``edge_constraints``       -- xpbd_core.py:715-727 (unique sorted edges)
* ``bend_constraints``       -- xpbd_core.py:730-747 (wing-opposite pairs)
* ``color_constraints``      -- xpbd_core.py:828-859 (greedy colouring, stable
  sort by colour, colour offsets)
* ``vertex_inverse_mass``    -- xpbd_core.py:862-881 (area / 3 lumping)
* ``hidden_tethers``         -- xpbd_core.py:750-825 (nearest hard pin)
* ``derive_hardness``        -- xpbd_core.py:213-244 (hardness -> compliances)

Scenes are generated from a seed: square grids split into triangles, a
closed box mesh and a closed torus mesh for the static SDF collider.  The
coordinate convention is the reference's: Z up, gravity along -Z.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_EPS = 1.0e-8
PIN_HARD_WEIGHT_THRESHOLD = 0.75


@dataclass
class ClothData:
    """Solver inputs of one cloth (the fields of the reference's ClothBuildData)."""

    positions_world: np.ndarray
    inv_mass: np.ndarray
    triangles: np.ndarray
    edges: np.ndarray
    edge_rest_lengths: np.ndarray
    edge_color_offsets: np.ndarray
    bends: np.ndarray
    bend_rest_lengths: np.ndarray
    bend_color_offsets: np.ndarray
    lra_edges: np.ndarray
    lra_rest_lengths: np.ndarray
    lra_color_offsets: np.ndarray
    pin_indices: np.ndarray
    pin_targets_world: np.ndarray
    pin_weights: np.ndarray
    rest_volume: float = 0.0


@dataclass
class SolverOptions:
    """Solver settings (field meaning of the reference's SolverOptions,
    xpbd_core.py:45-84; defaults are the add-on's UI defaults)."""

    dt: float = 1.0 / 60.0
    damping: float = 1.0
    gravity: tuple = (0.0, 0.0, -9.81)
    stretch_compliance: float = 1.0e-6
    stretch_optimization_enabled: bool = False
    stretch_optimization_strength: float = 0.0
    bend_compliance: float = 1.0e-4
    lra_compliance: float = 0.0
    collision_margin: float = 0.005
    use_ground: bool = False
    ground_height: float = 0.0
    use_wall: bool = False
    wall_origin: tuple = (0.0, 0.0, 0.0)
    wall_normal: tuple = (0.0, 0.0, 1.0)
    use_sphere: bool = False
    sphere_center: tuple = (0.0, 0.0, 0.0)
    sphere_radius: float = 0.0
    self_collision: bool = False
    self_collision_mode: int = 0
    cloth_thickness: float = 0.02
    self_collision_distance: float = 0.0
    self_collision_interval: int = 1
    max_self_collision_neighbors: int = 64
    fast_self_collision_passes: int = 4
    use_volume_pressure: bool = False
    volume_compliance: float = 1.0e-6
    pressure_strength: float = 0.0
    volume_target_scale: float = 1.0
    volume_solve_interval: int = 1
    self_probe_interval: int = 1
    self_surface_pair_interval: int = 1
    jitter_stabilizer_enabled: bool = False
    contact_friction: float = 0.35
    contact_tangent_damping: float = 0.2
    contact_compliance: float = 0.0
    static_sdf_voxel_size: float = 0.0
    static_sdf_band_voxels: int = 4
    static_sdf_max_resolution: int = 160


# ----------------------------------------------------------- topology ----
def grid_mesh(n: int, side: float = 1.0, z: float = 0.0) -> tuple[np.ndarray, np.ndarray]:
    """n x n vertices on a `side`-metre square in the XY plane, centred at the
    origin; every quad split along its (i, j)-(i+1, j+1) diagonal."""
    lin = (np.arange(n, dtype=np.float64) / (n - 1) - 0.5) * side
    xs, ys = np.meshgrid(lin, lin, indexing="xy")
    pos = np.stack([xs.ravel(), ys.ravel(), np.full(n * n, z)], axis=1).astype(np.float32)
    idx = np.arange(n * n, dtype=np.int32).reshape(n, n)
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, 1:].ravel()
    d = idx[1:, :-1].ravel()
    tris = np.empty((2 * len(a), 3), dtype=np.int32)
    tris[0::2] = np.stack([a, b, c], axis=1)
    tris[1::2] = np.stack([a, c, d], axis=1)
    return pos, tris


def edge_constraints(triangles: np.ndarray, rest: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    t = np.asarray(triangles, dtype=np.int64)
    if len(t) == 0:
        return np.empty((0, 2), np.int32), np.empty(0, np.float32)
    pairs = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    pairs = np.sort(pairs, axis=1)
    pairs = np.unique(pairs, axis=0).astype(np.int32)
    delta = rest[pairs[:, 1]] - rest[pairs[:, 0]]
    return pairs, np.maximum(np.linalg.norm(delta, axis=1), _EPS)


def set_native_prep(enabled: bool) -> None:
    """Whether the builders may call the library's host-side preprocessing
    (greedy colouring, bend pairs); off, they use only the Python
    restatement, and this module loads no native library (the benchmark's
    reference arm runs that way)."""
    global _PREP, _PREP_ENABLED
    _PREP_ENABLED = bool(enabled)
    _PREP = None
_PREP_ENABLED = True


def _native_prep():
    """The library's host-side preprocessing entry points, when it is built
    (same results as the Python loops below, which remain the restatement)."""
    global _PREP
    if not _PREP_ENABLED:
        return None
    if _PREP is None:
        try:
            import ctypes
            import os

            from .build import library_path

            path = os.environ.get("SSBL_NATIVE_DLL_PATH") or library_path()
            lib = ctypes.CDLL(path) if os.path.exists(path) else None
            if lib is not None and hasattr(lib, "xpbd_gb300_greedy_color"):
                pi = ctypes.POINTER(ctypes.c_int)
                lib.xpbd_gb300_greedy_color.argtypes = [pi, ctypes.c_int, ctypes.c_int, pi]
                lib.xpbd_gb300_greedy_color.restype = ctypes.c_int
                lib.xpbd_gb300_bend_pairs.argtypes = [pi, ctypes.c_int, pi, ctypes.c_int]
                lib.xpbd_gb300_bend_pairs.restype = ctypes.c_int
                if hasattr(lib, "xpbd_gb300_prepare_cloth_device"):
                    pf = ctypes.POINTER(ctypes.c_float)
                    lib.xpbd_gb300_prepare_cloth_device.argtypes = [
                        pf, ctypes.c_int, pi, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                        ctypes.POINTER(ctypes.c_ubyte), pi, pf, pf, pi, pf, pi]
                    lib.xpbd_gb300_prepare_cloth_device.restype = ctypes.c_int
                    lib.ssbl_last_error.restype = ctypes.c_char_p
                _PREP = lib
            else:
                _PREP = False
        except Exception:
            _PREP = False
    return _PREP or None


_PREP = None


def bend_pairs_py(triangles: np.ndarray) -> np.ndarray:
    """Bend pairs by the Python walk of xpbd_core.py:730-747."""
    first_opposite: dict[tuple[int, int], int] = {}
    pairs: set[tuple[int, int]] = set()
    for tri in np.asarray(triangles, dtype=np.int64):
        a, b, c = int(tri[0]), int(tri[1]), int(tri[2])
        for x, y, opp in ((a, b, c), (b, c, a), (c, a, b)):
            key = (x, y) if x < y else (y, x)
            prev = first_opposite.get(key)
            if prev is None:
                first_opposite[key] = opp
            elif prev != opp:
                pairs.add((prev, opp) if prev < opp else (opp, prev))
    return np.asarray(sorted(pairs), dtype=np.int32).reshape(-1, 2)


def bend_pairs(triangles: np.ndarray) -> np.ndarray:
    lib = _native_prep()
    tris = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
    if lib is None or len(tris) == 0:
        return bend_pairs_py(tris)
    import ctypes

    out = np.empty((3 * len(tris), 2), np.int32)
    pi = ctypes.POINTER(ctypes.c_int)
    n = lib.xpbd_gb300_bend_pairs(tris.ctypes.data_as(pi), len(tris), out.ctypes.data_as(pi), len(out))
    if n < 0:
        return bend_pairs_py(tris)
    return np.ascontiguousarray(out[:n])


def bend_constraints(triangles: np.ndarray, rest: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    arr = bend_pairs(triangles)
    if len(arr) == 0:
        return arr, np.empty(0, np.float32)
    delta = rest[arr[:, 1]] - rest[arr[:, 0]]
    return arr, np.maximum(np.linalg.norm(delta, axis=1), _EPS)


def color_constraints(pairs: np.ndarray, rest: np.ndarray, vertex_count: int):
    """Greedy first-fit colouring in constraint order, then a stable sort by
    colour; returns (pairs, rest, offsets)."""
    if len(pairs) == 0:
        return pairs.reshape(0, 2), np.asarray(rest, np.float32), np.asarray([0], np.int32)
    colors = greedy_colors(pairs, vertex_count)
    order = np.argsort(colors, kind="stable")
    counts = np.bincount(colors[order], minlength=int(colors.max()) + 1).astype(np.int32)
    offsets = np.concatenate(([0], np.cumsum(counts))).astype(np.int32)
    return (np.ascontiguousarray(pairs[order], np.int32), np.ascontiguousarray(np.asarray(rest)[order], np.float32), offsets)


def greedy_colors(pairs: np.ndarray, vertex_count: int) -> np.ndarray:
    """Greedy first-fit colour of each pair in order (native when built)."""
    lib = _native_prep()
    p = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    if lib is not None:
        import ctypes

        pi = ctypes.POINTER(ctypes.c_int)
        out = np.empty(len(p), np.int32)
        if lib.xpbd_gb300_greedy_color(p.ctypes.data_as(pi), len(p), int(vertex_count), out.ctypes.data_as(pi)) >= 0:
            return out
    return greedy_colors_py(p, vertex_count)


def greedy_colors_py(pairs: np.ndarray, vertex_count: int) -> np.ndarray:
    """Greedy first-fit colouring by the Python loop of xpbd_core.py:828-859."""
    used = [0] * vertex_count  # bitmask of colours per vertex
    colors = np.empty(len(pairs), dtype=np.int32)
    for k, (a, b) in enumerate(np.asarray(pairs, dtype=np.int64)):
        blocked = 0
        if 0 <= a < vertex_count:
            blocked |= used[a]
        if 0 <= b < vertex_count:
            blocked |= used[b]
        color = 0
        while (blocked >> color) & 1:
            color += 1
        colors[k] = color
        bit = 1 << color
        if 0 <= a < vertex_count:
            used[a] |= bit
        if 0 <= b < vertex_count:
            used[b] |= bit
    return colors


def cloth_inputs_device(rest: np.ndarray, triangles: np.ndarray, density: float, pin_mask: np.ndarray):
    """Edges, edge rest lengths, inverse masses, bend pairs and bend rest
    lengths computed on the GPU (xpbd_gb300_prepare_cloth_device);
    bit-identical to edge_constraints, vertex_inverse_mass and
    bend_constraints.  Needs the built library and a GPU."""
    import ctypes

    lib = _native_prep()
    if lib is None or not hasattr(lib, "xpbd_gb300_prepare_cloth_device"):
        raise RuntimeError("device preprocessing needs the built GB300 library")
    pos = np.ascontiguousarray(rest, np.float32)
    tris = np.ascontiguousarray(triangles, np.int32)
    hard = np.ascontiguousarray(pin_mask, np.uint8)
    V, T = len(pos), len(tris)
    edges = np.empty((max(3 * T, 1), 2), np.int32)
    edge_rest = np.empty(max(3 * T, 1), np.float32)
    inv = np.empty(max(V, 1), np.float32)
    bends = np.empty((max(3 * T, 1), 2), np.int32)
    bend_rest = np.empty(max(3 * T, 1), np.float32)
    nb = ctypes.c_int(0)
    pf, pi = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
    # the builders scale areas by max(density, eps) as a float32 factor
    n = lib.xpbd_gb300_prepare_cloth_device(
        pos.ctypes.data_as(pf), V, tris.ctypes.data_as(pi), T, float(np.float32(max(density, _EPS))), float(np.float32(_EPS)),
        hard.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), edges.ctypes.data_as(pi), edge_rest.ctypes.data_as(pf),
        inv.ctypes.data_as(pf), bends.ctypes.data_as(pi), bend_rest.ctypes.data_as(pf), ctypes.byref(nb))
    if n < 0:
        raise RuntimeError((lib.ssbl_last_error() or b"").decode() or "device preprocessing failed")
    return (edges[:n].copy(), edge_rest[:n].copy(), inv[:V].copy(), bends[:nb.value].copy(),
            bend_rest[:nb.value].copy())


def vertex_inverse_mass(rest: np.ndarray, triangles: np.ndarray, density: float, pin_mask: np.ndarray) -> np.ndarray:
    mass = np.zeros(len(rest), dtype=np.float64)
    p0, p1, p2 = rest[triangles[:, 0]], rest[triangles[:, 1]], rest[triangles[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0), axis=1)
    share = np.maximum(area * max(density, _EPS), _EPS) / 3.0
    for k in range(3):
        np.add.at(mass, triangles[:, k], share)
    mass[mass <= 0.0] = 1.0
    inv = 1.0 / mass
    inv[pin_mask] = 0.0
    return inv


def hidden_tethers(rest: np.ndarray, pin_mask: np.ndarray, slack: float) -> tuple[np.ndarray, np.ndarray]:
    """Each free vertex tethered to its nearest hard pin, rest = distance x slack."""
    pins = np.flatnonzero(pin_mask).astype(np.int32)
    free = np.flatnonzero(~pin_mask).astype(np.int32)
    if len(pins) == 0 or len(free) == 0:
        return np.empty((0, 2), np.int32), np.empty(0, np.float32)
    pp = rest[pins].astype(np.float64)
    fp = rest[free].astype(np.float64)
    try:  # the reference queries a k-d tree first (xpbd_core.py:771-784)
        from scipy.spatial import cKDTree

        dist, loc = cKDTree(pp).query(fp, k=1, workers=-1)
        nearest = pins[loc]
    except Exception:
        nearest = np.empty(len(free), dtype=np.int32)
        dist = np.empty(len(free), dtype=np.float64)
        for s in range(0, len(free), 2048):
            d = fp[s:s + 2048, None, :] - pp[None, :, :]
            dsq = np.einsum("cpi,cpi->cp", d, d)
            loc = np.argmin(dsq, axis=1)
            nearest[s:s + 2048] = pins[loc]
            dist[s:s + 2048] = np.sqrt(dsq[np.arange(len(loc)), loc])
    pairs = np.column_stack((nearest, free)).astype(np.int32)
    return pairs, np.maximum(dist * max(float(slack), 0.5), _EPS).astype(np.float32)


def _log_interp(soft: float, hard: float, h: float) -> float:
    h = min(max(h, 0.0), 1.0)
    return float(np.exp(np.log(soft) * (1.0 - h) + np.log(hard) * h))


def derive_hardness(hardness: float) -> dict:
    """Hardness slider -> compliances (xpbd_core.py:213-244)."""
    hardness = min(max(float(hardness), 0.0), 1.0)
    material = hardness * 0.70
    tether = hardness >= 0.5
    tether_h = ((hardness - 0.5) / 0.5) * 0.70 if tether else 0.0
    return {
        "stretch_compliance": _log_interp(8.0e-6, 1.0e-9, material),
        "stretch_optimization_enabled": hardness > 0.0,
        "stretch_optimization_strength": hardness,
        "bend_compliance": _log_interp(2.0e-3, 1.0e-9, material),
        "hidden_tether_enabled": tether,
        "hidden_tether_compliance": _log_interp(8.0e-4, 1.0e-9, tether_h),
        "hidden_tether_slack": float(np.interp(tether_h, [0.0, 1.0], [1.20, 0.95])),
    }


def build_cloth(
    positions: np.ndarray,
    triangles: np.ndarray,
    density: float,
    pin_weights_by_vertex: np.ndarray,
    tether_slack: float | None = None,
    device: bool = False,
) -> ClothData:
    """Constraint inputs of a cloth from its rest pose and per-vertex pin
    weights (the steps of xpbd_core.py:_build_cloth_data_uncached).  With
    `device`, edges, rest lengths and inverse masses come from the GPU
    (cloth_inputs_device), the same arrays bit for bit."""
    world = np.ascontiguousarray(positions, dtype=np.float32)
    tris = np.ascontiguousarray(triangles, dtype=np.int32)
    weights = np.asarray(pin_weights_by_vertex, dtype=np.float32)
    pin_mask = weights > 0.0
    hard = weights >= PIN_HARD_WEIGHT_THRESHOLD
    if device:
        edges, edge_rest, inv, bends, bend_rest = cloth_inputs_device(world, tris, density, hard)
    else:
        edges, edge_rest = edge_constraints(tris, world)
        bends, bend_rest = bend_constraints(tris, world)
        inv = None
    edges, edge_rest, edge_off = color_constraints(edges, edge_rest, len(world))
    bends, bend_rest, bend_off = color_constraints(bends, bend_rest, len(world))
    if tether_slack is not None:
        lra, lra_rest = hidden_tethers(world, hard, tether_slack)
    else:
        lra, lra_rest = np.empty((0, 2), np.int32), np.empty(0, np.float32)
    if inv is None:
        inv = vertex_inverse_mass(world, tris, density, hard)
    pins = np.flatnonzero(pin_mask).astype(np.int32)
    return ClothData(
        positions_world=world,
        inv_mass=np.ascontiguousarray(inv, np.float32),
        triangles=tris,
        edges=np.ascontiguousarray(edges, np.int32),
        edge_rest_lengths=np.ascontiguousarray(edge_rest, np.float32),
        edge_color_offsets=np.ascontiguousarray(edge_off, np.int32),
        bends=np.ascontiguousarray(bends, np.int32),
        bend_rest_lengths=np.ascontiguousarray(bend_rest, np.float32),
        bend_color_offsets=np.ascontiguousarray(bend_off, np.int32),
        lra_edges=np.ascontiguousarray(lra, np.int32),
        lra_rest_lengths=np.ascontiguousarray(lra_rest, np.float32),
        lra_color_offsets=np.asarray([0], np.int32),
        pin_indices=pins,
        pin_targets_world=np.ascontiguousarray(world[pins], np.float32),
        pin_weights=np.ascontiguousarray(weights[pins], np.float32),
    )


# ------------------------------------------------------------ colliders ---
def box_triangles(center, half) -> np.ndarray:
    """Closed axis-aligned box, 12 outward-wound triangles, (12, 3, 3) f32."""
    cx, cy, cz = center
    hx, hy, hz = half if np.ndim(half) else (half, half, half)
    v = np.array([[cx + sx * hx, cy + sy * hy, cz + sz * hz] for sz in (-1, 1) for sy in (-1, 1) for sx in (-1, 1)], np.float32)
    faces = [(0, 2, 3), (0, 3, 1), (4, 5, 7), (4, 7, 6), (0, 1, 5), (0, 5, 4),
             (2, 6, 7), (2, 7, 3), (0, 4, 6), (0, 6, 2), (1, 3, 7), (1, 7, 5)]
    return v[np.array(faces)].astype(np.float32)


def torus_triangles(center, major: float, minor: float, nu: int = 32, nv: int = 16) -> np.ndarray:
    """Closed torus around +Z, (2*nu*nv, 3, 3) f32."""
    cx, cy, cz = center
    u = np.arange(nu) * (2.0 * math.pi / nu)
    w = np.arange(nv) * (2.0 * math.pi / nv)
    uu, ww = np.meshgrid(u, w, indexing="ij")
    r = major + minor * np.cos(ww)
    pts = np.stack([cx + r * np.cos(uu), cy + r * np.sin(uu), cz + minor * np.sin(ww)], axis=-1).reshape(-1, 3)
    idx = np.arange(nu * nv).reshape(nu, nv)
    a = idx
    b = np.roll(idx, -1, axis=0)
    c = np.roll(np.roll(idx, -1, axis=0), -1, axis=1)
    d = np.roll(idx, -1, axis=1)
    faces = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return pts[faces].astype(np.float32)


def icosphere(center, radius: float, subdivisions: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """Closed, outward-wound sphere mesh: (vertices (N, 3) f32, indices
    (20 * 4^subdivisions, 3) i32)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
             (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts) * radius + np.asarray(center, np.float64)
    return v.astype(np.float32), np.array(faces, np.int32)


def ramp_triangles(center, size: float, n: int, tilt: float) -> np.ndarray:
    """Open n x n grid of 2 n^2 triangles (size m square, tilted by `tilt`
    radians about x), (2 n^2, 3, 3) f32, facing +z."""
    pos, tris = grid_mesh(n + 1, size, 0.0)
    c, s = math.cos(tilt), math.sin(tilt)
    y, z = pos[:, 1].astype(np.float64), pos[:, 2].astype(np.float64)
    rot = np.stack([pos[:, 0], c * y - s * z, s * y + c * z], axis=1) + np.asarray(center, np.float64)
    return rot[tris].astype(np.float32)


def particle_stream(count: int, center, spread: float, radius: float, seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Seeded particles (positions (count, 3), radii (count,)) in a slab
    of half-width `spread` around `center`, radii in [0.5, 1] x radius."""
    rng = np.random.default_rng(seed)
    p = np.asarray(center, np.float64) + rng.uniform(-spread, spread, size=(count, 3)) * np.array([1.0, 1.0, 0.25])
    r = rng.uniform(0.5, 1.0, size=count) * radius
    return p.astype(np.float32), r.astype(np.float32)


# --------------------------------------------------------- named scenes ---
@dataclass
class Scene:
    name: str
    cloth: ClothData
    options: SolverOptions
    static_triangles: np.ndarray  # (S, 3, 3) f32
    substeps: int
    iterations: int
    frames: int
    extent: float = 1.0
    meta: dict = field(default_factory=dict)


def plain_grid_scene(n: int = 32, frames: int = 120) -> Scene:
    """Plain XPBD: n x n grid, 1 m side, the two corners of the y = +0.5 edge
    hard-pinned, stretch 1e-7 / bend 1e-4, 0.2 kg/m^2, damping 0.99 per
    substep, ground plane z = -1, 60 fps x 10 substeps x 2 iterations."""
    pos, tris = grid_mesh(n, 1.0, 0.0)
    w = np.zeros(n * n, np.float32)
    w[(n - 1) * n] = 1.0
    w[n * n - 1] = 1.0
    cloth = build_cloth(pos, tris, 0.2, w)
    opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, gravity=(0.0, 0.0, -9.81), stretch_compliance=1.0e-7,
                        bend_compliance=1.0e-4, collision_margin=0.005, use_ground=True, ground_height=-1.0)
    return Scene(f"plain-grid-{n}", cloth, opt, np.empty((0, 3, 3), np.float32), 10, 2, frames, 1.0)


def collider_meshes() -> np.ndarray:
    """Static collider: a box below and beside the cloth plus a torus lying
    on it (box union torus, both closed)."""
    box = box_triangles((0.55, 0.0, -0.55), (0.25, 0.25, 0.25))
    torus = torus_triangles((-0.45, 0.1, -0.35), 0.22, 0.07, 32, 16)
    return np.concatenate([box, torus]).astype(np.float32)


def drop_scene(n: int = 100, frames: int = 200, seed: int = 0, self_mode: int = 2) -> Scene:
    """n x n grid (1 m) with seeded +-1 mm z jitter, dropped from z = 0.5 onto
    a sphere (r = 0.3 m, origin) and a 64^3 static SDF of box union torus;
    self collision (strict by default) with 2 mm thickness, friction 0.3."""
    rng = np.random.default_rng(seed)
    pos, tris = grid_mesh(n, 1.0, 0.5)
    pos[:, 2] += rng.uniform(-1.0e-3, 1.0e-3, size=len(pos)).astype(np.float32)
    cloth = build_cloth(pos, tris, 0.2, np.zeros(len(pos), np.float32))
    opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, stretch_compliance=1.0e-7, bend_compliance=1.0e-4,
                        collision_margin=0.002, cloth_thickness=0.002, use_sphere=True, sphere_center=(0.0, 0.0, 0.0),
                        sphere_radius=0.3, use_ground=True, ground_height=-1.0, self_collision=True,
                        self_collision_mode=self_mode, self_collision_interval=1 if self_mode == 2 else 2,
                        max_self_collision_neighbors=64 if self_mode == 2 else 32, fast_self_collision_passes=4,
                        contact_friction=0.3, static_sdf_max_resolution=64)
    return Scene(f"drop-{n}", cloth, opt, collider_meshes(), 10, 2, frames, 1.0)


def hardness_grid_scene(n: int = 32, hardness: float = 0.4, frames: int = 60) -> Scene:
    """The plain grid with the add-on's hardness mapping: compliances from the
    hardness slider, the hard-stretch (CG) path at strength = hardness, and
    hidden tethers to the pins when hardness >= 0.5 (xpbd_core.py:213-244)."""
    base = plain_grid_scene(n, frames)
    h = derive_hardness(hardness)
    w = np.zeros(len(base.cloth.positions_world), np.float32)
    w[base.cloth.pin_indices] = 1.0
    cloth = build_cloth(base.cloth.positions_world, base.cloth.triangles, 0.2, w,
                        tether_slack=h["hidden_tether_slack"] if h["hidden_tether_enabled"] else None)
    opt = base.options
    opt.stretch_compliance = h["stretch_compliance"]
    opt.bend_compliance = h["bend_compliance"]
    opt.stretch_optimization_enabled = h["stretch_optimization_enabled"]
    opt.stretch_optimization_strength = h["stretch_optimization_strength"]
    opt.lra_compliance = h["hidden_tether_compliance"] if h["hidden_tether_enabled"] else 0.0
    opt.cloth_thickness = 0.02
    return Scene(f"hardness-{hardness}-grid-{n}", cloth, opt, base.static_triangles, 10, 2, frames, 1.0)


_GRID_CACHE: dict[tuple, ClothData] = {}


def _unpinned_grid(n: int, z: float, side: float = 1.0) -> ClothData:
    """Constraint inputs of an unpinned n x n grid (cached: every cloth of a
    batch with the same side shares its topology and rest state)."""
    key = (n, z, side)
    if key not in _GRID_CACHE:
        pos, tris = grid_mesh(n, side, z)
        _GRID_CACHE[key] = build_cloth(pos, tris, 0.2, np.zeros(n * n, np.float32))
    return _GRID_CACHE[key]


def batched_scenes(count: int = 256, seed: int = 0, frames: int = 120, side_range: tuple = (16, 128),
                   only=None) -> list[Scene]:
    """Independent cloths of uneven sizes for the batched form: side drawn
    uniformly from `side_range` vertices (1 m cloths at z = 0.5), stretch and
    bend compliance each log-uniform in [1e-8, 1e-4], 2-8 random hard pins,
    self collision fast or strict with probability 0.5 (2 mm thickness), a
    sphere (r = 0.3 m) below and the ground at z = -1; 10 substeps x 2
    iterations.  `only` (cloth indices) builds just those cloths of the same
    seeded set."""
    rng = np.random.default_rng(seed)
    keep = None if only is None else set(int(k) for k in only)
    out = []
    for k in range(count):
        n = int(rng.integers(side_range[0], side_range[1] + 1))
        V = n * n
        pins = np.sort(rng.choice(V, size=int(rng.integers(2, 9)), replace=False)).astype(np.int32)
        if keep is not None and k not in keep:
            rng.uniform(-8.0, -4.0)
            rng.uniform(-8.0, -4.0)
            rng.random()
            continue
        base = _unpinned_grid(n, 0.5)
        inv = base.inv_mass.copy()
        inv[pins] = 0.0
        cloth = ClothData(
            positions_world=base.positions_world, inv_mass=np.ascontiguousarray(inv, np.float32),
            triangles=base.triangles, edges=base.edges, edge_rest_lengths=base.edge_rest_lengths,
            edge_color_offsets=base.edge_color_offsets, bends=base.bends, bend_rest_lengths=base.bend_rest_lengths,
            bend_color_offsets=base.bend_color_offsets, lra_edges=base.lra_edges, lra_rest_lengths=base.lra_rest_lengths,
            lra_color_offsets=base.lra_color_offsets, pin_indices=pins,
            pin_targets_world=np.ascontiguousarray(base.positions_world[pins], np.float32),
            pin_weights=np.ones(len(pins), np.float32))
        stretch = float(10.0 ** rng.uniform(-8.0, -4.0))
        bend = float(10.0 ** rng.uniform(-8.0, -4.0))
        fast = bool(rng.random() < 0.5)
        opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, stretch_compliance=stretch, bend_compliance=bend,
                            collision_margin=0.002, cloth_thickness=0.002, use_sphere=True,
                            sphere_center=(0.0, 0.0, 0.0), sphere_radius=0.3, use_ground=True, ground_height=-1.0,
                            self_collision=True, self_collision_mode=1 if fast else 2,
                            self_collision_interval=2 if fast else 1, max_self_collision_neighbors=32 if fast else 64,
                            fast_self_collision_passes=4, contact_friction=0.3)
        out.append(Scene(f"batch-{k}-grid-{n}", cloth, opt, np.empty((0, 3, 3), np.float32), 10, 2, frames, 1.0,
                         {"side": n, "fast": fast}))
    return out


def serving_requests(rate: float = 200.0, duration: float = 60.0, seed: int = 0, v_range: tuple = (1000, 250000),
                     horizon: tuple = (30, 240), classes: int = 16, max_requests: int | None = None) -> list:
    """Cloth solve requests for the serving form: Poisson arrivals at `rate`
    per second over `duration` seconds, vertex counts log-uniform in
    `v_range` (snapped to `classes` geometric grid sizes so cloths of one
    size share their topology), horizons uniform in `horizon` frames, a
    random sphere (r in [0.1, 0.5] m) and / or a static SDF collider (box,
    torus or both); strict self collision with 2 mm thickness as in the 10k
    drop scene; 10 substeps x 2 iterations.  Cloths keep a 1 cm vertex
    spacing, so a larger request is a larger cloth (0.3 m to 5 m), not a
    finer one."""
    from .serving import ClothRequest

    rng = np.random.default_rng(seed)
    lo, hi = math.sqrt(v_range[0]), math.sqrt(v_range[1])
    sides = sorted({int(round(lo * (hi / lo) ** (k / max(classes - 1, 1)))) for k in range(classes)})
    sdfs = [box_triangles((0.55, 0.0, -0.55), (0.25, 0.25, 0.25)), torus_triangles((-0.45, 0.1, -0.35), 0.22, 0.07, 32, 16)]
    sdfs.append(np.concatenate(sdfs).astype(np.float32))
    out, t = [], 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > duration or (max_requests is not None and len(out) >= max_requests):
            break
        v = math.exp(rng.uniform(math.log(v_range[0]), math.log(v_range[1])))
        n = min(sides, key=lambda s: abs(math.log(s * s) - math.log(v)))
        cloth = _unpinned_grid(n, 0.5, (n - 1) * 0.01)
        kind = int(rng.integers(0, 3))  # 0 sphere, 1 SDF, 2 both
        use_sphere = kind in (0, 2)
        static = sdfs[int(rng.integers(0, 3))] if kind in (1, 2) else np.empty((0, 3, 3), np.float32)
        opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, stretch_compliance=1.0e-7, bend_compliance=1.0e-4,
                            collision_margin=0.002, cloth_thickness=0.002, use_sphere=use_sphere,
                            sphere_center=(0.0, 0.0, 0.0), sphere_radius=float(rng.uniform(0.1, 0.5)), use_ground=True,
                            ground_height=-1.0, self_collision=True, self_collision_mode=2, self_collision_interval=1,
                            max_self_collision_neighbors=64, fast_self_collision_passes=4, contact_friction=0.3,
                            static_sdf_max_resolution=64)
        frames = int(rng.integers(horizon[0], horizon[1] + 1))
        out.append(ClothRequest(cloth, opt, static, frames, 10, 2, len(out), t))
    return out


def dynamic_scene(n: int = 32, frames: int = 60) -> Scene:
    """Cloth for the dynamic colliders: an unpinned n x n grid (1 m) at
    z = 0 with 2 mm thickness and 5 mm margin, friction 0.2, falling onto
    colliders that the caller moves every frame."""
    cloth = _unpinned_grid(n, 0.0)
    opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, stretch_compliance=1.0e-7, bend_compliance=1.0e-4,
                        collision_margin=0.005, cloth_thickness=0.002, contact_friction=0.2, use_ground=True,
                        ground_height=-1.0)
    return Scene(f"dynamic-{n}", cloth, opt, np.empty((0, 3, 3), np.float32), 10, 2, frames, 1.0)


def diff_scene(n: int = 64, frames: int = 60, stretch: float = 1.0e-7, bend: float = 1.0e-4) -> Scene:
    """Contact-free cloth for the differentiable form: n x n grid (1 m), the
    two corners of the y = +0.5 edge hard-pinned, 0.2 kg/m^2, damping 0.99
    per substep, gravity -9.81, no colliders; 10 substeps x 2 iterations."""
    pos, tris = grid_mesh(n, 1.0, 0.0)
    w = np.zeros(n * n, np.float32)
    w[(n - 1) * n] = 1.0
    w[n * n - 1] = 1.0
    cloth = build_cloth(pos, tris, 0.2, w)
    opt = SolverOptions(dt=1.0 / 60.0, damping=0.99, gravity=(0.0, 0.0, -9.81), stretch_compliance=stretch,
                        bend_compliance=bend, collision_margin=0.005)
    return Scene(f"diff-grid-{n}", cloth, opt, np.empty((0, 3, 3), np.float32), 10, 2, frames, 1.0)


def compliance_field(count: int, center: float, decades: float, seed: int) -> np.ndarray:
    """Seeded per-constraint compliances, log-uniform within +-`decades`
    around `center`."""
    rng = np.random.default_rng(seed)
    return (center * 10.0 ** rng.uniform(-decades, decades, count)).astype(np.float32)
