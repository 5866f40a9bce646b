"""Contact-group probe cases of the reference (tools/native_contact_group_probe.py:
analytic ground / wall / sphere / corner at :124-171, the static SDF plane at
:174-197, the self VV pair at :200-241): single vertices (and a 600-vertex
line for VV) driven into contacts with the probe's option set (:29-69).  The
probe asserts only finiteness and reports penetration, tangential drift and
contact counts; the tests built on these cases check those quantities in the
physically expected direction on the oracle, and GPU == oracle bit for bit."""
import numpy as np

from xpbd_gb300 import scene


def options(**over) -> scene.SolverOptions:
    """The probe's settings (native_contact_group_probe.py:29-69)."""
    values = dict(dt=1.0 / 60.0, damping=1.0, gravity=(0.0, 0.0, 0.0), stretch_compliance=0.0,
                  stretch_optimization_enabled=False, stretch_optimization_strength=0.0, bend_compliance=0.0,
                  lra_compliance=0.0, collision_margin=0.05, use_ground=False, ground_height=0.0, use_wall=False,
                  wall_origin=(0.0, 0.0, 0.0), wall_normal=(1.0, 0.0, 0.0), use_sphere=False,
                  sphere_center=(0.0, 0.0, 0.0), sphere_radius=0.0, self_collision=False, self_collision_mode=1,
                  cloth_thickness=0.04, self_collision_distance=0.0, self_collision_interval=1,
                  max_self_collision_neighbors=32, fast_self_collision_passes=4, use_volume_pressure=False,
                  volume_compliance=0.0, pressure_strength=0.0, volume_target_scale=1.0, volume_solve_interval=1,
                  self_probe_interval=4, self_surface_pair_interval=4, jitter_stabilizer_enabled=False,
                  contact_friction=4.0, contact_tangent_damping=1.0, contact_compliance=0.0,
                  static_sdf_voxel_size=0.02, static_sdf_band_voxels=3, static_sdf_max_resolution=64)
    values.update(over)
    return scene.SolverOptions(**values)


def cloth(positions, inv_mass=None) -> scene.ClothData:
    """Vertices without constraints (native_contact_group_probe.py:74-105)."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = len(pos)
    inv = np.ones(n, np.float32) if inv_mass is None else np.ascontiguousarray(inv_mass, np.float32)
    ei, ef = np.empty((0, 2), np.int32), np.empty(0, np.float32)
    return scene.ClothData(positions_world=pos, inv_mass=inv, triangles=np.empty((0, 3), np.int32), edges=ei,
                           edge_rest_lengths=ef, edge_color_offsets=np.empty(0, np.int32), bends=ei,
                           bend_rest_lengths=ef, bend_color_offsets=np.empty(0, np.int32), lra_edges=ei,
                           lra_rest_lengths=ef, lra_color_offsets=np.empty(0, np.int32),
                           pin_indices=np.empty(0, np.int32), pin_targets_world=np.empty((0, 3), np.float32),
                           pin_weights=np.empty(0, np.float32))


NO_STATIC = np.empty((0, 3, 3), np.float32)
PLANE = np.array([[[-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [1.0, 1.0, 0.0]],
                  [[-1.0, -1.0, 0.0], [1.0, 1.0, 0.0], [-1.0, 1.0, 0.0]]], np.float32)


def analytic(kind: str):
    """(cloth, options, static triangles, penetration(out), tangent(out)) of
    an analytic case (native_contact_group_probe.py:124-158)."""
    if kind == "ground":
        return (cloth([[0.0, 0.0, 0.02]]), options(use_ground=True, gravity=(6.0, 0.0, -6.0)), NO_STATIC,
                lambda o: max(0.0, 0.05 - float(o[0, 2])), lambda o: abs(float(o[0, 0])))
    if kind == "corner":
        return (cloth([[0.02, 0.0, 0.02]]),
                options(use_ground=True, use_wall=True, wall_normal=(1.0, 0.0, 0.0), gravity=(-6.0, 6.0, -6.0)), NO_STATIC,
                lambda o: max(0.0, 0.05 - float(o[0, 0]), 0.05 - float(o[0, 2])), lambda o: abs(float(o[0, 1])))
    if kind == "wall":
        return (cloth([[0.02, 0.0, 0.0]]), options(use_wall=True, gravity=(-6.0, 6.0, 0.0)), NO_STATIC,
                lambda o: max(0.0, 0.05 - float(o[0, 0])), lambda o: abs(float(o[0, 1])))
    if kind == "sphere":
        return (cloth([[0.30, 0.0, 0.0]]),
                options(use_sphere=True, sphere_radius=0.30, gravity=(0.0, 6.0, -1.0)), NO_STATIC,
                lambda o: max(0.0, 0.35 - float(np.linalg.norm(o[0]))), lambda o: abs(float(o[0, 1])))
    if kind == "static_sdf":
        return (cloth([[0.0, 0.0, 0.02]]), options(gravity=(6.0, 0.0, -6.0)), PLANE,
                lambda o: max(0.0, 0.05 - float(o[0, 2])), lambda o: abs(float(o[0, 0])))
    raise ValueError(kind)


KINDS = ["ground", "wall", "sphere", "corner", "static_sdf"]
STEPS, SUBSTEPS, ITERATIONS = 28, 4, 1


def free_tangent(kind: str) -> float:
    """Tangential distance a free vertex would cover under the case's
    gravity (6 m/s^2 along the tangent in every case) over the run."""
    t = STEPS / 60.0
    return 0.5 * 6.0 * t * t


def self_vv_line():
    """600 vertices 1 m apart on the x axis, vertex 599 then moved 3 cm from
    vertex 0; thickness 0.1 (native_contact_group_probe.py:200-221)."""
    n = 600
    pos = np.zeros((n, 3), np.float32)
    pos[:, 0] = np.arange(n, dtype=np.float32)
    close = pos.copy()
    close[-1] = [0.03, 0.0, 0.0]
    opts = options(self_collision=True, cloth_thickness=0.10, collision_margin=0.0, contact_friction=0.0,
                   contact_tangent_damping=0.0)
    return cloth(pos), opts, close


# ---- tools/abi41_self_collision_smoke.py: fast-mode self collision, 0.1
# thickness, no margin or friction (:26-67), one 1 x 6 step each -----------
def smoke_options() -> scene.SolverOptions:
    return options(self_collision=True, self_collision_mode=1, cloth_thickness=0.10, collision_margin=0.0,
                   contact_friction=0.0, contact_tangent_damping=0.0, static_sdf_voxel_size=0.0,
                   static_sdf_band_voxels=4, static_sdf_max_resolution=160, self_probe_interval=4,
                   self_surface_pair_interval=4)


def smoke_vv():
    """600 vertices on a line, the last moved 3 cm from vertex 0 (:70-90,
    :185-199); returns (cloth, moved positions, gap(out))."""
    cl = cloth(np.stack([np.arange(600, dtype=np.float32), np.zeros(600, np.float32), np.zeros(600, np.float32)], 1))
    close = cl.positions_world.copy()
    close[-1] = [0.03, 0.0, 0.0]
    return cl, close, lambda o: float(np.linalg.norm(o[-1] - o[0]))


def smoke_vt():
    """A pinned triangle and 63 far ones, vertex 599 moved 3 cm above the
    first (:93-132, :221-233); returns (cloth, moved positions, height(out))."""
    n, nt = 600, 64
    pos = np.zeros((n, 3), np.float32)
    inv = np.ones(n, np.float32)
    pos[0], pos[1], pos[2] = [-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [0.0, 1.0, 0.0]
    inv[:3] = 0.0
    for i in range(3, n):
        pos[i] = [20.0 + float(i), 20.0 + float(i % 7) * 0.25, float(i % 5) * 0.20]
    pos[n - 1] = [5.0, 5.0, 1.0]
    tris = np.array([[0, 1, 2]] + [[3 + t * 3, 4 + t * 3, 5 + t * 3] for t in range(1, nt)], np.int32)
    cl = cloth(pos, inv)
    cl.triangles = tris
    close = pos.copy()
    close[n - 1] = [0.0, -0.2, 0.03]
    return cl, close, lambda o: float(o[n - 1, 2])


def smoke_ee():
    """A pinned edge and a crossing edge moved 3 cm above it, 62 far edges
    (:135-176, :266-278); returns (cloth, moved positions, height(out))."""
    n, ne = 600, 64
    pos = np.zeros((n, 3), np.float32)
    inv = np.ones(n, np.float32)
    for i in range(n):
        pos[i] = [200.0 + float(i) * 3.0, 100.0 + float(i % 11), 0.0]
    pos[0], pos[1], pos[2], pos[3] = [-1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [5.0, -1.0, 0.0], [5.0, 1.0, 0.0]
    inv[:2] = 0.0
    edges = np.zeros((ne, 2), np.int32)
    edges[0], edges[1] = [0, 1], [2, 3]
    for e in range(2, ne):
        a = 4 + (e - 2) * 2
        pos[a] = [50.0 + float(e) * 4.0, 30.0, 0.0]
        pos[a + 1] = [51.0 + float(e) * 4.0, 30.0, 0.0]
        edges[e] = [a, a + 1]
    cl = cloth(pos, inv)
    cl.edges = edges
    cl.edge_rest_lengths = np.linalg.norm(pos[edges[:, 0]] - pos[edges[:, 1]], axis=1).astype(np.float32)
    close = pos.copy()
    close[2], close[3] = [0.0, -1.0, 0.03], [0.0, 1.0, 0.03]
    return cl, close, lambda o: float((o[2, 2] + o[3, 2]) * 0.5)


SMOKES = {"vv": smoke_vv, "vt": smoke_vt, "ee": smoke_ee}
