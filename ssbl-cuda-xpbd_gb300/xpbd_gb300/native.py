"""ctypes host interface of the GB300 XPBD library.

This module mirrors the reference's Python bridge (native_backend.py:
``_load_library`` :535, ``_config_from_options`` :712, ``NativeXpbdSolver``
:902-1463): same class and method names, same argument meaning, same errors
(``NativeBackendUnavailable`` when the library cannot be loaded,
``NativeSolverError`` carrying ``ssbl_last_error()`` when a call fails).  The
reference bridge itself can load this library unchanged through
``SSBL_NATIVE_DLL_PATH``; this module is the in-repo equivalent used by the
tests and the benchmark.

There is no CPU fallback: when the shared library is missing or no CUDA
device is present, construction raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .scene import ClothData, SolverOptions

_CAP_STRETCH_OPTIMIZATION = 1 << 0
_CAP_PIN_WEIGHTS = 1 << 1
_CAP_GLOBAL_DYNAMIC_SCENE = 1 << 2

F3 = ctypes.c_float * 3


class NativeBackendUnavailable(RuntimeError):
    pass


class NativeSolverError(RuntimeError):
    pass


class NativeConfig(ctypes.Structure):
    _fields_ = [
        ("vertex_count", ctypes.c_int), ("edge_count", ctypes.c_int), ("bend_count", ctypes.c_int),
        ("lra_count", ctypes.c_int), ("triangle_count", ctypes.c_int), ("static_triangle_count", ctypes.c_int),
        ("edge_color_count", ctypes.c_int), ("bend_color_count", ctypes.c_int), ("lra_color_count", ctypes.c_int),
        ("dt", ctypes.c_float), ("damping", ctypes.c_float), ("gravity", F3), ("stretch_compliance", ctypes.c_float),
        ("bend_compliance", ctypes.c_float), ("lra_compliance", ctypes.c_float), ("collision_margin", ctypes.c_float),
        ("use_ground", ctypes.c_int), ("ground_height", ctypes.c_float), ("use_wall", ctypes.c_int),
        ("wall_origin", F3), ("wall_normal", F3), ("use_sphere", ctypes.c_int), ("sphere_center", F3),
        ("sphere_radius", ctypes.c_float), ("self_collision", ctypes.c_int), ("self_collision_mode", ctypes.c_int),
        ("cloth_thickness", ctypes.c_float), ("self_collision_distance", ctypes.c_float),
        ("self_collision_interval", ctypes.c_int), ("max_self_collision_neighbors", ctypes.c_int),
        ("use_volume_pressure", ctypes.c_int), ("rest_volume", ctypes.c_float), ("volume_compliance", ctypes.c_float),
        ("pressure_strength", ctypes.c_float), ("volume_target_scale", ctypes.c_float),
        ("volume_solve_interval", ctypes.c_int), ("self_probe_interval", ctypes.c_int),
        ("self_surface_pair_interval", ctypes.c_int), ("jitter_stabilizer_enabled", ctypes.c_int),
        ("contact_friction", ctypes.c_float), ("contact_tangent_damping", ctypes.c_float),
        ("contact_compliance", ctypes.c_float), ("fast_self_collision_passes", ctypes.c_int),
        ("stretch_optimization_enabled", ctypes.c_int), ("stretch_optimization_strength", ctypes.c_float),
        ("static_sdf_voxel_size", ctypes.c_float), ("static_sdf_band_voxels", ctypes.c_int),
        ("static_sdf_max_resolution", ctypes.c_int),
    ]


_PF = ctypes.POINTER(ctypes.c_float)
_PI = ctypes.POINTER(ctypes.c_int)


class NativeMesh(ctypes.Structure):
    _fields_ = [
        ("positions", _PF), ("inv_mass", _PF), ("edges", _PI), ("edge_rest_lengths", _PF),
        ("edge_color_offsets", _PI), ("bends", _PI), ("bend_rest_lengths", _PF), ("bend_color_offsets", _PI),
        ("lra_edges", _PI), ("lra_rest_lengths", _PF), ("lra_color_offsets", _PI), ("triangles", _PI),
        ("static_triangles", _PF),
    ]


class NativeRuntimeColliders(ctypes.Structure):
    _fields_ = [
        ("use_ground", ctypes.c_int), ("ground_height", ctypes.c_float), ("use_wall", ctypes.c_int),
        ("wall_origin", F3), ("wall_normal", F3), ("use_sphere", ctypes.c_int), ("sphere_center", F3),
        ("sphere_radius", ctypes.c_float),
    ]


class NativeForceField(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int), ("use_min_distance", ctypes.c_int), ("use_max_distance", ctypes.c_int),
        ("seed", ctypes.c_int), ("strength", ctypes.c_float), ("origin", F3), ("direction", F3), ("axis", F3),
        ("falloff_power", ctypes.c_float), ("distance_min", ctypes.c_float), ("distance_max", ctypes.c_float),
        ("radial_min", ctypes.c_float), ("radial_max", ctypes.c_float), ("noise", ctypes.c_float),
        ("linear_drag", ctypes.c_float), ("quadratic_drag", ctypes.c_float), ("harmonic_damping", ctypes.c_float),
        ("flow", ctypes.c_float), ("size", ctypes.c_float), ("rest_length", ctypes.c_float),
        ("radial_falloff", ctypes.c_float), ("texture_nabla", ctypes.c_float), ("use_radial_min", ctypes.c_int),
        ("use_radial_max", ctypes.c_int), ("use_2d_force", ctypes.c_int), ("use_global_coords", ctypes.c_int),
        ("apply_to_location", ctypes.c_int),
    ]


class NativeFrameInputs(ctypes.Structure):
    _fields_ = [
        ("update_pin_targets", ctypes.c_int), ("pin_indices", _PI), ("pin_positions", _PF), ("pin_weights", _PF),
        ("pin_count", ctypes.c_int), ("update_runtime_colliders", ctypes.c_int),
        ("runtime_colliders", NativeRuntimeColliders), ("update_static_triangles", ctypes.c_int),
        ("static_triangles", _PF), ("static_triangle_count", ctypes.c_int), ("update_dynamic_triangles", ctypes.c_int),
        ("dynamic_triangles", _PF), ("dynamic_triangle_count", ctypes.c_int),
        ("update_dynamic_indexed_triangles", ctypes.c_int), ("dynamic_triangle_vertices", _PF),
        ("dynamic_triangle_vertex_count", ctypes.c_int), ("dynamic_triangle_indices", _PI),
        ("dynamic_indexed_triangle_count", ctypes.c_int), ("dynamic_triangle_topology_changed", ctypes.c_int),
        ("update_dynamic_particles", ctypes.c_int), ("dynamic_particle_positions", _PF),
        ("dynamic_particle_radii", _PF), ("dynamic_particle_inv_mass", _PF), ("dynamic_particle_slot_ids", _PI),
        ("dynamic_particle_phases", _PI), ("dynamic_particle_count", ctypes.c_int),
        ("update_force_fields", ctypes.c_int), ("force_fields", ctypes.POINTER(NativeForceField)),
        ("force_field_count", ctypes.c_int), ("unsupported_force_field_count", ctypes.c_int),
    ]


_DIAG_FLOATS = {
    "step_ms", "hash_build_ms", "constraints_ms", "volume_ms", "analytic_collision_ms", "static_collision_ms",
    "dynamic_collision_ms", "dynamic_particle_collision_ms", "self_hash_ms", "self_solve_ms", "self_probe_ms",
    "self_recovery_ms", "sync_ms", "diagnostics_fetch_ms", "min_gap", "jitter_max_correction",
    "fast_soft_repulsion_max_push", "fast_barrier_max_delta", "fast_overlap_island_max_delta",
    "fast_cc_overlap_max_delta", "abi41_max_smoothed_delta", "static_sdf_build_ms", "abi41_pcg_initial_residual",
    "abi41_pcg_final_residual", "abi41_pcg_max_delta", "dynamic_collider_pack_ms", "dynamic_triangle_upload_ms",
    "dynamic_particle_upload_ms", "abi41_pcg_solve_ms", "abi41_pcg_system_ms", "abi41_pcg_ad_ms",
    "abi41_direct_stretch_ms", "global_dynamic_scene_pack_ms", "global_dynamic_scene_upload_ms",
    "global_dynamic_hash_ms",
}
_DIAG_ORDER = """step_ms hash_build_ms constraints_ms volume_ms analytic_collision_ms static_collision_ms
dynamic_collision_ms dynamic_particle_collision_ms self_hash_ms self_solve_ms self_probe_ms self_recovery_ms sync_ms
diagnostics_fetch_ms candidate_count resolved_contacts min_gap ccd_clamp_count recovery_passes local_retry_count
jitter_stabilized_vertices jitter_rejected_vertices jitter_max_correction external_contact_cache_hits
external_contact_cache_misses external_contact_cache_count external_contact_cache_overflow
external_friction_corrections force_field_count unsupported_force_field_count dynamic_particle_count
dynamic_particle_candidate_count dynamic_particle_contacts dynamic_particle_overflow dynamic_triangle_count
static_triangle_count finite_flag fast_exact_vt_candidates fast_exact_vt_projected fast_exact_vt_guarded
fast_exact_vt_skipped_rest fast_soft_repulsion_candidates fast_soft_repulsion_applied fast_soft_repulsion_max_push
fast_hard_projection_count fast_manifold_contacts fast_manifold_reused fast_barrier_projected
fast_barrier_smoothed_vertices fast_barrier_overflow fast_barrier_max_delta fast_edge_edge_candidates
fast_edge_edge_contacts fast_triangle_pair_candidates fast_triangle_pair_contacts fast_triangle_pair_skipped_rest
fast_contact_classification_guarded fast_region_cluster_candidates fast_region_cluster_contacts
fast_region_cluster_guarded fast_overlap_island_candidates fast_overlap_island_clusters
fast_overlap_island_vertex_refs fast_overlap_island_applied_vertices fast_overlap_island_guarded
fast_overlap_island_max_delta fast_cc_overlap_components fast_cc_overlap_seed_triangles fast_cc_overlap_owned_vertices
fast_cc_overlap_union_edges fast_cc_overlap_guarded fast_cc_overlap_applied_vertices fast_cc_overlap_max_delta
abi41_soft_contact_count abi41_exact_impulse_contact_count abi41_edge_edge_contact_count abi41_max_smoothed_delta
abi41_hard_projection_fallbacks static_sdf_rebuild_count static_sdf_voxel_count static_sdf_grid_x static_sdf_grid_y
static_sdf_grid_z static_sdf_build_ms static_sdf_contact_count static_sdf_unsigned_fallback_count
abi41_pcg_iterations abi41_pcg_guarded abi41_pcg_csr_nnz abi41_pcg_texture_ready abi41_pcg_initial_residual
abi41_pcg_final_residual abi41_pcg_max_delta abi41_lra_tack_count abi41_bending_wing_count
abi41_bending_texture_ready abi41_tack_jitter_guarded abi41_bending_guarded dynamic_collider_pack_ms
dynamic_triangle_upload_ms dynamic_particle_upload_ms dynamic_collider_cache_hits dynamic_collider_cache_misses
abi41_pcg_solve_ms abi41_pcg_system_ms abi41_pcg_ad_ms abi41_direct_stretch_ms dynamic_pair_cache_hits
dynamic_pair_cache_misses dynamic_pair_cache_reused_triangles dynamic_pair_cache_reused_particles
dynamic_collision_skipped_launches self_collision_skipped_launches self_candidate_count self_filter_seen
self_filter_accepted_vv self_filter_accepted_vt self_filter_accepted_ee self_filter_rejected_rest
self_filter_rejected_duplicate self_filter_rejected_ownership self_filter_cache_hits self_filter_cache_misses
self_cluster_count self_cluster_owned_contacts dynamic_triangle_candidate_count dynamic_triangle_bucket_overflow
dynamic_triangle_large_primitive_count dynamic_triangle_aabb_reject_count dynamic_triangle_max_bucket_occupancy
global_dynamic_scene_pack_ms global_dynamic_scene_upload_ms global_dynamic_hash_ms global_dynamic_particle_count
global_dynamic_triangle_count global_dynamic_hash_overflow""".split()


class NativeDiagnostics(ctypes.Structure):
    _fields_ = [
        (n, ctypes.c_float if n in _DIAG_FLOATS else (ctypes.c_int if n == "finite_flag" else ctypes.c_longlong))
        for n in _DIAG_ORDER
    ]


# ------------------------------------------------------------ loading ----
_LIBS: dict = {}


def dll_path() -> str:
    """Library path: SSBL_NATIVE_DLL_PATH, else the in-tree build."""
    override = os.environ.get("SSBL_NATIVE_DLL_PATH")
    if override:
        return override
    from .build import library_path

    return library_path()


def _load_library(path: str | None = None):
    """Load (once per path) an ABI41 library: this repository's by default,
    or any drop-in of the same interface given by `path` (the parity tests
    load the reference's solver beside it)."""
    path = path or dll_path()
    if path in _LIBS:
        return _LIBS[path]
    if not os.path.exists(path):
        raise NativeBackendUnavailable(f"Missing GB300 XPBD library: {path} (run the package build first)")
    try:
        lib = ctypes.CDLL(path)
    except OSError as exc:
        raise NativeBackendUnavailable(f"Unable to load GB300 XPBD library: {exc}") from exc
    vp = ctypes.c_void_p
    sig = {
        "ssbl_create_solver": (vp, [ctypes.POINTER(NativeConfig), ctypes.POINTER(NativeMesh)]),
        "ssbl_destroy_solver": (ctypes.c_int, [vp]),
        "ssbl_reset_solver": (ctypes.c_int, [vp]),
        "ssbl_update_pin_targets": (ctypes.c_int, [vp, _PI, _PF, _PF, ctypes.c_int]),
        "ssbl_update_runtime_colliders": (ctypes.c_int, [vp, ctypes.POINTER(NativeRuntimeColliders)]),
        "ssbl_update_positions": (ctypes.c_int, [vp, _PF, ctypes.c_int]),
        "ssbl_update_static_triangles": (ctypes.c_int, [vp, _PF, ctypes.c_int]),
        "ssbl_update_dynamic_triangles": (ctypes.c_int, [vp, _PF, ctypes.c_int]),
        "ssbl_update_frame_inputs": (ctypes.c_int, [vp, ctypes.POINTER(NativeFrameInputs)]),
        "ssbl_step_solver": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "ssbl_step_solver_ex": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "ssbl_download_positions": (ctypes.c_int, [vp, _PF, ctypes.c_int]),
        "ssbl_get_diagnostics": (ctypes.c_int, [vp, ctypes.POINTER(NativeDiagnostics)]),
        "ssbl_capabilities": (ctypes.c_uint, []),
        "ssbl_create_global_dynamic_scene": (vp, []),
        "ssbl_destroy_global_dynamic_scene": (ctypes.c_int, [vp]),
        "ssbl_update_global_dynamic_scene": (ctypes.c_int, [vp, ctypes.POINTER(NativeGlobalSceneInputs)]),
        "ssbl_attach_global_dynamic_scene": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "ssbl_clear_global_dynamic_scene": (ctypes.c_int, [vp]),
        "ssbl_last_error": (ctypes.c_char_p, []),
        "xpbd_gb300_build_self_structures": (ctypes.c_int, [vp]),
        "xpbd_gb300_read_buffer": (ctypes.c_longlong, [vp, ctypes.c_int, vp, ctypes.c_longlong]),
        "xpbd_gb300_hash_info": (ctypes.c_int, [vp, _PI]),
        "xpbd_gb300_set_graph_capture": (ctypes.c_int, [vp, ctypes.c_int]),
        "xpbd_gb300_set_key_division": (ctypes.c_int, [vp, ctypes.c_int]),
        "xpbd_gb300_set_default_key_division": (ctypes.c_int, [ctypes.c_int]),
        "xpbd_gb300_last_step_launches": (ctypes.c_longlong, [vp]),
        "xpbd_gb300_synchronize": (ctypes.c_int, [vp]),
        "xpbd_gb300_stream": (vp, [vp]),
        "xpbd_gb300_profile_frame": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _PF,
                                                    ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
        "xpbd_gb300_profile_counters": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong)]),
        "xpbd_gb300_device_bytes": (ctypes.c_longlong, [vp]),
        "xpbd_gb300_set_launch_config": (ctypes.c_int, [vp, _PI, ctypes.c_int]),
        "xpbd_gb300_get_launch_config": (ctypes.c_int, [vp, _PI, ctypes.c_int]),
        "xpbd_gb300_solver_info": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong)]),
        "xpbd_gb300_autotune": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _PF]),
        "xpbd_gb300_prepare_graph": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "xpbd_gb300_batch_create": (vp, [ctypes.POINTER(NativeConfig), ctypes.POINTER(NativeMesh), ctypes.c_int]),
        "xpbd_gb300_batch_cloth_count": (ctypes.c_int, [vp]),
        "xpbd_gb300_batch_cloth_range": (ctypes.c_int, [vp, ctypes.c_int, _PI]),
        "xpbd_gb300_batch_update_pin_targets": (ctypes.c_int, [vp, ctypes.c_int, _PI, _PF, _PF, ctypes.c_int]),
        "xpbd_gb300_batch_update_runtime_colliders": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(NativeRuntimeColliders)]),
        "xpbd_gb300_batch_update_static_triangles": (ctypes.c_int, [vp, ctypes.c_int, _PF, ctypes.c_int]),
        "xpbd_gb300_batch_update_frame_inputs": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(NativeFrameInputs)]),
        "xpbd_gb300_batch_attach_global_dynamic_scene": (ctypes.c_int, [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int,
                                                                         ctypes.c_int]),
        "xpbd_gb300_batch_clear_global_dynamic_scene": (ctypes.c_int, [vp, ctypes.c_int]),
        "xpbd_gb300_batch_update_positions": (ctypes.c_int, [vp, ctypes.c_int, _PF, ctypes.c_int]),
        "xpbd_gb300_batch_download_positions": (ctypes.c_int, [vp, ctypes.c_int, _PF, ctypes.c_int]),
        "xpbd_gb300_batch_reset_cloth": (ctypes.c_int, [vp, ctypes.c_int]),
        "xpbd_gb300_batch_set_active": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
    _LIBS[path] = lib
    return lib


def _fp(a: np.ndarray):
    return _PF() if a is None or a.size == 0 else a.ctypes.data_as(_PF)


def _ip(a: np.ndarray):
    return _PI() if a is None or a.size == 0 else a.ctypes.data_as(_PI)


def _last_error(lib) -> str:
    raw = lib.ssbl_last_error()
    return raw.decode("utf-8", errors="replace") if raw else "GB300 XPBD call failed without an error message."


KEY_DIVISION = {"reference": 0, "ieee": 1}


def set_default_key_division(mode: str) -> None:
    """Cell-key division of the solvers and scenes created from now on in this
    process: "reference" (the default; the reference's fast-math division, so
    hash keys are its integers) or "ieee" (the correctly rounded quotient of
    the CPU oracle)."""
    lib = _load_library()
    if not lib.xpbd_gb300_set_default_key_division(KEY_DIVISION[mode]):
        raise NativeSolverError(_last_error(lib))


def capabilities(library: str | None = None) -> int:
    return int(_load_library(library).ssbl_capabilities())


def config_from_options(cloth: ClothData, options: SolverOptions, static_triangles: np.ndarray) -> NativeConfig:
    """Fill the ABI41 config exactly like native_backend.py:712-766."""
    c = NativeConfig()
    c.vertex_count = len(cloth.positions_world)
    c.edge_count = len(cloth.edges)
    c.bend_count = len(cloth.bends)
    c.lra_count = len(cloth.lra_edges)
    c.triangle_count = len(cloth.triangles)
    c.static_triangle_count = len(static_triangles)
    c.edge_color_count = max(len(cloth.edge_color_offsets) - 1, 0)
    c.bend_color_count = max(len(cloth.bend_color_offsets) - 1, 0)
    c.lra_color_count = max(len(cloth.lra_color_offsets) - 1, 0)
    o = options
    c.dt, c.damping = float(o.dt), float(o.damping)
    c.gravity = F3(*map(float, o.gravity))
    c.stretch_compliance, c.bend_compliance, c.lra_compliance = map(float, (o.stretch_compliance, o.bend_compliance, o.lra_compliance))
    c.collision_margin = float(o.collision_margin)
    c.use_ground, c.ground_height = int(o.use_ground), float(o.ground_height)
    c.use_wall = int(o.use_wall)
    c.wall_origin, c.wall_normal = F3(*map(float, o.wall_origin)), F3(*map(float, o.wall_normal))
    c.use_sphere, c.sphere_center, c.sphere_radius = int(o.use_sphere), F3(*map(float, o.sphere_center)), float(o.sphere_radius)
    c.self_collision, c.self_collision_mode = int(o.self_collision), int(o.self_collision_mode)
    c.cloth_thickness, c.self_collision_distance = float(o.cloth_thickness), float(o.self_collision_distance)
    c.self_collision_interval, c.max_self_collision_neighbors = int(o.self_collision_interval), int(o.max_self_collision_neighbors)
    c.use_volume_pressure, c.rest_volume = int(o.use_volume_pressure), float(cloth.rest_volume)
    c.volume_compliance, c.pressure_strength = float(o.volume_compliance), float(o.pressure_strength)
    c.volume_target_scale, c.volume_solve_interval = float(o.volume_target_scale), int(o.volume_solve_interval)
    c.self_probe_interval, c.self_surface_pair_interval = int(o.self_probe_interval), int(o.self_surface_pair_interval)
    c.jitter_stabilizer_enabled = int(o.jitter_stabilizer_enabled)
    c.contact_friction, c.contact_tangent_damping = float(o.contact_friction), float(o.contact_tangent_damping)
    c.contact_compliance, c.fast_self_collision_passes = float(o.contact_compliance), int(o.fast_self_collision_passes)
    c.stretch_optimization_enabled = int(o.stretch_optimization_enabled)
    c.stretch_optimization_strength = float(o.stretch_optimization_strength)
    c.static_sdf_voxel_size, c.static_sdf_band_voxels = float(o.static_sdf_voxel_size), int(o.static_sdf_band_voxels)
    c.static_sdf_max_resolution = int(o.static_sdf_max_resolution)
    return c


def colliders_from_options(o: SolverOptions) -> NativeRuntimeColliders:
    r = NativeRuntimeColliders()
    r.use_ground, r.ground_height, r.use_wall = int(o.use_ground), float(o.ground_height), int(o.use_wall)
    r.wall_origin, r.wall_normal = F3(*map(float, o.wall_origin)), F3(*map(float, o.wall_normal))
    r.use_sphere, r.sphere_center, r.sphere_radius = int(o.use_sphere), F3(*map(float, o.sphere_center)), float(o.sphere_radius)
    return r


def mesh_arrays(cloth: ClothData, static_triangles: np.ndarray) -> tuple[NativeMesh, list]:
    """ABI41 mesh struct plus the arrays it points into (keep them alive)."""
    keep = [
        np.ascontiguousarray(cloth.positions_world, np.float32), np.ascontiguousarray(cloth.inv_mass, np.float32),
        np.ascontiguousarray(cloth.edges, np.int32), np.ascontiguousarray(cloth.edge_rest_lengths, np.float32),
        np.ascontiguousarray(cloth.edge_color_offsets, np.int32), np.ascontiguousarray(cloth.bends, np.int32),
        np.ascontiguousarray(cloth.bend_rest_lengths, np.float32), np.ascontiguousarray(cloth.bend_color_offsets, np.int32),
        np.ascontiguousarray(cloth.lra_edges, np.int32), np.ascontiguousarray(cloth.lra_rest_lengths, np.float32),
        np.ascontiguousarray(cloth.lra_color_offsets, np.int32), np.ascontiguousarray(cloth.triangles, np.int32),
        np.ascontiguousarray(np.asarray(static_triangles, np.float32).reshape(-1, 3)),
    ]
    m = NativeMesh(_fp(keep[0]), _fp(keep[1]), _ip(keep[2]), _fp(keep[3]), _ip(keep[4]), _ip(keep[5]), _fp(keep[6]),
                   _ip(keep[7]), _ip(keep[8]), _fp(keep[9]), _ip(keep[10]), _ip(keep[11]), _fp(keep[12]))
    return m, keep


class NativeGlobalSceneInputs(ctypes.Structure):
    """SsblXpbdGlobalDynamicSceneInputs (native/include/ssbl_xpbd_cuda.h:299-312)."""

    _fields_ = [
        ("particle_positions", _PF), ("particle_prev_positions", _PF), ("particle_radii", _PF),
        ("particle_source_ids", _PI), ("particle_collision_layers", _PI), ("particle_count", ctypes.c_int),
        ("triangle_vertices", _PF), ("triangle_source_ids", _PI), ("triangle_collision_layers", _PI),
        ("triangle_count", ctypes.c_int), ("collision_margin", ctypes.c_float), ("cloth_thickness", ctypes.c_float),
    ]


def scene_inputs(triangles=None, particles=None, margin: float = 0.0, thickness: float = 0.0):
    """NativeGlobalSceneInputs (and the arrays it points to) from
    triangles = (rows (T, 3, 3), source ids (T,), layers (T,)) and
    particles = (positions (P, 3), previous positions (P, 3) or None,
    radii (P,), source ids (P,), layers (P,))."""
    fi = NativeGlobalSceneInputs()
    keep = []
    if triangles is not None:
        rows, src, layer = triangles
        t = np.ascontiguousarray(np.asarray(rows, np.float32).reshape(-1, 9))
        ts = np.ascontiguousarray(src, np.int32).reshape(-1)
        tl = np.ascontiguousarray(layer, np.int32).reshape(-1)
        if len(ts) != len(t) or len(tl) != len(t):
            raise ValueError("one source id and one layer per scene triangle")
        keep += [t, ts, tl]
        fi.triangle_vertices, fi.triangle_source_ids, fi.triangle_collision_layers = _fp(t), _ip(ts), _ip(tl)
        fi.triangle_count = len(t)
    if particles is not None:
        pos, prev, rad, src, layer = particles
        p = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1, 3))
        q = None if prev is None else np.ascontiguousarray(np.asarray(prev, np.float32).reshape(-1, 3))
        r = np.ascontiguousarray(rad, np.float32).reshape(-1)
        ps = np.ascontiguousarray(src, np.int32).reshape(-1)
        pl = np.ascontiguousarray(layer, np.int32).reshape(-1)
        if not (len(r) == len(ps) == len(pl) == len(p)) or (q is not None and len(q) != len(p)):
            raise ValueError("one previous position, radius, source id and layer per scene particle")
        keep += [p, r, ps, pl] + ([q] if q is not None else [])
        fi.particle_positions, fi.particle_radii = _fp(p), _fp(r)
        fi.particle_prev_positions = _fp(q) if q is not None else _PF()
        fi.particle_source_ids, fi.particle_collision_layers = _ip(ps), _ip(pl)
        fi.particle_count = len(p)
    fi.collision_margin = float(margin)
    fi.cloth_thickness = float(thickness)
    return fi, keep


class GlobalDynamicScene:
    """Shared dynamic scene (ssbl_create_global_dynamic_scene): colliders of
    many sources hashed once on the device; every attached cloth reads them
    through its source filter."""

    def __init__(self):
        self._lib = _load_library()
        self._handle = self._lib.ssbl_create_global_dynamic_scene()
        if not self._handle:
            raise NativeSolverError(_last_error(self._lib))

    @property
    def handle(self) -> int:
        return self._handle

    def update(self, triangles=None, particles=None, margin: float = 0.0, thickness: float = 0.0) -> None:
        fi, keep = scene_inputs(triangles, particles, margin, thickness)
        if not self._lib.ssbl_update_global_dynamic_scene(self._handle, ctypes.byref(fi)):
            raise NativeSolverError(_last_error(self._lib))
        del keep

    def close(self) -> None:
        if getattr(self, "_handle", None):
            self._lib.ssbl_destroy_global_dynamic_scene(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dynamic_frame_inputs(triangles, indexed, particles):
    fi = NativeFrameInputs()
    keep = []
    if triangles is not None:
        t = np.ascontiguousarray(np.asarray(triangles, np.float32).reshape(-1, 9))
        keep.append(t)
        fi.update_dynamic_triangles, fi.dynamic_triangles, fi.dynamic_triangle_count = 1, _fp(t), len(t)
    if indexed is not None:
        verts, idx, changed = indexed
        v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 3))
        ix = np.ascontiguousarray(np.asarray(idx, np.int32).reshape(-1, 3))
        keep += [v, ix]
        fi.update_dynamic_indexed_triangles = 1
        fi.dynamic_triangle_vertices, fi.dynamic_triangle_vertex_count = _fp(v), len(v)
        fi.dynamic_triangle_indices, fi.dynamic_indexed_triangle_count = _ip(ix), len(ix)
        fi.dynamic_triangle_topology_changed = 1 if changed else 0
    if particles is not None:
        pos, rad = particles
        p = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1, 3))
        r = np.ascontiguousarray(np.asarray(rad, np.float32).reshape(-1))
        if len(r) != len(p):
            raise ValueError("one radius per dynamic particle")
        keep += [p, r]
        fi.update_dynamic_particles = 1
        fi.dynamic_particle_positions, fi.dynamic_particle_radii, fi.dynamic_particle_count = _fp(p), _fp(r), len(p)
    return fi, keep


class NativeXpbdSolver:
    """One cloth on the GPU (the reference's NativeXpbdSolver interface)."""

    def __init__(self, cloth: ClothData, options: SolverOptions, static_triangles: np.ndarray,
                 library: str | None = None, key_division: str | None = None):
        self._lib = _load_library(library)
        caps = capabilities(library)
        if options.stretch_optimization_enabled and not caps & _CAP_STRETCH_OPTIMIZATION:
            raise NativeSolverError("Loaded CUDA solver library does not support hard stretch optimization.")
        if not caps & _CAP_PIN_WEIGHTS:
            raise NativeSolverError("Loaded CUDA solver library does not support vertex-group pin weights.")
        self._vertex_count = len(cloth.positions_world)
        self._positions_out = np.empty((self._vertex_count, 3), np.float32)
        self._static_triangle_count = len(static_triangles)
        cfg = config_from_options(cloth, options, static_triangles)
        mesh, keep = mesh_arrays(cloth, static_triangles)
        self._handle = self._lib.ssbl_create_solver(ctypes.byref(cfg), ctypes.byref(mesh))
        del keep
        if not self._handle:
            raise NativeSolverError(_last_error(self._lib))
        if key_division is not None:
            self.set_key_division(key_division)
        if len(cloth.pin_indices) > 0:
            self.update_pin_targets(cloth.pin_indices, cloth.pin_targets_world, cloth.pin_weights)

    @classmethod
    def from_raw(cls, config: NativeConfig, mesh: NativeMesh, pins=None, library: str | None = None) -> "NativeXpbdSolver":
        """Create from ABI41 structs directly (the pointers in `mesh` must
        stay valid for the call)."""
        self = cls.__new__(cls)
        self._lib = _load_library(library)
        self._vertex_count = int(config.vertex_count)
        self._positions_out = np.empty((self._vertex_count, 3), np.float32)
        self._static_triangle_count = int(config.static_triangle_count)
        self._handle = self._lib.ssbl_create_solver(ctypes.byref(config), ctypes.byref(mesh))
        if not self._handle:
            raise NativeSolverError(_last_error(self._lib))
        if pins is not None and len(pins[0]) > 0:
            self.update_pin_targets(*pins)
        return self

    @property
    def handle(self) -> int:
        return self._handle

    def close(self) -> None:
        if getattr(self, "_handle", None):
            self._lib.ssbl_clear_global_dynamic_scene(self._handle)
            self._lib.ssbl_destroy_solver(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, ok) -> None:
        if not ok:
            raise NativeSolverError(_last_error(self._lib))

    def reset(self) -> None:
        self._check(self._lib.ssbl_reset_solver(self._handle))

    def update_pin_targets(self, indices, positions, weights=None) -> None:
        idx = np.ascontiguousarray(indices, np.int32)
        pos = np.ascontiguousarray(positions, np.float32)
        w = np.ones(len(idx), np.float32) if weights is None else np.ascontiguousarray(weights, np.float32).reshape(-1)
        if len(idx) != len(pos) or len(idx) != len(w):
            raise NativeSolverError("Pin index, target, and weight arrays must have matching lengths.")
        self._check(self._lib.ssbl_update_pin_targets(self._handle, _ip(idx), _fp(pos), _fp(w), len(idx)))

    def update_runtime_colliders(self, options: SolverOptions) -> None:
        self._colliders = colliders_from_options(options)
        self._check(self._lib.ssbl_update_runtime_colliders(self._handle, ctypes.byref(self._colliders)))

    def update_positions(self, positions: np.ndarray) -> None:
        p = np.ascontiguousarray(positions, np.float32)
        if p.shape != (self._vertex_count, 3):
            raise NativeSolverError(f"Position upload expected shape ({self._vertex_count}, 3), got {tuple(p.shape)}.")
        self._check(self._lib.ssbl_update_positions(self._handle, _fp(p), p.size))

    def update_static_triangles(self, static_triangles: np.ndarray) -> None:
        n = len(static_triangles)
        if n <= 0 and self._static_triangle_count <= 0:
            return
        t = np.ascontiguousarray(np.asarray(static_triangles, np.float32).reshape(-1, 3))
        self._check(self._lib.ssbl_update_static_triangles(self._handle, _fp(t), n))
        self._static_triangle_count = n

    def update_frame_inputs(self, *, pin_indices=None, pin_positions=None, pin_weights=None, update_pin=False,
                            options: SolverOptions | None = None, static_triangles=None) -> None:
        fi = NativeFrameInputs()
        keep = []
        if update_pin:
            idx = np.ascontiguousarray(pin_indices, np.int32)
            pos = np.ascontiguousarray(pin_positions, np.float32)
            w = np.ones(len(idx), np.float32) if pin_weights is None else np.ascontiguousarray(pin_weights, np.float32)
            keep += [idx, pos, w]
            fi.update_pin_targets, fi.pin_indices, fi.pin_positions, fi.pin_weights, fi.pin_count = 1, _ip(idx), _fp(pos), _fp(w), len(idx)
        if options is not None:
            fi.update_runtime_colliders = 1
            fi.runtime_colliders = colliders_from_options(options)
        if static_triangles is not None:
            t = np.ascontiguousarray(np.asarray(static_triangles, np.float32).reshape(-1, 3))
            keep.append(t)
            fi.update_static_triangles, fi.static_triangles, fi.static_triangle_count = 1, _fp(t), len(t) // 3
        self._check(self._lib.ssbl_update_frame_inputs(self._handle, ctypes.byref(fi)))

    def update_force_fields(self, fields, unsupported: int = 0) -> None:
        """Replace the force fields (a sequence of NativeForceField, at most
        64) through ssbl_update_frame_inputs."""
        arr = (NativeForceField * max(len(fields), 1))(*fields)
        fi = NativeFrameInputs()
        fi.update_force_fields = 1
        fi.force_fields = ctypes.cast(arr, ctypes.POINTER(NativeForceField)) if len(fields) else None
        fi.force_field_count = len(fields)
        fi.unsupported_force_field_count = int(unsupported)
        self._check(self._lib.ssbl_update_frame_inputs(self._handle, ctypes.byref(fi)))

    def update_dynamic_colliders(self, *, triangles=None, indexed=None, particles=None) -> None:
        """Replace dynamic colliders through ssbl_update_frame_inputs.

        triangles: (T, 3, 3) plain triangles (unsigned response);
        indexed: (vertices (N, 3), indices (T, 3), topology_changed) of a
        closed mesh (signed response); particles: (positions (P, 3), radii
        (P,)).  An empty array clears that kind; None leaves it unchanged."""
        fi, keep = _dynamic_frame_inputs(triangles, indexed, particles)
        self._check(self._lib.ssbl_update_frame_inputs(self._handle, ctypes.byref(fi)))
        del keep

    def attach_global_scene(self, scene: "GlobalDynamicScene", target_source_id: int = 0, target_collision_layer: int = 0,
                            mode: int = 1) -> None:
        """Read the scene's colliders in the unsigned dynamic stage (mode 1:
        all but the target source, 2: only layers below the target's; 0:
        keep the own colliders)."""
        self._check(self._lib.ssbl_attach_global_dynamic_scene(self._handle, scene.handle, int(target_source_id),
                                                               int(target_collision_layer), int(mode)))
        self._scene_ref = scene

    def clear_global_scene(self) -> None:
        self._check(self._lib.ssbl_clear_global_dynamic_scene(self._handle))
        self._scene_ref = None

    def step(self, substeps: int, iterations: int, diagnostics: bool = True, synchronize: bool = True) -> None:
        fetch = 1 if diagnostics else 0
        sync = 1 if (synchronize or diagnostics) else 0
        self._check(self._lib.ssbl_step_solver_ex(self._handle, int(substeps), int(iterations), fetch, sync))

    def download_positions(self) -> np.ndarray:
        out = self._positions_out
        self._check(self._lib.ssbl_download_positions(self._handle, _fp(out), out.size))
        return out

    def diagnostics(self) -> dict:
        raw = NativeDiagnostics()
        self._check(self._lib.ssbl_get_diagnostics(self._handle, ctypes.byref(raw)))
        return {name: getattr(raw, name) for name, _ in NativeDiagnostics._fields_}

    # ---- GB300 extensions -------------------------------------------------
    def build_self_structures(self) -> None:
        self._check(self._lib.xpbd_gb300_build_self_structures(self._handle))

    def read_buffer(self, buffer_id: int, dtype, count: int) -> np.ndarray:
        out = np.empty(count, dtype=dtype)
        n = self._lib.xpbd_gb300_read_buffer(self._handle, int(buffer_id), out.ctypes.data, out.nbytes)
        if n < 0:
            raise NativeSolverError(_last_error(self._lib))
        return out[: n // out.itemsize]

    def hash_info(self) -> np.ndarray:
        out = np.zeros(6, np.int32)
        self._check(self._lib.xpbd_gb300_hash_info(self._handle, _ip(out)))
        return out

    def set_key_division(self, mode: str) -> None:
        """"reference" or "ieee" cell-key division (set_default_key_division)."""
        self._check(self._lib.xpbd_gb300_set_key_division(self._handle, KEY_DIVISION[mode]))

    def set_graph_capture(self, enabled: bool) -> None:
        self._check(self._lib.xpbd_gb300_set_graph_capture(self._handle, 1 if enabled else 0))

    def last_step_launches(self) -> int:
        return int(self._lib.xpbd_gb300_last_step_launches(self._handle))

    def synchronize(self) -> None:
        self._check(self._lib.xpbd_gb300_synchronize(self._handle))

    def prepare_graph(self, substeps: int, iterations: int) -> None:
        """Capture the frame graph now (no frame is run)."""
        self._check(self._lib.xpbd_gb300_prepare_graph(self._handle, int(substeps), int(iterations)))

    def device_bytes(self) -> int:
        """Device memory held by this solver."""
        return int(self._lib.xpbd_gb300_device_bytes(self._handle))

    LAUNCH_SLOTS = ("vertex_block", "hash_block", "prim_lanes", "warp_block", "query_block", "group_lanes",
                    "group_block", "dynamic_block", "fast_ee_form", "fused_frame", "tri_lanes", "neighbor_lanes")

    def launch_config(self) -> dict:
        """Effective launch configuration (block sizes and tiles) by slot."""
        out = np.zeros(len(self.LAUNCH_SLOTS), np.int32)
        self._check(self._lib.xpbd_gb300_get_launch_config(self._handle, _ip(out), len(out)))
        return {k: int(v) for k, v in zip(self.LAUNCH_SLOTS, out)}

    def set_launch_config(self, config) -> None:
        """Set slots from a dict (missing slots unchanged) or a sequence in
        LAUNCH_SLOTS order (0 = default).  Results do not depend on it."""
        cur = self.launch_config()
        if isinstance(config, dict):
            unknown = set(config) - set(self.LAUNCH_SLOTS)
            if unknown:
                raise NativeSolverError(f"unknown launch configuration slots: {sorted(unknown)}")
            cur.update({k: int(v) for k, v in config.items()})
            vals = [cur[k] for k in self.LAUNCH_SLOTS]
        else:
            vals = [int(x) for x in config]
        arr = np.ascontiguousarray(vals, np.int32)
        self._check(self._lib.xpbd_gb300_set_launch_config(self._handle, _ip(arr), len(arr)))

    def solver_info(self) -> dict:
        out = (ctypes.c_longlong * 8)()
        self._check(self._lib.xpbd_gb300_solver_info(self._handle, out))
        keys = ("cloths", "vertices", "edges", "triangles", "fast", "strict", "dynamic", "sdf")
        return {k: int(v) for k, v in zip(keys, out)}

    def autotune(self, substeps: int, iterations: int, rounds: int = 2, cache: bool = True) -> dict:
        """Pick the launch configuration for this workload (cached per device
        and workload, see xpbd_gb300.autotune).  The solver's state is
        unchanged."""
        from . import autotune as _tune

        return _tune.tune(self, int(substeps), int(iterations), rounds=rounds, use_cache=cache)

    def _autotune_native(self, substeps: int, iterations: int, rounds: int) -> tuple:
        ms = np.zeros(2, np.float32)
        self._check(self._lib.xpbd_gb300_autotune(self._handle, int(substeps), int(iterations), int(rounds), _fp(ms)))
        return float(ms[0]), float(ms[1])

    def stream(self) -> int:
        return int(self._lib.xpbd_gb300_stream(self._handle) or 0)

    KERNEL_KINDS = ("predict", "stretch_pass", "vertex_pass", "bend_color", "vertex_hash", "triangle_hash",
                    "edge_hash", "neighbors", "vertex_vertex", "vertex_triangle", "edge_edge", "island",
                    "self_apply", "copy", "pcg", "stretch_caps", "dynamic")

    def profile_frame(self, substeps: int, iterations: int) -> dict:
        n = len(self.KERNEL_KINDS)
        ms = np.zeros(n, np.float32)
        cnt = np.zeros(n, np.int64)
        self._check(self._lib.xpbd_gb300_profile_frame(self._handle, int(substeps), int(iterations), _fp(ms),
                                                        cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), n))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_KINDS)}

    def profile_counters(self) -> dict:
        """Work counters of the last profile_frame: EE / VT query items and
        bucket slots evaluated, entries of the last triangle / edge hash
        build, primitives hashed per build, the bucket counts and the EE
        candidate gathers (visited slots whose candidate id is above the
        query edge's)."""
        out = np.zeros(11, np.int64)
        self._check(self._lib.xpbd_gb300_profile_counters(self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        keys = ("ee_items", "ee_slots", "vt_items", "vt_slots", "tri_entries", "edge_entries", "tri_hashed", "edge_hashed",
                "tri_buckets", "edge_buckets", "ee_gathers")
        return {k: int(v) for k, v in zip(keys, out)}


class NativeXpbdBatch(NativeXpbdSolver):
    """Many independent cloths in one solver, stepped together: one launch
    sequence (one CUDA graph per frame) covers every cloth.  Each cloth's
    result is the same as when it runs alone.  ABI41 calls on the handle
    address all cloths (positions concatenated in cloth order); the per-cloth
    methods address one."""

    def __init__(self, items, key_division: str | None = None):
        """`items`: sequence of (ClothData, SolverOptions, static_triangles)."""
        self._lib = _load_library()
        items = list(items)
        if not items:
            raise NativeSolverError("A batch needs at least one cloth.")
        n = len(items)
        cfgs = (NativeConfig * n)()
        meshes = (NativeMesh * n)()
        keep = []
        for k, (cloth, options, static) in enumerate(items):
            cfgs[k] = config_from_options(cloth, options, static)
            meshes[k], kk = mesh_arrays(cloth, static)
            keep.append(kk)
        self._handle = self._lib.xpbd_gb300_batch_create(cfgs, meshes, n)
        del keep
        if not self._handle:
            raise NativeSolverError(_last_error(self._lib))
        self._cloth_count = n
        self._ranges = np.zeros((n, 4), np.int32)
        for k in range(n):
            self._check(self._lib.xpbd_gb300_batch_cloth_range(self._handle, k, _ip(self._ranges[k])))
        self._vertex_count = int(self._ranges[:, 1].sum())
        self._positions_out = np.empty((self._vertex_count, 3), np.float32)
        self._static_triangle_count = max(len(it[2]) for it in items)
        if key_division is not None:
            self.set_key_division(key_division)
        for k, (cloth, _, _) in enumerate(items):
            if len(cloth.pin_indices) > 0:
                self.update_cloth_pin_targets(k, cloth.pin_indices, cloth.pin_targets_world, cloth.pin_weights)

    @property
    def cloth_count(self) -> int:
        return self._cloth_count

    def cloth_vertices(self, cloth: int) -> tuple[int, int]:
        """(first vertex, vertex count) of a cloth in the concatenated arrays."""
        return int(self._ranges[cloth, 0]), int(self._ranges[cloth, 1])

    def update_cloth_pin_targets(self, cloth: int, indices, positions, weights=None) -> None:
        idx = np.ascontiguousarray(indices, np.int32)
        pos = np.ascontiguousarray(positions, np.float32)
        w = np.ones(len(idx), np.float32) if weights is None else np.ascontiguousarray(weights, np.float32).reshape(-1)
        if len(idx) != len(pos) or len(idx) != len(w):
            raise NativeSolverError("Pin index, target, and weight arrays must have matching lengths.")
        self._check(self._lib.xpbd_gb300_batch_update_pin_targets(self._handle, int(cloth), _ip(idx), _fp(pos), _fp(w), len(idx)))

    def update_cloth_colliders(self, cloth: int, options: SolverOptions) -> None:
        c = colliders_from_options(options)
        self._check(self._lib.xpbd_gb300_batch_update_runtime_colliders(self._handle, int(cloth), ctypes.byref(c)))

    def update_cloth_static_triangles(self, cloth: int, static_triangles: np.ndarray) -> None:
        t = np.ascontiguousarray(np.asarray(static_triangles, np.float32).reshape(-1, 3))
        self._check(self._lib.xpbd_gb300_batch_update_static_triangles(self._handle, int(cloth), _fp(t), len(t) // 3))

    def update_cloth_positions(self, cloth: int, positions: np.ndarray) -> None:
        p = np.ascontiguousarray(positions, np.float32)
        self._check(self._lib.xpbd_gb300_batch_update_positions(self._handle, int(cloth), _fp(p), p.size))

    def download_cloth_positions(self, cloth: int) -> np.ndarray:
        n = int(self._ranges[cloth, 1])
        out = np.empty((n, 3), np.float32)
        self._check(self._lib.xpbd_gb300_batch_download_positions(self._handle, int(cloth), _fp(out), out.size))
        return out

    def update_cloth_force_fields(self, cloth: int, fields, unsupported: int = 0) -> None:
        arr = (NativeForceField * max(len(fields), 1))(*fields)
        fi = NativeFrameInputs()
        fi.update_force_fields = 1
        fi.force_fields = ctypes.cast(arr, ctypes.POINTER(NativeForceField)) if len(fields) else None
        fi.force_field_count = len(fields)
        fi.unsupported_force_field_count = int(unsupported)
        self._check(self._lib.xpbd_gb300_batch_update_frame_inputs(self._handle, int(cloth), ctypes.byref(fi)))

    def update_cloth_dynamic_colliders(self, cloth: int, *, triangles=None, indexed=None, particles=None) -> None:
        """update_dynamic_colliders for one cloth of the batch."""
        fi, keep = _dynamic_frame_inputs(triangles, indexed, particles)
        self._check(self._lib.xpbd_gb300_batch_update_frame_inputs(self._handle, int(cloth), ctypes.byref(fi)))
        del keep

    def attach_cloth_global_scene(self, cloth: int, scene: "GlobalDynamicScene", target_source_id: int = 0,
                                  target_collision_layer: int = 0, mode: int = 1) -> None:
        self._check(self._lib.xpbd_gb300_batch_attach_global_dynamic_scene(
            self._handle, int(cloth), scene.handle, int(target_source_id), int(target_collision_layer), int(mode)))
        self._scene_ref = scene

    def clear_cloth_global_scene(self, cloth: int) -> None:
        self._check(self._lib.xpbd_gb300_batch_clear_global_dynamic_scene(self._handle, int(cloth)))

    def reset_cloth(self, cloth: int) -> None:
        self._check(self._lib.xpbd_gb300_batch_reset_cloth(self._handle, int(cloth)))

    def set_cloth_active(self, cloth: int, active: bool) -> None:
        self._check(self._lib.xpbd_gb300_batch_set_active(self._handle, int(cloth), 1 if active else 0))

    def cloth_range(self, cloth: int) -> tuple:
        """(first vertex, vertices, first edge, edges) of a cloth in the
        concatenation used by whole-handle transfers (the caller's order)."""
        return tuple(int(x) for x in self._ranges[cloth])

    def split_positions(self, positions: np.ndarray) -> list[np.ndarray]:
        """Per-cloth views of concatenated positions."""
        return [positions[s:s + n] for s, n in ((int(r[0]), int(r[1])) for r in self._ranges)]
