/*
 * ABI41 C interface of the GB300 XPBD cloth solver.
 *
 * This header declares the 20 entry points and the 6 structs that the
 * reference's ctypes bridge binds (native_backend.py:21-250 mirrors the
 * structs, native_backend.py:535-627 binds the functions).  The struct
 * layouts are part of the binary contract: field order, types and sizes
 * must stay identical to the reference header
 * (native/include/ssbl_xpbd_cuda.h:13-312), so that the unchanged bridge
 * can load this library through SSBL_NATIVE_DLL_PATH.  The sizes are
 * checked by static_asserts in the implementation (224 / 992 / 240 / 132
 * bytes for config / diagnostics / frame inputs / force field on LP64).
 *
 * Conventions shared by every entry point (reference
 * native/src/ssbl_xpbd_cuda_abi41.cu:228, 562-573, 9094-9098):
 *   - return 1 on success and 0 on failure; create returns NULL on failure;
 *   - the failure message is read with ssbl_last_error(); every entry point
 *     clears it first;
 *   - every input pointer is borrowed for the duration of the call only;
 *   - a handle is not safe to use from two threads at once.
 */
#pragma once

#ifdef _WIN32
#define SSBL_API __declspec(dllexport)
#else
#define SSBL_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Solver configuration (reference native/include/ssbl_xpbd_cuda.h:13-62). */
typedef struct SsblXpbdConfig {
    int vertex_count;
    int edge_count;
    int bend_count;
    int lra_count;
    int triangle_count;
    int static_triangle_count;
    int edge_color_count;
    int bend_color_count;
    int lra_color_count;
    float dt;
    float damping;                 /* per-substep velocity multiplier in [0, 1] */
    float gravity[3];              /* Z-up world */
    float stretch_compliance;
    float bend_compliance;
    float lra_compliance;
    float collision_margin;
    int use_ground;
    float ground_height;           /* ground plane is z = ground_height */
    int use_wall;
    float wall_origin[3];
    float wall_normal[3];
    int use_sphere;
    float sphere_center[3];
    float sphere_radius;
    int self_collision;
    int self_collision_mode;       /* 1 = fast (cluster filter), 2 = strict */
    float cloth_thickness;
    float self_collision_distance;
    int self_collision_interval;
    int max_self_collision_neighbors;
    int use_volume_pressure;
    float rest_volume;
    float volume_compliance;
    float pressure_strength;
    float volume_target_scale;
    int volume_solve_interval;
    int self_probe_interval;
    int self_surface_pair_interval;
    int jitter_stabilizer_enabled;
    float contact_friction;
    float contact_tangent_damping;
    float contact_compliance;
    int fast_self_collision_passes;
    int stretch_optimization_enabled;
    float stretch_optimization_strength;
    float static_sdf_voxel_size;
    int static_sdf_band_voxels;
    int static_sdf_max_resolution;
} SsblXpbdConfig;

/* Capability bits returned by ssbl_capabilities (reference abi.h:64-68). */
enum {
    SSBL_CAP_STRETCH_OPTIMIZATION = 1u << 0,
    SSBL_CAP_PIN_WEIGHTS = 1u << 1,
    SSBL_CAP_GLOBAL_DYNAMIC_SCENE = 1u << 2
};

/* Per-step diagnostics (reference native/include/ssbl_xpbd_cuda.h:70-207). */
typedef struct SsblXpbdDiagnostics {
    float step_ms;
    float hash_build_ms;
    float constraints_ms;
    float volume_ms;
    float analytic_collision_ms;
    float static_collision_ms;
    float dynamic_collision_ms;
    float dynamic_particle_collision_ms;
    float self_hash_ms;
    float self_solve_ms;
    float self_probe_ms;
    float self_recovery_ms;
    float sync_ms;
    float diagnostics_fetch_ms;
    long long candidate_count;
    long long resolved_contacts;
    float min_gap;
    long long ccd_clamp_count;
    long long recovery_passes;
    long long local_retry_count;
    long long jitter_stabilized_vertices;
    long long jitter_rejected_vertices;
    float jitter_max_correction;
    long long external_contact_cache_hits;
    long long external_contact_cache_misses;
    long long external_contact_cache_count;
    long long external_contact_cache_overflow;
    long long external_friction_corrections;
    long long force_field_count;
    long long unsupported_force_field_count;
    long long dynamic_particle_count;
    long long dynamic_particle_candidate_count;
    long long dynamic_particle_contacts;
    long long dynamic_particle_overflow;
    long long dynamic_triangle_count;
    long long static_triangle_count;
    int finite_flag;
    long long fast_exact_vt_candidates;
    long long fast_exact_vt_projected;
    long long fast_exact_vt_guarded;
    long long fast_exact_vt_skipped_rest;
    long long fast_soft_repulsion_candidates;
    long long fast_soft_repulsion_applied;
    float fast_soft_repulsion_max_push;
    long long fast_hard_projection_count;
    long long fast_manifold_contacts;
    long long fast_manifold_reused;
    long long fast_barrier_projected;
    long long fast_barrier_smoothed_vertices;
    long long fast_barrier_overflow;
    float fast_barrier_max_delta;
    long long fast_edge_edge_candidates;
    long long fast_edge_edge_contacts;
    long long fast_triangle_pair_candidates;
    long long fast_triangle_pair_contacts;
    long long fast_triangle_pair_skipped_rest;
    long long fast_contact_classification_guarded;
    long long fast_region_cluster_candidates;
    long long fast_region_cluster_contacts;
    long long fast_region_cluster_guarded;
    long long fast_overlap_island_candidates;
    long long fast_overlap_island_clusters;
    long long fast_overlap_island_vertex_refs;
    long long fast_overlap_island_applied_vertices;
    long long fast_overlap_island_guarded;
    float fast_overlap_island_max_delta;
    long long fast_cc_overlap_components;
    long long fast_cc_overlap_seed_triangles;
    long long fast_cc_overlap_owned_vertices;
    long long fast_cc_overlap_union_edges;
    long long fast_cc_overlap_guarded;
    long long fast_cc_overlap_applied_vertices;
    float fast_cc_overlap_max_delta;
    long long abi41_soft_contact_count;
    long long abi41_exact_impulse_contact_count;
    long long abi41_edge_edge_contact_count;
    float abi41_max_smoothed_delta;
    long long abi41_hard_projection_fallbacks;
    long long static_sdf_rebuild_count;
    long long static_sdf_voxel_count;
    long long static_sdf_grid_x;
    long long static_sdf_grid_y;
    long long static_sdf_grid_z;
    float static_sdf_build_ms;
    long long static_sdf_contact_count;
    long long static_sdf_unsigned_fallback_count;
    long long abi41_pcg_iterations;
    long long abi41_pcg_guarded;
    long long abi41_pcg_csr_nnz;
    long long abi41_pcg_texture_ready;
    float abi41_pcg_initial_residual;
    float abi41_pcg_final_residual;
    float abi41_pcg_max_delta;
    long long abi41_lra_tack_count;
    long long abi41_bending_wing_count;
    long long abi41_bending_texture_ready;
    long long abi41_tack_jitter_guarded;
    long long abi41_bending_guarded;
    float dynamic_collider_pack_ms;
    float dynamic_triangle_upload_ms;
    float dynamic_particle_upload_ms;
    long long dynamic_collider_cache_hits;
    long long dynamic_collider_cache_misses;
    float abi41_pcg_solve_ms;
    float abi41_pcg_system_ms;
    float abi41_pcg_ad_ms;
    float abi41_direct_stretch_ms;
    long long dynamic_pair_cache_hits;
    long long dynamic_pair_cache_misses;
    long long dynamic_pair_cache_reused_triangles;
    long long dynamic_pair_cache_reused_particles;
    long long dynamic_collision_skipped_launches;
    long long self_collision_skipped_launches;
    long long self_candidate_count;
    long long self_filter_seen;
    long long self_filter_accepted_vv;
    long long self_filter_accepted_vt;
    long long self_filter_accepted_ee;
    long long self_filter_rejected_rest;
    long long self_filter_rejected_duplicate;
    long long self_filter_rejected_ownership;
    long long self_filter_cache_hits;
    long long self_filter_cache_misses;
    long long self_cluster_count;
    long long self_cluster_owned_contacts;
    long long dynamic_triangle_candidate_count;
    long long dynamic_triangle_bucket_overflow;
    long long dynamic_triangle_large_primitive_count;
    long long dynamic_triangle_aabb_reject_count;
    long long dynamic_triangle_max_bucket_occupancy;
    float global_dynamic_scene_pack_ms;
    float global_dynamic_scene_upload_ms;
    float global_dynamic_hash_ms;
    long long global_dynamic_particle_count;
    long long global_dynamic_triangle_count;
    long long global_dynamic_hash_overflow;
} SsblXpbdDiagnostics;

/* Mesh arrays copied at create (reference abi.h:209-223). */
typedef struct SsblXpbdMesh {
    const float* positions;          /* V x 3, world space, also the rest pose */
    const float* inv_mass;           /* V; <= 0 marks a pinned / kinematic vertex */
    const int* edges;                /* E x 2 */
    const float* edge_rest_lengths;  /* E */
    const int* edge_color_offsets;   /* edge_color_count + 1 */
    const int* bends;                /* B x 2, wing-opposite vertex pairs */
    const float* bend_rest_lengths;  /* B */
    const int* bend_color_offsets;   /* bend_color_count + 1 */
    const int* lra_edges;            /* L x 2, (anchor, dynamic) */
    const float* lra_rest_lengths;   /* L */
    const int* lra_color_offsets;    /* lra_color_count + 1 */
    const int* triangles;            /* T x 3 */
    const float* static_triangles;   /* S x 9 */
} SsblXpbdMesh;

/* Analytic colliders (reference abi.h:225-234). */
typedef struct SsblXpbdRuntimeColliders {
    int use_ground;
    float ground_height;
    int use_wall;
    float wall_origin[3];
    float wall_normal[3];
    int use_sphere;
    float sphere_center[3];
    float sphere_radius;
} SsblXpbdRuntimeColliders;

/* Force-field record (reference abi.h:236-264). */
typedef struct SsblXpbdForceField {
    int type;
    int use_min_distance;
    int use_max_distance;
    int seed;
    float strength;
    float origin[3];
    float direction[3];
    float axis[3];
    float falloff_power;
    float distance_min;
    float distance_max;
    float radial_min;
    float radial_max;
    float noise;
    float linear_drag;
    float quadratic_drag;
    float harmonic_damping;
    float flow;
    float size;
    float rest_length;
    float radial_falloff;
    float texture_nabla;
    int use_radial_min;
    int use_radial_max;
    int use_2d_force;
    int use_global_coords;
    int apply_to_location;
} SsblXpbdForceField;

/* Per-frame inputs (reference abi.h:266-297). */
typedef struct SsblXpbdFrameInputs {
    int update_pin_targets;
    const int* pin_indices;
    const float* pin_positions;
    const float* pin_weights;
    int pin_count;
    int update_runtime_colliders;
    SsblXpbdRuntimeColliders runtime_colliders;
    int update_static_triangles;
    const float* static_triangles;
    int static_triangle_count;
    int update_dynamic_triangles;
    const float* dynamic_triangles;
    int dynamic_triangle_count;
    int update_dynamic_indexed_triangles;
    const float* dynamic_triangle_vertices;
    int dynamic_triangle_vertex_count;
    const int* dynamic_triangle_indices;
    int dynamic_indexed_triangle_count;
    int dynamic_triangle_topology_changed;
    int update_dynamic_particles;
    const float* dynamic_particle_positions;
    const float* dynamic_particle_radii;
    const float* dynamic_particle_inv_mass;
    const int* dynamic_particle_slot_ids;
    const int* dynamic_particle_phases;
    int dynamic_particle_count;
    int update_force_fields;
    const SsblXpbdForceField* force_fields;
    int force_field_count;
    int unsupported_force_field_count;
} SsblXpbdFrameInputs;

/* Shared cross-cloth collider scene (reference abi.h:299-312). */
typedef struct SsblXpbdGlobalDynamicSceneInputs {
    const float* particle_positions;
    const float* particle_prev_positions;
    const float* particle_radii;
    const int* particle_source_ids;
    const int* particle_collision_layers;
    int particle_count;
    const float* triangle_vertices;
    const int* triangle_source_ids;
    const int* triangle_collision_layers;
    int triangle_count;
    float collision_margin;
    float cloth_thickness;
} SsblXpbdGlobalDynamicSceneInputs;

/* Create a solver; copies every mesh array to the GPU and builds the static
 * SDF when static triangles are given.  Replaces abi41.cu:8791. */
SSBL_API void* ssbl_create_solver(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh);
/* Free a solver and all its device memory.  Replaces abi41.cu:8969. */
SSBL_API int ssbl_destroy_solver(void* handle);
/* pos = prev = rest, vel = 0.  Replaces abi41.cu:8975. */
SSBL_API int ssbl_reset_solver(void* handle);
/* Replace the pin set; weights may be NULL (all 1.0).  Replaces abi41.cu:8992. */
SSBL_API int ssbl_update_pin_targets(void* handle, const int* indices, const float* positions, const float* weights, int count);
/* Replace ground / wall / sphere.  Replaces abi41.cu:8997. */
SSBL_API int ssbl_update_runtime_colliders(void* handle, const SsblXpbdRuntimeColliders* inputs);
/* Set pos and prev (not vel).  Replaces abi41.cu:9007. */
SSBL_API int ssbl_update_positions(void* handle, const float* positions, int max_floats);
/* Replace the static collider; rebuilds the SDF.  Replaces abi41.cu:9021. */
SSBL_API int ssbl_update_static_triangles(void* handle, const float* triangles, int triangle_count);
/* Replace the dynamic triangle soup.  Replaces abi41.cu:9026. */
SSBL_API int ssbl_update_dynamic_triangles(void* handle, const float* triangles, int triangle_count);
/* Apply a batch of per-frame inputs.  Replaces abi41.cu:9035. */
SSBL_API int ssbl_update_frame_inputs(void* handle, const SsblXpbdFrameInputs* inputs);
/* = ssbl_step_solver_ex(handle, substeps, iterations, 1, 1).  Replaces abi41.cu:9400. */
SSBL_API int ssbl_step_solver(void* handle, int substeps, int iterations);
/* Advance one frame of `substeps` substeps with `iterations` constraint
 * iterations each.  Synchronises when force_sync or fetch_diagnostics.
 * Replaces abi41.cu:9087. */
SSBL_API int ssbl_step_solver_ex(void* handle, int substeps, int iterations, int fetch_diagnostics, int force_sync);
/* Copy V x 3 positions to the caller's buffer.  Replaces abi41.cu:9404. */
SSBL_API int ssbl_download_positions(void* handle, float* out_positions, int max_floats);
/* Copy the last step's diagnostics.  Replaces abi41.cu:9416. */
SSBL_API int ssbl_get_diagnostics(void* handle, SsblXpbdDiagnostics* out_diag);
/* Capability bits; 7 like the reference.  Replaces abi41.cu:9426. */
SSBL_API unsigned int ssbl_capabilities(void);
/* Global dynamic scene (cross-cloth colliders).  Replace abi41.cu:8733-8789. */
SSBL_API void* ssbl_create_global_dynamic_scene(void);
SSBL_API int ssbl_destroy_global_dynamic_scene(void* scene_handle);
SSBL_API int ssbl_update_global_dynamic_scene(void* scene_handle, const SsblXpbdGlobalDynamicSceneInputs* inputs);
SSBL_API int ssbl_attach_global_dynamic_scene(void* handle, void* scene_handle, int target_source_id, int target_collision_layer, int collision_mode);
SSBL_API int ssbl_clear_global_dynamic_scene(void* handle);
/* Message of the last failure on this thread's last call.  Replaces abi41.cu:9430. */
SSBL_API const char* ssbl_last_error(void);

#ifdef __cplusplus
}
#endif
