/*
 * Entry points of the GB300 XPBD library beyond the ABI41 set.  None of them
 * exists in the reference; they expose what the parity tests, the batched
 * form and the benchmark need.  Same conventions as ssbl_xpbd_cuda.h:
 * 1 = success, 0 = failure with ssbl_last_error() set.
 */
#pragma once

#include "ssbl_xpbd_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Internal buffers readable with xpbd_gb300_read_buffer. */
enum {
    XPBD_BUF_POSITIONS4 = 0,     /* float4 x V (xyz, effective inverse mass) */
    XPBD_BUF_PREV4 = 1,          /* float4 x V */
    XPBD_BUF_VEL4 = 2,           /* float4 x V */
    XPBD_BUF_VERTEX_CELLS = 3,   /* int4 x V: cell x, y, z, bucket */
    XPBD_BUF_VERTEX_BUCKET_START = 4, /* int x (vertex buckets + 1) */
    XPBD_BUF_VERTEX_BUCKET_ENTRIES = 5, /* int x V */
    XPBD_BUF_TRI_BUCKET_START = 6,     /* int x (triangle buckets + 1) */
    XPBD_BUF_TRI_BUCKET_ENTRIES = 7,   /* int x total entries */
    XPBD_BUF_EDGE_BUCKET_START = 8,
    XPBD_BUF_EDGE_BUCKET_ENTRIES = 9,
    XPBD_BUF_NEIGHBOR_COUNTS = 10,     /* int x V */
    XPBD_BUF_NEIGHBOR_INDICES = 11,    /* int x V x 32 */
    XPBD_BUF_STATIC_SDF = 12,          /* float x voxels */
    XPBD_BUF_COUNTERS = 13             /* uint64 x 38 */
};

/* Build the self-collision hashes and the vertex-vertex neighbour table from
 * the current positions without stepping (for integer parity checks). */
__attribute__((visibility("default"))) int xpbd_gb300_build_self_structures(void* handle);

/* Copy an internal buffer to host memory.  Returns the number of bytes
 * written, or -1 with ssbl_last_error() set. */
__attribute__((visibility("default"))) long long xpbd_gb300_read_buffer(void* handle, int buffer_id, void* out, long long max_bytes);

/* Sizes of the hash tables: out[0..2] = vertex / triangle / edge bucket
 * counts, out[3..5] = 1 when that hash is used (else brute force). */
__attribute__((visibility("default"))) int xpbd_gb300_hash_info(void* handle, int* out6);

/* Division of the spatial-hash cell keys, floor(x / cell) (no counterpart in
 * the reference; its keys are compiled with --use_fast_math, abi41.cu:654-656,
 * native/CMakeLists.txt:109).  mode 0 (the default): the reference's
 * approximate, flush-to-zero division, so cells, bucket ids and bucket
 * contents are the reference's integers; mode 1: the correctly rounded IEEE
 * quotient, which the CPU oracle reproduces bit for bit.  The two differ only
 * for quotients within a few ulp of an integer.  set_key_division applies to
 * one solver or batch (dynamic colliders uploaded afterwards);
 * set_default_key_division to the solvers and global dynamic scenes created
 * afterwards in this process. */
__attribute__((visibility("default"))) int xpbd_gb300_set_key_division(void* handle, int mode);
__attribute__((visibility("default"))) int xpbd_gb300_set_default_key_division(int mode);

/* Capture each frame's launch sequence as a CUDA graph (default 1). */
__attribute__((visibility("default"))) int xpbd_gb300_set_graph_capture(void* handle, int enabled);

/* Number of kernel launches (graph nodes count individually) issued by the
 * last ssbl_step_solver_ex call. */
__attribute__((visibility("default"))) long long xpbd_gb300_last_step_launches(void* handle);

/* The CUDA stream (cudaStream_t) all of the solver's work is issued on. */
__attribute__((visibility("default"))) void* xpbd_gb300_stream(void* handle);

/* Run one frame without graph capture, timing every launch with CUDA events
 * on the solver's stream; per kernel kind (17 kinds: predict, stretch pass,
 * other vertex pass, bend colour, vertex / triangle / edge hash, neighbour
 * table, VV, VT, EE, island, self apply, copy, CG solve, stretch caps,
 * dynamic colliders) write the summed milliseconds and the launch count
 * (kinds >= 17).  Advances the simulation by that frame. */
__attribute__((visibility("default"))) int xpbd_gb300_profile_frame(void* handle, int substeps, int iterations,
                                                                     float* kernel_ms, long long* kernel_launches, int kinds);

/* Shared dynamic scene for one cloth of a batch (ssbl_attach_global_dynamic_scene
 * attaches every cloth of a handle): the cloth's unsigned dynamic-collider
 * stage reads the scene's colliders except those of `target_source_id` (and,
 * with mode 2, those of layers not below `target_collision_layer`); mode 0
 * keeps it on its own colliders.  clear detaches the cloth. */
__attribute__((visibility("default"))) int xpbd_gb300_batch_attach_global_dynamic_scene(void* handle, int cloth, void* scene,
                                                                                        int target_source_id,
                                                                                        int target_collision_layer,
                                                                                        int collision_mode);
__attribute__((visibility("default"))) int xpbd_gb300_batch_clear_global_dynamic_scene(void* handle, int cloth);

/* PC2 point-cache writer (the reference's bake / realtime cache format,
 * session_manager.py:4624-4733): open for one cloth of a solver or batch
 * (cloth -1: every vertex of the handle in stored order), then one sample per
 * call from the cloth's current positions in object-local coordinates
 * (matrix_world_inv16: row-major 4x4, null = identity).  The transform runs
 * on the solver's stream, the copy to pinned memory on a side stream and the
 * file write on a writer thread, so stepping continues while samples drain.
 * close(commit = 1) writes the final header and renames the temporary file
 * into place; it returns the sample count or -1. */
__attribute__((visibility("default"))) void* xpbd_gb300_pc2_open(void* handle, int cloth, const char* path, int start_frame);
__attribute__((visibility("default"))) int xpbd_gb300_pc2_write(void* handle, void* writer, const float* matrix_world_inv16);
__attribute__((visibility("default"))) long long xpbd_gb300_pc2_close(void* writer, int commit);

/* Launch configuration (no counterpart in the reference): 12 slots, in order
 * block size of the per-vertex passes (default 128), of the hash count /
 * scatter kernels (256), lanes per primitive of the edge hash (1, 2, 4, 8
 * or 16; default 8), block size of the warp-per-item kernels (256), of
 * the thread-per-item queries (256), lanes per item of the strict group
 * queries (4, 8 or 16; default 8), block size of the group queries (256), of
 * the dynamic-collider pass (128), the form of the fast-mode edge-edge query
 * (8: groups of 8 lanes, 32: flattened warps; default 32), and whether
 * solvers whose cloths all fit one block (at most 1024 vertices, no self
 * collision, hard stretch or dynamic colliders) run each frame as one fused
 * launch, a block per cloth (1, default) or an 8-CTA thread-block cluster per
 * cloth exchanging through distributed shared memory (8), or as launched
 * kernels (2), lanes per primitive of the triangle hash (1, 2, 4, 8 or 16;
 * default 8), and lanes per vertex of the neighbour table and strict VV
 * responses (1, 2, 4, 8, 16 or 32; default 2).  Block sizes
 * are multiples of 32 up to 256; 0 selects the default.  No value changes a
 * result.  Setting drops the captured frame graphs. */
__attribute__((visibility("default"))) int xpbd_gb300_set_launch_config(void* handle, const int* values, int count);
__attribute__((visibility("default"))) int xpbd_gb300_get_launch_config(void* handle, int* out, int count);

/* Workload summary: out8 = cloths, vertices, edges, triangles, cloths with
 * fast self collision, with strict self collision, with dynamic colliders,
 * with a static SDF (the autotuner cache keys on it). */
__attribute__((visibility("default"))) int xpbd_gb300_solver_info(void* handle, long long* out8);

/* Autotuner: from the current state, time profiled frames (the fastest of
 * `rounds` per candidate, state restored before each) for each candidate of
 * each slot in turn, keep the fastest configuration and restore the state.
 * ms_out2 = {tuned frame ms, default frame ms} (summed kernel times). */
__attribute__((visibility("default"))) int xpbd_gb300_autotune(void* handle, int substeps, int iterations, int rounds,
                                                               float* ms_out2);

/* Work counters of the last xpbd_gb300_profile_frame, out[11]: EE query
 * items, EE bucket slots visited, VT query items (strict cloths), VT slots
 * evaluated; entries written by the frame's last triangle-hash build and
 * last edge-hash build; triangles and edges hashed per build; triangle and
 * edge bucket counts; EE candidate gathers (visited slots whose candidate's
 * id is above the query edge's, the pairs whose rows are read).  They size
 * the algorithmic bytes of the query kernels and of the hash builds. */
__attribute__((visibility("default"))) int xpbd_gb300_profile_counters(void* handle, long long* out);

/* No counterpart in the reference.  Vertex spatial hash that allocates no
 * device memory, for callers that cannot call cudaMalloc / cudaFree (a host
 * application whose pool owns all device memory, or a frame loop that cannot
 * absorb the device synchronisation those calls may cause).  Inputs and
 * outputs are the caller's device arrays: positions (x y z per vertex),
 * bucket_start (bucket_count + 1 ints), bucket_entries (vertex_count ints),
 * cells (4 ints per vertex, written as int4: 16-byte aligned; may be NULL).
 * bucket_count must be a power of two of at most 262144: the bucket counters
 * live in a fixed 1 MiB array inside the library, one per device, kept until
 * the process exits and shared by every call, so calls that overlap on the
 * GPU race.  Each call looks up that array's address in the current context;
 * the first call on a device also loads the library's device code, so make
 * it before any stream capture.  Buckets are ordered by a thread each, or by
 * a warp when one holds more than 32 members.  Work is queued on `stream`
 * (cudaStream_t, NULL = default).  Returns 1, or 0 with ssbl_last_error()
 * set. */
__attribute__((visibility("default"))) int xpbd_gb300_vertex_hash_noalloc(const float* positions, int vertex_count,
                                                                           float cell_size, int bucket_count,
                                                                           int* bucket_start, int* bucket_entries,
                                                                           int* cells, void* stream);

/* ---- Batched form (no counterpart in the reference) ----------------------
 * One solver for `cloth_count` independent cloths, stepped together by
 * ssbl_step_solver_ex: every launch of a frame covers all cloths and the
 * frame is captured as one CUDA graph.  configs[k] / meshes[k] have the
 * meaning of ssbl_create_solver's arguments (abi41.cu:8791); each cloth keeps
 * its own parameters, pins, colliders and static SDF, and its results are
 * the same bits as when it runs alone.  Hard stretch optimisation (the CG
 * path) is accepted only for cloth_count == 1.  The handle is accepted by
 * every ABI41 entry point, which then addresses all cloths: positions are
 * concatenated in cloth order, pin indices run over the concatenated
 * vertices, colliders and static triangles apply to every cloth, and the
 * diagnostics are sums over the cloths.  Destroy with ssbl_destroy_solver. */
__attribute__((visibility("default"))) void* xpbd_gb300_batch_create(const SsblXpbdConfig* configs,
                                                                      const SsblXpbdMesh* meshes, int cloth_count);
__attribute__((visibility("default"))) int xpbd_gb300_batch_cloth_count(void* handle);
/* out4 = first vertex, vertex count, first edge, edge count of the cloth. */
__attribute__((visibility("default"))) int xpbd_gb300_batch_cloth_range(void* handle, int cloth, int* out4);
/* Per-cloth forms of ssbl_update_pin_targets (indices local to the cloth),
 * ssbl_update_runtime_colliders, ssbl_update_static_triangles,
 * ssbl_update_frame_inputs, ssbl_update_positions, ssbl_download_positions
 * and ssbl_reset_solver. */
__attribute__((visibility("default"))) int xpbd_gb300_batch_update_pin_targets(void* handle, int cloth, const int* indices,
                                                                                const float* positions, const float* weights,
                                                                                int count);
__attribute__((visibility("default"))) int xpbd_gb300_batch_update_runtime_colliders(void* handle, int cloth,
                                                                                      const SsblXpbdRuntimeColliders* colliders);
__attribute__((visibility("default"))) int xpbd_gb300_batch_update_static_triangles(void* handle, int cloth,
                                                                                     const float* triangles, int triangle_count);
__attribute__((visibility("default"))) int xpbd_gb300_batch_update_frame_inputs(void* handle, int cloth,
                                                                                 const SsblXpbdFrameInputs* inputs);
__attribute__((visibility("default"))) int xpbd_gb300_batch_update_positions(void* handle, int cloth, const float* positions,
                                                                              int max_floats);
__attribute__((visibility("default"))) int xpbd_gb300_batch_download_positions(void* handle, int cloth, float* out,
                                                                                int max_floats);
__attribute__((visibility("default"))) int xpbd_gb300_batch_reset_cloth(void* handle, int cloth);
/* An inactive cloth is skipped by every kernel (its state stays as it is)
 * until it is activated again. */
__attribute__((visibility("default"))) int xpbd_gb300_batch_set_active(void* handle, int cloth, int active);

/* Capture and instantiate the frame graph for (substeps, iterations) and the
 * current collider kinds without running a frame, so the first step does
 * not pay for the capture (the serving loop prepares new solvers off the
 * stepping thread). */
__attribute__((visibility("default"))) int xpbd_gb300_prepare_graph(void* handle, int substeps, int iterations);

/* Device memory held by the solver (bytes of all its allocations), for
 * admission by a device-memory budget. */
__attribute__((visibility("default"))) long long xpbd_gb300_device_bytes(void* handle);

/* ---- Differentiable form (no counterpart in the reference) ---------------
 * A contact-free cloth (stretch and bend constraints, hard pins; no
 * colliders, self collision, tethers or hard-stretch path) rolled out from
 * its rest state with one compliance per edge and per bend, and the adjoint
 * of that rollout.  Array arguments of rollout / backward are DEVICE
 * pointers (float32): compliances of E and B values, positions and their
 * gradient of 3V values.  The rollout keeps every frame's starting state;
 * backward re-runs one frame at a time from those checkpoints. */
__attribute__((visibility("default"))) void* xpbd_gb300_diff_create(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh);
__attribute__((visibility("default"))) int xpbd_gb300_diff_destroy(void* handle);
/* Hard pins only (weight >= 0.75); softer pins are refused. */
__attribute__((visibility("default"))) int xpbd_gb300_diff_update_pin_targets(void* handle, const int* indices,
                                                                               const float* positions, const float* weights,
                                                                               int count);
__attribute__((visibility("default"))) int xpbd_gb300_diff_rollout(void* handle, const float* stretch_compliance,
                                                                    const float* bend_compliance, int frames, int substeps,
                                                                    int iterations, float* final_positions);
/* dL/d(compliance) of the last rollout for dL/d(final positions). */
__attribute__((visibility("default"))) int xpbd_gb300_diff_backward(void* handle, const float* grad_positions,
                                                                     float* grad_stretch, float* grad_bend);
__attribute__((visibility("default"))) void* xpbd_gb300_diff_stream(void* handle);
/* State at the start of frame `frame` of the last rollout (frame = frames:
 * the final state) as 3 x V float4 rows (positions, previous positions,
 * velocities; device array of 12 V floats), so a caller can evaluate other
 * derivatives along the rollout's own trajectory. */
__attribute__((visibility("default"))) int xpbd_gb300_diff_checkpoint(void* handle, int frame, float* out_rows);

/* Host-side input preprocessing of the cloth builders (no device work):
 * greedy first-fit colouring of constraint pairs in order (writes a colour
 * per pair, returns the colour count or -1) and the bend pairs of a triangle
 * mesh in increasing order (returns their count or -1). */
__attribute__((visibility("default"))) int xpbd_gb300_greedy_color(const int* pairs, int count, int vertex_count, int* colors);
__attribute__((visibility("default"))) int xpbd_gb300_bend_pairs(const int* triangles, int triangle_count, int* pairs,
                                                                  int max_pairs);
/* Device input preprocessing (replaces the per-element steps of the add-on's
 * cloth builder, xpbd_core.py:715-747 and 862-881): from rest positions
 * (V x 3), triangles (T x 3, indices in [0, V)), the area density factor
 * max(density, eps) and the hard-pin mask (V bytes, may be null), writes the
 * distinct triangle sides as (lower, upper) pairs in lexicographic order with
 * rest lengths max(|x_b - x_a|, eps) (room for 3T pairs), the inverse masses
 * (float64 area sums; 0 for hard pins) and, when `bends` is not null, the
 * bend pairs of xpbd_gb300_bend_pairs with their rest lengths (room for 3T;
 * count in *bend_count).  Returns the edge count, or -1 with
 * ssbl_last_error() set (an index outside the vertices included). */
__attribute__((visibility("default"))) int xpbd_gb300_prepare_cloth_device(const float* positions, int vertex_count,
                                                                            const int* triangles, int triangle_count,
                                                                            float density, float eps,
                                                                            const unsigned char* hard, int* edges,
                                                                            float* edge_rest, float* inv_mass, int* bends,
                                                                            float* bend_rest, int* bend_count);

/* Wait for the solver's stream. */
__attribute__((visibility("default"))) int xpbd_gb300_synchronize(void* handle);

#ifdef __cplusplus
}
#endif
