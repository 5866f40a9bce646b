/*
 * CPU oracle of the XPBD cloth step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solver's per-substep path
 * (native/src/ssbl_xpbd_cuda_abi41.cu, devin22ldh-afk/ssbl-cuda-xpbd), used
 * by the test suite, the smoke check and the benchmark's CPU baseline as the
 * checker.  The product library never links, loads or calls it.
 *
 * Semantics restated (each function in xpbd_oracle.c cites its reference
 * lines): prediction, weighted pins, snapshot-Jacobi stretch, tethers, bends
 * by colour, ground / sphere / wall contacts with friction, the static SDF
 * (build, trilinear sampling, contact), dynamic triangle / particle
 * colliders (hashes, unsigned and signed responses), self collision (vertex / triangle /
 * edge spatial hashes, neighbour table, VV / VT / EE responses, fast-mode
 * filters and overlap islands, averaging) and the velocity update, in the
 * reference's kernel order (abi41.cu:9165-9376).
 *
 * Where the reference is nondeterministic (float atomics, atomic bucket slot
 * order) the oracle fixes one order: constraint corrections are summed per
 * vertex in constraint-index order, hash buckets list primitive ids in
 * increasing order, and self-collision pushes are summed in 2^-32 m fixed
 * point.  Compiled with -ffp-contract=off, it performs the same IEEE
 * single-precision operations as the GPU kernels.
 */
#pragma once

#include "../include/ssbl_xpbd_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleSolver OracleSolver;
typedef struct OracleScene OracleScene;

OracleSolver* oracle_create(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh);
void oracle_destroy(OracleSolver* s);
const char* oracle_last_error(void);
int oracle_update_pin_targets(OracleSolver* s, const int* indices, const float* positions, const float* weights, int count);
int oracle_update_runtime_colliders(OracleSolver* s, const SsblXpbdRuntimeColliders* c);
int oracle_update_positions(OracleSolver* s, const float* positions, int max_floats);
int oracle_update_static_triangles(OracleSolver* s, const float* triangles, int count);
/* Force fields (at most 64) applied by the prediction from the next step. */
int oracle_update_force_fields(OracleSolver* s, const SsblXpbdForceField* fields, int count);
/* Dynamic colliders, replaced on each call (count 0 clears): plain
 * triangles (9 floats each, unsigned response), an indexed closed mesh
 * (signed response) and particles with radii. */
int oracle_update_dynamic_triangles(OracleSolver* s, const float* triangles, int count);
int oracle_update_dynamic_indexed(OracleSolver* s, const float* vertices, int vertex_count, const int* indices, int count,
                                  int topology_changed);
int oracle_update_dynamic_particles(OracleSolver* s, const float* positions, const float* radii, int count);
/* Shared dynamic scene: colliders of many sources with source ids and
 * collision layers; an attached solver's unsigned dynamic stage reads it
 * through its source filter (mode 0: own colliders, 1: all but its own
 * source, 2: only lower layers). */
OracleScene* oracle_scene_create(void);
void oracle_scene_destroy(OracleScene* g);
int oracle_scene_update(OracleScene* g, const SsblXpbdGlobalDynamicSceneInputs* inputs);
int oracle_scene_attach(OracleSolver* s, OracleScene* g, int target_source_id, int target_collision_layer, int mode);
int oracle_scene_clear(OracleSolver* s);
long long oracle_scene_overflow(const OracleScene* g);
int oracle_step(OracleSolver* s, int substeps, int iterations);
int oracle_download_positions(OracleSolver* s, float* out, int max_floats);
int oracle_download_state(OracleSolver* s, float* pos3, float* prev3, float* vel3);
/* Build the self-collision hashes and the neighbour table from the current
 * positions (no step), like xpbd_gb300_build_self_structures. */
int oracle_build_self_structures(OracleSolver* s);
/* Read integer structures: which = 3 vertex cells (int4 x V), 4 vertex bucket
 * start, 5 vertex bucket entries, 6/7 triangle start/entries, 8/9 edge
 * start/entries, 10 neighbour counts, 11 neighbour indices (V x 32),
 * 12 static SDF (float), 13 counters (uint64 x 38).  Returns bytes or -1. */
long long oracle_read_buffer(OracleSolver* s, int which, void* out, long long max_bytes);
int oracle_hash_info(OracleSolver* s, int* out6);
/* Dynamic colliders: triangles, large triangles, largest bucket, triangle
 * hash built, particles, particle hash built. */
int oracle_dynamic_info(OracleSolver* s, int* out6);
/* Threads used by the parallel loops (OpenMP builds); returns the count. */
int oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
