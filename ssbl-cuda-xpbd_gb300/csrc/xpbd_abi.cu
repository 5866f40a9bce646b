// C entry points of the GB300 XPBD library: the ABI41 set, the batch entry
// points and the extensions declared in include/xpbd_gb300.h.
//
// ABI41 entry points replace native/src/ssbl_xpbd_cuda_abi41.cu:8791-9432
// with the same return convention (1 / 0, NULL on failed create) and the same
// error strings where the reference defines them.  An ABI41 handle is a
// solver of one cloth; a batch handle (xpbd_gb300_batch_create) is accepted by
// every ABI41 entry point and then addresses all of its cloths at once
// (positions concatenated in cloth order, pin indices over the concatenated
// vertices, colliders and static triangles applied to every cloth).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "xpbd_host.cuh"

static_assert(sizeof(SsblXpbdConfig) == 224, "SsblXpbdConfig layout");
static_assert(sizeof(SsblXpbdDiagnostics) == 992, "SsblXpbdDiagnostics layout");
static_assert(sizeof(SsblXpbdFrameInputs) == 240, "SsblXpbdFrameInputs layout");
static_assert(sizeof(SsblXpbdForceField) == 132, "SsblXpbdForceField layout");

using namespace xg;
using namespace xg::host;

#define XG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

Solver* as_solver(void* h) { return reinterpret_cast<Solver*>(h); }

int ok_or_zero(bool ok) { return ok ? 1 : 0; }

bool frame_inputs(Solver* S, int cloth, const SsblXpbdFrameInputs* in) {
    if (!S || !in) return fail("invalid frame input update");
    if (in->update_pin_targets && !upload_pins(S, cloth, in->pin_indices, in->pin_positions, in->pin_weights, in->pin_count))
        return false;
    if (in->update_runtime_colliders && !set_colliders(S, cloth, in->runtime_colliders)) return false;
    if (in->update_dynamic_triangles && !upload_dynamic_triangles(S, cloth, in->dynamic_triangles, in->dynamic_triangle_count))
        return false;
    if (in->update_dynamic_indexed_triangles &&
        !upload_dynamic_indexed(S, cloth, in->dynamic_triangle_vertices, in->dynamic_triangle_vertex_count,
                                in->dynamic_triangle_indices, in->dynamic_indexed_triangle_count,
                                in->dynamic_triangle_topology_changed != 0))
        return false;
    if (in->update_dynamic_particles &&
        !upload_dynamic_particles(S, cloth, in->dynamic_particle_positions, in->dynamic_particle_radii, in->dynamic_particle_count))
        return false;
    if (in->update_static_triangles && !upload_static(S, cloth, in->static_triangles, in->static_triangle_count)) return false;
    if (in->update_force_fields &&
        !upload_fields(S, cloth, in->force_fields, in->force_field_count, in->unsupported_force_field_count))
        return false;
    int ff = 0, uff = 0;
    for (const Cloth& C : S->cl) {
        ff += C.force_field_count;
        uff += C.unsupported_force_field_count;
    }
    S->diag.force_field_count = ff;
    S->diag.unsupported_force_field_count = uff;
    return true;
}

}  // namespace

// ----------------------------------------------------------- ABI41 entry points

extern "C" SSBL_API void* ssbl_create_solver(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh) {
    g_error.clear();
    if (!config || !mesh) {
        fail("invalid ABI41 solver create request");
        return nullptr;
    }
    return create_solver(config, mesh, 1);
}

extern "C" SSBL_API int ssbl_destroy_solver(void* handle) {
    g_error.clear();
    free_solver(as_solver(handle));
    return 1;
}

extern "C" SSBL_API int ssbl_reset_solver(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return ok_or_zero(reset_cloths(S, -1));
}

extern "C" SSBL_API int ssbl_update_pin_targets(void* handle, const int* indices, const float* positions, const float* weights, int count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return ok_or_zero(upload_pins(S, -1, indices, positions, weights, count));
}

extern "C" SSBL_API int ssbl_update_runtime_colliders(void* handle, const SsblXpbdRuntimeColliders* inputs) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !inputs) return fail("invalid runtime collider update") ? 1 : 0;
    return ok_or_zero(set_colliders(S, -1, *inputs));
}

extern "C" SSBL_API int ssbl_update_positions(void* handle, const float* positions, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid position upload") ? 1 : 0;
    return ok_or_zero(upload_positions(S, -1, positions, max_floats));
}

extern "C" SSBL_API int ssbl_update_static_triangles(void* handle, const float* triangles, int triangle_count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid static triangle update") ? 1 : 0;
    return ok_or_zero(upload_static(S, -1, triangles, triangle_count));
}

extern "C" SSBL_API int ssbl_update_dynamic_triangles(void* handle, const float* triangles, int triangle_count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid dynamic triangle update") ? 1 : 0;
    return ok_or_zero(upload_dynamic_triangles(S, -1, triangles, triangle_count));
}

extern "C" SSBL_API int ssbl_update_frame_inputs(void* handle, const SsblXpbdFrameInputs* in) {
    g_error.clear();
    return ok_or_zero(frame_inputs(as_solver(handle), -1, in));
}

extern "C" SSBL_API int ssbl_step_solver_ex(void* handle, int substeps, int iterations, int fetch_diagnostics, int force_sync) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return ok_or_zero(step(S, substeps, iterations, fetch_diagnostics, force_sync));
}

extern "C" SSBL_API int ssbl_step_solver(void* handle, int substeps, int iterations) {
    return ssbl_step_solver_ex(handle, substeps, iterations, 1, 1);
}

extern "C" SSBL_API int ssbl_download_positions(void* handle, float* out, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid position download") ? 1 : 0;
    return ok_or_zero(download_positions(S, -1, out, max_floats));
}

extern "C" SSBL_API int ssbl_get_diagnostics(void* handle, SsblXpbdDiagnostics* out) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out) return fail("invalid diagnostics request") ? 1 : 0;
    *out = S->diag;
    return 1;
}

extern "C" SSBL_API unsigned int ssbl_capabilities(void) {
    return SSBL_CAP_STRETCH_OPTIMIZATION | SSBL_CAP_PIN_WEIGHTS | SSBL_CAP_GLOBAL_DYNAMIC_SCENE;
}

// Shared dynamic scene (abi41.cu:6597-6784, 8733-8789): colliders of many
// sources hashed once and read by every attached cloth through its source
// filter.  Attaching with mode 0 keeps the cloth on its own colliders.
extern "C" SSBL_API void* ssbl_create_global_dynamic_scene(void) {
    g_error.clear();
    return scene_create();
}

extern "C" SSBL_API int ssbl_destroy_global_dynamic_scene(void* scene) {
    g_error.clear();
    scene_destroy(reinterpret_cast<GlobalScene*>(scene));
    return 1;
}

extern "C" SSBL_API int ssbl_update_global_dynamic_scene(void* scene, const SsblXpbdGlobalDynamicSceneInputs* in) {
    g_error.clear();
    return ok_or_zero(scene_update(reinterpret_cast<GlobalScene*>(scene), in));
}

extern "C" SSBL_API int ssbl_attach_global_dynamic_scene(void* handle, void* scene, int target_source_id, int target_collision_layer,
                                                         int collision_mode) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !scene) return fail("invalid global dynamic scene attach") ? 1 : 0;
    return ok_or_zero(scene_attach(S, -1, reinterpret_cast<GlobalScene*>(scene), target_source_id, target_collision_layer, collision_mode));
}

extern "C" SSBL_API int ssbl_clear_global_dynamic_scene(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid global dynamic scene clear") ? 1 : 0;
    scene_detach(S, -1);
    return 1;
}

extern "C" SSBL_API const char* ssbl_last_error(void) { return g_error.c_str(); }

// ------------------------------------------------------------ batch entry points

XG_EXPORT void* xpbd_gb300_batch_create(const SsblXpbdConfig* configs, const SsblXpbdMesh* meshes, int cloth_count) {
    g_error.clear();
    if (!configs || !meshes || cloth_count < 1) {
        fail("invalid batch create request");
        return nullptr;
    }
    return create_solver(configs, meshes, cloth_count);
}

XG_EXPORT int xpbd_gb300_batch_cloth_count(void* handle) {
    Solver* S = as_solver(handle);
    return S ? S->K : -1;
}

XG_EXPORT int xpbd_gb300_batch_cloth_range(void* handle, int cloth, int* out4) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out4 || cloth < 0 || cloth >= S->K) return fail("invalid cloth index") ? 1 : 0;
    // offsets in the caller's cloth order (the order of whole-handle transfers)
    int estart = 0;
    for (int k = 0; k < cloth; ++k) estart += S->hp[S->ext2int[k]].E;
    const Params& P = S->hp[S->ext2int[cloth]];
    out4[0] = S->ext_vstart[cloth];
    out4[1] = P.V;
    out4[2] = estart;
    out4[3] = P.E;
    return 1;
}

XG_EXPORT int xpbd_gb300_batch_update_pin_targets(void* handle, int cloth, const int* indices, const float* positions,
                                                  const float* weights, int count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid cloth index") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(upload_pins(S, cloth, indices, positions, weights, count));
}

XG_EXPORT int xpbd_gb300_batch_update_runtime_colliders(void* handle, int cloth, const SsblXpbdRuntimeColliders* inputs) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !inputs || cloth < 0 || cloth >= S->K) return fail("invalid runtime collider update") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(set_colliders(S, cloth, *inputs));
}

XG_EXPORT int xpbd_gb300_batch_update_static_triangles(void* handle, int cloth, const float* triangles, int triangle_count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid static triangle update") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(upload_static(S, cloth, triangles, triangle_count));
}

XG_EXPORT int xpbd_gb300_batch_update_frame_inputs(void* handle, int cloth, const SsblXpbdFrameInputs* in) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid frame input update") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(frame_inputs(S, cloth, in));
}

XG_EXPORT int xpbd_gb300_batch_update_positions(void* handle, int cloth, const float* positions, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid position upload") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(upload_positions(S, cloth, positions, max_floats));
}

XG_EXPORT int xpbd_gb300_batch_download_positions(void* handle, int cloth, float* out, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid position download") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(download_positions(S, cloth, out, max_floats));
}

XG_EXPORT int xpbd_gb300_batch_attach_global_dynamic_scene(void* handle, int cloth, void* scene, int target_source_id,
                                                           int target_collision_layer, int collision_mode) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !scene || cloth < 0 || cloth >= S->K) return fail("invalid global dynamic scene attach") ? 1 : 0;
    return ok_or_zero(scene_attach(S, S->ext2int[cloth], reinterpret_cast<GlobalScene*>(scene), target_source_id,
                                   target_collision_layer, collision_mode));
}

XG_EXPORT int xpbd_gb300_batch_clear_global_dynamic_scene(void* handle, int cloth) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid global dynamic scene clear") ? 1 : 0;
    scene_detach(S, S->ext2int[cloth]);
    return 1;
}

XG_EXPORT int xpbd_gb300_batch_reset_cloth(void* handle, int cloth) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid cloth index") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(reset_cloths(S, cloth));
}

XG_EXPORT int xpbd_gb300_batch_set_active(void* handle, int cloth, int active) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth < 0 || cloth >= S->K) return fail("invalid cloth index") ? 1 : 0;
    cloth = S->ext2int[cloth];
    return ok_or_zero(set_active(S, cloth, active != 0));
}

// ------------------------------------------------------ GB300 extensions --

XG_EXPORT int xpbd_gb300_build_self_structures(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    if (!S->self_any || !S->nb_count) return fail("self collision is not enabled for this solver") ? 1 : 0;
    if (!sync_params(S)) return 0;
    // one scheduled substep outside the passes: every enabled cloth builds
    SelfVariants sv{};
    for (int k = 0; k < S->K; ++k) {
        const Params& P = S->hp[k];
        if (!P.self_on) continue;
        sv.hashed_v |= P.vhash != 0;
        sv.brute_v |= P.vhash == 0;
        sv.add_cloth(P, S->cl[k].fast);
    }
    const View v = S->view();
    if (S->nVB > 0) {
        cudaMemsetAsync(S->vb_count, 0, sizeof(int) * S->nVB, S->stream);
        self_build_vertex_hash(v, sv, S->nVB, S->stream);
    }
    if (S->nTB > 0) {
        cudaMemsetAsync(S->tb_count, 0, sizeof(int) * S->nTB, S->stream);
        self_build_triangle_hash(v, sv, S->nTB, 1, S->stream);
    }
    if (S->nEB > 0) {
        View ev = v;  // the edge hash lists its buckets of more than 32 members in trim segment 2
        const size_t trim_seg = (size_t)std::max(std::max(S->nVB, S->nTB), S->nEB);
        ev.trim_list = S->trim_list + 2 * trim_seg;
        ev.trim_count = S->trim_count + 2;
        reset_edge_hash(S, S->stream);
        self_build_edge_hash(ev, sv, S->nEB, 3, S->stream);
    }
    self_neighbors(v, 0, sv, S->stream);
    return (cuda_ok(cudaGetLastError(), "build self structures") && cuda_ok(cudaStreamSynchronize(S->stream), "build self structures")) ? 1 : 0;
}

namespace {

// The edge hash as a bucket CSR (start[nEB + 1], then the members bucket
// after bucket), as the triangle and vertex hashes are kept: a bucket of up
// to kEdgeSlots members lists its slots (a bucket of more than 32 with its 32
// smallest ids first, in increasing order), a larger one its full member
// list in increasing id order.
long long read_edge_buckets(Solver* S, bool starts, void* out, long long max_bytes) {
    const size_t nb = (size_t)S->nEB;
    std::vector<int> cnt(nb), first(nb);
    if (!cuda_ok(cudaStreamSynchronize(S->stream), "read edge hash") ||
        !cuda_ok(cudaMemcpy(cnt.data(), S->eb_count, sizeof(int) * nb, cudaMemcpyDeviceToHost), "read edge hash") ||
        !cuda_ok(cudaMemcpy(first.data(), S->eb_start, sizeof(int) * nb, cudaMemcpyDeviceToHost), "read edge hash"))
        return -1;
    std::vector<int> start(nb + 1, 0);
    for (size_t b = 0; b < nb; ++b) start[b + 1] = start[b] + cnt[b];
    if (starts) {
        const long long bytes = 4ll * (long long)(nb + 1);
        if (bytes > max_bytes) {
            fail("output buffer too small");
            return -1;
        }
        std::memcpy(out, start.data(), (size_t)bytes);
        return bytes;
    }
    const long long bytes = 4ll * start[nb];
    if (bytes > max_bytes) {
        fail("output buffer too small");
        return -1;
    }
    std::vector<int> slots(nb * kEdgeSlots);
    std::vector<int> all(std::max(start[nb], 1));
    if (!cuda_ok(cudaMemcpy(slots.data(), S->eb_slot, sizeof(int) * slots.size(), cudaMemcpyDeviceToHost), "read edge hash") ||
        (start[nb] > 0 && !cuda_ok(cudaMemcpy(all.data(), S->eb_ent, sizeof(int) * (size_t)start[nb], cudaMemcpyDeviceToHost),
                                   "read edge hash")))
        return -1;
    int* o = static_cast<int*>(out);
    for (size_t b = 0; b < nb; ++b) {
        const int n = cnt[b];
        int* dst = o + start[b];
        if (n <= kEdgeSlots) {
            std::memcpy(dst, slots.data() + b * kEdgeSlots, sizeof(int) * (size_t)n);
        } else {
            // overflow region [eb_start[b] - n, eb_start[b]) of the last build
            std::memcpy(dst, all.data() + (first[b] - n), sizeof(int) * (size_t)n);
            std::sort(dst, dst + n);
        }
    }
    return bytes;
}

}  // namespace

XG_EXPORT long long xpbd_gb300_read_buffer(void* handle, int id, void* out, long long max_bytes) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out) {
        fail("invalid buffer read");
        return -1;
    }
    const void* src = nullptr;
    long long bytes = 0;
    int total_t = 0;
    if ((id == XPBD_BUF_EDGE_BUCKET_START || id == XPBD_BUF_EDGE_BUCKET_ENTRIES) && S->eb_slot)
        return read_edge_buckets(S, id == XPBD_BUF_EDGE_BUCKET_START, out, max_bytes);
    if (id == XPBD_BUF_TRI_BUCKET_ENTRIES && S->tb_start) {
        const int* st = S->tb_start;
        const int nb = S->nTB;
        int total = 0;
        if (!cuda_ok(cudaStreamSynchronize(S->stream), "read bucket total") ||
            !cuda_ok(cudaMemcpy(&total, st + nb, sizeof(int), cudaMemcpyDeviceToHost), "read bucket total"))
            return -1;
        total_t = total;
    }
    const Params& P0 = S->hp[0];
    switch (id) {
        case XPBD_BUF_POSITIONS4: src = S->pos[0]; bytes = 16ll * S->nV; break;
        case XPBD_BUF_PREV4: src = S->prev; bytes = 16ll * S->nV; break;
        case XPBD_BUF_VEL4: src = S->vel; bytes = 16ll * S->nV; break;
        case XPBD_BUF_VERTEX_CELLS: src = S->vcell; bytes = 16ll * S->nV; break;
        case XPBD_BUF_VERTEX_BUCKET_START: src = S->vb_start; bytes = 4ll * (S->nVB + 1); break;
        case XPBD_BUF_VERTEX_BUCKET_ENTRIES: src = S->vb_ent; bytes = 4ll * S->nV; break;
        case XPBD_BUF_TRI_BUCKET_START: src = S->tb_start; bytes = 4ll * (S->nTB + 1); break;
        case XPBD_BUF_TRI_BUCKET_ENTRIES: src = S->tb_ent; bytes = 4ll * total_t; break;
        case XPBD_BUF_EDGE_BUCKET_START:
        case XPBD_BUF_EDGE_BUCKET_ENTRIES: src = nullptr; bytes = 0; break;  // no edge hash
        case XPBD_BUF_NEIGHBOR_COUNTS: src = S->nb_count; bytes = 4ll * S->nV; break;
        case XPBD_BUF_NEIGHBOR_INDICES: src = S->nb_idx; bytes = 4ll * S->nV * kNeighborSlots; break;
        case XPBD_BUF_STATIC_SDF:
            src = S->cl[0].grid ? S->cl[0].grid->sdf : nullptr;
            bytes = P0.sdf_ready ? 4ll * P0.sdf_dim[0] * P0.sdf_dim[1] * P0.sdf_dim[2] : 0;
            break;
        case XPBD_BUF_COUNTERS: src = S->counts; bytes = 8ll * kCntSlots; break;
        default: fail("unknown buffer id"); return -1;
    }
    if (!src && bytes > 0) {
        fail("buffer is not allocated for this solver");
        return -1;
    }
    if (!src) return 0;
    if (bytes > max_bytes) {
        fail("output buffer too small");
        return -1;
    }
    if (!cuda_ok(cudaStreamSynchronize(S->stream), "read buffer") ||
        (bytes > 0 && !cuda_ok(cudaMemcpy(out, src, (size_t)bytes, cudaMemcpyDeviceToHost), "read buffer")))
        return -1;
    return bytes;
}

XG_EXPORT int xpbd_gb300_hash_info(void* handle, int* out6) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out6) return fail("invalid hash info request") ? 1 : 0;
    out6[0] = S->nVB;
    out6[1] = S->nTB;
    out6[2] = S->nEB;
    out6[3] = S->K == 1 ? S->hp[0].vhash : (S->nVB > 0);
    out6[4] = S->K == 1 ? S->hp[0].thash : (S->nTB > 0);
    out6[5] = S->K == 1 ? S->hp[0].ehash : (S->nEB > 0);
    return 1;
}

XG_EXPORT int xpbd_gb300_set_graph_capture(void* handle, int enabled) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    S->use_graphs = enabled != 0;
    return 1;
}

XG_EXPORT int xpbd_gb300_set_key_division(void* handle, int mode) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    if (mode != 0 && mode != 1) return fail("key division mode must be 0 (reference) or 1 (IEEE)") ? 1 : 0;
    S->key_ieee = mode;
    for (Params& P : S->hp) P.key_ieee = mode;
    S->params_dirty = true;
    return 1;
}

XG_EXPORT int xpbd_gb300_set_default_key_division(int mode) {
    g_error.clear();
    if (mode != 0 && mode != 1) return fail("key division mode must be 0 (reference) or 1 (IEEE)") ? 1 : 0;
    g_default_key_ieee.store(mode);
    return 1;
}

XG_EXPORT long long xpbd_gb300_last_step_launches(void* handle) {
    Solver* S = as_solver(handle);
    return S ? S->last_launches : -1;
}

XG_EXPORT void* xpbd_gb300_stream(void* handle) {
    Solver* S = as_solver(handle);
    return S ? reinterpret_cast<void*>(S->stream) : nullptr;
}

XG_EXPORT int xpbd_gb300_profile_frame(void* handle, int substeps, int iterations, float* kernel_ms,
                                       long long* kernel_launches, int kinds) {
    g_error.clear();
    return ok_or_zero(profile_frame(as_solver(handle), substeps, iterations, kernel_ms, kernel_launches, kinds));
}

XG_EXPORT void* xpbd_gb300_pc2_open(void* handle, int cloth, const char* path, int start_frame) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || cloth >= S->K) {
        fail("invalid PC2 writer request");
        return nullptr;
    }
    return pc2_open(S, cloth < 0 ? -1 : S->ext2int[cloth], path, start_frame);
}

XG_EXPORT int xpbd_gb300_pc2_write(void* handle, void* writer, const float* matrix_world_inv16) {
    g_error.clear();
    return ok_or_zero(pc2_write(as_solver(handle), writer, matrix_world_inv16));
}

XG_EXPORT long long xpbd_gb300_pc2_close(void* writer, int commit) {
    g_error.clear();
    return pc2_close(writer, commit != 0);
}

XG_EXPORT int xpbd_gb300_set_launch_config(void* handle, const int* values, int count) {
    g_error.clear();
    return ok_or_zero(set_launch_config(as_solver(handle), values, count));
}

XG_EXPORT int xpbd_gb300_get_launch_config(void* handle, int* out, int count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out || count < 0) return fail("invalid launch configuration request") ? 1 : 0;
    for (int k = 0; k < count; ++k) out[k] = k < kTuneSlots ? effective_tune(S, k) : 0;
    return 1;
}

XG_EXPORT int xpbd_gb300_solver_info(void* handle, long long* out8) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out8) return fail("invalid solver info request") ? 1 : 0;
    long long fast = 0, strict = 0, dyn = 0, sdf = 0;
    for (int k = 0; k < S->K; ++k) {
        if (S->cl[k].self_enabled) (S->cl[k].fast ? fast : strict) += 1;
        dyn += S->hp[k].dyn ? 1 : 0;
        sdf += S->hp[k].sdf_ready ? 1 : 0;
    }
    out8[0] = S->K;
    out8[1] = S->nV;
    out8[2] = S->nE;
    out8[3] = S->nT;
    out8[4] = fast;
    out8[5] = strict;
    out8[6] = dyn;
    out8[7] = sdf;
    return 1;
}

XG_EXPORT int xpbd_gb300_autotune(void* handle, int substeps, int iterations, int rounds, float* ms_out2) {
    g_error.clear();
    return ok_or_zero(autotune(as_solver(handle), std::max(substeps, 1), std::max(iterations, 1), rounds, ms_out2));
}

XG_EXPORT int xpbd_gb300_profile_counters(void* handle, long long* out) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out) return fail("invalid profile counter request") ? 1 : 0;
    unsigned long long stripes[kPerfStripes * kPerfStride], c[kPerfSlots] = {};
    int entries[1] = {0};  // the triangle hash scan's total: entries of its last build
    if (!cuda_ok(cudaMemcpyAsync(stripes, S->perf, sizeof(stripes), cudaMemcpyDeviceToHost, S->stream), "read work counters") ||
        (S->tb_start && S->nTB > 0 &&
         !cuda_ok(cudaMemcpyAsync(&entries[0], S->tb_start + S->nTB, sizeof(int), cudaMemcpyDeviceToHost, S->stream),
                  "read triangle hash size")) ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "read work counters"))
        return 0;
    long long edge_entries = 0;  // the edge hash keeps counts, not starts: their sum
    if (S->eb_count && S->nEB > 0) {
        std::vector<int> cnt((size_t)S->nEB);
        if (!cuda_ok(cudaMemcpy(cnt.data(), S->eb_count, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost), "read edge hash size"))
            return 0;
        for (int x : cnt) edge_entries += x;
    }
    for (int q = 0; q < kPerfStripes; ++q)
        for (int k = 0; k < kPerfSlots; ++k) c[k] += stripes[q * kPerfStride + k];
    for (int k = 0; k < 4; ++k) out[k] = (long long)c[k];
    out[10] = (long long)c[kPerfEeGathers];
    long long tris = 0, edges = 0;
    for (const Params& P : S->hp) {
        if (!P.self_on) continue;
        if (P.thash) tris += P.T;
        if (P.ehash) edges += P.E;
    }
    out[4] = entries[0];
    out[5] = edge_entries;
    out[6] = tris;
    out[7] = edges;
    out[8] = S->nTB;
    out[9] = S->nEB;
    return 1;
}

XG_EXPORT int xpbd_gb300_prepare_graph(void* handle, int substeps, int iterations) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return ok_or_zero(prepare_graph(S, std::max(substeps, 1), std::max(iterations, 1)));
}

XG_EXPORT long long xpbd_gb300_device_bytes(void* handle) {
    Solver* S = as_solver(handle);
    return S ? S->device_bytes : -1;
}

XG_EXPORT int xpbd_gb300_synchronize(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return cuda_ok(cudaStreamSynchronize(S->stream), "synchronize") ? 1 : 0;
}
