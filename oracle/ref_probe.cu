// Test-only probe of the reference solver (test infrastructure, not part of
// the product).
//
// This translation unit includes the reference's solver source unchanged
// (native/src/ssbl_xpbd_cuda_abi41.cu, path given by REF_ABI41_SOURCE) and is
// compiled with the reference's own flags, so the library it makes is the
// reference solver plus a few read-only entry points below.  They reach the
// hash tables and the vertex-vertex neighbour lists that the reference keeps
// in its anonymous namespace and does not export through its ABI
// (abi41.cu:394-560 for the fields, 6834-6994 for the builders), so the
// parity tests can compare those integer structures with this repository's
// on identical input positions.
#ifndef REF_ABI41_SOURCE
#error "REF_ABI41_SOURCE must name the reference's ssbl_xpbd_cuda_abi41.cu"
#endif
#include REF_ABI41_SOURCE

namespace {

template <typename T>
long long probe_copy(const T* dev, long long count, void* out, long long max_bytes) {
    if (!dev || count <= 0) return 0;
    const long long bytes = count * (long long)sizeof(T);
    if (!out || bytes > max_bytes) return -1;
    if (cudaMemcpy(out, dev, (size_t)bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return bytes;
}

__global__ void refprobe_cell_kernel(const float* values, int n, float cell, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cell_coord(values[i], cell);
}

}  // namespace

// Buffers readable with refprobe_read.
enum {
    REFPROBE_VERTEX_CELLS = 0,        // int x 3V (written by the vertex hash build)
    REFPROBE_VERTEX_BUCKET_COUNTS = 1,  // int x vertex buckets (pre-clamp counts)
    REFPROBE_VERTEX_BUCKET_SLOTS = 2,   // int x vertex buckets x 32
    REFPROBE_TRI_CELLS = 3,           // int x 3T (lowest cell of each triangle's box)
    REFPROBE_TRI_BUCKET_COUNTS = 4,
    REFPROBE_TRI_BUCKET_SLOTS = 5,
    REFPROBE_EDGE_CELLS = 6,
    REFPROBE_EDGE_BUCKET_COUNTS = 7,
    REFPROBE_EDGE_BUCKET_SLOTS = 8,
    REFPROBE_NEIGHBOR_COUNTS = 9,     // unsigned x V
    REFPROBE_NEIGHBOR_SLOTS = 10,     // unsigned x V x 32
    REFPROBE_COUNTERS = 11,           // unsigned long long x 38
    REFPROBE_POSITIONS = 12,          // float x 3V
    REFPROBE_PREVIOUS = 13,           // float x 3V
    REFPROBE_VELOCITIES = 14          // float x 3V
};

extern "C" {

// out8 = vertex / triangle / edge bucket counts, the three "hash ready"
// flags, vertex count, slots per bucket; cells3 = the three cell sizes.
SSBL_API int refprobe_hash_info(void* handle, int* out8, float* cells3) {
    Abi41Solver* s = reinterpret_cast<Abi41Solver*>(handle);
    if (!s || !out8 || !cells3) return 0;
    out8[0] = s->self_hash_bucket_count;
    out8[1] = s->self_triangle_hash_bucket_count;
    out8[2] = s->self_edge_hash_bucket_count;
    out8[3] = s->self_hash_ready;
    out8[4] = s->self_triangle_hash_ready;
    out8[5] = s->self_edge_hash_ready;
    out8[6] = s->cfg.vertex_count;
    out8[7] = kAbi41SelfHashBucketSlots;
    cells3[0] = s->self_hash_cell_size;
    cells3[1] = s->self_triangle_hash_cell_size;
    cells3[2] = s->self_edge_hash_cell_size;
    return 1;
}

// Overwrite the current and previous positions (3V floats each; prev may be
// null to copy `pos`), as ssbl_update_positions does for both from one array.
SSBL_API int refprobe_set_state(void* handle, const float* pos, const float* prev) {
    Abi41Solver* s = reinterpret_cast<Abi41Solver*>(handle);
    if (!s || !pos) return 0;
    const size_t bytes = sizeof(Vec3) * (size_t)s->cfg.vertex_count;
    if (cudaMemcpy(s->pos, pos, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return 0;
    if (cudaMemcpy(s->prev, prev ? prev : pos, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return 0;
    return 1;
}

// Run the reference's own builders of the vertex, triangle and edge hashes
// and of the vertex-vertex neighbour table (abi41.cu:6834-6994) on the
// current positions, in the order of its step (abi41.cu:9272-9295), after
// clearing the diagnostic counters.
SSBL_API int refprobe_build_self_structures(void* handle) {
    Abi41Solver* s = reinterpret_cast<Abi41Solver*>(handle);
    if (!s) return 0;
    if (s->abi41_counts && cudaMemset(s->abi41_counts, 0, sizeof(unsigned long long) * kAbi41CountSlots) != cudaSuccess) {
        return 0;
    }
    const bool ok = build_self_collision_hash(s) && build_self_triangle_hash(s) && build_self_edge_hash(s) &&
                    build_self_neighbor_table(s);
    return ok && cudaDeviceSynchronize() == cudaSuccess ? 1 : 0;
}

// Copy one buffer (REFPROBE_*) to host memory; returns the bytes written, 0
// when the buffer does not exist, -1 on error or a short output buffer.
SSBL_API long long refprobe_read(void* handle, int which, void* out, long long max_bytes) {
    Abi41Solver* s = reinterpret_cast<Abi41Solver*>(handle);
    if (!s) return -1;
    const long long V = s->cfg.vertex_count, T = s->cfg.triangle_count, E = s->cfg.edge_count;
    switch (which) {
        case REFPROBE_VERTEX_CELLS: return probe_copy(s->self_cell_coords, 3 * V, out, max_bytes);
        case REFPROBE_VERTEX_BUCKET_COUNTS: return probe_copy(s->self_bucket_counts, (long long)s->self_hash_bucket_count, out, max_bytes);
        case REFPROBE_VERTEX_BUCKET_SLOTS:
            return probe_copy(s->self_bucket_indices, (long long)s->self_hash_bucket_count * kAbi41SelfHashBucketSlots, out, max_bytes);
        case REFPROBE_TRI_CELLS: return probe_copy(s->self_triangle_cell_coords, 3 * T, out, max_bytes);
        case REFPROBE_TRI_BUCKET_COUNTS:
            return probe_copy(s->self_triangle_bucket_counts, (long long)s->self_triangle_hash_bucket_count, out, max_bytes);
        case REFPROBE_TRI_BUCKET_SLOTS:
            return probe_copy(s->self_triangle_bucket_indices,
                              (long long)s->self_triangle_hash_bucket_count * kAbi41SelfTriangleHashBucketSlots, out, max_bytes);
        case REFPROBE_EDGE_CELLS: return probe_copy(s->self_edge_cell_coords, 3 * E, out, max_bytes);
        case REFPROBE_EDGE_BUCKET_COUNTS:
            return probe_copy(s->self_edge_bucket_counts, (long long)s->self_edge_hash_bucket_count, out, max_bytes);
        case REFPROBE_EDGE_BUCKET_SLOTS:
            return probe_copy(s->self_edge_bucket_indices,
                              (long long)s->self_edge_hash_bucket_count * kAbi41SelfEdgeHashBucketSlots, out, max_bytes);
        case REFPROBE_NEIGHBOR_COUNTS: return probe_copy(s->self_collision_counts, V, out, max_bytes);
        case REFPROBE_NEIGHBOR_SLOTS: return probe_copy(s->self_collision_indices, V * kAbi41SelfCollisionNeighborSlots, out, max_bytes);
        case REFPROBE_COUNTERS: return probe_copy(s->abi41_counts, (long long)kAbi41CountSlots, out, max_bytes);
        case REFPROBE_POSITIONS: return probe_copy(reinterpret_cast<const float*>(s->pos), 3 * V, out, max_bytes);
        case REFPROBE_PREVIOUS: return probe_copy(reinterpret_cast<const float*>(s->prev), 3 * V, out, max_bytes);
        case REFPROBE_VELOCITIES: return probe_copy(reinterpret_cast<const float*>(s->vel), 3 * V, out, max_bytes);
        default: return -1;
    }
}

// The reference's cell_coord (abi41.cu:654-656), as compiled in its own
// translation unit, applied to n host values.
SSBL_API int refprobe_cell_coords(const float* values, int n, float cell, int* out) {
    if (n <= 0) return 1;
    if (!values || !out) return 0;
    float* dv = nullptr;
    int* di = nullptr;
    bool ok = cudaMalloc(&dv, sizeof(float) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&di, sizeof(int) * (size_t)n) == cudaSuccess &&
              cudaMemcpy(dv, values, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
        refprobe_cell_kernel<<<(n + 255) / 256, 256>>>(dv, n, cell, di);
        ok = cudaGetLastError() == cudaSuccess &&
             cudaMemcpy(out, di, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    cudaFree(dv);
    cudaFree(di);
    return ok ? 1 : 0;
}

}  // extern "C"
