// Device preprocessing of a cloth's constraint inputs: the unique edges of a
// triangle mesh with their rest lengths, the bend pairs with theirs, and the
// per-vertex inverse masses from triangle areas, the per-element steps of the
// reference's input pipeline (xpbd_core.py:715-747 edges and bends, 862-881
// masses) that dominate the cost of building large cloths.  Greedy colouring
// stays on the host (xpbd_prep.cu): first-fit in constraint order is
// sequential by definition; so do the hidden tethers (a k-d tree query whose
// tie-breaking between equidistant pins a device argmin would not repeat).
//
// Results are bit-identical to the cloth builders' numpy restatement:
// * edges are the distinct (min, max) endpoint pairs of every triangle side
//   in lexicographic order (np.unique over rows): a CSR keyed by the lower
//   endpoint (count, scan, scatter), each row sorted and deduplicated;
// * rest length = max(|x_b - x_a|, eps) in float32 with the sum of squares
//   taken x, y, z in order (np.linalg.norm over a row of three);
// * bend pairs as xpbd_gb300_bend_pairs writes them (below), rest lengths
//   as for edges;
// * mass = float64 sum of float32 shares max(area * density, eps) / 3 in
//   np.add.at order (corner 0 of every triangle in index order, then corner
//   1, then 2): a CSR keyed by vertex with entries corner * T + t, sorted;
//   area = 0.5 |(x1 - x0) x (x2 - x0)| in float32; inverse mass 1 / mass
//   (mass 1 where nothing was added), 0 for hard-pinned vertices.
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "xpbd_solver.cuh"

#define XG_EXPORT extern "C" __attribute__((visibility("default")))

namespace xg {
namespace {

constexpr int kPrepThreads = 256;

inline int blocks_of(long long n) { return (int)((n + kPrepThreads - 1) / kPrepThreads); }

__device__ __forceinline__ void side(const int* tris, int t, int j, int* lo, int* hi) {
    const int a = tris[3 * t + j], b = tris[3 * t + (j + 1) % 3];
    *lo = min(a, b);
    *hi = max(a, b);
}

__global__ void k_side_count(const int* tris, int T, int* count) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 3ll * T) return;
    int lo, hi;
    side(tris, (int)(s / 3), (int)(s % 3), &lo, &hi);
    atomicAdd(&count[lo], 1);
}

__global__ void k_side_scatter(const int* tris, int T, int* cursor, int* ent) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 3ll * T) return;
    int lo, hi;
    side(tris, (int)(s / 3), (int)(s % 3), &lo, &hi);
    ent[atomicAdd(&cursor[lo], 1)] = hi;
}

// Sort one CSR row in place (insertion sort: rows are a vertex's incident
// sides or corners, a handful of entries on a manifold mesh).
__device__ void sort_row(int* r, int n) {
    for (int i = 1; i < n; ++i) {
        const int key = r[i];
        int j = i - 1;
        while (j >= 0 && r[j] > key) {
            r[j + 1] = r[j];
            --j;
        }
        r[j + 1] = key;
    }
}

// Row a: sort, keep distinct upper endpoints at the row's front, count them.
__global__ void k_side_unique(const int* start, int* ent, int V, int* distinct) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= V) return;
    int* r = ent + start[a];
    const int n = start[a + 1] - start[a];
    sort_row(r, n);
    int u = 0;
    for (int i = 0; i < n; ++i)
        if (u == 0 || r[i] != r[u - 1]) r[u++] = r[i];
    distinct[a] = u;
}

__global__ void k_edge_emit(const int* start, const int* ent, const int* edge_start, const float* pos, int V, float eps,
                            int* edges, float* rest) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= V) return;
    const int* r = ent + start[a];
    const int n = edge_start[a + 1] - edge_start[a];
    const float ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
    for (int i = 0; i < n; ++i) {
        const int b = r[i], e = edge_start[a] + i;
        const float dx = pos[3 * b] - ax, dy = pos[3 * b + 1] - ay, dz = pos[3 * b + 2] - az;
        const float len = sqrtf((dx * dx + dy * dy) + dz * dz);
        edges[2 * e] = a;
        edges[2 * e + 1] = b;
        rest[e] = fmaxf(len, eps);
    }
}

// Bend pairs (xpbd_core.py:730-747): sides keyed by their lower endpoint,
// entries (upper endpoint << 32 | side index s = 3 t + j), so a sorted row
// lists every edge's sides in triangle order.  The first side of an edge
// gives the reference opposite vertex; each later side whose opposite vertex
// differs yields the pair (min, max) of the two opposite vertices.  Pairs are
// written into the row's own slots (at most one per side).
__global__ void k_side_scatter64(const int* tris, int T, int* cursor, long long* ent) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 3ll * T) return;
    int lo, hi;
    side(tris, (int)(s / 3), (int)(s % 3), &lo, &hi);
    ent[atomicAdd(&cursor[lo], 1)] = ((long long)hi << 32) | (long long)s;
}

__global__ void k_bend_rows(const int* start, long long* ent, const int* tris, int V, int* pair_p, int* pair_q,
                            int* row_pairs) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= V) return;
    long long* r = ent + start[x];
    const int n = start[x + 1] - start[x];
    for (int i = 1; i < n; ++i) {
        const long long key = r[i];
        int j = i - 1;
        while (j >= 0 && r[j] > key) {
            r[j + 1] = r[j];
            --j;
        }
        r[j + 1] = key;
    }
    int m = 0, first_opp = 0;
    for (int i = 0; i < n; ++i) {
        const int y = (int)(r[i] >> 32), s = (int)(r[i] & 0xffffffffll);
        const int opp = tris[3 * (s / 3) + (s % 3 + 2) % 3];
        if (i == 0 || y != (int)(r[i - 1] >> 32)) {
            first_opp = opp;
        } else if (opp != first_opp) {
            pair_p[start[x] + m] = min(first_opp, opp);
            pair_q[start[x] + m] = max(first_opp, opp);
            ++m;
        }
    }
    row_pairs[x] = m;
}

__global__ void k_pair_count(const int* start, const int* pair_p, const int* row_pairs, int V, int* count) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= V) return;
    for (int i = 0; i < row_pairs[x]; ++i) atomicAdd(&count[pair_p[start[x] + i]], 1);
}

__global__ void k_pair_scatter(const int* start, const int* pair_p, const int* pair_q, const int* row_pairs, int V,
                               int* cursor, int* ent) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= V) return;
    for (int i = 0; i < row_pairs[x]; ++i) ent[atomicAdd(&cursor[pair_p[start[x] + i]], 1)] = pair_q[start[x] + i];
}

// Per triangle: max(area * density, eps) / 3 in float32.
__global__ void k_share(const int* tris, int T, const float* pos, float density, float eps, float* share) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
    const float ux = pos[3 * i1] - pos[3 * i0], uy = pos[3 * i1 + 1] - pos[3 * i0 + 1], uz = pos[3 * i1 + 2] - pos[3 * i0 + 2];
    const float vx = pos[3 * i2] - pos[3 * i0], vy = pos[3 * i2 + 1] - pos[3 * i0 + 1], vz = pos[3 * i2 + 2] - pos[3 * i0 + 2];
    const float cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    const float area = 0.5f * sqrtf((cx * cx + cy * cy) + cz * cz);
    share[t] = fmaxf(area * density, eps) / 3.0f;
}

__global__ void k_corner_count(const int* tris, int T, int* count) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 3ll * T) return;
    atomicAdd(&count[tris[3 * (c % T) + c / T]], 1);
}

// Entry key corner * T + t: sorted, it is np.add.at's order.
__global__ void k_corner_scatter(const int* tris, int T, int* cursor, int* ent) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 3ll * T) return;
    ent[atomicAdd(&cursor[tris[3 * (c % T) + c / T]], 1)] = (int)c;
}

__global__ void k_inverse_mass(const int* start, int* ent, const float* share, int T, const unsigned char* hard, int V,
                               float* inv) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    int* r = ent + start[v];
    const int n = start[v + 1] - start[v];
    sort_row(r, n);
    double mass = 0.0;
    for (int i = 0; i < n; ++i) mass += (double)share[r[i] % T];
    if (mass <= 0.0) mass = 1.0;
    inv[v] = (hard && hard[v]) ? 0.0f : (float)(1.0 / mass);
}

template <class T>
bool alloc(T** p, size_t n, std::vector<void*>* owned) {
    *p = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return false;
    owned->push_back(*p);
    return true;
}

}  // namespace
}  // namespace xg

using namespace xg;

// Edges, rest lengths, inverse masses and (when `bends` is given) bend pairs
// with their rest lengths of a cloth from its rest positions (V x 3 float),
// triangles (T x 3 int, indices in [0, V)), density and hard pin mask (V
// bytes, non-zero = pinned; may be null).  `edges` / `bends` hold room for
// 3T pairs, `edge_rest` / `bend_rest` for 3T floats, `inv_mass` for V
// floats; *bend_count receives the bend count.  Returns the number of edges,
// or -1 (ssbl_last_error() says why).
XG_EXPORT int xpbd_gb300_prepare_cloth_device(const float* positions, int vertex_count, const int* triangles,
                                              int triangle_count, float density, float eps, const unsigned char* hard,
                                              int* edges, float* edge_rest, float* inv_mass, int* bends,
                                              float* bend_rest, int* bend_count) {
    if (bend_count) *bend_count = 0;
    if (bends && (!bend_rest || !bend_count)) {
        set_last_error("invalid cloth preprocessing request");
        return -1;
    }
    const int V = vertex_count, T = triangle_count;
    if (V < 0 || T < 0 || (V > 0 && (!positions || !inv_mass)) || (T > 0 && (!triangles || !edges || !edge_rest)) ||
        3ll * T > (1ll << 30)) {
        set_last_error("invalid cloth preprocessing request");
        return -1;
    }
    for (long long i = 0; i < 3ll * T; ++i)
        if (triangles[i] < 0 || triangles[i] >= V) {
            set_last_error("triangle index " + std::to_string(triangles[i]) + " outside the " + std::to_string(V) +
                           " vertices");
            return -1;
        }
    if (V == 0) return 0;
    cudaStream_t st = nullptr;
    std::vector<void*> owned;
    auto finish = [&](int result, const char* what) {
        if (what) set_last_error(std::string("cloth preprocessing: ") + what + ": " + cudaGetErrorString(cudaGetLastError()));
        if (st) cudaStreamSynchronize(st);
        for (void* p : owned) cudaFree(p);
        if (st) cudaStreamDestroy(st);
        return what ? -1 : result;
    };
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return finish(0, "stream");
    float *d_pos, *d_rest, *d_share, *d_inv;
    int *d_tris, *d_count, *d_start, *d_ent, *d_distinct, *d_estart, *d_edges, *d_sums;
    unsigned char* d_hard = nullptr;
    const long long S = 3ll * T;
    const int sums = V / 4096 + 2;
    if (!alloc(&d_pos, 3ull * V, &owned) || !alloc(&d_tris, (size_t)S, &owned) || !alloc(&d_count, V, &owned) ||
        !alloc(&d_start, V + 1ull, &owned) || !alloc(&d_ent, (size_t)S, &owned) || !alloc(&d_distinct, V, &owned) ||
        !alloc(&d_estart, V + 1ull, &owned) || !alloc(&d_edges, 2ull * S, &owned) || !alloc(&d_rest, (size_t)S, &owned) ||
        !alloc(&d_share, (size_t)T, &owned) || !alloc(&d_inv, V, &owned) || !alloc(&d_sums, (size_t)sums, &owned) ||
        (hard && !alloc(&d_hard, V, &owned)))
        return finish(0, "device allocation");
    bool ok = cudaMemcpyAsync(d_pos, positions, sizeof(float) * 3 * V, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              (T == 0 || cudaMemcpyAsync(d_tris, triangles, sizeof(int) * S, cudaMemcpyHostToDevice, st) == cudaSuccess) &&
              (!hard || cudaMemcpyAsync(d_hard, hard, V, cudaMemcpyHostToDevice, st) == cudaSuccess);
    if (!ok) return finish(0, "upload");
    // unique edges and their rest lengths
    cudaMemsetAsync(d_count, 0, sizeof(int) * V, st);
    if (S > 0) k_side_count<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count);
    scan_bucket_counts(d_count, d_start, V, d_sums, st);  // d_count becomes the scatter cursor
    if (S > 0) k_side_scatter<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count, d_ent);
    k_side_unique<<<blocks_of(V), kPrepThreads, 0, st>>>(d_start, d_ent, V, d_distinct);
    scan_bucket_counts(d_distinct, d_estart, V, d_sums, st);
    k_edge_emit<<<blocks_of(V), kPrepThreads, 0, st>>>(d_start, d_ent, d_estart, d_pos, V, eps, d_edges, d_rest);
    int E = 0;
    if (cudaMemcpyAsync(&E, d_estart + V, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return finish(0, "edge build");
    // inverse masses (the side CSR is no longer needed: reuse its arrays)
    if (T > 0) k_share<<<blocks_of(T), kPrepThreads, 0, st>>>(d_tris, T, d_pos, density, eps, d_share);
    cudaMemsetAsync(d_count, 0, sizeof(int) * V, st);
    if (S > 0) k_corner_count<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count);
    scan_bucket_counts(d_count, d_start, V, d_sums, st);
    if (S > 0) k_corner_scatter<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count, d_ent);
    k_inverse_mass<<<blocks_of(V), kPrepThreads, 0, st>>>(d_start, d_ent, d_share, std::max(T, 1), d_hard, V, d_inv);
    // bend pairs: side CSR with (upper << 32 | side) entries, pairs per row,
    // then a CSR of the pairs by lower vertex, sorted and deduplicated
    int NB = 0;
    if (bends && S > 0) {
        long long* d_ent64;
        int *d_pp, *d_pq, *d_rowp, *d_bent, *d_bstart, *d_bedges;
        float* d_brest;
        if (!alloc(&d_ent64, (size_t)S, &owned) || !alloc(&d_pp, (size_t)S, &owned) || !alloc(&d_pq, (size_t)S, &owned) ||
            !alloc(&d_rowp, V, &owned) || !alloc(&d_bent, (size_t)S, &owned) || !alloc(&d_bstart, V + 1ull, &owned) ||
            !alloc(&d_bedges, 2ull * S, &owned) || !alloc(&d_brest, (size_t)S, &owned))
            return finish(0, "device allocation");
        int* d_side_start = d_estart;  // free after the edge emit: reuse for the side CSR offsets
        int* d_pstart = d_distinct;    // and for the pair CSR offsets' scratch counts
        cudaMemsetAsync(d_count, 0, sizeof(int) * V, st);
        k_side_count<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count);
        scan_bucket_counts(d_count, d_side_start, V, d_sums, st);
        k_side_scatter64<<<blocks_of(S), kPrepThreads, 0, st>>>(d_tris, T, d_count, d_ent64);
        k_bend_rows<<<blocks_of(V), kPrepThreads, 0, st>>>(d_side_start, d_ent64, d_tris, V, d_pp, d_pq, d_rowp);
        cudaMemsetAsync(d_count, 0, sizeof(int) * V, st);
        k_pair_count<<<blocks_of(V), kPrepThreads, 0, st>>>(d_side_start, d_pp, d_rowp, V, d_count);
        scan_bucket_counts(d_count, d_start, V, d_sums, st);
        k_pair_scatter<<<blocks_of(V), kPrepThreads, 0, st>>>(d_side_start, d_pp, d_pq, d_rowp, V, d_count, d_bent);
        k_side_unique<<<blocks_of(V), kPrepThreads, 0, st>>>(d_start, d_bent, V, d_pstart);
        scan_bucket_counts(d_pstart, d_bstart, V, d_sums, st);
        k_edge_emit<<<blocks_of(V), kPrepThreads, 0, st>>>(d_start, d_bent, d_bstart, d_pos, V, eps, d_bedges, d_brest);
        if (cudaMemcpyAsync(&NB, d_bstart + V, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return finish(0, "bend build");
        if (NB > 0 && (cudaMemcpyAsync(bends, d_bedges, sizeof(int) * 2 * NB, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                       cudaMemcpyAsync(bend_rest, d_brest, sizeof(float) * NB, cudaMemcpyDeviceToHost, st) != cudaSuccess))
            return finish(0, "bend download");
    }
    if (bend_count) *bend_count = NB;
    ok = (E == 0 || (cudaMemcpyAsync(edges, d_edges, sizeof(int) * 2 * E, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                     cudaMemcpyAsync(edge_rest, d_rest, sizeof(float) * E, cudaMemcpyDeviceToHost, st) == cudaSuccess)) &&
         cudaMemcpyAsync(inv_mass, d_inv, sizeof(float) * V, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    if (!ok) return finish(0, "download");
    return finish(E, nullptr);
}
