// Vertex spatial hash for callers that cannot allocate device memory.
//
// Some hosts of this solver own every byte of device memory themselves: an
// application that reserves the GPU up front through its own memory pool, or
// a frame loop that must never pay for the implicit device synchronisation a
// cudaMalloc or cudaFree can bring.  For them this file offers one extra entry
// point that builds the vertex spatial hash (the same counting sort as the
// solver's own hash build: cell per vertex, bucket counts, exclusive scan,
// scatter, members ordered by vertex id) without allocating anything.  The
// caller passes the positions and the output arrays; the only scratch, the
// per-bucket counters, lives in the file-scope array below.
//
// Limits and sharing:
//   * at most kNoAllocMaxBuckets buckets (1 MiB of counters); larger tables
//     are rejected with an error;
//   * the array exists once per device that loads the library and stays
//     allocated until the process exits;
//   * every call on a device uses the same array, which keeps what the last
//     call left there: each call clears the counters it uses first, and two
//     calls whose work overlaps on the GPU (different streams, or host threads
//     without ordering) race on it and corrupt each other's result;
//   * every call looks up the array's device address in the current context
//     (cudaGetSymbolAddress, with the caller's device current), so a device
//     reset or another context on the same device never leaves a stale
//     address behind; the first lookup on a device also loads the library's
//     device code there, so make the first call on a device before any
//     stream capture begins.
#include <climits>
#include <cmath>
#include <string>

#include "xpbd_solver.cuh"

namespace {

constexpr int kNoAllocMaxBuckets = 1 << 18;

// Bucket counters, then scatter cursors, of the last call on this device.
static __device__ __align__(256) int g_noalloc_bucket_scratch[kNoAllocMaxBuckets];

bool noalloc_fail(const std::string& msg) {
    xg::set_last_error(msg);
    return false;
}

// Device address of the scratch array in the current context.  In host code
// the array's name is only a host-side stand-in, never a device address.
bool scratch_for_current_device(int** out) {
    void* ptr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_bucket_scratch);
    if (err != cudaSuccess || !ptr)
        return noalloc_fail(std::string("cudaGetSymbolAddress of the hash scratch failed: ") + cudaGetErrorString(err));
    *out = static_cast<int*>(ptr);
    return true;
}

__global__ void k_zero(int* a, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = 0;
}

__global__ void k_cells(const float* __restrict__ pos, int n, float cell, int buckets, int* counts, int4* cells) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const int cx = xg::cell_of(x, cell, 0), cy = xg::cell_of(y, cell, 0), cz = xg::cell_of(z, cell, 0);
    const int b = (int)xg::bucket_of(cx, cy, cz, buckets);
    if (cells) cells[i] = make_int4(cx, cy, cz, b);
    atomicAdd(&counts[b], 1);
}

// Exclusive scan of counts into start[0..n], leaving the starts in counts as
// scatter cursors; one block, 4096 counters per round.
__global__ void __launch_bounds__(1024) k_scan_counts(int* counts, int* start, int n) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4096) {
        int v[4], sum = 0;
        for (int k = 0; k < 4; ++k) {
            const int idx = base + tid * 4 + k;
            v[k] = idx < n ? counts[idx] : 0;
            sum += v[k];
        }
        int inc = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) warp_tot[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int w = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        int run = carry + (warp ? warp_tot[warp - 1] : 0) + inc - sum;
        for (int k = 0; k < 4; ++k) {
            const int idx = base + tid * 4 + k;
            if (idx < n) {
                start[idx] = run;
                counts[idx] = run;
            }
            run += v[k];
        }
        __syncthreads();
        if (tid == 1023) carry = run;
        __syncthreads();
    }
    if (tid == 0) start[n] = carry;
}

__global__ void k_scatter(const float* __restrict__ pos, int n, float cell, int buckets, int* cursor, int* entries) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = (int)xg::bucket_of(xg::cell_of(pos[3 * i], cell, 0), xg::cell_of(pos[3 * i + 1], cell, 0),
                                     xg::cell_of(pos[3 * i + 2], cell, 0), buckets);
    entries[atomicAdd(&cursor[b], 1)] = i;
}

// Members of each bucket in increasing vertex id (the 32 smallest first when
// a bucket holds more, as the solver's queries read no further).  A thread
// orders its own bucket when it has at most 32 members; a crowded bucket
// (say a collapsed cloth with every vertex in one cell) is ordered by the
// whole warp: 32 rounds, each a warp-wide minimum over the unplaced members,
// O(n) steps per lane instead of O(32 n) on one thread.  Every thread of
// the grid reaches the ballot (no early return), so the full mask is valid.
__global__ void k_order(const int* start, int* entries, int buckets) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int s = 0, n = 0;
    if (b < buckets) {
        s = start[b];
        n = start[b + 1] - s;
    }
    if (n > 1 && n <= 32) {
        int* e = entries + s;
        for (int i = 0; i < n; ++i) {
            int best = i;
            for (int j = i + 1; j < n; ++j)
                if (e[j] < e[best]) best = j;
            const int t = e[i];
            e[i] = e[best];
            e[best] = t;
        }
    }
    unsigned crowded = __ballot_sync(0xffffffffu, n > 32);
    while (crowded) {
        const int src = __ffs(crowded) - 1;
        crowded &= crowded - 1;
        const int bs = __shfl_sync(0xffffffffu, s, src), bn = __shfl_sync(0xffffffffu, n, src);
        int* e = entries + bs;
        for (int i = 0; i < 32; ++i) {
            int best_v = INT_MAX, best_j = bn;
            for (int j = i + lane; j < bn; j += 32) {
                const int v = e[j];
                if (v < best_v) {
                    best_v = v;
                    best_j = j;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const int ov = __shfl_xor_sync(0xffffffffu, best_v, o);
                const int oj = __shfl_xor_sync(0xffffffffu, best_j, o);
                if (ov < best_v || (ov == best_v && oj < best_j)) {
                    best_v = ov;
                    best_j = oj;
                }
            }
            if (lane == 0 && best_j != i && best_j < bn) {
                e[best_j] = e[i];
                e[i] = best_v;
            }
            __syncwarp();
        }
    }
}

}  // namespace

// No counterpart in the reference.  Builds the vertex spatial hash of
// `vertex_count` positions (device memory, x y z per vertex) with cells of
// `cell_size` metres and `bucket_count` buckets (a power of two, at most
// 262144): bucket_start[0..bucket_count] (device, bucket_count + 1 ints),
// bucket_entries[0..vertex_count) (device) and, when non-null, cells (device,
// 4 ints per vertex: cell x, y, z, bucket; written as int4, so the pointer
// must be 16-byte aligned).  Work is queued on `stream`
// (a cudaStream_t; null = the default stream) and the call returns without
// waiting.  Returns 1, or 0 with the reason in ssbl_last_error().  Allocates
// nothing; see the notes at the top of this file.
extern "C" __attribute__((visibility("default"))) int xpbd_gb300_vertex_hash_noalloc(
    const float* positions, int vertex_count, float cell_size, int bucket_count, int* bucket_start, int* bucket_entries,
    int* cells, void* stream) {
    xg::set_last_error(std::string());
    // A launch error left pending by earlier, unrelated work on this thread
    // would otherwise be reported as this call's failure below.
    (void)cudaGetLastError();
    if (vertex_count < 0 || (vertex_count > 0 && (!positions || !bucket_entries)) || !bucket_start)
        return noalloc_fail("invalid vertex hash request") ? 1 : 0;
    if (!std::isfinite(cell_size) || cell_size <= 0.0f) return noalloc_fail("cell size must be finite and positive") ? 1 : 0;
    if (bucket_count <= 0 || (bucket_count & (bucket_count - 1)) != 0)
        return noalloc_fail("bucket count must be a positive power of two") ? 1 : 0;
    if (bucket_count > kNoAllocMaxBuckets)
        return noalloc_fail("bucket count exceeds the no-allocation limit of 262144 buckets") ? 1 : 0;
    int* scratch = nullptr;
    if (!scratch_for_current_device(&scratch)) return 0;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int threads = 256;
    k_zero<<<(bucket_count + threads - 1) / threads, threads, 0, s>>>(scratch, bucket_count);
    if (vertex_count > 0)
        k_cells<<<(vertex_count + threads - 1) / threads, threads, 0, s>>>(positions, vertex_count, cell_size, bucket_count,
                                                                           scratch, reinterpret_cast<int4*>(cells));
    k_scan_counts<<<1, 1024, 0, s>>>(scratch, bucket_start, bucket_count);
    if (vertex_count > 0)
        k_scatter<<<(vertex_count + threads - 1) / threads, threads, 0, s>>>(positions, vertex_count, cell_size,
                                                                             bucket_count, scratch, bucket_entries);
    k_order<<<(bucket_count + threads - 1) / threads, threads, 0, s>>>(bucket_start, bucket_entries, bucket_count);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return noalloc_fail(std::string("launch vertex hash: ") + cudaGetErrorString(err)) ? 1 : 0;
    return 1;
}
