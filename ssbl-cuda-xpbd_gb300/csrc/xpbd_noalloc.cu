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
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture begins.
#include <cmath>
#include <mutex>
#include <string>

#include "xpbd_solver.cuh"

namespace {

constexpr int kNoAllocMaxBuckets = 1 << 18;
constexpr int kMaxDevices = 64;

// Bucket counters, then scatter cursors, of the last call on this device.
static __device__ __align__(256) int g_noalloc_bucket_scratch[kNoAllocMaxBuckets];

// Host-side device addresses of the array, one per device, filled on the
// first call made with that device current.  The array's name itself is not
// a device address in host code.
int* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

bool noalloc_fail(const std::string& msg) {
    xg::set_last_error(msg);
    return false;
}

bool scratch_for_current_device(int** out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return noalloc_fail(std::string("no current CUDA device: ") + cudaGetErrorString(err));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail("CUDA device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        err = cudaGetSymbolAddress(&ptr, g_noalloc_bucket_scratch);
        if (err != cudaSuccess || !ptr)
            return noalloc_fail(std::string("cudaGetSymbolAddress of the hash scratch failed: ") + cudaGetErrorString(err));
        g_scratch_addr[dev] = static_cast<int*>(ptr);
    }
    *out = g_scratch_addr[dev];
    return true;
}

__global__ void k_zero(int* a, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = 0;
}

__global__ void k_cells(const float* __restrict__ pos, int n, float cell, int buckets, int* counts, int4* cells) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const int cx = xg::cell_of(x, cell), cy = xg::cell_of(y, cell), cz = xg::cell_of(z, cell);
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
    const int b = (int)xg::bucket_of(xg::cell_of(pos[3 * i], cell), xg::cell_of(pos[3 * i + 1], cell),
                                     xg::cell_of(pos[3 * i + 2], cell), buckets);
    entries[atomicAdd(&cursor[b], 1)] = i;
}

// Members of each bucket in increasing vertex id (the 32 smallest first when
// a bucket holds more, as the solver's queries read no further).
__global__ void k_order(const int* start, int* entries, int buckets) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    const int s = start[b], n = start[b + 1] - s;
    int* e = entries + s;
    if (n <= 1) return;
    const int keep = n <= 32 ? n : 32;
    for (int i = 0; i < keep; ++i) {
        int best = i;
        for (int j = i + 1; j < n; ++j)
            if (e[j] < e[best]) best = j;
        const int t = e[i];
        e[i] = e[best];
        e[best] = t;
    }
}

}  // namespace

// No counterpart in the reference.  Builds the vertex spatial hash of
// `vertex_count` positions (device memory, x y z per vertex) with cells of
// `cell_size` metres and `bucket_count` buckets (a power of two, at most
// 262144): bucket_start[0..bucket_count] (device, bucket_count + 1 ints),
// bucket_entries[0..vertex_count) (device) and, when non-null, cells (device,
// 4 ints per vertex: cell x, y, z, bucket).  Work is queued on `stream`
// (a cudaStream_t; null = the default stream) and the call returns without
// waiting.  Returns 1, or 0 with the reason in ssbl_last_error().  Allocates
// nothing; see the notes at the top of this file.
extern "C" __attribute__((visibility("default"))) int xpbd_gb300_vertex_hash_noalloc(
    const float* positions, int vertex_count, float cell_size, int bucket_count, int* bucket_start, int* bucket_entries,
    int* cells, void* stream) {
    xg::set_last_error(std::string());
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
