// Self collision: spatial hashes, the vertex-vertex neighbour table, and the
// vertex-vertex / vertex-triangle / edge-edge repulsion passes
// (reference native/src/ssbl_xpbd_cuda_abi41.cu:4542-5844, schedule at
// 9255-9339).
//
// Hash layout.  The reference inserts primitives into fixed 32-slot buckets
// with atomicAdd slot counters, so bucket contents depend on thread timing.
// Here the vertex and triangle hashes are a counting sort over the bucket id
// (count entries per bucket, exclusive-scan the counts into bucket starts,
// scatter the entries with atomic cursors), and the edge hash, by far the
// largest (about 20 cells per edge), keeps 64 member slots per bucket filled
// in one atomic pass (k_edge_insert; larger buckets get overflow regions).
// Either way each bucket's ids are then ordered so that its first
// min(count, 32) members are the 32 smallest primitive ids in increasing
// order where a query reads order.  Queries read exactly those members,
// which makes candidate order, the 32-slot caps and the fast-mode cluster
// filter deterministic.  Bucket ids, cell coordinates, pre-clamp counts and
// member multisets are the same integers as the reference's when no bucket
// overflows.
//
// Accumulation.  Pushes are scattered into per-vertex fixed-point int64
// accumulators (2^-32 m units) with integer atomics, so the per-vertex sums do
// not depend on the order of the atomics.
#include "xpbd_solver.cuh"

namespace xg {

namespace {


__device__ __forceinline__ float contact_radius(const Params& P) { return P.self_radius; }

__device__ __forceinline__ bool fast_mode(const Params& P) { return P.self_mode == 1; }

__device__ __forceinline__ void accumulate(const View& v, int i, F3 d) {
    if (i < 0 || i >= v.nV || !(__ldg(&v.inv_mass[i]) > 0.0f)) return;
    unsigned long long* a = reinterpret_cast<unsigned long long*>(&v.acc[i]);
    atomicAdd(a + 0, (unsigned long long)to_fix(d.x));
    atomicAdd(a + 1, (unsigned long long)to_fix(d.y));
    atomicAdd(a + 2, (unsigned long long)to_fix(d.z));
    atomicAdd(a + 3, 1ull);
}

// ---------------------------------------------------------------- filters --
// Fast-mode per-thread filters (abi41.cu:714-832).
__device__ int normal_bucket(float v) { return v > 0.45f ? 2 : (v < -0.45f ? 0 : 1); }

__device__ unsigned cluster_key(int pair_type, F3 point, F3 normal, float cell, int ieee) {
    const float c = fmaxf(cell, 1.0e-3f);
    unsigned key = bucket_of(cell_of(point.x, c, ieee), cell_of(point.y, c, ieee), cell_of(point.z, c, ieee), 1 << 20);
    const unsigned nk = (unsigned)normal_bucket(normal.x) | ((unsigned)normal_bucket(normal.y) << 2) |
                        ((unsigned)normal_bucket(normal.z) << 4);
    key ^= nk * 2654435761u;
    key ^= (unsigned)(pair_type + 1) * 2246822519u;
    return key;
}

struct Clusters {
    unsigned keys[16];
    unsigned char counts[16];
    int n;
};

__device__ int accept_slot(int pair_type) {
    return pair_type == 0 ? kCntFilterAcceptedVv : (pair_type == 1 ? kCntFilterAcceptedVt : kCntFilterAcceptedEe);
}

__device__ bool try_local_accept(const View& v, const Params& P, int pair_type, unsigned key, Clusters* cl) {
    if (!fast_mode(P)) return true;
    if (cl) {
        const int n = cl->n < 16 ? cl->n : 16;
        for (int i = 0; i < n; ++i) {
            if (cl->keys[i] == key) {
                if (cl->counts[i] >= 1) {
                    count1(v.counts, kCntFilterRejectedOwnership);
                    return false;
                }
                cl->counts[i] += 1;
                count1(v.counts, kCntClusterOwnedContacts);
                count1(v.counts, accept_slot(pair_type));
                return true;
            }
        }
        if (cl->n >= 16) {
            count1(v.counts, kCntFilterRejectedOwnership);
            return false;
        }
        cl->keys[cl->n] = key;
        cl->counts[cl->n] = 1;
        cl->n += 1;
        count1(v.counts, kCntClusterCount);
        count1(v.counts, kCntClusterOwnedContacts);
    }
    count1(v.counts, accept_slot(pair_type));
    return true;
}

struct Seen {
    int ids[64];
    int n;
};

__device__ bool try_note_seen(const View& v, const Params& P, int key, Seen* seen) {
    if (!fast_mode(P)) return true;
    count1(v.counts, kCntFilterSeen);
    if (!seen) return true;
    const int lim = seen->n < 64 ? seen->n : 64;
    for (int i = 0; i < lim; ++i) {
        if (seen->ids[i] == key) {
            count1(v.counts, kCntFilterRejectedDuplicate);
            return false;
        }
    }
    if (seen->n >= 64) {
        count1(v.counts, kCntSelfOverflow);
        count1(v.counts, kCntFilterRejectedOwnership);
        return false;
    }
    seen->ids[seen->n++] = key;
    return true;
}

__device__ __forceinline__ void filter_count(const View& v, const Params& P, int slot) {
    if (fast_mode(P)) count1(v.counts, slot);
}

// ------------------------------------------------------------- hash build --
// Cell range of a primitive's AABB grown by 1.8 r; ranges of more than 64
// cells collapse to the cell of `fallback` (abi41.cu:871-900).
struct CellRange {
    int x0, x1, y0, y1, z0, z1;
};

// *collapsed is set when the range collapsed (the caller counts it).
__device__ CellRange primitive_cells(F3 lo, F3 hi, F3 fallback, float cell, int ieee, bool* collapsed) {
    CellRange r{cell_of(lo.x, cell, ieee), cell_of(hi.x, cell, ieee), cell_of(lo.y, cell, ieee),
                cell_of(hi.y, cell, ieee), cell_of(lo.z, cell, ieee), cell_of(hi.z, cell, ieee)};
    const long long sx = (long long)r.x1 - r.x0 + 1, sy = (long long)r.y1 - r.y0 + 1, sz = (long long)r.z1 - r.z0 + 1;
    if (sx <= 0 || sy <= 0 || sz <= 0) return r;
    if (sx * sy * sz <= (long long)kMaxPrimitiveCells) return r;
    const int fx = cell_of(fallback.x, cell, ieee), fy = cell_of(fallback.y, cell, ieee), fz = cell_of(fallback.z, cell, ieee);
    *collapsed = true;
    return CellRange{fx, fx, fy, fy, fz, fz};
}

__device__ bool tri_valid(int nV, int4 t) {
    return t.x >= 0 && t.y >= 0 && t.z >= 0 && t.x < nV && t.y < nV && t.z < nV && t.x != t.y && t.y != t.z && t.x != t.z;
}

__device__ bool edge_valid(int nV, int2 e) { return e.x >= 0 && e.y >= 0 && e.x < nV && e.y < nV && e.x != e.y; }

__device__ CellRange tri_cells(const View& v, const Params& P, int t, bool* ok, bool* collapsed) {
    const int4 tr = __ldg(&v.tris[t]);
    *ok = tri_valid(v.nV, tr);
    if (!*ok) return CellRange{0, -1, 0, -1, 0, -1};
    const F3 a = f3(v.pos[tr.x]), b = f3(v.pos[tr.y]), c = f3(v.pos[tr.z]);
    const float m = contact_radius(P) * 1.8f;
    const F3 lo{fminf(a.x, fminf(b.x, c.x)) - m, fminf(a.y, fminf(b.y, c.y)) - m, fminf(a.z, fminf(b.z, c.z)) - m};
    const F3 hi{fmaxf(a.x, fmaxf(b.x, c.x)) + m, fmaxf(a.y, fmaxf(b.y, c.y)) + m, fmaxf(a.z, fmaxf(b.z, c.z)) + m};
    const F3 centroid = ((a + b) + c) * (1.0f / 3.0f);
    return primitive_cells(lo, hi, centroid, P.tcell, P.key_ieee, collapsed);
}

__device__ CellRange edge_cells(const View& v, const Params& P, int e, bool* ok, bool* collapsed) {
    const int2 ed = __ldg(&v.edges[e]);
    *ok = edge_valid(v.nV, ed);
    if (!*ok) return CellRange{0, -1, 0, -1, 0, -1};
    const F3 a = f3(v.pos[ed.x]), b = f3(v.pos[ed.y]);
    const float m = contact_radius(P) * 1.8f;
    const F3 lo{fminf(a.x, b.x) - m, fminf(a.y, b.y) - m, fminf(a.z, b.z) - m};
    const F3 hi{fmaxf(a.x, b.x) + m, fmaxf(a.y, b.y) + m, fmaxf(a.z, b.z) + m};
    const F3 mid = (a + b) * 0.5f;
    return primitive_cells(lo, hi, mid, P.ecell, P.key_ieee, collapsed);
}

__global__ void k_vhash_count(View v) {
    const int i = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= v.hi) return;
    const Params& P = params_v(v, i);
    if (!P.vhash || !self_scheduled(P, v)) return;
    const float4 p = v.pos[i];
    const int cx = cell_of(p.x, P.vcell, P.key_ieee), cy = cell_of(p.y, P.vcell, P.key_ieee), cz = cell_of(p.z, P.vcell, P.key_ieee);
    const int b = P.vbase + (int)bucket_of(cx, cy, cz, P.vbuckets);
    v.vcell[i] = make_int4(cx, cy, cz, b);
    atomicAdd(&v.vb_count[b], 1);  // overflow past 32 slots is counted from the totals in the scan
}

__global__ void k_vhash_scatter(View v) {
    const int i = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= v.hi) return;
    const Params& P = params_v(v, i);
    if (!P.vhash || !self_scheduled(P, v)) return;
    const int b = v.vcell[i].w;
    v.vb_ent[atomicAdd(&v.vb_count[b], 1)] = i;
}

// Triangle hash.  L threads per triangle (1, 2, 4, 8 or 16, a tile choice of
// the autotuner): thread r of triangle k walks the x rows r, r + L, ... of
// its cell box (at most 64 cells; rows indexed over (y, z)), so the cell
// coordinates come from one division per row rather than per cell.
// `scatter` = false counts entries per bucket; true writes them through the
// cursors left by the scan.  Entry order within a bucket is fixed afterwards
// by k_bucket_sort where a query depends on it.  Collapsed ranges are counted
// as guard events in the count pass, once per triangle: a ballot per warp, a
// sum per block (every thread reaches both).  Eight blocks per SM (32
// registers): the passes wait on their atomics (batch256 triangle hash 2.21
// -> 2.15 ms per frame).
template <int L>
__global__ void __launch_bounds__(kThreads, 8) k_tri_hash(View v, bool scatter) {
    __shared__ unsigned collapsed_s;  // the block's collapsed ranges: one global atomic per block
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = v.lo + (int)(t / L), r0 = (int)(t % L);
    if (threadIdx.x == 0) collapsed_s = 0u;
    __syncthreads();
    bool collapsed = false;
    if (k < v.hi) {
        const Params& P = params_t(v, k);
        if (P.thash && self_scheduled(P, v)) {
            bool ok = false;
            const CellRange r = tri_cells(v, P, k, &ok, &collapsed);
            const int nx = r.x1 - r.x0 + 1, ny = r.y1 - r.y0 + 1, nz = r.z1 - r.z0 + 1;
            if (ok && nx > 0 && ny > 0 && nz > 0) {
                for (int row = r0; row < ny * nz; row += L) {
                    const int y = r.y0 + row % ny, z = r.z0 + row / ny;
                    for (int x = r.x0; x <= r.x1; ++x) {
                        int* slot_counter = &v.tb_count[P.tbase + (int)bucket_of(x, y, z, P.tbuckets)];
                        if (scatter)
                            v.tb_ent[atomicAdd(slot_counter, 1)] = k;
                        else
                            atomicAdd(slot_counter, 1);  // no return value needed: a reduction
                    }
                }
            }
        }
    }
    if (!scatter) {
        const unsigned m = __ballot_sync(0xffffffffu, collapsed && r0 == 0);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(&collapsed_s, (unsigned)__popc(m));
        __syncthreads();
        if (threadIdx.x == 0 && collapsed_s) count_add(v.counts, kCntSelfOverflow, (unsigned long long)collapsed_s);
    }
}

// Exclusive scan of counts[0..n) into start[0..n] in three launches: block
// sums of 4096-count tiles, a scan of the block sums, then each tile's local
// scan plus its offset.  counts is overwritten with the starts so it serves
// as the scatter cursor.
constexpr int kScanTile = 4096;

__device__ __forceinline__ int block_exclusive_scan4(int (&vals)[4], int* warp_sums, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int local = vals[0] + vals[1] + vals[2] + vals[3];
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    *total = warp_sums[nw - 1];
    const int before = (wid > 0 ? warp_sums[wid - 1] : 0) + incl - local;
    __syncthreads();
    return before;
}

// Four consecutive counters from `base` (zero past n): one int4 load when
// the array is 16-byte aligned and the quad lies inside it (base is a
// multiple of 4).
__device__ __forceinline__ void load_quad(const int* a, int base, int n, int (&vals)[4]) {
    if (base + 3 < n && (reinterpret_cast<uintptr_t>(a) & 15u) == 0u) {
        const int4 q = *reinterpret_cast<const int4*>(a + base);
        vals[0] = q.x;
        vals[1] = q.y;
        vals[2] = q.z;
        vals[3] = q.w;
    } else {
        for (int k = 0; k < 4; ++k) vals[k] = base + k < n ? a[base + k] : 0;
    }
}

__device__ __forceinline__ void store_quad(int* a, int base, int n, const int (&vals)[4]) {
    if (base + 3 < n && (reinterpret_cast<uintptr_t>(a) & 15u) == 0u) {
        *reinterpret_cast<int4*>(a + base) = make_int4(vals[0], vals[1], vals[2], vals[3]);
    } else {
        for (int k = 0; k < 4; ++k)
            if (base + k < n) a[base + k] = vals[k];
    }
}

// Also adds the number of insertions past each bucket's 32 query slots,
// sum(max(0, count - 32)), to the overflow counter (the reference counts an
// overflow for every insertion that finds its bucket full, abi41.cu:4569).
// Buckets of more than 32 members are listed in `trim` (when given) for
// k_bucket_trim.
__global__ void __launch_bounds__(1024) k_scan_reduce(const int* counts, int n, int* block_sums,
                                                      unsigned long long* overflow, int* trim, int* trim_count) {
    __shared__ int ws[32];
    int vals[4];
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    int over = 0;
    load_quad(counts, base, n, vals);
    for (int k = 0; k < 4; ++k) {
        over += vals[k] > kBucketSlots ? vals[k] - kBucketSlots : 0;
        if (trim && vals[k] > kBucketSlots) trim[atomicAdd(trim_count, 1)] = base + k;
    }
    for (int o = 16; o > 0; o >>= 1) over += __shfl_down_sync(0xffffffffu, over, o);
    if (overflow && (threadIdx.x & 31) == 0 && over > 0) atomicAdd(overflow, (unsigned long long)over);
    int total;
    block_exclusive_scan4(vals, ws, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Exclusive scan of the block sums in place (one block, any count).
__global__ void __launch_bounds__(1024) k_scan_sums(int* sums, int n) {
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += kScanTile) {
        int vals[4];
        const int i0 = base + threadIdx.x * 4;
        for (int k = 0; k < 4; ++k) vals[k] = i0 + k < n ? sums[i0 + k] : 0;
        int total;
        int run = carry + block_exclusive_scan4(vals, ws, &total);
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) sums[i0 + k] = run;
            run += vals[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) k_scan_down(int* counts, int* start, int n, const int* block_offsets) {
    __shared__ int ws[32];
    int vals[4];
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    load_quad(counts, base, n, vals);
    int total;
    int run = block_offsets[blockIdx.x] + block_exclusive_scan4(vals, ws, &total);
    int starts[4];
    for (int k = 0; k < 4; ++k) {
        starts[k] = run;
        run += vals[k];
    }
    store_quad(start, base, n, starts);
    store_quad(counts, base, n, starts);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) start[n] = run;
}

void scan_counts(int* counts, int* start, int n, int* block_sums, unsigned long long* overflow, cudaStream_t s,
                 int* trim = nullptr, int* trim_count = nullptr) {
    const int blocks = (n + kScanTile - 1) / kScanTile;
    k_scan_reduce<<<blocks, 1024, 0, s>>>(counts, n, block_sums, overflow, trim, trim_count);
    k_scan_sums<<<1, 1024, 0, s>>>(block_sums, blocks);
    k_scan_down<<<blocks, 1024, 0, s>>>(counts, start, n, block_sums);
}

__device__ __forceinline__ int warp_global_id() { return (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); }

// ------------------------------------------------- edge hash (slotted) --
// The edge hash keeps each bucket's members in kEdgeSlots slots of its own
// (bucket b's at b * kEdgeSlots), filled in a single pass: an insertion takes
// the next slot from the bucket's counter, so the counts come from the same
// atomics that place the members, with no count pass and no scan.  A bucket
// whose count passes the 32 query slots is listed for ordering (its 32
// smallest ids first, in increasing order: queries read no further); one that
// passes kEdgeSlots is listed as an overflow, and its full member list is
// gathered into a region of its own (a fold or crumple that packs more than
// 64 edge boxes into one bucket): its slot members plus the insertions past
// them, which the insertion records as (bucket, edge); only when that record
// fills up are the cells walked a second time instead.
// Every insertion past the 32 query slots counts as an overflow guard event,
// as the reference counts an insertion into a full bucket (abi41.cu:5584-
// 5590), and so does a collapsed cell range.  Members end up where the
// reference's 32 slots would hold the same multiset whenever no bucket
// passes 32 (abi41.cu:5532-5593).

// Walks edge k's cells (rows r0, r0 + L, ... of its box) and calls f(bucket)
// for each; nothing when the edge is not hashed in this substep or pass.
template <int L, class F>
__device__ __forceinline__ void edge_cells_walk(const View& v, int k, int r0, bool* collapsed, F&& f) {
    const Params& P = params_e(v, k);
    if (!P.ehash || !self_scheduled(P, v)) return;
    bool ok = false;
    const CellRange r = edge_cells(v, P, k, &ok, collapsed);
    const int nx = r.x1 - r.x0 + 1, ny = r.y1 - r.y0 + 1, nz = r.z1 - r.z0 + 1;
    if (!ok || nx <= 0 || ny <= 0 || nz <= 0) return;
    for (int row = r0; row < ny * nz; row += L) {
        const int y = r.y0 + row % ny, z = r.z0 + row / ny;
        for (int x = r.x0; x <= r.x1; ++x) f(P.ebase + (int)bucket_of(x, y, z, P.ebuckets));
    }
}

// The same walk, handing the cells of a row to f four at a time (f(b, n):
// buckets b[0..n) in walk order), so an insertion can have four atomics in
// flight before it uses their results.
template <int L, class F>
__device__ __forceinline__ void edge_cells_walk4(const View& v, int k, int r0, bool* collapsed, F&& f) {
    const Params& P = params_e(v, k);
    if (!P.ehash || !self_scheduled(P, v)) return;
    bool ok = false;
    const CellRange r = edge_cells(v, P, k, &ok, collapsed);
    const int nx = r.x1 - r.x0 + 1, ny = r.y1 - r.y0 + 1, nz = r.z1 - r.z0 + 1;
    if (!ok || nx <= 0 || ny <= 0 || nz <= 0) return;
    for (int row = r0; row < ny * nz; row += L) {
        const int y = r.y0 + row % ny, z = r.z0 + row / ny;
        for (int x = r.x0; x <= r.x1; x += 4) {
            int b[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = P.ebase + (int)bucket_of(x + j, y, z, P.ebuckets);
            f(b, min(4, r.x1 - x + 1));
        }
    }
}

template <int L>
__global__ void __launch_bounds__(kThreads) k_edge_insert(View v) {
    __shared__ unsigned guard_s;  // the block's guard events: one global atomic per block
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = v.lo + (int)(t / L), r0 = (int)(t % L);
    if (threadIdx.x == 0) guard_s = 0u;
    __syncthreads();
    bool collapsed = false;
    unsigned past = 0u;
    if (k < v.hi) {
        edge_cells_walk4<L>(v, k, r0, &collapsed, [&](const int (&bs)[4], int n) {
            int slots[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) slots[j] = j < n ? atomicAdd(&v.eb_count[bs[j]], 1) : 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j >= n) continue;
                const int b = bs[j], slot = slots[j];
                if (slot < kEdgeSlots) v.eb_slot[edge_bucket_base(b) + slot] = k;
                if (slot >= kBucketSlots) {
                    ++past;
                    if (slot == kBucketSlots) v.trim_list[atomicAdd(v.trim_count, 1)] = b;
                    if (slot == kEdgeSlots) {
                        v.eb_ovf_list[atomicAdd(v.eb_ovf_count, 1)] = b;
                        atomicOr(&v.eb_ovf_bits[b >> 5], 1u << (b & 31));
                    }
                    if (slot >= kEdgeSlots) {
                        const unsigned long long q = atomicAdd(v.eb_late_count, 1ull);
                        if (q < (unsigned long long)v.eb_late_cap) v.eb_late[q] = make_int2(b, k);
                    }
                }
            }
        });
    }
    const unsigned events = __reduce_add_sync(0xffffffffu, past + ((collapsed && r0 == 0) ? 1u : 0u));
    if ((threadIdx.x & 31) == 0 && events) atomicAdd(&guard_s, events);
    __syncthreads();
    if (threadIdx.x == 0 && guard_s) count_add(v.counts, kCntSelfOverflow, (unsigned long long)guard_s);
}

// Whether every insertion past the slots was recorded in eb_late.
__device__ __forceinline__ bool edge_late_complete(const View& v) {
    return *v.eb_late_count <= (unsigned long long)v.eb_late_cap;
}

// Overflow regions: each listed bucket gets [start, start + count) of eb_ent,
// in list order (start also kept in eb_ovf_start); eb_start[b] then serves as
// the region's fill cursor, past the kEdgeSlots members the slots hold when
// the late insertions were all recorded.  One block; nothing to do in the
// usual build without overflow.
__global__ void __launch_bounds__(1024) k_edge_ovf_offsets(View v) {
    __shared__ int ws[32];
    __shared__ int carry;
    const int n = *v.eb_ovf_count;
    if (n == 0) return;
    const int skip = edge_late_complete(v) ? kEdgeSlots : 0;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += kScanTile) {
        int vals[4];
        const int i0 = base + threadIdx.x * 4;
        for (int q = 0; q < 4; ++q) vals[q] = i0 + q < n ? v.eb_count[v.eb_ovf_list[i0 + q]] : 0;
        int total;
        int run = carry + block_exclusive_scan4(vals, ws, &total);
        for (int q = 0; q < 4; ++q) {
            if (i0 + q < n) {
                v.eb_start[v.eb_ovf_list[i0 + q]] = run + skip;
                v.eb_ovf_start[i0 + q] = run;
            }
            run += vals[q];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

// Overflow regions from what the insertion kept: each listed bucket's
// kEdgeSlots slot members, then its recorded late insertions through the
// region's fill cursor.  A fixed grid striding over both; nothing to do
// without overflow, or when the late insertions did not all fit (the second
// walk below fills the regions then).
__global__ void __launch_bounds__(kThreads) k_edge_ovf_late(View v) {
    const int n = *v.eb_ovf_count;
    if (n == 0 || !edge_late_complete(v)) return;
    const long long threads = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long t = t0; t < (long long)n * kEdgeSlots; t += threads) {
        const int w = (int)(t / kEdgeSlots), i = (int)(t % kEdgeSlots);
        v.eb_ent[v.eb_ovf_start[w] + i] = v.eb_slot[edge_bucket_base(v.eb_ovf_list[w]) + i];
    }
    const long long late = (long long)*v.eb_late_count;
    for (long long t = t0; t < late; t += threads) {
        const int2 e = v.eb_late[t];
        v.eb_ent[atomicAdd(&v.eb_start[e.x], 1)] = e.y;
    }
}

// Second walk, only when some bucket overflowed and its late insertions were
// not all recorded: every insertion into an overflowing bucket is written to
// that bucket's region.  A fixed grid striding over the edges, so the usual
// build pays for a few hundred blocks that exit at once.
template <int L>
__global__ void __launch_bounds__(kThreads) k_edge_ovf_collect(View v) {
    if (*v.eb_ovf_count == 0 || edge_late_complete(v)) return;
    const long long threads = (long long)gridDim.x * blockDim.x;
    const long long items = (long long)(v.hi - v.lo) * L;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < items; t += threads) {
        const int k = v.lo + (int)(t / L), r0 = (int)(t % L);
        bool collapsed = false;
        edge_cells_walk<L>(v, k, r0, &collapsed, [&](int b) {
            if ((__ldg(&v.eb_ovf_bits[b >> 5]) >> (b & 31)) & 1u) v.eb_ent[atomicAdd(&v.eb_start[b], 1)] = k;
        });
    }
}

// The 32 smallest ids (with multiplicity) of each overflowing bucket's region,
// in increasing order, into its first 32 slots: one warp per bucket, 32
// rounds of a warp-wide minimum above the last value taken.
__global__ void __launch_bounds__(kThreads) k_edge_ovf_select(View v) {
    const int lane = threadIdx.x & 31;
    const int warps = (int)((gridDim.x * (long long)blockDim.x) >> 5);
    const int total = *v.eb_ovf_count;
    for (int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); w < total; w += warps) {
        const int b = v.eb_ovf_list[w];
        const int n = v.eb_count[b];
        const int* e = v.eb_ent + (v.eb_start[b] - n);
        int* out = v.eb_slot + edge_bucket_base(b);
        long long last = -1;  // ids are >= 0
        int filled = 0;
        while (filled < kBucketSlots) {
            int best = 0x7fffffff, mult = 0;
            for (int i = lane; i < n; i += 32) {
                const int id = e[i];
                if ((long long)id > last) {
                    if (id < best) {
                        best = id;
                        mult = 1;
                    } else if (id == best) {
                        ++mult;
                    }
                }
            }
            const int m = __reduce_min_sync(0xffffffffu, best);
            if (m == 0x7fffffff) break;
            const int c = __reduce_add_sync(0xffffffffu, best == m ? mult : 0);
            for (int q = lane; q < c && filled + q < kBucketSlots; q += 32) out[filled + q] = m;
            filled += c;
            last = m;
            __syncwarp();
        }
    }
}

// Buckets of 33 to kEdgeSlots members (listed by the insertion): all members
// sorted by id in place, so the 32 smallest come first.  One warp per bucket,
// two members per lane ranked against all members (ties by slot).
__global__ void __launch_bounds__(kThreads) k_edge_trim(View v) {
    const int lane = threadIdx.x & 31;
    const int warps = (int)((gridDim.x * (long long)blockDim.x) >> 5);
    const int total = *v.trim_count;
    for (int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); w < total; w += warps) {
        const int b = v.trim_list[w];
        const int n = v.eb_count[b];
        if (n > kEdgeSlots) continue;  // ordered by k_edge_ovf_select
        int* e = v.eb_slot + edge_bucket_base(b);
        const int k0 = lane < n ? e[lane] : 0x7fffffff, k1 = lane + 32 < n ? e[lane + 32] : 0x7fffffff;
        int r0 = 0, r1 = 0;
        for (int j = 0; j < 32; ++j) {
            const int a = __shfl_sync(0xffffffffu, k0, j), c = __shfl_sync(0xffffffffu, k1, j);
            r0 += (a < k0 || (a == k0 && j < lane)) ? 1 : 0;
            r0 += (c < k0) ? 1 : 0;  // slot j + 32 comes after slot lane
            r1 += (a <= k1) ? 1 : 0;  // slot j comes before slot lane + 32
            r1 += (c < k1 || (c == k1 && j < lane)) ? 1 : 0;
        }
        __syncwarp();
        if (lane < n) e[r0] = k0;
        if (lane + 32 < n) e[r1] = k1;
        __syncwarp();
    }
}


// Whether a cloth's queries depend on the order of a bucket's members: fast
// mode (order-dependent filters) or a candidate budget under 32.  Strict
// queries with a 32-candidate budget read every member of a bucket of up to
// 32 and sum their pushes in fixed point, so its order cannot change them.
__device__ __forceinline__ bool bucket_order_needed(const Params& P) {
    const int budget = min(max(P.max_neighbors, 1), kBucketSlots);
    return fast_mode(P) || budget < kBucketSlots;
}

// Sort e[0..n) (n <= N) in registers: bitonic network over N, padded with
// INT_MAX.
template <int N>
__device__ __forceinline__ void sort_small(int* e, int n) {
    int r[N];
#pragma unroll
    for (int k = 0; k < N; ++k) r[k] = k < n ? e[k] : 0x7fffffff;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const int l = k ^ stride;
                if (l > k) {
                    const int lo = min(r[k], r[l]), hi = max(r[k], r[l]);
                    const bool up = (k & size) == 0;
                    r[k] = up ? lo : hi;
                    r[l] = up ? hi : lo;
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (k < n) e[k] = r[k];
}

// sort_small for a bucket of the slotted edge hash: its slot block is
// 256-byte aligned and always holds kEdgeSlots ints, so the members are read
// as whole int4 quads (slots past n hold stale ids and are replaced by the
// padding) and whole quads are written back.
template <int N>
__device__ __forceinline__ void sort_small_slots(int* e, int n) {
    int r[N];
    const int4* q4 = reinterpret_cast<const int4*>(e);
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
        int4 t = make_int4(0, 0, 0, 0);
        if (4 * q < n) t = q4[q];
        r[4 * q] = t.x;
        r[4 * q + 1] = t.y;
        r[4 * q + 2] = t.z;
        r[4 * q + 3] = t.w;
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (k >= n) r[k] = 0x7fffffff;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const int l = k ^ stride;
                if (l > k) {
                    const int lo = min(r[k], r[l]), hi = max(r[k], r[l]);
                    const bool up = (k & size) == 0;
                    r[k] = up ? lo : hi;
                    r[l] = up ? hi : lo;
                }
            }
        }
    }
    int4* w4 = reinterpret_cast<int4*>(e);
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
        if (4 * q + 3 < n) {
            w4[q] = make_int4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
        } else {
#pragma unroll
            for (int k = 4 * q; k < 4 * q + 4; ++k)
                if (k < n) e[k] = r[k];
        }
    }
}

// Order bucket members by primitive id.  One warp per 32 consecutive buckets:
// each lane sorts its own bucket of up to 16 members in registers (bitonic
// network over 8, or 16 when a bucket of the warp needs it, padded with
// INT_MAX); a bucket of 17-32 members is sorted
// by the whole warp (each lane ranks one member against all others with
// shuffles); a larger one gets its 32 smallest ids moved to the front in
// order (queries read no further).
// `mode`: 0 order only buckets of more than 32, 1 order every bucket, 2 ask
// the cloth of the bucket's first member (bucket_order_needed), 3 order the
// buckets of up to 32 (k_bucket_trim has ordered the larger ones).  `kind`:
// 1 triangle, 2 edge buckets (for mode 2).
__global__ void __launch_bounds__(kThreads) k_bucket_sort(View v, const int* start, int* ent, int nbuckets, int kind,
                                                          int mode) {
    const int warp = warp_global_id();
    const int lane = threadIdx.x & 31;
    if (v.lo + (long long)warp * 32 >= v.hi || v.hi > nbuckets) return;
    const int b = v.lo + warp * 32 + lane;
    long long s = 0;  // first member: a CSR start, or the edge hash's slots (start == null)
    int n = 0;
    if (b < v.hi) {
        s = start ? start[b] : edge_bucket_base(b);
        n = start ? start[b + 1] - (int)s : v.eb_count[b];
    }
    bool need = n > kBucketSlots && mode != 3;
    if (n >= 2 && n <= kBucketSlots) {
        if (mode == 1 || mode == 3) {
            need = true;
        } else if (mode == 2) {
            const int first = ent[s];
            need = bucket_order_needed(kind == 1 ? params_t(v, first) : params_e(v, first));
        }
    }
    constexpr int kSmall = 16;
    const bool small = need && n <= kSmall;
    // the network size follows the warp's largest small bucket (8 or 16)
    if (__any_sync(0xffffffffu, small && n > 8)) {
        if (small && start) sort_small<16>(ent + s, n);
        if (small && !start) sort_small_slots<16>(ent + s, n);
    } else if (small) {
        if (start)
            sort_small<8>(ent + s, n);
        else
            sort_small_slots<8>(ent + s, n);
    }
    if (small) need = false;
    unsigned mask = __ballot_sync(0xffffffffu, need);
    while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        const long long sj = __shfl_sync(0xffffffffu, s, j);
        const int nj = __shfl_sync(0xffffffffu, n, j);
        int* e = ent + sj;
        if (nj <= kBucketSlots) {
            const int key = lane < nj ? e[lane] : 0x7fffffff;
            int rank = 0;
            for (int k = 0; k < 32; ++k) {
                const int o = __shfl_sync(0xffffffffu, key, k);
                rank += (o < key || (o == key && k < lane)) ? 1 : 0;
            }
            __syncwarp();
            if (lane < nj) e[rank] = key;
        } else if (lane == 0) {
            for (int i = 0; i < kBucketSlots; ++i) {
                int best = i;
                for (int q = i + 1; q < nj; ++q)
                    if (e[q] < e[best]) best = q;
                const int t = e[i];
                e[i] = e[best];
                e[best] = t;
            }
        }
        __syncwarp();
    }
}

// The listed buckets (more than 32 members) are put in increasing id order,
// so the 32 slots a query reads hold the bucket's 32 smallest ids.  One warp
// per bucket over a fixed grid: each lane ranks up to 8 members against all
// members (ties by position) and the warp writes them back by rank; larger
// buckets fall back to one lane selecting the 32 smallest.
constexpr int kTrimPerLane = 8;

__global__ void __launch_bounds__(kThreads) k_bucket_trim(const int* start, int* ent, const int* list, const int* count) {
    const int lane = threadIdx.x & 31;
    const int warps = (int)((gridDim.x * (long long)blockDim.x) >> 5);
    const int total = *count;
    for (int w = warp_global_id(); w < total; w += warps) {
        const int b = list[w];
        const int s = start[b], n = start[b + 1] - s;
        int* e = ent + s;
        if (n <= 32 * kTrimPerLane) {
            int key[kTrimPerLane], rank[kTrimPerLane];
#pragma unroll
            for (int q = 0; q < kTrimPerLane; ++q) {
                const int i = lane + 32 * q;
                key[q] = i < n ? e[i] : 0;
                rank[q] = 0;
                if (i < n)
                    for (int j = 0; j < n; ++j) {
                        const int o = e[j];
                        rank[q] += (o < key[q] || (o == key[q] && j < i)) ? 1 : 0;
                    }
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q < kTrimPerLane; ++q)
                if (lane + 32 * q < n) e[rank[q]] = key[q];
        } else if (lane == 0) {
            for (int i = 0; i < kBucketSlots; ++i) {
                int best = i;
                for (int q = i + 1; q < n; ++q)
                    if (e[q] < e[best]) best = q;
                const int t = e[i];
                e[i] = e[best];
                e[best] = t;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------- neighbour table --
// Rest-distance exclusion plus onset test on the current or previous
// positions (abi41.cu:4696-4717).
__device__ bool vv_valid(const View& v, int src, int other, float target, float onset) {
    if (src < 0 || other < 0 || src >= v.nV || other >= v.nV || src == other || target <= 0.0f || onset <= target ||
        !(__ldg(&v.inv_mass[src]) > 0.0f))
        return false;
    const F3 rd = f3(ld4(&v.rest[src])) - f3(ld4(&v.rest[other]));
    const float skip = fmaxf(onset * 1.25f, target * 2.5f);
    if (dot3(rd, rd) < skip * skip) return false;
    const F3 cd = f3(v.pos[src]) - f3(v.pos[other]);
    const F3 pd = f3(v.prev[src]) - f3(v.prev[other]);
    return dot3(cd, cd) < onset * onset || dot3(pd, pd) < onset * onset;
}

// Neighbour table without the vertex hash (cloths under 128 vertices): every
// vertex of the cloth in index order (abi41.cu:4790-4814).
__global__ void k_neighbors_brute(View v, int mode) {
    const int src = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (src >= v.hi) return;
    const Params& P = params_v(v, src);
    if (P.vhash || !self_scheduled(P, v) || (mode == 1 && !fast_mode(P)) || (mode == 2 && fast_mode(P))) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) {
        v.nb_count[src] = 0;
        return;
    }
    const float onset = fmaxf(target * 1.8f, target + kEps);
    int accepted = 0;
    for (int other = P.vstart; other < P.vstart + P.V && accepted < kNeighborSlots; ++other) {
        if (!vv_valid(v, src, other, target, onset)) continue;
        v.nb_idx[src * kNeighborSlots + accepted++] = other;
    }
    if (accepted >= kNeighborSlots) count1(v.counts, kCntSelfOverflow);
    v.nb_count[src] = accepted;
}

// -------------------------------------------------------- VV repulsion --
// Swept-sphere time of impact between the two vertices' prev->current paths,
// else an overlap push; responses clamped to 0.35 thickness
// (abi41.cu:4816-4951).
__global__ void __launch_bounds__(kThreads, 6) k_vv(View v) {
    const int src = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (src >= v.hi) return;
    const Params& P = params_v(v, src);
    if (!fast_mode(P) || !self_scheduled(P, v)) return;
    if (!(__ldg(&v.inv_mass[src]) > 0.0f)) return;
    const int count = v.nb_count[src];
    if (count == 0) return;
    const F3 pc = f3(v.pos[src]), pp = f3(v.prev[src]);
    const float target = contact_radius(P);
    const float r_self = target * 0.5f;
    const int lim = min(count, kNeighborSlots);
    Clusters cl;
    cl.n = 0;
    const bool fast = fast_mode(P);
    long long ax = 0, ay = 0, az = 0, aw = 0;
    for (int n = 0; n < lim; ++n) {
        const int other = v.nb_idx[src * kNeighborSlots + n];
        if (other < 0 || other >= v.nV || other == src) continue;
        if (fast)
            count1(v.counts, kCntFilterSeen);
        else
            count1(v.counts, kCntSelfCandidates);
        const F3 qc = f3(v.pos[other]), qp = f3(v.prev[other]);
        const float th = r_self + target * 0.5f;
        if (th <= 0.0f) continue;
        const bool other_pinned = !(__ldg(&v.inv_mass[other]) > 0.0f);
        const float scale = other_pinned ? 1.0f : 0.5f;
        F3 resp{0.0f, 0.0f, 0.0f};
        bool hit = false;
        const F3 d_ref = pp - qp;
        const float cc = dot3(d_ref, d_ref) - th * th;
        const F3 rel = (pc - pp) - (qc - qp);
        const float a = dot3(rel, rel);
        const float b = dot3(d_ref, rel);
        if (cc >= 0.0f && b < 0.0f && a > 1.0e-5f) {
            const float disc = b * b - a * cc;
            if (disc >= 0.0f) {
                const float t = (-b - sqrtf(disc)) / a;
                if (t > 0.0f && t <= 1.0f) {
                    const float s = 1.0f - t;
                    const F3 ph = pp * s + pc * t;
                    const F3 qh = qp * s + qc * t;
                    F3 nrm = ph - qh;
                    const float nl = dot3(nrm, nrm);
                    if (nl > kEps) {
                        nrm = nrm * (1.0f / sqrtf(nl));
                        const float vn = dot3((pc - ph) - (qc - qh), nrm);
                        if (vn > 0.0f) {
                            resp = nrm * (-vn * scale);
                            hit = true;
                        }
                    }
                }
            }
        }
        if (!hit) {
            const F3 delta = pc - qc;
            const float dsq = dot3(delta, delta);
            if (dsq >= th * th) continue;
            F3 nrm{0.0f, 0.0f, 1.0f};
            float dist = sqrtf(fmaxf(dsq, kEps));
            if (dsq > kEps) {
                nrm = delta * (1.0f / dist);
            } else {
                const F3 rd = f3(ld4(&v.rest[src])) - f3(ld4(&v.rest[other]));
                const float rl = dot3(rd, rd);
                if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
                dist = 0.0f;
            }
            resp = nrm * fminf((th - dist) * scale, th * 0.35f);
            hit = true;
        }
        if (hit && dot3(resp, resp) > kEps) {
            const float max_len = fmaxf(th * 0.35f, 1.0e-4f);
            const float rl = len3(resp);
            if (rl > max_len) resp = resp * (max_len / rl);
            if (fast) {
                const F3 nrm = resp * (1.0f / fmaxf(len3(resp), kEps));
                const F3 mid = (pc + qc) * 0.5f;
                const unsigned key = cluster_key(0, mid, nrm, fmaxf(th * 2.5f, 1.0e-3f), P.key_ieee);
                if (!try_local_accept(v, P, 0, key, &cl)) continue;
                count1(v.counts, kCntSelfCandidates);
            }
            ax += to_fix(resp.x);
            ay += to_fix(resp.y);
            az += to_fix(resp.z);
            aw += 1;
            count1(v.counts, kCntExactImpulseContacts);
        }
    }
    if (aw) {
        unsigned long long* acc = reinterpret_cast<unsigned long long*>(&v.acc[src]);
        atomicAdd(acc + 0, (unsigned long long)ax);
        atomicAdd(acc + 1, (unsigned long long)ay);
        atomicAdd(acc + 2, (unsigned long long)az);
        atomicAdd(acc + 3, (unsigned long long)aw);
    }
}

// --------------------------------------------------------- VT repulsion --
__device__ bool rest_vt_neighbor(const View& v, int vertex, int4 t, float target, float onset) {
    if (vertex == t.x || vertex == t.y || vertex == t.z) return true;
    const F3 rp = f3(ld4(&v.rest[vertex]));
    const F3 ra = f3(ld4(&v.rest[t.x])), rb = f3(ld4(&v.rest[t.y])), rc = f3(ld4(&v.rest[t.z]));
    const float skip = fmaxf(onset * 1.25f, target * 2.5f);
    if (point_triangle_far(rp, ra, rb, rc, skip)) return false;
    const F3 rd = rp - closest_on_triangle(rp, ra, rb, rc);
    return dot3(rd, rd) < skip * skip;
}

// Soft vertex-triangle push with barycentric split (abi41.cu:4990-5107).
// Returns whether the pair counts toward the vertex's neighbour budget.
__device__ bool vt_pair(const View& v, const Params& P, int vertex, int tri, float target, float onset, Clusters* cl) {
    if (tri < 0 || tri >= v.nT || target <= 0.0f || onset <= target) return false;
    const int4 t = __ldg(&v.tris[tri]);
    if (!tri_valid(v.nV, t)) return false;
    if (rest_vt_neighbor(v, vertex, t, target, onset)) {
        filter_count(v, P, kCntFilterRejectedRest);
        return false;
    }
    const F3 p = f3(v.pos[vertex]), a = f3(v.pos[t.x]), b = f3(v.pos[t.y]), c = f3(v.pos[t.z]);
    if (point_triangle_far(p, a, b, c, onset)) return false;
    const F3 q = closest_on_triangle(p, a, b, c);
    F3 d = p - q;
    const float dsq = dot3(d, d);
    float dist = sqrtf(fmaxf(dsq, kEps));
    if (dist >= onset) return false;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = d * (1.0f / dist);
    } else {
        nrm = cross3(b - a, c - a);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 rv = f3(ld4(&v.rest[vertex]));
            const F3 rd = rv - closest_on_triangle(rv, f3(ld4(&v.rest[t.x])), f3(ld4(&v.rest[t.y])), f3(ld4(&v.rest[t.z])));
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        d = nrm * dist;
        dist = 0.0f;
    }
    if (fast_mode(P)) {
        const unsigned key = cluster_key(1, q, F3{0.0f, 0.0f, 0.0f}, fmaxf(onset * 12.0f, 1.0e-3f), P.key_ieee);
        if (!try_local_accept(v, P, 1, key, cl)) return true;
    }
    count1(v.counts, kCntSelfCandidates);
    float wa, wb, wc;
    barycentric(q, a, b, c, &wa, &wb, &wc);
    const float pen = target - dist;
    float push;
    if (pen > 0.0f) {
        push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    } else {
        const float x = 1.0f - fminf(dist / onset, 1.0f);
        push = fminf(x * x * target * 0.06f, target * 0.04f);
    }
    const float wv = __ldg(&v.inv_mass[vertex]);
    const float wta = __ldg(&v.inv_mass[t.x]) * wa;
    const float wtb = __ldg(&v.inv_mass[t.y]) * wb;
    const float wtc = __ldg(&v.inv_mass[t.z]) * wc;
    const float total = wv + wta + wtb + wtc;
    if (push <= 0.0f || total <= 0.0f) return true;
    const F3 delta = nrm * (push / total);
    if (wv > 0.0f) accumulate(v, vertex, delta * wv);
    if (wta > 0.0f) accumulate(v, t.x, delta * (-wta));
    if (wtb > 0.0f) accumulate(v, t.y, delta * (-wtb));
    if (wtc > 0.0f) accumulate(v, t.z, delta * (-wtc));
    count1(v.counts, kCntSoftContacts);
    return true;
}

__device__ int neighbor_budget(const Params& P) {
    int m = P.max_neighbors;
    if (m < 1) m = 1;
    if (m > kBucketSlots) m = kBucketSlots;
    if (fast_mode(P) && m > 16) m = 16;
    return m;
}

// Vertex-triangle query over the vertex's own cell bucket only
// (abi41.cu:5109-5182).
__global__ void __launch_bounds__(kThreads) k_vt_hash(View v) {
    const int vertex = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (vertex >= v.hi) return;
    const Params& P = params_v(v, vertex);
    if (!P.thash || !fast_mode(P) || !self_scheduled(P, v)) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) return;
    const float onset = fmaxf(target * 1.8f, target + kEps);
    const int budget = neighbor_budget(P);
    const float4 p = v.pos[vertex];
    const int b = P.tbase + (int)bucket_of(cell_of(p.x, P.tcell, P.key_ieee), cell_of(p.y, P.tcell, P.key_ieee), cell_of(p.z, P.tcell, P.key_ieee), P.tbuckets);
    const int s = v.tb_start[b];
    const int lim = min(v.tb_start[b + 1] - s, kBucketSlots);
    int accepted = 0;
    Seen seen;
    seen.n = 0;
    Clusters cl;
    cl.n = 0;
    for (int k = 0; k < lim && accepted < budget; ++k) {
        const int tri = v.tb_ent[s + k];
        if (!try_note_seen(v, P, tri, &seen)) continue;
        if (vt_pair(v, P, vertex, tri, target, onset, &cl)) ++accepted;
    }
}

// Vertex-triangle query without the triangle hash (cloths under 64
// triangles): every triangle of the cloth (abi41.cu:5184-5224).
__global__ void __launch_bounds__(kThreads) k_vt_brute(View v) {
    const int vertex = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (vertex >= v.hi) return;
    const Params& P = params_v(v, vertex);
    if (P.thash || P.T <= 0 || !self_scheduled(P, v)) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) return;
    const float onset = fmaxf(target * 1.8f, target + kEps);
    const int budget = neighbor_budget(P);
    Clusters cl;
    cl.n = 0;
    int accepted = 0;
    for (int tri = P.tstart; tri < P.tstart + P.T && accepted < budget; ++tri) {
        if (!try_note_seen(v, P, tri, nullptr)) continue;
        if (vt_pair(v, P, vertex, tri, target, onset, &cl)) ++accepted;
    }
}

// --------------------------------------------------------- EE repulsion --
__device__ bool rest_ee_neighbor(const View& v, int2 ea, int2 eb, float target, float onset) {
    if (ea.x == eb.x || ea.x == eb.y || ea.y == eb.x || ea.y == eb.y) return true;
    const F3 a0 = f3(ld4(&v.rest[ea.x])), a1 = f3(ld4(&v.rest[ea.y]));
    const F3 b0 = f3(ld4(&v.rest[eb.x])), b1 = f3(ld4(&v.rest[eb.y]));
    const float skip = fmaxf(onset * 1.25f, target * 2.5f);
    if (segments_far(a0, a1, b0, b1, skip)) return false;
    float s, t;
    segment_params(a0, a1, b0, b1, &s, &t);
    const F3 d = (a0 + (a1 - a0) * s) - (b0 + (b1 - b0) * t);
    return dot3(d, d) < skip * skip;
}

// Soft edge-edge push split by the closest-point parameters
// (abi41.cu:5595-5722).
__device__ bool ee_pair(const View& v, const Params& P, int ia, int ib, float target, float onset, Clusters* cl) {
    if (ib <= ia || ia < 0 || ib < 0 || ia >= v.nE || ib >= v.nE || target <= 0.0f || onset <= target) return false;
    const int2 ea = __ldg(&v.edges[ia]), eb = __ldg(&v.edges[ib]);
    if (!edge_valid(v.nV, ea) || !edge_valid(v.nV, eb)) return false;
    if (rest_ee_neighbor(v, ea, eb, target, onset)) {
        filter_count(v, P, kCntFilterRejectedRest);
        return false;
    }
    const F3 a0 = f3(v.pos[ea.x]), a1 = f3(v.pos[ea.y]), b0 = f3(v.pos[eb.x]), b1 = f3(v.pos[eb.y]);
    if (segments_far(a0, a1, b0, b1, onset)) return false;
    float s, t;
    segment_params(a0, a1, b0, b1, &s, &t);
    const F3 pa = a0 + (a1 - a0) * s;
    const F3 pb = b0 + (b1 - b0) * t;
    const F3 d = pa - pb;
    const float dsq = dot3(d, d);
    float dist = sqrtf(fmaxf(dsq, kEps));
    if (dist >= onset) return false;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = d * (1.0f / dist);
    } else {
        nrm = cross3(a1 - a0, b1 - b0);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 r0 = f3(ld4(&v.rest[ea.x])), r1 = f3(ld4(&v.rest[ea.y]));
            const F3 r2 = f3(ld4(&v.rest[eb.x])), r3 = f3(ld4(&v.rest[eb.y]));
            float rs, rt;
            segment_params(r0, r1, r2, r3, &rs, &rt);
            const F3 rd = (r0 + (r1 - r0) * rs) - (r2 + (r3 - r2) * rt);
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        dist = 0.0f;
    }
    if (fast_mode(P)) {
        const unsigned key = cluster_key(2, (pa + pb) * 0.5f, F3{0.0f, 0.0f, 0.0f}, fmaxf(onset * 12.0f, 1.0e-3f), P.key_ieee);
        if (!try_local_accept(v, P, 2, key, cl)) return true;
    }
    count1(v.counts, kCntSelfCandidates);
    const float pen = target - dist;
    float push;
    if (pen > 0.0f) {
        push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    } else {
        const float x = 1.0f - fminf(dist / onset, 1.0f);
        push = fminf(x * x * target * 0.06f, target * 0.04f);
    }
    const float ma0 = __ldg(&v.inv_mass[ea.x]), ma1 = __ldg(&v.inv_mass[ea.y]);
    const float mb0 = __ldg(&v.inv_mass[eb.x]), mb1 = __ldg(&v.inv_mass[eb.y]);
    const float ws0 = 1.0f - s, ws1 = s, wt0 = 1.0f - t, wt1 = t;
    const float wa0 = ma0 * ws0, wa1 = ma1 * ws1, wb0 = mb0 * wt0, wb1 = mb1 * wt1;
    const float total = ma0 * ws0 * ws0 + ma1 * ws1 * ws1 + mb0 * wt0 * wt0 + mb1 * wt1 * wt1;
    if (push <= 0.0f || total <= 0.0f) return true;
    const F3 delta = nrm * (push / total);
    if (wa0 > 0.0f) accumulate(v, ea.x, delta * wa0);
    if (wa1 > 0.0f) accumulate(v, ea.y, delta * wa1);
    if (wb0 > 0.0f) accumulate(v, eb.x, delta * (-wb0));
    if (wb1 > 0.0f) accumulate(v, eb.y, delta * (-wb1));
    count1(v.counts, kCntEdgeEdgeContacts);
    return true;
}


// Edge-edge query without the edge hash (cloths under 64 edges): later edges
// of the cloth (abi41.cu:5804-5844).
__global__ void __launch_bounds__(kThreads) k_ee_brute(View v) {
    const int e = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (e >= v.hi) return;
    const Params& P = params_e(v, e);
    if (P.ehash || !self_scheduled(P, v)) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) return;
    const float onset = fmaxf(target * 1.8f, target + kEps);
    const int budget = neighbor_budget(P);
    Clusters cl;
    cl.n = 0;
    int accepted = 0;
    for (int other = e + 1; other < P.estart + P.E && accepted < budget; ++other) {
        if (!try_note_seen(v, P, other, nullptr)) continue;
        if (ee_pair(v, P, e, other, target, onset, &cl)) ++accepted;
    }
}

// ------------------------------------------- warp-per-item strict queries --
// Strict mode has no order-dependent filter, so each candidate can be tested
// by its own lane: one warp per vertex (or edge), one lane per cell or
// candidate slot.  Lane order equals the reference loop order, a ballot
// prefix gives each accepted candidate its rank, and the neighbour budget
// keeps the first `budget` accepted candidates exactly as the serial loop
// does.  Fixed-point sums make the accumulation order irrelevant.


__device__ __forceinline__ long long warp_sum64(long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// VV responses (strict): lane n handles neighbour n of the source vertex.
// The responses of one strict vertex against its neighbour table (lane n:
// neighbour n); shared by k_vv_warp and the fused neighbour kernel.
// Response of strict vertex src to neighbour `other` (abi41.cu:4816-4951):
// *candidate = 1 for a valid neighbour, returns 1 with the fixed-point push in
// ax / ay / az when it makes a contact.
__device__ __forceinline__ int vv_pair(const View& v, const Params& P, int src, int other, long long* pax, long long* pay,
                                       long long* paz, int* pcandidate) {
    long long ax = 0, ay = 0, az = 0;
    int candidate = 0, contact = 0;
    if (other >= 0 && other < v.nV && other != src) {
        candidate = 1;
        const F3 pc = f3(v.pos[src]), pp = f3(v.prev[src]);
        const float target = contact_radius(P);
        const float th = target * 0.5f + target * 0.5f;
        const F3 qc = f3(v.pos[other]), qp = f3(v.prev[other]);
        if (th > 0.0f) {
            const float scale = !(__ldg(&v.inv_mass[other]) > 0.0f) ? 1.0f : 0.5f;
            F3 resp{0.0f, 0.0f, 0.0f};
            bool hit = false;
            const F3 d_ref = pp - qp;
            const float cc = dot3(d_ref, d_ref) - th * th;
            const F3 rel = (pc - pp) - (qc - qp);
            const float a = dot3(rel, rel), b = dot3(d_ref, rel);
            if (cc >= 0.0f && b < 0.0f && a > 1.0e-5f) {
                const float disc = b * b - a * cc;
                if (disc >= 0.0f) {
                    const float t = (-b - sqrtf(disc)) / a;
                    if (t > 0.0f && t <= 1.0f) {
                        const float sg = 1.0f - t;
                        const F3 ph = pp * sg + pc * t, qh = qp * sg + qc * t;
                        F3 nrm = ph - qh;
                        const float nl = dot3(nrm, nrm);
                        if (nl > kEps) {
                            nrm = nrm * (1.0f / sqrtf(nl));
                            const float vn = dot3((pc - ph) - (qc - qh), nrm);
                            if (vn > 0.0f) {
                                resp = nrm * (-vn * scale);
                                hit = true;
                            }
                        }
                    }
                }
            }
            bool skip = false;
            if (!hit) {
                const F3 delta = pc - qc;
                const float dsq = dot3(delta, delta);
                if (dsq >= th * th) {
                    skip = true;
                } else {
                    F3 nrm{0.0f, 0.0f, 1.0f};
                    float dist = sqrtf(fmaxf(dsq, kEps));
                    if (dsq > kEps) {
                        nrm = delta * (1.0f / dist);
                    } else {
                        const F3 rd = f3(ld4(&v.rest[src])) - f3(ld4(&v.rest[other]));
                        const float rl = dot3(rd, rd);
                        if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
                        dist = 0.0f;
                    }
                    resp = nrm * fminf((th - dist) * scale, th * 0.35f);
                    hit = true;
                }
            }
            if (!skip && hit && dot3(resp, resp) > kEps) {
                const float max_len = fmaxf(th * 0.35f, 1.0e-4f);
                const float rl = len3(resp);
                if (rl > max_len) resp = resp * (max_len / rl);
                ax = to_fix(resp.x);
                ay = to_fix(resp.y);
                az = to_fix(resp.z);
                contact = 1;
            }
        }
    }
    *pax = ax;
    *pay = ay;
    *paz = az;
    *pcandidate = candidate;
    return contact;
}

__device__ __forceinline__ void vv_strict_warp(const View& v, const Params& P, int src, int lane) {
    const int count = min(v.nb_count[src], kNeighborSlots);
    if (count == 0) return;
    long long ax = 0, ay = 0, az = 0;
    int candidate = 0, contact = 0;
    if (lane < count) contact = vv_pair(v, P, src, v.nb_idx[src * kNeighborSlots + lane], &ax, &ay, &az, &candidate);
    const unsigned cand_mask = __ballot_sync(0xffffffffu, candidate);
    const unsigned hit_mask = __ballot_sync(0xffffffffu, contact);
    ax = warp_sum64(ax);
    ay = warp_sum64(ay);
    az = warp_sum64(az);
    if (lane == 0) {
        if (cand_mask) count_add(v.counts, kCntSelfCandidates, __popc(cand_mask));
        if (hit_mask) {
            count_add(v.counts, kCntExactImpulseContacts, __popc(hit_mask));
            unsigned long long* acc = reinterpret_cast<unsigned long long*>(&v.acc[src]);
            atomicAdd(acc + 0, (unsigned long long)ax);
            atomicAdd(acc + 1, (unsigned long long)ay);
            atomicAdd(acc + 2, (unsigned long long)az);
            atomicAdd(acc + 3, (unsigned long long)__popc(hit_mask));
        }
    }
}


// VV responses of strict cloths whose table k_neighbors_brute built (the
// hashed ones run fused into k_neighbors_group); `all` = 1 covers every
// strict cloth.
__global__ void __launch_bounds__(kThreads, 8) k_vv_warp(View v, int all) {
    const int src = v.lo + warp_global_id();
    const int lane = threadIdx.x & 31;
    if (src >= v.hi) return;
    const Params& P = params_v(v, src);
    if (fast_mode(P) || !self_scheduled(P, v) || (!all && P.vhash)) return;
    if (!(__ldg(&v.inv_mass[src]) > 0.0f)) return;
    vv_strict_warp(v, P, src, lane);
}


// VV neighbour table (abi41.cu:4756-4781) and, with kVv (strict passes), the
// VV responses computed from it at once (the next operation on that branch;
// positions do not change in between).  G lanes per vertex (a tile choice of
// the autotuner; 32 / G vertices per warp): lane l scans cells c = l, G + l,
// ... in rounds, cell c = (dz, dy, dx) = (c/9-1, c/3%3-1, c%3-1), the
// reference's nested-loop order; each round's hits are placed after the
// earlier cells' by a prefix sum over the vertex's lanes, so the table lists
// neighbours in walk order.  The VV responses take neighbours l, G + l, ...
// and sum their fixed-point pushes.  With few lanes per vertex the
// per-vertex set-up and response arithmetic of several vertices share one
// instruction stream (the table walk is issue-bound).
template <bool kVv, int G>
__global__ void __launch_bounds__(kThreads, 8) k_neighbors_group(View v, int mode) {
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const int src = v.lo + warp_global_id() * (32 / G) + lane / G;
    bool run = src < v.hi;
    const Params* P = nullptr;
    if (run) {
        P = &params_v(v, src);
        run = P->vhash && self_scheduled(*P, v) && !(mode == 1 && !fast_mode(*P)) && !(mode == 2 && fast_mode(*P));
    }
    float target = 0.0f;
    if (run) {
        target = contact_radius(*P);
        if (target <= 0.0f) {
            if (gl == 0) v.nb_count[src] = 0;
            run = false;
        }
    }
    const float onset = fmaxf(target * 1.8f, target + kEps);
    int cx = 0, cy = 0, cz = 0;
    if (run) {
        const float4 p = v.pos[src];
        cx = cell_of(p.x, P->vcell, P->key_ieee);
        cy = cell_of(p.y, P->vcell, P->key_ieee);
        cz = cell_of(p.z, P->vcell, P->key_ieee);
    }
    int total = 0;  // neighbours of the earlier rounds (the same in the vertex's lanes)
    if (G == 1) {
        // one lane per vertex: the cells in walk order, each neighbour
        // written to the table as it is found
        for (int c = 0; c < 27 && run; ++c) {
            const int qx = cx + c % 3 - 1, qy = cy + (c / 3) % 3 - 1, qz = cz + c / 9 - 1;
            const int b = P->vbase + (int)bucket_of(qx, qy, qz, P->vbuckets);
            const int st = v.vb_start[b];
            const int lim = min(v.vb_start[b + 1] - st, kBucketSlots);
            for (int k = 0; k < lim; ++k) {
                const int other = v.vb_ent[st + k];
                const int4 oc = v.vcell[other];
                if (oc.x != qx || oc.y != qy || oc.z != qz || !vv_valid(v, src, other, target, onset)) continue;
                if (total < kNeighborSlots) v.nb_idx[src * kNeighborSlots + total] = other;
                ++total;
            }
        }
    }
    for (int c0 = 0; G > 1 && c0 < 27; c0 += G) {
        const int c = c0 + gl;
        int found[kNeighborSlots];
        int nfound = 0;
        if (run && c < 27) {
            const int qx = cx + c % 3 - 1, qy = cy + (c / 3) % 3 - 1, qz = cz + c / 9 - 1;
            const int b = P->vbase + (int)bucket_of(qx, qy, qz, P->vbuckets);
            const int st = v.vb_start[b];
            const int lim = min(v.vb_start[b + 1] - st, kBucketSlots);
            for (int k = 0; k < lim; ++k) {
                const int other = v.vb_ent[st + k];
                const int4 oc = v.vcell[other];
                if (oc.x != qx || oc.y != qy || oc.z != qz || !vv_valid(v, src, other, target, onset)) continue;
                found[nfound++] = other;
            }
        }
        int incl = nfound;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o, G);
            if (gl >= o) incl += t;
        }
        const int offset = total + incl - nfound;
        for (int k = 0; k < nfound && offset + k < kNeighborSlots; ++k) v.nb_idx[src * kNeighborSlots + offset + k] = found[k];
        total += __shfl_sync(0xffffffffu, incl, G - 1, G);
    }
    if (run && gl == 0) {
        if (total >= kNeighborSlots) count1(v.counts, kCntSelfOverflow);
        v.nb_count[src] = min(total, kNeighborSlots);
    }
    if (!kVv) return;
    __syncwarp();  // the table's writes are visible to the whole warp
    const bool vv = run && __ldg(&v.inv_mass[src]) > 0.0f;
    const int count = vv ? min(total, kNeighborSlots) : 0;
    long long ax = 0, ay = 0, az = 0;
    int candidates = 0, contacts = 0;
    for (int n = gl; n < count; n += G) {
        long long px, py, pz;
        int cand = 0;
        if (vv_pair(v, *P, src, v.nb_idx[src * kNeighborSlots + n], &px, &py, &pz, &cand)) {
            ax += px;
            ay += py;
            az += pz;
            ++contacts;
        }
        candidates += cand;
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        ax += __shfl_down_sync(0xffffffffu, ax, o, G);
        ay += __shfl_down_sync(0xffffffffu, ay, o, G);
        az += __shfl_down_sync(0xffffffffu, az, o, G);
        candidates += __shfl_down_sync(0xffffffffu, candidates, o, G);
        contacts += __shfl_down_sync(0xffffffffu, contacts, o, G);
    }
    if (vv && gl == 0) {
        if (candidates) count_add(v.counts, kCntSelfCandidates, (unsigned long long)candidates);
        if (contacts) {
            count_add(v.counts, kCntExactImpulseContacts, (unsigned long long)contacts);
            unsigned long long* acc = reinterpret_cast<unsigned long long*>(&v.acc[src]);
            atomicAdd(acc + 0, (unsigned long long)ax);
            atomicAdd(acc + 1, (unsigned long long)ay);
            atomicAdd(acc + 2, (unsigned long long)az);
            atomicAdd(acc + 3, (unsigned long long)contacts);
        }
    }
}

// A soft push of up to four vertices decided by one lane, applied after the
// budget check.
struct SoftPush {
    F3 delta;
    int idx[4];
    float w[4];
    bool apply;  // push > 0 and total > 0
};

// Strict-mode vertex-triangle pair up to the accept decision
// (abi41.cu:4990-5107 without the fast-mode filter).  The current-distance
// test runs before the rest-pose test: both only reject, and strict mode
// counts neither, so the outcome is the same.
__device__ bool vt_eval(const View& v, int vertex, int tri, float target, float onset, SoftPush* out) {
    if (tri < 0 || tri >= v.nT) return false;
    const int4 t = __ldg(&v.tris[tri]);
    if (!tri_valid(v.nV, t)) return false;
    if (vertex == t.x || vertex == t.y || vertex == t.z) return false;
    const F3 p = f3(v.pos[vertex]), a = f3(v.pos[t.x]), b = f3(v.pos[t.y]), c = f3(v.pos[t.z]);
    if (point_triangle_far(p, a, b, c, onset)) return false;
    const F3 q = closest_on_triangle(p, a, b, c);
    const F3 d = p - q;
    const float dsq = dot3(d, d);
    float dist = sqrtf(fmaxf(dsq, kEps));
    if (dist >= onset) return false;
    if (rest_vt_neighbor(v, vertex, t, target, onset)) return false;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = d * (1.0f / dist);
    } else {
        nrm = cross3(b - a, c - a);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 rv = f3(ld4(&v.rest[vertex]));
            const F3 rd = rv - closest_on_triangle(rv, f3(ld4(&v.rest[t.x])), f3(ld4(&v.rest[t.y])), f3(ld4(&v.rest[t.z])));
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        dist = 0.0f;
    }
    float wa, wb, wc;
    barycentric(q, a, b, c, &wa, &wb, &wc);
    const float pen = target - dist;
    float push;
    if (pen > 0.0f) {
        push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    } else {
        const float x = 1.0f - fminf(dist / onset, 1.0f);
        push = fminf(x * x * target * 0.06f, target * 0.04f);
    }
    const float wv = __ldg(&v.inv_mass[vertex]);
    const float wta = __ldg(&v.inv_mass[t.x]) * wa, wtb = __ldg(&v.inv_mass[t.y]) * wb, wtc = __ldg(&v.inv_mass[t.z]) * wc;
    const float total = wv + wta + wtb + wtc;
    out->apply = push > 0.0f && total > 0.0f;
    if (out->apply) {
        out->delta = nrm * (push / total);
        out->idx[0] = vertex;
        out->idx[1] = t.x;
        out->idx[2] = t.y;
        out->idx[3] = t.z;
        out->w[0] = wv;
        out->w[1] = -wta;
        out->w[2] = -wtb;
        out->w[3] = -wtc;
    }
    return true;
}

// Strict-mode edge-edge pair up to the accept decision (abi41.cu:5595-5722
// without the fast-mode filter; current distance tested before the rest
// pose, as above).
__device__ bool ee_eval(const View& v, int ia, int ib, float target, float onset, SoftPush* out) {
    if (ib <= ia || ia < 0 || ib < 0 || ia >= v.nE || ib >= v.nE) return false;
    const int2 ea = __ldg(&v.edges[ia]), eb = __ldg(&v.edges[ib]);
    if (!edge_valid(v.nV, ea) || !edge_valid(v.nV, eb)) return false;
    if (ea.x == eb.x || ea.x == eb.y || ea.y == eb.x || ea.y == eb.y) return false;
    const F3 a0 = f3(v.pos[ea.x]), a1 = f3(v.pos[ea.y]), b0 = f3(v.pos[eb.x]), b1 = f3(v.pos[eb.y]);
    if (segments_far(a0, a1, b0, b1, onset)) return false;
    float s, t;
    segment_params(a0, a1, b0, b1, &s, &t);
    const F3 pa = a0 + (a1 - a0) * s;
    const F3 pb = b0 + (b1 - b0) * t;
    const F3 d = pa - pb;
    const float dsq = dot3(d, d);
    float dist = sqrtf(fmaxf(dsq, kEps));
    if (dist >= onset) return false;
    if (rest_ee_neighbor(v, ea, eb, target, onset)) return false;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = d * (1.0f / dist);
    } else {
        nrm = cross3(a1 - a0, b1 - b0);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 r0 = f3(ld4(&v.rest[ea.x])), r1 = f3(ld4(&v.rest[ea.y]));
            const F3 r2 = f3(ld4(&v.rest[eb.x])), r3 = f3(ld4(&v.rest[eb.y]));
            float rs, rt;
            segment_params(r0, r1, r2, r3, &rs, &rt);
            const F3 rd = (r0 + (r1 - r0) * rs) - (r2 + (r3 - r2) * rt);
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        dist = 0.0f;
    }
    const float pen = target - dist;
    float push;
    if (pen > 0.0f) {
        push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    } else {
        const float x = 1.0f - fminf(dist / onset, 1.0f);
        push = fminf(x * x * target * 0.06f, target * 0.04f);
    }
    const float ma0 = __ldg(&v.inv_mass[ea.x]), ma1 = __ldg(&v.inv_mass[ea.y]);
    const float mb0 = __ldg(&v.inv_mass[eb.x]), mb1 = __ldg(&v.inv_mass[eb.y]);
    const float ws0 = 1.0f - s, ws1 = s, wt0 = 1.0f - t, wt1 = t;
    const float total = ma0 * ws0 * ws0 + ma1 * ws1 * ws1 + mb0 * wt0 * wt0 + mb1 * wt1 * wt1;
    out->apply = push > 0.0f && total > 0.0f;
    if (out->apply) {
        out->delta = nrm * (push / total);
        out->idx[0] = ea.x;
        out->idx[1] = ea.y;
        out->idx[2] = eb.x;
        out->idx[3] = eb.y;
        out->w[0] = ma0 * ws0;
        out->w[1] = ma1 * ws1;
        out->w[2] = -(mb0 * wt0);
        out->w[3] = -(mb1 * wt1);
    }
    return true;
}

// Strict VT / EE queries: a group of kQueryLanes lanes per query item walks
// the item's bucket slots in chunks of kQueryLanes, lane k of a chunk taking
// slot base + k.  Accepted pairs are ranked in slot order across the chunks
// and the first `budget` of them are taken, as when one thread walks the
// slots in order (abi41.cu:5129-5143, 5724-5758); evaluation has no side
// effects, so the walk stops once the budget is reached.  Groups of 8 keep
// most lanes busy for the typical 1-16 occupied slots and put four items'
// dependent load chains in flight per warp.
// The lanes per item (4, 8 or 16) are a tile choice of the autotuner: the
// ranking in slot order makes the outcome independent of it.  The fast EE
// query keeps groups of 8.
constexpr int kQueryLanes = 8;

template <int L = kQueryLanes>
__device__ __forceinline__ unsigned group_mask() {
    const int lane = threadIdx.x & 31;
    return ((1u << L) - 1u) << (lane & ~(L - 1));
}

// Take the accepted pairs of one chunk whose rank (after `prior` earlier
// acceptances) is within the budget: candidate counter for each, the push for
// those that have one.  Returns the group's acceptances in this chunk.
template <int L = kQueryLanes>
__device__ __forceinline__ int commit_chunk(const View& v, bool accepted, const SoftPush& sp, int prior, int budget,
                                           int contact_slot) {
    const unsigned gm = group_mask<L>();
    const int lane = threadIdx.x & 31;
    const unsigned acc_mask = __ballot_sync(gm, accepted) & gm;
    const int rank = prior + __popc(acc_mask & ((1u << lane) - 1u));
    const bool take = accepted && rank < budget;
    const bool push = take && sp.apply;
    const unsigned take_mask = __ballot_sync(gm, take) & gm;
    const unsigned push_mask = __ballot_sync(gm, push) & gm;
    if ((lane & (L - 1)) == 0) {
        if (take_mask) count_add(v.counts, kCntSelfCandidates, __popc(take_mask));
        if (push_mask) count_add(v.counts, contact_slot, __popc(push_mask));
    }
    if (push) {
        for (int k = 0; k < 4; ++k) {
            // the reference skips a vertex whose share is not positive (w > 0,
            // or -w > 0 for the far side); the sign was folded into w
            const float w = sp.w[k];
            const bool far = (contact_slot == kCntSoftContacts) ? (k > 0) : (k > 1);
            if ((far ? -w : w) > 0.0f) accumulate(v, sp.idx[k], sp.delta * w);
        }
    }
    return __popc(acc_mask);
}

template <int L = kQueryLanes>
__device__ __forceinline__ int group_item() {
    return (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) / L);
}

// Strict VT: the vertex's own cell bucket (abi41.cu:5129-5143).
template <int L>
__global__ void __launch_bounds__(kThreads, 4) k_vt_warp(View v) {
    const int vertex = v.lo + group_item<L>();
    const int gl = threadIdx.x & (L - 1);
    if (vertex >= v.hi) return;
    const Params& P = params_v(v, vertex);
    if (!P.thash || fast_mode(P) || !self_scheduled(P, v) || neighbor_budget(P) >= kBucketSlots) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) return;
    const float onset = fmaxf(target * 1.8f, target + kEps);
    const float4 p = v.pos[vertex];
    const int b = P.tbase + (int)bucket_of(cell_of(p.x, P.tcell, P.key_ieee), cell_of(p.y, P.tcell, P.key_ieee), cell_of(p.z, P.tcell, P.key_ieee), P.tbuckets);
    const int st = v.tb_start[b];
    const int lim = min(v.tb_start[b + 1] - st, kBucketSlots);
    const int budget = neighbor_budget(P);
    int prior = 0, evaluated = 0;
    for (int base = 0; base < lim && prior < budget; base += L) {
        SoftPush sp;
        sp.apply = false;
        const int slot = base + gl;
        evaluated += min(lim - base, L);
        const bool accepted = slot < lim && vt_eval(v, vertex, v.tb_ent[st + slot], target, onset, &sp);
        prior += commit_chunk<L>(v, accepted, sp, prior, budget, kCntSoftContacts);
    }
    if (v.perf && gl == 0) {
        perf_add(v.perf, kPerfVtItems, 1ull);
        perf_add(v.perf, kPerfVtSlots, (unsigned long long)evaluated);
    }
}

// Strict EE: the bucket of the edge midpoint's cell (abi41.cu:5724-5758).
template <int L>
__global__ void __launch_bounds__(kThreads, 4) k_ee_warp(View v) {
    const int e = v.lo + group_item<L>();
    const int gl = threadIdx.x & (L - 1);
    if (e >= v.hi) return;
    const Params& P = params_e(v, e);
    if (!P.ehash || fast_mode(P) || !self_scheduled(P, v) || neighbor_budget(P) >= kBucketSlots) return;
    const int2 ed = __ldg(&v.edges[e]);
    if (!edge_valid(v.nV, ed)) return;
    const float target = contact_radius(P);
    if (target <= 0.0f) return;
    const float onset = fmaxf(target * 1.8f, target + kEps);
    const F3 mid = (f3(v.pos[ed.x]) + f3(v.pos[ed.y])) * 0.5f;
    const int b = P.ebase + (int)bucket_of(cell_of(mid.x, P.ecell, P.key_ieee), cell_of(mid.y, P.ecell, P.key_ieee), cell_of(mid.z, P.ecell, P.key_ieee), P.ebuckets);
    const int* mem = v.eb_slot + edge_bucket_base(b);
    const int lim = edge_bucket_size(v, b);
    const int budget = neighbor_budget(P);
    int prior = 0, evaluated = 0, gathered = 0;
    for (int base = 0; base < lim && prior < budget; base += L) {
        SoftPush sp;
        sp.apply = false;
        const int slot = base + gl;
        evaluated += min(lim - base, L);
        const int other = slot < lim ? mem[slot] : -1;
        gathered += other > e ? 1 : 0;
        const bool accepted = slot < lim && ee_eval(v, e, other, target, onset, &sp);
        prior += commit_chunk<L>(v, accepted, sp, prior, budget, kCntEdgeEdgeContacts);
    }
    if (v.perf) {
        perf_add(v.perf, kPerfEeGathers, (unsigned long long)gathered);
        if (gl == 0) {
            perf_add(v.perf, kPerfEeItems, 1ull);
            perf_add(v.perf, kPerfEeSlots, (unsigned long long)evaluated);
        }
    }
}

// Strict VT query for cloths whose candidate budget is at least the 32 query
// slots: every accepted pair of an item's slots is taken, so the pairs are
// independent and their order does not matter (pushes are summed in fixed
// point).  One warp per 32 consecutive query vertices lays their bucket
// slots end to end and evaluates 32 (vertex, slot) pairs per round, so the
// lanes stay busy however the slot counts vary.  The same pairs, counters
// and pushes as the 8-lane group kernel, which keeps the cloths with a
// smaller budget.
__global__ void __launch_bounds__(kThreads, 6) k_flat_vt(View v) {
    const int lane = threadIdx.x & 31;
    const int item = v.lo + warp_global_id() * 32 + lane;
    int st = 0, lim = 0;
    float target = 0.0f, onset = 0.0f;
    bool counted = false;
    if (item < v.hi) {
        const Params& P = params_v(v, item);
        if (P.thash && !fast_mode(P) && self_scheduled(P, v) && neighbor_budget(P) >= kBucketSlots) {
            const F3 q = f3(v.pos[item]);
            target = contact_radius(P);
            if (target > 0.0f) {
                onset = fmaxf(target * 1.8f, target + kEps);
                const int b = P.tbase + (int)bucket_of(cell_of(q.x, P.tcell, P.key_ieee), cell_of(q.y, P.tcell, P.key_ieee),
                                                       cell_of(q.z, P.tcell, P.key_ieee), P.tbuckets);
                st = v.tb_start[b];
                lim = min(v.tb_start[b + 1] - st, kBucketSlots);
                counted = true;
            }
        }
    }
    int incl = lim;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - lim;
    unsigned takes = 0, pushes = 0;
    for (int base = 0; base < total; base += 32) {
        const int w = base + lane;
        int j = 0;  // owner: the first lane whose inclusive slot count exceeds w
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (__shfl_sync(0xffffffffu, incl, j + step - 1) <= w) j += step;
        const int o_item = __shfl_sync(0xffffffffu, item, j);
        const int o_first = __shfl_sync(0xffffffffu, st, j) - __shfl_sync(0xffffffffu, excl, j);
        const float o_target = __shfl_sync(0xffffffffu, target, j), o_onset = __shfl_sync(0xffffffffu, onset, j);
        SoftPush sp;
        sp.apply = false;
        const bool accepted = w < total && vt_eval(v, o_item, v.tb_ent[o_first + w], o_target, o_onset, &sp);
        const bool push = accepted && sp.apply;
        takes += __popc(__ballot_sync(0xffffffffu, accepted));
        pushes += __popc(__ballot_sync(0xffffffffu, push));
        if (push) {
            for (int k = 0; k < 4; ++k) {
                const float wk = sp.w[k];
                if ((k > 0 ? -wk : wk) > 0.0f) accumulate(v, sp.idx[k], sp.delta * wk);
            }
        }
    }
    const unsigned items = __popc(__ballot_sync(0xffffffffu, counted));
    if (lane == 0) {
        count_add(v.counts, kCntSelfCandidates, takes);
        count_add(v.counts, kCntSoftContacts, pushes);
        if (v.perf && items) {
            perf_add(v.perf, kPerfVtItems, (unsigned long long)items);
            perf_add(v.perf, kPerfVtSlots, (unsigned long long)total);
        }
    }
}

// Strict edge-edge query for cloths whose candidate budget covers the 32
// query slots, flattened like k_flat_vt with one more step: a pair (item a,
// candidate b) counts only when b > a (it is evaluated from its lower edge),
// which about two thirds of the bucket slots fail as soon as their id is
// read.  Round after round the warp reads 32 slot ids (the items' slots laid
// end to end), keeps the surviving pairs in a 128-entry ring in shared memory
// (owner lane, candidate), and evaluates them 32 at a time whenever 32 are
// waiting, so the evaluation rounds carry only pairs that can be taken.
// Pushes go through the integer accumulators and the counters through warp
// ballots, so the result does not depend on the order of evaluation.
constexpr int kEeRing = 128;

__global__ void __launch_bounds__(kThreads, 6) k_flat_ee(View v) {
    __shared__ int2 ring_s[kThreads / 32][kEeRing];
    const int lane = threadIdx.x & 31;
    int2* ring = ring_s[threadIdx.x >> 5];
    const int item = v.lo + warp_global_id() * 32 + lane;
    long long st = 0;
    int lim = 0;
    float target = 0.0f, onset = 0.0f;
    bool counted = false;
    if (item < v.hi) {
        const Params& P = params_e(v, item);
        bool want = P.ehash && !fast_mode(P) && self_scheduled(P, v) && neighbor_budget(P) >= kBucketSlots;
        F3 q{0.0f, 0.0f, 0.0f};
        if (want) {
            const int2 ed = __ldg(&v.edges[item]);
            want = edge_valid(v.nV, ed);
            if (want) q = (f3(v.pos[ed.x]) + f3(v.pos[ed.y])) * 0.5f;
        }
        if (want) target = contact_radius(P);
        if (want && target > 0.0f) {
            onset = fmaxf(target * 1.8f, target + kEps);
            const int b = P.ebase + (int)bucket_of(cell_of(q.x, P.ecell, P.key_ieee), cell_of(q.y, P.ecell, P.key_ieee),
                                                   cell_of(q.z, P.ecell, P.key_ieee), P.ebuckets);
            st = edge_bucket_base(b);
            lim = edge_bucket_size(v, b);
            counted = true;
        }
    }
    int incl = lim;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - lim;
    unsigned takes = 0, pushes = 0, gathers = 0;
    int head = 0, tail = 0;  // warp-uniform ring positions
    auto drain = [&](int n) {
        const int2 e = lane < n ? ring[(head + lane) & (kEeRing - 1)] : make_int2(0, -1);
        const int o_item = __shfl_sync(0xffffffffu, item, e.x);
        const float o_target = __shfl_sync(0xffffffffu, target, e.x), o_onset = __shfl_sync(0xffffffffu, onset, e.x);
        SoftPush sp;
        sp.apply = false;
        const bool accepted = lane < n && ee_eval(v, o_item, e.y, o_target, o_onset, &sp);
        const bool push = accepted && sp.apply;
        takes += __popc(__ballot_sync(0xffffffffu, accepted));
        pushes += __popc(__ballot_sync(0xffffffffu, push));
        if (push) {
            for (int k = 0; k < 4; ++k) {
                const float wk = sp.w[k];
                if ((k > 1 ? -wk : wk) > 0.0f) accumulate(v, sp.idx[k], sp.delta * wk);
            }
        }
        head += n;
        __syncwarp();
    };
    const unsigned lower = (1u << lane) - 1u;
    // Two rounds of 32 slot ids per step, both loads issued before either
    // is used; the ring holds what two rounds add to fewer than 32 waiting.
    for (int base = 0; base < total; base += 64) {
        int jr[2], other[2], owner[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int w = base + 32 * r + lane;
            int j = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, incl, j + step - 1) <= w) j += step;
            jr[r] = j;
            owner[r] = __shfl_sync(0xffffffffu, item, j);
            const long long o_first = __shfl_sync(0xffffffffu, st, j) - __shfl_sync(0xffffffffu, excl, j);
            other[r] = w < total ? v.eb_slot[o_first + w] : -1;
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const bool keep = base + 32 * r + lane < total && other[r] > owner[r];
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) ring[(tail + __popc(m & lower)) & (kEeRing - 1)] = make_int2(jr[r], other[r]);
            tail += __popc(m);
            gathers += __popc(m);
        }
        __syncwarp();
        while (tail - head >= 32) drain(32);
    }
    if (tail > head) drain(tail - head);
    const unsigned items = __popc(__ballot_sync(0xffffffffu, counted));
    if (lane == 0) {
        count_add(v.counts, kCntSelfCandidates, takes);
        count_add(v.counts, kCntEdgeEdgeContacts, pushes);
        if (v.perf && items) {
            perf_add(v.perf, kPerfEeItems, (unsigned long long)items);
            perf_add(v.perf, kPerfEeSlots, (unsigned long long)total);
            perf_add(v.perf, kPerfEeGathers, (unsigned long long)gathers);
        }
    }
}

// Fast-mode edge-edge pair as ee_pair walks it (rest test first, then the
// current distance), without the cluster filter.  Returns 0 (no pair),
// 1 (rejected by the rest pose), 2 (beyond the onset distance) or 3 (a
// candidate: *key is its cluster key, *out its push).
// kPush = false stops at the class and key (the push is left unset).
template <bool kPush = true>
__device__ int ee_fast_classify(const View& v, int ia, int ib, float target, float onset, int ieee, SoftPush* out,
                                unsigned* key) {
    if (ib <= ia || ia < 0 || ib < 0 || ia >= v.nE || ib >= v.nE || target <= 0.0f || onset <= target) return 0;
    const int2 ea = __ldg(&v.edges[ia]), eb = __ldg(&v.edges[ib]);
    if (!edge_valid(v.nV, ea) || !edge_valid(v.nV, eb)) return 0;
    if (rest_ee_neighbor(v, ea, eb, target, onset)) return 1;
    const F3 a0 = f3(v.pos[ea.x]), a1 = f3(v.pos[ea.y]), b0 = f3(v.pos[eb.x]), b1 = f3(v.pos[eb.y]);
    if (segments_far(a0, a1, b0, b1, onset)) return 2;
    float s, t;
    segment_params(a0, a1, b0, b1, &s, &t);
    const F3 pa = a0 + (a1 - a0) * s;
    const F3 pb = b0 + (b1 - b0) * t;
    const F3 d = pa - pb;
    const float dsq = dot3(d, d);
    float dist = sqrtf(fmaxf(dsq, kEps));
    if (dist >= onset) return 2;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = d * (1.0f / dist);
    } else {
        nrm = cross3(a1 - a0, b1 - b0);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 r0 = f3(ld4(&v.rest[ea.x])), r1 = f3(ld4(&v.rest[ea.y]));
            const F3 r2 = f3(ld4(&v.rest[eb.x])), r3 = f3(ld4(&v.rest[eb.y]));
            float rs, rt;
            segment_params(r0, r1, r2, r3, &rs, &rt);
            const F3 rd = (r0 + (r1 - r0) * rs) - (r2 + (r3 - r2) * rt);
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        dist = 0.0f;
    }
    *key = cluster_key(2, (pa + pb) * 0.5f, F3{0.0f, 0.0f, 0.0f}, fmaxf(onset * 12.0f, 1.0e-3f), ieee);
    if (!kPush) return 3;
    const float pen = target - dist;
    float push;
    if (pen > 0.0f) {
        push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    } else {
        const float x = 1.0f - fminf(dist / onset, 1.0f);
        push = fminf(x * x * target * 0.06f, target * 0.04f);
    }
    const float ma0 = __ldg(&v.inv_mass[ea.x]), ma1 = __ldg(&v.inv_mass[ea.y]);
    const float mb0 = __ldg(&v.inv_mass[eb.x]), mb1 = __ldg(&v.inv_mass[eb.y]);
    const float ws0 = 1.0f - s, ws1 = s, wt0 = 1.0f - t, wt1 = t;
    const float total = ma0 * ws0 * ws0 + ma1 * ws1 * ws1 + mb0 * wt0 * wt0 + mb1 * wt1 * wt1;
    out->apply = push > 0.0f && total > 0.0f;
    if (out->apply) {
        out->delta = nrm * (push / total);
        out->idx[0] = ea.x;
        out->idx[1] = ea.y;
        out->idx[2] = eb.x;
        out->idx[3] = eb.y;
        out->w[0] = ma0 * ws0;
        out->w[1] = ma1 * ws1;
        out->w[2] = -(mb0 * wt0);
        out->w[3] = -(mb1 * wt1);
    }
    return 3;
}

__device__ __forceinline__ int nth_set_bit(unsigned m, int n) {
    for (int i = 0; i < n; ++i) m &= m - 1;
    return __ffs(m) - 1;
}

// Fast-mode EE query, flattened: the same outcome as k_ee_fast.  Phase 1
// classifies every (item, slot) pair of a warp's 32 items past the item's
// own id in its ordered bucket (the earlier slots give no pair), 32 pairs per round
// with the slots of the items laid end to end (duplicate = the same id as the
// slot before; classify is side-effect free, so pairs past an item's budget
// cut may be classified for nothing); classes and cluster keys go to shared
// memory.  Phase 2 gives each lane its item and walks the slots in order:
// visited / duplicate / rest-pose counts, the budget of passing pairs, the
// cluster filter on up to 16 held keys, and for each taken pair the push,
// recomputed by the same classify call, accumulated in fixed point.
constexpr int kFastWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads, 4) k_ee_fast_flat(View v) {
    __shared__ unsigned char cls_s[kFastWarps][32 * kBucketSlots];
    __shared__ unsigned key_s[kFastWarps][32 * kBucketSlots];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int e = v.lo + warp_global_id() * 32 + lane;
    bool run = e < v.hi;
    const Params* P = nullptr;
    if (run) {
        P = &params_e(v, e);
        run = P->ehash && fast_mode(*P) && self_scheduled(*P, v);
    }
    int2 ed = make_int2(-1, -1);
    if (run) {
        ed = __ldg(&v.edges[e]);
        run = edge_valid(v.nV, ed) && contact_radius(*P) > 0.0f;
    }
    long long st = 0;
    int lim = 0, budget = 0;
    float target = 0.0f, onset = 0.0f;
    if (run) {
        target = contact_radius(*P);
        onset = fmaxf(target * 1.8f, target + kEps);
        budget = neighbor_budget(*P);
        const F3 mid = (f3(v.pos[ed.x]) + f3(v.pos[ed.y])) * 0.5f;
        const int b =
            P->ebase + (int)bucket_of(cell_of(mid.x, P->ecell, P->key_ieee), cell_of(mid.y, P->ecell, P->key_ieee), cell_of(mid.z, P->ecell, P->key_ieee), P->ebuckets);
        st = edge_bucket_base(b);
        lim = edge_bucket_size(v, b);
    }
    // A fast cloth's bucket lists its members in increasing id order, and a
    // pair is taken from its lower edge: the members up to this edge's own
    // id form a prefix whose slots are each visited (seen) and give no pair,
    // an id equal to the one before being a duplicate.  Only the slots after
    // the prefix are classified.
    int skip = 0, skip_dup = 0;
    if (run) {
        int lo = 0, hi = lim;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (v.eb_slot[st + mid] > e)
                hi = mid;
            else
                lo = mid + 1;
        }
        skip = lo;
        for (int j = 1; j < skip; ++j) skip_dup += v.eb_slot[st + j] == v.eb_slot[st + j - 1] ? 1 : 0;
    }
    const int cnt = lim - skip;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - cnt - skip;  // so that slot = w - excl starts after the prefix
    unsigned char* cls_w = cls_s[wib];
    unsigned* key_w = key_s[wib];
    for (int base = 0; base < total; base += 32) {
        const int w = base + lane;
        int j = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (__shfl_sync(0xffffffffu, incl, j + step - 1) <= w) j += step;
        const int o_item = __shfl_sync(0xffffffffu, e, j);
        const long long o_st = __shfl_sync(0xffffffffu, st, j);
        const int o_excl = __shfl_sync(0xffffffffu, excl, j);
        const float o_target = __shfl_sync(0xffffffffu, target, j), o_onset = __shfl_sync(0xffffffffu, onset, j);
        const int o_ieee = __shfl_sync(0xffffffffu, run ? P->key_ieee : 0, j);
        if (w < total) {
            const int slot = w - o_excl;
            const int id = v.eb_slot[o_st + slot];
            const bool dup = slot > 0 && id == v.eb_slot[o_st + slot - 1];
            SoftPush sp;
            sp.apply = false;
            unsigned key = 0u;
            const int cls = dup ? 4 : ee_fast_classify<false>(v, o_item, id, o_target, o_onset, o_ieee, &sp, &key);
            cls_w[j * kBucketSlots + slot] = (unsigned char)cls;
            key_w[j * kBucketSlots + slot] = key;
        }
    }
    __syncwarp();
    int c_seen = skip, c_dup = skip_dup, c_rest = 0, c_own = 0, c_acc = 0, c_contact = 0, visited = skip;
    if (run) {
        unsigned keys[16];
        int nkeys = 0, passed = 0;
        for (int slot = skip; slot < lim && passed < budget; ++slot) {
            ++visited;
            ++c_seen;
            const int cls = cls_w[lane * kBucketSlots + slot];
            if (cls == 4) {
                ++c_dup;
                continue;
            }
            if (cls == 1) ++c_rest;
            if (cls != 3) continue;
            ++passed;
            const unsigned key = key_w[lane * kBucketSlots + slot];
            bool first = true;
#pragma unroll
            for (int q = 0; q < 16; ++q) first = first && !(q < nkeys && keys[q] == key);
            if (!(first && nkeys < 16)) {
                ++c_own;
                continue;
            }
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (q == nkeys) keys[q] = key;
            ++nkeys;
            ++c_acc;
            SoftPush sp;
            sp.apply = false;
            unsigned k2 = 0u;
            ee_fast_classify(v, e, v.eb_slot[st + slot], target, onset, P->key_ieee, &sp, &k2);
            if (sp.apply) {
                ++c_contact;
                for (int k = 0; k < 4; ++k) {
                    const float wk = sp.w[k];
                    if ((k > 1 ? -wk : wk) > 0.0f) accumulate(v, sp.idx[k], sp.delta * wk);
                }
            }
        }
    }
    const int sums[6] = {c_seen, c_dup, c_rest, c_own, c_acc, c_contact};
    const int slots[6] = {kCntFilterSeen, kCntFilterRejectedDuplicate, kCntFilterRejectedRest, kCntFilterRejectedOwnership,
                          kCntFilterAcceptedEe, kCntEdgeEdgeContacts};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int t = __reduce_add_sync(0xffffffffu, sums[q]);
        if (lane == 0 && t > 0) count_add(v.counts, slots[q], (unsigned long long)t);
    }
    if (v.perf) {
        const int items = __reduce_add_sync(0xffffffffu, run ? 1 : 0);
        const int slots_total = __reduce_add_sync(0xffffffffu, visited);
        if (lane == 0) {
            perf_add(v.perf, kPerfEeItems, (unsigned long long)items);
            perf_add(v.perf, kPerfEeSlots, (unsigned long long)slots_total);
            perf_add(v.perf, kPerfEeGathers, (unsigned long long)total);
        }
    }
    const int acc_total = __reduce_add_sync(0xffffffffu, c_acc);
    if (lane == 0 && acc_total > 0) {
        count_add(v.counts, kCntClusterCount, (unsigned long long)acc_total);
        count_add(v.counts, kCntClusterOwnedContacts, (unsigned long long)acc_total);
        count_add(v.counts, kCntSelfCandidates, (unsigned long long)acc_total);
    }
}

// Fast-mode EE query in groups of kQueryLanes lanes with the exact outcome of
// the serial walk of k_ee_hash (abi41.cu:5724-5802 with the filters of
// 714-832): slots are visited in order until `budget` pairs have passed the
// distance test; a slot whose edge id appeared at an earlier slot is a
// duplicate; a passing pair is accepted when its cluster key is new and fewer
// than 16 keys are held.  Fast-mode buckets are ordered by id (k_bucket_sort
// orders every bucket of a fast cloth, and the first 32 members of larger
// ones), so a duplicate is the same id as the slot before it.  The group
// carries the accepted keys in registers (lane g holds keys g and g + 8).
// Counters are summed per warp and added once at the end.
__global__ void __launch_bounds__(kThreads, 3) k_ee_fast(View v) {
    const int e = v.lo + group_item();
    const int lane = threadIdx.x & 31;
    const int gl = lane & (kQueryLanes - 1);
    const int gbase = lane & ~(kQueryLanes - 1);
    const unsigned gm = group_mask();
    int c_seen = 0, c_dup = 0, c_rest = 0, c_own = 0, c_acc = 0, c_contact = 0;
    bool run = e < v.hi;
    const Params* P = nullptr;
    if (run) {
        P = &params_e(v, e);
        run = P->ehash && fast_mode(*P) && self_scheduled(*P, v);
    }
    int2 ed = make_int2(-1, -1);
    if (run) {
        ed = __ldg(&v.edges[e]);
        run = edge_valid(v.nV, ed) && contact_radius(*P) > 0.0f;
    }
    long long st = 0;
    int lim = 0, budget = 0;
    float target = 0.0f, onset = 0.0f;
    if (run) {
        target = contact_radius(*P);
        onset = fmaxf(target * 1.8f, target + kEps);
        budget = neighbor_budget(*P);
        const F3 mid = (f3(v.pos[ed.x]) + f3(v.pos[ed.y])) * 0.5f;
        const int b =
            P->ebase + (int)bucket_of(cell_of(mid.x, P->ecell, P->key_ieee), cell_of(mid.y, P->ecell, P->key_ieee), cell_of(mid.z, P->ecell, P->key_ieee), P->ebuckets);
        st = edge_bucket_base(b);
        lim = edge_bucket_size(v, b);
    }
    // the members up to this edge's own id (a prefix of the ordered bucket)
    // are seen and give no pair, as in k_ee_fast_flat
    int skip = 0, skip_dup = 0;
    if (run) {
        int lo = 0, hi = lim;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (v.eb_slot[st + mid] > e)
                hi = mid;
            else
                lo = mid + 1;
        }
        skip = lo;
        if (gl == 0)
            for (int j = 1; j < skip; ++j) skip_dup += v.eb_slot[st + j] == v.eb_slot[st + j - 1] ? 1 : 0;
    }
    unsigned keys[2] = {0u, 0u};
    int nkeys = 0, accepted = 0, last_id = skip > 0 ? v.eb_slot[st + skip - 1] : -1;
    int evaluated = gl == 0 ? skip : 0;
    if (gl == 0) {
        c_seen += skip;
        c_dup += skip_dup;
    }
    for (int c = 0; c < kBucketSlots / kQueryLanes; ++c) {
        if (!(run && skip + c * kQueryLanes < lim && accepted < budget)) break;  // uniform within the group
        {
            const int slot = skip + c * kQueryLanes + gl;
            const bool valid = slot < lim;
            evaluated += valid ? 1 : 0;
            const int id = valid ? v.eb_slot[st + slot] : -1;
            const int before = __shfl_sync(gm, id, gbase + ((gl + kQueryLanes - 1) & (kQueryLanes - 1)));
            const bool dup = valid && id == (gl == 0 ? last_id : before);
            last_id = __shfl_sync(gm, id, gbase + kQueryLanes - 1);
            SoftPush sp;
            sp.apply = false;
            unsigned key = 0u;
            const int cls = (valid && !dup) ? ee_fast_classify(v, e, id, target, onset, P->key_ieee, &sp, &key) : 0;
            const unsigned pass_mask = (__ballot_sync(gm, cls == 3) >> gbase) & 0xffu;
            const int remaining = budget - accepted;
            const int cut = __popc(pass_mask) >= remaining ? nth_set_bit(pass_mask, remaining - 1) : kQueryLanes;
            const bool visited = valid && gl <= cut;
            c_seen += visited ? 1 : 0;
            c_dup += (visited && dup) ? 1 : 0;
            c_rest += (visited && cls == 1) ? 1 : 0;
            const bool cand = visited && cls == 3;
            const unsigned cand_mask = (__ballot_sync(gm, cand) >> gbase) & 0xffu;
            if (cand_mask == 0u) {
                accepted += __popc(pass_mask & ((cut >= kQueryLanes) ? 0xffu : ((2u << cut) - 1u)));
                continue;
            }
            // cluster filter: new key among the held ones and the earlier
            // candidates of this chunk, while fewer than 16 keys are held
            bool first = cand;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const unsigned hk = __shfl_sync(gm, keys[j >> 3], gbase + (j & 7));
                first = first && !(j < nkeys && hk == key);
            }
#pragma unroll
            for (int j = 0; j < kQueryLanes; ++j) {
                const unsigned ok = __shfl_sync(gm, key, gbase + j);
                first = first && !(j < gl && ((cand_mask >> j) & 1u) && ok == key);
            }
            const unsigned first_mask = (__ballot_sync(gm, first) >> gbase) & 0xffu;
            const int rank = __popc(first_mask & ((1u << gl) - 1u));
            const bool take = first && nkeys + rank < 16;
            const unsigned take_mask = (__ballot_sync(gm, take) >> gbase) & 0xffu;
            c_own += (cand && !take) ? 1 : 0;
            if (take) {
                c_acc += 1;
                if (sp.apply) {
                    c_contact += 1;
                    for (int k = 0; k < 4; ++k) {
                        const float w = sp.w[k];
                        if ((k > 1 ? -w : w) > 0.0f) accumulate(v, sp.idx[k], sp.delta * w);
                    }
                }
            }
            // append the taken keys in slot order: key position q is held by
            // lane q % 8 in register q / 8
            const int ntake = __popc(take_mask);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = gl + h * kQueryLanes;
                const bool mine = q >= nkeys && q < nkeys + ntake;
                const int src = mine ? nth_set_bit(take_mask, q - nkeys) : gl;
                const unsigned got = __shfl_sync(gm, key, gbase + src);
                if (mine) keys[h] = got;
            }
            nkeys += ntake;
            accepted += __popc(pass_mask & ((cut >= kQueryLanes) ? 0xffu : ((2u << cut) - 1u)));
        }
    }
    // one atomic per counter and warp
    const int sums[6] = {c_seen, c_dup, c_rest, c_own, c_acc, c_contact};
    const int slots[6] = {kCntFilterSeen, kCntFilterRejectedDuplicate, kCntFilterRejectedRest, kCntFilterRejectedOwnership,
                          kCntFilterAcceptedEe, kCntEdgeEdgeContacts};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int total = __reduce_add_sync(0xffffffffu, sums[q]);
        if (lane == 0 && total > 0) count_add(v.counts, slots[q], (unsigned long long)total);
    }
    if (v.perf) {
        const int items = __reduce_add_sync(0xffffffffu, (run && gl == 0) ? 1 : 0);
        const int slots_total = __reduce_add_sync(0xffffffffu, evaluated);
        const int gathers = __reduce_add_sync(0xffffffffu, evaluated - (gl == 0 ? skip : 0));
        if (lane == 0) {
            perf_add(v.perf, kPerfEeItems, (unsigned long long)items);
            perf_add(v.perf, kPerfEeSlots, (unsigned long long)slots_total);
            perf_add(v.perf, kPerfEeGathers, (unsigned long long)gathers);
        }
    }
    const int acc_total = __reduce_add_sync(0xffffffffu, c_acc);
    if (lane == 0 && acc_total > 0) {
        count_add(v.counts, kCntClusterCount, (unsigned long long)acc_total);
        count_add(v.counts, kCntClusterOwnedContacts, (unsigned long long)acc_total);
        count_add(v.counts, kCntSelfCandidates, (unsigned long long)acc_total);
    }
}

// ------------------------------------------------- fast overlap islands --
// Fast mode, final pass: aggregate push for a vertex buried in >= 3 nearby
// triangles of the 27-cell neighbourhood (abi41.cu:5226-5439).
//
// One candidate slot of the walk, everything but the duplicate check: 0 =
// skipped, 1 = skipped with a guard count, 2 = a contact with its
// penetration, normal and inverse-mass term.
struct IslandHit {
    float pen, wterm;
    F3 nrm;
};

__device__ int island_eval(const View& v, int vertex, F3 p, F3 pp, float target, float onset, int tri, IslandHit* out) {
    if (tri < 0 || tri >= v.nT) return 1;
    const int4 t = __ldg(&v.tris[tri]);
    if (!tri_valid(v.nV, t)) return 0;
    // The reference tests the rest pose, then finiteness, then the current
    // distance.  Both the rest and the distance test only skip the
    // candidate, so for finite positions the (cheaper, usually failing)
    // distance test runs first; non-finite positions keep the reference
    // order, which decides the guard count.
    const F3 a = f3(v.pos[t.x]), b2 = f3(v.pos[t.y]), c = f3(v.pos[t.z]);
    const F3 ap = f3(v.prev[t.x]), bp = f3(v.prev[t.y]), cp = f3(v.prev[t.z]);
    const bool finite = finite3(a) && finite3(b2) && finite3(c) && finite3(ap) && finite3(bp) && finite3(cp);
    F3 q{0.0f, 0.0f, 0.0f};
    float dsq = 0.0f, dist = 0.0f;
    if (finite) {
        if (point_triangle_far(p, a, b2, c, target)) return 0;
        q = closest_on_triangle(p, a, b2, c);
        const F3 d0 = p - q;
        dsq = dot3(d0, d0);
        dist = sqrtf(fmaxf(dsq, kEps));
        if (dist >= target) return 0;
    }
    if (rest_vt_neighbor(v, vertex, t, target, onset)) return 0;
    if (!finite) return 1;
    F3 delta = p - q;
    F3 nrm{0.0f, 0.0f, 1.0f};
    if (dsq > kEps) {
        nrm = delta * (1.0f / dist);
    } else {
        nrm = cross3(b2 - a, c - a);
        const float nl = dot3(nrm, nrm);
        if (nl > kEps) {
            nrm = nrm * (1.0f / sqrtf(nl));
        } else {
            const F3 rv = f3(ld4(&v.rest[vertex]));
            const F3 rd = rv - closest_on_triangle(rv, f3(ld4(&v.rest[t.x])), f3(ld4(&v.rest[t.y])), f3(ld4(&v.rest[t.z])));
            const float rl = dot3(rd, rd);
            if (rl > kEps) nrm = rd * (1.0f / sqrtf(rl));
        }
        delta = nrm * dist;
        dist = 0.0f;
    }
    if (!finite3(nrm)) return 1;
    const F3 qprev = closest_on_triangle(pp, ap, bp, cp);
    const F3 pdelta = pp - qprev;
    if (dot3(pdelta, nrm) > target * 0.25f && dot3(delta, nrm) > -target * 0.10f) return 0;
    float wa, wb, wc;
    barycentric(q, a, b2, c, &wa, &wb, &wc);
    const float pen = target - dist;
    if (pen <= 0.0f) return 0;
    out->pen = pen;
    out->nrm = nrm;
    out->wterm = __ldg(&v.inv_mass[t.x]) * wa + __ldg(&v.inv_mass[t.y]) * wb + __ldg(&v.inv_mass[t.z]) * wc;
    return 2;
}

// G lanes per vertex (32 / G vertices per warp).  The 27 cells (dz, dy, dx)
// = (c/9-1, c/3%3-1, c%3-1), the serial walk's order, are read in rounds of
// G (lane l: cell c0 + l); a round's slots are laid end to end (prefix sum
// over the vertex's lanes) and evaluated G at a time, one slot per lane; then
// the vertex's lanes replay those slots in walk order with the walk's rules
// -- stop at max_contacts contacts or scan_limit slots, skip a triangle
// already accepted, count guards of visited slots only -- and sum the
// accepted contacts in that order (every lane of the vertex holds the same
// sums; the accepted ids are spread over its lanes for the duplicate test).
// Loop bounds are the warp's maximum so the shuffles stay converged.
constexpr int kIslandLanes = 4;  // lanes per vertex of the island walk

template <int G>
__global__ void __launch_bounds__(kThreads, 4) k_island(View v) {
    constexpr int kHeld = (48 + G - 1) / G;  // accepted ids per lane (at most 48 per vertex)
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (lane & ~(G - 1));
    const int vertex = v.lo + warp_global_id() * (32 / G) + lane / G;
    bool run = vertex < v.hi;
    const Params* P = nullptr;
    if (run) {
        P = &params_v(v, vertex);
        run = fast_mode(*P) && P->thash && P->T > 0 && self_scheduled(*P, v) && v.pass == P->self_passes - 1 &&
              __ldg(&v.inv_mass[vertex]) > 0.0f;
    }
    float target = 0.0f;
    if (run) {
        target = contact_radius(*P);
        run = target > 0.0f;
    }
    const float onset = fmaxf(target * 1.8f, target + kEps);
    F3 p{0.0f, 0.0f, 0.0f}, pp{0.0f, 0.0f, 0.0f};
    int guards = 0;
    if (run) {
        p = f3(v.pos[vertex]);
        pp = f3(v.prev[vertex]);
        if (!finite3(p) || !finite3(pp)) {
            guards = 1;
            run = false;
        }
    }
    int max_contacts = 3, scan_limit = 30, cx = 0, cy = 0, cz = 0;
    if (run) {
        const int maxn = P->max_neighbors < 1 ? 1 : P->max_neighbors;
        max_contacts = min(max(maxn * 2, 3), 48);
        scan_limit = max_contacts * 10;
        cx = cell_of(p.x, P->tcell, P->key_ieee);
        cy = cell_of(p.y, P->tcell, P->key_ieee);
        cz = cell_of(p.z, P->tcell, P->key_ieee);
    }
    int contacts = 0, scanned = 0;
    int held[kHeld];
#pragma unroll
    for (int q = 0; q < kHeld; ++q) held[q] = -1;
    float pen_sum = 0.0f, wsum = 0.0f, max_pen = 0.0f;
    F3 axis{0.0f, 0.0f, 0.0f}, best{0.0f, 0.0f, 1.0f};
    bool stop = !run;
    for (int c0 = 0; c0 < 27; c0 += G) {
        const int c = c0 + gl;
        int st = 0, lim = 0;
        if (!stop && c < 27) {
            const int b = P->tbase + (int)bucket_of(cx + c % 3 - 1, cy + (c / 3) % 3 - 1, cz + c / 9 - 1, P->tbuckets);
            st = v.tb_start[b];
            lim = min(v.tb_start[b + 1] - st, kBucketSlots);
        }
        int incl = lim;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o, G);
            if (gl >= o) incl += t;
        }
        const int round_total = __shfl_sync(0xffffffffu, incl, G - 1, G);
        const int excl = incl - lim;
        const int warp_total = __reduce_max_sync(0xffffffffu, stop ? 0 : round_total);
        for (int base = 0; base < warp_total; base += G) {
            const int g = base + gl;
            int j = 0;  // owner lane: the first of the vertex's lanes whose inclusive count exceeds g
#pragma unroll
            for (int step = G / 2; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, incl, j + step - 1, G) <= g) j += step;
            const int o_first = __shfl_sync(0xffffffffu, st, j, G) - __shfl_sync(0xffffffffu, excl, j, G);
            int tri = -1, code = 0;
            IslandHit h{0.0f, 0.0f, F3{0.0f, 0.0f, 0.0f}};
            if (!stop && g < round_total) {
                tri = v.tb_ent[o_first + g];
                code = island_eval(v, vertex, p, pp, target, onset, tri, &h);
            }
            // Replay in walk order.  A triangle gives the same code every
            // time this vertex meets it, and only contacts (code 2) enter
            // the accepted set, so a slot of code 0 or 1 is never a
            // duplicate: it only advances the scan count (and the guard
            // count for code 1) under the walk's two limits, which stay
            // fixed until the next contact.  Such runs are settled in one
            // step from ballot masks; only the contacts go through the
            // serial duplicate test, one per iteration.
            const int n = stop ? 0 : max(min(G, round_total - base), 0);
            const int first = lane & ~(G - 1);
            const unsigned m1 = (__ballot_sync(0xffffffffu, code == 1) & gmask) >> first;
            unsigned m2 = (__ballot_sync(0xffffffffu, code == 2) & gmask) >> first;
            const int warp_c2 = __reduce_max_sync(0xffffffffu, __popc(m2));
            int pos = 0;
            auto run_plain = [&](int end) {  // slots [pos, end), none of them a contact
                if (stop || end <= pos) return;
                if (contacts >= max_contacts || scanned >= scan_limit) {
                    stop = true;
                    return;
                }
                const int take = min(end - pos, scan_limit - scanned);
                const unsigned span = take >= 32 ? 0xffffffffu : (1u << take) - 1u;
                guards += __popc(m1 & (span << pos));
                scanned += take;
                if (take < end - pos) stop = true;
                pos = end;
            };
            for (int it = 0; it < warp_c2; ++it) {
                const int k = m2 ? __ffs(m2) - 1 : n;
                run_plain(k);
                bool live = m2 != 0u && !stop;
                if (live && (contacts >= max_contacts || scanned >= scan_limit)) {
                    stop = true;
                    live = false;
                }
                const int src = m2 ? k : 0;
                const int t_k = __shfl_sync(0xffffffffu, tri, src, G);
                const float pen_k = __shfl_sync(0xffffffffu, h.pen, src, G), w_k = __shfl_sync(0xffffffffu, h.wterm, src, G);
                const F3 n_k{__shfl_sync(0xffffffffu, h.nrm.x, src, G), __shfl_sync(0xffffffffu, h.nrm.y, src, G),
                             __shfl_sync(0xffffffffu, h.nrm.z, src, G)};
                bool mine = false;
#pragma unroll
                for (int q = 0; q < kHeld; ++q) mine = mine || (q * G + gl < contacts && held[q] == t_k);
                const bool dup = (__ballot_sync(0xffffffffu, live && mine) & gmask) != 0u;
                if (m2) {
                    m2 &= m2 - 1u;
                    pos = k + 1;
                }
                if (!live) continue;
                ++scanned;
                if (dup) continue;
                if (gl == contacts % G) {
#pragma unroll
                    for (int q = 0; q < kHeld; ++q)
                        if (q == contacts / G) held[q] = t_k;
                }
                ++contacts;
                pen_sum += pen_k;
                wsum += w_k;
                axis = axis + n_k * pen_k;
                if (pen_k > max_pen) {
                    max_pen = pen_k;
                    best = n_k;
                }
            }
            run_plain(n);
        }
    }
    if (gl != 0) return;
    if (guards > 0) count_add(v.counts, kCntIslandGuarded, (unsigned long long)guards);
    if (contacts <= 0) return;
    count_add(v.counts, kCntIslandCandidates, (unsigned long long)contacts);
    if (contacts < 3) {
        count1(v.counts, kCntIslandGuarded);
        return;
    }
    const float avg_pen = pen_sum / (float)contacts;
    if (avg_pen < target * 0.04f) {
        count1(v.counts, kCntIslandGuarded);
        return;
    }
    const float alen = len3(axis);
    const F3 agg = alen > kEps ? axis * (1.0f / alen) : best;
    const float sw = __ldg(&v.inv_mass[vertex]);
    const float sample = wsum / (float)contacts;
    const float share = sw / fmaxf(sw + sample, kEps);
    const float max_delta = fmaxf(target * 0.30f, 1.0e-5f);
    const float dl = fminf(avg_pen * 0.50f * share, max_delta);
    if (!finite3(agg) || !isfinite(dl) || dl <= kEps) {
        count1(v.counts, kCntIslandGuarded);
        return;
    }
    accumulate(v, vertex, agg * dl);
    count1(v.counts, kCntIslandClusters);
    count_add(v.counts, kCntIslandVertexRefs, (unsigned long long)contacts);
    count1(v.counts, kCntIslandAppliedVertices);
    if (isfinite(dl) && dl > 0.0f) {
        const unsigned long long micro = (unsigned long long)(fminf(dl, 1024.0f) * 1000000.0f);
        atomicMax(&v.counts[kCntIslandMaxDeltaMicro], micro);
    }
}

// Average the accumulated pushes, clamp to 0.35 r, apply with a 0.55 prev
// shift, and clear the accumulators for the next pass (abi41.cu:4953-4988).
__global__ void __launch_bounds__(kThreads) k_self_apply(View v) {
    const int i = v.lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= v.hi) return;
    const Params& P = params_v(v, i);
    if (!self_scheduled(P, v)) return;
    const Acc4 a = v.acc[i];
    if (a.w == 0) return;  // every push adds a weight: nothing accumulated, the row is still zero
    v.acc[i] = Acc4{0, 0, 0, 0};
    if (!(__ldg(&v.inv_mass[i]) > 0.0f) || a.w <= 0) return;
    F3 avg = F3{from_fix(a.x), from_fix(a.y), from_fix(a.z)} * (1.0f / (float)a.w);
    const float max_delta = fmaxf(contact_radius(P) * 0.35f, 1.0e-4f);
    const float dl = len3(avg);
    if (dl > max_delta) avg = avg * (max_delta / dl);
    const float4 p = v.pos[i];
    v.pos[i] = f4(f3(p) + avg, p.w);
    v.prev[i] = f4(f3(v.prev[i]) + avg * 0.55f, 0.0f);
    const float al = len3(avg);
    if (al > 0.0f) atomicMax(v.max_delta_bits, __float_as_uint(al));
}

}  // namespace

// Host-side entry points used by the solver orchestration.
namespace {

View ranged(const View& v, const ItemRange& r) {
    View out = v;
    out.lo = r.lo;
    out.hi = r.hi;
    return out;
}

// Threads of a launch over `items` with `per_item` lanes each, in blocks of b.
inline int grid(long long items, int per_item, int b) { return grid_for(items * per_item, b); }

constexpr int kTrimBlocks = 152 * 4;  // fixed grid of the trim pass (4 blocks per SM)

template <int L>
void tri_pass(const View& iv, int blocks, int b, bool scatter, cudaStream_t s) {
    k_tri_hash<L><<<blocks, b, 0, s>>>(iv, scatter);
}

void tri_pass_lanes(const View& iv, long long items, int lanes, int b, bool scatter, cudaStream_t s) {
    switch (lanes) {
        case 1: tri_pass<1>(iv, grid(items, 1, b), b, scatter, s); break;
        case 2: tri_pass<2>(iv, grid(items, 2, b), b, scatter, s); break;
        case 4: tri_pass<4>(iv, grid(items, 4, b), b, scatter, s); break;
        case 16: tri_pass<16>(iv, grid(items, 16, b), b, scatter, s); break;
        default: tri_pass<8>(iv, grid(items, 8, b), b, scatter, s); break;
    }
}

template <int G>
void neighbors_group(const View& v, const ItemRange& r, bool vv, int mode, int b, cudaStream_t s) {
    if (vv)
        k_neighbors_group<true, G><<<grid(r.size(), G, b), b, 0, s>>>(ranged(v, r), mode);
    else
        k_neighbors_group<false, G><<<grid(r.size(), G, b), b, 0, s>>>(ranged(v, r), mode);
}

void bucket_order(const View& v, const ItemRange& buckets, const int* start, int* ent, int nb, int kind, int mode,
                  cudaStream_t s) {
    if (buckets.size() == 0) return;
    const int b = tune_of(v.tune, kTuneWarpBlock);
    k_bucket_sort<<<grid((buckets.size() + 31) / 32, 32, b), b, 0, s>>>(ranged(v, buckets), start, ent, nb, kind, mode);
}

void bucket_trim(const View& v, const int* start, int* ent, cudaStream_t s) {
    k_bucket_trim<<<kTrimBlocks, kThreads, 0, s>>>(start, ent, v.trim_list, v.trim_count);
}

void tri_hash(const View& v, const ItemRange& items, const ItemRange& buckets, const ItemRange& ordered, int nb, int order,
              cudaStream_t s) {
    if (items.size() == 0) return;
    const View iv = ranged(v, items);
    const int b = tune_of(v.tune, kTuneHashBlock), lanes = tune_of(v.tune, kTuneTriLanes);
    tri_pass_lanes(iv, items.size(), lanes, b, false, s);
    scan_counts(v.tb_count, v.tb_start, nb, v.scan_tmp, v.counts ? v.counts + kCntSelfOverflow : nullptr, s, v.trim_list,
                v.trim_count);
    tri_pass_lanes(iv, items.size(), lanes, b, true, s);
    if (v.trim_list) {
        // overflowing buckets of every cloth from the scan's list, then every
        // bucket of the cloths whose queries follow bucket order
        bucket_trim(v, v.tb_start, v.tb_ent, s);
        if (order != 0) bucket_order(v, ordered, v.tb_start, v.tb_ent, nb, 1, 3, s);
    } else {
        bucket_order(v, buckets, v.tb_start, v.tb_ent, nb, 1, order, s);
    }
}

template <int L>
void group_queries(const View& v, const SelfVariants& sv, int b, cudaStream_t s, bool edges) {
    if (edges)
        k_ee_warp<L><<<grid(sv.e_strict.size(), L, b), b, 0, s>>>(ranged(v, sv.e_strict));
    else
        k_vt_warp<L><<<grid(sv.v_strict.size(), L, b), b, 0, s>>>(ranged(v, sv.v_strict));
}

void group_queries_lanes(const View& v, const SelfVariants& sv, cudaStream_t s, bool edges) {
    const int b = tune_of(v.tune, kTuneGroupBlock);
    switch (tune_of(v.tune, kTuneGroupLanes)) {
        case 4: group_queries<4>(v, sv, b, s, edges); break;
        case 16: group_queries<16>(v, sv, b, s, edges); break;
        default: group_queries<8>(v, sv, b, s, edges); break;
    }
}

}  // namespace

void scan_bucket_counts(int* counts, int* start, int n, int* block_sums, cudaStream_t s) {
    if (n > 0) scan_counts(counts, start, n, block_sums, nullptr, s);
}

void self_build_vertex_hash(const View& v, const SelfVariants& sv, int nb, cudaStream_t s) {
    const ItemRange& r = sv.v_all;
    if (r.size() == 0) return;
    const View iv = ranged(v, r);
    const int b = tune_of(v.tune, kTuneHashBlock);
    k_vhash_count<<<grid(r.size(), 1, b), b, 0, s>>>(iv);
    scan_counts(v.vb_count, v.vb_start, nb, v.scan_tmp, v.counts ? v.counts + kCntSelfOverflow : nullptr, s);
    k_vhash_scatter<<<grid(r.size(), 1, b), b, 0, s>>>(iv);
    bucket_order(v, sv.vb, v.vb_start, v.vb_ent, nb, 0, 1, s);
}
void self_build_triangle_hash(const View& v, const SelfVariants& sv, int nb, int order, cudaStream_t s) {
    tri_hash(v, sv.t_all, sv.tb, sv.tb_ord, nb, order, s);
}
// The slotted edge hash: insertion, the overflow regions (kernels that exit
// at once when no bucket overflowed), ordering of the listed buckets of more
// than 32 members, then of the buckets of up to 32 where queries follow
// bucket order (order 1 / 2: the cloths that need it, 3: every bucket).
// The counts, overflow bits and counters and the trim count must be zero.
void self_build_edge_hash(const View& v, const SelfVariants& sv, int nb, int order, cudaStream_t s) {
    const ItemRange& items = sv.e_all;
    if (items.size() == 0) return;
    const View iv = ranged(v, items);
    const int b = tune_of(v.tune, kTuneHashBlock), lanes = tune_of(v.tune, kTunePrimLanes);
    const long long n = items.size();
    switch (lanes) {
        case 1: k_edge_insert<1><<<grid(n, 1, b), b, 0, s>>>(iv); break;
        case 2: k_edge_insert<2><<<grid(n, 2, b), b, 0, s>>>(iv); break;
        case 4: k_edge_insert<4><<<grid(n, 4, b), b, 0, s>>>(iv); break;
        case 16: k_edge_insert<16><<<grid(n, 16, b), b, 0, s>>>(iv); break;
        default: k_edge_insert<8><<<grid(n, 8, b), b, 0, s>>>(iv); break;
    }
    k_edge_ovf_offsets<<<1, 1024, 0, s>>>(v);
    k_edge_ovf_late<<<kTrimBlocks, kThreads, 0, s>>>(v);
    switch (lanes) {
        case 1: k_edge_ovf_collect<1><<<kTrimBlocks, kThreads, 0, s>>>(iv); break;
        case 2: k_edge_ovf_collect<2><<<kTrimBlocks, kThreads, 0, s>>>(iv); break;
        case 4: k_edge_ovf_collect<4><<<kTrimBlocks, kThreads, 0, s>>>(iv); break;
        case 16: k_edge_ovf_collect<16><<<kTrimBlocks, kThreads, 0, s>>>(iv); break;
        default: k_edge_ovf_collect<8><<<kTrimBlocks, kThreads, 0, s>>>(iv); break;
    }
    k_edge_ovf_select<<<kTrimBlocks, kThreads, 0, s>>>(v);
    k_edge_trim<<<kTrimBlocks, kThreads, 0, s>>>(v);
    if (order != 0) bucket_order(v, order == 3 ? sv.eb : sv.eb_ord, nullptr, v.eb_slot, nb, 2, 3, s);
}

void self_neighbors(const View& v, int mode, const SelfVariants& sv, cudaStream_t s) {
    const ItemRange& r = mode == 1 ? sv.v_fast : (mode == 2 ? sv.v_strict : sv.v_all);
    if (r.size() == 0) return;
    const int wb = tune_of(v.tune, kTuneWarpBlock), qb = tune_of(v.tune, kTuneQueryBlock);
    if (sv.hashed_v) {
        const bool vv = mode == 2;  // strict passes: VV responses fused
        switch (tune_of(v.tune, kTuneNeighborLanes)) {
            case 1: neighbors_group<1>(v, r, vv, mode, wb, s); break;
            case 4: neighbors_group<4>(v, r, vv, mode, wb, s); break;
            case 8: neighbors_group<8>(v, r, vv, mode, wb, s); break;
            case 16: neighbors_group<16>(v, r, vv, mode, wb, s); break;
            case 32: neighbors_group<32>(v, r, vv, mode, wb, s); break;
            default: neighbors_group<2>(v, r, vv, mode, wb, s); break;
        }
    }
    if (sv.brute_v) k_neighbors_brute<<<grid(r.size(), 1, qb), qb, 0, s>>>(ranged(v, r), mode);
}
void self_vv(const View& v, const SelfVariants& sv, cudaStream_t s) {
    const int wb = tune_of(v.tune, kTuneWarpBlock), qb = tune_of(v.tune, kTuneQueryBlock);
    // hashed strict cloths get their responses in the fused neighbour kernel
    if (sv.strict && sv.brute_v && sv.v_strict.size() > 0)
        k_vv_warp<<<grid(sv.v_strict.size(), 32, wb), wb, 0, s>>>(ranged(v, sv.v_strict), 0);
    if (sv.fast && sv.v_fast.size() > 0) k_vv<<<grid(sv.v_fast.size(), 1, qb), qb, 0, s>>>(ranged(v, sv.v_fast));
}
void self_vt(const View& v, const SelfVariants& sv, cudaStream_t s) {
    const int wb = tune_of(v.tune, kTuneWarpBlock), qb = tune_of(v.tune, kTuneQueryBlock);
    if (sv.hashed_t && sv.strict_wide && sv.v_strict.size() > 0)
        k_flat_vt<<<grid(sv.v_strict.size(), 1, wb), wb, 0, s>>>(ranged(v, sv.v_strict));
    if (sv.hashed_t && sv.strict_narrow && sv.v_strict.size() > 0) group_queries_lanes(v, sv, s, false);
    if (sv.hashed_t && sv.fast && sv.v_fast.size() > 0)
        k_vt_hash<<<grid(sv.v_fast.size(), 1, qb), qb, 0, s>>>(ranged(v, sv.v_fast));
    if (sv.brute_t && sv.v_all.size() > 0) k_vt_brute<<<grid(sv.v_all.size(), 1, qb), qb, 0, s>>>(ranged(v, sv.v_all));
}
void self_ee(const View& v, const SelfVariants& sv, cudaStream_t s) {
    const int wb = tune_of(v.tune, kTuneWarpBlock), qb = tune_of(v.tune, kTuneQueryBlock);
    const int gb = tune_of(v.tune, kTuneGroupBlock);
    if (sv.hashed_e && sv.strict_wide && sv.e_strict.size() > 0)
        k_flat_ee<<<grid(sv.e_strict.size(), 1, wb), wb, 0, s>>>(ranged(v, sv.e_strict));
    if (sv.hashed_e && sv.strict_narrow && sv.e_strict.size() > 0) group_queries_lanes(v, sv, s, true);
    if (sv.hashed_e && sv.fast && sv.e_fast.size() > 0) {
        if (tune_of(v.tune, kTuneFastEeForm) == 32) {
            const int fb = min(wb, kThreads);  // the shared arrays hold kThreads / 32 warps
            k_ee_fast_flat<<<grid(sv.e_fast.size(), 1, fb), fb, 0, s>>>(ranged(v, sv.e_fast));
        } else {
            k_ee_fast<<<grid(sv.e_fast.size(), kQueryLanes, gb), gb, 0, s>>>(ranged(v, sv.e_fast));
        }
    }
    if (sv.brute_e && sv.e_all.size() > 0) k_ee_brute<<<grid(sv.e_all.size(), 1, qb), qb, 0, s>>>(ranged(v, sv.e_all));
}
void self_island(const View& v, const SelfVariants& sv, cudaStream_t s) {
    const int wb = tune_of(v.tune, kTuneWarpBlock);
    constexpr int G = kIslandLanes;
    if (sv.v_fast.size() > 0) k_island<G><<<grid(sv.v_fast.size(), G, wb), wb, 0, s>>>(ranged(v, sv.v_fast));
}
void self_apply(const View& v, const SelfVariants& sv, cudaStream_t s) {
    const int qb = tune_of(v.tune, kTuneQueryBlock);
    if (sv.v_all.size() > 0) k_self_apply<<<grid(sv.v_all.size(), 1, qb), qb, 0, s>>>(ranged(v, sv.v_all));
}

}  // namespace xg
