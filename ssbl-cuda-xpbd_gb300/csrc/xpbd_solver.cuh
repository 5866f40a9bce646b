// Device-side state of one cloth solver and the declarations shared by the
// CUDA translation units of the GB300 XPBD library.
//
// Layout in HBM (one allocation per array, 256-byte aligned by cudaMalloc):
//   pos[2]   float4 x V   ping-pong; .w = effective inverse mass (0 = pinned)
//   prev     float4 x V   previous position (.w unused)
//   vel      float4 x V
//   rest     float4 x V   rest pose (.w unused)
//   spring   CSR by vertex: off[V+1], ent[2E] = {other | side<<31, rest}
//   tether   CSR by vertex: off[V+1], ent[2L] = {other | side<<31, rest}
//   bends    int2 x B sorted by colour, rest f32 x B (colour ranges on host)
//   tris     int4 x T {a, b, c, 0}
//   edges    int2 x E
//   pins     per vertex: target float4, weight f32 (-1 = none), relaxation f32
// float4 rows make every gather of a neighbour one 16-byte load and carry the
// inverse mass with the position, which the constraint kernels need together.
#pragma once

#include <string>

#include "../../include/ssbl_xpbd_cuda.h"
#include "xpbd_math.cuh"

namespace xg {

constexpr int kThreads = 256;
constexpr int kNeighborSlots = 32;    // VV neighbour table width (abi41.cu:38)
constexpr int kBucketSlots = 32;      // per-bucket query cap (abi41.cu:29, 32, 36)
constexpr int kEdgeSlots = 64;        // member slots per edge-hash bucket (more: overflow regions)
constexpr int kMaxPrimitiveCells = 64;
constexpr int kSideBit = (int)0x80000000u;

// Fixed-point self-collision accumulator of one vertex: delta x, y, z in
// 2^-32 m units and the number of contributions.
struct __align__(32) Acc4 {
    long long x, y, z, w;
};

// Counter slots of the diagnostics block (same meaning as abi41.cu:41-78).
enum Counter {
    kCntSoftContacts = 0,
    kCntExactImpulseContacts = 1,
    kCntEdgeEdgeContacts = 2,
    kCntHardFallbacks = 3,
    kCntDynParCandidates = 4,
    kCntDynParContacts = 5,
    kCntDynParOverflow = 6,
    kCntTrianglePairs = 7,
    kCntSelfCandidates = 9,
    kCntSelfOverflow = 10,
    kCntStaticSdfContacts = 11,
    kCntLraTacks = 12,
    kCntBendingWings = 13,
    kCntTackGuards = 14,
    kCntBendingGuards = 15,
    kCntIslandCandidates = 16,
    kCntIslandClusters = 17,
    kCntIslandVertexRefs = 18,
    kCntIslandAppliedVertices = 19,
    kCntIslandGuarded = 20,
    kCntIslandMaxDeltaMicro = 21,
    kCntFilterSeen = 22,
    kCntFilterAcceptedVv = 23,
    kCntFilterAcceptedVt = 24,
    kCntFilterAcceptedEe = 25,
    kCntFilterRejectedRest = 26,
    kCntFilterRejectedDuplicate = 27,
    kCntFilterRejectedOwnership = 28,
    kCntFilterCacheHits = 29,
    kCntFilterCacheMisses = 30,
    kCntClusterCount = 31,
    kCntClusterOwnedContacts = 32,
    kCntFrictionCorrections = 33,
    kCntDynTriCandidates = 34,
    kCntDynTriOverflow = 35,
    kCntDynTriLarge = 36,
    kCntDynTriAabbRejects = 37,
    kCntSlots = 38
};

// Scalar slots of the CG solve (same roles as abi41.cu:158-164).
enum PcgSlot { kRedDAD = 0, kRedRZ = 1, kRedRZNext = 2, kRedStatus = 3, kRedInitialRZ = 4, kRedIterations = 5, kRedSlots = 8 };

// Dynamic colliders of one cloth (moving triangle meshes and particles,
// uploaded every frame): geometry, per-triangle bounds, and the spatial
// hashes built at upload (bucket members in increasing id order).
struct DynSet {
    // triangles
    int tri_count;
    int signed_mode;      // 1 for indexed (closed, animated) meshes
    int motion_valid;     // previous centres belong to the same triangles
    int tri_hashed;       // hash built (>= 64 triangles), else brute force
    float tri_cell;
    int tri_buckets;
    const float4* tris;   // 3 rows per triangle
    const float4* amin;   // bounds per triangle
    const float4* amax;
    const float4* center;
    const float4* prev_center;
    const float* radius;
    const int4* cmin;     // cell span per triangle (hash margin = collision margin)
    const int4* cmax;
    const int* tstart;    // [tri_buckets + 1]
    const int* tent;
    const int* large;     // triangles spanning more than 64 cells, increasing id
    int large_count;
    // particles
    int par_count;
    int par_motion_valid;
    int par_hashed;       // hash built (>= 128 particles), else brute force
    float par_cell;
    int par_buckets;
    const float4* par_pos;
    const float4* par_prev;
    const float* par_radius;
    const int4* par_cellc;
    const int* pstart;    // [par_buckets + 1]
    const int* pent;      // first 16 members of a bucket are queried
    // shared scene only: source id and collision layer per primitive
    const int* tri_src;
    const int* tri_layer;
    const int* par_src;
    const int* par_layer;
    int key_ieee;         // cell-key division of both hashes (xpbd_math.cuh)
};

// Parameters of one cloth.  A solver holds one or more cloths concatenated
// in every per-vertex / per-constraint array (a batch); each kernel reads the
// parameters of the cloth its item belongs to.  They live in device memory so
// a captured CUDA graph stays valid when the caller moves a collider, the
// pins or the static SDF of a cloth.
struct Params {
    // this cloth's ranges in the concatenated arrays
    int vstart, V, estart, E, tstart, T, B, L;
    int active;      // 0: every kernel skips this cloth's items
    float sub_dt;    // frame dt / substeps of the current step
    float frame_dt;  // collider motion interval: cfg.dt when positive, else sub_dt
    float damping;
    float gravity[3];
    float stretch_compliance;
    float bend_compliance;
    float lra_compliance;
    float margin;
    float thickness;
    float friction;
    float tangent_damping;
    int use_ground;
    float ground_height;
    int use_wall;
    float wall_origin[3];
    float wall_normal[3];
    int use_sphere;
    float sphere_center[3];
    float sphere_radius;
    // static SDF of this cloth's collider
    int sdf_ready;
    int sdf_signed;
    int sdf_dim[3];
    float sdf_origin[3];
    float sdf_voxel;
    int static_tri_count;
    const float* sdf;
    const float4* static_tris;  // 3 per triangle
    // self collision
    int self_on;           // enabled with a positive contact distance
    int self_interval;
    int self_passes;
    float self_radius;     // contact target distance r
    int self_mode;         // 1 fast, 2 strict
    int max_neighbors;     // cfg.max_self_collision_neighbors as given
    float vcell, tcell, ecell;
    int vbuckets, tbuckets, ebuckets;  // this cloth's table sizes
    int vbase, tbase, ebase;           // offsets of its tables in the shared bucket arrays
    int vhash, thash, ehash;           // hash in use (else brute force)
    int key_ieee;                      // cell-key division: 0 the reference's, 1 IEEE (xpbd_math.cuh)
    float stretch_strength;            // clamp01(stretch_optimization_strength)
    // hard-stretch optimisation: this cloth runs the CG stretch solve in
    // place of the spring gather (and, at strength >= 0.95, the averaged
    // polish and ratio caps); its CG blocks are [pcg_block0, + pcg_nblocks)
    int pcg_on, pcg_hard, pcg_block0, pcg_nblocks;
    int cap_jacobi;  // no caller edge colouring: each cap pass is one Jacobi pass over the cloth's edges
    // external accelerations of the prediction (force fields, volume pressure)
    const SsblXpbdForceField* fields;  // field_count records (device)
    int field_count;
    int pressure_on;                   // use_volume_pressure with a positive strength
    float pressure_strength;
    float pressure_accel_scale;
    float pressure_impulse_rest_scale;
    float pressure_velocity_rest_scale;
    float pressure_velocity_length_scale;
    int needs_normal;                  // pressure or fields: vertex normals are gathered
    const DynSet* dyn;                 // dynamic colliders (device), null when none
    // shared dynamic scene (cross-cloth collision, abi41.cu:3984-3997):
    // with a non-zero mode it replaces the cloth's own unsigned colliders;
    // primitives of the target source id are skipped, and with mode 2 only
    // lower collision layers collide
    const DynSet* gdyn;
    int gd_mode, gd_target_source, gd_target_layer;
};

// Buffers of the hard-stretch CG solve and the averaged caps.
struct PcgView {
    float4* diag;        // 2 rows per vertex: symmetric 3x3 block
    float4* pinv;        // 2 rows per vertex: block-Jacobi inverse
    float4* r;
    float4* z;
    float4* d;
    float4* q;
    float4* offdiag;     // per stretch-CSR entry: edge normal xyz, stiffness
    float4* avg;         // averaged caps: sum xyz, count
    float* red;          // kRedSlots scalars per cloth
    float* partials;     // one per warp of the solve grid (each cloth's warps contiguous)
    unsigned* ticket;    // last-block ticket per cloth
    const int* blk_cloth;  // cloth of each block of the solve grid
    unsigned long long* guard;
    unsigned* max_delta_bits;
};

// Launch configuration of the kernel classes (block sizes and tiles), chosen
// by the autotuner; 0 selects the built-in default.  None of them changes a
// result: every kernel's per-item arithmetic and its fixed-point sums are the
// same for any block size, lanes per primitive or lanes per query item.
enum TuneSlot {
    kTuneVertexBlock = 0,  // per-vertex constraint passes and prediction (default 128)
    kTuneHashBlock,        // hash count / scatter kernels (256)
    kTunePrimLanes,        // lanes per primitive of the edge hash: 1, 2, 4, 8, 16 (8)
    kTuneWarpBlock,        // warp-per-item kernels: neighbour table, strict VV, flat queries, bucket order (256)
    kTuneQueryBlock,       // thread-per-item queries: fast VV / VT, brute queries, islands, apply (256)
    kTuneGroupLanes,       // lanes per item of the strict group queries: 4, 8, 16 (8)
    kTuneGroupBlock,       // group query kernels (256)
    kTuneDynamicBlock,     // dynamic colliders (128)
    kTuneFastEeForm,       // fast-mode EE query: 8 = groups of 8 lanes, 32 = one warp per 32 items, flattened (32)
    kTuneFusedFrame,       // small cloths: 1 = whole frame in one block per cloth, 8 = in an 8-CTA cluster per cloth,
                           // 2 = launched kernels (1)
    kTuneTriLanes,         // lanes per primitive of the triangle hash: 1, 2, 4, 8, 16 (8)
    kTuneNeighborLanes,    // lanes per vertex of the neighbour table (+ strict VV): 1, 2, 4, 8, 16, 32 (2)
    kTuneSlots
};
struct LaunchTune {
    short v[kTuneSlots];
};
constexpr short kTuneDefault[kTuneSlots] = {128, 256, 8, 256, 256, 8, 256, 128, 32, 0, 8, 2};
constexpr int kMaxBlock = 256;  // the kernels' launch bounds
inline int tune_of(const LaunchTune& t, int slot) { return t.v[slot] > 0 ? t.v[slot] : kTuneDefault[slot]; }
inline int grid_for(long long threads, int block) { return (int)((threads + block - 1) / block); }

// Device pointers of one solver, passed by value to each kernel, plus the
// launch context of the frame schedule.
struct View {
    const Params* P;      // one per cloth
    const int* vcloth;    // cloth of each vertex / edge / triangle (null for one cloth)
    const int* ecloth;
    const int* tcloth;
    int nV, nE, nT, nB, K;  // totals over all cloths
    int substep, substeps;  // position in the frame schedule
    int pass;               // self-collision pass (-1 outside the passes)
    int last_it;            // launch belongs to the last iteration
    float4* pos_in;       // snapshot read by gathers
    float4* pos;          // position written by this kernel / in place
    float4* prev;
    float4* vel;
    const float4* rest;
    const float* inv_mass;
    const int* sp_off;
    const int2* sp_ent;
    const int* te_off;
    const int2* te_ent;
    const int* bj_off;    // bends as a gather when no colours are given
    const int2* bj_ent;
    const int2* bends;
    const float* bend_rest;
    const int4* tris;
    const int2* edges;
    const float* edge_rest;
    const float4* pin_target;  // per vertex
    const float* pin_weight;   // per vertex; -1 = no pin
    const float* pin_relax;    // per vertex soft-pin relaxation
    const int* vt_off;         // vertex -> incident triangles (triangle order)
    const int* vt_tri;
    const float* p_area;       // volume pressure: area share and rest scale per vertex
    const float* p_rest;
    unsigned long long* counts;
    // self collision
    int4* vcell;            // cx, cy, cz, global bucket per vertex
    int* vb_count;          // [all cloths' vertex buckets]
    int* vb_start;          // [+1]
    int* vb_ent;            // [nV]
    int* tb_count;
    int* tb_start;
    int* tb_ent;
    // edge hash: bucket b's members in eb_slot[b * kEdgeSlots ...], its count
    // in eb_count[b]; buckets of more than kEdgeSlots members are listed in
    // eb_ovf_list (bit set in eb_ovf_bits) and their full member lists kept
    // in eb_ent at [eb_start[b] - eb_count[b], eb_start[b]); the insertions
    // past a bucket's kEdgeSlots slots are recorded as (bucket, edge) in
    // eb_late while eb_late_count stays within eb_late_cap
    int* eb_count;
    int* eb_start;
    int* eb_ent;
    int* eb_slot;
    unsigned* eb_ovf_bits;
    int* eb_ovf_list;
    int* eb_ovf_count;
    int* eb_ovf_start;      // [eb_ovf_list index] first entry of the bucket's region
    int2* eb_late;
    unsigned long long* eb_late_count;
    long long eb_late_cap;
    int* scan_tmp;          // block sums of the bucket scans
    int* trim_list;         // buckets of more than 32 members found by the scan (null: none kept)
    int* trim_count;
    int* nb_count;          // [nV]
    int* nb_idx;            // [nV * 32]
    Acc4* acc;              // fixed-point delta xyz + contact weight
    unsigned* max_delta_bits;
    // work counters of a profiled frame (null otherwise): query items and
    // bucket slots evaluated by the EE and VT queries
    unsigned long long* perf;
    // item range [lo, hi) of a self-collision launch (vertices, edges,
    // triangles or buckets, by kernel); set by the launchers
    int lo, hi;
    LaunchTune tune;  // read by the launchers only
};

// EE gathers: visited slots whose candidate id is above the query edge's
// (the pairs whose indices and rows are read; a pair is taken from its lower
// edge, so the others end at the id).
enum PerfSlot { kPerfEeItems = 0, kPerfEeSlots = 1, kPerfVtItems = 2, kPerfVtSlots = 3, kPerfEeGathers = 4, kPerfSlots = 5 };
// The work counters are kept in kPerfStripes copies 64 bytes apart, a block
// adding to copy blockIdx.x % kPerfStripes, and summed on the host: one
// counter address taking an atomic from every warp of a query launch would
// serialise in one L2 slice and slow the profiled kernels themselves.
constexpr int kPerfStripes = 32;
constexpr int kPerfStride = 8;

__device__ __forceinline__ int cloth_of(const int* map, int i) { return map ? __ldg(&map[i]) : 0; }
__device__ __forceinline__ const Params& params_v(const View& v, int i) { return v.P[cloth_of(v.vcloth, i)]; }
__device__ __forceinline__ const Params& params_e(const View& v, int e) { return v.P[cloth_of(v.ecloth, e)]; }
__device__ __forceinline__ const Params& params_t(const View& v, int t) { return v.P[cloth_of(v.tcloth, t)]; }

// First member slot of edge-hash bucket b and the members a query reads
// (at most the 32 query slots).
__device__ __forceinline__ long long edge_bucket_base(int b) { return (long long)b * kEdgeSlots; }
__device__ __forceinline__ int edge_bucket_size(const View& v, int b) { return min(v.eb_count[b], kBucketSlots); }

// Whether a cloth runs self collision in this substep (and, inside the
// passes, in this pass) (abi41.cu:9255-9262, 9291).
__device__ __forceinline__ bool self_scheduled(const Params& P, const View& v) {
    if (!P.active || !P.self_on) return false;
    if (!(((v.substep + 1) % P.self_interval) == 0 || v.substep == v.substeps - 1)) return false;
    return v.pass < 0 || v.pass < P.self_passes;
}

// Warp-aggregated counter increment: one atomic per warp, lane count from the
// active mask.
__device__ __forceinline__ void count1(unsigned long long* counts, int slot) {
    if (!counts) return;
    const unsigned mask = __activemask();
    if ((threadIdx.x & 31) == (__ffs(mask) - 1)) atomicAdd(&counts[slot], (unsigned long long)__popc(mask));
}

__device__ __forceinline__ void perf_add(unsigned long long* perf, int slot, unsigned long long v) {
    if (perf && v) atomicAdd(&perf[(blockIdx.x % kPerfStripes) * kPerfStride + slot], v);
}

__device__ __forceinline__ void count_add(unsigned long long* counts, int slot, unsigned long long v) {
    if (counts && v) atomicAdd(&counts[slot], v);
}

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// Set the message returned by ssbl_last_error() (defined in xpbd_abi.cu).
void set_last_error(const std::string& msg);

// ---- host launchers (defined in the .cu files) ----
// Blocks of the CG solve grid for a cloth of V vertices (each cloth of a
// batch gets the grid a one-cloth solver of its size would launch).
int pcg_blocks(int V);
void pcg_solve(const View& v, const PcgView& g, int blocks, cudaStream_t s, long long* launches);
void pcg_averaged_pass(const View& v, const PcgView& g, int V, bool tiny, cudaStream_t s);
// kind: 0 normal cap, 1 tiny cap, 2 extreme cap; over the colour-sorted cap
// edges [start, start + count) (v.edges / v.edge_rest / v.nE point at them)
void pcg_cap_range(const View& v, int start, int count, int kind, cudaStream_t s);
void pcg_cap_jacobi(const View& v, const PcgView& g, int V, int kind, cudaStream_t s);
void launch_predict(const View& v, int V, cudaStream_t s);
// pass flags for launch_vertex_pass
enum PassFlags : unsigned {
    kPassSpring = 1u,
    kPassPin = 2u,
    kPassAnalytic = 4u,
    kPassSdf = 8u,
    kPassPinPolish = 16u,
    kPassVelocity = 32u,
    kPassTether = 64u,
    kPassBend = 128u,
};
void launch_vertex_pass(const View& v, int V, unsigned flags, cudaStream_t s);

// One operation of a recorded frame (the launches of the normal schedule):
// kind 0 prediction, 1 vertex pass (flags), 2 bends of colour `color`,
// 3 copy of buffer `in_buf` into `out_buf`.  in_buf / out_buf: index of the
// position buffer read / written.
struct FrameOp {
    int kind;
    unsigned flags;
    int in_buf, out_buf;
    int substep, last_it;
    int color;
};
// The whole frame of each cloth in one block (cloths of at most 1024
// vertices without self collision, hard stretch or dynamic colliders): the
// recorded operations run in order with a block barrier between them.
// bend_ranges[color * K + cloth] = {first bend, count} of that cloth's bends
// of the colour.
void launch_frame_fused(const View& v, const FrameOp* ops, int nops, float4* buf0, float4* buf1, const int2* bend_ranges,
                        int K, int block, cudaStream_t s);
// The same with a thread-block cluster of `cluster` CTAs per cloth (each
// holding a full copy of the state, cap vertices per array) exchanging their
// slices through distributed shared memory after every operation.
void launch_frame_cluster(const View& v, const FrameOp* ops, int nops, float4* buf0, const int2* bend_ranges, int K, int cap,
                          int cluster, int block, cudaStream_t s);
void launch_bend_color(const View& v, int start, int count, cudaStream_t s);
void launch_copy_pos(float4* dst, const float4* src, int V, cudaStream_t s);
void launch_pin_scatter(const int* idx, const float4* target, const float* weight, const float* relax, int n,
                        float4* pin_target, float* pin_weight, float* pin_relax, int nV, cudaStream_t s);
void launch_pack_positions(float* dst, const float4* src, int V, cudaStream_t s);
void launch_sdf_build(const View& v, int cloth, int voxels, cudaStream_t s);

// dynamic colliders: collision passes over all vertices (cloths without
// colliders of the kind skip); `which` 0 unsigned triangles + particles
// (cloths in unsigned mode), 1 signed triangles + particles, 2 signed
// triangles inside-only
void launch_dynamic_collision(const View& v, int V, int which, cudaStream_t s);
constexpr int kSignedInsidePasses = 6;  // inside-only passes at the final constraints (abi41.cu:80)
// exclusive scan of bucket counts into starts (counts become cursors)
void scan_bucket_counts(int* counts, int* start, int n, int* block_sums, cudaStream_t s);

// Contiguous item range covering the cloths added to it.
struct ItemRange {
    int lo = 0, hi = 0;
    void add(int start, int n) {
        if (n <= 0) return;
        if (hi <= lo) {
            lo = start;
            hi = start + n;
        } else {
            lo = lo < start ? lo : start;
            hi = hi > start + n ? hi : start + n;
        }
    }
    int size() const { return hi > lo ? hi - lo : 0; }
};

// The kernel variants some scheduled cloth needs and the item ranges of the
// scheduled cloths.  Cloths are stored grouped by self-collision mode, so a
// mode's range holds no items of the other mode's cloths.
struct SelfVariants {
    bool fast, strict, hashed_v, brute_v, hashed_t, brute_t, hashed_e, brute_e;
    bool strict_wide, strict_narrow;  // strict cloths with a candidate budget of >= 32 / < 32 slots
    ItemRange v_all, v_fast, v_strict, e_all, e_fast, e_strict, t_all, vb, tb, eb;
    ItemRange tb_ord, eb_ord;  // bucket ranges of cloths whose queries need every bucket ordered
    void add_cloth(const Params& P, bool is_fast) {
        v_all.add(P.vstart, P.V);
        (is_fast ? v_fast : v_strict).add(P.vstart, P.V);
        e_all.add(P.estart, P.E);
        (is_fast ? e_fast : e_strict).add(P.estart, P.E);
        t_all.add(P.tstart, P.T);
        if (P.vhash) vb.add(P.vbase, P.vbuckets);
        if (P.thash) tb.add(P.tbase, P.tbuckets);
        if (P.ehash) eb.add(P.ebase, P.ebuckets);
    }
};

// self collision (bucket counts must be zeroed before each hash build; nb =
// total buckets over all cloths).  Each launcher runs the kernel variants
// that some cloth needs, over the item range of that variant's cloths;
// every item still skips cloths of another mode / table kind.
void self_build_vertex_hash(const View& v, const SelfVariants& sv, int nb, cudaStream_t s);
// `order`: 0 orders only buckets of more than 32 members (enough for strict
// queries with a 32-candidate budget), 1 orders every bucket, 2 asks each
// bucket's cloth
void self_build_triangle_hash(const View& v, const SelfVariants& sv, int nb, int order, cudaStream_t s);
void self_build_edge_hash(const View& v, const SelfVariants& sv, int nb, int order, cudaStream_t s);
// `mode`: 1 fast cloths only, 2 strict only, 0 both
void self_neighbors(const View& v, int mode, const SelfVariants& sv, cudaStream_t s);
void self_vv(const View& v, const SelfVariants& sv, cudaStream_t s);
void self_vt(const View& v, const SelfVariants& sv, cudaStream_t s);
void self_ee(const View& v, const SelfVariants& sv, cudaStream_t s);
void self_island(const View& v, const SelfVariants& sv, cudaStream_t s);
void self_apply(const View& v, const SelfVariants& sv, cudaStream_t s);

}  // namespace xg
