// Host-side solver object shared by the C entry points (xpbd_abi.cu) and the
// solver implementation (xpbd_host.cu).
//
// One Solver holds K >= 1 independent cloths concatenated in every device
// array: cloth k owns vertices [vstart, vstart + V), edges, triangles, bends
// and tethers likewise, and its own ranges of the self-collision bucket
// tables.  An ABI41 handle is a solver of one cloth; the batch entry points
// create solvers of many.  Every cloth of a solver steps with the same
// substeps / iterations, in one launch sequence captured as one CUDA graph.
#pragma once

#include <atomic>
#include <chrono>
#include <map>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/ssbl_xpbd_cuda.h"
#include "../../include/xpbd_gb300.h"
#include "xpbd_solver.cuh"

namespace xg {
namespace host {

constexpr int kMaxFieldRecords = 64;  // force fields per cloth (abi41.cu:166)

extern thread_local std::string g_error;
// Device bytes of the solver being built or updated on this thread: every
// successful dalloc adds to it while an AllocAccount is in scope.
extern thread_local long long* g_alloc_account;
// Cell-key division given to solvers and shared scenes when they are created
// (0 the reference's, 1 IEEE; xpbd_math.cuh).
extern std::atomic<int> g_default_key_ieee;

struct AllocAccount {
    long long* prev;
    explicit AllocAccount(long long* target) : prev(g_alloc_account) { g_alloc_account = target; }
    ~AllocAccount() { g_alloc_account = prev; }
};

inline bool fail(const std::string& msg) {
    g_error = msg.empty() ? std::string("unknown GB300 XPBD error") : msg;
    return false;
}

inline bool cuda_ok(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return true;
    g_error = std::string(what) + ": " + cudaGetErrorString(err);
    return false;
}

template <class T>
bool dalloc(T** p, size_t n, const char* what) {
    *p = nullptr;
    if (n == 0) return true;
    if (!cuda_ok(cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * n), what)) return false;
    if (g_alloc_account) *g_alloc_account += (long long)(sizeof(T) * n);
    return true;
}

template <class T>
bool dupload(T* dst, const T* src, size_t n, cudaStream_t s, const char* what) {
    if (n == 0) return true;
    return cuda_ok(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, s), what);
}

inline int next_pow2(int value) {
    int r = 1;
    value = value < 1 ? 1 : value;
    while (r < value && r < (1 << 30)) r <<= 1;
    return r;
}

inline double ms_since(std::chrono::high_resolution_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
}

// Kernel kinds of the per-kernel profile (xpbd_gb300_profile_frame).
enum KernelKind {
    kKPredict = 0,
    kKStretchPass = 1,   // stretch gather + per-vertex contact stages
    kKVertexPass = 2,    // tether / Jacobi-bend gather or stages only
    kKBendColor = 3,
    kKVertexHash = 4,
    kKTriangleHash = 5,
    kKEdgeHash = 6,
    kKNeighbors = 7,
    kKVertexVertex = 8,
    kKVertexTriangle = 9,
    kKEdgeEdge = 10,
    kKIsland = 11,
    kKSelfApply = 12,
    kKCopy = 13,
    kKPcg = 14,          // CG solve (build + 8 iterations)
    kKStretchCaps = 15,  // averaged polish and colour-range ratio caps
    kKDynamic = 16,      // dynamic-collider contacts
    kKinds = 17
};

struct GraphKey {
    int substeps, iterations, analytic, sdf, normals;
    int dyn;  // bit 0: some cloth has unsigned dynamic colliders, bit 1: signed
    bool operator<(const GraphKey& o) const {
        return std::tie(substeps, iterations, analytic, sdf, normals, dyn) <
               std::tie(o.substeps, o.iterations, o.analytic, o.sdf, o.normals, o.dyn);
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    long long cache_hits = 0, cache_misses = 0;
    long long pcg_solves = 0;
};

struct FrameStats {
    long long launches = 0;
    long long cache_hits = 0, cache_misses = 0;
    long long pcg_solves = 0;
};

// Optional per-launch event pairs, recorded when profiling a frame.
struct Profile {
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
};

// A static SDF grid on the device, shared by every cloth whose collider
// triangles and SDF settings are identical (serving many requests against
// the same collider builds its grid once).  Reference counted.
struct SdfGrid {
    int device = 0;
    std::vector<float> tris;      // the collider triangles it was built from
    float voxel_setting = 0.0f;   // config values that size the grid
    int band = 0, max_res = 0;
    float margin = 0.0f;
    float* sdf = nullptr;
    float4* tris_dev = nullptr;
    int dim[3] = {0, 0, 0};
    float origin[3] = {0.0f, 0.0f, 0.0f};
    float voxel = 0.0f;
    int is_signed = 0;
    long long bytes = 0;
    int refs = 0;
};

// Dynamic colliders of one cloth: device buffers (grown, never shrunk) and
// the descriptor the kernels read.
struct DynHost {
    DynSet h{};                   // host copy of the descriptor
    DynSet* dev = nullptr;        // device copy (Params.dyn)
    float4* tris = nullptr;       // 3 rows per triangle
    float4* verts = nullptr;      // indexed mesh vertices
    int* idx = nullptr;           // indexed mesh triples
    float4 *amin = nullptr, *amax = nullptr, *center = nullptr, *prev_center = nullptr;
    float* radius = nullptr;
    int4 *cmin = nullptr, *cmax = nullptr;
    int* large = nullptr;
    int *lflag = nullptr, *lpos = nullptr;  // large flags and their scan
    int *tcount = nullptr, *tstart = nullptr, *tent = nullptr, *scan_tmp = nullptr;
    int* small = nullptr;         // large count, max bucket occupancy
    float4 *ppos = nullptr, *pprev = nullptr;
    float* prad = nullptr;
    int4* pcell = nullptr;
    int *pcount = nullptr, *pstart = nullptr, *pent = nullptr, *pscan = nullptr;
    int tris_cap = 0, verts_cap = 0, idx_cap = 0, bounds_cap = 0, tb_cap = 0, tent_cap = 0;
    int par_cap = 0, pb_cap = 0;
    int tri_upload_count = 0;     // triangles of the last upload (motion continuity)
    int topology_count = -1;      // triangles of the uploaded index buffer
    int par_upload_count = 0;
    unsigned long long radius_signature = 0;
    int large_count = 0;          // triangles spanning more than 64 cells
    int max_occupancy = 0;        // largest bucket of the triangle hash
};

struct Solver;

// Shared dynamic scene: colliders of many sources (other cloths' proxies,
// props) hashed once, read by every attached cloth with its own source
// filter.  Updates wait for the device to be idle, so no attached solver's
// frame reads it while it changes.
struct GlobalScene {
    DynHost dyn;
    int *tri_src = nullptr, *tri_layer = nullptr, *par_src = nullptr, *par_layer = nullptr;
    int tri_meta_cap = 0, par_meta_cap = 0;
    unsigned long long* overflow = nullptr;  // particles past the 16 queried slots of a bucket
    float margin = 0.0f, thickness = 0.0f;
    int key_ieee = 0;  // cell-key division of the scene's hashes (xpbd_math.cuh)
    long long hash_overflow = 0;
    float upload_ms = 0.0f;
    long long device_bytes = 0;
    cudaStream_t stream = nullptr;
    std::set<std::pair<Solver*, int>> attached;  // (solver, cloth) pairs reading it
};

// Host-side state of one cloth of a solver.
struct Cloth {
    SsblXpbdConfig cfg{};               // sanitised copy of the caller's config
    SsblXpbdRuntimeColliders colliders{};
    std::vector<int> bend_colors;       // caller's colour offsets (local)
    std::vector<int> edge_colors;
    bool self_enabled = false;          // self collision on with a positive radius
    int interval = 1, passes = 1;       // self-collision schedule
    bool fast = false;
    bool order_buckets = true;          // queries depend on bucket member order
    // static SDF of this cloth's collider (shared grid, null when none)
    SdfGrid* grid = nullptr;
    long long sdf_rebuilds = 0, sdf_unsigned = 0;
    float sdf_build_ms = 0.0f;
    int pin_count = 0;
    int wing_count = 0;
    int force_field_count = 0;
    int unsupported_force_field_count = 0;
    SsblXpbdForceField* fields_dev = nullptr;  // device copy of the cloth's force fields
    int fields_capacity = 0;
    bool pressure_on = false;
    DynHost dyn;
    GlobalScene* gscene = nullptr;      // attached shared scene (may be detached: gd_mode 0)
};

struct Solver {
    int K = 0;
    int key_ieee = 0;  // cell-key division (xpbd_math.cuh): 0 the reference's, 1 IEEE
    // Cloths are stored grouped by self-collision mode (none, fast, strict;
    // caller order within a group) so that each mode-specific kernel covers
    // contiguous items.  The batch entry points take the caller's cloth
    // index (ext2int maps it); concatenated whole-handle transfers use the
    // caller's order (ext_vstart: vertex offsets in that order).
    bool permuted = false;
    std::vector<int> ext2int, int2ext, ext_vstart;
    std::vector<Cloth> cl;
    std::vector<Params> hp;     // one per cloth
    Params* dp = nullptr;
    bool params_dirty = true;
    cudaStream_t stream = nullptr;
    // side streams for independent self-collision work (captured into the
    // frame graph as parallel branches), with fork / join events
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[3] = {nullptr, nullptr, nullptr};

    int nV = 0, nE = 0, nT = 0, nB = 0, nL = 0;   // totals over the cloths
    int nVB = 0, nTB = 0, nEB = 0;                // total bucket counts
    int* vcloth = nullptr;                        // cloth maps (K > 1 only)
    int* ecloth = nullptr;
    int* tcloth = nullptr;

    float4* pos[2] = {nullptr, nullptr};
    float4* prev = nullptr;
    float4* vel = nullptr;
    float4* rest = nullptr;  // .w = effective inverse mass
    float* inv_mass = nullptr;
    int* sp_off = nullptr;
    int2* sp_ent = nullptr;
    int* te_off = nullptr;
    int2* te_ent = nullptr;
    int* vt_off = nullptr;  // vertex -> incident triangles (normals for pressure / fields)
    int* vt_tri = nullptr;
    float* p_area = nullptr;  // volume pressure per vertex (any cloth with pressure)
    float* p_rest = nullptr;
    int* bj_off = nullptr;  // bends as a Jacobi gather (cloths without colours)
    int2* bj_ent = nullptr;
    int2* bends = nullptr;  // coloured bends merged by (colour, cloth)
    float* bend_rest = nullptr;
    int4* tris = nullptr;
    int2* edges = nullptr;
    float* edge_rest = nullptr;
    float4* pin_target = nullptr;
    float* pin_weight = nullptr;
    float* pin_relax = nullptr;
    unsigned long long* counts = nullptr;
    unsigned* max_delta_bits = nullptr;
    float* pack = nullptr;

    std::vector<float> h_w;      // effective inverse mass per vertex
    std::vector<float> h_inv;    // inverse mass as given
    std::vector<float> h_pin_weight;
    std::vector<float4> h_pin_target;
    std::vector<float> h_pin_relax;
    int pin_relax_iterations = -1;
    // pin updates: current pinned vertices, change marks, device staging
    std::vector<int> pin_set, pin_changed, pin_mark, pin_kept;
    int pin_epoch = 0;
    std::vector<float4> h_stage_target;
    std::vector<float> h_stage_weight, h_stage_relax;
    int* stage_idx = nullptr;
    float4* stage_target = nullptr;
    float* stage_weight = nullptr;
    float* stage_relax = nullptr;
    int stage_capacity = 0;
    std::vector<int> bend_colors;   // merged colour offsets into `bends`
    bool jacobi_bends = false;      // some cloth gathers its bends

    // self collision
    bool self_any = false;
    int4* vcell = nullptr;
    int *vb_count = nullptr, *vb_start = nullptr, *vb_ent = nullptr;
    int *tb_count = nullptr, *tb_start = nullptr, *tb_ent = nullptr;
    int *eb_count = nullptr, *eb_start = nullptr, *eb_ent = nullptr;
    int *eb_slot = nullptr, *eb_ovf_list = nullptr, *eb_ovf_count = nullptr, *eb_ovf_start = nullptr;
    unsigned* eb_ovf_bits = nullptr;
    long long eb_ovf_cap = 0;  // entries of eb_ovf_list
    int2* eb_late = nullptr;   // insertions past a bucket's slots, as (bucket, edge)
    unsigned long long* eb_late_count = nullptr;
    long long eb_late_cap = 0;
    int* nb_count = nullptr;
    int* nb_idx = nullptr;
    int* scan_tmp = nullptr;  // three segments: vertex, triangle, edge hash scans
    int* trim_list = nullptr;  // three segments: buckets of more than 32 members per hash
    int* trim_count = nullptr; // three list lengths
    int scan_seg = 0;
    Acc4* acc = nullptr;
    unsigned long long* perf = nullptr;  // kPerfSlots work counters of a profiled frame

    // hard-stretch optimisation (every cloth that enables it)
    bool pcg_on = false;         // some cloth runs the CG stretch solve
    bool pcg_hard = false;       // some cloth runs the averaged polish and caps
    bool cap_jacobi = false;     // some such cloth has no edge colouring (Jacobi caps)
    bool spring_any = false;     // some cloth with edges keeps the spring gather
    PcgView pcg{};
    int* pcg_blk = nullptr;      // cloth of each block of the CG grid
    int pcg_blocks = 0;          // CG grid: the one-cloth grids of those cloths end to end
    int2* cap_edges = nullptr;   // edges sorted by colour for the caps (colours of all cloths merged)
    float* cap_rest = nullptr;
    int cap_count = 0;
    std::vector<int> cap_colors; // colour offsets into cap_edges
    int pcg_nnz = 0;
    long long pcg_iterations = 0;

    LaunchTune tune{};           // launch configuration (0 = default per slot)
    // fused frames (cloths small enough for one block each): the recorded
    // operations per frame schedule, and each cloth's bends per colour
    std::vector<FrameOp>* rec = nullptr;  // set while recording a frame's operations
    bool rec_unsupported = false;         // a launch without a fused form was recorded
    std::map<GraphKey, std::pair<FrameOp*, int>> fused_ops;
    std::vector<int2> h_bend_ranges;      // [colours x K]: first bend, count
    int2* bend_ranges = nullptr;
    long long device_bytes = 0;  // sum of the solver's device allocations
    std::map<GraphKey, GraphEntry> graphs;
    bool use_graphs = true;
    long long last_launches = 0;
    SsblXpbdDiagnostics diag{};

    View view() const;
    void drop_graphs();
};

// Creation of a solver for `count` cloths (count == 1: the ABI41 handle).
// Returns nullptr with g_error set on failure.
Solver* create_solver(const SsblXpbdConfig* configs, const SsblXpbdMesh* meshes, int count);
void free_solver(Solver* S);
void reset_edge_hash(Solver* S, cudaStream_t s);
void reset_triangle_hash(Solver* S, cudaStream_t s);

// Cloth-level updates; cloth < 0 applies to every cloth (pins then take
// indices over the concatenated vertices).
bool upload_pins(Solver* S, int cloth, const int* indices, const float* positions, const float* weights, int count);
bool set_colliders(Solver* S, int cloth, const SsblXpbdRuntimeColliders& c);
bool upload_static(Solver* S, int cloth, const float* tris, int count);
bool upload_fields(Solver* S, int cloth, const SsblXpbdForceField* fields, int count, int unsupported);
bool upload_positions(Solver* S, int cloth, const float* positions, int max_floats);
bool download_positions(Solver* S, int cloth, float* out, int max_floats);
bool reset_cloths(Solver* S, int cloth);
bool set_active(Solver* S, int cloth, bool active);
// Dynamic colliders of a cloth (cloth < 0: every cloth), replaced on each
// upload; defined in xpbd_dynamic.cu.
bool upload_dynamic_triangles(Solver* S, int cloth, const float* tris, int count);
bool upload_dynamic_indexed(Solver* S, int cloth, const float* verts, int vcount, const int* idx, int count,
                            bool topology_changed);
bool upload_dynamic_particles(Solver* S, int cloth, const float* pos, const float* radii, int count);
void free_dynamic(Cloth& C);
// Shared dynamic scene (xpbd_dynamic.cu).  cloth < 0 attaches / detaches
// every cloth of the solver.
GlobalScene* scene_create();
void scene_destroy(GlobalScene* G);
bool scene_update(GlobalScene* G, const SsblXpbdGlobalDynamicSceneInputs* in);
bool scene_attach(Solver* S, int cloth, GlobalScene* G, int source_id, int layer, int mode);
void scene_detach(Solver* S, int cloth);
void sdf_diagnostics(Solver* S);

// One frame: prepare parameters, launch (graph or direct), optionally fetch.
bool prepare_step(Solver* S, int substeps, int iterations);
bool run_frame(Solver* S, int substeps, int iterations, FrameStats* st);
bool prepare_graph(Solver* S, int substeps, int iterations);  // capture without launching
void enqueue_frame(Solver* S, int substeps, int iterations, FrameStats* st, Profile* prof = nullptr);
bool fetch_counts(Solver* S, const FrameStats& st);
bool sync_params(Solver* S);
bool step(Solver* S, int substeps, int iterations, int fetch_diagnostics, int force_sync);

// PC2 point-cache writer of one cloth (cloth < 0: all vertices), in
// xpbd_pc2.cu.
void* pc2_open(Solver* S, int cloth, const char* path, int start_frame);
bool pc2_write(Solver* S, void* writer, const float* matrix16);
long long pc2_close(void* writer, bool commit);

// Launch configuration: set (validated; captured graphs are dropped) and the
// autotuner, which measures profiled frames from the current state (restored
// after every trial and at the end, so tuning changes no result) and keeps
// the configuration with the shortest frame.  ms_out: {tuned, default}.
bool set_launch_config(Solver* S, const int* values, int n);
int effective_tune(const Solver* S, int slot);
bool autotune(Solver* S, int substeps, int iterations, int rounds, float* ms_out);
// One profiled frame: per-kind milliseconds and launches (kinds >= kKinds).
bool profile_frame(Solver* S, int substeps, int iterations, float* kernel_ms, long long* kernel_launches, int kinds);

}  // namespace host
}  // namespace xg
