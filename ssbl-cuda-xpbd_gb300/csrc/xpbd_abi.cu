// Host side of the GB300 XPBD library: the ABI41 C entry points, solver
// creation (CSR builds, hash sizing, static SDF), and the per-frame launch
// schedule, captured once per configuration as a CUDA graph.
//
// Entry points replace native/src/ssbl_xpbd_cuda_abi41.cu:8791-9432 with the
// same return convention (1 / 0, NULL on failed create) and the same error
// strings where the reference defines them.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/ssbl_xpbd_cuda.h"
#include "../../include/xpbd_gb300.h"
#include "xpbd_solver.cuh"

static_assert(sizeof(SsblXpbdConfig) == 224, "SsblXpbdConfig layout");
static_assert(sizeof(SsblXpbdDiagnostics) == 992, "SsblXpbdDiagnostics layout");
static_assert(sizeof(SsblXpbdFrameInputs) == 240, "SsblXpbdFrameInputs layout");
static_assert(sizeof(SsblXpbdForceField) == 132, "SsblXpbdForceField layout");

using namespace xg;

namespace {

thread_local std::string g_error;

bool fail(const char* msg) {
    g_error = msg ? msg : "unknown GB300 XPBD error";
    return false;
}

bool cuda_ok(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return true;
    g_error = std::string(what) + ": " + cudaGetErrorString(err);
    return false;
}

template <class T>
bool dalloc(T** p, size_t n, const char* what) {
    *p = nullptr;
    if (n == 0) return true;
    return cuda_ok(cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * n), what);
}

template <class T>
bool dupload(T* dst, const T* src, size_t n, cudaStream_t s, const char* what) {
    if (n == 0) return true;
    return cuda_ok(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, s), what);
}

int next_pow2(int value) {
    int r = 1;
    value = std::max(value, 1);
    while (r < value && r < (1 << 30)) r <<= 1;
    return r;
}

double ms_since(std::chrono::high_resolution_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
}

// Vertex -> constraint CSR: for each vertex the incident constraints in
// increasing constraint index, tagged with the vertex's side (bit 31 set when
// the vertex is the constraint's second endpoint).
void build_pair_csr(int V, const std::vector<int2>& pairs, const std::vector<float>& rest, std::vector<int>* off,
                    std::vector<int2>* ent) {
    off->assign(V + 1, 0);
    for (const int2& p : pairs) {
        if (p.x < 0 || p.y < 0 || p.x >= V || p.y >= V || p.x == p.y) continue;
        (*off)[p.x + 1]++;
        (*off)[p.y + 1]++;
    }
    for (int i = 0; i < V; ++i) (*off)[i + 1] += (*off)[i];
    ent->assign((*off)[V], make_int2(0, 0));
    std::vector<int> cur(off->begin(), off->end() - 1);
    for (size_t k = 0; k < pairs.size(); ++k) {
        const int2 p = pairs[k];
        if (p.x < 0 || p.y < 0 || p.x >= V || p.y >= V || p.x == p.y) continue;
        int bits;
        std::memcpy(&bits, &rest[k], 4);
        (*ent)[cur[p.x]++] = make_int2(p.y, bits);
        (*ent)[cur[p.y]++] = make_int2(p.x | kSideBit, bits);
    }
}

// Closed-mesh test for the SDF sign: weld vertices on a 1e-6 grid and require
// every undirected edge to have exactly two incident triangles
// (abi41.cu:6026-6063).
struct QKey {
    long long x, y, z;
    bool operator==(const QKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct QKeyHash {
    size_t operator()(const QKey& k) const {
        uint64_t h = (uint64_t)k.x * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)k.y + 0x632BE59BD9B4E019ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)k.z + 0x85EBCA77C2B2AE63ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

bool mesh_is_closed(const float* tris, int count) {
    if (!tris || count <= 0) return false;
    std::unordered_map<QKey, int, QKeyHash> ids;
    std::unordered_map<uint64_t, int> edges;
    auto vid = [&](const float* v) {
        const QKey k{std::llround((double)v[0] * 1000000.0), std::llround((double)v[1] * 1000000.0),
                     std::llround((double)v[2] * 1000000.0)};
        auto it = ids.find(k);
        if (it != ids.end()) return it->second;
        const int id = (int)ids.size();
        ids.emplace(k, id);
        return id;
    };
    auto ekey = [](int a, int b) {
        const unsigned lo = (unsigned)std::min(a, b), hi = (unsigned)std::max(a, b);
        return ((uint64_t)lo << 32) | hi;
    };
    for (int t = 0; t < count; ++t) {
        const float* p = tris + t * 9;
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(p[k])) return false;
        const int a = vid(p), b = vid(p + 3), c = vid(p + 6);
        if (a == b || b == c || c == a) continue;
        edges[ekey(a, b)] += 1;
        edges[ekey(b, c)] += 1;
        edges[ekey(c, a)] += 1;
    }
    if (edges.empty()) return false;
    for (const auto& e : edges)
        if (e.second != 2) return false;
    return true;
}

struct GraphKey {
    int substeps, iterations, analytic, sdf;
    bool operator<(const GraphKey& o) const {
        return std::tie(substeps, iterations, analytic, sdf) < std::tie(o.substeps, o.iterations, o.analytic, o.sdf);
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    long long cache_hits = 0, cache_misses = 0;
    long long pcg_solves = 0;
};

struct Solver {
    SsblXpbdConfig cfg{};
    SsblXpbdRuntimeColliders colliders{};
    Params hp{};
    Params* dp = nullptr;
    bool params_dirty = true;
    cudaStream_t stream = nullptr;

    float4* pos[2] = {nullptr, nullptr};
    float4* prev = nullptr;
    float4* vel = nullptr;
    float4* rest = nullptr;  // .w = effective inverse mass
    float* inv_mass = nullptr;
    int* sp_off = nullptr;
    int2* sp_ent = nullptr;
    int* te_off = nullptr;
    int2* te_ent = nullptr;
    int* bj_off = nullptr;  // bends as a Jacobi gather (no colours given)
    int2* bj_ent = nullptr;
    int2* bends = nullptr;
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
    int pin_count = 0;
    int pin_relax_iterations = -1;
    std::vector<int> edge_colors, bend_colors;

    // static SDF
    float* sdf = nullptr;
    int sdf_capacity = 0;
    float4* static_tris = nullptr;
    int static_capacity = 0;
    long long sdf_rebuilds = 0, sdf_unsigned = 0;
    float sdf_build_ms = 0.0f;

    // self collision
    bool self_on = false;
    int4* vcell = nullptr;
    int *vb_count = nullptr, *vb_start = nullptr, *vb_ent = nullptr;
    int *tb_count = nullptr, *tb_start = nullptr, *tb_ent = nullptr;
    int *eb_count = nullptr, *eb_start = nullptr, *eb_ent = nullptr;
    int* nb_count = nullptr;
    int* nb_idx = nullptr;
    int* scan_tmp = nullptr;
    Acc4* acc = nullptr;

    // dynamic colliders (accepted, see step)
    int dynamic_triangle_count = 0;
    int dynamic_particle_count = 0;
    int force_field_count = 0;
    int unsupported_force_field_count = 0;

    int wing_count = 0;  // triangle pairs sharing an edge (bending wings)

    // hard-stretch optimisation (CG solve and caps)
    bool pcg_on = false;
    PcgView pcg{};
    int2* cap_edges = nullptr;   // edges sorted by colour for the caps
    float* cap_rest = nullptr;
    std::vector<int> cap_colors; // colour offsets into cap_edges
    int pcg_nnz = 0;
    long long pcg_iterations = 0;

    std::map<GraphKey, GraphEntry> graphs;
    bool use_graphs = true;
    long long last_launches = 0;
    SsblXpbdDiagnostics diag{};

    View view() const {
        View v{};
        v.P = dp;
        v.pos_in = pos[0];
        v.pos = pos[0];
        v.prev = prev;
        v.vel = vel;
        v.rest = rest;
        v.inv_mass = inv_mass;
        v.sp_off = sp_off;
        v.sp_ent = sp_ent;
        v.te_off = te_off;
        v.te_ent = te_ent;
        v.bj_off = bj_off;
        v.bj_ent = bj_ent;
        v.bends = bends;
        v.bend_rest = bend_rest;
        v.tris = tris;
        v.edges = edges;
        v.edge_rest = edge_rest;
        v.pin_target = pin_target;
        v.pin_weight = pin_weight;
        v.pin_relax = pin_relax;
        v.counts = counts;
        v.sdf = sdf;
        v.static_tris = static_tris;
        v.vcell = vcell;
        v.vb_count = vb_count;
        v.vb_start = vb_start;
        v.vb_ent = vb_ent;
        v.tb_count = tb_count;
        v.tb_start = tb_start;
        v.tb_ent = tb_ent;
        v.eb_count = eb_count;
        v.eb_start = eb_start;
        v.eb_ent = eb_ent;
        v.nb_count = nb_count;
        v.nb_idx = nb_idx;
        v.scan_tmp = scan_tmp;
        v.acc = acc;
        v.max_delta_bits = max_delta_bits;
        return v;
    }

    void drop_graphs() {
        for (auto& g : graphs)
            if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
        graphs.clear();
    }
};

void free_solver(Solver* S) {
    if (!S) return;
    if (S->stream) cudaStreamSynchronize(S->stream);
    S->drop_graphs();
    void* ptrs[] = {S->dp,        S->pos[0],   S->pos[1],     S->prev,     S->vel,       S->rest,       S->inv_mass,
                    S->sp_off,    S->sp_ent,   S->te_off,     S->te_ent,   S->bj_off,    S->bj_ent,     S->bends,
                    S->bend_rest, S->tris,     S->edges,      S->edge_rest, S->pin_target, S->pin_weight, S->pin_relax,
                    S->counts,    S->max_delta_bits, S->pack, S->sdf,      S->static_tris, S->vcell,    S->vb_count,
                    S->vb_start,  S->vb_ent,   S->tb_count,   S->tb_start, S->tb_ent,    S->eb_count,   S->eb_start,
                    S->eb_ent,    S->nb_count, S->nb_idx,     S->acc,      S->scan_tmp,  S->pcg.diag,   S->pcg.pinv,
                    S->pcg.r,     S->pcg.z,    S->pcg.d,      S->pcg.q,    S->pcg.offdiag, S->pcg.avg,  S->pcg.red,
                    S->pcg.partials, S->pcg.ticket, S->pcg.guard, S->pcg.max_delta_bits, S->cap_edges, S->cap_rest};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

float self_radius(const SsblXpbdConfig& c) {
    const float req = std::max(c.self_collision_distance, 0.0f);
    if (req > 0.0f) return req;
    return std::max(std::max(c.cloth_thickness, c.collision_margin), 0.0f);
}

void load_colliders(Solver* S) {
    Params& P = S->hp;
    const SsblXpbdRuntimeColliders& c = S->colliders;
    P.use_ground = c.use_ground;
    P.ground_height = c.ground_height;
    P.use_wall = c.use_wall;
    std::memcpy(P.wall_origin, c.wall_origin, sizeof(P.wall_origin));
    std::memcpy(P.wall_normal, c.wall_normal, sizeof(P.wall_normal));
    P.use_sphere = c.use_sphere;
    std::memcpy(P.sphere_center, c.sphere_center, sizeof(P.sphere_center));
    P.sphere_radius = c.sphere_radius;
    S->params_dirty = true;
}

bool sync_params(Solver* S) {
    if (!S->params_dirty) return true;
    if (!cuda_ok(cudaMemcpyAsync(S->dp, &S->hp, sizeof(Params), cudaMemcpyHostToDevice, S->stream), "upload solver parameters"))
        return false;
    S->params_dirty = false;
    return true;
}

// Soft-pin relaxation 1 - (1 - clamp(w / 0.75))^(1/(I+1)) (abi41.cu:3466-3477).
float pin_soft_relaxation(float weight, float exponent) {
    if (!std::isfinite(weight) || weight < 0.05f) return 0.0f;
    const float total = std::min(std::max(weight / 0.75f, 0.0f), 1.0f);
    if (total >= 1.0f) return 1.0f;
    const float remaining = std::max(1.0f - total, 0.0f);
    const float relax = 1.0f - std::pow(remaining, std::max(exponent, 1.0e-4f));
    return std::isfinite(relax) ? std::min(std::max(relax, 0.0f), 1.0f) : total;
}

bool upload_pin_relax(Solver* S, int iterations) {
    if (S->pin_relax_iterations == iterations) return true;
    const int V = S->cfg.vertex_count;
    const float exponent = 1.0f / (float)std::max(iterations + 1, 1);
    for (int i = 0; i < V; ++i) S->h_pin_relax[i] = pin_soft_relaxation(S->h_pin_weight[i], exponent);
    if (!dupload(S->pin_relax, S->h_pin_relax.data(), V, S->stream, "pin relaxation upload")) return false;
    S->pin_relax_iterations = iterations;
    return true;
}

bool upload_pins(Solver* S, const int* indices, const float* positions, const float* weights, int count) {
    if (!S) return fail("invalid solver handle");
    if (count < 0) return fail("invalid pin count");
    const int V = S->cfg.vertex_count;
    if (count > 0 && (!indices || !positions)) return fail("pin arrays are required when pin count is nonzero");
    std::fill(S->h_pin_weight.begin(), S->h_pin_weight.end(), -1.0f);
    for (int k = 0; k < count; ++k) {
        const int i = indices[k];
        if (i < 0 || i >= V) continue;
        S->h_pin_weight[i] = weights ? weights[k] : 1.0f;
        S->h_pin_target[i] = make_float4(positions[k * 3 + 0], positions[k * 3 + 1], positions[k * 3 + 2], 0.0f);
    }
    S->pin_count = count;
    S->pin_relax_iterations = -1;
    return dupload(S->pin_weight, S->h_pin_weight.data(), V, S->stream, "pin weight upload") &&
           dupload(S->pin_target, S->h_pin_target.data(), V, S->stream, "pin target upload") &&
           cuda_ok(cudaStreamSynchronize(S->stream), "pin upload");
}

// Static SDF: grid sizing (abi41.cu:6123-6218) and the device build.
bool build_static_sdf(Solver* S, const float* tris, int count) {
    Params& P = S->hp;
    P.sdf_ready = 0;
    P.sdf_dim[0] = P.sdf_dim[1] = P.sdf_dim[2] = 0;
    P.sdf_origin[0] = P.sdf_origin[1] = P.sdf_origin[2] = 0.0f;
    P.sdf_voxel = 0.0f;
    P.sdf_signed = 0;
    P.static_tri_count = std::max(count, 0);
    S->params_dirty = true;
    S->sdf_build_ms = 0.0f;
    if (count <= 0) return true;
    if (!tris) return fail("static triangle data is required for SDF build");
    const auto t0 = std::chrono::high_resolution_clock::now();
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < count * 3; ++k) {
        const float* v = tris + k * 3;
        if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2]))
            return fail("static triangle data contains non-finite coordinates");
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], v[a]);
            hi[a] = std::max(hi[a], v[a]);
        }
    }
    const SsblXpbdConfig& c = S->cfg;
    float voxel = (std::isfinite(c.static_sdf_voxel_size) && c.static_sdf_voxel_size > 0.0f)
                      ? c.static_sdf_voxel_size
                      : std::max(std::max(c.collision_margin, 0.0f) * 0.5f, 0.002f);
    const int band = std::max(c.static_sdf_band_voxels > 0 ? c.static_sdf_band_voxels : 4, 1);
    const int max_res = std::max(c.static_sdf_max_resolution > 0 ? c.static_sdf_max_resolution : 160, 16);
    const float margin = std::max(c.collision_margin, 0.0f);
    const float expand = margin + (float)band * voxel + voxel * 2.0f;
    float ext[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = lo[a] - expand;
        hi[a] = hi[a] + expand;
        ext[a] = std::max(hi[a] - lo[a], voxel);
    }
    const float largest = std::max(ext[0], std::max(ext[1], ext[2]));
    if (largest / voxel + 1.0f > (float)max_res) voxel = largest / (float)std::max(max_res - 1, 1);
    voxel = std::max(voxel, 1.0e-5f);
    int dim[3];
    for (int a = 0; a < 3; ++a) dim[a] = std::min(std::max((int)std::ceil(ext[a] / voxel) + 1, 2), max_res);
    const long long voxels_ll = (long long)dim[0] * dim[1] * dim[2];
    if (voxels_ll <= 0 || voxels_ll > 0x7fffffffll) return fail("static SDF grid is too large");
    const int voxels = (int)voxels_ll;
    if (voxels > S->sdf_capacity) {
        cudaFree(S->sdf);
        S->sdf = nullptr;
        S->sdf_capacity = 0;
        S->drop_graphs();
        if (!dalloc(&S->sdf, voxels, "static SDF allocation")) return false;
        S->sdf_capacity = voxels;
    }
    if (count > S->static_capacity) {
        cudaFree(S->static_tris);
        S->static_tris = nullptr;
        S->static_capacity = 0;
        S->drop_graphs();
        if (!dalloc(&S->static_tris, (size_t)count * 3, "static triangle upload")) return false;
        S->static_capacity = count;
    }
    std::vector<float4> t4((size_t)count * 3);
    for (int k = 0; k < count * 3; ++k) t4[k] = make_float4(tris[k * 3], tris[k * 3 + 1], tris[k * 3 + 2], 0.0f);
    if (!dupload(S->static_tris, t4.data(), t4.size(), S->stream, "static triangle upload")) return false;
    for (int a = 0; a < 3; ++a) {
        P.sdf_dim[a] = dim[a];
        P.sdf_origin[a] = lo[a];
    }
    P.sdf_voxel = voxel;
    P.sdf_signed = mesh_is_closed(tris, count) ? 1 : 0;
    if (!P.sdf_signed) S->sdf_unsigned += 1;
    if (!sync_params(S)) return false;
    launch_sdf_build(S->view(), voxels, S->stream);
    if (!cuda_ok(cudaGetLastError(), "build static SDF") || !cuda_ok(cudaStreamSynchronize(S->stream), "sync static SDF build"))
        return false;
    P.sdf_ready = 1;
    S->params_dirty = true;
    S->sdf_rebuilds += 1;
    S->sdf_build_ms = (float)ms_since(t0);
    return true;
}

// Static SDF fields of the diagnostics block (abi41.cu:6105-6121).
void sdf_diagnostics(Solver* S) {
    SsblXpbdDiagnostics& d = S->diag;
    const Params& P = S->hp;
    d.static_triangle_count = P.static_tri_count;
    d.static_sdf_rebuild_count = S->sdf_rebuilds;
    d.static_sdf_unsigned_fallback_count = S->sdf_unsigned;
    d.static_sdf_build_ms = S->sdf_build_ms;
    d.static_sdf_grid_x = P.sdf_dim[0];
    d.static_sdf_grid_y = P.sdf_dim[1];
    d.static_sdf_grid_z = P.sdf_dim[2];
    d.static_sdf_voxel_count = P.sdf_ready ? (long long)P.sdf_dim[0] * P.sdf_dim[1] * P.sdf_dim[2] : 0;
}

bool upload_static(Solver* S, const float* tris, int count) {
    if (!S) return fail("invalid static triangle update");
    count = std::max(count, 0);
    S->cfg.static_triangle_count = count;
    if (count > 0 && !tris) return fail("static triangle data is required when triangle count is nonzero");
    const bool ok = build_static_sdf(S, tris, count);
    sdf_diagnostics(S);
    return ok;
}

// Number of bending wings: triangle pairs on an edge with distinct opposite
// vertices (abi41.cu:7193-7302).  Reported in the diagnostics only.
int count_wings(int V, const std::vector<int4>& tris) {
    std::unordered_map<uint64_t, int> first_opposite;
    int wings = 0;
    for (const int4& t : tris) {
        const int ids[3] = {t.x, t.y, t.z};
        if (t.x >= V || t.y >= V || t.z >= V) continue;
        for (int e = 0; e < 3; ++e) {
            const int x = ids[e], y = ids[(e + 1) % 3], opp = ids[(e + 2) % 3];
            const uint64_t key = ((uint64_t)(unsigned)std::min(x, y) << 32) | (unsigned)std::max(x, y);
            auto it = first_opposite.find(key);
            if (it == first_opposite.end()) {
                first_opposite.emplace(key, opp);
            } else if (it->second != opp) {
                ++wings;
            }
        }
    }
    return wings;
}

// ------------------------------------------------------------ the frame --
// Kernel kinds for the per-kernel profile (xpbd_gb300_profile_frame).
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
    kKinds = 16
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

// Issue one frame: `substeps` substeps of `iterations` iterations, following
// the reference schedule (abi41.cu:9165-9376).  Per-vertex stages of an
// iteration are fused into one pass; a pass starts at every stretch /
// tether / Jacobi-bend gather and around the work that needs all vertices
// (bends by colour, self collision).
void enqueue_frame(Solver* S, int substeps, int iterations, FrameStats* st, Profile* prof = nullptr) {
    const SsblXpbdConfig& c = S->cfg;
    const Params& P = S->hp;
    const int V = c.vertex_count, E = c.edge_count, T = c.triangle_count, B = c.bend_count, L = c.lra_count;
    const float dt = c.dt / (float)substeps;
    const bool analytic = P.use_ground || P.use_wall || P.use_sphere;
    const bool sdf = P.sdf_ready != 0;
    const bool pcg = S->pcg_on;
    const bool spring = E > 0 && !pcg;
    const bool hard = pcg && P.stretch_strength >= 0.95f;
    View base = S->view();
    int cur = 0;
    unsigned pending = 0;
    int gather = 0;  // 0 none, 1 stretch, 2 tethers, 3 bends without colours
    auto timed = [&](int kind, int launches, auto&& fn) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, S->stream);
        }
        fn();
        if (prof) {
            cudaEventRecord(b, S->stream);
            prof->marks.push_back({kind, {a, b}});
        }
        st->launches += launches;
    };
    auto flush = [&]() {
        if (!pending && !gather) return;
        View v = base;
        v.pos_in = S->pos[cur];
        const unsigned gflag = gather == 1 ? kPassSpring : (gather == 2 ? kPassTether : (gather == 3 ? kPassBend : 0u));
        v.pos = gather ? S->pos[cur ^ 1] : S->pos[cur];
        timed(gather == 1 ? kKStretchPass : kKVertexPass, 1, [&] { launch_vertex_pass(v, V, dt, gflag | pending, S->stream); });
        if (gather) cur ^= 1;
        pending = 0;
        gather = 0;
    };
    auto cur_view = [&]() {
        View v = base;
        v.pos_in = S->pos[cur];
        v.pos = S->pos[cur];
        return v;
    };
    // colour-range caps over the colour-sorted edge arrays
    auto caps = [&](int kind, int passes, bool both_ways) {
        View cv = base;
        cv.pos_in = S->pos[cur];
        cv.pos = S->pos[cur];
        cv.edges = S->cap_edges;
        cv.edge_rest = S->cap_rest;
        const int ncol = (int)S->cap_colors.size() - 1;
        timed(kKStretchCaps, 0, [&] {
            for (int p = 0; p < passes; ++p) {
                for (int k = 0; k < ncol; ++k) {
                    const int n = S->cap_colors[k + 1] - S->cap_colors[k];
                    if (n > 0) {
                        pcg_cap_range(cv, S->cap_colors[k], n, dt, kind, S->stream);
                        st->launches += 1;
                    }
                }
                if (both_ways)
                    for (int k = ncol - 1; k >= 0; --k) {
                        const int n = S->cap_colors[k + 1] - S->cap_colors[k];
                        if (n > 0) {
                            pcg_cap_range(cv, S->cap_colors[k], n, dt, kind, S->stream);
                            st->launches += 1;
                        }
                    }
            }
        });
    };
    auto averaged = [&](bool tiny) {
        View av = base;
        av.pos_in = S->pos[cur];
        av.pos = S->pos[cur];
        timed(kKStretchCaps, 2, [&] { pcg_averaged_pass(av, S->pcg, V, tiny, S->stream); });
    };
    const bool self_enabled = S->self_on && c.self_collision && V > 0 && P.self_radius > 0.0f;
    const int interval = std::max(c.self_collision_interval, 1);
    const int passes = std::max(1, std::min(c.fast_self_collision_passes, 8));
    const bool fast = c.self_collision_mode == 1;
    for (int s = 0; s < substeps; ++s) {
        View pv = cur_view();
        timed(kKPredict, 1, [&] { launch_predict(pv, V, dt, S->stream); });
        for (int it = 0; it < iterations; ++it) {
            const bool last_it = it == iterations - 1;
            const bool final_c = (s == substeps - 1) && last_it;
            flush();
            if (spring) gather = 1;
            if (pcg && last_it) {
                // CG stretch solve, then (hardness >= 0.95) the averaged
                // polish with normal and tiny caps, and the extreme caps
                // (abi41.cu:9183-9201, 7806-7857, 7974-7995)
                View gv = cur_view();
                timed(kKPcg, 0, [&] { pcg_solve(gv, S->pcg, V, S->stream, &st->launches); });
                st->pcg_solves += 1;
                if (hard) {
                    for (int polish = 0; polish < 2; ++polish) {
                        averaged(false);
                        caps(0, 2, true);
                        for (int tiny = 0; tiny < 2; ++tiny) {
                            averaged(true);
                            caps(1, 3, false);
                        }
                    }
                    caps(2, 3, false);
                }
            }
            if (final_c && L > 0) {
                flush();
                gather = 2;
            }
            if (final_c && B > 0) {
                if (!S->bend_colors.empty()) {
                    flush();
                    View bv = cur_view();
                    for (size_t k = 0; k + 1 < S->bend_colors.size(); ++k) {
                        const int start = S->bend_colors[k], n = S->bend_colors[k + 1] - start;
                        if (n > 0) timed(kKBendColor, 1, [&] { launch_bend_color(bv, start, n, dt, S->stream); });
                    }
                } else {
                    flush();
                    gather = 3;
                }
            }
            pending |= kPassPin;
            if (analytic) pending |= kPassAnalytic;
            if (sdf) pending |= kPassSdf;
            const bool self_run = self_enabled && last_it && (((s + 1) % interval) == 0 || s == substeps - 1);
            if (self_run) {
                flush();
                View sv = cur_view();
                if (P.vhash)
                    timed(kKVertexHash, 6, [&] {
                        cudaMemsetAsync(S->vb_count, 0, sizeof(int) * P.vbuckets, S->stream);
                        self_build_vertex_hash(sv, V, P.vbuckets, S->stream);
                    });
                // strict queries with a 32-candidate budget do not depend on
                // the order of buckets of <= 32 members
                const bool order = fast || std::min(std::max(c.max_self_collision_neighbors, 1), 32) < 32;
                if (P.thash)
                    timed(kKTriangleHash, 6, [&] {
                        cudaMemsetAsync(S->tb_count, 0, sizeof(int) * P.tbuckets, S->stream);
                        self_build_triangle_hash(sv, T, P.tbuckets, order, S->stream);
                    });
                if (P.ehash)
                    timed(kKEdgeHash, 6, [&] {
                        cudaMemsetAsync(S->eb_count, 0, sizeof(int) * P.ebuckets, S->stream);
                        self_build_edge_hash(sv, E, P.ebuckets, order, S->stream);
                    });
                if (fast) {
                    timed(kKNeighbors, 1, [&] { self_neighbors(sv, V, P.vhash != 0, S->stream); });
                    st->cache_hits += (long long)V * (passes > 1 ? passes - 1 : 0);
                    st->cache_misses += (long long)V;
                }
                for (int pass = 0; pass < passes; ++pass) {
                    if (!fast) timed(kKNeighbors, 1, [&] { self_neighbors(sv, V, P.vhash != 0, S->stream); });
                    timed(kKVertexVertex, 1, [&] { self_vv(sv, V, !fast, S->stream); });
                    if (T > 0) timed(kKVertexTriangle, 1, [&] { self_vt(sv, V, P.thash != 0, !fast, S->stream); });
                    if (E > 0) timed(kKEdgeEdge, 1, [&] { self_ee(sv, E, P.ehash != 0, !fast, S->stream); });
                    if (pass == passes - 1 && fast && T > 0 && P.thash) timed(kKIsland, 1, [&] { self_island(sv, V, S->stream); });
                    timed(kKSelfApply, 1, [&] { self_apply(sv, V, S->stream); });
                }
            }
            // final ratio caps after the contacts (abi41.cu:9346-9350, 7997-8027)
            if (pcg && final_c && hard) {
                flush();
                caps(0, 2, true);
                caps(2, 3, false);
                caps(1, 3, false);
            }
            // Final pin polish whenever a contact stage ran (the dynamic
            // collider stage counts as running on every last iteration).
            if (analytic || sdf || last_it || self_run) pending |= kPassPinPolish;
        }
        pending |= kPassVelocity;
        flush();
    }
    if (cur != 0) timed(kKCopy, 1, [&] { launch_copy_pos(S->pos[0], S->pos[1], V, S->stream); });
}

bool run_frame(Solver* S, int substeps, int iterations, FrameStats* st) {
    if (!S->use_graphs) {
        enqueue_frame(S, substeps, iterations, st);
        return cuda_ok(cudaGetLastError(), "launch GB300 XPBD frame");
    }
    const GraphKey key{substeps, iterations,
                       (S->hp.use_ground || S->hp.use_wall || S->hp.use_sphere) ? 1 : 0, S->hp.sdf_ready};
    auto it = S->graphs.find(key);
    if (it == S->graphs.end()) {
        GraphEntry g;
        FrameStats cst;
        if (!cuda_ok(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal), "begin frame capture"))
            return false;
        enqueue_frame(S, substeps, iterations, &cst);
        cudaGraph_t graph = nullptr;
        if (!cuda_ok(cudaStreamEndCapture(S->stream, &graph), "end frame capture")) return false;
        const cudaError_t err = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (!cuda_ok(err, "instantiate frame graph")) return false;
        g.launches = cst.launches;
        g.cache_hits = cst.cache_hits;
        g.cache_misses = cst.cache_misses;
        g.pcg_solves = cst.pcg_solves;
        it = S->graphs.emplace(key, g).first;
    }
    st->launches += it->second.launches;
    st->cache_hits += it->second.cache_hits;
    st->cache_misses += it->second.cache_misses;
    st->pcg_solves += it->second.pcg_solves;
    return cuda_ok(cudaGraphLaunch(it->second.exec, S->stream), "launch frame graph");
}

bool fetch_counts(Solver* S, const FrameStats& st) {
    unsigned long long c[kCntSlots];
    unsigned mbits = 0;
    if (!cuda_ok(cudaMemcpyAsync(c, S->counts, sizeof(c), cudaMemcpyDeviceToHost, S->stream), "fetch ABI41 diagnostics") ||
        !cuda_ok(cudaMemcpyAsync(&mbits, S->max_delta_bits, sizeof(unsigned), cudaMemcpyDeviceToHost, S->stream),
                 "fetch self max smoothed delta") ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "fetch diagnostics"))
        return false;
    SsblXpbdDiagnostics& d = S->diag;
    d.abi41_soft_contact_count = (long long)c[kCntSoftContacts];
    d.abi41_exact_impulse_contact_count = (long long)c[kCntExactImpulseContacts];
    d.abi41_edge_edge_contact_count = (long long)c[kCntEdgeEdgeContacts];
    d.abi41_hard_projection_fallbacks = (long long)c[kCntHardFallbacks];
    std::memcpy(&d.abi41_max_smoothed_delta, &mbits, 4);
    d.fast_soft_repulsion_candidates = (long long)c[kCntSelfCandidates];
    d.fast_soft_repulsion_applied = (long long)c[kCntSoftContacts];
    d.external_friction_corrections = (long long)c[kCntFrictionCorrections];
    d.self_candidate_count = (long long)c[kCntSelfCandidates];
    d.static_sdf_contact_count = (long long)c[kCntStaticSdfContacts];
    d.candidate_count = (long long)(c[kCntSelfCandidates] + c[kCntStaticSdfContacts]);
    d.abi41_lra_tack_count = (long long)c[kCntLraTacks];
    d.abi41_bending_wing_count = c[kCntBendingWings] > 0 ? (long long)c[kCntBendingWings] : (long long)S->wing_count;
    d.abi41_bending_texture_ready = S->wing_count > 0 ? 1 : 0;
    d.abi41_tack_jitter_guarded = (long long)c[kCntTackGuards];
    d.abi41_bending_guarded = (long long)c[kCntBendingGuards];
    d.fast_overlap_island_candidates = (long long)c[kCntIslandCandidates];
    d.fast_overlap_island_clusters = (long long)c[kCntIslandClusters];
    d.fast_overlap_island_vertex_refs = (long long)c[kCntIslandVertexRefs];
    d.fast_overlap_island_applied_vertices = (long long)c[kCntIslandAppliedVertices];
    d.fast_overlap_island_guarded = (long long)c[kCntIslandGuarded];
    d.fast_overlap_island_max_delta = (float)c[kCntIslandMaxDeltaMicro] * 1.0e-6f;
    d.self_filter_seen = (long long)c[kCntFilterSeen];
    d.self_filter_accepted_vv = (long long)c[kCntFilterAcceptedVv];
    d.self_filter_accepted_vt = (long long)c[kCntFilterAcceptedVt];
    d.self_filter_accepted_ee = (long long)c[kCntFilterAcceptedEe];
    d.self_filter_rejected_rest = (long long)c[kCntFilterRejectedRest];
    d.self_filter_rejected_duplicate = (long long)c[kCntFilterRejectedDuplicate];
    d.self_filter_rejected_ownership = (long long)c[kCntFilterRejectedOwnership];
    d.self_filter_cache_hits = S->cfg.self_collision_mode == 1 ? st.cache_hits : 0;
    d.self_filter_cache_misses = S->cfg.self_collision_mode == 1 ? st.cache_misses : 0;
    d.self_cluster_count = (long long)c[kCntClusterCount];
    d.self_cluster_owned_contacts = (long long)c[kCntClusterOwnedContacts];
    if (S->pcg_on) {
        // residual diagnostics from the scalar slots (abi41.cu:7586-7624)
        float red[kRedSlots];
        unsigned long long guard = 0;
        unsigned mbits = 0;
        if (!cuda_ok(cudaMemcpyAsync(red, S->pcg.red, sizeof(red), cudaMemcpyDeviceToHost, S->stream), "fetch PCG reductions") ||
            !cuda_ok(cudaMemcpyAsync(&guard, S->pcg.guard, sizeof(guard), cudaMemcpyDeviceToHost, S->stream), "fetch PCG guard count") ||
            !cuda_ok(cudaMemcpyAsync(&mbits, S->pcg.max_delta_bits, 4, cudaMemcpyDeviceToHost, S->stream), "fetch PCG max delta") ||
            !cuda_ok(cudaStreamSynchronize(S->stream), "fetch PCG diagnostics"))
            return false;
        d.abi41_pcg_csr_nnz = S->pcg_nnz;
        d.abi41_pcg_texture_ready = 1;
        d.abi41_pcg_iterations = S->pcg_iterations;
        float initial = red[kRedInitialRZ];
        if ((!std::isfinite(initial) || initial <= 0.0f) && std::isfinite(red[kRedRZ]) && red[kRedRZ] >= 0.0f) initial = red[kRedRZ];
        if (std::isfinite(initial) && initial >= 0.0f) {
            d.abi41_pcg_initial_residual = std::sqrt(std::max(initial, 0.0f));
            d.abi41_pcg_final_residual = d.abi41_pcg_initial_residual;
        }
        const float status = red[kRedStatus];
        const float final_rz = status == 2.0f ? red[kRedRZ] : red[kRedRZNext];
        if ((status == 0.0f || status == 2.0f) && std::isfinite(final_rz) && final_rz >= 0.0f)
            d.abi41_pcg_final_residual = std::sqrt(std::max(final_rz, 0.0f));
        else if (status != 0.0f && status != 2.0f)
            d.abi41_pcg_guarded += 1;
        d.abi41_pcg_guarded += (long long)guard;
        std::memcpy(&d.abi41_pcg_max_delta, &mbits, 4);
    }
    return true;
}

Solver* as_solver(void* h) { return reinterpret_cast<Solver*>(h); }

}  // namespace

namespace xg {
// Lets entry points defined in other translation units report through
// ssbl_last_error().
void set_last_error(const std::string& msg) { g_error = msg; }
}  // namespace xg

// ----------------------------------------------------------- C entry points

extern "C" SSBL_API void* ssbl_create_solver(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh) {
    g_error.clear();
    if (!config || config->vertex_count < 0 || config->edge_count < 0 || config->triangle_count < 0 ||
        !std::isfinite(config->dt) || !(config->dt > 0.0f) || !mesh || !mesh->positions || !mesh->inv_mass) {
        fail("invalid ABI41 solver create request");
        return nullptr;
    }
    Solver* S = new Solver();
    SsblXpbdConfig& c = S->cfg;
    c = *config;
    c.vertex_count = std::max(c.vertex_count, 0);
    c.edge_count = std::max(c.edge_count, 0);
    c.bend_count = std::max(c.bend_count, 0);
    c.lra_count = std::max(c.lra_count, 0);
    c.triangle_count = std::max(c.triangle_count, 0);
    c.damping = std::isfinite(c.damping) ? std::max(0.0f, std::min(c.damping, 1.0f)) : 1.0f;
    if (!std::isfinite(c.bend_compliance) || c.bend_compliance < 0.0f) c.bend_compliance = 0.0f;
    if (!std::isfinite(c.lra_compliance) || c.lra_compliance < 0.0f) c.lra_compliance = 0.0f;
    if (!std::isfinite(c.stretch_optimization_strength)) c.stretch_optimization_strength = 0.0f;
    c.stretch_optimization_strength = std::min(std::max(c.stretch_optimization_strength, 0.0f), 1.0f);
    c.stretch_optimization_enabled =
        (c.edge_count > 0 && c.stretch_optimization_enabled && c.stretch_optimization_strength > 0.0f) ? 1 : 0;
    const int V = c.vertex_count, E = c.edge_count, B = c.bend_count, L = c.lra_count, T = c.triangle_count;
    auto bail = [&](const char* msg) -> void* {
        if (msg) fail(msg);
        free_solver(S);
        return nullptr;
    };
    if (c.use_volume_pressure && c.pressure_strength > 0.0f)
        return bail("volume pressure is not supported by this build of the GB300 solver");
    if (B > 0 && (!mesh->bends || !mesh->bend_rest_lengths))
        return bail("ABI41 bend constraints require bend pairs and rest lengths");
    if (L > 0 && (!mesh->lra_edges || !mesh->lra_rest_lengths))
        return bail("ABI41 LRA constraints require edge pairs and rest lengths");
    if (c.edge_color_count > 0) {
        if (!mesh->edge_color_offsets) return bail("ABI41 edge color offsets are required");
        S->edge_colors.assign(mesh->edge_color_offsets, mesh->edge_color_offsets + c.edge_color_count + 1);
    }
    if (c.bend_color_count > 0) {
        if (!mesh->bend_color_offsets) return bail("ABI41 bend color offsets are required");
        S->bend_colors.assign(mesh->bend_color_offsets, mesh->bend_color_offsets + c.bend_color_count + 1);
    }
    S->colliders.use_ground = c.use_ground;
    S->colliders.ground_height = c.ground_height;
    S->colliders.use_wall = c.use_wall;
    std::memcpy(S->colliders.wall_origin, c.wall_origin, sizeof(c.wall_origin));
    std::memcpy(S->colliders.wall_normal, c.wall_normal, sizeof(c.wall_normal));
    S->colliders.use_sphere = c.use_sphere;
    std::memcpy(S->colliders.sphere_center, c.sphere_center, sizeof(c.sphere_center));
    S->colliders.sphere_radius = c.sphere_radius;

    if (!cuda_ok(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking), "create solver stream")) return bail(nullptr);

    // vertices
    S->h_inv.assign(mesh->inv_mass, mesh->inv_mass + V);
    S->h_w.resize(V);
    std::vector<float4> rest4(V), zero4(V, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < V; ++i) {
        S->h_w[i] = S->h_inv[i] > 0.0f ? S->h_inv[i] : 0.0f;
        rest4[i] = make_float4(mesh->positions[i * 3], mesh->positions[i * 3 + 1], mesh->positions[i * 3 + 2], S->h_w[i]);
    }
    // constraints
    std::vector<int2> springs(E);
    std::vector<float> spring_rest(E);
    for (int e = 0; e < E; ++e) {
        const int i = mesh->edges ? mesh->edges[e * 2] : 0, j = mesh->edges ? mesh->edges[e * 2 + 1] : 0;
        springs[e] = make_int2(std::max(i, 0), std::max(j, 0));
        spring_rest[e] = mesh->edge_rest_lengths ? mesh->edge_rest_lengths[e] : 0.0f;
    }
    std::vector<int> sp_off, te_off, bj_off;
    std::vector<int2> sp_ent, te_ent, bj_ent;
    build_pair_csr(V, springs, spring_rest, &sp_off, &sp_ent);
    std::vector<int2> tethers(L), bends(B);
    std::vector<float> tether_rest(L), bend_rest(B);
    for (int k = 0; k < L; ++k) {
        tethers[k] = make_int2(mesh->lra_edges[k * 2], mesh->lra_edges[k * 2 + 1]);
        tether_rest[k] = mesh->lra_rest_lengths[k];
    }
    for (int k = 0; k < B; ++k) {
        bends[k] = make_int2(mesh->bends[k * 2], mesh->bends[k * 2 + 1]);
        bend_rest[k] = mesh->bend_rest_lengths[k];
    }
    build_pair_csr(V, tethers, tether_rest, &te_off, &te_ent);
    if (S->bend_colors.empty() && B > 0) build_pair_csr(V, bends, bend_rest, &bj_off, &bj_ent);
    std::vector<int4> tris(T);
    for (int t = 0; t < T; ++t) {
        const int* tr = mesh->triangles ? mesh->triangles + t * 3 : nullptr;
        tris[t] = make_int4(tr ? std::max(tr[0], 0) : 0, tr ? std::max(tr[1], 0) : 0, tr ? std::max(tr[2], 0) : 0, 0);
    }
    S->wing_count = T > 1 ? count_wings(V, tris) : 0;
    S->h_pin_weight.assign(V, -1.0f);
    S->h_pin_target.assign(V, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    S->h_pin_relax.assign(V, 0.0f);

    // parameters
    Params& P = S->hp;
    P.V = V;
    P.E = E;
    P.T = T;
    P.B = B;
    P.L = L;
    P.damping = c.damping;
    for (int a = 0; a < 3; ++a) P.gravity[a] = c.gravity[a];
    P.stretch_compliance = c.stretch_compliance;
    P.bend_compliance = c.bend_compliance;
    P.lra_compliance = c.lra_compliance;
    P.margin = c.collision_margin;
    P.thickness = c.cloth_thickness;
    P.friction = c.contact_friction;
    P.tangent_damping = c.contact_tangent_damping;
    load_colliders(S);
    const float radius = self_radius(c);
    P.self_radius = radius;
    P.self_mode = c.self_collision_mode;
    P.max_neighbors = c.max_self_collision_neighbors;
    P.stretch_strength = c.stretch_optimization_strength;
    S->pcg_on = c.stretch_optimization_enabled != 0;
    S->self_on = c.self_collision != 0;
    if (S->self_on && radius > 0.0f) {
        const float cell = std::max(radius * 1.8f, 1.0e-3f);
        P.vcell = P.tcell = P.ecell = cell;
        P.vhash = V >= 128;
        P.thash = T >= 64;
        P.ehash = E >= 64;
        P.vbuckets = P.vhash ? next_pow2(std::max(1024, V * 4)) : 0;
        P.tbuckets = P.thash ? next_pow2(std::max(1024, T * 4)) : 0;
        P.ebuckets = P.ehash ? next_pow2(std::max(1024, E * 4)) : 0;
    }

    bool ok = dalloc(&S->dp, 1, "parameter allocation") && dalloc(&S->pos[0], V, "position allocation") &&
              dalloc(&S->pos[1], V, "position allocation") && dalloc(&S->prev, V, "previous position allocation") &&
              dalloc(&S->vel, V, "velocity allocation") && dalloc(&S->rest, V, "rest position allocation") &&
              dalloc(&S->inv_mass, V, "inverse mass allocation") && dalloc(&S->sp_off, V + 1, "spring CSR allocation") &&
              dalloc(&S->sp_ent, sp_ent.size(), "spring CSR allocation") &&
              dalloc(&S->te_off, V + 1, "tether CSR allocation") && dalloc(&S->te_ent, te_ent.size(), "tether CSR allocation") &&
              dalloc(&S->bends, B, "bend pair allocation") && dalloc(&S->bend_rest, B, "bend rest allocation") &&
              dalloc(&S->tris, T, "triangle allocation") && dalloc(&S->edges, E, "edge allocation") &&
              dalloc(&S->edge_rest, E, "edge rest allocation") && dalloc(&S->pin_target, V, "pin target allocation") &&
              dalloc(&S->pin_weight, V, "pin weight allocation") && dalloc(&S->pin_relax, V, "pin relaxation allocation") &&
              dalloc(&S->counts, kCntSlots, "ABI41 diagnostic allocation") &&
              dalloc(&S->max_delta_bits, 1, "self max smoothed delta allocation") &&
              dalloc(&S->pack, (size_t)V * 3, "download staging allocation");
    if (ok && !bj_off.empty())
        ok = dalloc(&S->bj_off, V + 1, "bend CSR allocation") && dalloc(&S->bj_ent, bj_ent.size(), "bend CSR allocation");
    if (ok && S->self_on && radius > 0.0f) {
        ok = dalloc(&S->nb_count, V, "self collision count allocation") &&
             dalloc(&S->nb_idx, (size_t)V * kNeighborSlots, "self collision index allocation") &&
             dalloc(&S->acc, V, "self accumulation allocation") &&
             dalloc(&S->scan_tmp, (size_t)std::max(std::max(P.vbuckets, P.tbuckets), P.ebuckets) / 4096 + 2,
                    "bucket scan allocation");
        if (ok && P.vhash)
            ok = dalloc(&S->vcell, V, "self collision cell allocation") &&
                 dalloc(&S->vb_count, P.vbuckets, "self collision hash count allocation") &&
                 dalloc(&S->vb_start, P.vbuckets + 1, "self collision hash start allocation") &&
                 dalloc(&S->vb_ent, V, "self collision hash index allocation");
        if (ok && P.thash)
            ok = dalloc(&S->tb_count, P.tbuckets, "self triangle hash count allocation") &&
                 dalloc(&S->tb_start, P.tbuckets + 1, "self triangle hash start allocation") &&
                 dalloc(&S->tb_ent, (size_t)T * kMaxPrimitiveCells, "self triangle hash index allocation");
        if (ok && P.ehash)
            ok = dalloc(&S->eb_count, P.ebuckets, "self edge hash count allocation") &&
                 dalloc(&S->eb_start, P.ebuckets + 1, "self edge hash start allocation") &&
                 dalloc(&S->eb_ent, (size_t)E * kMaxPrimitiveCells, "self edge hash index allocation");
    }
    // hard-stretch buffers; caps need edges grouped by colour: the caller's
    // colouring when given (edges already sorted by colour), else a greedy
    // first-fit colouring in edge order
    std::vector<int2> cap_edges;
    std::vector<float> cap_rest;
    if (ok && S->pcg_on) {
        S->pcg_nnz = (int)sp_ent.size();
        if (S->pcg_nnz == 0) return bail("PCG stretch optimization found no valid CSR edges");
        if (!S->edge_colors.empty()) {
            cap_edges = springs;
            cap_rest = spring_rest;
            S->cap_colors = S->edge_colors;
        } else {
            std::vector<int> color(E, 0);
            std::vector<std::vector<int>> used(V);
            int ncol = 0;
            for (int e = 0; e < E; ++e) {
                const int a = springs[e].x, b = springs[e].y;
                int k = 0;
                auto taken = [&](int v, int col) {
                    return v >= 0 && v < V && std::find(used[v].begin(), used[v].end(), col) != used[v].end();
                };
                while (taken(a, k) || taken(b, k)) ++k;
                color[e] = k;
                if (a >= 0 && a < V) used[a].push_back(k);
                if (b >= 0 && b < V) used[b].push_back(k);
                ncol = std::max(ncol, k + 1);
            }
            S->cap_colors.assign(ncol + 1, 0);
            for (int e = 0; e < E; ++e) S->cap_colors[color[e] + 1]++;
            for (int k = 0; k < ncol; ++k) S->cap_colors[k + 1] += S->cap_colors[k];
            std::vector<int> cursor(S->cap_colors.begin(), S->cap_colors.end() - 1);
            cap_edges.resize(E);
            cap_rest.resize(E);
            for (int e = 0; e < E; ++e) {
                const int at = cursor[color[e]]++;
                cap_edges[at] = springs[e];
                cap_rest[at] = spring_rest[e];
            }
        }
        PcgView& g = S->pcg;
        ok = dalloc(&g.diag, 2 * (size_t)V, "PCG diagonal block allocation") &&
             dalloc(&g.pinv, 2 * (size_t)V, "PCG preconditioner allocation") && dalloc(&g.r, V, "PCG residual allocation") &&
             dalloc(&g.z, V, "PCG preconditioned residual allocation") && dalloc(&g.d, V, "PCG search direction allocation") &&
             dalloc(&g.q, V, "PCG A*d allocation") && dalloc(&g.offdiag, sp_ent.size(), "PCG offdiagonal allocation") &&
             dalloc(&g.avg, V, "stretch cap accumulation allocation") && dalloc(&g.red, kRedSlots, "PCG reduction allocation") &&
             dalloc(&g.partials, pcg_warp_partials(V), "PCG partial sum allocation") &&
             dalloc(&g.ticket, 1, "PCG ticket allocation") && dalloc(&g.guard, 1, "PCG guard counter allocation") &&
             dalloc(&g.max_delta_bits, 1, "PCG max delta allocation") && dalloc(&S->cap_edges, E, "cap edge allocation") &&
             dalloc(&S->cap_rest, E, "cap rest allocation");
    }
    if (!ok) return bail(nullptr);
    cudaStream_t st = S->stream;
    ok = dupload(S->pos[0], rest4.data(), V, st, "position upload") && dupload(S->pos[1], rest4.data(), V, st, "position upload") &&
         dupload(S->prev, rest4.data(), V, st, "previous position upload") && dupload(S->vel, zero4.data(), V, st, "velocity upload") &&
         dupload(S->rest, rest4.data(), V, st, "rest position upload") &&
         dupload(S->inv_mass, S->h_inv.data(), V, st, "inverse mass upload") &&
         dupload(S->sp_off, sp_off.data(), sp_off.size(), st, "spring CSR upload") &&
         dupload(S->sp_ent, sp_ent.data(), sp_ent.size(), st, "spring CSR upload") &&
         dupload(S->te_off, te_off.data(), te_off.size(), st, "tether CSR upload") &&
         dupload(S->te_ent, te_ent.data(), te_ent.size(), st, "tether CSR upload") &&
         dupload(S->bj_off, bj_off.data(), bj_off.size(), st, "bend CSR upload") &&
         dupload(S->bj_ent, bj_ent.data(), bj_ent.size(), st, "bend CSR upload") &&
         dupload(S->bends, bends.data(), B, st, "bend pair upload") && dupload(S->bend_rest, bend_rest.data(), B, st, "bend rest upload") &&
         dupload(S->tris, tris.data(), T, st, "triangle upload") && dupload(S->edges, springs.data(), E, st, "edge upload") &&
         dupload(S->edge_rest, spring_rest.data(), E, st, "edge rest upload") &&
         dupload(S->pin_weight, S->h_pin_weight.data(), V, st, "pin weight upload") &&
         dupload(S->pin_target, S->h_pin_target.data(), V, st, "pin target upload") &&
         dupload(S->pin_relax, S->h_pin_relax.data(), V, st, "pin relaxation upload") &&
         cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, st), "reset ABI41 diagnostics") &&
         cuda_ok(cudaMemsetAsync(S->max_delta_bits, 0, sizeof(unsigned), st), "reset self max smoothed delta") &&
         (!S->acc || cuda_ok(cudaMemsetAsync(S->acc, 0, sizeof(Acc4) * V, st), "reset self accumulation")) &&
         (!S->nb_count || cuda_ok(cudaMemsetAsync(S->nb_count, 0, sizeof(int) * V, st), "reset neighbor table")) &&
         sync_params(S) && cuda_ok(cudaStreamSynchronize(st), "solver upload");
    if (ok && S->pcg_on)
        ok = dupload(S->cap_edges, cap_edges.data(), E, st, "cap edge upload") &&
             dupload(S->cap_rest, cap_rest.data(), E, st, "cap rest upload") &&
             cuda_ok(cudaMemsetAsync(S->pcg.ticket, 0, sizeof(unsigned), st), "reset PCG ticket") &&
             cuda_ok(cudaMemsetAsync(S->pcg.red, 0, sizeof(float) * kRedSlots, st), "reset PCG reductions") &&
             cuda_ok(cudaStreamSynchronize(st), "PCG buffer upload");
    if (!ok) return bail(nullptr);
    S->diag.finite_flag = 1;
    S->diag.abi41_bending_wing_count = S->wing_count;
    S->diag.abi41_bending_texture_ready = S->wing_count > 0 ? 1 : 0;
    if (!upload_static(S, mesh->static_triangles, std::max(config->static_triangle_count, 0))) return bail(nullptr);
    return S;
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
    const int V = S->cfg.vertex_count;
    if (!cuda_ok(cudaMemcpyAsync(S->pos[0], S->rest, sizeof(float4) * V, cudaMemcpyDeviceToDevice, S->stream), "reset positions") ||
        !cuda_ok(cudaMemcpyAsync(S->prev, S->rest, sizeof(float4) * V, cudaMemcpyDeviceToDevice, S->stream), "reset previous positions") ||
        !cuda_ok(cudaMemsetAsync(S->vel, 0, sizeof(float4) * V, S->stream), "reset velocities") ||
        !cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, S->stream), "reset ABI41 diagnostics") ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "reset solver"))
        return 0;
    S->diag = SsblXpbdDiagnostics{};
    S->diag.finite_flag = 1;
    return 1;
}

extern "C" SSBL_API int ssbl_update_pin_targets(void* handle, const int* indices, const float* positions, const float* weights, int count) {
    g_error.clear();
    return upload_pins(as_solver(handle), indices, positions, weights, count) ? 1 : 0;
}

extern "C" SSBL_API int ssbl_update_runtime_colliders(void* handle, const SsblXpbdRuntimeColliders* inputs) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !inputs) return fail("invalid runtime collider update") ? 1 : 0;
    S->colliders = *inputs;
    load_colliders(S);
    return 1;
}

extern "C" SSBL_API int ssbl_update_positions(void* handle, const float* positions, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !positions || max_floats < S->cfg.vertex_count * 3) return fail("invalid position upload") ? 1 : 0;
    const int V = S->cfg.vertex_count;
    std::vector<float4> p4(V);
    for (int i = 0; i < V; ++i) p4[i] = make_float4(positions[i * 3], positions[i * 3 + 1], positions[i * 3 + 2], S->h_w[i]);
    return (dupload(S->pos[0], p4.data(), V, S->stream, "upload positions") &&
            dupload(S->prev, p4.data(), V, S->stream, "upload previous positions") &&
            cuda_ok(cudaStreamSynchronize(S->stream), "upload positions"))
               ? 1
               : 0;
}

extern "C" SSBL_API int ssbl_update_static_triangles(void* handle, const float* triangles, int triangle_count) {
    g_error.clear();
    return upload_static(as_solver(handle), triangles, triangle_count) ? 1 : 0;
}

extern "C" SSBL_API int ssbl_update_dynamic_triangles(void* handle, const float* triangles, int triangle_count) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid dynamic triangle update") ? 1 : 0;
    if (triangle_count > 0 && triangles) return fail("dynamic triangle colliders are not supported by this build of the GB300 solver") ? 1 : 0;
    S->dynamic_triangle_count = 0;
    return 1;
}

extern "C" SSBL_API int ssbl_update_frame_inputs(void* handle, const SsblXpbdFrameInputs* in) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !in) return fail("invalid frame input update") ? 1 : 0;
    if (in->update_pin_targets && !upload_pins(S, in->pin_indices, in->pin_positions, in->pin_weights, in->pin_count)) return 0;
    if (in->update_runtime_colliders) {
        S->colliders = in->runtime_colliders;
        load_colliders(S);
    }
    if (in->update_dynamic_triangles && in->dynamic_triangle_count > 0)
        return fail("dynamic triangle colliders are not supported by this build of the GB300 solver") ? 1 : 0;
    if (in->update_dynamic_indexed_triangles && in->dynamic_indexed_triangle_count > 0)
        return fail("dynamic triangle colliders are not supported by this build of the GB300 solver") ? 1 : 0;
    if (in->update_dynamic_particles && in->dynamic_particle_count > 0)
        return fail("dynamic particle colliders are not supported by this build of the GB300 solver") ? 1 : 0;
    if (in->update_static_triangles && !upload_static(S, in->static_triangles, in->static_triangle_count)) return 0;
    if (in->update_force_fields) {
        if (in->force_field_count < 0 || in->force_field_count > 64) return fail("force field count exceeds SSBL maximum") ? 1 : 0;
        if (in->force_field_count > 0) return fail("force fields are not supported by this build of the GB300 solver") ? 1 : 0;
        S->force_field_count = 0;
        S->unsupported_force_field_count = std::max(in->unsupported_force_field_count, 0);
    }
    S->diag.force_field_count = S->force_field_count;
    S->diag.unsupported_force_field_count = S->unsupported_force_field_count;
    return 1;
}

extern "C" SSBL_API int ssbl_step_solver_ex(void* handle, int substeps, int iterations, int fetch_diagnostics, int force_sync) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    const auto t0 = std::chrono::high_resolution_clock::now();
    S->diag = SsblXpbdDiagnostics{};
    S->diag.finite_flag = 1;
    S->diag.force_field_count = S->force_field_count;
    S->diag.unsupported_force_field_count = S->unsupported_force_field_count;
    sdf_diagnostics(S);
    substeps = std::max(substeps, 1);
    iterations = std::max(iterations, 1);
    if (!cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, S->stream), "reset ABI41 diagnostics") ||
        !cuda_ok(cudaMemsetAsync(S->max_delta_bits, 0, sizeof(unsigned), S->stream), "reset self max smoothed delta") ||
        !upload_pin_relax(S, iterations) || !sync_params(S))
        return 0;
    if (S->pcg_on &&
        (!cuda_ok(cudaMemsetAsync(S->pcg.guard, 0, sizeof(unsigned long long), S->stream), "reset PCG guard count") ||
         !cuda_ok(cudaMemsetAsync(S->pcg.max_delta_bits, 0, sizeof(unsigned), S->stream), "reset PCG max delta") ||
         !cuda_ok(cudaMemsetAsync(S->pcg.red, 0, sizeof(float) * kRedSlots, S->stream), "reset PCG reductions")))
        return 0;
    FrameStats st;
    if (!run_frame(S, substeps, iterations, &st)) return 0;
    S->last_launches = st.launches;
    S->pcg_iterations = st.pcg_solves * 8;
    if (force_sync || fetch_diagnostics) {
        const auto ts = std::chrono::high_resolution_clock::now();
        if (!cuda_ok(cudaStreamSynchronize(S->stream), "ABI41 solver step")) return 0;
        S->diag.sync_ms = (float)ms_since(ts);
    }
    if (fetch_diagnostics && !fetch_counts(S, st)) return 0;
    S->diag.step_ms = (float)ms_since(t0);
    S->diag.constraints_ms = S->diag.step_ms;
    S->diag.resolved_contacts = S->diag.abi41_soft_contact_count + S->diag.abi41_exact_impulse_contact_count +
                                S->diag.abi41_edge_edge_contact_count + S->diag.static_sdf_contact_count;
    return 1;
}

extern "C" SSBL_API int ssbl_step_solver(void* handle, int substeps, int iterations) {
    return ssbl_step_solver_ex(handle, substeps, iterations, 1, 1);
}

extern "C" SSBL_API int ssbl_download_positions(void* handle, float* out, int max_floats) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out || max_floats < S->cfg.vertex_count * 3) return fail("invalid position download") ? 1 : 0;
    const int V = S->cfg.vertex_count;
    launch_pack_positions(S->pack, S->pos[0], V, S->stream);
    return (cuda_ok(cudaGetLastError(), "pack positions") &&
            cuda_ok(cudaMemcpyAsync(out, S->pack, sizeof(float) * 3 * V, cudaMemcpyDeviceToHost, S->stream), "download ABI41 positions") &&
            cuda_ok(cudaStreamSynchronize(S->stream), "download ABI41 positions"))
               ? 1
               : 0;
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

// The global dynamic scene shares dynamic colliders between cloths; this
// build keeps the handle life cycle and rejects cross-cloth collision modes.
namespace {
struct GlobalScene {
    int particle_count = 0;
    int triangle_count = 0;
};
}  // namespace

extern "C" SSBL_API void* ssbl_create_global_dynamic_scene(void) {
    g_error.clear();
    return new GlobalScene();
}

extern "C" SSBL_API int ssbl_destroy_global_dynamic_scene(void* scene) {
    g_error.clear();
    delete reinterpret_cast<GlobalScene*>(scene);
    return 1;
}

extern "C" SSBL_API int ssbl_update_global_dynamic_scene(void* scene, const SsblXpbdGlobalDynamicSceneInputs* in) {
    g_error.clear();
    GlobalScene* G = reinterpret_cast<GlobalScene*>(scene);
    if (!G || !in) return fail("invalid global dynamic scene update") ? 1 : 0;
    G->particle_count = std::max(in->particle_count, 0);
    G->triangle_count = std::max(in->triangle_count, 0);
    return 1;
}

extern "C" SSBL_API int ssbl_attach_global_dynamic_scene(void* handle, void* scene, int, int, int collision_mode) {
    g_error.clear();
    if (!handle || !scene) return fail("invalid global dynamic scene attach") ? 1 : 0;
    GlobalScene* G = reinterpret_cast<GlobalScene*>(scene);
    if (collision_mode != 0 && (G->particle_count > 0 || G->triangle_count > 0))
        return fail("cross-cloth collision through the global dynamic scene is not supported by this build of the GB300 solver") ? 1 : 0;
    return 1;
}

extern "C" SSBL_API int ssbl_clear_global_dynamic_scene(void* handle) {
    g_error.clear();
    return handle ? 1 : (fail("invalid solver handle") ? 1 : 0);
}

extern "C" SSBL_API const char* ssbl_last_error(void) { return g_error.c_str(); }

// ------------------------------------------------------ GB300 extensions --

extern "C" __attribute__((visibility("default"))) int xpbd_gb300_build_self_structures(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    if (!S->self_on || !S->nb_count) return fail("self collision is not enabled for this solver") ? 1 : 0;
    if (!sync_params(S)) return 0;
    const Params& P = S->hp;
    const View v = S->view();
    if (P.vhash) {
        cudaMemsetAsync(S->vb_count, 0, sizeof(int) * P.vbuckets, S->stream);
        self_build_vertex_hash(v, P.V, P.vbuckets, S->stream);
    }
    if (P.thash) {
        cudaMemsetAsync(S->tb_count, 0, sizeof(int) * P.tbuckets, S->stream);
        self_build_triangle_hash(v, P.T, P.tbuckets, true, S->stream);
    }
    if (P.ehash) {
        cudaMemsetAsync(S->eb_count, 0, sizeof(int) * P.ebuckets, S->stream);
        self_build_edge_hash(v, P.E, P.ebuckets, true, S->stream);
    }
    self_neighbors(v, P.V, P.vhash != 0, S->stream);
    return (cuda_ok(cudaGetLastError(), "build self structures") && cuda_ok(cudaStreamSynchronize(S->stream), "build self structures")) ? 1 : 0;
}

extern "C" __attribute__((visibility("default"))) long long xpbd_gb300_read_buffer(void* handle, int id, void* out, long long max_bytes) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out) {
        fail("invalid buffer read");
        return -1;
    }
    const Params& P = S->hp;
    const void* src = nullptr;
    long long bytes = 0;
    int total_t = 0, total_e = 0;
    if ((id == XPBD_BUF_TRI_BUCKET_ENTRIES && S->tb_start) || (id == XPBD_BUF_EDGE_BUCKET_ENTRIES && S->eb_start)) {
        const int* st = id == XPBD_BUF_TRI_BUCKET_ENTRIES ? S->tb_start : S->eb_start;
        const int nb = id == XPBD_BUF_TRI_BUCKET_ENTRIES ? P.tbuckets : P.ebuckets;
        int total = 0;
        if (!cuda_ok(cudaMemcpy(&total, st + nb, sizeof(int), cudaMemcpyDeviceToHost), "read bucket total")) return -1;
        (id == XPBD_BUF_TRI_BUCKET_ENTRIES ? total_t : total_e) = total;
    }
    switch (id) {
        case XPBD_BUF_POSITIONS4: src = S->pos[0]; bytes = 16ll * P.V; break;
        case XPBD_BUF_PREV4: src = S->prev; bytes = 16ll * P.V; break;
        case XPBD_BUF_VEL4: src = S->vel; bytes = 16ll * P.V; break;
        case XPBD_BUF_VERTEX_CELLS: src = S->vcell; bytes = 16ll * P.V; break;
        case XPBD_BUF_VERTEX_BUCKET_START: src = S->vb_start; bytes = 4ll * (P.vbuckets + 1); break;
        case XPBD_BUF_VERTEX_BUCKET_ENTRIES: src = S->vb_ent; bytes = 4ll * P.V; break;
        case XPBD_BUF_TRI_BUCKET_START: src = S->tb_start; bytes = 4ll * (P.tbuckets + 1); break;
        case XPBD_BUF_TRI_BUCKET_ENTRIES: src = S->tb_ent; bytes = 4ll * total_t; break;
        case XPBD_BUF_EDGE_BUCKET_START: src = S->eb_start; bytes = 4ll * (P.ebuckets + 1); break;
        case XPBD_BUF_EDGE_BUCKET_ENTRIES: src = S->eb_ent; bytes = 4ll * total_e; break;
        case XPBD_BUF_NEIGHBOR_COUNTS: src = S->nb_count; bytes = 4ll * P.V; break;
        case XPBD_BUF_NEIGHBOR_INDICES: src = S->nb_idx; bytes = 4ll * P.V * kNeighborSlots; break;
        case XPBD_BUF_STATIC_SDF:
            src = S->sdf;
            bytes = P.sdf_ready ? 4ll * P.sdf_dim[0] * P.sdf_dim[1] * P.sdf_dim[2] : 0;
            break;
        case XPBD_BUF_COUNTERS: src = S->counts; bytes = 8ll * kCntSlots; break;
        default: fail("unknown buffer id"); return -1;
    }
    if (!src) {
        fail("buffer is not allocated for this solver");
        return -1;
    }
    if (bytes > max_bytes) {
        fail("output buffer too small");
        return -1;
    }
    if (!cuda_ok(cudaStreamSynchronize(S->stream), "read buffer") ||
        (bytes > 0 && !cuda_ok(cudaMemcpy(out, src, (size_t)bytes, cudaMemcpyDeviceToHost), "read buffer")))
        return -1;
    return bytes;
}

extern "C" __attribute__((visibility("default"))) int xpbd_gb300_hash_info(void* handle, int* out6) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !out6) return fail("invalid hash info request") ? 1 : 0;
    out6[0] = S->hp.vbuckets;
    out6[1] = S->hp.tbuckets;
    out6[2] = S->hp.ebuckets;
    out6[3] = S->hp.vhash;
    out6[4] = S->hp.thash;
    out6[5] = S->hp.ehash;
    return 1;
}

extern "C" __attribute__((visibility("default"))) int xpbd_gb300_set_graph_capture(void* handle, int enabled) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    S->use_graphs = enabled != 0;
    return 1;
}

extern "C" __attribute__((visibility("default"))) long long xpbd_gb300_last_step_launches(void* handle) {
    Solver* S = as_solver(handle);
    return S ? S->last_launches : -1;
}

extern "C" __attribute__((visibility("default"))) void* xpbd_gb300_stream(void* handle) {
    Solver* S = as_solver(handle);
    return S ? reinterpret_cast<void*>(S->stream) : nullptr;
}

extern "C" __attribute__((visibility("default"))) int xpbd_gb300_profile_frame(void* handle, int substeps, int iterations,
                                                                               float* kernel_ms, long long* kernel_launches,
                                                                               int kinds) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S || !kernel_ms || !kernel_launches || kinds < kKinds) return fail("invalid profile request") ? 1 : 0;
    substeps = std::max(substeps, 1);
    iterations = std::max(iterations, 1);
    if (!upload_pin_relax(S, iterations) || !sync_params(S)) return 0;
    for (int k = 0; k < kinds; ++k) {
        kernel_ms[k] = 0.0f;
        kernel_launches[k] = 0;
    }
    FrameStats st;
    Profile prof;
    enqueue_frame(S, substeps, iterations, &st, &prof);
    if (!cuda_ok(cudaGetLastError(), "profile frame") || !cuda_ok(cudaStreamSynchronize(S->stream), "profile frame")) return 0;
    for (auto& m : prof.marks) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, m.second.first, m.second.second);
        kernel_ms[m.first] += ms;
        kernel_launches[m.first] += 1;
        cudaEventDestroy(m.second.first);
        cudaEventDestroy(m.second.second);
    }
    return 1;
}

extern "C" __attribute__((visibility("default"))) int xpbd_gb300_synchronize(void* handle) {
    g_error.clear();
    Solver* S = as_solver(handle);
    if (!S) return fail("invalid solver handle") ? 1 : 0;
    return cuda_ok(cudaStreamSynchronize(S->stream), "synchronize") ? 1 : 0;
}
