// Solver creation (CSR builds, hash sizing, static SDF), cloth-level
// updates and the per-frame launch schedule of the GB300 XPBD library.
//
// A solver holds one or more cloths concatenated in its device arrays (the
// layout is described in xpbd_host.cuh).  The schedule below is the
// reference's single-cloth schedule (native/src/ssbl_xpbd_cuda_abi41.cu:
// 9165-9376); every kernel reads the parameters of the cloth its item belongs
// to, so a cloth stepped inside a batch follows exactly the sequence of
// per-vertex operations it follows alone and its results are the same bits.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <unordered_map>

#include "xpbd_host.cuh"

namespace xg {
namespace host {

thread_local std::string g_error;
thread_local long long* g_alloc_account = nullptr;
std::atomic<int> g_default_key_ieee{0};

namespace {

constexpr int kInvalid = -1;  // index outside its cloth: invalid in every kernel

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

// Number of bending wings: triangle pairs on an edge with distinct opposite
// vertices (abi41.cu:7193-7302).  Reported in the diagnostics only.
int count_wings(int V, const std::vector<int4>& tris, size_t begin, size_t end) {
    std::unordered_map<uint64_t, int> first_opposite;
    int wings = 0;
    for (size_t k = begin; k < end; ++k) {
        const int4 t = tris[k];
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

// ---- volume pressure preprocessing (abi41.cu:7413-7584, 8816-8903) ----

// A tuning constant of the pressure model, overridable from the environment
// under the reference's variable names, clamped to its range.
float env_scale(const char* name, float value, float lo, float hi) {
    const char* raw = std::getenv(name);
    if (raw && raw[0]) {
        char* end = nullptr;
        const float v = std::strtof(raw, &end);
        if (end != raw && std::isfinite(v)) value = v;
    }
    return std::max(lo, std::min(value, hi));
}

// Area share of each vertex: a third of every incident triangle's rest area,
// capped at 16 x the mean vertex area; all zero without a valid triangle.
std::vector<float> pressure_area_shares(int V, const std::vector<int4>& tris, size_t t0, size_t t1, const float* pos) {
    std::vector<float> shares(V, 0.0f);
    double total = 0.0;
    int valid = 0;
    for (size_t k = t0; k < t1; ++k) {
        const int4 t = tris[k];
        if (t.x < 0 || t.y < 0 || t.z < 0 || t.x >= V || t.y >= V || t.z >= V) continue;
        const F3 a = F3{pos[3 * t.x], pos[3 * t.x + 1], pos[3 * t.x + 2]};
        const F3 b = F3{pos[3 * t.y], pos[3 * t.y + 1], pos[3 * t.y + 2]};
        const F3 c = F3{pos[3 * t.z], pos[3 * t.z + 1], pos[3 * t.z + 2]};
        const F3 n = cross3(b - a, c - a);
        const float sq4 = dot3(n, n);
        if (!std::isfinite(sq4) || sq4 <= 0.0f) continue;
        const float area = 0.5f * std::sqrt(sq4);
        if (!std::isfinite(area) || area <= 0.0f) continue;
        const float share = area / 3.0f;
        shares[t.x] += share;
        shares[t.y] += share;
        shares[t.z] += share;
        total += (double)area;
        ++valid;
    }
    if (valid <= 0 || !(total > 0.0) || !std::isfinite(total)) return std::vector<float>(V, 0.0f);
    const float mean = (float)(total / (double)std::max(V, 1));
    const float cap = std::max(mean * 16.0f, 1.0e-12f);
    for (float& x : shares) x = (!std::isfinite(x) || x <= 0.0f) ? 0.0f : std::min(x, cap);
    return shares;
}

// Rest length scale of each vertex: the mean rest length of its edges (else
// the square root of its area share), clamped to [0.02, 16] x the mean.
std::vector<float> pressure_rest_scales(int V, const int* edges, const float* rest, int E, const std::vector<float>& shares) {
    std::vector<float> scales(V, 0.0f);
    std::vector<double> sum(V, 0.0);
    std::vector<int> cnt(V, 0);
    for (int e = 0; e < E; ++e) {
        const int i = std::max(edges ? edges[2 * e] : 0, 0), j = std::max(edges ? edges[2 * e + 1] : 0, 0);
        const float r = rest ? rest[e] : 0.0f;
        if (i >= V || j >= V || !std::isfinite(r) || r <= 0.0f) continue;
        sum[i] += (double)r;
        sum[j] += (double)r;
        cnt[i] += 1;
        cnt[j] += 1;
    }
    double total = 0.0;
    int valid = 0;
    for (int i = 0; i < V; ++i) {
        float x = 0.0f;
        if (cnt[i] > 0)
            x = (float)(sum[i] / (double)cnt[i]);
        else if (std::isfinite(shares[i]) && shares[i] > 0.0f)
            x = std::sqrt(shares[i]);
        if (std::isfinite(x) && x > 0.0f) {
            scales[i] = x;
            total += (double)x;
            ++valid;
        }
    }
    const float mean = valid > 0 ? (float)(total / (double)valid) : 1.0f;
    const float lo = std::max(mean * 0.02f, 1.0e-7f), hi = std::max(mean * 16.0f, lo);
    for (float& x : scales) {
        if (!std::isfinite(x) || x <= 0.0f) x = mean;
        x = std::max(lo, std::min(x, hi));
    }
    return scales;
}

// Length scale of the outward-speed trim: max(bounding-box diagonal x object
// scale, 4 x the mean rest scale).
float pressure_velocity_length(int V, const float* pos, const std::vector<float>& scales, float object_scale) {
    float mean = 0.0f;
    int n = 0;
    for (float x : scales)
        if (std::isfinite(x) && x > 0.0f) {
            mean += x;
            ++n;
        }
    mean = n > 0 ? mean / (float)n : 1.0f;
    bool any = false;
    F3 lo{0.0f, 0.0f, 0.0f}, hi{0.0f, 0.0f, 0.0f};
    for (int i = 0; i < V; ++i) {
        const F3 p{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        if (!finite3(p)) continue;
        if (!any) {
            lo = hi = p;
            any = true;
        } else {
            lo = F3{std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
            hi = F3{std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
        }
    }
    if (!any) return std::max(mean, 1.0e-6f);
    const F3 span = hi - lo;
    const float diag = std::sqrt(std::max(dot3(span, span), 0.0f));
    if (!std::isfinite(diag) || diag <= 0.0f) return std::max(mean, 1.0e-6f);
    const float obj = std::isfinite(object_scale) && object_scale > 0.0f ? object_scale : 0.08f;
    return std::max(diag * obj, mean * 4.0f);
}

float self_radius(const SsblXpbdConfig& c) {
    const float req = std::max(c.self_collision_distance, 0.0f);
    if (req > 0.0f) return req;
    return std::max(std::max(c.cloth_thickness, c.collision_margin), 0.0f);
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

// Config sanitising of ssbl_create_solver (abi41.cu:8791-8840).
void sanitize(SsblXpbdConfig& c) {
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
}

void load_colliders(Params& P, const SsblXpbdRuntimeColliders& c) {
    P.use_ground = c.use_ground;
    P.ground_height = c.ground_height;
    P.use_wall = c.use_wall;
    std::memcpy(P.wall_origin, c.wall_origin, sizeof(P.wall_origin));
    std::memcpy(P.wall_normal, c.wall_normal, sizeof(P.wall_normal));
    P.use_sphere = c.use_sphere;
    std::memcpy(P.sphere_center, c.sphere_center, sizeof(P.sphere_center));
    P.sphere_radius = c.sphere_radius;
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

std::mutex g_sdf_mutex;
std::vector<SdfGrid*> g_sdf_cache;

// Drop a cloth's reference to its SDF grid; the last reference frees it.
void release_grid(Solver* S, Cloth& c) {
    if (!c.grid) return;
    std::lock_guard<std::mutex> lock(g_sdf_mutex);
    SdfGrid* g = c.grid;
    c.grid = nullptr;
    S->device_bytes -= g->bytes;
    if (--g->refs > 0) return;
    g_sdf_cache.erase(std::remove(g_sdf_cache.begin(), g_sdf_cache.end(), g), g_sdf_cache.end());
    dfree(g->sdf);
    dfree(g->tris_dev);
    delete g;
}

}  // namespace

namespace {

// Zeroes up to six int arrays in one launch: one graph node where a memset
// per array would be one node each, on the path every hash build waits on.
// Arrays whose start is 16-byte aligned are written as int4 quads.
struct ZeroSpans {
    int* p[6];
    long long n[6];
    int count;
};

__global__ void k_zero_spans(ZeroSpans z) {
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long step = (long long)gridDim.x * blockDim.x;
    for (int k = 0; k < z.count; ++k) {
        int* p = z.p[k];
        const long long n = z.n[k];
        long long quads = 0;
        if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0u) {
            quads = n / 4;
            int4* p4 = reinterpret_cast<int4*>(p);
            for (long long i = t0; i < quads; i += step) p4[i] = make_int4(0, 0, 0, 0);
        }
        for (long long i = 4 * quads + t0; i < n; i += step) p[i] = 0;
    }
}

void zero_spans(const ZeroSpans& z, cudaStream_t s) {
    long long work = 0;
    for (int k = 0; k < z.count; ++k) work += (z.n[k] + 3) / 4;
    const long long blocks = std::min<long long>(std::max<long long>((work + 255) / 256, 1), 152 * 8);
    k_zero_spans<<<(int)blocks, 256, 0, s>>>(z);
}

}  // namespace

// Zero what the slotted edge hash counts from: bucket counts, overflow bits,
// list count and record count, and the edge hash's trim list (segment 2).
void reset_edge_hash(Solver* S, cudaStream_t s) {
    ZeroSpans z{};
    z.p[0] = S->eb_count;
    z.n[0] = S->nEB;
    z.p[1] = reinterpret_cast<int*>(S->eb_ovf_bits);
    z.n[1] = ((long long)S->nEB + 31) / 32;
    z.p[2] = S->eb_ovf_count;
    z.n[2] = 1;
    z.p[3] = reinterpret_cast<int*>(S->eb_late_count);
    z.n[3] = 2;
    z.p[4] = S->trim_count + 2;
    z.n[4] = 1;
    z.count = 5;
    zero_spans(z, s);
}

// Zero the triangle hash's bucket counts and its trim list count (segment 1).
void reset_triangle_hash(Solver* S, cudaStream_t s) {
    ZeroSpans z{};
    z.p[0] = S->tb_count;
    z.n[0] = S->nTB;
    z.p[1] = S->trim_count + 1;
    z.n[1] = 1;
    z.count = 2;
    zero_spans(z, s);
}


View Solver::view() const {
    View v{};
    v.tune = tune;
    v.P = dp;
    v.vcloth = vcloth;
    v.ecloth = ecloth;
    v.tcloth = tcloth;
    v.nV = nV;
    v.nE = nE;
    v.nT = nT;
    v.nB = bend_colors.empty() ? 0 : bend_colors.back();
    v.K = K;
    v.substep = 0;
    v.substeps = 1;
    v.pass = -1;
    v.last_it = 1;
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
    v.vt_off = vt_off;
    v.vt_tri = vt_tri;
    v.p_area = p_area;
    v.p_rest = p_rest;
    v.counts = counts;
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
    v.eb_slot = eb_slot;
    v.eb_ovf_bits = eb_ovf_bits;
    v.eb_ovf_list = eb_ovf_list;
    v.eb_ovf_count = eb_ovf_count;
    v.eb_ovf_start = eb_ovf_start;
    v.eb_late = eb_late;
    v.eb_late_count = eb_late_count;
    v.eb_late_cap = eb_late_cap;
    v.nb_count = nb_count;
    v.nb_idx = nb_idx;
    v.scan_tmp = scan_tmp;
    v.acc = acc;
    v.max_delta_bits = max_delta_bits;
    return v;
}

void Solver::drop_graphs() {
    for (auto& g : graphs)
        if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    graphs.clear();
}

void free_solver(Solver* S) {
    if (!S) return;
    if (S->stream) cudaStreamSynchronize(S->stream);
    S->drop_graphs();
    scene_detach(S, -1);
    for (Cloth& c : S->cl) {
        release_grid(S, c);
        dfree(c.fields_dev);
        free_dynamic(c);
    }
    dfree(S->vt_off);
    dfree(S->vt_tri);
    dfree(S->p_area);
    dfree(S->p_rest);
    dfree(S->dp);
    dfree(S->vcloth);
    dfree(S->ecloth);
    dfree(S->tcloth);
    dfree(S->pos[0]);
    dfree(S->pos[1]);
    dfree(S->prev);
    dfree(S->vel);
    dfree(S->rest);
    dfree(S->inv_mass);
    dfree(S->sp_off);
    dfree(S->sp_ent);
    dfree(S->te_off);
    dfree(S->te_ent);
    dfree(S->bj_off);
    dfree(S->bj_ent);
    dfree(S->bends);
    dfree(S->bend_rest);
    dfree(S->tris);
    dfree(S->edges);
    dfree(S->edge_rest);
    dfree(S->pin_target);
    dfree(S->pin_weight);
    dfree(S->pin_relax);
    dfree(S->counts);
    dfree(S->perf);
    dfree(S->max_delta_bits);
    dfree(S->pack);
    dfree(S->vcell);
    dfree(S->vb_count);
    dfree(S->vb_start);
    dfree(S->vb_ent);
    dfree(S->tb_count);
    dfree(S->tb_start);
    dfree(S->tb_ent);
    dfree(S->eb_count);
    dfree(S->eb_start);
    dfree(S->eb_ent);
    dfree(S->eb_slot);
    dfree(S->eb_ovf_bits);
    dfree(S->eb_ovf_list);
    dfree(S->eb_ovf_start);
    dfree(S->eb_ovf_count);
    dfree(S->eb_late);
    dfree(S->eb_late_count);
    dfree(S->nb_count);
    dfree(S->nb_idx);
    dfree(S->acc);
    dfree(S->scan_tmp);
    dfree(S->trim_list);
    dfree(S->trim_count);
    dfree(S->bend_ranges);
    for (auto& f : S->fused_ops) dfree(f.second.first);
    S->fused_ops.clear();
    PcgView& g = S->pcg;
    dfree(g.diag);
    dfree(g.pinv);
    dfree(g.r);
    dfree(g.z);
    dfree(g.d);
    dfree(g.q);
    dfree(g.offdiag);
    dfree(g.avg);
    dfree(g.red);
    dfree(g.partials);
    dfree(g.ticket);
    dfree(g.guard);
    dfree(g.max_delta_bits);
    dfree(S->pcg_blk);
    dfree(S->cap_edges);
    dfree(S->cap_rest);
    dfree(S->stage_idx);
    dfree(S->stage_target);
    dfree(S->stage_weight);
    dfree(S->stage_relax);
    for (int k = 0; k < 3; ++k) {
        if (S->aux[k]) cudaStreamDestroy(S->aux[k]);
        if (S->ev_join[k]) cudaEventDestroy(S->ev_join[k]);
    }
    if (S->ev_fork) cudaEventDestroy(S->ev_fork);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

bool sync_params(Solver* S) {
    if (!S->params_dirty) return true;
    if (!cuda_ok(cudaMemcpyAsync(S->dp, S->hp.data(), sizeof(Params) * S->K, cudaMemcpyHostToDevice, S->stream),
                 "upload solver parameters"))
        return false;
    S->params_dirty = false;
    return true;
}

namespace {

bool upload_pin_relax(Solver* S, int iterations) {
    if (S->pin_relax_iterations == iterations) return true;
    const float exponent = 1.0f / (float)std::max(iterations + 1, 1);
    for (int i = 0; i < S->nV; ++i) S->h_pin_relax[i] = pin_soft_relaxation(S->h_pin_weight[i], exponent);
    if (!dupload(S->pin_relax, S->h_pin_relax.data(), S->nV, S->stream, "pin relaxation upload")) return false;
    S->pin_relax_iterations = iterations;
    return true;
}

// Static SDF of one cloth: grid sizing (abi41.cu:6123-6218) and the device
// build.
bool build_static_sdf(Solver* S, int k, const float* tris, int count) {
    Params& P = S->hp[k];
    Cloth& C = S->cl[k];
    P.sdf_ready = 0;
    P.sdf_dim[0] = P.sdf_dim[1] = P.sdf_dim[2] = 0;
    P.sdf_origin[0] = P.sdf_origin[1] = P.sdf_origin[2] = 0.0f;
    P.sdf_voxel = 0.0f;
    P.sdf_signed = 0;
    P.static_tri_count = std::max(count, 0);
    S->params_dirty = true;
    C.sdf_build_ms = 0.0f;
    if (count <= 0) return true;
    if (!tris) return fail("static triangle data is required for SDF build");
    const auto t0 = std::chrono::high_resolution_clock::now();
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int q = 0; q < count * 3; ++q) {
        const float* v = tris + q * 3;
        if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2]))
            return fail("static triangle data contains non-finite coordinates");
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], v[a]);
            hi[a] = std::max(hi[a], v[a]);
        }
    }
    const SsblXpbdConfig& c = C.cfg;
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
    int device = 0;
    cudaGetDevice(&device);
    std::unique_lock<std::mutex> lock(g_sdf_mutex);
    SdfGrid* grid = nullptr;
    for (SdfGrid* g : g_sdf_cache)
        if (g->device == device && g->voxel_setting == c.static_sdf_voxel_size && g->band == band &&
            g->max_res == max_res && g->margin == margin && g->tris.size() == (size_t)count * 9 &&
            std::memcmp(g->tris.data(), tris, sizeof(float) * 9 * (size_t)count) == 0) {
            grid = g;
            break;
        }
    if (grid) {
        grid->refs += 1;
    } else {
        grid = new SdfGrid();
        grid->device = device;
        grid->tris.assign(tris, tris + (size_t)count * 9);
        grid->voxel_setting = c.static_sdf_voxel_size;
        grid->band = band;
        grid->max_res = max_res;
        grid->margin = margin;
        long long bytes = 0;
        {
            AllocAccount account(&bytes);
            if (!dalloc(&grid->sdf, voxels, "static SDF allocation") ||
                !dalloc(&grid->tris_dev, (size_t)count * 3, "static triangle upload")) {
                dfree(grid->sdf);
                delete grid;
                return false;
            }
        }
        grid->bytes = bytes;
        std::vector<float4> t4((size_t)count * 3);
        for (int q = 0; q < count * 3; ++q) t4[q] = make_float4(tris[q * 3], tris[q * 3 + 1], tris[q * 3 + 2], 0.0f);
        for (int a = 0; a < 3; ++a) {
            grid->dim[a] = dim[a];
            grid->origin[a] = lo[a];
        }
        grid->voxel = voxel;
        grid->is_signed = mesh_is_closed(tris, count) ? 1 : 0;
        // build it with this cloth's parameters pointing at the new grid
        for (int a = 0; a < 3; ++a) {
            P.sdf_dim[a] = dim[a];
            P.sdf_origin[a] = lo[a];
        }
        P.sdf_voxel = voxel;
        P.sdf = grid->sdf;
        P.static_tris = grid->tris_dev;
        P.sdf_signed = grid->is_signed;
        S->params_dirty = true;
        if (!dupload(grid->tris_dev, t4.data(), t4.size(), S->stream, "static triangle upload") || !sync_params(S)) {
            dfree(grid->sdf);
            dfree(grid->tris_dev);
            delete grid;
            return false;
        }
        launch_sdf_build(S->view(), k, voxels, S->stream);
        if (!cuda_ok(cudaGetLastError(), "build static SDF") ||
            !cuda_ok(cudaStreamSynchronize(S->stream), "sync static SDF build")) {
            dfree(grid->sdf);
            dfree(grid->tris_dev);
            delete grid;
            return false;
        }
        grid->refs = 1;
        g_sdf_cache.push_back(grid);
    }
    lock.unlock();
    release_grid(S, C);
    C.grid = grid;
    S->device_bytes += grid->bytes;
    for (int a = 0; a < 3; ++a) {
        P.sdf_dim[a] = grid->dim[a];
        P.sdf_origin[a] = grid->origin[a];
    }
    P.sdf_voxel = grid->voxel;
    P.sdf = grid->sdf;
    P.static_tris = grid->tris_dev;
    P.sdf_signed = grid->is_signed;
    if (!P.sdf_signed) C.sdf_unsigned += 1;
    P.sdf_ready = 1;
    S->params_dirty = true;
    C.sdf_rebuilds += 1;
    C.sdf_build_ms = (float)ms_since(t0);
    return true;
}

struct Range {
    int lo, hi;
};

Range cloth_range(const Solver* S, int cloth) {
    if (cloth < 0) return Range{0, S->nV};
    return Range{S->hp[cloth].vstart, S->hp[cloth].vstart + S->hp[cloth].V};
}

bool valid_cloth(const Solver* S, int cloth) { return S && cloth < S->K; }

// Vertex index over the caller-ordered concatenation -> stored index (-1
// outside).
int internal_vertex(const Solver* S, int i) {
    if (i < 0 || i >= S->ext_vstart[S->K]) return -1;
    const int k = (int)(std::upper_bound(S->ext_vstart.begin(), S->ext_vstart.end(), i) - S->ext_vstart.begin()) - 1;
    return S->hp[S->ext2int[k]].vstart + (i - S->ext_vstart[k]);
}

// Stored vertex index -> index over the caller-ordered concatenation.
int external_vertex(const Solver* S, int i) {
    int lo = 0, hi = S->K - 1;  // last cloth whose vstart <= i
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (S->hp[mid].vstart <= i) lo = mid; else hi = mid - 1;
    }
    return S->ext_vstart[S->int2ext[lo]] + (i - S->hp[lo].vstart);
}

}  // namespace

// Static SDF fields of the diagnostics block (abi41.cu:6105-6121), summed
// over the cloths; the grid shape is the first cloth's with a grid.
void sdf_diagnostics(Solver* S) {
    SsblXpbdDiagnostics& d = S->diag;
    d.static_triangle_count = 0;
    d.static_sdf_rebuild_count = 0;
    d.static_sdf_unsigned_fallback_count = 0;
    d.static_sdf_build_ms = 0.0f;
    d.static_sdf_grid_x = d.static_sdf_grid_y = d.static_sdf_grid_z = 0;
    d.static_sdf_voxel_count = 0;
    bool shaped = false;
    for (int e = 0; e < S->K; ++e) {  // the caller's cloth order
        const int k = S->ext2int.empty() ? e : S->ext2int[e];
        const bool last = e == S->K - 1;
        const Params& P = S->hp[k];
        const Cloth& C = S->cl[k];
        d.static_triangle_count += P.static_tri_count;
        d.static_sdf_rebuild_count += C.sdf_rebuilds;
        d.static_sdf_unsigned_fallback_count += C.sdf_unsigned;
        d.static_sdf_build_ms += C.sdf_build_ms;
        if (!shaped && (P.sdf_ready || last)) {
            d.static_sdf_grid_x = P.sdf_dim[0];
            d.static_sdf_grid_y = P.sdf_dim[1];
            d.static_sdf_grid_z = P.sdf_dim[2];
            shaped = P.sdf_ready != 0;
        }
        d.static_sdf_voxel_count += P.sdf_ready ? (long long)P.sdf_dim[0] * P.sdf_dim[1] * P.sdf_dim[2] : 0;
    }
    if (!shaped && S->K > 0) {
        const Params& P0 = S->hp[S->ext2int.empty() ? 0 : S->ext2int[0]];
        d.static_sdf_grid_x = P0.sdf_dim[0];
        d.static_sdf_grid_y = P0.sdf_dim[1];
        d.static_sdf_grid_z = P0.sdf_dim[2];
    }
}

bool upload_static(Solver* S, int cloth, const float* tris, int count) {
    if (!valid_cloth(S, cloth)) return fail("invalid static triangle update");
    count = std::max(count, 0);
    if (count > 0 && !tris) return fail("static triangle data is required when triangle count is nonzero");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    bool ok = true;
    for (int k = k0; k < k1 && ok; ++k) {
        S->cl[k].cfg.static_triangle_count = count;
        ok = build_static_sdf(S, k, tris, count);
    }
    sdf_diagnostics(S);
    return ok;
}

// Pin update: the new set replaces the cloth's (or, for cloth < 0, every
// cloth's) pins; a vertex listed twice keeps its last entry.  Only the
// vertices whose pin changes (old pins cleared, new pins set) travel to the
// device, as a compact list scattered by a kernel.
bool upload_pins(Solver* S, int cloth, const int* indices, const float* positions, const float* weights, int count) {
    if (!valid_cloth(S, cloth)) return fail("invalid solver handle");
    if (count < 0) return fail("invalid pin count");
    if (count > 0 && (!indices || !positions)) return fail("pin arrays are required when pin count is nonzero");
    const Range r = cloth_range(S, cloth);
    std::vector<int>& mod = S->pin_changed;
    mod.clear();
    auto mark = [&](int i) {
        if (S->pin_mark[i] != S->pin_epoch) {
            S->pin_mark[i] = S->pin_epoch;
            mod.push_back(i);
        }
    };
    ++S->pin_epoch;
    std::vector<int> keep;
    keep.reserve(S->pin_set.size());
    for (int i : S->pin_set) {
        if (i >= r.lo && i < r.hi) {
            S->h_pin_weight[i] = -1.0f;
            mark(i);
        } else {
            keep.push_back(i);
        }
    }
    for (int k = 0; k < count; ++k) {
        const int i = (cloth < 0 && S->permuted) ? internal_vertex(S, indices[k]) : r.lo + indices[k];
        if (indices[k] < 0 || i < r.lo || i >= r.hi) continue;
        S->h_pin_weight[i] = weights ? weights[k] : 1.0f;
        S->h_pin_target[i] = make_float4(positions[k * 3 + 0], positions[k * 3 + 1], positions[k * 3 + 2], 0.0f);
        mark(i);
        if (S->pin_kept[i] != S->pin_epoch) {
            S->pin_kept[i] = S->pin_epoch;
            keep.push_back(i);
        }
    }
    S->pin_set.swap(keep);
    if (cloth >= 0)
        S->cl[cloth].pin_count = count;
    else if (S->K == 1)
        S->cl[0].pin_count = count;
    const int n = (int)mod.size();
    if (n == 0) return true;
    const float exponent = 1.0f / (float)std::max(S->pin_relax_iterations + 1, 1);
    S->h_stage_target.resize(n);
    S->h_stage_weight.resize(n);
    S->h_stage_relax.resize(n);
    for (int k = 0; k < n; ++k) {
        const int i = mod[k];
        S->h_stage_target[k] = S->h_pin_target[i];
        S->h_stage_weight[k] = S->h_pin_weight[i];
        S->h_pin_relax[i] = S->pin_relax_iterations >= 0 ? pin_soft_relaxation(S->h_pin_weight[i], exponent) : 0.0f;
        S->h_stage_relax[k] = S->h_pin_relax[i];
    }
    AllocAccount account(&S->device_bytes);
    if (n > S->stage_capacity) {
        if (!cuda_ok(cudaStreamSynchronize(S->stream), "pin staging reallocation")) return false;
        S->device_bytes -= (long long)(sizeof(int) + sizeof(float4) + 2 * sizeof(float)) * S->stage_capacity;
        dfree(S->stage_idx);
        dfree(S->stage_target);
        dfree(S->stage_weight);
        dfree(S->stage_relax);
        S->stage_capacity = 0;
        const int cap = std::max(n, 256);
        if (!dalloc(&S->stage_idx, cap, "pin staging allocation") || !dalloc(&S->stage_target, cap, "pin staging allocation") ||
            !dalloc(&S->stage_weight, cap, "pin staging allocation") || !dalloc(&S->stage_relax, cap, "pin staging allocation"))
            return false;
        S->stage_capacity = cap;
    }
    if (!dupload(S->stage_idx, mod.data(), n, S->stream, "pin index upload") ||
        !dupload(S->stage_target, S->h_stage_target.data(), n, S->stream, "pin target upload") ||
        !dupload(S->stage_weight, S->h_stage_weight.data(), n, S->stream, "pin weight upload") ||
        !dupload(S->stage_relax, S->h_stage_relax.data(), n, S->stream, "pin relaxation upload"))
        return false;
    launch_pin_scatter(S->stage_idx, S->stage_target, S->stage_weight, S->stage_relax, n, S->pin_target, S->pin_weight,
                       S->pin_relax, S->nV, S->stream);
    return cuda_ok(cudaGetLastError(), "pin upload");
}

bool set_colliders(Solver* S, int cloth, const SsblXpbdRuntimeColliders& c) {
    if (!valid_cloth(S, cloth)) return fail("invalid runtime collider update");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    for (int k = k0; k < k1; ++k) {
        S->cl[k].colliders = c;
        load_colliders(S->hp[k], c);
    }
    S->params_dirty = true;
    return true;
}

// Force fields of a cloth (cloth < 0: every cloth), at most 64
// (abi41.cu:5920-5960).
bool upload_fields(Solver* S, int cloth, const SsblXpbdForceField* fields, int count, int unsupported) {
    if (!valid_cloth(S, cloth)) return fail("invalid force field update");
    if (count < 0 || count > kMaxFieldRecords) return fail("force field count exceeds SSBL maximum");
    if (count > 0 && !fields) return fail("missing force field data");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    AllocAccount account(&S->device_bytes);
    for (int k = k0; k < k1; ++k) {
        Cloth& C = S->cl[k];
        C.unsupported_force_field_count = std::max(unsupported, 0);
        if (count > C.fields_capacity) {
            if (!cuda_ok(cudaStreamSynchronize(S->stream), "force field reallocation")) return false;
            S->device_bytes -= (long long)sizeof(SsblXpbdForceField) * C.fields_capacity;
            dfree(C.fields_dev);
            C.fields_capacity = 0;
            if (!dalloc(&C.fields_dev, count, "force field allocation")) return false;
            C.fields_capacity = count;
        }
        if (count > 0 && !dupload(C.fields_dev, fields, count, S->stream, "upload force fields")) return false;
        C.force_field_count = count;
        Params& P = S->hp[k];
        P.fields = C.fields_dev;
        P.field_count = count;
        P.needs_normal = (P.pressure_on || count > 0) ? 1 : 0;
    }
    S->params_dirty = true;
    return cuda_ok(cudaStreamSynchronize(S->stream), "upload force fields");
}

bool upload_positions(Solver* S, int cloth, const float* positions, int max_floats) {
    if (!valid_cloth(S, cloth) || !positions) return fail("invalid position upload");
    const Range r = cloth_range(S, cloth);
    const int n = r.hi - r.lo;
    if (max_floats < n * 3) return fail("invalid position upload");
    std::vector<float4> p4(n);
    for (int i = 0; i < n; ++i) {
        // a whole-handle upload lists the cloths in the caller's order
        const int src = (cloth < 0 && S->permuted) ? external_vertex(S, i) : i;
        p4[i] = make_float4(positions[src * 3], positions[src * 3 + 1], positions[src * 3 + 2], S->h_w[r.lo + i]);
    }
    return dupload(S->pos[0] + r.lo, p4.data(), n, S->stream, "upload positions") &&
           dupload(S->prev + r.lo, p4.data(), n, S->stream, "upload previous positions") &&
           cuda_ok(cudaStreamSynchronize(S->stream), "upload positions");
}

bool download_positions(Solver* S, int cloth, float* out, int max_floats) {
    if (!valid_cloth(S, cloth) || !out) return fail("invalid position download");
    const Range r = cloth_range(S, cloth);
    const int n = r.hi - r.lo;
    if (max_floats < n * 3) return fail("invalid position download");
    launch_pack_positions(S->pack + 3ll * r.lo, S->pos[0] + r.lo, n, S->stream);
    if (cloth < 0 && S->permuted) {
        // whole handle: each cloth's block goes to its place in the caller's order
        if (!cuda_ok(cudaGetLastError(), "pack positions")) return false;
        for (int k = 0; k < S->K; ++k) {
            const Params& P = S->hp[S->ext2int[k]];
            if (P.V > 0 && !cuda_ok(cudaMemcpyAsync(out + 3ll * S->ext_vstart[k], S->pack + 3ll * P.vstart, sizeof(float) * 3 * P.V,
                                                    cudaMemcpyDeviceToHost, S->stream),
                                    "download ABI41 positions"))
                return false;
        }
        return cuda_ok(cudaStreamSynchronize(S->stream), "download ABI41 positions");
    }
    return cuda_ok(cudaGetLastError(), "pack positions") &&
           cuda_ok(cudaMemcpyAsync(out, S->pack + 3ll * r.lo, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, S->stream),
                   "download ABI41 positions") &&
           cuda_ok(cudaStreamSynchronize(S->stream), "download ABI41 positions");
}

bool reset_cloths(Solver* S, int cloth) {
    if (!valid_cloth(S, cloth)) return fail("invalid solver handle");
    const Range r = cloth_range(S, cloth);
    const size_t n = (size_t)(r.hi - r.lo);
    if (!cuda_ok(cudaMemcpyAsync(S->pos[0] + r.lo, S->rest + r.lo, sizeof(float4) * n, cudaMemcpyDeviceToDevice, S->stream),
                 "reset positions") ||
        !cuda_ok(cudaMemcpyAsync(S->prev + r.lo, S->rest + r.lo, sizeof(float4) * n, cudaMemcpyDeviceToDevice, S->stream),
                 "reset previous positions") ||
        !cuda_ok(cudaMemsetAsync(S->vel + r.lo, 0, sizeof(float4) * n, S->stream), "reset velocities") ||
        !cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, S->stream), "reset ABI41 diagnostics") ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "reset solver"))
        return false;
    S->diag = SsblXpbdDiagnostics{};
    S->diag.finite_flag = 1;
    return true;
}

bool set_active(Solver* S, int cloth, bool active) {
    if (!valid_cloth(S, cloth)) return fail("invalid cloth index");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    for (int k = k0; k < k1; ++k) S->hp[k].active = active ? 1 : 0;
    S->params_dirty = true;
    return true;
}

// ------------------------------------------------------------ creation --

Solver* create_solver(const SsblXpbdConfig* in_configs, const SsblXpbdMesh* in_meshes, int K) {
    if (!in_configs || !in_meshes || K < 1) {
        fail("invalid ABI41 solver create request");
        return nullptr;
    }
    Solver* S = new Solver();
    AllocAccount account(&S->device_bytes);
    S->K = K;
    S->key_ieee = g_default_key_ieee.load();
    S->cl.resize(K);
    S->hp.assign(K, Params{});
    // internal order: grouped by self-collision mode, stable within a group
    S->int2ext.resize(K);
    for (int k = 0; k < K; ++k) S->int2ext[k] = k;
    // none, fast, strict with a budget under 32 slots, strict: the cloths
    // whose queries depend on bucket order (fast, small-budget strict) form
    // one contiguous run, and so do the strict ones
    auto mode_key = [&](int k) {
        const SsblXpbdConfig& c = in_configs[k];
        if (!c.self_collision) return 0;
        if (c.self_collision_mode == 1) return 1;
        return std::min(std::max(c.max_self_collision_neighbors, 1), kBucketSlots) < kBucketSlots ? 2 : 3;
    };
    std::stable_sort(S->int2ext.begin(), S->int2ext.end(), [&](int a, int b) { return mode_key(a) < mode_key(b); });
    S->ext2int.resize(K);
    S->ext_vstart.assign(K + 1, 0);
    std::vector<SsblXpbdConfig> cfg_sorted(K);
    std::vector<SsblXpbdMesh> mesh_sorted(K);
    for (int k = 0; k < K; ++k) {
        S->ext2int[S->int2ext[k]] = k;
        S->permuted |= S->int2ext[k] != k;
        cfg_sorted[k] = in_configs[S->int2ext[k]];
        mesh_sorted[k] = in_meshes[S->int2ext[k]];
    }
    for (int k = 0; k < K; ++k) S->ext_vstart[k + 1] = S->ext_vstart[k] + std::max(in_configs[k].vertex_count, 0);
    const SsblXpbdConfig* configs = cfg_sorted.data();
    const SsblXpbdMesh* meshes = mesh_sorted.data();
    auto bail = [&](int k, const std::string& msg) -> Solver* {
        if (!msg.empty()) fail(K > 1 ? "batch cloth " + std::to_string(S->int2ext[k]) + ": " + msg : msg);
        free_solver(S);
        return nullptr;
    };

    // Per-cloth validation and ranges in the concatenated arrays.
    long long tv = 0, te = 0, tt = 0, tl = 0;
    for (int k = 0; k < K; ++k) {
        const SsblXpbdConfig* config = &configs[k];
        const SsblXpbdMesh* mesh = &meshes[k];
        if (config->vertex_count < 0 || config->edge_count < 0 || config->triangle_count < 0 || !std::isfinite(config->dt) ||
            !(config->dt > 0.0f) || !mesh->positions || !mesh->inv_mass)
            return bail(k, "invalid ABI41 solver create request");
        Cloth& C = S->cl[k];
        SsblXpbdConfig& c = C.cfg;
        c = *config;
        sanitize(c);
        if (c.bend_count > 0 && (!mesh->bends || !mesh->bend_rest_lengths))
            return bail(k, "ABI41 bend constraints require bend pairs and rest lengths");
        if (c.lra_count > 0 && (!mesh->lra_edges || !mesh->lra_rest_lengths))
            return bail(k, "ABI41 LRA constraints require edge pairs and rest lengths");
        if (c.edge_color_count > 0) {
            if (!mesh->edge_color_offsets) return bail(k, "ABI41 edge color offsets are required");
            C.edge_colors.assign(mesh->edge_color_offsets, mesh->edge_color_offsets + c.edge_color_count + 1);
        }
        if (c.bend_color_count > 0) {
            if (!mesh->bend_color_offsets) return bail(k, "ABI41 bend color offsets are required");
            C.bend_colors.assign(mesh->bend_color_offsets, mesh->bend_color_offsets + c.bend_color_count + 1);
        }
        C.colliders.use_ground = c.use_ground;
        C.colliders.ground_height = c.ground_height;
        C.colliders.use_wall = c.use_wall;
        std::memcpy(C.colliders.wall_origin, c.wall_origin, sizeof(c.wall_origin));
        std::memcpy(C.colliders.wall_normal, c.wall_normal, sizeof(c.wall_normal));
        C.colliders.use_sphere = c.use_sphere;
        std::memcpy(C.colliders.sphere_center, c.sphere_center, sizeof(c.sphere_center));
        C.colliders.sphere_radius = c.sphere_radius;
        Params& P = S->hp[k];
        P.vstart = (int)tv;
        P.estart = (int)te;
        P.tstart = (int)tt;
        P.V = c.vertex_count;
        P.E = c.edge_count;
        P.T = c.triangle_count;
        P.B = c.bend_count;
        P.L = c.lra_count;
        tv += P.V;
        te += P.E;
        tt += P.T;
        tl += P.L;
    }
    if (tv > (1 << 30) || te > (1 << 30) || tt > (1 << 30) || tl > (1 << 30)) return bail(0, "batch is too large");
    S->nV = (int)tv;
    S->nE = (int)te;
    S->nT = (int)tt;
    S->nL = (int)tl;
    const int nV = S->nV, nE = S->nE, nT = S->nT;

    if (!cuda_ok(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking), "create solver stream")) return bail(0, "");
    for (int k = 0; k < 3; ++k)
        if (!cuda_ok(cudaStreamCreateWithFlags(&S->aux[k], cudaStreamNonBlocking), "create solver stream") ||
            !cuda_ok(cudaEventCreateWithFlags(&S->ev_join[k], cudaEventDisableTiming), "create solver event"))
            return bail(0, "");
    if (!cuda_ok(cudaEventCreateWithFlags(&S->ev_fork, cudaEventDisableTiming), "create solver event")) return bail(0, "");

    // Concatenated host arrays; indices outside their cloth become -1.
    S->h_inv.resize(nV);
    S->h_w.resize(nV);
    std::vector<float4> rest4(nV), zero4(nV, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    std::vector<int2> springs(nE), tethers(S->nL), jbends;
    std::vector<float> spring_rest(nE), tether_rest(S->nL), jbend_rest;
    std::vector<int4> tris(nT);
    std::vector<int> vmap, emap, tmap;
    if (K > 1) {
        vmap.resize(nV);
        emap.resize(nE);
        tmap.resize(nT);
    }
    int max_colors = 0;
    for (int k = 0; k < K; ++k) max_colors = std::max(max_colors, (int)S->cl[k].bend_colors.size() - 1);
    std::vector<std::vector<int2>> color_bends(std::max(max_colors, 0));
    std::vector<int2> bend_local((size_t)std::max(max_colors, 0) * K, make_int2(0, 0));  // within the colour
    std::vector<std::vector<float>> color_rest(std::max(max_colors, 0));
    int lpos = 0;
    for (int k = 0; k < K; ++k) {
        const SsblXpbdMesh* mesh = &meshes[k];
        Cloth& C = S->cl[k];
        const SsblXpbdConfig& c = C.cfg;
        const Params& P = S->hp[k];
        const int V = P.V, E = P.E, T = P.T, B = P.B, L = P.L, vs = P.vstart;
        auto gidx = [&](int i) { return (i >= 0 && i < V) ? vs + i : kInvalid; };
        for (int i = 0; i < V; ++i) {
            const float im = mesh->inv_mass[i];
            S->h_inv[vs + i] = im;
            S->h_w[vs + i] = im > 0.0f ? im : 0.0f;
            rest4[vs + i] = make_float4(mesh->positions[i * 3], mesh->positions[i * 3 + 1], mesh->positions[i * 3 + 2], S->h_w[vs + i]);
            if (K > 1) vmap[vs + i] = k;
        }
        for (int e = 0; e < E; ++e) {
            const int i = mesh->edges ? mesh->edges[e * 2] : 0, j = mesh->edges ? mesh->edges[e * 2 + 1] : 0;
            springs[P.estart + e] = make_int2(gidx(std::max(i, 0)), gidx(std::max(j, 0)));
            spring_rest[P.estart + e] = mesh->edge_rest_lengths ? mesh->edge_rest_lengths[e] : 0.0f;
            if (K > 1) emap[P.estart + e] = k;
        }
        for (int q = 0; q < L; ++q) {
            tethers[lpos + q] = make_int2(gidx(mesh->lra_edges[q * 2]), gidx(mesh->lra_edges[q * 2 + 1]));
            tether_rest[lpos + q] = mesh->lra_rest_lengths[q];
        }
        lpos += L;
        if (B > 0 && C.bend_colors.empty()) {
            for (int q = 0; q < B; ++q) {
                jbends.push_back(make_int2(gidx(mesh->bends[q * 2]), gidx(mesh->bends[q * 2 + 1])));
                jbend_rest.push_back(mesh->bend_rest_lengths[q]);
            }
            S->jacobi_bends = true;
        } else if (B > 0) {
            // bends of colour j: the caller's range [off_j, off_j+1), clipped
            // to the cloth's bends
            for (size_t j = 0; j + 1 < C.bend_colors.size(); ++j) {
                const int b0 = std::max(C.bend_colors[j], 0), b1 = std::min(C.bend_colors[j + 1], B);
                bend_local[j * K + k] = make_int2((int)color_bends[j].size(), std::max(b1 - b0, 0));
                for (int q = b0; q < b1; ++q) {
                    color_bends[j].push_back(make_int2(gidx(mesh->bends[q * 2]), gidx(mesh->bends[q * 2 + 1])));
                    color_rest[j].push_back(mesh->bend_rest_lengths[q]);
                }
            }
        }
        for (int t = 0; t < T; ++t) {
            const int* tr = mesh->triangles ? mesh->triangles + t * 3 : nullptr;
            const int a = tr ? std::max(tr[0], 0) : 0, b = tr ? std::max(tr[1], 0) : 0, cc = tr ? std::max(tr[2], 0) : 0;
            tris[P.tstart + t] = make_int4(a, b, cc, 0);  // local for the wing count
            if (K > 1) tmap[P.tstart + t] = k;
        }
        C.wing_count = T > 1 ? count_wings(V, tris, P.tstart, P.tstart + T) : 0;
        for (int t = 0; t < T; ++t) {
            int4& tr = tris[P.tstart + t];
            tr = make_int4(gidx(tr.x), gidx(tr.y), gidx(tr.z), 0);
        }
        (void)c;
    }
    std::vector<int2> cbends;
    std::vector<float> cbend_rest;
    S->bend_colors.assign(1, 0);
    for (int j = 0; j < max_colors; ++j) {
        cbends.insert(cbends.end(), color_bends[j].begin(), color_bends[j].end());
        cbend_rest.insert(cbend_rest.end(), color_rest[j].begin(), color_rest[j].end());
        S->bend_colors.push_back((int)cbends.size());
    }
    if (cbends.empty()) S->bend_colors.clear();
    S->nB = (int)cbends.size();
    S->h_bend_ranges.assign(bend_local.size(), make_int2(0, 0));
    for (int j = 0; j < max_colors && !cbends.empty(); ++j)
        for (int k = 0; k < K; ++k) {
            const int2 r = bend_local[(size_t)j * K + k];
            S->h_bend_ranges[(size_t)j * K + k] = make_int2(S->bend_colors[j] + r.x, r.y);
        }

    std::vector<int> sp_off, te_off, bj_off;
    std::vector<int2> sp_ent, te_ent, bj_ent;
    build_pair_csr(nV, springs, spring_rest, &sp_off, &sp_ent);
    build_pair_csr(nV, tethers, tether_rest, &te_off, &te_ent);
    if (S->jacobi_bends) build_pair_csr(nV, jbends, jbend_rest, &bj_off, &bj_ent);
    S->h_pin_weight.assign(nV, -1.0f);
    S->h_pin_target.assign(nV, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    S->h_pin_relax.assign(nV, 0.0f);
    // vertex -> incident triangles in triangle order (vertex normals)
    std::vector<int> vt_off(nV + 1, 0), vt_tri;
    for (int t = 0; t < nT; ++t) {
        const int4 tr = tris[t];
        const int ids[3] = {tr.x, tr.y, tr.z};
        for (int a = 0; a < 3; ++a)
            if (ids[a] >= 0 && ids[a] < nV) vt_off[ids[a] + 1]++;
    }
    for (int i = 0; i < nV; ++i) vt_off[i + 1] += vt_off[i];
    vt_tri.assign(vt_off[nV], -1);
    {
        std::vector<int> cur(vt_off.begin(), vt_off.end() - 1);
        for (int t = 0; t < nT; ++t) {
            const int4 tr = tris[t];
            const int ids[3] = {tr.x, tr.y, tr.z};
            for (int a = 0; a < 3; ++a)
                if (ids[a] >= 0 && ids[a] < nV) vt_tri[cur[ids[a]]++] = t;
        }
    }
    // volume pressure shares and scales per cloth
    const float accel_scale = env_scale("SSBL_ABI41_PRESSURE_UI_ACCEL_SCALE", 1792.0f, 1.0f, 8192.0f);
    const float impulse_scale = env_scale("SSBL_ABI41_PRESSURE_IMPULSE_REST_SCALE", 0.85f, 0.05f, 8.0f);
    const float velocity_scale = env_scale("SSBL_ABI41_PRESSURE_VELOCITY_REST_SCALE", 2.25f, 0.10f, 16.0f);
    const float object_scale = env_scale("SSBL_ABI41_PRESSURE_VELOCITY_OBJECT_SCALE", 0.08f, 0.005f, 1.0f);
    std::vector<float> p_area, p_rest;
    bool any_pressure = false;
    for (int k = 0; k < K; ++k) {
        const SsblXpbdConfig& c = S->cl[k].cfg;
        S->cl[k].pressure_on = c.use_volume_pressure && c.pressure_strength > 0.0f && std::isfinite(c.pressure_strength);
        any_pressure |= S->cl[k].pressure_on;
    }
    if (any_pressure) {
        p_area.assign(nV, 0.0f);
        p_rest.assign(nV, 0.0f);
        for (int k = 0; k < K; ++k) {
            Params& P = S->hp[k];
            const SsblXpbdMesh* mesh = &meshes[k];
            // local triangle indices (negative indices clamped to 0 as at create)
            std::vector<int4> lt(P.T);
            for (int t = 0; t < P.T; ++t) {
                const int* tr = mesh->triangles ? mesh->triangles + 3 * t : nullptr;
                lt[t] = make_int4(tr ? std::max(tr[0], 0) : 0, tr ? std::max(tr[1], 0) : 0, tr ? std::max(tr[2], 0) : 0, 0);
            }
            const std::vector<float> a = pressure_area_shares(P.V, lt, 0, lt.size(), mesh->positions);
            const std::vector<float> r = pressure_rest_scales(P.V, mesh->edges, mesh->edge_rest_lengths, P.E, a);
            std::copy(a.begin(), a.end(), p_area.begin() + P.vstart);
            std::copy(r.begin(), r.end(), p_rest.begin() + P.vstart);
            P.pressure_velocity_length_scale = pressure_velocity_length(P.V, mesh->positions, r, object_scale);
        }
    }
    S->pin_mark.assign(nV, 0);
    S->pin_kept.assign(nV, 0);

    // Parameters and self-collision table sizes.
    int wings = 0;
    for (int k = 0; k < K; ++k) {
        Cloth& C = S->cl[k];
        const SsblXpbdConfig& c = C.cfg;
        Params& P = S->hp[k];
        P.active = 1;
        P.sub_dt = c.dt;
        P.frame_dt = c.dt;
        P.damping = c.damping;
        for (int a = 0; a < 3; ++a) P.gravity[a] = c.gravity[a];
        P.stretch_compliance = c.stretch_compliance;
        P.bend_compliance = c.bend_compliance;
        P.lra_compliance = c.lra_compliance;
        P.margin = c.collision_margin;
        P.thickness = c.cloth_thickness;
        P.friction = c.contact_friction;
        P.tangent_damping = c.contact_tangent_damping;
        load_colliders(P, C.colliders);
        const float radius = self_radius(c);
        P.self_radius = radius;
        P.key_ieee = S->key_ieee;
        P.self_mode = c.self_collision_mode;
        P.max_neighbors = c.max_self_collision_neighbors;
        P.stretch_strength = c.stretch_optimization_strength;
        P.pressure_on = C.pressure_on ? 1 : 0;
        P.pressure_strength = std::max(c.pressure_strength, 0.0f);
        P.pressure_accel_scale = accel_scale;
        P.pressure_impulse_rest_scale = impulse_scale;
        P.pressure_velocity_rest_scale = velocity_scale;
        P.needs_normal = P.pressure_on;
        P.fields = nullptr;
        P.field_count = 0;
        C.self_enabled = c.self_collision != 0 && radius > 0.0f && P.V > 0;
        C.interval = std::max(c.self_collision_interval, 1);
        C.passes = std::max(1, std::min(c.fast_self_collision_passes, 8));
        C.fast = c.self_collision_mode == 1;
        C.order_buckets = C.fast || std::min(std::max(c.max_self_collision_neighbors, 1), 32) < 32;
        P.self_on = C.self_enabled ? 1 : 0;
        P.self_interval = C.interval;
        P.self_passes = C.passes;
        if (C.self_enabled) {
            S->self_any = true;
            const float cell = std::max(radius * 1.8f, 1.0e-3f);
            P.vcell = P.tcell = P.ecell = cell;
            P.vhash = P.V >= 128;
            P.thash = P.T >= 64;
            P.ehash = P.E >= 64;
            P.vbuckets = P.vhash ? next_pow2(std::max(1024, P.V * 4)) : 0;
            P.tbuckets = P.thash ? next_pow2(std::max(1024, P.T * 4)) : 0;
            P.ebuckets = P.ehash ? next_pow2(std::max(1024, P.E * 4)) : 0;
            if ((long long)S->nVB + P.vbuckets > (1ll << 30) || (long long)S->nTB + P.tbuckets > (1ll << 30) ||
                (long long)S->nEB + P.ebuckets > (1ll << 30))
                return bail(k, "self collision tables are too large");
            P.vbase = S->nVB;
            P.tbase = S->nTB;
            P.ebase = S->nEB;
            S->nVB += P.vbuckets;
            S->nTB += P.tbuckets;
            S->nEB += P.ebuckets;
        }
        wings += C.wing_count;
    }
    long long tri_entries = 0, edge_entries = 0;
    for (int k = 0; k < K; ++k) {
        if (S->hp[k].thash) tri_entries += (long long)S->hp[k].T * kMaxPrimitiveCells;
        if (S->hp[k].ehash) edge_entries += (long long)S->hp[k].E * kMaxPrimitiveCells;
    }
    S->pcg_on = S->spring_any = false;
    for (int k = 0; k < K; ++k) {
        const bool on = S->cl[k].cfg.stretch_optimization_enabled != 0;
        S->pcg_on |= on;
        S->spring_any |= !on && S->hp[k].E > 0;
    }

    bool ok = dalloc(&S->dp, K, "parameter allocation") && dalloc(&S->pos[0], nV, "position allocation") &&
              dalloc(&S->pos[1], nV, "position allocation") && dalloc(&S->prev, nV, "previous position allocation") &&
              dalloc(&S->vel, nV, "velocity allocation") && dalloc(&S->rest, nV, "rest position allocation") &&
              dalloc(&S->inv_mass, nV, "inverse mass allocation") && dalloc(&S->sp_off, nV + 1, "spring CSR allocation") &&
              dalloc(&S->sp_ent, sp_ent.size(), "spring CSR allocation") &&
              dalloc(&S->te_off, nV + 1, "tether CSR allocation") && dalloc(&S->te_ent, te_ent.size(), "tether CSR allocation") &&
              dalloc(&S->bends, cbends.size(), "bend pair allocation") &&
              dalloc(&S->bend_rest, cbend_rest.size(), "bend rest allocation") && dalloc(&S->tris, nT, "triangle allocation") &&
              dalloc(&S->edges, nE, "edge allocation") && dalloc(&S->edge_rest, nE, "edge rest allocation") &&
              dalloc(&S->pin_target, nV, "pin target allocation") && dalloc(&S->pin_weight, nV, "pin weight allocation") &&
              dalloc(&S->pin_relax, nV, "pin relaxation allocation") &&
              dalloc(&S->counts, kCntSlots, "ABI41 diagnostic allocation") && dalloc(&S->perf, kPerfStripes * kPerfStride, "work counter allocation") &&
              dalloc(&S->max_delta_bits, 1, "self max smoothed delta allocation") &&
              dalloc(&S->pack, (size_t)nV * 3, "download staging allocation");
    if (ok && !S->h_bend_ranges.empty())
        ok = dalloc(&S->bend_ranges, S->h_bend_ranges.size(), "bend range allocation");
    if (ok && K > 1)
        ok = dalloc(&S->vcloth, nV, "cloth map allocation") && dalloc(&S->ecloth, nE, "cloth map allocation") &&
             dalloc(&S->tcloth, nT, "cloth map allocation");
    if (ok && S->jacobi_bends)
        ok = dalloc(&S->bj_off, nV + 1, "bend CSR allocation") && dalloc(&S->bj_ent, bj_ent.size(), "bend CSR allocation");
    if (ok && nT > 0)
        ok = dalloc(&S->vt_off, nV + 1, "incident triangle allocation") &&
             dalloc(&S->vt_tri, vt_tri.size(), "incident triangle allocation");
    if (ok && any_pressure)
        ok = dalloc(&S->p_area, nV, "pressure area allocation") && dalloc(&S->p_rest, nV, "pressure scale allocation");
    if (ok && S->self_any) {
        ok = dalloc(&S->nb_count, nV, "self collision count allocation") &&
             dalloc(&S->nb_idx, (size_t)nV * kNeighborSlots, "self collision index allocation") &&
             dalloc(&S->acc, nV, "self accumulation allocation") &&
             dalloc(&S->scan_tmp, 3 * ((size_t)std::max(std::max(S->nVB, S->nTB), S->nEB) / 4096 + 2), "bucket scan allocation");
        S->scan_seg = std::max(std::max(S->nVB, S->nTB), S->nEB) / 4096 + 2;
        if (ok && S->nVB > 0)
            ok = dalloc(&S->vcell, nV, "self collision cell allocation") &&
                 dalloc(&S->vb_count, S->nVB, "self collision hash count allocation") &&
                 dalloc(&S->vb_start, S->nVB + 1, "self collision hash start allocation") &&
                 dalloc(&S->vb_ent, nV, "self collision hash index allocation");
        // overflowing buckets (more than 32 members) listed by the scans
        if (ok)
            ok = dalloc(&S->trim_list, (size_t)std::max(std::max(S->nVB, S->nTB), S->nEB) * 3, "bucket trim list allocation") &&
                 dalloc(&S->trim_count, 3, "bucket trim list allocation");
        if (ok && S->nTB > 0)
            ok = dalloc(&S->tb_count, S->nTB, "self triangle hash count allocation") &&
                 dalloc(&S->tb_start, S->nTB + 1, "self triangle hash start allocation") &&
                 dalloc(&S->tb_ent, (size_t)tri_entries, "self triangle hash index allocation");
        if (ok && S->nEB > 0) {
            // a bucket past kEdgeSlots members holds at least kEdgeSlots + 1 entries
            S->eb_ovf_cap = std::min<long long>(S->nEB, edge_entries / (kEdgeSlots + 1) + 1);
            // room for the insertions past the slots of a crowded build (the
            // hashed edges' count, at least 2^20); a build with more falls
            // back to a second walk of the cells.  XPBD_GB300_EDGE_LATE_CAP
            // lowers it (tests run the fallback that way).
            S->eb_late_cap = std::min<long long>(edge_entries, std::max<long long>(1ll << 20, edge_entries / kMaxPrimitiveCells));
            if (const char* raw = std::getenv("XPBD_GB300_EDGE_LATE_CAP")) {
                const long long cap = std::atoll(raw);
                if (cap >= 0) S->eb_late_cap = std::min(S->eb_late_cap, cap);
            }
            ok = dalloc(&S->eb_count, S->nEB, "self edge hash count allocation") &&
                 dalloc(&S->eb_start, S->nEB + 1, "self edge hash start allocation") &&
                 dalloc(&S->eb_ent, (size_t)edge_entries, "self edge hash index allocation") &&
                 dalloc(&S->eb_slot, (size_t)S->nEB * kEdgeSlots, "self edge hash slot allocation") &&
                 dalloc(&S->eb_ovf_bits, ((size_t)S->nEB + 31) / 32, "self edge hash overflow allocation") &&
                 dalloc(&S->eb_ovf_list, (size_t)S->eb_ovf_cap, "self edge hash overflow allocation") &&
                 dalloc(&S->eb_ovf_start, (size_t)S->eb_ovf_cap, "self edge hash overflow allocation") &&
                 dalloc(&S->eb_ovf_count, 1, "self edge hash overflow allocation") &&
                 dalloc(&S->eb_late, (size_t)std::max<long long>(S->eb_late_cap, 1), "self edge hash overflow allocation") &&
                 dalloc(&S->eb_late_count, 1, "self edge hash overflow allocation");
        }
    }
    // Hard-stretch buffers.  The caps follow the caller's edge colouring when
    // one is given (edges already sorted by colour; each pass sweeps the
    // colours forward then backward, abi41.cu:7769-7793); without one each
    // pass is a single Jacobi pass over all of the cloth's edges
    // (abi41.cu:7794-7801), run as a per-vertex gather (P.cap_jacobi).
    // In a batch colour c of every coloured cloth with the hard polish forms
    // cap launch c (cloths share no vertex); a caller's offsets are clamped to
    // the cloth's edges, which is what the bounds check of a one-cloth launch
    // does with them.
    std::vector<int2> cap_edges;
    std::vector<float> cap_rest;
    std::vector<int> blk_cloth;
    if (ok && S->pcg_on) {
        S->pcg_nnz = 0;
        S->pcg_blocks = 0;
        S->pcg_hard = false;
        S->cap_jacobi = false;
        std::vector<std::vector<int>> col_off(K), col_order(K);
        int ncol = 0;
        for (int k = 0; k < K; ++k) {
            Params& P = S->hp[k];
            P.pcg_on = S->cl[k].cfg.stretch_optimization_enabled != 0 ? 1 : 0;
            P.pcg_hard = P.pcg_on && P.stretch_strength >= 0.95f ? 1 : 0;
            P.pcg_block0 = S->pcg_blocks;
            P.pcg_nblocks = 0;
            if (!P.pcg_on) continue;
            const int nnz = sp_off[P.vstart + P.V] - sp_off[P.vstart];
            if (nnz == 0) return bail(k, "PCG stretch optimization found no valid CSR edges");
            S->pcg_nnz += nnz;
            P.pcg_nblocks = pcg_blocks(P.V);
            S->pcg_blocks += P.pcg_nblocks;
            blk_cloth.insert(blk_cloth.end(), P.pcg_nblocks, k);
            P.cap_jacobi = 0;
            if (!P.pcg_hard) continue;
            S->pcg_hard = true;
            if (S->cl[k].edge_colors.empty()) {
                P.cap_jacobi = 1;
                S->cap_jacobi = true;
                continue;
            }
            col_off[k] = S->cl[k].edge_colors;
            col_order[k].resize(P.E);
            for (int e = 0; e < P.E; ++e) col_order[k][e] = e;
            ncol = std::max(ncol, (int)col_off[k].size() - 1);
        }
        S->cap_colors.assign(1, 0);
        for (int c = 0; c < ncol; ++c) {
            for (int k = 0; k < K; ++k) {
                const Params& P = S->hp[k];
                if (!P.pcg_hard || c + 1 >= (int)col_off[k].size()) continue;
                const int lo = std::min(std::max(col_off[k][c], 0), P.E), hi = std::min(std::max(col_off[k][c + 1], 0), P.E);
                for (int e = lo; e < hi; ++e) {
                    const int ge = P.estart + col_order[k][e];
                    cap_edges.push_back(springs[ge]);
                    cap_rest.push_back(spring_rest[ge]);
                }
            }
            S->cap_colors.push_back((int)cap_edges.size());
        }
        S->cap_count = (int)cap_edges.size();
        PcgView& g = S->pcg;
        ok = dalloc(&g.diag, 2 * (size_t)nV, "PCG diagonal block allocation") &&
             dalloc(&g.pinv, 2 * (size_t)nV, "PCG preconditioner allocation") && dalloc(&g.r, nV, "PCG residual allocation") &&
             dalloc(&g.z, nV, "PCG preconditioned residual allocation") && dalloc(&g.d, nV, "PCG search direction allocation") &&
             dalloc(&g.q, nV, "PCG A*d allocation") && dalloc(&g.offdiag, sp_ent.size(), "PCG offdiagonal allocation") &&
             dalloc(&g.avg, nV, "stretch cap accumulation allocation") &&
             dalloc(&g.red, (size_t)K * kRedSlots, "PCG reduction allocation") &&
             dalloc(&g.partials, (size_t)S->pcg_blocks * (kThreads / 32), "PCG partial sum allocation") &&
             dalloc(&g.ticket, K, "PCG ticket allocation") && dalloc(&g.guard, 1, "PCG guard counter allocation") &&
             dalloc(&g.max_delta_bits, 1, "PCG max delta allocation") &&
             dalloc(&S->pcg_blk, S->pcg_blocks, "PCG block map allocation") &&
             dalloc(&S->cap_edges, std::max(S->cap_count, 1), "cap edge allocation") &&
             dalloc(&S->cap_rest, std::max(S->cap_count, 1), "cap rest allocation");
        g.blk_cloth = S->pcg_blk;
    }
    if (!ok) return bail(0, "");
    cudaStream_t st = S->stream;
    ok = dupload(S->pos[0], rest4.data(), nV, st, "position upload") && dupload(S->pos[1], rest4.data(), nV, st, "position upload") &&
         dupload(S->prev, rest4.data(), nV, st, "previous position upload") &&
         dupload(S->vel, zero4.data(), nV, st, "velocity upload") && dupload(S->rest, rest4.data(), nV, st, "rest position upload") &&
         dupload(S->inv_mass, S->h_inv.data(), nV, st, "inverse mass upload") &&
         dupload(S->sp_off, sp_off.data(), sp_off.size(), st, "spring CSR upload") &&
         dupload(S->sp_ent, sp_ent.data(), sp_ent.size(), st, "spring CSR upload") &&
         dupload(S->te_off, te_off.data(), te_off.size(), st, "tether CSR upload") &&
         dupload(S->te_ent, te_ent.data(), te_ent.size(), st, "tether CSR upload") &&
         dupload(S->bj_off, bj_off.data(), bj_off.size(), st, "bend CSR upload") &&
         dupload(S->bj_ent, bj_ent.data(), bj_ent.size(), st, "bend CSR upload") &&
         dupload(S->bends, cbends.data(), cbends.size(), st, "bend pair upload") &&
         (S->h_bend_ranges.empty() ||
          dupload(S->bend_ranges, S->h_bend_ranges.data(), S->h_bend_ranges.size(), st, "bend range upload")) &&
         dupload(S->bend_rest, cbend_rest.data(), cbend_rest.size(), st, "bend rest upload") &&
         dupload(S->tris, tris.data(), nT, st, "triangle upload") && dupload(S->edges, springs.data(), nE, st, "edge upload") &&
         dupload(S->edge_rest, spring_rest.data(), nE, st, "edge rest upload") &&
         dupload(S->pin_weight, S->h_pin_weight.data(), nV, st, "pin weight upload") &&
         dupload(S->pin_target, S->h_pin_target.data(), nV, st, "pin target upload") &&
         dupload(S->pin_relax, S->h_pin_relax.data(), nV, st, "pin relaxation upload") &&
         (!S->vt_off || (dupload(S->vt_off, vt_off.data(), vt_off.size(), st, "incident triangle upload") &&
                         dupload(S->vt_tri, vt_tri.data(), vt_tri.size(), st, "incident triangle upload"))) &&
         dupload(S->p_area, p_area.data(), p_area.size(), st, "pressure area upload") &&
         dupload(S->p_rest, p_rest.data(), p_rest.size(), st, "pressure scale upload") &&
         dupload(S->vcloth, vmap.data(), vmap.size(), st, "cloth map upload") &&
         dupload(S->ecloth, emap.data(), emap.size(), st, "cloth map upload") &&
         dupload(S->tcloth, tmap.data(), tmap.size(), st, "cloth map upload") &&
         cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, st), "reset ABI41 diagnostics") &&
         cuda_ok(cudaMemsetAsync(S->max_delta_bits, 0, sizeof(unsigned), st), "reset self max smoothed delta") &&
         (!S->acc || cuda_ok(cudaMemsetAsync(S->acc, 0, sizeof(Acc4) * nV, st), "reset self accumulation")) &&
         (!S->nb_count || cuda_ok(cudaMemsetAsync(S->nb_count, 0, sizeof(int) * nV, st), "reset neighbor table")) &&
         sync_params(S) && cuda_ok(cudaStreamSynchronize(st), "solver upload");
    if (ok && S->pcg_on)
        ok = (S->cap_count == 0 || (dupload(S->cap_edges, cap_edges.data(), S->cap_count, st, "cap edge upload") &&
                                    dupload(S->cap_rest, cap_rest.data(), S->cap_count, st, "cap rest upload"))) &&
             dupload(S->pcg_blk, blk_cloth.data(), blk_cloth.size(), st, "PCG block map upload") &&
             cuda_ok(cudaMemsetAsync(S->pcg.ticket, 0, sizeof(unsigned) * K, st), "reset PCG ticket") &&
             cuda_ok(cudaMemsetAsync(S->pcg.red, 0, sizeof(float) * kRedSlots * K, st), "reset PCG reductions") &&
             cuda_ok(cudaStreamSynchronize(st), "PCG buffer upload");
    if (!ok) return bail(0, "");
    S->diag.finite_flag = 1;
    S->diag.abi41_bending_wing_count = wings;
    S->diag.abi41_bending_texture_ready = wings > 0 ? 1 : 0;
    for (int k = 0; k < K; ++k)
        if (!upload_static(S, k, meshes[k].static_triangles, std::max(configs[k].static_triangle_count, 0))) return bail(k, "");
    return S;
}

// ------------------------------------------------------------ the frame --

namespace {

// Self-collision work of one substep: which cloths run it and which kernel
// variants they need.
struct SelfPlan {
    bool run = false;
    int passes = 0;
    bool vhash = false, thash = false, ehash = false, any_t = false, any_e = false, island = false;
    bool t_order = false, t_plain = false, e_order = false, e_plain = false;  // bucket order needs
    unsigned island_passes = 0;  // passes in which some cloth runs its overlap islands
    SelfVariants sv{};
    long long hits = 0, misses = 0;
};

SelfPlan plan_self(const Solver* S, int s, int substeps) {
    SelfPlan p;
    for (int k = 0; k < S->K; ++k) {
        const Cloth& C = S->cl[k];
        const Params& P = S->hp[k];
        if (!C.self_enabled || !P.active) continue;
        if (!(((s + 1) % C.interval) == 0 || s == substeps - 1)) continue;
        p.run = true;
        p.passes = std::max(p.passes, C.passes);
        p.vhash |= P.vhash != 0;
        p.thash |= P.thash != 0;
        p.ehash |= P.ehash != 0;
        if (P.thash) (C.order_buckets ? p.t_order : p.t_plain) = true;
        if (P.ehash) (C.order_buckets ? p.e_order : p.e_plain) = true;
        if (C.order_buckets) {
            if (P.thash) p.sv.tb_ord.add(P.tbase, P.tbuckets);
            if (P.ehash) p.sv.eb_ord.add(P.ebase, P.ebuckets);
        }
        p.any_t |= P.T > 0;
        p.any_e |= P.E > 0;
        p.sv.fast |= C.fast;
        p.sv.strict |= !C.fast;
        if (!C.fast) (std::min(std::max(P.max_neighbors, 1), kBucketSlots) >= kBucketSlots ? p.sv.strict_wide : p.sv.strict_narrow) = true;
        p.sv.add_cloth(P, C.fast);
        p.sv.hashed_v |= P.vhash != 0;
        p.sv.brute_v |= P.vhash == 0;
        p.sv.hashed_t |= P.thash != 0 && P.T > 0;
        p.sv.brute_t |= P.thash == 0 && P.T > 0;
        p.sv.hashed_e |= P.ehash != 0 && P.E > 0;
        p.sv.brute_e |= P.ehash == 0 && P.E > 0;
        if (C.fast && P.T > 0 && P.thash != 0) {
            p.island = true;
            p.island_passes |= 1u << (std::min(std::max(P.self_passes, 1), 31) - 1);  // islands run in a cloth's final pass
        }
        if (C.fast) {
            p.hits += (long long)P.V * (C.passes > 1 ? C.passes - 1 : 0);
            p.misses += (long long)P.V;
        }
    }
    return p;
}

// Bucket ordering mode of a hash build: 1 every bucket, 0 only buckets past
// the 32 query slots, 2 decided per bucket from its cloth.
int order_mode(bool need, bool plain) { return need ? (plain ? 2 : 1) : 0; }

}  // namespace

// Issue one frame: `substeps` substeps of `iterations` iterations, following
// the reference schedule (abi41.cu:9165-9376).  Per-vertex stages of an
// iteration are fused into one pass; a pass starts at every stretch /
// tether / Jacobi-bend gather and around the work that needs all vertices
// (bends by colour, self collision).
// Kinds of dynamic colliders present: bit 0 unsigned (plain triangles and
// particles), bit 1 signed (indexed meshes, with their particles).
int dynamic_kinds(const Solver* S) {
    int kinds = 0;
    for (int k = 0; k < S->K; ++k) {
        const Params& P = S->hp[k];
        const GlobalScene* G = S->cl[k].gscene;
        const bool shared = P.gd_mode != 0 && G && (G->dyn.h.tri_count > 0 || G->dyn.h.par_count > 0);
        if (shared) kinds |= 1;
        if (!P.dyn) continue;
        // own colliders: signed meshes keep their passes; unsigned ones give
        // way to an attached shared scene (abi41.cu:9239)
        if (S->cl[k].dyn.h.signed_mode)
            kinds |= 2;
        else if (P.gd_mode == 0)
            kinds |= 1;
    }
    return kinds;
}

int buf_index(const Solver* S, const float4* p) { return p == S->pos[0] ? 0 : 1; }

GraphKey frame_key(const Solver* S, int substeps, int iterations) {
    int analytic = 0, sdf = 0, normals = 0;
    for (const Params& P : S->hp) {
        analytic |= (P.use_ground || P.use_wall || P.use_sphere) ? 1 : 0;
        sdf |= P.sdf_ready ? 1 : 0;
        normals |= P.needs_normal ? 1 : 0;
    }
    return GraphKey{substeps, iterations, analytic, sdf, normals, dynamic_kinds(S)};
}

// Whether every cloth fits one block and uses only stages the fused frame
// runs (no self collision, hard stretch or dynamic colliders).
// Fused frame form: 1 one block per cloth (default), 8 an 8-CTA cluster per
// cloth, 2 launched kernels.  On a 32x32 cloth the block form measured 0.174
// ms per frame, the launched kernels 0.19 ms and the cluster 0.227 ms (its
// per-operation exchange and cluster barrier cost more than the seven extra
// SMs save).
int fused_mode(const Solver* S) {
    const int m = S->tune.v[kTuneFusedFrame];
    return m > 0 ? m : 1;
}

bool fused_ok(const Solver* S) {
    if (fused_mode(S) == 2 || S->pcg_on || S->nV == 0) return false;
    for (int k = 0; k < S->K; ++k) {
        const Params& P = S->hp[k];
        if (P.V > 1024 || S->cl[k].self_enabled || P.dyn || P.gd_mode != 0) return false;
    }
    return true;
}

int fused_block(const Solver* S) {
    int m = 32;
    for (const Params& P : S->hp) m = std::max(m, P.V);
    return std::min((m + 31) / 32 * 32, 1024);
}

void enqueue_frame(Solver* S, int substeps, int iterations, FrameStats* st, Profile* prof) {
    const int nV = S->nV;
    const int dyn = dynamic_kinds(S);
    if (!prof && !S->rec) {
        const auto f = S->fused_ops.find(frame_key(S, substeps, iterations));
        if (f != S->fused_ops.end() && f->second.first && fused_ok(S)) {
            View v = S->view();
            v.substeps = substeps;
            v.pass = -1;
            if (fused_mode(S) == 8)
                launch_frame_cluster(v, f->second.first, f->second.second, S->pos[0], S->bend_ranges, S->K, fused_block(S), 8, 128,
                                     S->stream);
            else
                launch_frame_fused(v, f->second.first, f->second.second, S->pos[0], S->pos[1], S->bend_ranges, S->K,
                                   fused_block(S), S->stream);
            st->launches += 1;
            return;
        }
    }
    bool analytic = false, sdf = false, normals = false;
    for (const Params& P : S->hp) {
        analytic |= P.use_ground || P.use_wall || P.use_sphere;
        sdf |= P.sdf_ready != 0;
        normals |= P.needs_normal != 0;
    }
    // cloths with the CG stretch solve skip the spring gather of a pass that
    // other cloths of the batch need (their vertices pass through unchanged)
    const bool pcg = S->pcg_on;
    const bool spring = S->spring_any;
    const bool hard = S->pcg_hard;
    const bool colored_bends = !S->bend_colors.empty();
    View base = S->view();
    base.substeps = substeps;
    if (prof) {
        base.perf = S->perf;
        cudaMemsetAsync(S->perf, 0, sizeof(unsigned long long) * kPerfStripes * kPerfStride, S->stream);
    }
    int cur = 0;
    unsigned pending = 0;
    int pending_last = 0;  // last_it of the iteration that queued `pending`
    int gather = 0;        // 0 none, 1 stretch, 2 tethers, 3 bends without colours
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
        v.last_it = pending_last;
        v.pos_in = S->pos[cur];
        const unsigned gflag = gather == 1 ? kPassSpring : (gather == 2 ? kPassTether : (gather == 3 ? kPassBend : 0u));
        v.pos = gather ? S->pos[cur ^ 1] : S->pos[cur];
        if (S->rec)
            S->rec->push_back(FrameOp{1, gflag | pending, buf_index(S, v.pos_in), buf_index(S, v.pos), v.substep, v.last_it, 0});
        else
            timed(gather == 1 ? kKStretchPass : kKVertexPass, 1, [&] { launch_vertex_pass(v, nV, gflag | pending, S->stream); });
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
        View cv = cur_view();
        cv.edges = S->cap_edges;
        cv.edge_rest = S->cap_rest;
        cv.nE = S->cap_count;
        const int ncol = (int)S->cap_colors.size() - 1;
        timed(kKStretchCaps, 0, [&] {
            for (int p = 0; p < passes; ++p) {
                if (S->cap_jacobi) {
                    pcg_cap_jacobi(cv, S->pcg, nV, kind, S->stream);
                    st->launches += 2;
                }
                for (int k = 0; k < ncol; ++k) {
                    const int n = S->cap_colors[k + 1] - S->cap_colors[k];
                    if (n > 0) {
                        pcg_cap_range(cv, S->cap_colors[k], n, kind, S->stream);
                        st->launches += 1;
                    }
                }
                if (both_ways)
                    for (int k = ncol - 1; k >= 0; --k) {
                        const int n = S->cap_colors[k + 1] - S->cap_colors[k];
                        if (n > 0) {
                            pcg_cap_range(cv, S->cap_colors[k], n, kind, S->stream);
                            st->launches += 1;
                        }
                    }
            }
        });
    };
    auto averaged = [&](bool tiny) {
        View av = cur_view();
        timed(kKStretchCaps, 2, [&] { pcg_averaged_pass(av, S->pcg, nV, tiny, S->stream); });
    };
    for (int s = 0; s < substeps; ++s) {
        base.substep = s;
        const SelfPlan sp = plan_self(S, s, substeps);
        View pv = cur_view();
        if (normals) pv.pos = S->pos[cur ^ 1];  // vertex normals read the snapshot
        if (S->rec)
            S->rec->push_back(FrameOp{0, 0u, buf_index(S, pv.pos_in), buf_index(S, pv.pos), s, 0, 0});
        else
            timed(kKPredict, 1, [&] { launch_predict(pv, nV, S->stream); });
        if (normals) cur ^= 1;
        for (int it = 0; it < iterations; ++it) {
            const bool last_it = it == iterations - 1;
            const bool final_c = (s == substeps - 1) && last_it;
            flush();
            base.last_it = last_it ? 1 : 0;
            if (spring) gather = 1;
            if (pcg && last_it) {
                if (S->rec) S->rec_unsupported = true;
                // CG stretch solve, then (hardness >= 0.95) the averaged
                // polish with normal and tiny caps, and the extreme caps
                // (abi41.cu:9183-9201, 7806-7857, 7974-7995)
                View gv = cur_view();
                timed(kKPcg, 0, [&] { pcg_solve(gv, S->pcg, S->pcg_blocks, S->stream, &st->launches); });
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
            if (final_c && S->nL > 0) {
                flush();
                gather = 2;
            }
            if (final_c && colored_bends) {
                flush();
                View bv = cur_view();
                for (size_t k = 0; k + 1 < S->bend_colors.size(); ++k) {
                    const int start = S->bend_colors[k], n = S->bend_colors[k + 1] - start;
                    if (n > 0 && S->rec)
                        S->rec->push_back(FrameOp{2, 0u, buf_index(S, bv.pos_in), buf_index(S, bv.pos), s, 1, (int)k});
                    else if (n > 0)
                        timed(kKBendColor, 1, [&] { launch_bend_color(bv, start, n, S->stream); });
                }
            }
            if (final_c && S->jacobi_bends) {
                flush();
                gather = 3;
            }
            pending |= kPassPin;
            if (analytic) pending |= kPassAnalytic;
            if (sdf) pending |= kPassSdf;
            pending_last = base.last_it;
            // unsigned dynamic colliders after the static contacts of the
            // last iteration (abi41.cu:9234-9254)
            if (last_it && (dyn & 1)) {
                if (S->rec) S->rec_unsupported = true;
                flush();
                View dv = cur_view();
                timed(kKDynamic, 1, [&] { launch_dynamic_collision(dv, nV, 0, S->stream); });
            }
            const bool self_run = last_it && sp.run;
            if (self_run) {
                if (S->rec) S->rec_unsupported = true;
                flush();
                // Independent self-collision work runs on side streams: the
                // three hash builds, then in each pass the VV, VT and EE
                // queries (and the fast-mode islands).  They only add to the
                // integer accumulators and counters, so the result does not
                // depend on their interleaving.  A profiled frame keeps
                // everything on the solver stream so each kind is timed alone.
                const bool par = prof == nullptr;
                auto lane_stream = [&](int k) { return par ? S->aux[k] : S->stream; };
                auto fork = [&]() {
                    if (!par) return;
                    cudaEventRecord(S->ev_fork, S->stream);
                    for (int k = 0; k < 3; ++k) cudaStreamWaitEvent(S->aux[k], S->ev_fork, 0);
                };
                auto join = [&]() {
                    if (!par) return;
                    for (int k = 0; k < 3; ++k) {
                        cudaEventRecord(S->ev_join[k], S->aux[k]);
                        cudaStreamWaitEvent(S->stream, S->ev_join[k], 0);
                    }
                };
                View sv = cur_view();
                View hv[3] = {sv, sv, sv};
                const size_t trim_seg = (size_t)std::max(std::max(S->nVB, S->nTB), S->nEB);
                for (int k = 0; k < 3; ++k) {
                    hv[k].scan_tmp = S->scan_tmp + (size_t)k * S->scan_seg;
                    hv[k].trim_list = S->trim_list + (size_t)k * trim_seg;
                    hv[k].trim_count = S->trim_count + k;
                }
                fork();
                if (sp.vhash)
                    timed(kKVertexHash, 6, [&] {
                        cudaMemsetAsync(S->vb_count, 0, sizeof(int) * S->nVB, lane_stream(0));
                        self_build_vertex_hash(hv[0], sp.sv, S->nVB, lane_stream(0));
                    });
                if (sp.thash)
                    // zeroing, count, three scan kernels, scatter, trim (+ ordering)
                    timed(kKTriangleHash, 7 + (order_mode(sp.t_order, sp.t_plain) != 0), [&] {
                        reset_triangle_hash(S, lane_stream(1));
                        self_build_triangle_hash(hv[1], sp.sv, S->nTB, order_mode(sp.t_order, sp.t_plain), lane_stream(1));
                    });
                if (sp.ehash)
                    // zeroing, insertion, four overflow kernels, trim (+ ordering)
                    timed(kKEdgeHash, 7 + (order_mode(sp.e_order, sp.e_plain) != 0), [&] {
                        reset_edge_hash(S, lane_stream(2));
                        self_build_edge_hash(hv[2], sp.sv, S->nEB, order_mode(sp.e_order, sp.e_plain), lane_stream(2));
                    });
                // No join here: each branch's first pass needs only its own
                // hash (neighbour table + VV: the vertex hash, VT + islands:
                // the triangle hash, EE: the edge hash), so the queries of the
                // finished branches overlap the longer builds.
                if (sp.sv.fast) {
                    timed(kKNeighbors, 1, [&] { self_neighbors(sv, 1, sp.sv, lane_stream(0)); });
                    st->cache_hits += sp.hits;
                    st->cache_misses += sp.misses;
                }
                for (int pass = 0; pass < sp.passes; ++pass) {
                    View pv2 = sv;
                    pv2.pass = pass;
                    if (pass > 0) fork();
                    if (sp.sv.strict) timed(kKNeighbors, 1, [&] { self_neighbors(pv2, 2, sp.sv, lane_stream(0)); });
                    timed(kKVertexVertex, 1, [&] { self_vv(pv2, sp.sv, lane_stream(0)); });
                    if (sp.any_t) timed(kKVertexTriangle, 1, [&] { self_vt(pv2, sp.sv, lane_stream(1)); });
                    if (sp.island && ((sp.island_passes >> pass) & 1u))
                        timed(kKIsland, 1, [&] { self_island(pv2, sp.sv, lane_stream(1)); });
                    if (sp.any_e) timed(kKEdgeEdge, 1, [&] { self_ee(pv2, sp.sv, lane_stream(2)); });
                    join();
                    timed(kKSelfApply, 1, [&] { self_apply(pv2, sp.sv, S->stream); });
                }
            }
            // signed dynamic colliders after self collision (abi41.cu:9340-9345)
            if (last_it && (dyn & 2)) {
                flush();
                View dv = cur_view();
                timed(kKDynamic, 1, [&] { launch_dynamic_collision(dv, nV, 1, S->stream); });
            }
            // final ratio caps after the contacts (abi41.cu:9346-9350, 7997-8027)
            if (pcg && final_c && hard) {
                flush();
                caps(0, 2, true);
                caps(2, 3, false);
                caps(1, 3, false);
            }
            // inside-only signed passes at the final constraints (abi41.cu:9351-9360)
            if (final_c && (dyn & 2)) {
                flush();
                View dv = cur_view();
                for (int pass = 0; pass < kSignedInsidePasses; ++pass)
                    timed(kKDynamic, 1, [&] { launch_dynamic_collision(dv, nV, 2, S->stream); });
            }
            // Final pin polish whenever a contact stage ran: analytic
            // colliders, the SDF, or any last iteration (the dynamic
            // collider stage counts as running on every last iteration);
            // the pass applies it per cloth.
            if (analytic || sdf || last_it) pending |= kPassPinPolish;
        }
        pending |= kPassVelocity;
        flush();
    }
    if (cur != 0 && S->rec)
        S->rec->push_back(FrameOp{3, 0u, 1, 0, 0, 0, 0});
    else if (cur != 0)
        timed(kKCopy, 1, [&] { launch_copy_pos(S->pos[0], S->pos[1], nV, S->stream); });
}

namespace {

// The frame graph for (substeps, iterations) and the current collider kinds,
// captured and instantiated on first use.
// Record the frame's operations for the fused form (once per schedule key);
// outside any stream capture, since it allocates and uploads.
bool prepare_fused(Solver* S, int substeps, int iterations) {
    if (!fused_ok(S)) return true;
    const GraphKey key = frame_key(S, substeps, iterations);
    if (S->fused_ops.count(key)) return true;
    std::vector<FrameOp> ops;
    FrameStats dummy;
    S->rec = &ops;
    S->rec_unsupported = false;
    enqueue_frame(S, substeps, iterations, &dummy, nullptr);
    S->rec = nullptr;
    if (S->rec_unsupported || ops.empty()) {
        S->fused_ops[key] = {nullptr, 0};
        return true;
    }
    AllocAccount account(&S->device_bytes);
    FrameOp* dev = nullptr;
    if (!dalloc(&dev, ops.size(), "fused frame allocation") || !dupload(dev, ops.data(), ops.size(), S->stream, "fused frame upload") ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "fused frame upload"))
        return false;
    S->fused_ops[key] = {dev, (int)ops.size()};
    return true;
}

GraphEntry* ensure_graph(Solver* S, int substeps, int iterations) {
    int analytic = 0, sdf = 0, normals = 0;
    for (const Params& P : S->hp) {
        analytic |= (P.use_ground || P.use_wall || P.use_sphere) ? 1 : 0;
        sdf |= P.sdf_ready ? 1 : 0;
        normals |= P.needs_normal ? 1 : 0;
    }
    const GraphKey key{substeps, iterations, analytic, sdf, normals, dynamic_kinds(S)};
    auto it = S->graphs.find(key);
    if (it == S->graphs.end()) {
        if (!prepare_fused(S, substeps, iterations)) return nullptr;
        GraphEntry g;
        FrameStats cst;
        if (!cuda_ok(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal), "begin frame capture"))
            return nullptr;
        enqueue_frame(S, substeps, iterations, &cst);
        cudaGraph_t graph = nullptr;
        if (!cuda_ok(cudaStreamEndCapture(S->stream, &graph), "end frame capture")) return nullptr;
        const cudaError_t err = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (!cuda_ok(err, "instantiate frame graph")) return nullptr;
        g.launches = cst.launches;
        g.cache_hits = cst.cache_hits;
        g.cache_misses = cst.cache_misses;
        g.pcg_solves = cst.pcg_solves;
        it = S->graphs.emplace(key, g).first;
    }
    return &it->second;
}

}  // namespace

bool prepare_graph(Solver* S, int substeps, int iterations) {
    if (!S->use_graphs) return true;
    return ensure_graph(S, substeps, iterations) != nullptr;
}

bool run_frame(Solver* S, int substeps, int iterations, FrameStats* st) {
    if (!S->use_graphs) {
        if (!prepare_fused(S, substeps, iterations)) return false;
        enqueue_frame(S, substeps, iterations, st);
        return cuda_ok(cudaGetLastError(), "launch GB300 XPBD frame");
    }
    GraphEntry* g = ensure_graph(S, substeps, iterations);
    if (!g) return false;
    st->launches += g->launches;
    st->cache_hits += g->cache_hits;
    st->cache_misses += g->cache_misses;
    st->pcg_solves += g->pcg_solves;
    return cuda_ok(cudaGraphLaunch(g->exec, S->stream), "launch frame graph");
}

bool fetch_counts(Solver* S, const FrameStats& st) {
    unsigned long long c[kCntSlots];
    unsigned mbits = 0;
    if (!cuda_ok(cudaMemcpyAsync(c, S->counts, sizeof(c), cudaMemcpyDeviceToHost, S->stream), "fetch ABI41 diagnostics") ||
        !cuda_ok(cudaMemcpyAsync(&mbits, S->max_delta_bits, sizeof(unsigned), cudaMemcpyDeviceToHost, S->stream),
                 "fetch self max smoothed delta") ||
        !cuda_ok(cudaStreamSynchronize(S->stream), "fetch diagnostics"))
        return false;
    int wings = 0;
    for (const Cloth& C : S->cl) wings += C.wing_count;
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
    d.candidate_count = (long long)(c[kCntDynParCandidates] + c[kCntDynTriCandidates] + c[kCntSelfCandidates] +
                                   c[kCntStaticSdfContacts]);
    // dynamic colliders (abi41.cu:8078-8117): the hashes are built at upload,
    // so the per-build figures (large triangles, largest bucket) come from
    // the host copies
    d.dynamic_particle_candidate_count = (long long)c[kCntDynParCandidates];
    d.dynamic_particle_contacts = (long long)c[kCntDynParContacts];
    d.dynamic_particle_overflow = 0;
    d.dynamic_triangle_candidate_count = (long long)c[kCntDynTriCandidates];
    d.dynamic_triangle_bucket_overflow = (long long)c[kCntDynTriOverflow];
    d.dynamic_triangle_aabb_reject_count = (long long)c[kCntDynTriAabbRejects];
    long long large = 0, occupancy = 0;
    for (const Cloth& C : S->cl) {
        if (!C.dyn.h.tri_hashed || C.dyn.h.tri_count <= 0) continue;
        large += C.dyn.large_count;
        occupancy = std::max(occupancy, (long long)C.dyn.max_occupancy);
    }
    d.dynamic_triangle_large_primitive_count = large;
    d.dynamic_triangle_max_bucket_occupancy = occupancy;
    d.fast_triangle_pair_candidates = d.dynamic_triangle_candidate_count;
    d.fast_triangle_pair_contacts = (long long)c[kCntTrianglePairs];
    d.fast_triangle_pair_skipped_rest = d.dynamic_triangle_aabb_reject_count;
    d.abi41_lra_tack_count = (long long)c[kCntLraTacks];
    d.abi41_bending_wing_count = c[kCntBendingWings] > 0 ? (long long)c[kCntBendingWings] : (long long)wings;
    d.abi41_bending_texture_ready = wings > 0 ? 1 : 0;
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
    d.self_filter_cache_hits = st.cache_hits;      // counted for fast-mode cloths only
    d.self_filter_cache_misses = st.cache_misses;
    d.self_cluster_count = (long long)c[kCntClusterCount];
    d.self_cluster_owned_contacts = (long long)c[kCntClusterOwnedContacts];
    if (S->pcg_on) {
        // residual diagnostics from the scalar slots (abi41.cu:7586-7624);
        // in a batch the residuals are those of the stacked systems (square
        // root of the summed r.z of the solving cloths) and every cloth's
        // guarded status counts
        std::vector<float> red((size_t)S->K * kRedSlots);
        unsigned long long guard = 0;
        unsigned pbits = 0;
        if (!cuda_ok(cudaMemcpyAsync(red.data(), S->pcg.red, sizeof(float) * red.size(), cudaMemcpyDeviceToHost, S->stream),
                     "fetch PCG reductions") ||
            !cuda_ok(cudaMemcpyAsync(&guard, S->pcg.guard, sizeof(guard), cudaMemcpyDeviceToHost, S->stream), "fetch PCG guard count") ||
            !cuda_ok(cudaMemcpyAsync(&pbits, S->pcg.max_delta_bits, 4, cudaMemcpyDeviceToHost, S->stream), "fetch PCG max delta") ||
            !cuda_ok(cudaStreamSynchronize(S->stream), "fetch PCG diagnostics"))
            return false;
        d.abi41_pcg_csr_nnz = S->pcg_nnz;
        d.abi41_pcg_texture_ready = 1;
        d.abi41_pcg_iterations = S->pcg_iterations;
        bool have_initial = false, have_final = false;
        float initial_sum = 0.0f, final_sum = 0.0f;
        for (int k = 0; k < S->K; ++k) {
            if (!S->hp[k].pcg_on) continue;
            const float* R = red.data() + (size_t)k * kRedSlots;
            float initial = R[kRedInitialRZ];
            if ((!std::isfinite(initial) || initial <= 0.0f) && std::isfinite(R[kRedRZ]) && R[kRedRZ] >= 0.0f) initial = R[kRedRZ];
            const bool init_ok = std::isfinite(initial) && initial >= 0.0f;
            if (init_ok) {
                initial_sum += initial;
                have_initial = true;
            }
            const float status = R[kRedStatus];
            const float final_rz = status == 2.0f ? R[kRedRZ] : R[kRedRZNext];
            if ((status == 0.0f || status == 2.0f) && std::isfinite(final_rz) && final_rz >= 0.0f) {
                final_sum += final_rz;
                have_final = true;
            } else {
                if (init_ok) final_sum += initial;  // a cloth without a final value reports its initial one
                if (status != 0.0f && status != 2.0f) d.abi41_pcg_guarded += 1;
            }
        }
        if (have_initial) d.abi41_pcg_initial_residual = std::sqrt(std::max(initial_sum, 0.0f));
        if (have_initial || have_final) d.abi41_pcg_final_residual = std::sqrt(std::max(final_sum, 0.0f));
        d.abi41_pcg_guarded += (long long)guard;
        std::memcpy(&d.abi41_pcg_max_delta, &pbits, 4);
    }
    return true;
}

// Per-step preparation: sub-step length of each cloth, pin relaxation for
// this iteration count, parameter upload and counter resets.
bool prepare_step(Solver* S, int substeps, int iterations) {
    for (int k = 0; k < S->K; ++k) {
        const float sub_dt = S->cl[k].cfg.dt / (float)substeps;
        if (S->hp[k].sub_dt != sub_dt) {
            S->hp[k].sub_dt = sub_dt;
            S->params_dirty = true;
        }
    }
    if (!cuda_ok(cudaMemsetAsync(S->counts, 0, sizeof(unsigned long long) * kCntSlots, S->stream), "reset ABI41 diagnostics") ||
        !cuda_ok(cudaMemsetAsync(S->max_delta_bits, 0, sizeof(unsigned), S->stream), "reset self max smoothed delta") ||
        !upload_pin_relax(S, iterations) || !sync_params(S))
        return false;
    if (S->pcg_on &&
        (!cuda_ok(cudaMemsetAsync(S->pcg.guard, 0, sizeof(unsigned long long), S->stream), "reset PCG guard count") ||
         !cuda_ok(cudaMemsetAsync(S->pcg.max_delta_bits, 0, sizeof(unsigned), S->stream), "reset PCG max delta") ||
         !cuda_ok(cudaMemsetAsync(S->pcg.red, 0, sizeof(float) * kRedSlots * S->K, S->stream), "reset PCG reductions")))
        return false;
    return true;
}

bool step(Solver* S, int substeps, int iterations, int fetch_diagnostics, int force_sync) {
    const auto t0 = std::chrono::high_resolution_clock::now();
    int ff = 0, uff = 0;
    for (const Cloth& C : S->cl) {
        ff += C.force_field_count;
        uff += C.unsupported_force_field_count;
    }
    S->diag = SsblXpbdDiagnostics{};
    S->diag.finite_flag = 1;
    S->diag.force_field_count = ff;
    S->diag.unsupported_force_field_count = uff;
    for (int k = 0; k < S->K; ++k) {
        const Cloth& C = S->cl[k];
        const GlobalScene* G = S->hp[k].gd_mode != 0 ? C.gscene : nullptr;
        if (G) {
            // a cloth on the shared scene reports the scene (abi41.cu:9109-9122)
            S->diag.dynamic_triangle_count += G->dyn.h.tri_count;
            S->diag.dynamic_particle_count += G->dyn.h.par_count;
            S->diag.global_dynamic_triangle_count += G->dyn.h.tri_count;
            S->diag.global_dynamic_particle_count += G->dyn.h.par_count;
            S->diag.global_dynamic_hash_overflow += G->hash_overflow;
            S->diag.global_dynamic_scene_upload_ms += G->upload_ms;
        } else {
            S->diag.dynamic_triangle_count += C.dyn.h.tri_count;
            S->diag.dynamic_particle_count += C.dyn.h.par_count;
        }
    }
    sdf_diagnostics(S);
    substeps = std::max(substeps, 1);
    iterations = std::max(iterations, 1);
    if (!prepare_step(S, substeps, iterations)) return false;
    FrameStats st;
    if (!run_frame(S, substeps, iterations, &st)) return false;
    S->last_launches = st.launches;
    S->pcg_iterations = st.pcg_solves * 8;
    if (force_sync || fetch_diagnostics) {
        const auto ts = std::chrono::high_resolution_clock::now();
        if (!cuda_ok(cudaStreamSynchronize(S->stream), "ABI41 solver step")) return false;
        S->diag.sync_ms = (float)ms_since(ts);
    }
    if (fetch_diagnostics && !fetch_counts(S, st)) return false;
    S->diag.step_ms = (float)ms_since(t0);
    S->diag.constraints_ms = S->diag.step_ms;
    S->diag.resolved_contacts = S->diag.abi41_soft_contact_count + S->diag.abi41_exact_impulse_contact_count +
                                S->diag.abi41_edge_edge_contact_count + S->diag.static_sdf_contact_count;
    return true;
}

bool profile_frame(Solver* S, int substeps, int iterations, float* kernel_ms, long long* kernel_launches, int kinds) {
    if (!S || !kernel_ms || !kernel_launches || kinds < kKinds) return fail("invalid profile request");
    substeps = std::max(substeps, 1);
    iterations = std::max(iterations, 1);
    if (!prepare_step(S, substeps, iterations)) return false;
    for (int k = 0; k < kinds; ++k) {
        kernel_ms[k] = 0.0f;
        kernel_launches[k] = 0;
    }
    FrameStats st;
    Profile prof;
    enqueue_frame(S, substeps, iterations, &st, &prof);
    const bool ok = cuda_ok(cudaGetLastError(), "profile frame") && cuda_ok(cudaStreamSynchronize(S->stream), "profile frame");
    for (auto& m : prof.marks) {
        float ms = 0.0f;
        if (ok) cudaEventElapsedTime(&ms, m.second.first, m.second.second);
        kernel_ms[m.first] += ms;
        kernel_launches[m.first] += 1;
        cudaEventDestroy(m.second.first);
        cudaEventDestroy(m.second.second);
    }
    return ok;
}

namespace {

bool tune_value_ok(int slot, int v) {
    if (v == 0) return true;
    if (slot == kTuneGroupLanes) return v == 4 || v == 8 || v == 16;
    if (slot == kTunePrimLanes || slot == kTuneTriLanes) return v == 1 || v == 2 || v == 4 || v == 8 || v == 16;
    if (slot == kTuneNeighborLanes) return v == 1 || v == 2 || v == 4 || v == 8 || v == 16 || v == 32;
    if (slot == kTuneFastEeForm) return v == 8 || v == 32;
    if (slot == kTuneFusedFrame) return v == 1 || v == 2 || v == 8;
    return v >= 32 && v <= kMaxBlock && v % 32 == 0;
}

}  // namespace

int effective_tune(const Solver* S, int slot) { return slot == kTuneFusedFrame ? fused_mode(S) : tune_of(S->tune, slot); }

bool set_launch_config(Solver* S, const int* values, int n) {
    if (!S || (!values && n > 0) || n < 0 || n > kTuneSlots) return fail("invalid launch configuration");
    LaunchTune t = S->tune;
    for (int k = 0; k < n; ++k) {
        if (!tune_value_ok(k, values[k])) return fail("invalid launch configuration value for slot " + std::to_string(k));
        t.v[k] = (short)values[k];
    }
    if (std::memcmp(&t, &S->tune, sizeof(t)) != 0) {
        if (!cuda_ok(cudaStreamSynchronize(S->stream), "launch configuration")) return false;
        S->tune = t;
        S->drop_graphs();
    }
    return true;
}

// Coordinate descent over the slots, one sweep, each candidate timed as the
// fastest of `rounds` profiled frames from the same saved state.
bool autotune(Solver* S, int substeps, int iterations, int rounds, float* ms_out) {
    if (!S) return fail("invalid solver handle");
    rounds = std::max(rounds, 1);
    const size_t n = (size_t)std::max(S->nV, 1);
    float4 *spos = nullptr, *sprev = nullptr, *svel = nullptr;
    {
        AllocAccount none(nullptr);
        if (!dalloc(&spos, n, "autotune state") || !dalloc(&sprev, n, "autotune state") || !dalloc(&svel, n, "autotune state")) {
            cudaFree(spos);
            cudaFree(sprev);
            return false;
        }
    }
    auto copy = [&](float4* dst, const float4* src) {
        return cuda_ok(cudaMemcpyAsync(dst, src, sizeof(float4) * (size_t)S->nV, cudaMemcpyDeviceToDevice, S->stream), "autotune state");
    };
    bool ok = cuda_ok(cudaStreamSynchronize(S->stream), "autotune") && copy(spos, S->pos[0]) && copy(sprev, S->prev) &&
              copy(svel, S->vel);
    std::vector<float> kms(kKinds);
    std::vector<long long> kn(kKinds);
    auto measure = [&](float* out) {
        float best = 0.0f;
        for (int r = 0; r < rounds && ok; ++r) {
            ok = copy(S->pos[0], spos) && copy(S->prev, sprev) && copy(S->vel, svel) &&
                 profile_frame(S, substeps, iterations, kms.data(), kn.data(), kKinds);
            float total = 0.0f;
            for (float x : kms) total += x;
            if (r == 0 || total < best) best = total;
        }
        *out = best;
        return ok;
    };
    int dyn = 0, narrow = 0, fast_any = 0;
    for (int k = 0; k < S->K; ++k) {
        fast_any |= (S->cl[k].self_enabled && S->cl[k].fast) ? 1 : 0;
        dyn |= S->hp[k].dyn ? 1 : 0;
        narrow |= (S->cl[k].self_enabled && !S->cl[k].fast && std::min(std::max(S->hp[k].max_neighbors, 1), kBucketSlots) < kBucketSlots) ? 1 : 0;
    }
    const std::vector<std::vector<short>> cand = {
        {64, 128, 256},   // vertex passes
        {64, 128, 256},   // hash count / scatter
        {1, 2, 4, 8, 16}, // lanes per edge of the edge hash
        {128, 256},       // warp kernels
        {64, 128, 256},   // thread-per-item queries
        {4, 8, 16},       // group lanes
        {128, 256},       // group block
        {64, 128, 256},   // dynamic colliders
        {8, 32},          // fast EE: groups of 8 lanes or flattened warps
        {1, 2, 8},        // small cloths: fused frame (block or cluster per cloth) or launched kernels
        {1, 2, 4, 16},    // lanes per triangle of the triangle hash
        {1, 2, 4, 8},     // lanes per vertex of the neighbour table
    };
    const LaunchTune start = S->tune;
    LaunchTune best = start;
    for (int k = 0; k < kTuneSlots; ++k) best.v[k] = (short)tune_of(start, k);
    S->tune = best;
    S->drop_graphs();
    float best_ms = 0.0f, default_ms = 0.0f;
    if (ok) ok = measure(&default_ms);
    best_ms = default_ms;
    for (int slot = 0; slot < kTuneSlots && ok; ++slot) {
        if (slot == kTuneDynamicBlock && !dyn) continue;
        if ((slot == kTuneGroupLanes || slot == kTuneGroupBlock) && !narrow && !S->self_any) continue;
        if (slot == kTuneFastEeForm && !fast_any) continue;
        // profiled frames are never fused, so the fused form is not a
        // candidate here (it replaces a frame's launches by one)
        if (slot == kTuneFusedFrame) continue;
        for (short c : cand[slot]) {
            if (c == best.v[slot]) continue;
            LaunchTune t = best;
            t.v[slot] = c;
            S->tune = t;
            float ms = 0.0f;
            if (!measure(&ms)) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    }
    S->tune = ok ? best : start;
    S->drop_graphs();
    const bool restored = copy(S->pos[0], spos) && copy(S->prev, sprev) && copy(S->vel, svel) &&
                          cuda_ok(cudaStreamSynchronize(S->stream), "autotune restore");
    cudaFree(spos);
    cudaFree(sprev);
    cudaFree(svel);
    S->diag = SsblXpbdDiagnostics{};
    S->diag.finite_flag = 1;
    if (ms_out) {
        ms_out[0] = best_ms;
        ms_out[1] = default_ms;
    }
    return ok && restored;
}

}  // namespace host

// Lets entry points defined in other translation units report through
// ssbl_last_error().
void set_last_error(const std::string& msg) { host::g_error = msg; }

}  // namespace xg
