// Differentiable rollout of the contact-free XPBD step: per-constraint stretch
// and bend compliances in, final positions out, and a hand-written adjoint
// that returns dL/d(compliance) for a loss gradient dL/d(final positions).
//
// Forward: the solver's own schedule and arithmetic for a cloth without
// contacts (prediction, stretch gathers with the pin stage, bends by colour
// once per frame, velocity update; native/src/ssbl_xpbd_cuda_abi41.cu:
// 9165-9376), with each constraint's compliance read from an array.  With
// equal compliances it produces the solver's bits (shared arithmetic in
// xpbd_constraint.cuh).
//
// Checkpointing: the state (x, prev, v) at the start of every frame is kept.
// The backward pass walks the frames in reverse; for each it re-runs the
// frame forward from its checkpoint, recording the state before every
// operation (and the positions before every bend colour), then propagates
// the adjoint through the operations in reverse.  Branch decisions (caps,
// velocity clamp, sign tests) are those of the forward; the adjoint is the
// derivative of the active branch.
//
// Adjoint of one stretch use (edge e = (i, j), delta = xj - xi, len = |delta|,
// W = wi + wj, a = k / dt^2): corr = s delta with s = -0.18 (len - rest) /
// ((W + a) len); d corr / d delta = s I + q delta delta^T, q = -0.18 rest /
// ((W + a) len^3); d corr / d a = -s delta / (W + a).  A capped correction
// corr = m sign(s) delta / len has d corr / d delta = m sign(s) (I - n n^T) /
// len and no dependence on a.  Bends have the same form with 0.10.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "xpbd_constraint.cuh"
#include "xpbd_host.cuh"

using namespace xg;
using namespace xg::host;

#define XG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

constexpr int kDiffThreads = 128;
inline int dblocks(int n) { return (n + kDiffThreads - 1) / kDiffThreads; }

enum DiffPass : unsigned { kDGather = 1u, kDPin = 2u, kDVelocity = 4u };

struct DState {
    float4* p;     // xyz, .w = effective inverse mass
    float4* prev;
    float4* vel;
};

struct DView {
    int V, E, B;
    float dt, damping, thickness;
    float gravity[3];
    const float4* rest;       // .w = effective inverse mass
    const int* off;           // vertex -> stretch CSR
    const int2* ent;          // {other | side << 31, edge}
    const float* edge_rest;
    const int2* bends;        // caller order
    const float* bend_rest;
    const int* pinned;        // 1 = hard pin
    const float4* target;
    const float* kst;         // per-edge stretch compliance
    const float* kbd;         // per-bend compliance
};

__device__ __forceinline__ float4 row(const float4* a, int i) { return a[i]; }

// ------------------------------------------------------------- forward --

__global__ void k_d_predict(DView d, DState in, DState out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    const float4 p4 = row(in.p, i);
    const float w = p4.w;
    F3 p, vel;
    const F3 prev = f3(p4);
    if (!(w > 0.0f)) {
        vel = F3{0.0f, 0.0f, 0.0f};
        p = f3(d.rest[i]);
    } else {
        const F3 accel = F3{d.gravity[0], d.gravity[1], d.gravity[2]} + F3{0.0f, 0.0f, 0.0f};
        vel = f3(row(in.vel, i)) + accel * d.dt;
        vel = vel * d.damping;
        p = f3(p4) + vel * d.dt;
    }
    F3 pv = prev;
    if (d.pinned[i]) {
        p = f3(d.target[i]);
        pv = p;
        vel = F3{0.0f, 0.0f, 0.0f};
    }
    out.p[i] = f4(p, w);
    out.prev[i] = f4(pv, 0.0f);
    out.vel[i] = f4(vel, 0.0f);
}

__global__ void k_d_pass(DView d, unsigned flags, DState in, DState out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    const float4 p4 = row(in.p, i);
    F3 p = f3(p4), prev = f3(row(in.prev, i)), vel = f3(row(in.vel, i));
    if (flags & kDGather) {
        F3 dp = p, dprev = prev;
        for (int k = d.off[i]; k < d.off[i + 1]; ++k) {
            const int2 e = d.ent[k];
            const bool self_is_j = (e.x & kSideBit) != 0;
            const float4 q4 = row(in.p, e.x & 0x7fffffff);
            const float4 pi = self_is_j ? q4 : p4, pj = self_is_j ? p4 : q4;
            F3 corr;
            float c;
            bool clamped;
            if (!stretch_correction(pi, pj, d.edge_rest[e.y], d.kst[e.y], d.dt, &corr, &c, &clamped)) continue;
            const float wself = self_is_j ? pj.w : pi.w;
            if (wself > 0.0f) {
                const F3 dd = self_is_j ? corr * pj.w : corr * (-pi.w);
                dp = dp + dd;
                if (c > 0.0f) dprev = dprev + dd * 0.08f;
            }
        }
        p = dp;
        prev = dprev;
    }
    if ((flags & kDPin) && d.pinned[i]) {
        p = f3(d.target[i]);
        prev = p;
        vel = F3{0.0f, 0.0f, 0.0f};
    }
    if (flags & kDVelocity) vel = velocity_update(p, prev, vel, p4.w, d.thickness, d.dt);
    out.p[i] = f4(p, p4.w);
    out.prev[i] = f4(prev, 0.0f);
    out.vel[i] = f4(vel, 0.0f);
}

// One bend colour, in place (no two bends of a colour share a vertex).
__global__ void k_d_bend(DView d, const int* order, int start, int count, DState s) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int b = order[start + k];
    if (b < 0 || b >= d.B) return;
    const int2 pr = d.bends[b];
    const int i = pr.x, j = pr.y;
    if (i < 0 || j < 0 || i >= d.V || j >= d.V || i == j) return;
    const float4 pi4 = s.p[i], pj4 = s.p[j];
    F3 corr;
    bool guard, clamped;
    if (!bend_correction_k(pi4, pj4, d.bend_rest[b], d.kbd[b], d.thickness, d.dt, &corr, &guard, &clamped)) return;
    if (pi4.w > 0.0f) {
        const F3 dd = corr * (-pi4.w);
        s.p[i] = f4(f3(pi4) + dd, pi4.w);
        s.prev[i] = f4(f3(s.prev[i]) + dd * 0.06f, 0.0f);
    }
    if (pj4.w > 0.0f) {
        const F3 dd = corr * pj4.w;
        s.p[j] = f4(f3(pj4) + dd, pj4.w);
        s.prev[j] = f4(f3(s.prev[j]) + dd * 0.06f, 0.0f);
    }
}

// ------------------------------------------------------------- adjoint --

// J^T g for corr = s delta (+ cap): returns d(corr . g)/d delta and, through
// `dk`, d(corr . g)/d compliance.
__device__ __forceinline__ F3 corr_adjoint(F3 delta, float len, float rest, float weight, float alpha, float gain, bool clamped,
                                           float max_corr, float dt, float compliance, F3 g, float* dk) {
    const float inv = 1.0f / (weight + alpha);
    const float s = -gain * (len - rest) * inv / len;
    if (clamped) {
        const F3 n = delta * (1.0f / len);
        const float sg = s < 0.0f ? -1.0f : 1.0f;
        *dk = 0.0f;
        return (g - n * dot3(n, g)) * (max_corr * sg / len);
    }
    const float q = -gain * rest * inv / (len * len * len);
    const float dg = dot3(delta, g);
    // d corr / d a = -s delta / (W + a); d a / d k = 1 / dt^2 for k > 0
    *dk = compliance > 0.0f ? (-s * inv * dg) / fmaxf(dt * dt, kEps) : 0.0f;
    return g * s + delta * (q * dg);
}

// Velocity and pin stages of a pass, backwards: adjoint at the pass output
// (ap, aq = prev, av) to the adjoint after the gather (mid arrays).
__global__ void k_d_stage_back(DView d, unsigned flags, DState in, DState out, const float4* ap, const float4* aq,
                               const float4* av, float4* mp, float4* mq, float4* mv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    F3 gp = f3(ap[i]), gq = f3(aq[i]), gv = f3(av[i]);
    const float w = in.p[i].w;
    if (flags & kDVelocity) {
        F3 np{0.0f, 0.0f, 0.0f}, nq{0.0f, 0.0f, 0.0f}, nv{0.0f, 0.0f, 0.0f};
        // velocity stage inputs: x and prev after the pin stage (= pass
        // output), velocity after the pin stage
        const bool pinned = (flags & kDPin) && d.pinned[i];
        if (w > 0.0f) {
            const float sdt = fmaxf(d.dt, kEps);
            const F3 p = f3(out.p[i]), prev = f3(out.prev[i]);
            const F3 base = pinned ? F3{0.0f, 0.0f, 0.0f} : f3(in.vel[i]);
            const F3 measured = (p - prev) * (1.0f / sdt);
            const F3 proj = measured - base;
            const float pdb = dot3(proj, base);
            const float scale = (isfinite(pdb) && pdb > 0.0f) ? 0.9f : 1.0f;
            const float max_delta = fmaxf(2.0e-4f, fmaxf(d.thickness, 0.0f) * 0.35f);
            const float max_speed = max_delta / sdt;
            const F3 fb = proj * scale;
            const float fspeed = len3(fb);
            F3 gproj;
            if (scale < 1.0f && isfinite(fspeed) && fspeed > max_speed && fspeed > kEps) {
                const float plen = len3(proj);
                const F3 n = proj * (1.0f / plen);
                gproj = (gv - n * dot3(n, gv)) * (max_speed / plen);
            } else {
                gproj = gv * scale;
            }
            np = gproj * (1.0f / sdt);
            nq = gproj * (-1.0f / sdt);
            nv = gv - gproj;
        }
        gp = gp + np;
        gq = gq + nq;
        gv = nv;
    }
    if ((flags & kDPin) && d.pinned[i]) {
        gp = F3{0.0f, 0.0f, 0.0f};
        gq = F3{0.0f, 0.0f, 0.0f};
        gv = F3{0.0f, 0.0f, 0.0f};
    }
    mp[i] = f4(gp, 0.0f);
    mq[i] = f4(gq, 0.0f);
    mv[i] = f4(gv, 0.0f);
}

// Stretch gather, backwards: adjoint after the gather (mid) to the adjoint of
// the pass input; each edge's compliance gradient is added by its first
// endpoint (one writer per edge, so the sum is deterministic).
__global__ void k_d_gather_back(DView d, DState in, const float4* mp, const float4* mq, const float4* mv, float4* ap,
                                float4* aq, float4* av, float* gk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    const float4 p4 = in.p[i];
    F3 acc = f3(mp[i]);
    for (int k = d.off[i]; k < d.off[i + 1]; ++k) {
        const int2 e = d.ent[k];
        const bool self_is_j = (e.x & kSideBit) != 0;
        const int o = e.x & 0x7fffffff;
        const float4 q4 = in.p[o];
        const float4 pi = self_is_j ? q4 : p4, pj = self_is_j ? p4 : q4;
        const int ii = self_is_j ? o : i, jj = self_is_j ? i : o;
        const float wi = pi.w, wj = pj.w, weight = wi + wj;
        if (weight <= 0.0f) continue;
        const float rest = d.edge_rest[e.y], kc = d.kst[e.y];
        const F3 delta = f3(pj) - f3(pi);
        const float len = sqrtf(fmaxf(dot3(delta, delta), kEps));
        const float c = len - rest;
        const float alpha = fmaxf(kc, 0.0f) / fmaxf(d.dt * d.dt, kEps);
        F3 corr;
        float cc;
        bool clamped;
        stretch_correction(pi, pj, rest, kc, d.dt, &corr, &cc, &clamped);
        const float kp = c > 0.0f ? 0.08f : 0.0f;
        const F3 gi = (f3(mp[ii]) + f3(mq[ii]) * kp) * wi, gj = (f3(mp[jj]) + f3(mq[jj]) * kp) * wj;
        const F3 g = gj - gi;
        const float max_corr = fmaxf(0.0025f, fminf(fmaxf(rest, 0.0f) * 0.10f, 0.025f));
        float dk;
        const F3 adelta = corr_adjoint(delta, len, rest, weight, alpha, 0.18f, clamped, max_corr, d.dt, kc, g, &dk);
        acc = self_is_j ? acc + adelta : acc - adelta;
        if (!self_is_j) gk[e.y] += dk;
    }
    ap[i] = f4(acc, 0.0f);
    aq[i] = mq[i];
    av[i] = mv[i];
}

// One bend colour backwards, in place on the adjoint (positions before the
// colour in `before`).
__global__ void k_d_bend_back(DView d, const int* order, int start, int count, const float4* before, float4* ap,
                              const float4* aq, float* gk) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int b = order[start + k];
    if (b < 0 || b >= d.B) return;
    const int2 pr = d.bends[b];
    const int i = pr.x, j = pr.y;
    if (i < 0 || j < 0 || i >= d.V || j >= d.V || i == j) return;
    const float4 pi4 = before[i], pj4 = before[j];
    const float rest = d.bend_rest[b], kc = d.kbd[b];
    F3 corr;
    bool guard, clamped;
    if (!bend_correction_k(pi4, pj4, rest, kc, d.thickness, d.dt, &corr, &guard, &clamped)) return;
    const float wi = pi4.w, wj = pj4.w, weight = wi + wj;
    const F3 delta = f3(pj4) - f3(pi4);
    const float len_sq = len_sq_xyz(delta);
    const float inv_len = 1.0f / sqrtf(len_sq);
    const float len = len_sq * inv_len;
    const float alpha = fmaxf(kc, 0.0f) / fmaxf(d.dt * d.dt, kEps);
    const F3 gi = wi > 0.0f ? (f3(ap[i]) + f3(aq[i]) * 0.06f) * wi : F3{0.0f, 0.0f, 0.0f};
    const F3 gj = wj > 0.0f ? (f3(ap[j]) + f3(aq[j]) * 0.06f) * wj : F3{0.0f, 0.0f, 0.0f};
    const F3 g = gj - gi;
    const float max_corr = fmaxf(2.5e-4f, fminf(fmaxf(rest, d.thickness) * 0.08f, 0.020f));
    float dk;
    const F3 adelta = corr_adjoint(delta, len, rest, weight, alpha, 0.10f, clamped, max_corr, d.dt, kc, g, &dk);
    ap[j] = f4(f3(ap[j]) + adelta, 0.0f);
    ap[i] = f4(f3(ap[i]) - adelta, 0.0f);
    gk[b] += dk;
}

// Prediction (and the pin stage after it), backwards.
__global__ void k_d_predict_back(DView d, DState in, float4* ap, float4* aq, float4* av) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.V) return;
    F3 gp = f3(ap[i]), gq = f3(aq[i]), gv = f3(av[i]);
    if (d.pinned[i]) gp = gq = gv = F3{0.0f, 0.0f, 0.0f};
    const float w = in.p[i].w;
    F3 np, nv;
    if (w > 0.0f) {
        // vel' = (v + g dt) c; x' = x + vel' dt; prev' = x
        const F3 gvel = gv + gp * d.dt;
        nv = gvel * d.damping;
        np = gp + gq;
    } else {
        nv = F3{0.0f, 0.0f, 0.0f};
        np = gq;
    }
    ap[i] = f4(np, 0.0f);
    aq[i] = f4(F3{0.0f, 0.0f, 0.0f}, 0.0f);
    av[i] = f4(nv, 0.0f);
}

__global__ void k_d_copy_state(DState src, DState dst, int V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    dst.p[i] = src.p[i];
    dst.prev[i] = src.prev[i];
    dst.vel[i] = src.vel[i];
}

__global__ void k_d_pack(const float4* p, float* out, int V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 q = p[i];
    out[3 * i] = q.x;
    out[3 * i + 1] = q.y;
    out[3 * i + 2] = q.z;
}

__global__ void k_d_unpack_grad(const float* g, float4* ap, float4* aq, float4* av, int V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    ap[i] = make_float4(g[3 * i], g[3 * i + 1], g[3 * i + 2], 0.0f);
    aq[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    av[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ---------------------------------------------------------------- host --

struct Op {
    int kind;        // 0 predict, 1 pass, 2 bends
    unsigned flags;  // pass stages
};

struct DiffSolver {
    SsblXpbdConfig cfg{};
    int V = 0, E = 0, B = 0;
    cudaStream_t stream = nullptr;
    float4* rest = nullptr;
    int* off = nullptr;
    int2* ent = nullptr;
    float* edge_rest = nullptr;
    int2* bends = nullptr;
    float* bend_rest = nullptr;
    int* order = nullptr;           // bend ids by colour
    std::vector<int> colors;        // colour offsets into `order`
    int* pinned = nullptr;
    float4* target = nullptr;
    std::vector<int> h_pinned;
    std::vector<float4> h_target;
    float* kst = nullptr;           // compliance of the last rollout (device copies)
    float* kbd = nullptr;
    float4* init = nullptr;         // initial state (3 rows of V)
    float4* ck = nullptr;           // checkpoints: (frames + 1) x 3 x V
    int ck_frames = 0;
    float4* tape = nullptr;         // states before each op of a frame, + colour snapshots
    size_t tape_states = 0;
    float4* adj = nullptr;          // 6 x V adjoint rows (output + mid)
    int frames = 0, substeps = 0, iterations = 0;
    std::vector<Op> ops;

    DView view(float dt) const {
        DView d{};
        d.V = V;
        d.E = E;
        d.B = B;
        d.dt = dt;
        d.damping = cfg.damping;
        d.thickness = cfg.cloth_thickness;
        for (int a = 0; a < 3; ++a) d.gravity[a] = cfg.gravity[a];
        d.rest = rest;
        d.off = off;
        d.ent = ent;
        d.edge_rest = edge_rest;
        d.bends = bends;
        d.bend_rest = bend_rest;
        d.pinned = pinned;
        d.target = target;
        d.kst = kst;
        d.kbd = kbd;
        return d;
    }
    DState state_at(float4* base) const { return DState{base, base + V, base + 2 * (size_t)V}; }
};

void free_diff(DiffSolver* D) {
    if (!D) return;
    if (D->stream) cudaStreamSynchronize(D->stream);
    void* ptrs[] = {D->rest, D->off, D->ent, D->edge_rest, D->bends, D->bend_rest, D->order, D->pinned,
                    D->target, D->kst, D->kbd, D->init, D->ck, D->tape, D->adj};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (D->stream) cudaStreamDestroy(D->stream);
    delete D;
}

// The frame's operations in the solver's order for a contact-free cloth with
// coloured bends (the schedule of enqueue_frame without contact stages).
std::vector<Op> frame_ops(int substeps, int iterations, bool bends) {
    std::vector<Op> ops;
    for (int s = 0; s < substeps; ++s) {
        const bool final_sub = s == substeps - 1;
        ops.push_back(Op{0, 0u});
        for (int it = 1; it < iterations; ++it) ops.push_back(Op{1, kDGather | kDPin});
        if (final_sub && bends) {
            ops.push_back(Op{1, kDGather});
            ops.push_back(Op{2, 0u});
            ops.push_back(Op{1, kDPin | kDVelocity});
        } else {
            ops.push_back(Op{1, kDGather | kDPin | kDVelocity});
        }
    }
    return ops;
}

bool ensure_buffers(DiffSolver* D, int frames) {
    const size_t V = (size_t)D->V;
    const size_t states = D->ops.size() + 1;
    const size_t ncol = D->colors.empty() ? 0 : D->colors.size() - 1;
    const size_t need = states * 3 * V + ncol * V;
    if (need > D->tape_states) {
        if (D->tape) cudaFree(D->tape);
        D->tape = nullptr;
        D->tape_states = 0;
        if (!dalloc(&D->tape, need, "rollout tape allocation")) return false;
        D->tape_states = need;
    }
    if (frames > D->ck_frames) {
        if (D->ck) cudaFree(D->ck);
        D->ck = nullptr;
        D->ck_frames = 0;
        if (!dalloc(&D->ck, (size_t)(frames + 1) * 3 * V, "checkpoint allocation")) return false;
        D->ck_frames = frames;
    }
    return true;
}

// One frame forward from `in` to `out`; with `record`, the state before every
// op goes to the tape (op k at state k) and the positions before every bend
// colour after the states.
void run_frame_ops(DiffSolver* D, DState in, DState out, bool record) {
    const float dt = D->cfg.dt / (float)D->substeps;
    const DView d = D->view(dt);
    const int V = D->V;
    const size_t ops = D->ops.size();
    float4* colour_base = D->tape + (ops + 1) * 3 * (size_t)V;
    // ping-pong between two tape slots when not recording
    DState cur = in;
    for (size_t k = 0; k < ops; ++k) {
        DState next = record ? D->state_at(D->tape + (k + 1) * 3 * (size_t)V) : (k + 1 == ops ? out : D->state_at(D->tape + ((k & 1) ? 0 : 3 * (size_t)V)));
        if (record && k == 0) k_d_copy_state<<<dblocks(V), kDiffThreads, 0, D->stream>>>(cur, D->state_at(D->tape), V);
        const Op& op = D->ops[k];
        if (op.kind == 0) {
            k_d_predict<<<dblocks(V), kDiffThreads, 0, D->stream>>>(d, cur, next);
        } else if (op.kind == 1) {
            k_d_pass<<<dblocks(V), kDiffThreads, 0, D->stream>>>(d, op.flags, cur, next);
        } else {
            k_d_copy_state<<<dblocks(V), kDiffThreads, 0, D->stream>>>(cur, next, V);
            for (size_t c = 0; c + 1 < D->colors.size(); ++c) {
                const int start = D->colors[c], n = D->colors[c + 1] - start;
                if (record)
                    cudaMemcpyAsync(colour_base + c * (size_t)V, next.p, sizeof(float4) * V, cudaMemcpyDeviceToDevice, D->stream);
                if (n > 0) k_d_bend<<<dblocks(n), kDiffThreads, 0, D->stream>>>(d, D->order, start, n, next);
            }
        }
        cur = next;
    }
    if (record) k_d_copy_state<<<dblocks(V), kDiffThreads, 0, D->stream>>>(cur, out, V);
}

// Backward through one recorded frame: the adjoint in adj rows 0-2 at the
// frame end becomes the adjoint at the frame start.
void back_frame_ops(DiffSolver* D, float* gst, float* gbd) {
    const float dt = D->cfg.dt / (float)D->substeps;
    const DView d = D->view(dt);
    const int V = D->V;
    const size_t ops = D->ops.size();
    float4* ap = D->adj;
    float4* aq = D->adj + V;
    float4* av = D->adj + 2 * (size_t)V;
    float4* mp = D->adj + 3 * (size_t)V;
    float4* mq = D->adj + 4 * (size_t)V;
    float4* mv = D->adj + 5 * (size_t)V;
    const float4* colour_base = D->tape + (ops + 1) * 3 * (size_t)V;
    for (size_t k = ops; k-- > 0;) {
        const DState in = D->state_at(D->tape + k * 3 * (size_t)V);
        const DState out = D->state_at(D->tape + (k + 1) * 3 * (size_t)V);
        const Op& op = D->ops[k];
        if (op.kind == 0) {
            k_d_predict_back<<<dblocks(V), kDiffThreads, 0, D->stream>>>(d, in, ap, aq, av);
        } else if (op.kind == 1) {
            k_d_stage_back<<<dblocks(V), kDiffThreads, 0, D->stream>>>(d, op.flags, in, out, ap, aq, av, mp, mq, mv);
            if (op.flags & kDGather) {
                k_d_gather_back<<<dblocks(V), kDiffThreads, 0, D->stream>>>(d, in, mp, mq, mv, ap, aq, av, gst);
            } else {
                cudaMemcpyAsync(ap, mp, sizeof(float4) * 3 * (size_t)V, cudaMemcpyDeviceToDevice, D->stream);
            }
        } else {
            for (size_t c = D->colors.size() - 1; c-- > 0;) {
                const int start = D->colors[c], n = D->colors[c + 1] - start;
                if (n > 0)
                    k_d_bend_back<<<dblocks(n), kDiffThreads, 0, D->stream>>>(d, D->order, start, n, colour_base + c * (size_t)V,
                                                                             ap, aq, gbd);
            }
        }
    }
}

DiffSolver* as_diff(void* h) { return reinterpret_cast<DiffSolver*>(h); }

}  // namespace

// ------------------------------------------------------------ entry points

XG_EXPORT void* xpbd_gb300_diff_create(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh) {
    g_error.clear();
    if (!config || !mesh || !mesh->positions || !mesh->inv_mass || config->vertex_count <= 0 || config->edge_count < 0 ||
        config->bend_count < 0 || !std::isfinite(config->dt) || !(config->dt > 0.0f)) {
        fail("invalid differentiable rollout create request");
        return nullptr;
    }
    const SsblXpbdConfig& c = *config;
    if (c.use_ground || c.use_wall || c.use_sphere || c.static_triangle_count > 0 || c.self_collision)
        return fail("the differentiable rollout covers the contact-free step: colliders and self collision must be off"),
               nullptr;
    if (c.lra_count > 0 || c.stretch_optimization_enabled || (c.use_volume_pressure && c.pressure_strength > 0.0f))
        return fail("the differentiable rollout covers stretch and bend constraints only"), nullptr;
    if (c.bend_count > 0 && (c.bend_color_count <= 0 || !mesh->bend_color_offsets || !mesh->bends || !mesh->bend_rest_lengths))
        return fail("the differentiable rollout needs coloured bends"), nullptr;
    if (c.edge_count > 0 && (!mesh->edges || !mesh->edge_rest_lengths))
        return fail("the differentiable rollout needs edge pairs and rest lengths"), nullptr;
    DiffSolver* D = new DiffSolver();
    D->cfg = c;
    D->cfg.damping = std::isfinite(c.damping) ? std::max(0.0f, std::min(c.damping, 1.0f)) : 1.0f;
    const int V = c.vertex_count, E = c.edge_count, B = c.bend_count;
    D->V = V;
    D->E = E;
    D->B = B;
    std::vector<float4> rest4(V), zero(V, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < V; ++i) {
        const float w = mesh->inv_mass[i] > 0.0f ? mesh->inv_mass[i] : 0.0f;
        rest4[i] = make_float4(mesh->positions[3 * i], mesh->positions[3 * i + 1], mesh->positions[3 * i + 2], w);
    }
    // vertex -> edge CSR in edge order, entries {other | side, edge}
    std::vector<int> off(V + 1, 0);
    std::vector<int2> edges(E);
    for (int e = 0; e < E; ++e) {
        edges[e] = make_int2(std::max(mesh->edges[2 * e], 0), std::max(mesh->edges[2 * e + 1], 0));
        const int2 p = edges[e];
        if (p.x >= V || p.y >= V || p.x == p.y) continue;
        off[p.x + 1]++;
        off[p.y + 1]++;
    }
    for (int i = 0; i < V; ++i) off[i + 1] += off[i];
    std::vector<int2> ent(off[V]);
    std::vector<int> cur(off.begin(), off.end() - 1);
    for (int e = 0; e < E; ++e) {
        const int2 p = edges[e];
        if (p.x >= V || p.y >= V || p.x == p.y) continue;
        ent[cur[p.x]++] = make_int2(p.y, e);
        ent[cur[p.y]++] = make_int2(p.x | kSideBit, e);
    }
    std::vector<int2> bends(B);
    for (int b = 0; b < B; ++b) bends[b] = make_int2(mesh->bends[2 * b], mesh->bends[2 * b + 1]);
    std::vector<int> order;
    D->colors.assign(1, 0);
    for (int k = 0; k < c.bend_color_count; ++k) {
        const int b0 = std::max(mesh->bend_color_offsets[k], 0), b1 = std::min(mesh->bend_color_offsets[k + 1], B);
        for (int b = b0; b < b1; ++b) order.push_back(b);
        D->colors.push_back((int)order.size());
    }
    if (order.empty()) D->colors.clear();
    D->h_pinned.assign(V, 0);
    D->h_target.assign(V, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    std::vector<float> kst(E, std::max(c.stretch_compliance, 0.0f)), kbd(B, std::max(c.bend_compliance, 0.0f));
    bool ok = cuda_ok(cudaStreamCreateWithFlags(&D->stream, cudaStreamNonBlocking), "create rollout stream") &&
              dalloc(&D->rest, V, "rollout allocation") && dalloc(&D->off, V + 1, "rollout allocation") &&
              dalloc(&D->ent, ent.size(), "rollout allocation") && dalloc(&D->edge_rest, E, "rollout allocation") &&
              dalloc(&D->bends, B, "rollout allocation") && dalloc(&D->bend_rest, B, "rollout allocation") &&
              dalloc(&D->order, order.size(), "rollout allocation") && dalloc(&D->pinned, V, "rollout allocation") &&
              dalloc(&D->target, V, "rollout allocation") && dalloc(&D->kst, E, "rollout allocation") &&
              dalloc(&D->kbd, B, "rollout allocation") && dalloc(&D->init, 3 * (size_t)V, "rollout allocation") &&
              dalloc(&D->adj, 6 * (size_t)V, "rollout allocation");
    if (ok)
        ok = dupload(D->rest, rest4.data(), V, D->stream, "rollout upload") &&
             dupload(D->off, off.data(), off.size(), D->stream, "rollout upload") &&
             dupload(D->ent, ent.data(), ent.size(), D->stream, "rollout upload") &&
             dupload(D->edge_rest, mesh->edge_rest_lengths, E, D->stream, "rollout upload") &&
             dupload(D->bends, bends.data(), B, D->stream, "rollout upload") &&
             dupload(D->bend_rest, mesh->bend_rest_lengths, B, D->stream, "rollout upload") &&
             dupload(D->order, order.data(), order.size(), D->stream, "rollout upload") &&
             dupload(D->pinned, D->h_pinned.data(), V, D->stream, "rollout upload") &&
             dupload(D->target, D->h_target.data(), V, D->stream, "rollout upload") &&
             dupload(D->kst, kst.data(), E, D->stream, "rollout upload") &&
             dupload(D->kbd, kbd.data(), B, D->stream, "rollout upload") &&
             dupload(D->init, rest4.data(), V, D->stream, "rollout upload") &&
             dupload(D->init + V, rest4.data(), V, D->stream, "rollout upload") &&
             dupload(D->init + 2 * (size_t)V, zero.data(), V, D->stream, "rollout upload") &&
             cuda_ok(cudaStreamSynchronize(D->stream), "rollout upload");
    if (!ok) {
        free_diff(D);
        return nullptr;
    }
    return D;
}

XG_EXPORT int xpbd_gb300_diff_destroy(void* handle) {
    free_diff(as_diff(handle));
    return 1;
}

// Hard pins (weight >= 0.75): the vertex is held at its target.  Softer pins
// are not differentiated and are refused.
XG_EXPORT int xpbd_gb300_diff_update_pin_targets(void* handle, const int* indices, const float* positions,
                                                 const float* weights, int count) {
    g_error.clear();
    DiffSolver* D = as_diff(handle);
    if (!D || count < 0 || (count > 0 && (!indices || !positions))) return fail("invalid pin update") ? 1 : 0;
    std::fill(D->h_pinned.begin(), D->h_pinned.end(), 0);
    for (int k = 0; k < count; ++k) {
        const int i = indices[k];
        if (i < 0 || i >= D->V) continue;
        const float w = weights ? weights[k] : 1.0f;
        if (!std::isfinite(w) || w < 0.05f) {
            D->h_pinned[i] = 0;
            continue;
        }
        if (w < 0.75f) return fail("the differentiable rollout supports hard pins only (weight >= 0.75)") ? 1 : 0;
        D->h_pinned[i] = 1;
        D->h_target[i] = make_float4(positions[3 * k], positions[3 * k + 1], positions[3 * k + 2], 0.0f);
    }
    return (dupload(D->pinned, D->h_pinned.data(), D->V, D->stream, "pin upload") &&
            dupload(D->target, D->h_target.data(), D->V, D->stream, "pin upload") &&
            cuda_ok(cudaStreamSynchronize(D->stream), "pin upload"))
               ? 1
               : 0;
}

// Roll out `frames` frames from the rest state with the given per-edge and
// per-bend compliances (device arrays of E and B floats; null keeps the
// config values) and write the final positions (device array of 3V floats).
// Every frame's starting state is kept for xpbd_gb300_diff_backward.
XG_EXPORT int xpbd_gb300_diff_rollout(void* handle, const float* stretch_compliance, const float* bend_compliance, int frames,
                                      int substeps, int iterations, float* final_positions) {
    g_error.clear();
    DiffSolver* D = as_diff(handle);
    if (!D || frames < 1 || !final_positions) return fail("invalid rollout request") ? 1 : 0;
    D->frames = frames;
    D->substeps = std::max(substeps, 1);
    D->iterations = std::max(iterations, 1);
    D->ops = frame_ops(D->substeps, D->iterations, !D->colors.empty());
    if (!ensure_buffers(D, frames)) return 0;
    const int V = D->V;
    if ((stretch_compliance && D->E > 0 &&
         !cuda_ok(cudaMemcpyAsync(D->kst, stretch_compliance, sizeof(float) * D->E, cudaMemcpyDeviceToDevice, D->stream),
                  "copy stretch compliance")) ||
        (bend_compliance && D->B > 0 &&
         !cuda_ok(cudaMemcpyAsync(D->kbd, bend_compliance, sizeof(float) * D->B, cudaMemcpyDeviceToDevice, D->stream),
                  "copy bend compliance")))
        return 0;
    // checkpoint 0 = initial state with the pins applied by the first predict
    cudaMemcpyAsync(D->ck, D->init, sizeof(float4) * 3 * (size_t)V, cudaMemcpyDeviceToDevice, D->stream);
    for (int f = 0; f < frames; ++f)
        run_frame_ops(D, D->state_at(D->ck + (size_t)f * 3 * V), D->state_at(D->ck + (size_t)(f + 1) * 3 * V), false);
    k_d_pack<<<dblocks(V), kDiffThreads, 0, D->stream>>>(D->ck + (size_t)frames * 3 * V, final_positions, V);
    return (cuda_ok(cudaGetLastError(), "rollout") && cuda_ok(cudaStreamSynchronize(D->stream), "rollout")) ? 1 : 0;
}

// Gradient of a loss with dL/d(final positions) = grad_positions (device, 3V
// floats) with respect to the compliances of the last rollout: writes
// grad_stretch (E floats) and grad_bend (B floats), device arrays.
XG_EXPORT int xpbd_gb300_diff_backward(void* handle, const float* grad_positions, float* grad_stretch, float* grad_bend) {
    g_error.clear();
    DiffSolver* D = as_diff(handle);
    if (!D || D->frames < 1 || !grad_positions || (D->E > 0 && !grad_stretch) || (D->B > 0 && !grad_bend))
        return fail("invalid backward request (run a rollout first)") ? 1 : 0;
    const int V = D->V;
    if ((D->E > 0 && !cuda_ok(cudaMemsetAsync(grad_stretch, 0, sizeof(float) * D->E, D->stream), "clear gradient")) ||
        (D->B > 0 && !cuda_ok(cudaMemsetAsync(grad_bend, 0, sizeof(float) * D->B, D->stream), "clear gradient")))
        return 0;
    k_d_unpack_grad<<<dblocks(V), kDiffThreads, 0, D->stream>>>(grad_positions, D->adj, D->adj + V, D->adj + 2 * (size_t)V, V);
    for (int f = D->frames - 1; f >= 0; --f) {
        // re-run frame f from its checkpoint, recording the tape
        DState start = D->state_at(D->ck + (size_t)f * 3 * V);
        DState end = D->state_at(D->tape + D->ops.size() * 3 * (size_t)V);
        run_frame_ops(D, start, end, true);
        back_frame_ops(D, grad_stretch, grad_bend);
    }
    return (cuda_ok(cudaGetLastError(), "rollout backward") && cuda_ok(cudaStreamSynchronize(D->stream), "rollout backward"))
               ? 1
               : 0;
}

// Copy the state at the start of frame `frame` of the last rollout (frame =
// frames: its final state): positions, previous positions and velocities as
// 3 x V float4 rows into `out_rows` (device array of 12 V floats).
XG_EXPORT int xpbd_gb300_diff_checkpoint(void* handle, int frame, float* out_rows) {
    g_error.clear();
    DiffSolver* D = as_diff(handle);
    if (!D || D->frames < 1 || frame < 0 || frame > D->frames || !out_rows)
        return fail("invalid checkpoint request (run a rollout first; frame in [0, frames])") ? 1 : 0;
    const size_t n = 3 * (size_t)D->V;
    return (cuda_ok(cudaMemcpyAsync(out_rows, D->ck + (size_t)frame * n, sizeof(float4) * n, cudaMemcpyDeviceToDevice,
                                    D->stream),
                    "copy checkpoint") &&
            cuda_ok(cudaStreamSynchronize(D->stream), "copy checkpoint"))
               ? 1
               : 0;
}

XG_EXPORT void* xpbd_gb300_diff_stream(void* handle) {
    DiffSolver* D = as_diff(handle);
    return D ? reinterpret_cast<void*>(D->stream) : nullptr;
}
