// Hard-stretch optimisation: the block-Jacobi preconditioned CG stretch solve
// and the ratio caps / averaged polish around it (reference
// native/src/ssbl_xpbd_cuda_abi41.cu:1982-2708, 3032-3464, 7626-8027).
//
// System assembly and every per-vertex sum are gathers over the vertex ->
// edge CSR in edge order (the reference scatters with float atomics).  The CG
// dot products are reduced deterministically: a shuffle-down tree inside each
// 32-vertex warp, partials stored per warp, and the last block to finish
// (atomic ticket, no waiting) sums the partials in a fixed order -- lane l
// adds partials l, l+32, ... then a shuffle-down tree.  The device-side
// alpha / beta / status logic is the reference's (abi41.cu:3320-3464).
//
// In a batch every cloth that enables the optimisation solves its own system:
// the solve grid is the concatenation of the grids one-cloth solvers of
// those cloths would launch (a block belongs to one cloth), each cloth has
// its own partials segment, ticket and scalar slots, so its reductions, its
// alpha / beta and its status follow exactly the one-cloth sequence.
#include "xpbd_solver.cuh"

namespace xg {

namespace {

constexpr float kStatusOk = 0.0f, kStatusBadResidual = 1.0f, kStatusZeroResidual = 2.0f, kStatusBadDad = 3.0f,
                kStatusBadAlpha = 4.0f;

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

struct Sym {
    float m11, m12, m13, m22, m23, m33;
};

__device__ __forceinline__ Sym sym_load(const float4* a, int i) {
    const float4 u = a[2 * i], w = a[2 * i + 1];
    return Sym{u.x, u.y, u.z, u.w, w.x, w.y};
}
__device__ __forceinline__ void sym_store(float4* a, int i, Sym m) {
    a[2 * i] = make_float4(m.m11, m.m12, m.m13, m.m22);
    a[2 * i + 1] = make_float4(m.m23, m.m33, 0.0f, 0.0f);
}
// m * v + acc with the reference's fused chains (abi41.cu:1125-1131).
__device__ __forceinline__ F3 sym_madd(Sym m, F3 v, F3 acc) {
    return F3{fmaf(m.m13, v.z, fmaf(m.m12, v.y, fmaf(m.m11, v.x, acc.x))),
              fmaf(m.m23, v.z, fmaf(m.m22, v.y, fmaf(m.m12, v.x, acc.y))),
              fmaf(m.m33, v.z, fmaf(m.m23, v.y, fmaf(m.m13, v.x, acc.z)))};
}
__device__ __forceinline__ Sym sym_outer(F3 n, float s) {
    return Sym{n.x * n.x * s, n.x * n.y * s, n.x * n.z * s, n.y * n.y * s, n.y * n.z * s, n.z * n.z * s};
}
__device__ __forceinline__ Sym sym_add(Sym a, Sym b) {
    return Sym{a.m11 + b.m11, a.m12 + b.m12, a.m13 + b.m13, a.m22 + b.m22, a.m23 + b.m23, a.m33 + b.m33};
}
// Inverse of a symmetric 3x3 block, diagonal fallback when singular
// (abi41.cu:1158-1189).
__device__ Sym sym_inverse_or_diag(Sym m, unsigned long long* guard) {
    const float a = m.m11, b = m.m12, c = m.m13, d = m.m22, e = m.m23, f = m.m33;
    const float df_ee = fmaf(d, f, -e * e);
    const float bf_ce = fmaf(b, f, -c * e);
    const float be_cd = fmaf(b, e, -c * d);
    const float det = fmaf(c, be_cd, fmaf(-b, bf_ce, a * df_ee));
    if (isfinite(det) && fabsf(det) > 1.0e-12f) {
        const float inv = 1.0f / det;
        return Sym{df_ee * inv,
                   fmaf(c, e, -b * f) * inv,
                   be_cd * inv,
                   fmaf(a, f, -c * c) * inv,
                   fmaf(b, c, -a * e) * inv,
                   fmaf(a, d, -b * b) * inv};
    }
    if (guard) atomicAdd(guard, 1ull);
    return Sym{1.0f / fmaxf(fabsf(a), 1.0e-4f), 0.0f, 0.0f, 1.0f / fmaxf(fabsf(d), 1.0e-4f), 0.0f,
               1.0f / fmaxf(fabsf(f), 1.0e-4f)};
}

// Per-edge projection bound (abi41.cu:1070-1089).
__device__ float projection_limit(const Params& P, float rest) {
    const float base = fmaxf(1.0e-5f, fminf(fmaxf(rest, P.thickness) * 0.5f, 0.25f));
    if (P.stretch_strength < 0.95f || !isfinite(P.thickness) || P.thickness <= kEps) return base;
    const float hard = fmaxf(1.0e-5f, fminf(fmaxf(rest * 0.18f, P.thickness * 0.06f), 0.0035f));
    return fminf(base, hard);
}
// Per-iteration position write-back bound (abi41.cu:1091-1104).
__device__ float writeback_limit(const Params& P) {
    if (P.stretch_strength < 0.95f || !isfinite(P.thickness) || P.thickness <= kEps) return 0.25f;
    return fmaxf(2.5e-4f, fminf(P.thickness * 0.035f, 9.0e-4f));
}

// ---------------------------------------------------- fixed-order sums --
__device__ __forceinline__ float warp_tree(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// The vertex of this thread in the solve grid: the block's cloth, its local
// vertex index and its global one.
struct PcgItem {
    int cloth, local, i;
    bool valid;
};
__device__ __forceinline__ PcgItem pcg_item(const View& v, const PcgView& g) {
    const int c = __ldg(&g.blk_cloth[blockIdx.x]);
    const Params& P = v.P[c];
    const int local = (blockIdx.x - P.pcg_block0) * blockDim.x + threadIdx.x;
    return PcgItem{c, local, P.vstart + local, local < P.V};
}

// Store this warp's tree partial; the last block of the cloth to finish
// returns true in every thread of its first warp together with the cloth's
// total in `*total`.
__device__ bool reduce_partials(const PcgView& g, const Params& P, int cloth, float v, float* total) {
    __shared__ bool last;
    const float w = warp_tree(v);
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int gw = blockIdx.x * wpb + (threadIdx.x >> 5);
    if (lane == 0) g.partials[gw] = w;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned ticket = atomicAdd(&g.ticket[cloth], 1u);
        last = ticket == (unsigned)(P.pcg_nblocks - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x >= 32) return false;
    __threadfence();
    const int nw = P.pcg_nblocks * wpb;
    const volatile float* part = g.partials + (long long)P.pcg_block0 * wpb;
    float s = 0.0f;
    for (int k = lane; k < nw; k += 32) s += part[k];
    s = warp_tree(s);
    *total = __shfl_sync(0xffffffffu, s, 0);
    if (lane == 0) g.ticket[cloth] = 0u;
    return true;
}

__device__ __forceinline__ float4 z4() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }

// ------------------------------------------------------- system build --
// Assembly gathered per vertex (abi41.cu:3085-3186) fused with the
// preconditioner / initial residual (abi41.cu:3188-3226) and the iteration
// set-up (abi41.cu:3071-3083).
__global__ void __launch_bounds__(kThreads) k_pcg_build(View v, PcgView g) {
    const PcgItem it = pcg_item(v, g);
    const Params& P = v.P[it.cloth];
    const int i = it.i;
    float rz = 0.0f;
    if (it.valid) {
        const float4 p4 = v.pos[i];
        const float wi_self = p4.w;
        Sym diag{1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f};
        F3 rhs{0.0f, 0.0f, 0.0f};
        const float strength = clamp01f(P.stretch_strength * 2.5f);
        const int begin = v.sp_off[i], end = v.sp_off[i + 1];
        for (int k = begin; k < end; ++k) {
            const int2 e = __ldg(&v.sp_ent[k]);
            const bool self_is_j = (e.x & kSideBit) != 0;
            const float4 q4 = v.pos[e.x & 0x7fffffff];
            const float4 pi = self_is_j ? q4 : p4, pj = self_is_j ? p4 : q4;
            const float rest = __int_as_float(e.y);
            float4 off = z4();
            const float wi = pi.w, wj = pj.w, weight = wi + wj;
            const bool ai = wi > 0.0f, aj = wj > 0.0f;
            bool ok = isfinite(weight) && weight > 0.0f && isfinite(rest) && rest > kEps && finite3(f3(pi)) && finite3(f3(pj));
            F3 normal{0.0f, 0.0f, 0.0f};
            float projected = 0.0f;
            if (ok) {
                const F3 delta = f3(pj) - f3(pi);
                const float len_sq = dot3(delta, delta);
                ok = isfinite(len_sq) && len_sq > kEps;
                if (ok) {
                    const float len = sqrtf(len_sq);
                    const float err = len - rest;
                    ok = isfinite(err) && fabsf(err) > 1.0e-6f && strength > 0.0f;
                    if (ok) {
                        const float lim = projection_limit(P, rest);
                        projected = fmaxf(-lim, fminf(err * strength, lim));
                        ok = isfinite(projected) && fabsf(projected) > 1.0e-7f;
                        normal = delta * (1.0f / len);
                    }
                }
            }
            if (ok) {
                const F3 desired = normal * (projected / weight);
                const float stiff = fmaxf(strength, 1.0e-3f);
                const bool mine = self_is_j ? aj : ai;
                if (mine) {
                    rhs = rhs + (self_is_j ? desired * (-wj) : desired * wi);
                    diag = sym_add(diag, sym_outer(normal, stiff));
                }
                if (ai && aj) off = make_float4(normal.x, normal.y, normal.z, stiff);
            }
            g.offdiag[k] = off;
        }
        sym_store(g.diag, i, diag);
        if (!(wi_self > 0.0f)) {
            g.r[i] = z4();
            g.z[i] = z4();
            g.d[i] = z4();
            sym_store(g.pinv, i, Sym{1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f});
        } else {
            const Sym inv = sym_inverse_or_diag(diag, g.guard);
            const F3 z = sym_madd(inv, rhs, F3{0.0f, 0.0f, 0.0f});
            sym_store(g.pinv, i, inv);
            g.r[i] = f4(rhs, 0.0f);
            g.z[i] = f4(z, 0.0f);
            g.d[i] = f4(z, 0.0f);
            rz = dot3(rhs, z);
        }
    }
    float total;
    if (reduce_partials(g, P, it.cloth, rz, &total) && (threadIdx.x & 31) == 0) {
        float* R = g.red + it.cloth * kRedSlots;
        R[kRedRZ] = total;
        R[kRedInitialRZ] = total;
        R[kRedIterations] = 0.0f;
        R[kRedDAD] = 0.0f;
        R[kRedRZNext] = 0.0f;
        R[kRedStatus] = kStatusOk;
    }
}

// q = A d, partial d.q (abi41.cu:3228-3267); the last block publishes dAd.
__global__ void __launch_bounds__(kThreads) k_pcg_ad(View v, PcgView g) {
    const PcgItem it = pcg_item(v, g);
    const Params& P = v.P[it.cloth];
    const int i = it.i;
    float* R = g.red + it.cloth * kRedSlots;
    const bool status_ok = R[kRedStatus] == kStatusOk;
    float dq = 0.0f;
    if (status_ok && it.valid) {
        if (!(v.pos[i].w > 0.0f)) {
            g.q[i] = z4();
        } else {
            const F3 di = f3(g.d[i]);
            F3 q = sym_madd(sym_load(g.diag, i), di, F3{0.0f, 0.0f, 0.0f});
            const int begin = v.sp_off[i], end = v.sp_off[i + 1];
            for (int k = begin; k < end; ++k) {
                const float4 o = g.offdiag[k];
                const int col = __ldg(&v.sp_ent[k]).x & 0x7fffffff;
                // inactive entries hold a zero block (+0 entries, like the
                // reference's cleared texels)
                Sym nb{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                if (o.w != 0.0f) {
                    const Sym b = sym_outer(F3{o.x, o.y, o.z}, o.w);
                    nb = Sym{-b.m11, -b.m12, -b.m13, -b.m22, -b.m23, -b.m33};
                }
                q = sym_madd(nb, f3(g.d[col]), q);
            }
            g.q[i] = f4(q, 0.0f);
            dq = dot3(di, q);
        }
    }
    float total;
    if (reduce_partials(g, P, it.cloth, dq, &total) && (threadIdx.x & 31) == 0) R[kRedDAD] = R[kRedDAD] + total;
}

// Device alpha, solution / residual / preconditioned residual update with the
// incremental position write-back, partial r.z (abi41.cu:3320-3405).
__global__ void __launch_bounds__(kThreads) k_pcg_update(View v, PcgView g) {
    const PcgItem it = pcg_item(v, g);
    const Params& P = v.P[it.cloth];
    const int i = it.i;
    float* R = g.red + it.cloth * kRedSlots;
    const float rz_old = R[kRedRZ], dad = R[kRedDAD];
    float status = kStatusOk, alpha = 0.0f;
    if (!isfinite(rz_old) || rz_old < 0.0f) {
        status = kStatusBadResidual;
    } else if (rz_old <= 1.0e-14f) {
        status = kStatusZeroResidual;
    } else if (!isfinite(dad) || dad <= 1.0e-14f) {
        status = kStatusBadDad;
    } else {
        alpha = rz_old / dad;
        if (!isfinite(alpha)) status = kStatusBadAlpha;
    }
    float rz = 0.0f;
    if (status == kStatusOk && it.valid) {
        const float4 p4 = v.pos[i];
        if (!(p4.w > 0.0f)) {
            g.r[i] = z4();
            g.z[i] = z4();
        } else {
            const F3 di = f3(g.d[i]);
            const F3 qi = f3(g.q[i]);
            const F3 ri = f3(g.r[i]);
            const F3 res{fmaf(qi.x, -alpha, ri.x), fmaf(qi.y, -alpha, ri.y), fmaf(qi.z, -alpha, ri.z)};
            const F3 safe_res = finite3(res) ? res : F3{0.0f, 0.0f, 0.0f};
            const F3 z = sym_madd(sym_load(g.pinv, i), safe_res, F3{0.0f, 0.0f, 0.0f});
            g.r[i] = f4(safe_res, 0.0f);
            g.z[i] = f4(z, 0.0f);
            rz = dot3(safe_res, z);
            F3 delta = di * alpha;
            const float len = len3(delta);
            const float max_delta = writeback_limit(P);
            if (len > max_delta) {
                delta = delta * (max_delta / fmaxf(len, kEps));
                count1(v.counts, kCntHardFallbacks);
            }
            v.pos[i] = f4(f3(p4) + delta, p4.w);
            v.prev[i] = f4(f3(v.prev[i]) + delta * 0.08f, 0.0f);
            const float dl = len3(delta);
            if (dl > 0.0f) atomicMax(g.max_delta_bits, __float_as_uint(dl));
        }
    }
    if (status != kStatusOk) {
        if (it.local == 0) {
            R[kRedStatus] = status;
            if (status != kStatusZeroResidual) atomicAdd(g.guard, 1ull);
        }
        return;
    }
    float total;
    if (reduce_partials(g, P, it.cloth, rz, &total) && (threadIdx.x & 31) == 0) {
        R[kRedRZNext] = R[kRedRZNext] + total;
        R[kRedIterations] = R[kRedIterations] + 1.0f;
    }
}

// Device beta and d = z + beta d (abi41.cu:3421-3450); the last block then
// advances the scalar slots (abi41.cu:3452-3464).
__global__ void __launch_bounds__(kThreads) k_pcg_dir(View v, PcgView g) {
    const PcgItem it = pcg_item(v, g);
    const Params& P = v.P[it.cloth];
    const int i = it.i;
    float* R = g.red + it.cloth * kRedSlots;
    const float status = R[kRedStatus], rz_old = R[kRedRZ], rz_new = R[kRedRZNext];
    const bool ok = status == kStatusOk && isfinite(rz_old) && isfinite(rz_new) && rz_old > 1.0e-14f && rz_new >= 0.0f;
    const float beta = ok ? rz_new / rz_old : 0.0f;
    if (ok && isfinite(beta) && it.valid) {
        if (!(v.pos[i].w > 0.0f)) {
            g.d[i] = z4();
        } else {
            const F3 d = f3(g.d[i]), z = f3(g.z[i]);
            g.d[i] = make_float4(fmaf(d.x, beta, z.x), fmaf(d.y, beta, z.y), fmaf(d.z, beta, z.z), 0.0f);
        }
    }
    float total;
    if (reduce_partials(g, P, it.cloth, 0.0f, &total) && threadIdx.x == 0) {
        if (status == kStatusOk && isfinite(rz_new) && rz_new >= 0.0f) {
            R[kRedRZ] = rz_new;
            R[kRedDAD] = 0.0f;
            R[kRedRZNext] = 0.0f;
            R[kRedStatus] = kStatusOk;
        }
    }
}

// ------------------------------------------------------- averaged caps --
// Edge correction shared by the averaged polish / tiny passes, seen from one
// endpoint (abi41.cu:1995-2082, 2399-2467).  Returns false when the edge
// contributes nothing to this vertex.
__device__ bool averaged_delta(const Params& P, bool tiny, float4 pi, float4 pj, F3 prev_i, F3 prev_j, float rest,
                               bool self_is_j, F3* out) {
    const float wi = pi.w, wj = pj.w, weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return false;
    if (tiny) {
        if (!isfinite(rest) || rest <= kEps || rest > 7.5e-4f) return false;
        if (!finite3(f3(pi)) || !finite3(f3(pj))) return false;
    } else {
        if (!isfinite(rest) || rest <= kEps) return false;
        if (!finite3(f3(pi)) || !finite3(f3(pj)) || !finite3(prev_i) || !finite3(prev_j)) return false;
    }
    const F3 edge = f3(pj) - f3(pi);
    const float len_sq = dot3(edge, edge);
    if (!isfinite(len_sq) || len_sq <= 1.0e-14f) return false;
    const float len = sqrtf(len_sq);
    float target, relax, max_delta;
    if (tiny) {
        target = rest * 1.06f;
        relax = 1.0f;
        max_delta = fminf(fmaxf(rest * 3.0f, 2.5e-4f), 8.0e-4f);
    } else {
        target = rest * (P.stretch_strength >= 0.95f ? 1.08f : 1.18f);
        relax = 0.90f;
        max_delta = fmaxf(5.0e-4f, fminf(fmaxf(rest * 2.0f, P.thickness * 0.25f), 0.008f));
    }
    const float excess = len - target;
    if (!isfinite(excess) || excess <= 0.0f) return false;
    const F3 corr = edge * (-relax * excess / fmaxf(weight * len, kEps));
    if (!finite3(corr) || (tiny ? len3(corr) <= 1.0e-20f : false)) return false;
    if (!tiny) {
        const float cl = len3(corr);
        if (!isfinite(cl) || cl <= 1.0e-20f) return false;
    }
    const float w = self_is_j ? wj : wi;
    if (!(w > 0.0f)) return false;
    const F3 d = limit_delta(self_is_j ? corr * wj : corr * (-wi), max_delta);
    if (!finite3(d) || !(len3(d) > 0.0f)) return false;
    *out = d;
    return true;
}

// Gather of the averaged corrections of a vertex's edges into sum / count.
// Vertices of cloths without the hard polish are left alone.
__global__ void __launch_bounds__(kThreads) k_avg_gather(View v, PcgView g, int tiny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nV) return;
    const Params& P = params_v(v, i);
    if (!P.pcg_hard) return;
    const float4 p4 = v.pos[i];
    const F3 prev_self = f3(v.prev[i]);
    F3 sum{0.0f, 0.0f, 0.0f};
    float count = 0.0f;
    const int begin = v.sp_off[i], end = v.sp_off[i + 1];
    for (int k = begin; k < end; ++k) {
        const int2 e = __ldg(&v.sp_ent[k]);
        const bool self_is_j = (e.x & kSideBit) != 0;
        const int o = e.x & 0x7fffffff;
        const float4 q4 = v.pos[o];
        const F3 prev_o = tiny ? F3{0.0f, 0.0f, 0.0f} : f3(v.prev[o]);
        F3 d;
        if (averaged_delta(P, tiny != 0, self_is_j ? q4 : p4, self_is_j ? p4 : q4, self_is_j ? prev_o : prev_self,
                           self_is_j ? prev_self : prev_o, __int_as_float(e.y), self_is_j, &d)) {
            sum = sum + d;
            count += 1.0f;
        }
    }
    g.avg[i] = f4(sum, count);
}

// Apply the averaged corrections (abi41.cu:2084-2112, 2469-2494).
__global__ void __launch_bounds__(kThreads) k_avg_apply(View v, PcgView g, int tiny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nV) return;
    const Params& P = params_v(v, i);
    if (!P.pcg_hard) return;
    const float4 p4 = v.pos[i];
    if (!(p4.w > 0.0f)) return;
    const float4 a = g.avg[i];
    const float count = a.w;
    if (!isfinite(count) || count <= 0.0f) return;
    F3 delta = F3{a.x, a.y, a.z} * (1.0f / count);
    if (!finite3(delta)) {
        count1(v.counts, kCntHardFallbacks);
        return;
    }
    const float max_delta = tiny ? fminf(fmaxf(P.thickness * 0.015f, 2.5e-4f), 9.0e-4f)
                                 : fmaxf(5.0e-4f, fminf(fmaxf(P.thickness * 0.20f, 1.0e-3f), 0.005f));
    delta = limit_delta(delta, max_delta);
    if (!finite3(delta) || !(len3(delta) > 0.0f)) return;
    v.pos[i] = f4(f3(p4) + delta, p4.w);
    v.prev[i] = f4(f3(v.prev[i]) + delta * (tiny ? 0.24f : 0.16f), 0.0f);
}

// ------------------------------------------------------------ ratio caps --
// One edge of a ratio cap: normal (kind 0, abi41.cu:2249-2362), tiny (1,
// 2496-2601) or extreme (2, 2603-2708).  Writes each endpoint's position
// correction d and previous-position shift pd; ok = false where that
// endpoint gets nothing.  Returns false when the edge is skipped.
struct CapSide {
    F3 d, pd;
    bool ok;
};

__device__ bool cap_edge(const Params& P, int kind, float rest, float4 pi4, float4 pj4, F3 qi, F3 qj, CapSide* si, CapSide* sj) {
    si->ok = sj->ok = false;
    const bool tiny = kind == 1;
    if (!isfinite(rest) || rest <= kEps) return false;
    if (tiny ? rest > 7.5e-4f : rest <= 7.5e-4f) return false;
    const float dt = P.sub_dt;
    const float wi = pi4.w, wj = pj4.w, weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return false;
    const F3 pi = f3(pi4), pj = f3(pj4);
    if (!finite3(pi) || !finite3(pj) || !finite3(qi) || !finite3(qj)) return false;
    const F3 edge = pj - pi;
    const float len_sq = dot3(edge, edge);
    if (!isfinite(len_sq) || len_sq <= 1.0e-14f) return false;
    const float len = sqrtf(len_sq);
    const bool high = P.stretch_strength >= 0.95f;
    float start_ratio, target_ratio, max_delta, prev_sync;
    if (kind == 0) {
        start_ratio = high ? 1.12f : 1.32f;
        target_ratio = high ? 1.04f : 1.22f;
        max_delta = fminf(fmaxf(rest * 0.60f, P.thickness * 0.10f), 0.010f);
        prev_sync = 0.08f;
    } else if (kind == 1) {
        start_ratio = 1.35f;
        target_ratio = 1.12f;
        max_delta = fminf(fmaxf(rest * 6.0f, 5.0e-4f), 1.5e-3f);
        prev_sync = 1.0f;
    } else {
        start_ratio = 1.24f;
        target_ratio = 1.10f;
        max_delta = fminf(fmaxf(rest * 1.25f, P.thickness * 0.10f), 0.006f);
        prev_sync = 0.30f;
    }
    if (!isfinite(len) || len <= rest * start_ratio) return false;
    const float excess = len - rest * target_ratio;
    if (!isfinite(excess) || excess <= 0.0f) return false;
    const F3 corr = edge * (-excess / fmaxf(weight * len, kEps));
    if (!finite3(corr) || len3(corr) <= 1.0e-20f) return false;
    F3 pdi{0.0f, 0.0f, 0.0f}, pdj{0.0f, 0.0f, 0.0f};
    const F3 normal = edge * (1.0f / fmaxf(len, kEps));
    const float sdt = kind == 0 ? fmaxf(dt, kEps) : dt;
    if (isfinite(sdt) && sdt > kEps) {
        const float inv_dt = 1.0f / sdt;
        const F3 vi = (pi - qi) * inv_dt, vj = (pj - qj) * inv_dt;
        const float sep = dot3(vj - vi, normal);
        if (isfinite(sep) && sep > 0.0f) {
            const float trim = sep * sdt * 1.0f / weight;
            if (wi > 0.0f) pdi = pdi + normal * (-wi * trim);
            if (wj > 0.0f) pdj = pdj + normal * (wj * trim);
        }
    }
    if (wi > 0.0f) {
        const F3 d = limit_delta(corr * (-wi), max_delta);
        if (finite3(d) && len3(d) > 0.0f) *si = CapSide{d, pdi + d * prev_sync, true};
    }
    if (wj > 0.0f) {
        const F3 d = limit_delta(corr * wj, max_delta);
        if (finite3(d) && len3(d) > 0.0f) *sj = CapSide{d, pdj + d * prev_sync, true};
    }
    return true;
}

// Caps applied in place one edge colour at a time (no two edges of a colour
// share a vertex), over a caller's edge colouring.  In a batch a launch
// covers one colour of every cloth that uses its colouring; the time step is
// the cloth's substep length.
__global__ void __launch_bounds__(kThreads) k_cap_range(View v, int start, int count, int kind) {
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    if (local >= count) return;
    const int s = start + local;
    if (s < 0 || s >= v.nE) return;
    const int2 ed = __ldg(&v.edges[s]);
    const int i = ed.x, j = ed.y;
    if (i < 0 || j < 0 || i >= v.nV || j >= v.nV || i == j) return;
    const Params& P = params_v(v, i);
    const float4 pi4 = v.pos[i], pj4 = v.pos[j];
    const F3 qi = f3(v.prev[i]), qj = f3(v.prev[j]);
    CapSide si, sj;
    if (!cap_edge(P, kind, __ldg(&v.edge_rest[s]), pi4, pj4, qi, qj, &si, &sj)) return;
    if (si.ok) {
        v.pos[i] = f4(f3(pi4) + si.d, pi4.w);
        v.prev[i] = f4(qi + si.pd, 0.0f);
    }
    if (sj.ok) {
        v.pos[j] = f4(f3(pj4) + sj.d, pj4.w);
        v.prev[j] = f4(qj + sj.pd, 0.0f);
    }
}

// Caps of a cloth without a caller's colouring: the reference launches one
// kernel over every edge, each adding its corrections to both endpoints with
// float atomics (abi41.cu:7794-7801), i.e. a Jacobi pass.  Here every edge
// sees the positions and previous positions at the start of the pass and
// each vertex adds its edges' corrections in edge order (vertex -> edge CSR)
// into pos_out / prev_out; k_cap_store copies them back.
__global__ void __launch_bounds__(kThreads) k_cap_jacobi(View v, int kind, float4* pos_out, float4* prev_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nV) return;
    const Params& P = params_v(v, i);
    if (!P.pcg_hard || !P.cap_jacobi) return;
    const float4 self4 = v.pos[i];
    const F3 self_prev = f3(v.prev[i]);
    F3 p = f3(self4), q = self_prev;
    for (int k = v.sp_off[i]; k < v.sp_off[i + 1]; ++k) {
        const int2 e = __ldg(&v.sp_ent[k]);
        const bool self_is_j = (e.x & kSideBit) != 0;
        const int o = e.x & 0x7fffffff;
        const float4 o4 = v.pos[o];
        const F3 oq = f3(v.prev[o]);
        CapSide si, sj;
        if (!cap_edge(P, kind, __int_as_float(e.y), self_is_j ? o4 : self4, self_is_j ? self4 : o4, self_is_j ? oq : self_prev,
                      self_is_j ? self_prev : oq, &si, &sj))
            continue;
        const CapSide& me = self_is_j ? sj : si;
        if (me.ok) {
            p = p + me.d;
            q = q + me.pd;
        }
    }
    pos_out[i] = f4(p, self4.w);
    prev_out[i] = f4(q, 0.0f);
}

__global__ void __launch_bounds__(kThreads) k_cap_store(View v, const float4* pos_in, const float4* prev_in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nV) return;
    const Params& P = params_v(v, i);
    if (!P.pcg_hard || !P.cap_jacobi) return;
    v.pos[i] = pos_in[i];
    v.prev[i] = prev_in[i];
}

}  // namespace

int pcg_blocks(int V) { return V > 0 ? blocks_for(V) : 0; }

void pcg_solve(const View& v, const PcgView& g, int blocks, cudaStream_t s, long long* launches) {
    if (blocks <= 0) return;
    const int b = blocks;
    k_pcg_build<<<b, kThreads, 0, s>>>(v, g);
    for (int it = 0; it < 8; ++it) {
        k_pcg_ad<<<b, kThreads, 0, s>>>(v, g);
        k_pcg_update<<<b, kThreads, 0, s>>>(v, g);
        *launches += 2;
        if (it + 1 < 8) {
            k_pcg_dir<<<b, kThreads, 0, s>>>(v, g);
            *launches += 1;
        }
    }
    *launches += 1;
}

void pcg_averaged_pass(const View& v, const PcgView& g, int V, bool tiny, cudaStream_t s) {
    if (V <= 0) return;
    k_avg_gather<<<blocks_for(V), kThreads, 0, s>>>(v, g, tiny ? 1 : 0);
    k_avg_apply<<<blocks_for(V), kThreads, 0, s>>>(v, g, tiny ? 1 : 0);
}

void pcg_cap_range(const View& v, int start, int count, int kind, cudaStream_t s) {
    if (count > 0) k_cap_range<<<blocks_for(count), kThreads, 0, s>>>(v, start, count, kind);
}

void pcg_cap_jacobi(const View& v, const PcgView& g, int V, int kind, cudaStream_t s) {
    if (V <= 0) return;
    k_cap_jacobi<<<blocks_for(V), kThreads, 0, s>>>(v, kind, g.r, g.z);
    k_cap_store<<<blocks_for(V), kThreads, 0, s>>>(v, g.r, g.z);
}

}  // namespace xg
