// Per-vertex kernels of one XPBD substep: prediction, the fused constraint /
// contact pass, bends per colour, and the position pack for downloads.
//
// The reference launches one kernel per stage over every vertex or
// constraint (native/src/ssbl_xpbd_cuda_abi41.cu:9165-9376): integrate, pins,
// springs (float atomics into pos), pins, analytic contacts, SDF contacts,
// pins, velocity.  Pins, analytic contacts, SDF contacts and the velocity
// update only read and write the vertex they act on, so this library runs
// them as stages of one per-vertex kernel.  Stretch (and the once-per-frame
// tethers) become a gather over a vertex->constraint CSR that reads a
// snapshot of the positions (ping-pong buffer) and sums the corrections of
// the incident constraints in constraint order: the same snapshot-Jacobi
// update as the reference's atomics, without float atomics, and therefore
// deterministic.
#include "xpbd_constraint.cuh"
#include <cooperative_groups.h>

#include "xpbd_contact.cuh"
#include "xpbd_fields.cuh"
#include "xpbd_solver.cuh"

namespace xg {

namespace {

struct VState {
    F3 p, prev, vel;
    float w;  // effective inverse mass
};

// Weighted pin projection of one vertex (abi41.cu:3466-3509).  Pins are
// stored per vertex (weight -1 = no pin; a vertex listed twice keeps its last
// entry) and the relaxation 1 - (1 - s)^(1/(I+1)) is precomputed on the host.
__device__ void pin_stage(const View& v, int i, float inv_mass, float dt, VState* s) {
    const float weight = __ldg(&v.pin_weight[i]);
    if (!isfinite(weight) || weight < 0.05f) return;
    const F3 target = f3(ld4(&v.pin_target[i]));
    if (weight >= 0.75f || inv_mass <= 0.0f) {
        s->p = target;
        s->prev = target;
        s->vel = F3{0.0f, 0.0f, 0.0f};
        return;
    }
    const float relax = __ldg(&v.pin_relax[i]);
    if (relax <= 0.0f) return;
    const F3 corrected = s->p + (target - s->p) * relax;
    const F3 damped = s->vel * fmaxf(1.0f - relax, 0.0f);
    s->p = corrected;
    s->prev = corrected - damped * fmaxf(dt, kEps);
    s->vel = damped;
}

// Ground plane (z up), sphere and wall (abi41.cu:3511-3590).
__device__ void analytic_stage(const Params& P, unsigned long long* counts, float inv_mass, float dt, VState* s) {
    if (inv_mass <= 0.0f) return;
    F3 p = s->p;
    F3 vel = s->vel;
    bool contacted = false;
    const float margin = fmaxf(P.margin, 0.0f);
    const float sdt = fmaxf(dt, kEps);
    if (P.use_ground && p.z < P.ground_height + margin) {
        const float target_z = P.ground_height + margin;
        const float pen = target_z - p.z;
        const F3 n{0.0f, 0.0f, 1.0f};
        const float inward = fmaxf(-dot3(vel, n), 0.0f);
        p.z = target_z;
        contact_response(P, counts, n, inward + pen / sdt, &vel);
        contacted = true;
    }
    if (P.use_sphere && P.sphere_radius > 0.0f) {
        const F3 c{P.sphere_center[0], P.sphere_center[1], P.sphere_center[2]};
        const F3 d = p - c;
        const float dist = sqrtf(fmaxf(dot3(d, d), kEps));
        const float target = P.sphere_radius + margin;
        if (dist < target) {
            const F3 n = dist > kEps ? d * (1.0f / dist) : F3{0.0f, 0.0f, 1.0f};
            const float pen = target - dist;
            const float inward = fmaxf(-dot3(vel, n), 0.0f);
            p = c + n * target;
            contact_response(P, counts, n, inward + pen / sdt, &vel);
            contacted = true;
        }
    }
    if (P.use_wall) {
        const F3 o{P.wall_origin[0], P.wall_origin[1], P.wall_origin[2]};
        F3 n{P.wall_normal[0], P.wall_normal[1], P.wall_normal[2]};
        const float nlen = sqrtf(fmaxf(dot3(n, n), kEps));
        n = n * (1.0f / nlen);
        const float gap = dot3(p - o, n);
        if (gap < margin) {
            const float pen = margin - gap;
            const float inward = fmaxf(-dot3(vel, n), 0.0f);
            p = p + n * (margin - gap);
            contact_response(P, counts, n, inward + pen / sdt, &vel);
            contacted = true;
        }
    }
    s->p = p;
    if (contacted) {
        s->vel = vel;
        s->prev = p - vel * sdt;
    }
}

__device__ __forceinline__ int sdf_index(const Params& P, int x, int y, int z) {
    return (z * P.sdf_dim[1] + y) * P.sdf_dim[0] + x;
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }

__device__ float sdf_trilinear(const Params& P, const float* sdf, float gx, float gy, float gz) {
    const int x0 = min(max((int)floorf(gx), 0), P.sdf_dim[0] - 1);
    const int y0 = min(max((int)floorf(gy), 0), P.sdf_dim[1] - 1);
    const int z0 = min(max((int)floorf(gz), 0), P.sdf_dim[2] - 1);
    const int x1 = min(x0 + 1, P.sdf_dim[0] - 1);
    const int y1 = min(y0 + 1, P.sdf_dim[1] - 1);
    const int z1 = min(z0 + 1, P.sdf_dim[2] - 1);
    const float tx = gx - (float)x0, ty = gy - (float)y0, tz = gz - (float)z0;
    const float c000 = __ldg(&sdf[sdf_index(P, x0, y0, z0)]);
    const float c100 = __ldg(&sdf[sdf_index(P, x1, y0, z0)]);
    const float c010 = __ldg(&sdf[sdf_index(P, x0, y1, z0)]);
    const float c110 = __ldg(&sdf[sdf_index(P, x1, y1, z0)]);
    const float c001 = __ldg(&sdf[sdf_index(P, x0, y0, z1)]);
    const float c101 = __ldg(&sdf[sdf_index(P, x1, y0, z1)]);
    const float c011 = __ldg(&sdf[sdf_index(P, x0, y1, z1)]);
    const float c111 = __ldg(&sdf[sdf_index(P, x1, y1, z1)]);
    const float c0 = lerpf(lerpf(c000, c100, tx), lerpf(c010, c110, tx), ty);
    const float c1 = lerpf(lerpf(c001, c101, tx), lerpf(c011, c111, tx), ty);
    return lerpf(c0, c1, tz);
}

// Trilinear sample inside the grid, false outside (abi41.cu:1645-1691).
__device__ bool sdf_sample(const Params& P, const float* sdf, F3 p, float* out) {
    if (P.sdf_dim[0] < 2 || P.sdf_dim[1] < 2 || P.sdf_dim[2] < 2 || P.sdf_voxel <= 0.0f) return false;
    const float inv = 1.0f / P.sdf_voxel;
    const float gx = (p.x - P.sdf_origin[0]) * inv;
    const float gy = (p.y - P.sdf_origin[1]) * inv;
    const float gz = (p.z - P.sdf_origin[2]) * inv;
    if (gx < 0.0f || gy < 0.0f || gz < 0.0f || gx > (float)(P.sdf_dim[0] - 1) || gy > (float)(P.sdf_dim[1] - 1) ||
        gz > (float)(P.sdf_dim[2] - 1))
        return false;
    *out = sdf_trilinear(P, sdf, gx, gy, gz);
    return isfinite(*out);
}

// Sample with the point clamped into the grid (abi41.cu:1693-1723).
__device__ float sdf_sample_clamped(const Params& P, const float* sdf, F3 p) {
    const float inv = 1.0f / fmaxf(P.sdf_voxel, kEps);
    const float gx = fminf(fmaxf((p.x - P.sdf_origin[0]) * inv, 0.0f), (float)(P.sdf_dim[0] - 1));
    const float gy = fminf(fmaxf((p.y - P.sdf_origin[1]) * inv, 0.0f), (float)(P.sdf_dim[1] - 1));
    const float gz = fminf(fmaxf((p.z - P.sdf_origin[2]) * inv, 0.0f), (float)(P.sdf_dim[2] - 1));
    return sdf_trilinear(P, sdf, gx, gy, gz);
}

// Normal of the nearest static triangle, used when the SDF gradient vanishes
// (abi41.cu:1749-1769).
__device__ F3 nearest_static_normal(const Params& P, const float4* tris, F3 p) {
    F3 best{0.0f, 0.0f, 1.0f};
    float best_sq = 3.402823466e+38f;
    for (int t = 0; t < P.static_tri_count; ++t) {
        const F3 a = f3(ld4(&tris[t * 3 + 0])), b = f3(ld4(&tris[t * 3 + 1])), c = f3(ld4(&tris[t * 3 + 2]));
        const F3 d = p - closest_on_triangle(p, a, b, c);
        const float dsq = dot3(d, d);
        if (dsq < best_sq) {
            best_sq = dsq;
            best = dsq > kEps * kEps ? normalize_or(d, best) : normalize_or(cross3(b - a, c - a), best);
        }
    }
    return normalize_or(best, F3{0.0f, 0.0f, 1.0f});
}

// Central-difference SDF gradient (abi41.cu:1771-1785).
__device__ F3 sdf_normal(const Params& P, const float* sdf, const float4* tris, F3 p) {
    const float h = fmaxf(P.sdf_voxel, 1.0e-5f);
    const float dx = sdf_sample_clamped(P, sdf, p + F3{h, 0.0f, 0.0f}) - sdf_sample_clamped(P, sdf, p + F3{-h, 0.0f, 0.0f});
    const float dy = sdf_sample_clamped(P, sdf, p + F3{0.0f, h, 0.0f}) - sdf_sample_clamped(P, sdf, p + F3{0.0f, -h, 0.0f});
    const float dz = sdf_sample_clamped(P, sdf, p + F3{0.0f, 0.0f, h}) - sdf_sample_clamped(P, sdf, p + F3{0.0f, 0.0f, -h});
    const F3 n{dx, dy, dz};
    const float lsq = dot3(n, n);
    if (!isfinite(lsq) || lsq <= 1.0e-12f) return nearest_static_normal(P, tris, p);
    return n * (1.0f / sqrtf(lsq));
}

// Static SDF contact (abi41.cu:1831-1867).
__device__ void sdf_stage(const View& v, const Params& P, float inv_mass, float dt, VState* s) {
    if (inv_mass <= 0.0f || !P.sdf_ready) return;
    const float margin = fmaxf(P.margin, 0.0f);
    if (margin <= 0.0f) return;
    float d = 0.0f;
    if (!sdf_sample(P, P.sdf, s->p, &d) || d >= margin) return;
    const F3 n = sdf_normal(P, P.sdf, P.static_tris, s->p);
    if (!finite3(n)) return;
    const float pen = margin - d;
    if (!isfinite(pen) || pen <= 0.0f) return;
    const F3 corrected = s->p + n * pen;
    F3 vel = s->vel;
    const float inward = fmaxf(-dot3(vel, n), 0.0f);
    contact_response(P, v.counts, n, inward + pen / fmaxf(dt, kEps), &vel);
    s->p = corrected;
    s->vel = vel;
    s->prev = corrected - vel * fmaxf(dt, kEps);
    count1(v.counts, kCntStaticSdfContacts);
}

// v = v + feedback(measured - v) with the aligned-feedback clamp
// (abi41.cu:5846-5884); the arithmetic is velocity_update.
__device__ void velocity_stage(const Params& P, float dt, VState* s) {
    s->vel = velocity_update(s->p, s->prev, s->vel, s->w, P.thickness, dt);
}

// Stretch constraint of edge (i, j) seen from one of its endpoints
// (abi41.cu:1927-1980): the correction is computed in the edge's own
// orientation so both endpoints get bit-identical values.
__device__ __forceinline__ void spring_term(const Params& P, unsigned long long* counts, float dt, float4 pi, float4 pj,
                                            float rest, bool self_is_j, F3* dp, F3* dprev) {
    F3 corr;
    float c;
    bool clamped;
    if (!stretch_correction(pi, pj, rest, P.stretch_compliance, dt, &corr, &c, &clamped)) return;
    if (clamped && !self_is_j) count1(counts, kCntHardFallbacks);
    const float wi = pi.w, wj = pj.w;
    const float wself = self_is_j ? wj : wi;
    if (wself > 0.0f) {
        const F3 d = self_is_j ? corr * wj : corr * (-wi);
        *dp = *dp + d;
        if (c > 0.0f) *dprev = *dprev + d * 0.08f;
    }
}

// Long-range tether (anchor i, dynamic j) seen from one endpoint
// (abi41.cu:2710-2803).
__device__ __forceinline__ void tether_term(const Params& P, unsigned long long* counts, float dt, float4 pi4, float4 pj4,
                                            float rest, bool self_is_j, F3* dp, F3* dprev) {
    const bool counter = !self_is_j;  // count once per tether
    const float wi = pi4.w, wj = pj4.w;
    const float weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) {
        if (counter) count1(counts, kCntTackGuards);
        return;
    }
    const F3 pi = f3(pi4), pj = f3(pj4);
    if (!finite3(pi) || !finite3(pj)) {
        if (counter) count1(counts, kCntTackGuards);
        return;
    }
    F3 dx = pj - pi;
    const float len_sq = len_sq_xyz(dx);
    if (!isfinite(len_sq) || len_sq <= 1.0e-10f || !isfinite(rest) || rest <= kEps) {
        if (counter) count1(counts, kCntTackGuards);
        return;
    }
    const float inv_len = 1.0f / sqrtf(len_sq);
    const float len = len_sq * inv_len;
    const float stretch = len - rest;
    if (!isfinite(stretch) || stretch <= 0.0f) return;
    dx = dx * inv_len;
    const float base_c = fmaxf(P.lra_compliance, 1.0e-12f);
    const float stiff = (1.0f / base_c) * 500000.0f;
    const float alpha = (base_c / 500000.0f) / fmaxf(dt * dt, kEps);
    const float sw = stiff / fmaxf(stiff + 500000.0f, 1.0f);
    const float dlambda = -stretch / fmaxf(weight + alpha, kEps);
    F3 corr = dx * (0.35f * sw * dlambda);
    if (!finite3(corr)) {
        if (counter) count1(counts, kCntTackGuards);
        return;
    }
    const float corr_len = len3(corr);
    const float max_corr = fmaxf(5.0e-4f, fminf(fmaxf(rest, P.thickness) * 0.20f, 0.035f));
    if (!isfinite(corr_len) || corr_len <= 0.0f) return;
    if (corr_len > max_corr) {
        corr = corr * (max_corr / fmaxf(corr_len, kEps));
        if (counter) count1(counts, kCntTackGuards);
    }
    const bool has_th = P.thickness > 0.0f;
    const float cap = has_th ? 0.0025f : 0.012f;
    const float rest_limit = fmaxf(rest, 0.0f) * (has_th ? 0.02f : 0.08f);
    const float th_limit = has_th ? P.thickness * 0.12f : cap;
    const float applied = fmaxf(5.0e-4f, fminf(fminf(rest_limit, th_limit), cap));
    if (self_is_j) {
        if (wj > 0.0f) {
            const F3 d = limit_delta(corr * (wj / fmaxf(weight, kEps)), applied);
            *dp = *dp + d;
            *dprev = *dprev + d * 0.32f;
        }
    } else if (wi > 0.0f) {
        const F3 d = limit_delta(corr * (-wi / fmaxf(weight, kEps)), applied);
        *dp = *dp + d;
        *dprev = *dprev + d * 0.32f;
    }
    if (counter) count1(counts, kCntLraTacks);
}

// Bend distance constraint between the two wing-opposite vertices, shared by
// the per-colour kernel and the Jacobi gather used when no colours are given
// (abi41.cu:2805-2884 and 2886-2970).  Returns false when the constraint is
// skipped; `guard` is set when the reference would count a guard.
__device__ __forceinline__ bool bend_correction(const Params& P, float dt, float4 pi4, float4 pj4, float rest, F3* corr_out,
                                                bool* guard) {
    bool clamped;
    return bend_correction_k(pi4, pj4, rest, P.bend_compliance, P.thickness, dt, corr_out, guard, &clamped);
}

__device__ __forceinline__ void bend_term(const Params& P, unsigned long long* counts, float dt, float4 pi, float4 pj,
                                          float rest, bool self_is_j, F3* dp, F3* dprev) {
    F3 corr;
    bool guard;
    const bool applied = bend_correction(P, dt, pi, pj, rest, &corr, &guard);
    if (!self_is_j) {
        if (guard) count1(counts, kCntBendingGuards);
        if (applied) count1(counts, kCntBendingWings);
    }
    if (!applied) return;
    const float wself = self_is_j ? pj.w : pi.w;
    if (wself > 0.0f) {
        const F3 d = self_is_j ? corr * pj.w : corr * (-pi.w);
        *dp = *dp + d;
        *dprev = *dprev + d * 0.06f;
    }
}

// Area-weighted normal of a vertex from its incident triangles in the
// snapshot positions (abi41.cu:1213-1261; 1/sqrt in IEEE arithmetic).
__device__ bool vertex_normal(const View& v, int i, F3* out) {
    if (!v.vt_off) return false;
    const int begin = __ldg(&v.vt_off[i]), end = __ldg(&v.vt_off[i + 1]);
    if (end <= begin) return false;
    F3 acc{0.0f, 0.0f, 0.0f};
    for (int k = begin; k < end; ++k) {
        const int t = __ldg(&v.vt_tri[k]);
        if (t < 0 || t >= v.nT) continue;
        const int4 tr = __ldg(&v.tris[t]);
        if (tr.x < 0 || tr.y < 0 || tr.z < 0 || tr.x >= v.nV || tr.y >= v.nV || tr.z >= v.nV) continue;
        const F3 p0 = f3(v.pos_in[tr.x]), p1 = f3(v.pos_in[tr.y]), p2 = f3(v.pos_in[tr.z]);
        const F3 n = cross3(p1 - p0, p2 - p0);
        const float l2 = dot3(n, n);
        if (!isfinite(l2) || l2 <= 1.0e-10f) continue;
        acc = acc + n * (1.0f / sqrtf(l2));
    }
    const float a2 = dot3(acc, acc);
    if (!isfinite(a2) || a2 <= 1.0e-10f) return false;
    *out = acc * (1.0f / sqrtf(a2));
    return true;
}

// Integrate (abi41.cu:1869-1925): gravity, volume pressure along the vertex
// normal, force fields, damping, pressure speed trims; fixed vertices return
// to rest.  Reads the snapshot `pos_in` and writes `pos` (the same buffer
// unless vertex normals are gathered).
__device__ __forceinline__ void predict_item(const View& v, int i) {
    const Params& P = params_v(v, i);
    const float4 p4 = v.pos_in[i];
    if (!P.active) {
        if (v.pos != v.pos_in) v.pos[i] = p4;
        return;
    }
    const float dt = P.sub_dt;
    const float inv_mass = __ldg(&v.inv_mass[i]);
    VState s;
    s.w = p4.w;
    s.prev = f3(p4);
    if (!(p4.w > 0.0f)) {
        s.vel = F3{0.0f, 0.0f, 0.0f};
        s.p = f3(ld4(&v.rest[i]));
    } else {
        F3 normal{0.0f, 0.0f, 0.0f};
        const bool has_normal = P.needs_normal && vertex_normal(v, i, &normal);
        F3 accel = F3{P.gravity[0], P.gravity[1], P.gravity[2]} + F3{0.0f, 0.0f, 0.0f};
        const bool pressure = P.pressure_on && has_normal;
        const float area = pressure ? __ldg(&v.p_area[i]) : 0.0f;
        if (pressure && isfinite(area) && area > 0.0f)
            accel = accel + normal * (P.pressure_strength * P.pressure_accel_scale * area * inv_mass);
        if (P.field_count > 0) {
            F3 fa{0.0f, 0.0f, 0.0f};
            const F3 vel0 = f3(v.vel[i]);
            const int n = min(P.field_count, kMaxFields);
            for (int k = 0; k < n; ++k) fa = fa + field_accel(P.fields[k], f3(p4), vel0, normal, has_normal);
            accel = accel + cap_field_accel(fa);
        }
        F3 vel = f3(v.vel[i]) + accel * dt;
        vel = vel * P.damping;
        if (pressure) {
            const float rest = __ldg(&v.p_rest[i]);
            if (isfinite(rest) && rest > kEps && isfinite(dt) && dt > kEps) {
                const float pa = fmaxf(P.pressure_strength, 0.0f) * fmaxf(P.pressure_accel_scale, 0.0f) * fmaxf(area, 0.0f) *
                                 fmaxf(inv_mass, 0.0f);
                const float max_delta = fmaxf(rest * fmaxf(P.pressure_impulse_rest_scale, 0.0f), 1.0e-7f);
                const float delta = pa * dt * dt;
                if (isfinite(delta) && delta > max_delta) vel = vel - normal * ((delta - max_delta) / dt);
                const float vrest = fmaxf(rest, fmaxf(P.pressure_velocity_length_scale, 0.0f));
                const float max_out = fmaxf(vrest * fmaxf(P.pressure_velocity_rest_scale, 0.0f) / dt, 1.0e-6f);
                const float out = dot3(vel, normal);
                if (isfinite(out) && out > max_out) vel = vel - normal * (out - max_out);
            }
        }
        s.vel = vel;
        s.p = f3(p4) + vel * dt;
    }
    pin_stage(v, i, inv_mass, dt, &s);
    v.pos[i] = f4(s.p, s.w);
    v.prev[i] = f4(s.prev, 0.0f);
    v.vel[i] = f4(s.vel, 0.0f);
}

__global__ void __launch_bounds__(kThreads) k_predict(View v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.nV) predict_item(v, i);
}

__device__ __forceinline__ void vertex_pass_item(const View& v, int i, unsigned flags) {
    const Params& P = params_v(v, i);
    const float dt = P.sub_dt;
    const float4 p4 = v.pos_in[i];
    if (!P.active) {
        if (v.pos != v.pos_in) v.pos[i] = p4;  // keep the ping-pong buffers in step
        return;
    }
    VState s;
    s.w = p4.w;
    s.p = f3(p4);
    s.prev = f3(v.prev[i]);
    s.vel = f3(v.vel[i]);
    const float inv_mass = __ldg(&v.inv_mass[i]);
    // a cloth with the CG stretch solve has no spring gather (in a batch the
    // pass still carries its vertices to the other buffer)
    const unsigned gather = flags & (P.pcg_on ? (kPassTether | kPassBend) : (kPassSpring | kPassTether | kPassBend));
    if (gather) {
        const int kind = (gather & kPassSpring) ? 0 : ((gather & kPassTether) ? 1 : 2);
        const int* off = kind == 0 ? v.sp_off : (kind == 1 ? v.te_off : v.bj_off);
        const int2* ent = kind == 0 ? v.sp_ent : (kind == 1 ? v.te_ent : v.bj_ent);
        const int begin = __ldg(&off[i]), end = __ldg(&off[i + 1]);
        F3 dp = s.p, dprev = s.prev;
        for (int k = begin; k < end; ++k) {
            const int2 e = __ldg(&ent[k]);
            const bool self_is_j = (e.x & kSideBit) != 0;
            const float4 q4 = v.pos_in[e.x & 0x7fffffff];
            const float rest = __int_as_float(e.y);
            const float4 pi = self_is_j ? q4 : p4;
            const float4 pj = self_is_j ? p4 : q4;
            if (kind == 0)
                spring_term(P, v.counts, dt, pi, pj, rest, self_is_j, &dp, &dprev);
            else if (kind == 1)
                tether_term(P, v.counts, dt, pi, pj, rest, self_is_j, &dp, &dprev);
            else
                bend_term(P, v.counts, dt, pi, pj, rest, self_is_j, &dp, &dprev);
        }
        s.p = dp;
        s.prev = dprev;
    }
    if (flags & kPassPin) pin_stage(v, i, inv_mass, dt, &s);
    if (flags & kPassAnalytic) analytic_stage(P, v.counts, inv_mass, dt, &s);
    if (flags & kPassSdf) sdf_stage(v, P, inv_mass, dt, &s);
    // final pin polish when this cloth ran a contact stage in this iteration
    // (analytic colliders, SDF, or any last iteration; abi41.cu:9360-9369)
    if ((flags & kPassPinPolish) &&
        (v.last_it || P.use_ground || P.use_wall || P.use_sphere || P.sdf_ready))
        pin_stage(v, i, inv_mass, dt, &s);
    if (flags & kPassVelocity) velocity_stage(P, dt, &s);
    v.pos[i] = f4(s.p, s.w);
    v.prev[i] = f4(s.prev, 0.0f);
    v.vel[i] = f4(s.vel, 0.0f);
}

// Six 256-thread blocks per SM (40 registers): the gathers are latency
// bound, and the extra resident warps outweigh the spills (batch256 stretch
// passes 2.05 -> 1.85 ms per frame; five blocks 1.98).
__global__ void __launch_bounds__(kThreads, 6) k_vertex_pass(View v, unsigned flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.nV) vertex_pass_item(v, i, flags);
}

// Bend constraints of one colour, applied in place: no two bends of a colour
// share a vertex (abi41.cu:2886-2970).
__device__ __forceinline__ void bend_item(const View& v, int b) {
    if (b < 0 || b >= v.nB) {
        count1(v.counts, kCntBendingGuards);
        return;
    }
    const int2 pr = __ldg(&v.bends[b]);
    const int i = pr.x, j = pr.y;
    if (i < 0 || j < 0 || i >= v.nV || j >= v.nV || i == j) {
        count1(v.counts, kCntBendingGuards);
        return;
    }
    const Params& P = params_v(v, i);
    if (!P.active) return;
    const float dt = P.sub_dt;
    const float4 pi4 = v.pos[i], pj4 = v.pos[j];
    F3 corr;
    bool guard;
    const bool applied = bend_correction(P, dt, pi4, pj4, __ldg(&v.bend_rest[b]), &corr, &guard);
    if (guard) count1(v.counts, kCntBendingGuards);
    if (!applied) return;
    if (pi4.w > 0.0f) {
        const F3 d = corr * (-pi4.w);
        v.pos[i] = f4(f3(pi4) + d, pi4.w);
        v.prev[i] = f4(f3(v.prev[i]) + d * 0.06f, 0.0f);
    }
    if (pj4.w > 0.0f) {
        const F3 d = corr * pj4.w;
        v.pos[j] = f4(f3(pj4) + d, pj4.w);
        v.prev[j] = f4(f3(v.prev[j]) + d * 0.06f, 0.0f);
    }
    count1(v.counts, kCntBendingWings);
}

__global__ void __launch_bounds__(kThreads) k_bend_color(View v, int start, int count) {
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    if (local < count) bend_item(v, start + local);
}

__global__ void k_copy_pos(float4* dst, const float4* src, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

__global__ void k_pack_positions(float* dst, const float4* src, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = src[i];
    dst[i * 3 + 0] = p.x;
    dst[i * 3 + 1] = p.y;
    dst[i * 3 + 2] = p.z;
}

// Scatter of changed pin entries (vertices whose pin was set or cleared).
__global__ void k_pin_scatter(const int* idx, const float4* target, const float* weight, const float* relax, int n,
                              float4* pin_target, float* pin_weight, float* pin_relax, int nV) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = idx[k];
    if (i < 0 || i >= nV) return;
    pin_target[i] = target[k];
    pin_weight[i] = weight[k];
    pin_relax[i] = relax[k];
}

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

// The per-vertex passes are latency bound (gathers of neighbours): by default
// 128-thread blocks spread a 10k-vertex cloth over twice as many SMs.
// One block per cloth; the cloth's positions (both ping-pong buffers),
// previous positions and velocities live in shared memory for the whole
// frame, so the neighbour gathers and the per-vertex stages touch no global
// memory for state.  Every operation of the recorded frame sweeps the cloth's
// items with the block's threads, then the block synchronises.  The state
// pointers of the View are offset by the cloth's first vertex, so the item
// functions index them with global vertex indices as in the launched form.
__global__ void __launch_bounds__(1024) k_frame_fused(View base, const FrameOp* ops, int nops, float4* buf0,
                                                       const int2* bend_ranges, int K) {
    extern __shared__ float4 sm[];
    const int k = blockIdx.x;
    if (k >= K) return;
    const Params& P = base.P[k];
    const int v0 = P.vstart, n = P.V, v1 = P.vstart + P.V;
    const int cap = (int)(blockDim.x);  // vertices per state array in shared memory
    float4* s0 = sm;
    float4* s1 = sm + cap;
    float4* sprev = sm + 2 * cap;
    float4* svel = sm + 3 * cap;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s0[i] = buf0[v0 + i];
        sprev[i] = base.prev[v0 + i];
        svel[i] = base.vel[v0 + i];
    }
    __syncthreads();
    View v = base;
    v.prev = sprev - v0;
    v.vel = svel - v0;
    float4* b0 = s0 - v0;
    float4* b1 = s1 - v0;
    for (int o = 0; o < nops; ++o) {
        const FrameOp op = ops[o];
        v.pos_in = op.in_buf ? b1 : b0;
        v.pos = op.out_buf ? b1 : b0;
        v.substep = op.substep;
        v.last_it = op.last_it;
        if (op.kind == 0) {
            for (int i = v0 + (int)threadIdx.x; i < v1; i += blockDim.x) predict_item(v, i);
        } else if (op.kind == 1) {
            for (int i = v0 + (int)threadIdx.x; i < v1; i += blockDim.x) vertex_pass_item(v, i, op.flags);
        } else if (op.kind == 2) {
            const int2 r = bend_ranges[op.color * K + k];
            for (int b = r.x + (int)threadIdx.x; b < r.x + r.y; b += blockDim.x) bend_item(v, b);
        } else {
            for (int i = v0 + (int)threadIdx.x; i < v1; i += blockDim.x) v.pos[i] = v.pos_in[i];
        }
        __syncthreads();
    }
    // a frame ends with its result in buffer 0
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        buf0[v0 + i] = s0[i];
        base.prev[v0 + i] = sprev[i];
        base.vel[v0 + i] = svel[i];
    }
}

// Cluster form of the fused frame: a thread-block cluster of C CTAs (C SMs)
// per cloth.  Each CTA holds a full copy of the cloth's state in its shared
// memory and computes the vertex operations for its slice of the vertices;
// after each operation it writes its slice of the arrays the operation wrote
// into the other CTAs' copies (distributed shared memory), then the cluster
// synchronises.  Bend colours are computed by every CTA on its own copy
// (identical work, identical results), so their scattered writes need no
// exchange.  Within an operation the incoming copies touch only other
// slices of the arrays being written (gathers read the other buffer; the
// previous positions and velocities are read for the own vertex only).
namespace cgx = cooperative_groups;

__global__ void __launch_bounds__(256) k_frame_cluster(View base, const FrameOp* ops, int nops, float4* buf0,
                                                        const int2* bend_ranges, int K, int cap) {
    extern __shared__ float4 sm[];
    cgx::cluster_group cluster = cgx::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int r = (int)cluster.block_rank();
    const int k = (int)(blockIdx.x / C);
    if (k >= K) return;  // uniform over the cluster
    const Params& P = base.P[k];
    const int v0 = P.vstart, n = P.V;
    const int chunk = (n + C - 1) / C;
    const int lo = min(r * chunk, n), hi = min(lo + chunk, n);
    float4* s0 = sm;
    float4* s1 = sm + cap;
    float4* sprev = sm + 2 * cap;
    float4* svel = sm + 3 * cap;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s0[i] = buf0[v0 + i];
        sprev[i] = base.prev[v0 + i];
        svel[i] = base.vel[v0 + i];
    }
    cluster.sync();  // every copy is complete before any CTA writes into another
    View v = base;
    v.prev = sprev - v0;
    v.vel = svel - v0;
    float4* b0 = s0 - v0;
    float4* b1 = s1 - v0;
    for (int o = 0; o < nops; ++o) {
        const FrameOp op = ops[o];
        v.pos_in = op.in_buf ? b1 : b0;
        v.pos = op.out_buf ? b1 : b0;
        v.substep = op.substep;
        v.last_it = op.last_it;
        if (op.kind == 2) {
            // every CTA applies the colour to its copy; one of them counts
            View bv = v;
            if (r != 0) bv.counts = nullptr;
            const int2 rg = bend_ranges[op.color * K + k];
            for (int b = rg.x + (int)threadIdx.x; b < rg.x + rg.y; b += blockDim.x) bend_item(bv, b);
        } else {
            for (int i = v0 + lo + (int)threadIdx.x; i < v0 + hi; i += blockDim.x) {
                if (op.kind == 0)
                    predict_item(v, i);
                else if (op.kind == 1)
                    vertex_pass_item(v, i, op.flags);
                else
                    v.pos[i] = v.pos_in[i];
            }
            __syncthreads();
            // the own slice of the written arrays into every other copy
            const int out = op.out_buf ? 1 : 0;
            const bool state = op.kind != 3;
            for (int q = 1; q < C; ++q) {
                const int dst = (r + q) % C;
                float4* rem = cluster.map_shared_rank(sm, dst);
                for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
                    rem[out * cap + i] = sm[out * cap + i];
                    if (state) {
                        rem[2 * cap + i] = sprev[i];
                        rem[3 * cap + i] = svel[i];
                    }
                }
            }
        }
        cluster.sync();
    }
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
        buf0[v0 + i] = s0[i];
        base.prev[v0 + i] = sprev[i];
        base.vel[v0 + i] = svel[i];
    }
}

// cluster > 1: one cluster of that many CTAs per cloth (block threads each)
void launch_frame_cluster(const View& v, const FrameOp* ops, int nops, float4* buf0, const int2* bend_ranges, int K, int cap,
                          int cluster, int block, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_frame_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 1024 * (int)sizeof(float4));
        configured = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(K * cluster), 1, 1);
    cfg.blockDim = dim3((unsigned)block, 1, 1);
    cfg.dynamicSmemBytes = (size_t)4 * cap * sizeof(float4);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (K > 0) cudaLaunchKernelEx(&cfg, k_frame_cluster, v, ops, nops, buf0, bend_ranges, K, cap);
}

void launch_frame_fused(const View& v, const FrameOp* ops, int nops, float4* buf0, float4* buf1, const int2* bend_ranges,
                        int K, int block, cudaStream_t s) {
    (void)buf1;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_frame_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 1024 * (int)sizeof(float4));
        configured = true;
    }
    const size_t smem = (size_t)4 * block * sizeof(float4);
    if (K > 0) k_frame_fused<<<K, block, smem, s>>>(v, ops, nops, buf0, bend_ranges, K);
}

void launch_predict(const View& v, int V, cudaStream_t s) {
    const int b = tune_of(v.tune, kTuneVertexBlock);
    if (V > 0) k_predict<<<grid_for(V, b), b, 0, s>>>(v);
}

void launch_vertex_pass(const View& v, int V, unsigned flags, cudaStream_t s) {
    const int b = tune_of(v.tune, kTuneVertexBlock);
    if (V > 0) k_vertex_pass<<<grid_for(V, b), b, 0, s>>>(v, flags);
}

void launch_bend_color(const View& v, int start, int count, cudaStream_t s) {
    const int b = tune_of(v.tune, kTuneVertexBlock);
    if (count > 0) k_bend_color<<<grid_for(count, b), b, 0, s>>>(v, start, count);
}

void launch_pin_scatter(const int* idx, const float4* target, const float* weight, const float* relax, int n,
                        float4* pin_target, float* pin_weight, float* pin_relax, int nV, cudaStream_t s) {
    if (n > 0) k_pin_scatter<<<blocks_for(n), kThreads, 0, s>>>(idx, target, weight, relax, n, pin_target, pin_weight, pin_relax, nV);
}

void launch_copy_pos(float4* dst, const float4* src, int V, cudaStream_t s) {
    if (V > 0) k_copy_pos<<<blocks_for(V), kThreads, 0, s>>>(dst, src, V);
}

void launch_pack_positions(float* dst, const float4* src, int V, cudaStream_t s) {
    if (V > 0) k_pack_positions<<<blocks_for(V), kThreads, 0, s>>>(dst, src, V);
}

}  // namespace xg
