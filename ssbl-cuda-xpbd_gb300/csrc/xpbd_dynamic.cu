// Dynamic colliders: moving triangle meshes (plain triangles, unsigned
// response; indexed meshes, signed response) and particles, uploaded each
// frame (native/src/ssbl_xpbd_cuda_abi41.cu:8333-8696 uploads, 6220-6449
// hashes, 3592-4540 queries and responses).
//
// The reference builds the collider hashes on every step with a host prefix
// sum between two kernels (a device-to-host round trip per step) and fills
// buckets in atomic arrival order, so the candidate order — which decides
// ties of the closest / deepest contact and the order of the signed
// response's weighted average — changes from run to run.  Here the hashes
// are built once per upload, entirely on the device (count, scan, scatter,
// then each bucket sorted by id), and every query walks its candidates in
// increasing id order: the same contacts in the same order on every run.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "xpbd_contact.cuh"
#include "xpbd_host.cuh"

namespace xg {

namespace {

constexpr int kThreadsDyn = 128;
inline int dyn_blocks(int n) { return (n + kThreadsDyn - 1) / kThreadsDyn; }

constexpr int kTriHashMin = 64;         // abi41.cu:39
constexpr int kParHashMin = 128;        // abi41.cu:25
constexpr int kParSlots = 16;           // abi41.cu:26
constexpr int kDynMaxCells = 64;        // abi41.cu:79
constexpr float kNeighborImpulse = 0.5f;

// ------------------------------------------------------------ bounds / hash

// Per triangle: bounds, centre, radius and (hashed meshes) the cell span of
// the bounds grown by the collision margin; an invalid span collapses to
// the centre's cell (abi41.cu:3686-3760).
__global__ void k_dyn_bounds(const float4* tris, int T, float cell, float margin, bool spans, int ieee, float4* amin,
                             float4* amax, float4* center, float* radius, int4* cmin, int4* cmax) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const F3 a = f3(tris[3 * t]), b = f3(tris[3 * t + 1]), c = f3(tris[3 * t + 2]);
    const F3 lo{fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z))};
    const F3 hi{fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z))};
    const F3 ce = (a + b + c) * (1.0f / 3.0f);
    const F3 da = a - ce, db = b - ce, dc = c - ce;
    const float r = sqrtf(fmaxf(fmaxf(dot3(da, da), dot3(db, db)), dot3(dc, dc)));
    amin[t] = f4(lo, 0.0f);
    amax[t] = f4(hi, 0.0f);
    center[t] = f4(ce, 0.0f);
    radius[t] = r;
    if (!spans) return;
    const float cs = fmaxf(cell, 1.0e-3f);
    int x0 = cell_of(lo.x - margin, cs, ieee), y0 = cell_of(lo.y - margin, cs, ieee), z0 = cell_of(lo.z - margin, cs, ieee);
    int x1 = cell_of(hi.x + margin, cs, ieee), y1 = cell_of(hi.y + margin, cs, ieee), z1 = cell_of(hi.z + margin, cs, ieee);
    const long long sx = (long long)x1 - x0 + 1, sy = (long long)y1 - y0 + 1, sz = (long long)z1 - z0 + 1;
    if (!(sx > 0 && sy > 0 && sz > 0)) {
        x0 = x1 = cell_of(ce.x, cs, ieee);
        y0 = y1 = cell_of(ce.y, cs, ieee);
        z0 = z1 = cell_of(ce.z, cs, ieee);
    }
    cmin[t] = make_int4(x0, y0, z0, 0);
    cmax[t] = make_int4(x1, y1, z1, 0);
}

__device__ __forceinline__ long long span_cells(int4 a, int4 b) {
    const long long sx = (long long)b.x - a.x + 1, sy = (long long)b.y - a.y + 1, sz = (long long)b.z - a.z + 1;
    return (sx > 0 && sy > 0 && sz > 0) ? sx * sy * sz : 0;
}

// Count (scatter = false) or place (scatter = true) every cell of every
// triangle; a triangle over 64 cells is flagged for the large list instead
// (abi41.cu:3763-3930).  `occupancy` receives the largest bucket count.
__global__ void k_dyn_tri_hash(int T, const int4* cmin, const int4* cmax, int nb, int* cnt, int* ent, bool scatter,
                               int* large_flag, int* occupancy) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int4 a = cmin[t], b = cmax[t];
    const long long cells = span_cells(a, b);
    if (!scatter) large_flag[t] = cells > kDynMaxCells ? 1 : 0;
    if (cells <= 0 || cells > kDynMaxCells) return;
    for (int z = a.z; z <= b.z; ++z)
        for (int y = a.y; y <= b.y; ++y)
            for (int x = a.x; x <= b.x; ++x) {
                int* c = &cnt[bucket_of(x, y, z, nb)];
                const int slot = atomicAdd(c, 1);
                if (scatter)
                    ent[slot] = t;
                else
                    atomicMax(occupancy, slot + 1);
            }
}

// Large triangles in increasing id order: `pos` is the exclusive scan of
// the large flags.
__global__ void k_dyn_large_list(int T, const int4* cmin, const int4* cmax, const int* pos, int* large) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    if (span_cells(cmin[t], cmax[t]) > kDynMaxCells) large[pos[t]] = t;
}

// Particle cells and bucket counts / placement.
__global__ void k_dyn_par_hash(const float4* pos, int n, float cell, int nb, int ieee, int4* cellc, int* cnt, int* ent,
                               bool scatter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const int cx = cell_of(p.x, cell, ieee), cy = cell_of(p.y, cell, ieee), cz = cell_of(p.z, cell, ieee);
    int* c = &cnt[bucket_of(cx, cy, cz, nb)];
    if (scatter) {
        ent[atomicAdd(c, 1)] = i;
    } else {
        cellc[i] = make_int4(cx, cy, cz, 0);
        atomicAdd(c, 1);
    }
}

// Sort each bucket's members by id (shell sort in place; buckets are small).
__global__ void k_dyn_sort_buckets(const int* start, int* ent, int nb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int s = start[b], n = start[b + 1] - s;
    int* e = ent + s;
    for (int gap = n / 2; gap > 0; gap /= 2)
        for (int i = gap; i < n; ++i) {
            const int x = e[i];
            int j = i;
            while (j >= gap && e[j - gap] > x) {
                e[j] = e[j - gap];
                j -= gap;
            }
            e[j] = x;
        }
}

// Particles past the 16 queried per bucket (the reference counts one
// overflow per insertion into a full bucket, abi41.cu:4350).
__global__ void k_dyn_overflow(const int* start, int nb, unsigned long long* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int n = start[b + 1] - start[b];
    if (n > kParSlots) atomicAdd(out, (unsigned long long)(n - kParSlots));
}

// Indexed mesh: triangle rows from the vertex and index arrays; an index
// out of range gives a degenerate triangle at the origin (abi41.cu:3663-3684).
__global__ void k_dyn_from_indices(const float4* verts, int nv, const int* idx, int T, float4* tris) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
    if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv) {
        tris[3 * t] = tris[3 * t + 1] = tris[3 * t + 2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    tris[3 * t] = verts[a];
    tris[3 * t + 1] = verts[b];
    tris[3 * t + 2] = verts[c];
}

// ----------------------------------------------------------------- queries

struct DynBest {
    F3 delta, velocity, acc;
    float penetration, distance, acc_w;
};

__device__ __forceinline__ float point_box_sq(F3 p, F3 lo, F3 hi) {
    const F3 q{fminf(fmaxf(p.x, lo.x), hi.x), fminf(fmaxf(p.y, lo.y), hi.y), fminf(fmaxf(p.z, lo.z), hi.z)};
    const F3 d = p - q;
    return dot3(d, d);
}

// Source filter of the shared scene (abi41.cu:3984-3997): the target's own
// source is skipped, and mode 2 keeps only lower collision layers.
__device__ __forceinline__ bool source_enabled(const Params& P, int source, int layer) {
    if (P.gd_mode == 0) return true;
    if (P.gd_target_source != 0 && source == P.gd_target_source) return false;
    if (P.gd_mode == 2) return layer < P.gd_target_layer;
    return true;
}

// One candidate triangle (abi41.cu:3998-4111).
__device__ void dyn_tri_candidate(const Params& P, const DynSet& D, int t, F3 p, float collider_dt, bool inside, float qm, float cm,
                                  DynBest* b, unsigned* candidates, unsigned* rejects) {
    if (t < 0 || t >= D.tri_count) return;
    if (D.tri_src && !source_enabled(P, D.tri_src[t], D.tri_layer ? D.tri_layer[t] : 0)) return;
    *candidates += 1;
    if (point_box_sq(p, f3(D.amin[t]), f3(D.amax[t])) > qm * qm) {
        *rejects += 1;
        return;
    }
    const F3 dc = p - f3(D.center[t]);
    const float rr = D.radius[t] + qm;
    if (dot3(dc, dc) > rr * rr) {
        *rejects += 1;
        return;
    }
    const F3 a = f3(D.tris[3 * t]), bb = f3(D.tris[3 * t + 1]), c = f3(D.tris[3 * t + 2]);
    const F3 q = closest_on_triangle(p, a, bb, c);
    const F3 d = p - q;
    const float dsq = dot3(d, d);
    const float dist = sqrtf(fmaxf(dsq, kEps));
    const F3 tn = cross3(bb - a, c - a);
    const float tl = sqrtf(fmaxf(dot3(tn, tn), kEps));
    const F3 tri_normal = tn * (1.0f / tl);
    F3 normal = dsq > kEps * 4.0f ? d * (1.0f / fmaxf(dist, kEps)) : tri_normal;
    float pen = cm - dist;
    if (D.signed_mode) {
        const float sd = dot3(d, tri_normal);
        if (inside) {
            const float target = 0.001f;
            if (sd >= target) return;
            pen = target - sd;
        } else {
            pen = cm - sd;
        }
        normal = tri_normal;
        if (pen <= 0.0f) return;
        const F3 delta = normal * pen;
        if (!inside && finite3(delta)) {
            const float w = fmaxf(pen, kEps);
            b->acc = b->acc + delta * w;
            b->acc_w += w;
        }
        if (dist < b->distance) {
            F3 vel{0.0f, 0.0f, 0.0f};
            if (D.motion_valid && collider_dt > kEps) vel = (f3(D.center[t]) - f3(D.prev_center[t])) * (1.0f / collider_dt);
            b->distance = dist;
            b->penetration = pen;
            b->delta = delta;
            b->velocity = vel;
        }
    } else {
        if (dist >= cm) return;
        if (pen > b->penetration) {
            b->penetration = pen;
            b->delta = normal * pen;
        }
    }
}

// Signed response of a vertex (abi41.cu:991-1065): relaxed, capped
// projection along the contact normal; the collider's normal velocity is
// kept, the relative velocity loses its inward part (inside-only) or gets
// the static-contact friction response with the outward part retained at
// one eighth.
__device__ void signed_response(const View& v, const Params& P, int i, F3 p, F3 raw, F3 collider_vel, float proxy, float dt,
                                bool inside) {
    if (!finite3(p) || !finite3(raw)) return;
    const float rl = len3(raw);
    if (!isfinite(rl) || rl <= kEps) return;
    const F3 n = raw * (1.0f / rl);
    F3 applied = raw * (1.0f / 3.0f);
    const float basis = fmaxf(fmaxf(P.thickness, 0.0f), fmaxf(P.margin, 0.0f));
    const float cap = inside ? fmaxf(3.0e-3f, basis * 16.0f) : fmaxf(5.0e-4f, basis * 3.0f);
    applied = limit_delta(applied, cap);
    const float al = len3(applied);
    if (!isfinite(al) || al <= kEps) return;
    const float sdt = fmaxf(dt, kEps);
    const F3 corrected = p + applied;
    F3 vel = f3(v.vel[i]);
    F3 base{0.0f, 0.0f, 0.0f};
    if (finite3(collider_vel)) {
        const float cn = dot3(collider_vel, n);
        if (isfinite(cn)) base = n * cn;
    }
    if (inside) {
        if (!finite3(vel)) vel = F3{0.0f, 0.0f, 0.0f};
        F3 rel = vel - base;
        const float ns = dot3(rel, n);
        if (isfinite(ns) && ns < 0.0f) {
            rel = rel - n * ns;
            vel = base + rel;
        }
    } else {
        F3 rel = vel - base;
        const float inward = fmaxf(-dot3(rel, n), 0.0f);
        const float depth = fmaxf(fmaxf(proxy, rl), al);
        contact_response(P, v.counts, n, inward + depth / sdt, &rel);
        const float out = dot3(rel, n);
        if (out > 0.0f) rel = rel - n * (out * (1.0f - 1.0f / 8.0f));
        vel = base + rel;
    }
    if (!finite3(vel)) vel = F3{0.0f, 0.0f, 0.0f};
    const float w = v.pos[i].w;
    v.pos[i] = f4(corrected, w);
    v.vel[i] = f4(vel, 0.0f);
    v.prev[i] = f4(corrected - vel * sdt, 0.0f);
}

__device__ __forceinline__ F3 local_average(F3 acc, float w, F3 fallback) {
    if (w > 0.0f && finite3(acc)) {
        const F3 avg = acc * (1.0f / w);
        const float al = len3(avg), fl = len3(fallback);
        if (finite3(avg) && isfinite(al) && isfinite(fl) && al > kEps && fl > kEps) return avg * (fl / al);
    }
    return fallback;
}

__device__ __forceinline__ void warp_count(unsigned long long* counts, int slot, unsigned value) {
    const unsigned mask = __activemask();
    const unsigned total = __reduce_add_sync(mask, value);
    if ((threadIdx.x & 31) == (__ffs(mask) - 1) && total) count_add(counts, slot, total);
}

// Triangle contact of one vertex (abi41.cu:4247-4323).
__device__ void dyn_triangles(const View& v, const Params& P, const DynSet& D, int i, bool inside) {
    const float sub_dt = P.sub_dt;
    const float collider_dt = (isfinite(P.frame_dt) && P.frame_dt > kEps) ? P.frame_dt : fmaxf(sub_dt, kEps);
    float cm = fmaxf(P.margin, 0.0f);
    if (D.signed_mode) cm = fmaxf(cm, fmaxf(P.thickness, 0.0f) * 0.75f);
    float qm = cm;
    if (D.signed_mode) {
        const float animated = fmaxf(fmaxf(cm * 2.0f, 0.04f), fmaxf(D.tri_cell, 0.0f) * 1.25f);
        qm = fminf(fmaxf(animated, cm), 0.08f);
    }
    if (cm <= 0.0f || qm <= 0.0f) return;
    const F3 p = f3(v.pos[i]);
    DynBest b{F3{0.0f, 0.0f, 0.0f}, F3{0.0f, 0.0f, 0.0f}, F3{0.0f, 0.0f, 0.0f}, 0.0f, 3.402823466e+38f, 0.0f};
    unsigned candidates = 0, rejects = 0;
    if (D.tri_hashed) {
        const int cx = cell_of(p.x, D.tri_cell, D.key_ieee), cy = cell_of(p.y, D.tri_cell, D.key_ieee),
                  cz = cell_of(p.z, D.tri_cell, D.key_ieee);
        int R = 0;
        if (D.signed_mode) {
            if (!inside) {
                R = 1;
            } else {
                const float cs = fmaxf(D.tri_cell, 1.0e-3f);
                R = min(max((int)ceilf(fmaxf(qm, 0.0f) / cs), 1), 4);
            }
        }
        for (int dz = -R; dz <= R; ++dz)
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx) {
                    const int qx = cx + dx, qy = cy + dy, qz = cz + dz;
                    const unsigned bk = bucket_of(qx, qy, qz, D.tri_buckets);
                    const int s0 = D.tstart[bk], s1 = max(D.tstart[bk + 1], s0);
                    for (int k = s0; k < s1; ++k) {
                        const int t = D.tent[k];
                        if (t < 0 || t >= D.tri_count) continue;
                        // each triangle once: in the cell of its span nearest the vertex's cell
                        const int4 lo = D.cmin[t], hi = D.cmax[t];
                        if (qx != min(max(cx, lo.x), hi.x) || qy != min(max(cy, lo.y), hi.y) || qz != min(max(cz, lo.z), hi.z))
                            continue;
                        dyn_tri_candidate(P, D, t, p, collider_dt, inside, qm, cm, &b, &candidates, &rejects);
                    }
                }
        for (int k = 0; k < D.large_count; ++k) dyn_tri_candidate(P, D, D.large[k], p, collider_dt, inside, qm, cm, &b, &candidates, &rejects);
    } else {
        for (int t = 0; t < D.tri_count; ++t) dyn_tri_candidate(P, D, t, p, collider_dt, inside, qm, cm, &b, &candidates, &rejects);
    }
    warp_count(v.counts, kCntDynTriCandidates, candidates);
    warp_count(v.counts, kCntDynTriAabbRejects, rejects);
    if (!(b.penetration > 0.0f)) return;
    count1(v.counts, kCntTrianglePairs);
    if (D.signed_mode) {
        signed_response(v, P, i, p, local_average(b.acc, b.acc_w, b.delta), b.velocity, b.penetration, sub_dt, inside);
    } else {
        const F3 applied = b.delta * kNeighborImpulse;
        const F3 np = p + applied;
        F3 vel = f3(v.vel[i]);
        const float vn = dot3(vel, applied);
        if (vn < 0.0f) {
            const float l2 = fmaxf(dot3(applied, applied), kEps);
            vel = vel - applied * (kNeighborImpulse * vn / l2);
        }
        const float w = v.pos[i].w;
        v.pos[i] = f4(np, w);
        v.vel[i] = f4(vel, 0.0f);
        v.prev[i] = f4(np - vel * fmaxf(sub_dt, kEps), 0.0f);
    }
    count1(v.counts, kCntExactImpulseContacts);
}

// Particle contact of one vertex (abi41.cu:4354-4511).
__device__ void dyn_particles(const View& v, const Params& P, const DynSet& D, int i) {
    const float sub_dt = P.sub_dt;
    const float collider_dt = (isfinite(P.frame_dt) && P.frame_dt > kEps) ? P.frame_dt : fmaxf(sub_dt, kEps);
    const F3 p = f3(v.pos[i]);
    const float margin = fmaxf(P.margin, 0.0f);
    F3 best_delta{0.0f, 0.0f, 0.0f}, best_vel{0.0f, 0.0f, 0.0f}, acc{0.0f, 0.0f, 0.0f};
    float best = 0.0f, acc_w = 0.0f;
    unsigned candidates = 0;
    auto consider = [&](int k) {
        if (k < 0 || k >= D.par_count) return;
        if (D.par_src && !source_enabled(P, D.par_src[k], D.par_layer ? D.par_layer[k] : 0)) return;
        const F3 c = f3(D.par_pos[k]);
        const float r = fmaxf(D.par_radius[k], 0.0f) + margin;
        if (r <= 0.0f) return;
        const F3 d = p - c;
        const float dist = sqrtf(fmaxf(dot3(d, d), kEps));
        if (dist >= r) return;
        candidates += 1;
        const F3 n = dist > kEps ? d * (1.0f / dist) : F3{0.0f, 0.0f, 1.0f};
        const float pen = r - dist;
        const F3 delta = n * pen;
        if (D.signed_mode && finite3(delta)) {
            const float w = fmaxf(pen, kEps);
            acc = acc + delta * w;
            acc_w += w;
        }
        if (pen > best) {
            F3 pv{0.0f, 0.0f, 0.0f};
            if (D.par_motion_valid && collider_dt > kEps) pv = (c - f3(D.par_prev[k])) * (1.0f / collider_dt);
            best = pen;
            best_delta = delta;
            best_vel = pv;
        }
    };
    if (D.par_hashed) {
        const int cx = cell_of(p.x, D.par_cell, D.key_ieee), cy = cell_of(p.y, D.par_cell, D.key_ieee),
                  cz = cell_of(p.z, D.par_cell, D.key_ieee);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int qx = cx + dx, qy = cy + dy, qz = cz + dz;
                    const unsigned bk = bucket_of(qx, qy, qz, D.par_buckets);
                    const int s0 = D.pstart[bk], n = min(D.pstart[bk + 1] - s0, kParSlots);
                    for (int s = 0; s < n; ++s) {
                        const int k = D.pent[s0 + s];
                        const int4 kc = D.par_cellc[k];
                        if (kc.x != qx || kc.y != qy || kc.z != qz) continue;
                        consider(k);
                    }
                }
    } else {
        for (int k = 0; k < D.par_count; ++k) consider(k);
    }
    warp_count(v.counts, kCntDynParCandidates, candidates);
    if (!(best > 0.0f)) return;
    if (D.signed_mode) {
        signed_response(v, P, i, p, local_average(acc, acc_w, best_delta), best_vel, best, sub_dt, false);
    } else {
        const float w = v.pos[i].w;
        v.pos[i] = f4(p + best_delta * kNeighborImpulse, w);
    }
    count1(v.counts, kCntExactImpulseContacts);
    count1(v.counts, kCntDynParContacts);
}

// which: 0 unsigned meshes (triangles then particles), 1 signed meshes
// (triangles then particles, outside contacts), 2 signed meshes inside-only.
__global__ void __launch_bounds__(kMaxBlock) k_dynamic(View v, int which) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nV) return;
    const Params& P = params_v(v, i);
    if (!P.active) return;
    // the unsigned stage reads the shared scene when one is attached, else
    // the cloth's own unsigned colliders; the signed stages read the cloth's
    // own indexed mesh (abi41.cu:9234-9360)
    const DynSet* Dp = nullptr;
    if (which == 0)
        Dp = (P.gd_mode != 0 && P.gdyn) ? P.gdyn : ((P.dyn && !P.dyn->signed_mode) ? P.dyn : nullptr);
    else
        Dp = (P.dyn && P.dyn->signed_mode) ? P.dyn : nullptr;
    if (!Dp) return;
    if (__ldg(&v.inv_mass[i]) <= 0.0f) return;
    const DynSet& D = *Dp;
    if (D.tri_count > 0) dyn_triangles(v, P, D, i, which == 2);
    if (which != 2 && D.par_count > 0) dyn_particles(v, P, D, i);
}

}  // namespace

void launch_dynamic_collision(const View& v, int V, int which, cudaStream_t s) {
    const int b = tune_of(v.tune, kTuneDynamicBlock);
    if (V > 0) k_dynamic<<<grid_for(V, b), b, 0, s>>>(v, which);
}

namespace host {

namespace {

// Where an upload allocates and launches: the owner's stream and device byte
// account, and the margin / thickness that size the hash cells and spans
// (the cloth's configuration, or a shared scene's own values).
struct DynCtx {
    cudaStream_t st;
    long long* bytes;
    float margin;
    float thickness;
    int key_ieee;  // cell-key division of the hashes built
};

DynCtx cloth_ctx(Solver* S, int k) {
    const SsblXpbdConfig& c = S->cl[k].cfg;
    return DynCtx{S->stream, &S->device_bytes, std::max(c.collision_margin, 0.0f), std::max(c.cloth_thickness, 0.0f),
                  S->key_ieee};
}

// (Re)allocate a device array of at least n elements; the old contents are
// dropped.  Work in flight on the owner's stream is finished first.
template <class T>
bool realloc_dev(const DynCtx& c, T** p, size_t old_n, size_t n, const char* what) {
    if (*p) {
        if (!cuda_ok(cudaStreamSynchronize(c.st), what)) return false;
        cudaFree(*p);
        *c.bytes -= (long long)(sizeof(T) * old_n);
        *p = nullptr;
    }
    return dalloc(p, std::max<size_t>(n, 1), what);
}

// Cell size of a triangle source (abi41.cu:8319-8331): the largest triangle
// extent plus two margins for plain meshes; finer for indexed meshes and the
// shared scene.
float tri_cell_size(float max_extent, float margin, float thickness, bool fine_cells) {
    const float extent_cell = std::max(std::max(max_extent + margin * 2.0f, thickness), 1.0e-3f);
    if (!fine_cells) return extent_cell;
    const float fine = std::max(std::max(thickness * 1.5f, margin * 4.0f), 0.02f);
    return std::max(std::min(extent_cell, fine), 1.0e-3f);
}

float tri_extent(const float* a, const float* b, const float* c) {
    const float lx = std::min(a[0], std::min(b[0], c[0])), hx = std::max(a[0], std::max(b[0], c[0]));
    const float ly = std::min(a[1], std::min(b[1], c[1])), hy = std::max(a[1], std::max(b[1], c[1]));
    const float lz = std::min(a[2], std::min(b[2], c[2])), hz = std::max(a[2], std::max(b[2], c[2]));
    return std::max(hx - lx, std::max(hy - ly, hz - lz));
}

float rows_max_extent(const float* tris, int count) {
    float m = 0.0f;
    for (int t = 0; t < count; ++t) {
        const float e = tri_extent(tris + 9 * t, tris + 9 * t + 3, tris + 9 * t + 6);
        if (std::isfinite(e) && e >= 0.0f) m = std::max(m, e);
    }
    return m;
}

// Bounds, cell spans and (>= 64 triangles) the hash of the triangles whose
// rows are in D.tris (abi41.cu:3686-3760, 6220-6392).
bool finish_triangles(const DynCtx& c, DynHost& D, int T, bool signed_mode, bool motion_valid, float cell) {
    cudaStream_t st = c.st;
    const bool hashed = T >= kTriHashMin;
    if (T > D.bounds_cap) {
        const size_t o = (size_t)D.bounds_cap, n = (size_t)T;
        if (!realloc_dev(c, &D.amin, o, n, "dynamic triangle bounds") || !realloc_dev(c, &D.amax, o, n, "dynamic triangle bounds") ||
            !realloc_dev(c, &D.center, o, n, "dynamic triangle bounds") ||
            !realloc_dev(c, &D.prev_center, o, n, "dynamic triangle bounds") ||
            !realloc_dev(c, &D.radius, o, n, "dynamic triangle bounds") || !realloc_dev(c, &D.cmin, o, n, "dynamic triangle cells") ||
            !realloc_dev(c, &D.cmax, o, n, "dynamic triangle cells") || !realloc_dev(c, &D.large, o, n, "dynamic triangle large list") ||
            !realloc_dev(c, &D.lflag, o, n, "dynamic triangle large list") ||
            !realloc_dev(c, &D.lpos, o + 1, n + 1, "dynamic triangle large list"))
            return false;
        D.bounds_cap = T;
    }
    if (!D.small && !dalloc(&D.small, 4, "dynamic triangle hash")) return false;
    if (motion_valid &&
        !cuda_ok(cudaMemcpyAsync(D.prev_center, D.center, sizeof(float4) * T, cudaMemcpyDeviceToDevice, st), "keep dynamic centres"))
        return false;
    k_dyn_bounds<<<dyn_blocks(T), kThreadsDyn, 0, st>>>(D.tris, T, cell, c.margin, hashed, c.key_ieee, D.amin, D.amax, D.center,
                                                         D.radius, D.cmin, D.cmax);
    if (!motion_valid &&
        !cuda_ok(cudaMemcpyAsync(D.prev_center, D.center, sizeof(float4) * T, cudaMemcpyDeviceToDevice, st), "init dynamic centres"))
        return false;
    DynSet& h = D.h;
    h.key_ieee = c.key_ieee;
    h.tri_count = T;
    h.signed_mode = signed_mode ? 1 : 0;
    h.motion_valid = motion_valid ? 1 : 0;
    h.tri_hashed = hashed ? 1 : 0;
    h.tri_cell = cell;
    h.tri_buckets = 0;
    h.large_count = 0;
    D.large_count = 0;
    D.max_occupancy = 0;
    if (hashed) {
        const int nb = next_pow2(std::max(1024, T * 4));
        if (nb > D.tb_cap) {
            const size_t o = (size_t)D.tb_cap;
            if (!realloc_dev(c, &D.tcount, o, (size_t)nb, "dynamic triangle hash") ||
                !realloc_dev(c, &D.tstart, o + 1, (size_t)nb + 1, "dynamic triangle hash") ||
                !realloc_dev(c, &D.scan_tmp, o / 4096 + 2, (size_t)nb / 4096 + 2, "dynamic triangle hash"))
                return false;
            D.tb_cap = nb;
        }
        if (!cuda_ok(cudaMemsetAsync(D.tcount, 0, sizeof(int) * nb, st), "reset dynamic triangle hash") ||
            !cuda_ok(cudaMemsetAsync(D.small, 0, sizeof(int) * 4, st), "reset dynamic triangle hash"))
            return false;
        k_dyn_tri_hash<<<dyn_blocks(T), kThreadsDyn, 0, st>>>(T, D.cmin, D.cmax, nb, D.tcount, nullptr, false, D.lflag, D.small);
        scan_bucket_counts(D.tcount, D.tstart, nb, D.scan_tmp, st);
        scan_bucket_counts(D.lflag, D.lpos, T, D.scan_tmp, st);  // T <= nb / 4: the block sums fit
        int got[3] = {0, 0, 0};
        if (!cuda_ok(cudaMemcpyAsync(&got[0], D.tstart + nb, sizeof(int), cudaMemcpyDeviceToHost, st), "dynamic triangle hash") ||
            !cuda_ok(cudaMemcpyAsync(&got[1], D.lpos + T, sizeof(int), cudaMemcpyDeviceToHost, st), "dynamic triangle hash") ||
            !cuda_ok(cudaMemcpyAsync(&got[2], D.small, sizeof(int), cudaMemcpyDeviceToHost, st), "dynamic triangle hash") ||
            !cuda_ok(cudaStreamSynchronize(st), "dynamic triangle hash"))
            return false;
        if (got[0] > D.tent_cap) {
            if (!realloc_dev(c, &D.tent, (size_t)D.tent_cap, (size_t)got[0], "dynamic triangle hash")) return false;
            D.tent_cap = got[0];
        }
        k_dyn_tri_hash<<<dyn_blocks(T), kThreadsDyn, 0, st>>>(T, D.cmin, D.cmax, nb, D.tcount, D.tent, true, nullptr, nullptr);
        k_dyn_large_list<<<dyn_blocks(T), kThreadsDyn, 0, st>>>(T, D.cmin, D.cmax, D.lpos, D.large);
        k_dyn_sort_buckets<<<dyn_blocks(nb), kThreadsDyn, 0, st>>>(D.tstart, D.tent, nb);
        h.tri_buckets = nb;
        h.large_count = got[1];
        D.large_count = got[1];
        D.max_occupancy = got[2];
    }
    h.tris = D.tris;
    h.amin = D.amin;
    h.amax = D.amax;
    h.center = D.center;
    h.prev_center = D.prev_center;
    h.radius = D.radius;
    h.cmin = D.cmin;
    h.cmax = D.cmax;
    h.tstart = D.tstart;
    h.tent = D.tent;
    h.large = D.large;
    return cuda_ok(cudaGetLastError(), "dynamic triangle hash");
}

// Plain triangle rows (9 floats each) into D.tris.
bool put_rows(const DynCtx& c, DynHost& D, const float* tris, int count) {
    if (count > D.tris_cap) {
        if (!realloc_dev(c, &D.tris, (size_t)D.tris_cap * 3, (size_t)count * 3, "dynamic triangle upload")) return false;
        D.tris_cap = count;
    }
    std::vector<float4> rows((size_t)count * 3);
    for (int q = 0; q < count * 3; ++q) rows[q] = make_float4(tris[3 * q], tris[3 * q + 1], tris[3 * q + 2], 0.0f);
    return dupload(D.tris, rows.data(), rows.size(), c.st, "dynamic triangle upload");
}

void clear_triangles(DynHost& D) {
    D.h.tri_count = 0;
    D.h.signed_mode = 0;
    D.h.motion_valid = 0;
    D.h.tri_hashed = 0;
    D.h.large_count = 0;
    D.tri_upload_count = 0;
    D.large_count = 0;
    D.max_occupancy = 0;
}

void clear_particles(DynHost& D) {
    D.h.par_count = 0;
    D.h.par_motion_valid = 0;
    D.h.par_hashed = 0;
    D.par_upload_count = 0;
    D.radius_signature = 0;
}

// Particles (abi41.cu:8566-8696, 6595-6665 for the shared scene; hash
// 6395-6449).  prev: the previous positions given by the caller (the shared
// scene), or null to keep the last upload's positions as previous.
bool put_particles(const DynCtx& c, DynHost& D, const float* pos, const float* prev, const float* radii, int count,
                   unsigned long long* overflow_out) {
    uint64_t sig = 1469598103934665603ull ^ (uint64_t)count;
    float max_r = 0.0f;
    std::vector<float4> p4(count), q4;
    for (int q = 0; q < count; ++q) {
        float r = std::isfinite(radii[q]) ? radii[q] : 0.0f;
        r = std::max(r, 0.0f);
        max_r = std::max(max_r, r);
        uint32_t bits;
        std::memcpy(&bits, &r, 4);
        sig ^= (uint64_t)bits;
        sig *= 1099511628211ull;
        p4[q] = make_float4(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], 0.0f);
    }
    DynSet& h = D.h;
    cudaStream_t st = c.st;
    if (h.par_cell <= 0.0f || D.radius_signature != sig || D.par_upload_count != count) {
        h.par_cell = std::max(std::max(max_r + c.margin, c.thickness), 1.0e-3f);
        D.radius_signature = sig;
    }
    const bool motion = D.par_upload_count == count;
    if (count > D.par_cap) {
        const size_t o = (size_t)D.par_cap, n = (size_t)count;
        if (!realloc_dev(c, &D.ppos, o, n, "dynamic particle upload") || !realloc_dev(c, &D.pprev, o, n, "dynamic particle upload") ||
            !realloc_dev(c, &D.prad, o, n, "dynamic particle upload") || !realloc_dev(c, &D.pcell, o, n, "dynamic particle hash") ||
            !realloc_dev(c, &D.pent, o, n, "dynamic particle hash"))
            return false;
        D.par_cap = count;
    }
    if (prev) {
        q4.resize(count);
        for (int q = 0; q < count; ++q) q4[q] = make_float4(prev[3 * q], prev[3 * q + 1], prev[3 * q + 2], 0.0f);
        if (!dupload(D.pprev, q4.data(), (size_t)count, st, "dynamic particle previous upload")) return false;
    } else if (motion && !cuda_ok(cudaMemcpyAsync(D.pprev, D.ppos, sizeof(float4) * count, cudaMemcpyDeviceToDevice, st),
                                  "keep dynamic particle positions")) {
        return false;
    }
    if (!dupload(D.ppos, p4.data(), (size_t)count, st, "dynamic particle upload") ||
        !dupload(D.prad, radii, (size_t)count, st, "dynamic particle radius upload"))
        return false;
    if (!prev && !motion &&
        !cuda_ok(cudaMemcpyAsync(D.pprev, D.ppos, sizeof(float4) * count, cudaMemcpyDeviceToDevice, st), "init dynamic particle positions"))
        return false;
    h.key_ieee = c.key_ieee;
    h.par_count = count;
    h.par_motion_valid = motion ? 1 : 0;
    h.par_hashed = count >= kParHashMin ? 1 : 0;
    h.par_buckets = 0;
    if (h.par_hashed) {
        const int nb = next_pow2(std::max(1024, count * 4));
        if (nb > D.pb_cap) {
            const size_t o = (size_t)D.pb_cap;
            if (!realloc_dev(c, &D.pcount, o, (size_t)nb, "dynamic particle hash") ||
                !realloc_dev(c, &D.pstart, o + 1, (size_t)nb + 1, "dynamic particle hash") ||
                !realloc_dev(c, &D.pscan, o / 4096 + 2, (size_t)nb / 4096 + 2, "dynamic particle hash"))
                return false;
            D.pb_cap = nb;
        }
        if (!cuda_ok(cudaMemsetAsync(D.pcount, 0, sizeof(int) * nb, st), "reset dynamic particle hash")) return false;
        k_dyn_par_hash<<<dyn_blocks(count), kThreadsDyn, 0, st>>>(D.ppos, count, h.par_cell, nb, c.key_ieee, D.pcell, D.pcount,
                                                                   nullptr, false);
        scan_bucket_counts(D.pcount, D.pstart, nb, D.pscan, st);
        k_dyn_par_hash<<<dyn_blocks(count), kThreadsDyn, 0, st>>>(D.ppos, count, h.par_cell, nb, c.key_ieee, D.pcell, D.pcount,
                                                                   D.pent, true);
        k_dyn_sort_buckets<<<dyn_blocks(nb), kThreadsDyn, 0, st>>>(D.pstart, D.pent, nb);
        if (overflow_out) k_dyn_overflow<<<dyn_blocks(nb), kThreadsDyn, 0, st>>>(D.pstart, nb, overflow_out);
        h.par_buckets = nb;
    }
    h.par_pos = D.ppos;
    h.par_prev = D.pprev;
    h.par_radius = D.prad;
    h.par_cellc = D.pcell;
    h.pstart = D.pstart;
    h.pent = D.pent;
    D.par_upload_count = count;
    return cuda_ok(cudaGetLastError(), "dynamic particle hash");
}

// Copy the descriptor to the device (allocated on first use).
bool publish_set(const DynCtx& c, DynHost& D) {
    if (!D.dev && !dalloc(&D.dev, 1, "dynamic collider descriptor")) return false;
    return dupload(D.dev, &D.h, 1, c.st, "dynamic collider descriptor") && cuda_ok(cudaStreamSynchronize(c.st), "dynamic collider upload");
}

// Point the cloth's parameters at its descriptor (null when it has no
// dynamic collider).
bool publish(Solver* S, int k) {
    DynHost& D = S->cl[k].dyn;
    if (!publish_set(cloth_ctx(S, k), D)) return false;
    const bool any = D.h.tri_count > 0 || D.h.par_count > 0;
    S->hp[k].dyn = any ? D.dev : nullptr;
    S->params_dirty = true;
    return true;
}

void free_set(DynHost& D) {
    void* ptrs[] = {D.tris, D.verts, D.idx, D.amin, D.amax, D.center, D.prev_center, D.radius, D.cmin, D.cmax, D.large, D.lflag,
                    D.lpos, D.tcount, D.tstart, D.tent, D.scan_tmp, D.small, D.ppos, D.pprev, D.prad, D.pcell, D.pcount, D.pstart,
                    D.pent, D.pscan, D.dev};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    D = DynHost{};
}

}  // namespace

void free_dynamic(Cloth& C) { free_set(C.dyn); }

// Plain dynamic triangles (unsigned response), 9 floats per triangle
// (abi41.cu:8333-8413).
bool upload_dynamic_triangles(Solver* S, int cloth, const float* tris, int count) {
    if (!S || cloth >= S->K) return fail("invalid dynamic triangle update");
    count = std::max(count, 0);
    if (count > 0 && !tris) return fail("dynamic triangle data is required when triangle count is nonzero");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    AllocAccount account(&S->device_bytes);
    const float max_extent = rows_max_extent(tris, count);
    for (int k = k0; k < k1; ++k) {
        DynHost& D = S->cl[k].dyn;
        if (count == 0) {
            clear_triangles(D);
            if (!publish(S, k)) return false;
            continue;
        }
        const DynCtx c = cloth_ctx(S, k);
        const bool motion = D.tri_upload_count == count;
        if (!put_rows(c, D, tris, count) ||
            !finish_triangles(c, D, count, false, motion, tri_cell_size(max_extent, c.margin, c.thickness, false)))
            return false;
        D.tri_upload_count = count;
        if (!publish(S, k)) return false;
    }
    return true;
}

// Indexed dynamic mesh (signed response): vertices and index triples
// (abi41.cu:8415-8564).
bool upload_dynamic_indexed(Solver* S, int cloth, const float* verts, int vcount, const int* idx, int count, bool topology_changed) {
    if (!S || cloth >= S->K) return fail("invalid dynamic indexed triangle update");
    vcount = std::max(vcount, 0);
    count = std::max(count, 0);
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    AllocAccount account(&S->device_bytes);
    if (vcount == 0 || count == 0) {
        for (int k = k0; k < k1; ++k) {
            clear_triangles(S->cl[k].dyn);
            if (!publish(S, k)) return false;
        }
        return true;
    }
    if (!verts || !idx) return fail("dynamic indexed triangle positions and indices are required when count is nonzero");
    float max_extent = 0.0f;
    for (int t = 0; t < count; ++t) {
        const int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
        if (a < 0 || b < 0 || c < 0 || a >= vcount || b >= vcount || c >= vcount) continue;
        const float e = tri_extent(verts + 3 * a, verts + 3 * b, verts + 3 * c);
        if (std::isfinite(e) && e >= 0.0f) max_extent = std::max(max_extent, e);
    }
    std::vector<float4> v4(vcount);
    for (int i = 0; i < vcount; ++i) v4[i] = make_float4(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2], 0.0f);
    for (int k = k0; k < k1; ++k) {
        DynHost& D = S->cl[k].dyn;
        const DynCtx cx = cloth_ctx(S, k);
        if (vcount > D.verts_cap) {
            if (!realloc_dev(cx, &D.verts, (size_t)D.verts_cap, (size_t)vcount, "dynamic triangle vertex upload")) return false;
            D.verts_cap = vcount;
        }
        if (!dupload(D.verts, v4.data(), (size_t)vcount, S->stream, "dynamic triangle vertex upload")) return false;
        if (topology_changed || count != D.topology_count || count > D.idx_cap) {
            if (count > D.idx_cap) {
                if (!realloc_dev(cx, &D.idx, (size_t)D.idx_cap * 3, (size_t)count * 3, "dynamic triangle index upload")) return false;
                D.idx_cap = count;
            }
            if (!dupload(D.idx, idx, (size_t)3 * count, S->stream, "dynamic triangle index upload")) return false;
            D.topology_count = count;
        }
        if (count > D.tris_cap) {
            if (!realloc_dev(cx, &D.tris, (size_t)D.tris_cap * 3, (size_t)count * 3, "dynamic indexed triangle allocation")) return false;
            D.tris_cap = count;
        }
        const bool motion = !topology_changed && D.tri_upload_count == count;
        k_dyn_from_indices<<<dyn_blocks(count), kThreadsDyn, 0, S->stream>>>(D.verts, vcount, D.idx, count, D.tris);
        if (!finish_triangles(cx, D, count, true, motion, tri_cell_size(max_extent, cx.margin, cx.thickness, true))) return false;
        D.tri_upload_count = count;
        if (!publish(S, k)) return false;
    }
    return true;
}

// Dynamic particles of a cloth (abi41.cu:8566-8696).
bool upload_dynamic_particles(Solver* S, int cloth, const float* pos, const float* radii, int count) {
    if (!S || cloth >= S->K) return fail("invalid dynamic particle update");
    count = std::max(count, 0);
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    AllocAccount account(&S->device_bytes);
    if (count > 0 && (!pos || !radii)) return fail("dynamic particle position/radius data is required when particle count is nonzero");
    for (int k = k0; k < k1; ++k) {
        DynHost& D = S->cl[k].dyn;
        if (count == 0)
            clear_particles(D);
        else if (!put_particles(cloth_ctx(S, k), D, pos, nullptr, radii, count, nullptr))
            return false;
        if (!publish(S, k)) return false;
    }
    return true;
}

// ------------------------------------------------------ shared scene --

GlobalScene* scene_create() {
    GlobalScene* G = new GlobalScene();
    G->key_ieee = g_default_key_ieee.load();
    if (!cuda_ok(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking), "global dynamic scene stream")) {
        delete G;
        return nullptr;
    }
    return G;
}

void scene_destroy(GlobalScene* G) {
    if (!G) return;
    // solvers still attached stop using it before its memory goes
    for (const auto& a : std::vector<std::pair<Solver*, int>>(G->attached.begin(), G->attached.end())) scene_detach(a.first, a.second);
    cudaDeviceSynchronize();
    free_set(G->dyn);
    void* ptrs[] = {G->tri_src, G->tri_layer, G->par_src, G->par_layer, G->overflow};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (G->stream) cudaStreamDestroy(G->stream);
    delete G;
}

// abi41.cu:6597-6784: triangles as plain rows with fine hash cells and the
// unsigned response, particles with the caller's previous positions, source
// ids and collision layers per primitive.
bool scene_update(GlobalScene* G, const SsblXpbdGlobalDynamicSceneInputs* in) {
    if (!G || !in) return fail("invalid global dynamic scene update");
    const auto t0 = std::chrono::high_resolution_clock::now();
    const int P = std::max(in->particle_count, 0), T = std::max(in->triangle_count, 0);
    if (P > 0 && (!in->particle_positions || !in->particle_radii || !in->particle_source_ids || !in->particle_collision_layers))
        return fail("global dynamic particle arrays are incomplete");
    if (T > 0 && (!in->triangle_vertices || !in->triangle_source_ids || !in->triangle_collision_layers))
        return fail("global dynamic triangle arrays are incomplete");
    // solvers read the scene from their own streams: let their frames finish
    if (!cuda_ok(cudaDeviceSynchronize(), "global dynamic scene update")) return false;
    G->margin = std::max(in->collision_margin, 0.0f);
    G->thickness = std::max(in->cloth_thickness, 0.0f);
    G->hash_overflow = 0;
    AllocAccount account(&G->device_bytes);
    const DynCtx c{G->stream, &G->device_bytes, G->margin, G->thickness, G->key_ieee};
    DynHost& D = G->dyn;
    if (!G->overflow && !dalloc(&G->overflow, 1, "global dynamic scene counters")) return false;
    if (!cuda_ok(cudaMemsetAsync(G->overflow, 0, sizeof(unsigned long long), c.st), "global dynamic scene counters")) return false;
    if (P == 0) {
        clear_particles(D);
    } else {
        if (P > G->par_meta_cap) {
            if (!realloc_dev(c, &G->par_src, (size_t)G->par_meta_cap, (size_t)P, "global dynamic particle source ids") ||
                !realloc_dev(c, &G->par_layer, (size_t)G->par_meta_cap, (size_t)P, "global dynamic particle layers"))
                return false;
            G->par_meta_cap = P;
        }
        if (!dupload(G->par_src, in->particle_source_ids, (size_t)P, c.st, "global dynamic particle source upload") ||
            !dupload(G->par_layer, in->particle_collision_layers, (size_t)P, c.st, "global dynamic particle layer upload") ||
            !put_particles(c, D, in->particle_positions, in->particle_prev_positions ? in->particle_prev_positions : in->particle_positions,
                           in->particle_radii, P, G->overflow))
            return false;
    }
    if (T == 0) {
        clear_triangles(D);
    } else {
        if (T > G->tri_meta_cap) {
            if (!realloc_dev(c, &G->tri_src, (size_t)G->tri_meta_cap, (size_t)T, "global dynamic triangle source ids") ||
                !realloc_dev(c, &G->tri_layer, (size_t)G->tri_meta_cap, (size_t)T, "global dynamic triangle layers"))
                return false;
            G->tri_meta_cap = T;
        }
        const bool motion = D.tri_upload_count == T;
        if (!dupload(G->tri_src, in->triangle_source_ids, (size_t)T, c.st, "global dynamic triangle source upload") ||
            !dupload(G->tri_layer, in->triangle_collision_layers, (size_t)T, c.st, "global dynamic triangle layer upload") ||
            !put_rows(c, D, in->triangle_vertices, T) ||
            !finish_triangles(c, D, T, false, motion, tri_cell_size(rows_max_extent(in->triangle_vertices, T), c.margin, c.thickness, true)))
            return false;
        D.tri_upload_count = T;
    }
    D.h.tri_src = T > 0 ? G->tri_src : nullptr;
    D.h.tri_layer = T > 0 ? G->tri_layer : nullptr;
    D.h.par_src = P > 0 ? G->par_src : nullptr;
    D.h.par_layer = P > 0 ? G->par_layer : nullptr;
    unsigned long long over = 0;
    if (!publish_set(c, D) ||
        !cuda_ok(cudaMemcpyAsync(&over, G->overflow, sizeof(over), cudaMemcpyDeviceToHost, c.st), "global dynamic scene counters") ||
        !cuda_ok(cudaStreamSynchronize(c.st), "global dynamic scene update"))
        return false;
    G->hash_overflow = (long long)over;
    G->upload_ms = (float)ms_since(t0);
    // attached solvers re-check which stages their frame graph needs
    for (const auto& a : G->attached) a.first->params_dirty = true;
    return true;
}

bool scene_attach(Solver* S, int cloth, GlobalScene* G, int source_id, int layer, int mode) {
    if (!S || !G || cloth >= S->K) return fail("invalid global dynamic scene attach");
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    for (int k = k0; k < k1; ++k) {
        Cloth& C = S->cl[k];
        if (C.gscene && C.gscene != G) C.gscene->attached.erase({S, k});
        if (!G->dyn.dev) {
            AllocAccount account(&G->device_bytes);
            if (!publish_set(DynCtx{G->stream, &G->device_bytes, G->margin, G->thickness, G->key_ieee}, G->dyn)) return false;
        }
        C.gscene = G;
        G->attached.insert({S, k});
        Params& P = S->hp[k];
        P.gdyn = G->dyn.dev;
        P.gd_mode = mode;
        P.gd_target_source = source_id;
        P.gd_target_layer = layer;
    }
    S->params_dirty = true;
    return true;
}

void scene_detach(Solver* S, int cloth) {
    if (!S) return;
    const int k0 = cloth < 0 ? 0 : cloth, k1 = cloth < 0 ? S->K : cloth + 1;
    for (int k = k0; k < k1 && k < S->K; ++k) {
        Cloth& C = S->cl[k];
        if (C.gscene) C.gscene->attached.erase({S, k});
        C.gscene = nullptr;
        Params& P = S->hp[k];
        P.gdyn = nullptr;
        P.gd_mode = 0;
        P.gd_target_source = 0;
        P.gd_target_layer = 0;
    }
    S->params_dirty = true;
}

}  // namespace host

}  // namespace xg
