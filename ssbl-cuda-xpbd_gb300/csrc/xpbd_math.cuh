// Small-vector arithmetic shared by every kernel of the GB300 XPBD solver.
//
// Every product-sum that the reference evaluates with an explicit fused
// multiply-add (dot and cross products, native/src/ssbl_xpbd_cuda_abi41.cu:
// 625-636) is written here with fmaf; everything else is a plain IEEE
// single-precision operation.  The library is compiled with -fmad=false and
// IEEE division / square root, so no other contraction happens and each
// kernel computes exactly the same bits as a C restatement compiled with
// -ffp-contract=off.  That is what makes the solver deterministic and
// bit-comparable with the CPU oracle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define XG_HD __host__ __device__ __forceinline__

namespace xg {

constexpr float kEps = 1.0e-7f;

struct F3 {
    float x, y, z;
};

XG_HD F3 f3(float x, float y, float z) { return F3{x, y, z}; }
XG_HD F3 f3(float4 v) { return F3{v.x, v.y, v.z}; }
XG_HD float4 f4(F3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
XG_HD F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
XG_HD F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
XG_HD F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
XG_HD F3 neg(F3 a) { return F3{-a.x, -a.y, -a.z}; }

// dot(a, b) = a.z*b.z + (a.y*b.y + a.x*b.x) with two fused steps.
XG_HD float dot3(F3 a, F3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }

XG_HD F3 cross3(F3 a, F3 b) {
    return F3{fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x))};
}

XG_HD float len3(F3 a) { return sqrtf(fmaxf(dot3(a, a), 0.0f)); }

// x*x + y*y + z*z accumulated from z outwards; the reference uses this order
// for tethers and bends (abi41.cu:2747, 2849).
XG_HD float len_sq_xyz(F3 d) { return fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)); }

XG_HD bool finite3(F3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

XG_HD float clamp01f(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

XG_HD F3 normalize_or(F3 v, F3 fallback) {
    const float len = len3(v);
    if (!isfinite(len) || len <= kEps) return fallback;
    return v * (1.0f / len);
}

// Scale `delta` down to `max_len` (abi41.cu:951-960).
XG_HD F3 limit_delta(F3 delta, float max_len) {
    if (!finite3(delta) || !isfinite(max_len) || max_len <= 0.0f) return F3{0.0f, 0.0f, 0.0f};
    const float len = len3(delta);
    if (!isfinite(len) || len <= kEps) return F3{0.0f, 0.0f, 0.0f};
    return len > max_len ? delta * (max_len / len) : delta;
}

// Grid cell of one coordinate: floor(value / max(cell, 1e-7)) (abi41.cu:
// 654-656).  The reference is compiled with --use_fast_math, which makes its
// float division the approximate, flush-to-zero division of the PTX ISA
// (div.approx.ftz.f32: at most 2 ulp from the exact quotient); near a cell
// boundary that quotient can fall on the other side of an integer from the
// correctly rounded one, so hash keys computed with IEEE division differ
// from the reference's in rare cases.  `ieee` = 0 (the default of every
// solver) uses the reference's division, so cells, bucket ids and bucket
// contents are the reference's integers; `ieee` = 1 uses the correctly
// rounded quotient, which is what the CPU oracle computes.
__device__ __forceinline__ float key_quotient(float value, float cell, int ieee) {
    if (ieee) return __fdiv_rn(value, cell);
    float q;
    asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(q) : "f"(value), "f"(cell));
    return q;
}
__device__ __forceinline__ int cell_of(float value, float cell_size, int ieee) {
    return (int)floorf(key_quotient(value, fmaxf(cell_size, kEps), ieee));
}

// Spatial-hash bucket of a cell: the three large primes of Teschner et al.,
// "Optimized Spatial Hashing for Collision Detection of Deformable Objects"
// (VMV 2003), xor-combined and masked to a power-of-two table
// (abi41.cu:658-664).
XG_HD unsigned bucket_of(int x, int y, int z, int bucket_count) {
    const unsigned h = (unsigned)x * 73856093u ^ (unsigned)y * 19349663u ^ (unsigned)z * 83492791u;
    return bucket_count > 0 ? (h & (unsigned)(bucket_count - 1)) : 0u;
}

// Closest point on triangle abc to p: the region classification of Ericson,
// "Real-Time Collision Detection" (2005) section 5.1.5, with the guarded
// divisions of abi41.cu:1589-1635.
XG_HD F3 closest_on_triangle(F3 p, F3 a, F3 b, F3 c) {
    const F3 ab = b - a, ac = c - a, ap = p - a;
    const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    const F3 bp = p - b;
    const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return a + ab * (d1 / fmaxf(d1 - d3, kEps));
    const F3 cp = p - c;
    const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return a + ac * (d2 / fmaxf(d2 - d6, kEps));
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return b + (c - b) * ((d4 - d3) / fmaxf((d4 - d3) + (d5 - d6), kEps));
    const float denom = 1.0f / fmaxf(va + vb + vc, kEps);
    const float v = vb * denom, w = vc * denom;
    return a + (ab * v + ac * w);
}

// Clamped barycentric weights of a point on triangle abc (abi41.cu:4588-4614).
XG_HD void barycentric(F3 p, F3 a, F3 b, F3 c, float* wa, float* wb, float* wc) {
    const F3 v0 = b - a, v1 = c - a, v2 = p - a;
    const float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
    const float d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    const float denom = d00 * d11 - d01 * d01;
    if (fabsf(denom) <= kEps) {
        *wa = *wb = *wc = 1.0f / 3.0f;
        return;
    }
    float v = (d11 * d20 - d01 * d21) / denom;
    float w = (d00 * d21 - d01 * d20) / denom;
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    w = fminf(fmaxf(w, 0.0f), 1.0f - v);
    const float u = fmaxf(1.0f - v - w, 0.0f);
    const float sum = fmaxf(u + v + w, kEps);
    *wa = u / sum;
    *wb = v / sum;
    *wc = w / sum;
}

// Closest-point parameters of segments p1q1 and p2q2 (Ericson section 5.1.9,
// guarded as in abi41.cu:5458-5505).
XG_HD void segment_params(F3 p1, F3 q1, F3 p2, F3 q2, float* s, float* t) {
    const F3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    const float a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
    if (a <= kEps && e <= kEps) {
        *s = 0.0f;
        *t = 0.0f;
        return;
    }
    if (a <= kEps) {
        *s = 0.0f;
        *t = clamp01f(f / fmaxf(e, kEps));
        return;
    }
    const float c = dot3(d1, r);
    if (e <= kEps) {
        *t = 0.0f;
        *s = clamp01f(-c / fmaxf(a, kEps));
        return;
    }
    const float b = dot3(d1, d2);
    const float denom = a * e - b * b;
    *s = fabsf(denom) > kEps ? clamp01f((b * f - c * e) / denom) : 0.0f;
    const float tnom = b * (*s) + f;
    if (tnom < 0.0f) {
        *t = 0.0f;
        *s = clamp01f(-c / fmaxf(a, kEps));
    } else if (tnom > e) {
        *t = 1.0f;
        *s = clamp01f((b - c) / fmaxf(a, kEps));
    } else {
        *t = tnom / e;
    }
}

// Early rejection that cannot change a result.  The closest points computed
// by closest_on_triangle / segment_params are convex combinations of the
// corners, so their exact distance is at least the largest per-axis gap
// between the primitives' boxes; the float computation deviates from it by
// a few units in the last place of the largest coordinate magnitude.  When
// the gap exceeds `limit` by a relative 1e-5 plus 4e-6 x that magnitude
// (well above the rounding), the computed distance is not below `limit`, so
// a test "distance < limit" would fail anyway.  Non-finite input never takes
// the shortcut.
XG_HD float abs_max4(F3 a, F3 b, F3 c, F3 d) {
    const float ma = fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z)));
    const float mb = fmaxf(fabsf(b.x), fmaxf(fabsf(b.y), fabsf(b.z)));
    const float mc = fmaxf(fabsf(c.x), fmaxf(fabsf(c.y), fabsf(c.z)));
    const float md = fmaxf(fabsf(d.x), fmaxf(fabsf(d.y), fabsf(d.z)));
    return fmaxf(fmaxf(ma, mb), fmaxf(mc, md));
}

XG_HD bool gap_proves_far(float gap, float magnitude, bool finite, float limit) {
    return finite && gap > limit * 1.00001f + magnitude * 4.0e-6f;
}

XG_HD bool segments_far(F3 a0, F3 a1, F3 b0, F3 b1, float limit) {
    const float gx = fmaxf(fminf(b0.x, b1.x) - fmaxf(a0.x, a1.x), fminf(a0.x, a1.x) - fmaxf(b0.x, b1.x));
    const float gy = fmaxf(fminf(b0.y, b1.y) - fmaxf(a0.y, a1.y), fminf(a0.y, a1.y) - fmaxf(b0.y, b1.y));
    const float gz = fmaxf(fminf(b0.z, b1.z) - fmaxf(a0.z, a1.z), fminf(a0.z, a1.z) - fmaxf(b0.z, b1.z));
    const bool finite = finite3(a0) && finite3(a1) && finite3(b0) && finite3(b1);
    return gap_proves_far(fmaxf(gx, fmaxf(gy, gz)), abs_max4(a0, a1, b0, b1), finite, limit);
}

XG_HD bool point_triangle_far(F3 p, F3 a, F3 b, F3 c, float limit) {
    const float gx = fmaxf(fminf(a.x, fminf(b.x, c.x)) - p.x, p.x - fmaxf(a.x, fmaxf(b.x, c.x)));
    const float gy = fmaxf(fminf(a.y, fminf(b.y, c.y)) - p.y, p.y - fmaxf(a.y, fmaxf(b.y, c.y)));
    const float gz = fmaxf(fminf(a.z, fminf(b.z, c.z)) - p.z, p.z - fmaxf(a.z, fmaxf(b.z, c.z)));
    const bool finite = finite3(p) && finite3(a) && finite3(b) && finite3(c);
    return gap_proves_far(fmaxf(gx, fmaxf(gy, gz)), abs_max4(p, a, b, c), finite, limit);
}

// Fixed-point accumulation of position deltas: 2^32 units per metre.  Integer
// addition is associative, so scatter sums come out the same whatever order
// the atomics land in; the CPU oracle quantises the same way.
constexpr float kFixScale = 4294967296.0f;
constexpr float kFixInv = 1.0f / 4294967296.0f;

XG_HD long long to_fix(float v) {
    if (!(fabsf(v) < 1.0e6f)) return 0;  // non-finite or absurd deltas contribute nothing
#if defined(__CUDA_ARCH__)
    return __float2ll_rn(v * kFixScale);
#else
    return llrintf(v * kFixScale);
#endif
}

XG_HD float from_fix(long long v) { return (float)v * kFixInv; }

}  // namespace xg
