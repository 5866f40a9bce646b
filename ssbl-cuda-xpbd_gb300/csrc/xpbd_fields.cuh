// External accelerations of the prediction step: Blender-style force fields
// and the volume-pressure push along the vertex normal
// (native/src/ssbl_xpbd_cuda_abi41.cu:1213-1261, 1262-1558, 1869-1925).
//
// Field kinds and their accelerations at position p with velocity v (d = p -
// origin, r = d without its axis component when the field is 2-D, f = the
// falloff factor, s = strength * f):
//   wind        s * max(0, 1 + noise * n(p)) * (dir . normal) * dir, front faces only
//   force       s * d / |d|;  charge: additionally / max(|d|^2, 0.01)
//   vortex      s * unit(axis x d_radial)
//   harmonic    (-s (|d| - rest) - (v . u) damping |s|) u, u = d / |d|
//   Lennard-Jones  s (q^12 - q^6) d / |d|, q = min(max(rest, size, 0.1) / max(|d|, 1e-3), 6)
//   magnet      s * (v x unit(dir))
//   drag        -(linear + quadratic |v|) v (linear = |s| when both are 0)
//   turbulence  s * (2 T(q) - 1) per axis, T a three-octave gradient noise
//   texture     s * (n(q), n(q + 7 salt), n(q + 13 salt)), q = d * frequency
// then plus -flow * f * v (except harmonic and drag), each field and the sum
// capped at 5000 m/s^2.  n(p) = 2 fract(sin(p . (12.9898, 78.233, 37.719) +
// (seed + salt) 19.191) * 43758.5453) - 1.
//
// The turbulence noise here hashes lattice points with its own integer mix
// instead of the Blender permutation table the reference embeds, so
// turbulence fields give different (equally distributed) values than the
// reference; every other kind follows the reference's formulas.
#pragma once

#include "../../include/ssbl_xpbd_cuda.h"
#include "xpbd_math.cuh"

namespace xg {

constexpr int kFieldWind = 1, kFieldForce = 2, kFieldVortex = 3, kFieldTurbulence = 4, kFieldCharge = 5,
              kFieldHarmonic = 6, kFieldLennardJones = 7, kFieldMagnet = 8, kFieldDrag = 9, kFieldTexture = 10;
constexpr int kMaxFields = 64;
constexpr float kMaxFieldAccel = 5000.0f;

XG_HD F3 f3a(const float* a) { return F3{a[0], a[1], a[2]}; }

__device__ __forceinline__ float field_noise(F3 p, int seed, float salt) {
    const float x = sinf(p.x * 12.9898f + p.y * 78.233f + p.z * 37.719f + ((float)seed + salt) * 19.191f) * 43758.5453f;
    return (x - floorf(x)) * 2.0f - 1.0f;
}

// Lattice hash of the turbulence noise (own integer mix, 8 bits).
__device__ __forceinline__ int lattice_hash(int i) {
    unsigned h = (unsigned)i * 0x9E3779B1u;
    h ^= h >> 15;
    h *= 0x85EBCA77u;
    h ^= h >> 13;
    return (int)(h & 255u);
}

__device__ __forceinline__ float noise_grad(int h, float x, float y, float z) {
    h &= 15;
    const float u = h < 8 ? x : y;
    const float v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

__device__ __forceinline__ float noise_fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
__device__ __forceinline__ float noise_lerp(float t, float a, float b) { return a + t * (b - a); }

// Gradient noise in [-1, 1] (improved-noise construction, Perlin 2002).
__device__ float gradient_noise(float x, float y, float z) {
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
    x -= fx;
    y -= fy;
    z -= fz;
    const float u = noise_fade(x), v = noise_fade(y), w = noise_fade(z);
    const int A = lattice_hash(X) + Y, B = lattice_hash(X + 1) + Y;
    const int AA = lattice_hash(A) + Z, AB = lattice_hash(A + 1) + Z;
    const int BA = lattice_hash(B) + Z, BB = lattice_hash(B + 1) + Z;
    const float x0 = noise_lerp(u, noise_grad(lattice_hash(AA), x, y, z), noise_grad(lattice_hash(BA), x - 1.0f, y, z));
    const float x1 = noise_lerp(u, noise_grad(lattice_hash(AB), x, y - 1.0f, z), noise_grad(lattice_hash(BB), x - 1.0f, y - 1.0f, z));
    const float x2 = noise_lerp(u, noise_grad(lattice_hash(AA + 1), x, y, z - 1.0f),
                                noise_grad(lattice_hash(BA + 1), x - 1.0f, y, z - 1.0f));
    const float x3 = noise_lerp(u, noise_grad(lattice_hash(AB + 1), x, y - 1.0f, z - 1.0f),
                                noise_grad(lattice_hash(BB + 1), x - 1.0f, y - 1.0f, z - 1.0f));
    return noise_lerp(w, noise_lerp(v, x0, x1), noise_lerp(v, x2, x3));
}

// Three octaves of unsigned noise, normalised to [0, 1].
__device__ float turbulence3(float size, float x, float y, float z) {
    if (size != 0.0f && isfinite(size)) {
        const float inv = 1.0f / size;
        x *= inv;
        y *= inv;
        z *= inv;
    }
    float sum = 0.0f, amp = 1.0f, scale = 1.0f;
    for (int o = 0; o < 3; ++o) {
        sum += (0.5f + 0.5f * gradient_noise(scale * x, scale * y, scale * z)) * amp;
        amp *= 0.5f;
        scale *= 2.0f;
    }
    return sum * (4.0f / 7.0f);
}

__device__ float field_falloff(const SsblXpbdForceField& f, float dist, float rdist) {
    if (!isfinite(dist)) return 0.0f;
    const float dmin = fmaxf(f.distance_min, 0.0f), dmax = fmaxf(f.distance_max, 0.0f);
    const float rmin = fmaxf(f.radial_min, 0.0f), rmax = fmaxf(f.radial_max, 0.0f);
    if (f.use_max_distance && dmax > 0.0f && dist >= dmax) return 0.0f;
    if (f.use_radial_max && rmax > 0.0f && rdist >= rmax) return 0.0f;
    float k = 1.0f;
    if (f.use_max_distance && dmax > dmin && dist > dmin) k *= clamp01f((dmax - dist) / fmaxf(dmax - dmin, kEps));
    if (f.use_min_distance && f.falloff_power > 0.0f && dist > dmin) {
        const float ref = fmaxf(dmin, 1.0e-4f);
        k *= powf(ref / fmaxf(dist, ref), f.falloff_power);
    }
    if (f.use_radial_max && rmax > rmin && rdist > rmin) k *= clamp01f((rmax - rdist) / fmaxf(rmax - rmin, kEps));
    if (f.use_radial_min && f.radial_falloff > 0.0f && rdist > rmin) {
        const float ref = fmaxf(rmin, 1.0e-4f);
        k *= powf(ref / fmaxf(rdist, ref), f.radial_falloff);
    }
    return isfinite(k) ? k : 0.0f;
}

__device__ __forceinline__ F3 cap_field_accel(F3 a) {
    const float l = len3(a);
    if (!isfinite(l) || l <= kMaxFieldAccel) return isfinite(l) ? a : F3{0.0f, 0.0f, 0.0f};
    return a * (kMaxFieldAccel / fmaxf(l, kEps));
}

__device__ __forceinline__ F3 with_flow(const SsblXpbdForceField& f, F3 a, F3 vel, float falloff) {
    if (f.type != kFieldHarmonic && f.type != kFieldDrag) {
        const float flow = isfinite(f.flow) ? f.flow : 0.0f;
        if (fabsf(flow) > 1.0e-6f && falloff != 0.0f) a = a + vel * (-flow * falloff);
    }
    return cap_field_accel(a);
}

__device__ F3 field_accel(const SsblXpbdForceField& f, F3 p, F3 vel, F3 normal, bool has_normal) {
    const F3 zero{0.0f, 0.0f, 0.0f};
    if (!isfinite(f.strength) || f.strength == 0.0f || f.apply_to_location == 0) return zero;
    const F3 d = p - f3a(f.origin);
    const F3 axis = normalize_or(f3a(f.axis), F3{0.0f, 0.0f, 1.0f});
    const F3 rd = f.use_2d_force ? d - axis * dot3(d, axis) : d;
    const float dist = len3(d), rdist = len3(rd);
    const float falloff = field_falloff(f, dist, rdist);
    const float s = f.strength * falloff;
    if (s == 0.0f || !isfinite(s)) return zero;
    switch (f.type) {
        case kFieldWind: {
            if (!has_normal) return zero;
            const F3 dir = normalize_or(f3a(f.direction), zero);
            const float proj = dot3(dir, normal);
            if (!isfinite(proj) || proj <= 0.0f) return zero;
            float m = s * proj;
            if (f.noise > 0.0f) m *= fmaxf(0.0f, 1.0f + f.noise * field_noise(p, f.seed, 0.0f));
            return with_flow(f, dir * m, vel, falloff);
        }
        case kFieldForce:
        case kFieldCharge: {
            const F3 sd = f.use_2d_force ? rd : d;
            const float sdist = f.use_2d_force ? rdist : dist;
            if (sdist <= 1.0e-6f) return zero;
            float k = s / fmaxf(sdist, kEps);
            if (f.type == kFieldCharge) k /= fmaxf(sdist * sdist, 0.01f);
            return with_flow(f, sd * k, vel, falloff);
        }
        case kFieldVortex: {
            const F3 radial = d - axis * dot3(d, axis);
            if (dot3(radial, radial) <= 1.0e-10f) return zero;
            return with_flow(f, normalize_or(cross3(axis, radial), zero) * s, vel, falloff);
        }
        case kFieldHarmonic: {
            const float sdist = f.use_2d_force ? rdist : dist;
            const F3 sd = f.use_2d_force ? rd : d;
            if (sdist <= 1.0e-6f) return zero;
            const F3 u = sd * (1.0f / fmaxf(sdist, kEps));
            const float spring = -s * (sdist - fmaxf(f.rest_length, 0.0f));
            const float damp = -dot3(vel, u) * fmaxf(f.harmonic_damping, 0.0f) * fabsf(s);
            return with_flow(f, u * (spring + damp), vel, falloff);
        }
        case kFieldLennardJones: {
            if (dist <= 1.0e-6f) return zero;
            const F3 u = d * (1.0f / fmaxf(dist, kEps));
            const float radius = fmaxf(f.rest_length, fmaxf(f.size, 0.1f));
            const float q = fminf(radius / fmaxf(dist, 1.0e-3f), 6.0f);
            const float q2 = q * q, q6 = q2 * q2 * q2;
            return with_flow(f, u * (s * (q6 * q6 - q6)), vel, falloff);
        }
        case kFieldMagnet: {
            const F3 ax = normalize_or(f3a(f.direction), zero);
            return with_flow(f, cross3(vel, ax) * s, vel, falloff);
        }
        case kFieldDrag: {
            const float speed = len3(vel);
            if (speed <= 1.0e-6f) return zero;
            float lin = fmaxf(f.linear_drag, 0.0f);
            const float quad = fmaxf(f.quadratic_drag, 0.0f);
            if (lin <= 0.0f && quad <= 0.0f) lin = fabsf(s);
            return with_flow(f, vel * (-(lin + quad * speed)), vel, falloff);
        }
        case kFieldTurbulence: {
            const F3 q = f.use_global_coords ? p : d + axis;
            const F3 n{-1.0f + 2.0f * turbulence3(f.size, q.x, q.y, q.z), -1.0f + 2.0f * turbulence3(f.size, q.y, q.z, q.x),
                       -1.0f + 2.0f * turbulence3(f.size, q.z, q.x, q.y)};
            return with_flow(f, n * s, vel, falloff);
        }
        case kFieldTexture: {
            float freq = fmaxf(fmaxf(f.noise, f.texture_nabla), 0.25f);
            if (f.size > 1.0e-6f) freq = fmaxf(freq, 1.0f / f.size);
            const F3 q = d * freq;
            const F3 n{field_noise(q, f.seed, 0.0f), field_noise(q, f.seed, 7.0f), field_noise(q, f.seed, 13.0f)};
            return with_flow(f, n * s, vel, falloff);
        }
        default:
            return zero;
    }
}

}  // namespace xg
