// Constraint and velocity arithmetic shared by the solver kernels and the
// differentiable rollout: the stretch and bend corrections of one constraint
// and the velocity update of one vertex, written once so both compute the
// same bits.  Each takes its compliance as an argument (the rollout has one
// per constraint).
#pragma once

#include "xpbd_math.cuh"

namespace xg {

// Stretch correction of edge (i, j), in the edge's orientation (abi41.cu:
// 1927-1980): corr = (pj - pi) * 0.18 * dlambda / len, dlambda = -C / (wi +
// wj + compliance / dt^2), C = len - rest, capped at max(2.5 mm, min(0.1
// rest, 25 mm)).  Returns false when both endpoints are fixed.
__device__ __forceinline__ bool stretch_correction(float4 pi, float4 pj, float rest, float compliance, float dt, F3* corr_out,
                                                   float* c_out, bool* clamped) {
    const float wi = pi.w, wj = pj.w;
    const float weight = wi + wj;
    *clamped = false;
    if (weight <= 0.0f) return false;
    const F3 delta = f3(pj) - f3(pi);
    const float len = sqrtf(fmaxf(dot3(delta, delta), kEps));
    const float c = len - rest;
    const float alpha = fmaxf(compliance, 0.0f) / fmaxf(dt * dt, kEps);
    const float dlambda = -c / (weight + alpha);
    F3 corr = delta * (0.18f * dlambda / fmaxf(len, kEps));
    const float corr_len = sqrtf(fmaxf(dot3(corr, corr), 0.0f));
    const float max_corr = fmaxf(0.0025f, fminf(fmaxf(rest, 0.0f) * 0.10f, 0.025f));
    if (corr_len > max_corr) {
        corr = corr * (max_corr / fmaxf(corr_len, kEps));
        *clamped = true;
    }
    *corr_out = corr;
    *c_out = c;
    return true;
}

// Bend distance correction between the two wing-opposite vertices
// (abi41.cu:2805-2884, 2886-2970): corr = (pj - pi) * 0.10 * dlambda / len,
// capped at max(0.25 mm, min(0.08 max(rest, thickness), 20 mm)).  Returns
// false when the constraint is skipped; `guard` is set when the reference
// would count a guard.
__device__ __forceinline__ bool bend_correction_k(float4 pi4, float4 pj4, float rest, float compliance, float thickness,
                                                  float dt, F3* corr_out, bool* guard, bool* clamped) {
    *guard = false;
    *clamped = false;
    const float wi = pi4.w, wj = pj4.w;
    const float weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return false;
    if (!isfinite(rest) || rest <= kEps) {
        *guard = true;
        return false;
    }
    const F3 pi = f3(pi4), pj = f3(pj4);
    if (!finite3(pi) || !finite3(pj)) {
        *guard = true;
        return false;
    }
    const F3 delta = pj - pi;
    const float len_sq = len_sq_xyz(delta);
    if (!isfinite(len_sq) || len_sq <= 1.0e-10f) {
        *guard = true;
        return false;
    }
    const float inv_len = 1.0f / sqrtf(len_sq);
    const float len = len_sq * inv_len;
    const float c = len - rest;
    if (!isfinite(c) || fabsf(c) <= 1.0e-6f) return false;
    const float alpha = fmaxf(compliance, 0.0f) / fmaxf(dt * dt, kEps);
    const float dlambda = -c / fmaxf(weight + alpha, kEps);
    F3 corr = delta * (0.10f * dlambda * inv_len);
    if (!finite3(corr)) {
        *guard = true;
        return false;
    }
    const float corr_len = len3(corr);
    const float max_corr = fmaxf(2.5e-4f, fminf(fmaxf(rest, thickness) * 0.08f, 0.020f));
    if (!isfinite(corr_len) || corr_len <= 0.0f) return false;
    if (corr_len > max_corr) {
        corr = corr * (max_corr / fmaxf(corr_len, kEps));
        *guard = true;
        *clamped = true;
    }
    *corr_out = corr;
    return true;
}

// Velocity of a vertex at the end of a substep: v + feedback(measured - v)
// with the aligned-feedback clamp (abi41.cu:5846-5884); fixed vertices
// (w <= 0) stop.
__device__ __forceinline__ F3 velocity_update(F3 p, F3 prev, F3 vel, float w, float thickness, float dt) {
    if (w <= 0.0f) return F3{0.0f, 0.0f, 0.0f};
    const float sdt = fmaxf(dt, kEps);
    const F3 measured = (p - prev) * (1.0f / sdt);
    const F3 base = vel;
    if (!finite3(measured) || !finite3(base)) return F3{0.0f, 0.0f, 0.0f};
    const F3 proj = measured - base;
    const float pdb = dot3(proj, base);
    const float scale = (isfinite(pdb) && pdb > 0.0f) ? 0.9f : 1.0f;
    const float max_delta = fmaxf(2.0e-4f, fmaxf(thickness, 0.0f) * 0.35f);
    const float max_speed = max_delta / sdt;
    F3 fb = proj * scale;
    const float fspeed = len3(fb);
    if (scale < 1.0f && isfinite(fspeed) && fspeed > max_speed && fspeed > kEps) fb = fb * (max_speed / fspeed);
    if (!finite3(fb)) fb = F3{0.0f, 0.0f, 0.0f};
    return base + fb;
}

}  // namespace xg
