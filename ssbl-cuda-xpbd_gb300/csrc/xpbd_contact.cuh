// Velocity response of a contact, shared by the static-collider stages and
// the dynamic-collider kernels.
#pragma once

#include "xpbd_solver.cuh"

namespace xg {

// Velocity response of a static contact with unit normal n: remove the inward
// normal velocity, damp the tangent, then Coulomb-style friction bounded by
// friction * normal_proxy (abi41.cu:910-949).
__device__ __forceinline__ bool contact_response(const Params& P, unsigned long long* counts, F3 n, float normal_proxy, F3* vel) {
    if (!finite3(n) || !finite3(*vel)) return false;
    const float vn = dot3(*vel, n);
    if (vn < 0.0f) *vel = *vel - n * vn;
    bool corrected = false;
    F3 tangent = *vel - n * dot3(*vel, n);
    float tlen = len3(tangent);
    const float damping = clamp01f(P.tangent_damping);
    if (damping > 0.0f && tlen > 1.0e-6f) {
        *vel = *vel - tangent * damping;
        corrected = true;
    }
    tangent = *vel - n * dot3(*vel, n);
    tlen = len3(tangent);
    const float friction = fmaxf(P.friction, 0.0f);
    if (friction > 0.0f && normal_proxy > 0.0f && tlen > 1.0e-6f) {
        const float drop = fminf(tlen, friction * normal_proxy);
        if (drop > 1.0e-7f) {
            *vel = *vel - tangent * (drop / fmaxf(tlen, kEps));
            corrected = true;
        }
    }
    if (corrected) count1(counts, kCntFrictionCorrections);
    return corrected;
}

}  // namespace xg
