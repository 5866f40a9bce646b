// Static signed-distance grid built on the GPU from the static collider's
// triangles (reference native/src/ssbl_xpbd_cuda_abi41.cu:1787-1829 and the
// host sizing at 6123-6218).
//
// One thread per voxel takes the minimum closest-point distance over every
// static triangle and, when the collider mesh is closed, the parity of +x ray
// crossings for the sign.  The triangles are streamed through shared memory
// in tiles so each block reads every triangle once from L2 instead of once
// per thread.
#include "xpbd_solver.cuh"

namespace xg {

namespace {

constexpr int kSdfTile = 256;  // triangles per shared-memory tile (3 x 16 B each)

// Moller-Trumbore test of the ray p + t (1, 0, 0), t > 1e-6, against abc
// with the tolerances of abi41.cu:1725-1747.
__device__ bool ray_x_hits(F3 p, F3 a, F3 b, F3 c) {
    const F3 dir{1.0f, 0.0f, 0.0f};
    const F3 e1 = b - a, e2 = c - a;
    const F3 h = cross3(dir, e2);
    const float det = dot3(e1, h);
    if (fabsf(det) <= 1.0e-8f) return false;
    const float inv_det = 1.0f / det;
    const F3 s = p - a;
    const float u = inv_det * dot3(s, h);
    if (u < -1.0e-5f || u > 1.0f + 1.0e-5f) return false;
    const F3 q = cross3(s, e1);
    const float v = inv_det * dot3(dir, q);
    if (v < -1.0e-5f || u + v > 1.0f + 1.0e-5f) return false;
    const float t = inv_det * dot3(e2, q);
    return t > 1.0e-6f;
}

__global__ void __launch_bounds__(kThreads) k_sdf_build(View v, int cloth, int voxels) {
    __shared__ float4 tile[kSdfTile * 3];
    const Params& P = v.P[cloth];
    const int voxel = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = P.sdf_dim[0], ny = P.sdf_dim[1];
    const int x = voxel % nx, y = (voxel / nx) % ny, z = voxel / (nx * ny);
    const float vs = P.sdf_voxel;
    const F3 p = F3{P.sdf_origin[0], P.sdf_origin[1], P.sdf_origin[2]} + F3{(float)x * vs, (float)y * vs, (float)z * vs};
    const F3 ray = p + F3{0.0f, vs * 1.37e-4f, vs * 2.11e-4f};
    const int T = P.static_tri_count;
    const bool is_signed = P.sdf_signed != 0;
    float best = 3.402823466e+38f;
    int parity = 0;
    for (int base = 0; base < T; base += kSdfTile) {
        const int n = min(kSdfTile, T - base);
        __syncthreads();
        for (int k = threadIdx.x; k < n * 3; k += blockDim.x) tile[k] = ld4(&P.static_tris[base * 3 + k]);
        __syncthreads();
        if (voxel < voxels) {
            for (int t = 0; t < n; ++t) {
                const F3 a = f3(tile[t * 3 + 0]), b = f3(tile[t * 3 + 1]), c = f3(tile[t * 3 + 2]);
                const F3 d = p - closest_on_triangle(p, a, b, c);
                best = fminf(best, dot3(d, d));
                if (is_signed && ray_x_hits(ray, a, b, c)) parity ^= 1;
            }
        }
    }
    if (voxel >= voxels) return;
    float dist = sqrtf(fmaxf(best, 0.0f));
    if (is_signed && parity) dist = -dist;
    const_cast<float*>(P.sdf)[voxel] = dist;
}

}  // namespace

void launch_sdf_build(const View& v, int cloth, int voxels, cudaStream_t s) {
    if (voxels > 0) k_sdf_build<<<(voxels + kThreads - 1) / kThreads, kThreads, 0, s>>>(v, cloth, voxels);
}

}  // namespace xg
