// Render-side surface data in device buffers: per-triangle corner positions
// and flat normals from the engine's current positions (the reference fills
// OpenGL vertex buffers with PopulateTriPos + RecalculateNormals,
// utilities.cu:93-107, 147-183).
#include "engine.h"

namespace pdgb {

// One thread per triangle.  Corners are emitted as X[t0], X[t2], X[t1]
// (the reference's winding flip); the normal is cross(p1 - p0, p2 - p0),
// scaled by rsqrt of its squared length when that exceeds 1e-12.
// Triangles with a corner id >= nv write zeros.
__global__ void k_render_surface(int n, const uint32_t* __restrict__ tris, const int* __restrict__ viperm, int nv,
                                 const float4* __restrict__ x, float* pos, float4* nor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t a = tris[3 * (size_t)i], b = tris[3 * (size_t)i + 1], c = tris[3 * (size_t)i + 2];
    float* out = pos + 9 * (size_t)i;
    float4* on = nor + 3 * (size_t)i;
    if (a >= (uint32_t)nv || b >= (uint32_t)nv || c >= (uint32_t)nv) {
        for (int k = 0; k < 9; ++k) out[k] = 0.f;
        for (int k = 0; k < 3; ++k) on[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 p0 = x[viperm[a]], p1 = x[viperm[c]], p2 = x[viperm[b]];
    out[0] = p0.x; out[1] = p0.y; out[2] = p0.z;
    out[3] = p1.x; out[4] = p1.y; out[5] = p1.z;
    out[6] = p2.x; out[7] = p2.y; out[8] = p2.z;
    const float e1x = p1.x - p0.x, e1y = p1.y - p0.y, e1z = p1.z - p0.z;
    const float e2x = p2.x - p0.x, e2y = p2.y - p0.y, e2z = p2.z - p0.z;
    float nx = e1y * e2z - e2y * e1z;
    float ny = e1z * e2x - e2z * e1x;
    float nz = e1x * e2y - e2x * e1y;
    const float len2 = nx * nx + ny * ny + nz * nz;
    if (len2 > 1e-12f) {
        const float r = rsqrtf(len2);
        nx *= r;
        ny *= r;
        nz *= r;
    }
    const float4 nn = make_float4(nx, ny, nz, 0.f);
    on[0] = nn;
    on[1] = nn;
    on[2] = nn;
}

void launch_render_surface(int n, const uint32_t* tris, const int* viperm, int nv, const float4* x, float* pos,
                           float* nor, cudaStream_t s) {
    if (n > 0) k_render_surface<<<(n + 255) / 256, 256, 0, s>>>(n, tris, viperm, nv, x, pos, (float4*)nor);
}

}  // namespace pdgb
