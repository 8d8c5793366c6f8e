// Scene-term kernels outside the per-iteration path: drag set-up (caller
// arrays or the reference's mouse selection), the Cholesky-path RHS
// overwrite of dragged rows, and state copies for XTilde.
#include "scene.cuh"

namespace pdgb {

__global__ void k_gather_drag(int nv, const int* __restrict__ vperm, const float* __restrict__ w,
                              const float* __restrict__ off, float* drag_w, float4* drag_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int o = vperm[i];
    drag_w[i] = w ? w[o] : 0.f;
    if (off) drag_off[i] = make_float4(off[3 * o], off[3 * o + 1], off[3 * o + 2], 0.f);
}

// Selection around a grabbed vertex (Control_Kernel,
// simulationContext.cu:201-218): every free vertex gets its offset from the
// grabbed one; those within sqrt(radius_sq) get the drag weight.  Pinned
// vertices and select_v = -1 get weight 0 and keep their offset.
__global__ void k_drag_select(int nv, const float4* __restrict__ x, const float4* __restrict__ coef, int select_v,
                              float control_mag, double radius_sq, float* drag_w, float4* drag_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float w = 0.f;
    if (coef[i].z == 0.f && select_v != -1) {
        const float4 a = x[i], g = x[select_v];
        const float3 d = make_float3(a.x - g.x, a.y - g.y, a.z - g.z);
        drag_off[i] = make_float4(d.x, d.y, d.z, 0.f);
        const float dist2 = dot3f(d, d);
        if ((double)dist2 < radius_sq) w = control_mag;
    }
    drag_w[i] = w;
}

// Cholesky path: computeDBCLocal overwrites the RHS rows of dragged
// vertices with target * weight (pdUtil.cu:159-164) after the local step
// has added into them; base holds that value for dragged rows.
__global__ void k_drag_rhs(int nv, SceneArgs sc, const float4* __restrict__ base, float4* b, const int* done) {
    if (done && *done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    if (drag_weight(sc, i) > 0.f) b[i] = base[i];
}

__global__ void k_copy_state(int nv, const float4* __restrict__ src, float4* dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) dst[i] = src[i];
}

void launch_gather_drag(int nv, const int* vperm, const float* w, const float* off, float* drag_w, float4* drag_off,
                        cudaStream_t s) {
    if (nv > 0) k_gather_drag<<<(nv + 255) / 256, 256, 0, s>>>(nv, vperm, w, off, drag_w, drag_off);
}

void launch_drag_select(int nv, const float4* x, const float4* coef, int select_v, float control_mag,
                        double radius_sq, float* drag_w, float4* drag_off, cudaStream_t s) {
    if (nv > 0)
        k_drag_select<<<(nv + 255) / 256, 256, 0, s>>>(nv, x, coef, select_v, control_mag, radius_sq, drag_w,
                                                       drag_off);
}

void launch_drag_rhs(int nv, const SceneArgs& sc, const float4* base, float4* b, const int* done, cudaStream_t s) {
    if (nv > 0) k_drag_rhs<<<(nv + 255) / 256, 256, 0, s>>>(nv, sc, base, b, done);
}

void launch_copy_state(int nv, const float4* src, float4* dst, cudaStream_t s) {
    if (nv > 0) k_copy_state<<<(nv + 255) / 256, 256, 0, s>>>(nv, src, dst);
}

}  // namespace pdgb
