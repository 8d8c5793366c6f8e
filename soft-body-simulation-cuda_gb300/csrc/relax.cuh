// The 0.9 under-relaxation of the Jacobi iterate (device code).
//
// 0.9 is a double literal in the reference's Chebyshev kernel
// (pdUtil.cu:221), so 0.9 * (x - s) + s is evaluated in double there.
// Splitting 0.9 into a float head and tail keeps the product exact to ~1e-15
// without FP64 arithmetic on the GPU.
#pragma once

namespace pdgb {

__device__ __forceinline__ float relax09(float nx, float s) {
    const float d = nx - s;
    constexpr float kHi = 0.9f;
    constexpr float kLo = (float)(0.9 - (double)0.9f);
    return fmaf(kHi, d, fmaf(kLo, d, s));
}

}  // namespace pdgb
