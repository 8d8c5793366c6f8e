/*
 * Keyword shim that lets g++ compile the reference's PD kernels
 * (src/simulation/solver/projective/pdUtil.cu and the templates of
 * src/simulation/solver/solverUtil.cuh) as ordinary C++ functions.
 * TEST INFRASTRUCTURE ONLY: it builds oracle/_ref, the CPU run of the
 * reference's own PD arithmetic used to pin the oracle and make fixtures.
 *
 * - __global__/__device__/__host__ expand to nothing; a "launch" is a loop
 *   that sets blockIdx/threadIdx and calls the kernel function.
 * - atomicAdd on float is a plain read-add-write (the loop is serial, so
 *   contributions land in thread order).
 * - The three round-to-nearest intrinsics the reference's SVD uses
 *   (external/svd3_cuda/svd3_cuda.h) are given their IEEE meaning:
 *   __fadd_rn/__fsub_rn are single-rounded float add/sub (kept apart from
 *   multiplies by -ffp-contract=off), __frsqrt_rn is 1/sqrt(x) rounded to
 *   float, computed here via double (one extra rounding step, so it may
 *   differ from a correctly rounded result in the last bit on rare inputs).
 * - CUDA's max(float, float) is fmaxf.
 */
#pragma once
#include <cmath>
#include <cstdint>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __inline__ inline

struct refshim_dim3 {
    unsigned x, y, z;
};
extern thread_local refshim_dim3 blockIdx, threadIdx, blockDim, gridDim;

inline float atomicAdd(float* a, float v) {
    float old = *a;
    *a = old + v;
    return old;
}
inline double atomicAdd(double* a, double v) {
    double old = *a;
    *a = old + v;
    return old;
}
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __frsqrt_rn(float x) { return (float)(1.0 / std::sqrt((double)x)); }
inline float max(float a, float b) { return std::fmax(a, b); }

typedef int cudaEvent_t;
inline int cudaEventCreate(cudaEvent_t*) { return 0; }
inline int cudaEventRecord(cudaEvent_t, int = 0) { return 0; }
inline int cudaEventSynchronize(cudaEvent_t) { return 0; }
inline int cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) {
    *ms = 0.f;
    return 0;
}
inline int cudaEventDestroy(cudaEvent_t) { return 0; }

/* Serial emulation of kernel<<<blocks, tpb>>>(...). */
template <class F> inline void refshim_launch(int blocks, int tpb, F&& body) {
    blockDim = {(unsigned)tpb, 1u, 1u};
    gridDim = {(unsigned)blocks, 1u, 1u};
    for (int b = 0; b < blocks; ++b)
        for (int t = 0; t < tpb; ++t) {
            blockIdx = {(unsigned)b, 0u, 0u};
            threadIdx = {(unsigned)t, 0u, 0u};
            body();
        }
}
