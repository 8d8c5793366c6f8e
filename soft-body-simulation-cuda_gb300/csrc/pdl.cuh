// Programmatic dependent launch (sm_90 and later), shared by the step
// kernels.  A kernel launched with programmatic stream serialization may be
// scheduled before its predecessor on the stream has finished: once every
// CTA of the predecessor has executed pdl_trigger (or exited).  Until its
// own pdl_wait returns -- after the predecessor grid has completed and its
// writes are visible -- it may only read data that no earlier kernel of
// the chain writes (layouts, coefficients, factor blocks).  Every CTA of a
// kernel launched this way waits before it can exit, so each grid
// completes after its predecessor and the order holds along the chain.
#pragma once
#include <cuda_runtime.h>

#include "engine.h"

namespace pdgb {

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

template <typename... P, typename... A>
inline void launch_pdl(void (*kernel)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PDGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kernel, args...));
}

}  // namespace pdgb
