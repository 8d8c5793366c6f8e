// Device-side interface of the supernodal triangular solves.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "cholesky.h"

namespace pdgb {

constexpr int kFwdThreads = 128;       // rows per forward item (one row per thread)
constexpr int kFwdCols = 256;          // pivot columns per forward item
constexpr int kBwdThreads = 128;       // 4 warps; one warp per column
constexpr int kBwdColsPerItem = 16;    // pivot columns per backward item
constexpr int kBwdChunk = 2048;        // rows of z staged per pass (32 KB)

struct CholArgs {
    const int* fwd_items;  // int4 per item
    const int* bwd_items;  // int4 per item
    const int* sk;
    const int* sm;
    const int64_t* moff;
    const int* roff;
    const int* rows;
    const float* mval;
    float4* r;  // right-hand side in, destroyed (forward updates)
    float4* y;  // forward result (must be zero on entry)
    float4* x;  // solution out
    const int* done;  // early-exit flag of the step (tol rule), may be null
};

// Convergence state of one step of the Cholesky path (device memory).
struct StepState {
    int done;            // set once sqrt(err) < tol: later iterations are skipped
    int iterations;      // iterations run in the current step
    unsigned count;      // blocks that added their partial error sum
    float err_acc;       // sum of squared changes (float, as the reference)
};

struct CholVertexArgs {
    int nv;
    int iteration;
    float tol;
    StepState* st;
    float4* prev;
    float4* sn;
    float4* y;
    float4* b;
    const float4* base;
    const float4* coef;
    const float4* pin_rhs;
    float4* x;
    float4* v;
    float dt_inv;
};

void launch_chol_solve(const CholArgs& a, const std::vector<SolveLevel>& levels, cudaStream_t s);
void launch_chol_vertex(const CholVertexArgs& a, cudaStream_t s);
void launch_chol_finish(const CholVertexArgs& a, cudaStream_t s);

}  // namespace pdgb
