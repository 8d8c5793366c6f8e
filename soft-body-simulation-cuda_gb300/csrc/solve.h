// Device-side interface of the supernodal triangular solves.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "cholesky.h"
#include "engine.h"

namespace pdgb {

constexpr int kCtaSolveThreads = 1024; // whole-solve-in-one-CTA kernel: 32 warps
constexpr int kClusterCtas = 8;           // CTAs per body in the cluster solve
constexpr int kClusterSolveThreads = 512; // per CTA of the cluster solve: 16 warps

struct CholArgs {
    const int* fwd_items;  // kItemInts per item
    const int* bwd_items;  // kItemInts per item
    const int* rows;
    const float* mval;       // M_s column major
    const int4* levels;      // {fwd_begin, fwd_end, bwd_begin, bwd_end} per level, body-major
    const int* body_level;   // [nbodies + 1]: levels of body b (CTA solve)
    const int* body_order;   // CTA -> body (largest factor first)
    float4* r;  // right-hand side in, destroyed (forward updates)
    float4* y;  // forward result (must be zero on entry)
    float4* x;  // solution out
    const int* done;  // early-exit flag of the step (tol rule), may be null
    const int* fwd_blocks;  // CTA block items (per-level launches)
    const int* bwd_blocks;
    const int* fwd_small;   // warp items of small supernodes (per-level launches)
    const int* bwd_small;
    const int* tiny;        // tiny supernode descriptors (per-level launches)
    const int* zstage;      // backward z-staging items (per-level launches)
    float4* zbuf;           // staged z of the block supernodes
};

constexpr int kBlockThreads = 128;      // block-item kernels: 4 warps
constexpr int kSmallThreads = 256;      // small-supernode kernels: one warp item per warp
constexpr int kStageThreads = 128;      // backward z staging: one CTA per 128-row chunk (kStageRows)

// Grid-wide barrier of the persistent solve (device memory): arrivals and
// generation are cleared before each launch; timeout is set when a wait
// ran out of its spin limit and stays set until the state is set again.
struct GridSync {
    unsigned arrive;
    unsigned gen;
    int timeout;
    int pad;
};

// Convergence state of one step of the Cholesky path (device memory).
struct StepState {
    int done;            // set once sqrt(err) < tol: later iterations are skipped
    int iterations;      // iterations run in the current step
    unsigned count;      // blocks that added their partial error sum
    float err_acc;       // sum of squared changes (float, as the reference)
    int nonfinite;       // a step ended with a non-finite position or velocity (sticky)
    int local_timeout;   // a bulk-copy wait of the pipelined local step ran out (sticky)
    GridSync bar;        // barrier of the persistent solve
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
    SceneArgs sc;
};

// One launch per level and direction (large systems).
void launch_chol_solve_levels(const CholArgs& a, const std::vector<SolveLevel>& levels, cudaStream_t s);
// Whether a level's warp items go into its block launch: when there are
// block items and at most kMixWarpsPerBlock warp items per block item.  The
// leaf levels of a batch, with many warp items and few blocks, keep their
// own launch of 256-thread CTAs (merging every level measured 2 % faster on
// the 40^3 cube and 2 % slower on the 512-body batch; 8 or 32 per block:
// the same on the batch, 32 better on the cube).
constexpr int kMixWarpsPerBlock = 32;
inline bool mix_level(int nb, int nw) { return nb > 0 && nw > 0 && nw <= kMixWarpsPerBlock * nb; }
// The whole solve in one persistent cooperative launch over the GPU (all
// bodies of a batch), levels separated by a bounded grid barrier; levels is
// the device copy of the per-level item ranges.
void launch_chol_solve_persistent(const CholArgs& a, const SolveLevel* levels, int nl, GridSync* bar,
                                  long long spin_limit, cudaStream_t s);
// The grid barrier on its own (check entry point).
void launch_grid_sync_check(GridSync* bar, int ctas, int rounds, int missing, long long spin_limit, cudaStream_t s);
int persistent_grid();
// Spin iterations (about 100 ns each) before a barrier wait gives up.
constexpr long long kPersistSpinLimit = 1ll << 24;
// The whole solve of one body in one CTA, levels separated by
// __syncthreads; one CTA per body (small systems and batches of bodies).
void launch_chol_solve_cta(const CholArgs& a, int nbodies, cudaStream_t s);
// The whole solve of one body in one thread-block cluster of kClusterCtas
// CTAs, levels separated by cluster barriers; one cluster per body.
void launch_chol_solve_cluster(const CholArgs& a, int nbodies, cudaStream_t s);

// Distributed-shared-memory solve of one body (DsmPlan): one 8-CTA cluster;
// factor blocks, row lists and the three vectors stay on chip, levels are
// separated by cluster barriers.
struct DsmArgs {
    const float* mcopy;    // each CTA's M_s blocks, as laid out in its shared memory
    const int* mcopy_ptr;  // [kClusterCtas + 1], multiples of 4
    const int* rcopy;      // each CTA's row lists
    const int* rcopy_ptr;
    const int* items;      // kItemInts per item
    const int4* lvl;       // [kClusterCtas][nlevels]
    int nlevels;
    int n;
    int slots;
    int m_area;            // float index of the staged M area
    int r_area;            // int index of the staged row area
};
void launch_chol_solve_dsm(const CholArgs& a, const DsmArgs& d, size_t smem_bytes, cudaStream_t s);
// FP64-residual iterative refinement of the global solve:
//   bsave = b (before the solve destroys it);
//   r = bsave - K x0 in double (K: FP64 CSR over vertex ids), b = r, y = 0;
//   solve K dx = b with the FP32 factor; x0 += dx.
struct RefineArgs {
    int nv;
    const int* rowptr;
    const int* colind;
    const double* val;
    const float4* bsave;
    const float4* x0;
    float4* b;
    float4* y;
    float4* dx;
    float4* x;
    const int* done;
};
void launch_copy_rhs(int nv, const float4* b, float4* bsave, const int* done, cudaStream_t s);
void launch_refine_residual(const RefineArgs& a, cudaStream_t s);
void launch_refine_update(const RefineArgs& a, cudaStream_t s);

void launch_chol_vertex(const CholVertexArgs& a, cudaStream_t s);
void launch_chol_finish(const CholVertexArgs& a, cudaStream_t s);
// Multi-request forms (serving; no early exit): entries {request, first vertex}.
void launch_chol_vertex_multi(const CholVertexArgs* req, const int2* list, const int* count, int grid,
                              cudaStream_t s);
void launch_chol_finish_multi(const CholVertexArgs* req, const int2* list, const int* count, int grid,
                              cudaStream_t s);

}  // namespace pdgb
