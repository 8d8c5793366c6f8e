// Level-scheduled supernodal triangular solves (sm_103a) and the Cholesky
// path's per-iteration vertex kernel.
//
// Replaces the reference's global step CholeskySpLinearSolver::Solve
// (cholesky.cu:184-192: permute, cusolverSpScsrcholSolve, unpermute) and the
// error check computeError (pdSolver.cu:186-191, 243-253).  The factor is
// stored per supernode as M_s = [L_ss^-1 ; L_os L_ss^-1] (see cholesky.h);
// three right-hand sides (x, y, z) travel together as float4.  Row lists
// hold engine vertex ids, so no permutation pass is needed.
#include "engine.h"
#include "solve.h"
#include "pdl.cuh"
#include "scene.cuh"

#include <cooperative_groups.h>

#include <cstdlib>

namespace pdgb {

// The per-level kernels are launched with programmatic dependent launch
// (pdl.cuh): each triggers its dependents at entry and, before its wait,
// reads only its item descriptors, factor blocks and row ids -- never r, y,
// x, z or the early-exit flag, which earlier kernels write.

// Forward warp item {moff, roff, m, k, r0, c0, c1}: lane = row r0 + lane of
// M_s; sum over pivot columns c0..c1 of M_s[row, c] r[pivot c]; pivot rows
// add the sum to y, off-diagonal rows subtract it from r (ancestor columns,
// solved at a later level).  The chunk's pivot right-hand sides are staged
// in warp-private shared memory 32 at a time; the column loop issues 8
// independent loads of M before using them (memory-level parallelism for
// the few, large supernodes at the top of the tree).
__device__ __forceinline__ void fwd_warp_item(const CholArgs& a, const int* w, float4* stage, int lane) {
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int roff = h0.z, m = h0.w, k = h1.x, r0 = h1.y, c0 = h1.z, c1 = h1.w;
    const int* rows = a.rows + roff;
    const int row = r0 + lane;
    const bool valid = row < m;
    const int cend = !valid ? c0 : (row < k ? min(c1, row + 1) : c1);
    const float* Mr = a.mval + moff + row;
    const int vid = valid ? __ldg(&rows[row]) : 0;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int cb = c0; cb < c1; cb += 32) {
        const int nc = min(32, c1 - cb);
        __syncwarp();
        if (lane < nc) stage[lane] = a.r[__ldg(&rows[cb + lane])];
        __syncwarp();
        for (int c = cb; c < cb + nc; c += 8) {
            float mv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) mv[q] = (c + q < cend) ? __ldg(Mr + (size_t)(c + q) * m) : 0.f;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (c + q < cb + nc) {
                    const float4 v = stage[c + q - cb];
                    ax = fmaf(mv[q], v.x, ax);
                    ay = fmaf(mv[q], v.y, ay);
                    az = fmaf(mv[q], v.z, az);
                }
            }
        }
    }
    if (!valid) return;
    if (row < k) atomicAdd(&a.y[vid], make_float4(ax, ay, az, 0.f));
    else atomicAdd(&a.r[vid], make_float4(-ax, -ay, -az, 0.f));
}

// L2 prefetch of a forward warp item's static data (row ids and up to 16
// columns of the lane's row of M_s), issued before the grid dependency wait.
__device__ __forceinline__ void fwd_warp_prefetch(const CholArgs& a, const int* w, int lane) {
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int m = h0.w, k = h1.x, row = h1.y + lane, c0 = h1.z, c1 = h1.w;
    if (row >= m) return;
    const int cend = min(row < k ? min(c1, row + 1) : c1, c0 + 16);
    const float* Mr = a.mval + moff + row;
    for (int c = c0; c < cend; ++c) prefetch_l2(Mr + (size_t)c * m);
    if (lane == 0) prefetch_l2(a.rows + h0.z + h1.y);
}

// Backward warp item {moff, roff, m, k, c}: x[pivot c] = sum_{i >= c}
// M_s[i, c] z_i with z = [y_pivots ; -x_offdiag]; lanes stride over rows
// (a coalesced column of M_s, 4 independent loads in flight per lane),
// then a warp reduction.  One column per warp keeps the large supernodes at
// the top of the tree spread over many warps.  No atomics.
__device__ __forceinline__ void bwd_warp_item(const CholArgs& a, const int* w, float4* stage, int lane) {
    (void)stage;
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int roff = h0.z, m = h0.w, k = h1.x, c = h1.y;
    const int* rows = a.rows + roff;
    const float* Mc = a.mval + moff + (size_t)c * m;
    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll 4
    for (int i = c + lane; i < m; i += 32) {
        const int vid = __ldg(&rows[i]);
        const float mv = __ldg(Mc + i);
        float4 z;
        if (i < k) z = a.y[vid];
        else {
            const float4 xv = a.x[vid];
            z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
        }
        ax = fmaf(mv, z.x, ax);
        ay = fmaf(mv, z.y, ay);
        az = fmaf(mv, z.z, az);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, off);
        ay += __shfl_xor_sync(0xffffffffu, ay, off);
        az += __shfl_xor_sync(0xffffffffu, az, off);
    }
    if (lane == 0) a.x[__ldg(&rows[c])] = make_float4(ax, ay, az, 0.f);
}

// Backward warp item with its first 64 rows of M_s and row ids loaded
// into registers before the grid dependency wait (the small supernodes of
// the per-level kernels have fewer rows than that); same sums, same order
// as bwd_warp_item.
__device__ __forceinline__ void bwd_warp_item_pre(const CholArgs& a, const int* w, int lane, bool item) {
    int m = 0, k = 0, c = 0;
    const int* rows = a.rows;
    const float* Mc = a.mval;
    float mv[2] = {0.f, 0.f};
    int vid[2] = {0, 0};
    if (item) {
        const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
        const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
        const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
        m = h0.w;
        k = h1.x;
        c = h1.y;
        rows = a.rows + h0.z;
        Mc = a.mval + moff + (size_t)c * m;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int i = c + lane + 32 * t;
            if (i < m) {
                mv[t] = __ldg(Mc + i);
                vid[t] = __ldg(&rows[i]);
            }
        }
    }
    pdl_wait();
    if ((a.done && *a.done) || !item) return;
    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int i = c + lane + 32 * t;
        if (i < m) {
            float4 z;
            if (i < k) z = a.y[vid[t]];
            else {
                const float4 xv = a.x[vid[t]];
                z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
            }
            ax = fmaf(mv[t], z.x, ax);
            ay = fmaf(mv[t], z.y, ay);
            az = fmaf(mv[t], z.z, az);
        }
    }
    for (int i = c + lane + 64; i < m; i += 32) {
        const int v = __ldg(&rows[i]);
        const float mvi = __ldg(Mc + i);
        float4 z;
        if (i < k) z = a.y[v];
        else {
            const float4 xv = a.x[v];
            z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
        }
        ax = fmaf(mvi, z.x, ax);
        ay = fmaf(mvi, z.y, ay);
        az = fmaf(mvi, z.z, az);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, off);
        ay += __shfl_xor_sync(0xffffffffu, ay, off);
        az += __shfl_xor_sync(0xffffffffu, az, off);
    }
    if (lane == 0) a.x[__ldg(&rows[c])] = make_float4(ax, ay, az, 0.f);
}

// ---- per-level launches with CTA block items.
// Forward block {moff, roff, m, k, r0, c0, c1}: the pivot right-hand sides
// r[c0 .. c1) are staged in shared memory once; thread t owns row r0 + t and
// streams its row of M_s (column-major, so a warp's loads of one column are
// contiguous), 8 independent loads in flight.  Pivot rows add into y,
// off-diagonal rows subtract from r (ancestor pivots, read at a later level).
// Static part of a forward block item (no vector reads): the thread's row of
// M_s (at most kFwdBlockCols columns, zero past cend), its vertex id and
// the staging index.
struct FwdBlockPre {
    float mv[kFwdBlockCols];
    int vid, sv, ncols, row, k;
    bool active;
};

__device__ __forceinline__ void fwd_block_load(const CholArgs& a, int item, FwdBlockPre& p) {
    const int* w = a.fwd_blocks + (size_t)kItemInts * item;
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int roff = h0.z, m = h0.w, k = h1.x, r0 = h1.y, c0 = h1.z, c1 = h1.w;
    const int* rows = a.rows + roff;
    const int row = r0 + threadIdx.x;
    const bool active = row < m && row < r0 + kFwdBlockRows;
    const int cend = !active ? c0 : (row < k ? min(c1, row + 1) : c1);
    const float* Mr = a.mval + moff + row;
#pragma unroll
    for (int q = 0; q < kFwdBlockCols; ++q) p.mv[q] = (c0 + q < cend) ? __ldg(Mr + (size_t)(c0 + q) * m) : 0.f;
    p.vid = active ? __ldg(&rows[row]) : 0;
    p.ncols = c1 - c0;
    p.sv = (int)threadIdx.x < p.ncols ? __ldg(&rows[c0 + threadIdx.x]) : 0;
    p.row = row;
    p.k = k;
    p.active = active;
}

// Vector part: stage the pivot right-hand sides (one barrier of the whole
// CTA), then the thread's row sum into y (pivot rows) or r (ancestor rows).
__device__ __forceinline__ void fwd_block_run(const CholArgs& a, const FwdBlockPre& p, float4* rs) {
    if (threadIdx.x < kFwdBlockCols)
        rs[threadIdx.x] = (int)threadIdx.x < p.ncols ? a.r[p.sv] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    if (!p.active) return;
    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
    for (int q = 0; q < kFwdBlockCols; ++q) {
        const float4 v = rs[q];
        ax = fmaf(p.mv[q], v.x, ax);
        ay = fmaf(p.mv[q], v.y, ay);
        az = fmaf(p.mv[q], v.z, az);
    }
    if (p.row < p.k) atomicAdd(&a.y[p.vid], make_float4(ax, ay, az, 0.f));
    else atomicAdd(&a.r[p.vid], make_float4(-ax, -ay, -az, 0.f));
}

__global__ void __launch_bounds__(kBlockThreads) k_chol_fwd_block(CholArgs a, int item0) {
    __shared__ float4 rs[kFwdBlockCols];
    pdl_trigger();
    FwdBlockPre p;
    fwd_block_load(a, item0 + blockIdx.x, p);  // static data before the wait
    pdl_wait();
    if (a.done && *a.done) return;
    fwd_block_run(a, p, rs);
}

// Backward z staging {roff, m, k, r0, zoff}: z = [y_pivots ; -x_offdiag]
// over rows r0 .. r0 + kStageRows of the supernode, gathered once per level
// into zbuf[zoff ..] so that the backward blocks of all its column groups
// read it contiguously.  For a supernode whose columns are split into row
// chunks, x at the pivot rows is cleared here: the backward blocks of the
// level add their chunk sums into it.
__device__ __forceinline__ void zstage_item(const CholArgs& a, int item, bool pdl) {
    const int* w = a.zstage + (size_t)kItemInts * item;
    const int roff = __ldg(w + 2), m = __ldg(w + 3), k = __ldg(w + 4), r0 = __ldg(w + 5), split = __ldg(w + 6),
              zoff = __ldg(w + 7);
    const int* rows = a.rows + roff;
    const int r1 = min(m, r0 + kStageRows);
    const int i0 = r0 + threadIdx.x;
    const int vid0 = i0 < r1 ? __ldg(&rows[i0]) : 0;
    if (pdl) {
        pdl_wait();
        if (a.done && *a.done) return;
    }
    for (int i = i0; i < r1; i += kStageThreads) {
        const int vid = i == i0 ? vid0 : __ldg(&rows[i]);
        float4 z;
        if (i < k) {
            z = a.y[vid];
            if (split) a.x[vid] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const float4 xv = a.x[vid];
            z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
        }
        a.zbuf[zoff + i] = z;
    }
}

__global__ void __launch_bounds__(kStageThreads) k_chol_bwd_zstage(CholArgs a, int item0) {
    pdl_trigger();
    zstage_item(a, item0 + blockIdx.x, true);
}

// Static part of a backward block item: the warp's first 256 rows of each
// of its columns in registers (a whole 256-row chunk).
constexpr int kBwdPre = 8;
struct BwdBlockPre {
    float mpre[kBwdPre][kBwdWarpCols];
    const float* Mc;
    const int* rows;
    const float4* z;
    int m, r0, rend, cw, nc, ib;
    bool live;
};

__device__ __forceinline__ void bwd_block_load(const CholArgs& a, int item, BwdBlockPre& p) {
    const int* w = a.bwd_blocks + (size_t)kItemInts * item;
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(w));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(w) + 1);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int roff = h0.z, m = h0.w, r0 = h1.x, c0 = h1.y & ((1 << kBwdColShift) - 1),
              c1 = c0 + (int)((unsigned)h1.y >> kBwdColShift), rend = h1.z, zoff = h1.w;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = c0 + kBwdWarpCols * warp;  // first column of this warp
    p.nc = min(kBwdWarpCols, c1 - cw);
    p.Mc = a.mval + moff + (size_t)cw * m;
    p.rows = a.rows + roff;
    p.z = a.zbuf + zoff;
    p.m = m;
    p.r0 = r0;
    p.rend = rend;
    p.cw = cw;
    p.live = cw < c1 && cw < rend;
    p.ib = max(cw, r0) + lane;
#pragma unroll
    for (int t = 0; t < kBwdPre; ++t) {
        const int i = p.ib + 32 * t;
#pragma unroll
        for (int j = 0; j < kBwdWarpCols; ++j)
            p.mpre[t][j] =
                (p.live && j < p.nc && i < rend && i >= cw + j) ? __ldg(p.Mc + (size_t)j * m + i) : 0.f;
    }
}

// Vector part: the staged z against the warp's columns, warp reductions,
// sums stored (whole column) or added (row chunk) into x.  Warp-level only.
__device__ __forceinline__ void bwd_block_run(const CholArgs& a, const BwdBlockPre& p) {
    if (!p.live) return;
    const int lane = threadIdx.x & 31;
    float acc[kBwdWarpCols][3];
#pragma unroll
    for (int j = 0; j < kBwdWarpCols; ++j) acc[j][0] = acc[j][1] = acc[j][2] = 0.f;
#pragma unroll
    for (int t = 0; t < kBwdPre; ++t) {
        const int i = p.ib + 32 * t;
        if (i < p.rend) {
            const float4 zz = p.z[i];
#pragma unroll
            for (int j = 0; j < kBwdWarpCols; ++j) {
                if (j < p.nc && i >= p.cw + j) {
                    acc[j][0] = fmaf(p.mpre[t][j], zz.x, acc[j][0]);
                    acc[j][1] = fmaf(p.mpre[t][j], zz.y, acc[j][1]);
                    acc[j][2] = fmaf(p.mpre[t][j], zz.z, acc[j][2]);
                }
            }
        }
    }
#pragma unroll 2
    for (int i = p.ib + 32 * kBwdPre; i < p.rend; i += 32) {
        const float4 zz = p.z[i];
#pragma unroll
        for (int j = 0; j < kBwdWarpCols; ++j) {
            if (j < p.nc && i >= p.cw + j) {
                const float mv = __ldg(p.Mc + (size_t)j * p.m + i);
                acc[j][0] = fmaf(mv, zz.x, acc[j][0]);
                acc[j][1] = fmaf(mv, zz.y, acc[j][1]);
                acc[j][2] = fmaf(mv, zz.z, acc[j][2]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kBwdWarpCols; ++j) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            acc[j][0] += __shfl_xor_sync(0xffffffffu, acc[j][0], off);
            acc[j][1] += __shfl_xor_sync(0xffffffffu, acc[j][1], off);
            acc[j][2] += __shfl_xor_sync(0xffffffffu, acc[j][2], off);
        }
        if (lane == 0 && j < p.nc) {
            float4* xc = &a.x[__ldg(&p.rows[p.cw + j])];
            const float4 sum = make_float4(acc[j][0], acc[j][1], acc[j][2], 0.f);
            if (p.r0 == 0 && p.rend == p.m) *xc = sum;  // the whole column in one item
            else atomicAdd(xc, sum);
        }
    }
}

// Backward block {moff, roff, m, r0, c0 | ncols, r1, zoff}: warp w owns the
// kBwdWarpCols consecutive columns c0 + kBwdWarpCols w .. over the rows
// r0 .. r1; lanes stride the rows, each z (staged, contiguous) is loaded
// once and used for all of the warp's columns (contiguous loads of M_s, one
// per column), then a warp reduction per column whose sum is added into x.
// Column c uses rows i >= c only.  The warp's first 256 rows of each column
// are loaded into registers before the wait; longer columns of whole-column
// items stream the rest afterwards.
__global__ void __launch_bounds__(kBlockThreads) k_chol_bwd_block(CholArgs a, int item0) {
    pdl_trigger();
    BwdBlockPre p;
    bwd_block_load(a, item0 + blockIdx.x, p);
    pdl_wait();
    if (a.done && *a.done) return;
    bwd_block_run(a, p);
}

// Small supernodes of a level (per-level launches): one warp item per warp,
// in kernels of their own so that the many warps of the leaf levels are not
// limited by the block kernels' registers and shared memory.
__global__ void __launch_bounds__(kSmallThreads) k_chol_fwd_small(CholArgs a, int item0, int nitems) {
    __shared__ float4 stage[kSmallThreads / 32][32];
    pdl_trigger();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int it = blockIdx.x * (kSmallThreads / 32) + warp;
    if (it < nitems) fwd_warp_prefetch(a, a.fwd_small + (size_t)kItemInts * (item0 + it), lane);
    pdl_wait();
    if (a.done && *a.done) return;
    if (it < nitems) fwd_warp_item(a, a.fwd_small + (size_t)kItemInts * (item0 + it), stage[warp], lane);
}

__global__ void __launch_bounds__(kSmallThreads) k_chol_bwd_small(CholArgs a, int item0, int nitems) {
    pdl_trigger();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int it = blockIdx.x * (kSmallThreads / 32) + warp;
    bwd_warp_item_pre(a, a.bwd_small + (size_t)kItemInts * (item0 + min(it, nitems - 1)), lane, it < nitems);
}

// L2 prefetch of a tiny supernode's columns of M_s and row ids.
__device__ __forceinline__ void tiny_prefetch(const CholArgs& a, int item) {
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(a.tiny + (size_t)kItemInts * item));
    const float* M = a.mval + ((int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32));
    const int m = h0.w, k = __ldg(a.tiny + (size_t)kItemInts * item + 4);
    for (int i = 0; i < k * m; i += 32) prefetch_l2(M + i);
    prefetch_l2(a.rows + h0.z);
}

// Tiny supernodes (at most kTinyCols pivots, kTinyRows rows): one thread
// solves a whole supernode, so the many leaves of a level cost one thread
// each instead of one warp per item.  Forward: pivot rows store y (only this
// supernode writes them), off-diagonal rows subtract from r.  Backward:
// x_c = sum_{i >= c} M[i, c] z_i over the supernode's rows.
__device__ __forceinline__ void fwd_tiny_item(const CholArgs& a, int item) {
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(a.tiny + (size_t)kItemInts * item));
    const int k = __ldg(a.tiny + (size_t)kItemInts * item + 4);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int m = h0.w;
    const int* rows = a.rows + h0.z;
    const float* M = a.mval + moff;
    float4 rc[kTinyCols];
#pragma unroll
    for (int c = 0; c < kTinyCols; ++c) rc[c] = c < k ? a.r[__ldg(&rows[c])] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int i = 0; i < m; ++i) {
        float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
        for (int c = 0; c < kTinyCols; ++c) {
            if (c < k && c <= i) {
                const float mv = __ldg(M + (size_t)c * m + i);
                ax = fmaf(mv, rc[c].x, ax);
                ay = fmaf(mv, rc[c].y, ay);
                az = fmaf(mv, rc[c].z, az);
            }
        }
        const int vid = __ldg(&rows[i]);
        if (i < k) a.y[vid] = make_float4(ax, ay, az, 0.f);
        else atomicAdd(&a.r[vid], make_float4(-ax, -ay, -az, 0.f));
    }
}

__device__ __forceinline__ void bwd_tiny_item(const CholArgs& a, int item) {
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(a.tiny + (size_t)kItemInts * item));
    const int k = __ldg(a.tiny + (size_t)kItemInts * item + 4);
    const int64_t moff = (int64_t)(uint32_t)h0.x | ((int64_t)h0.y << 32);
    const int m = h0.w;
    const int* rows = a.rows + h0.z;
    const float* M = a.mval + moff;
    float acc[kTinyCols][3];
#pragma unroll
    for (int c = 0; c < kTinyCols; ++c) acc[c][0] = acc[c][1] = acc[c][2] = 0.f;
#pragma unroll 4
    for (int i = 0; i < m; ++i) {
        const int vid = __ldg(&rows[i]);
        float4 z;
        if (i < k) z = a.y[vid];
        else {
            const float4 xv = a.x[vid];
            z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
        }
#pragma unroll
        for (int c = 0; c < kTinyCols; ++c) {
            if (c < k && c <= i) {
                const float mv = __ldg(M + (size_t)c * m + i);
                acc[c][0] = fmaf(mv, z.x, acc[c][0]);
                acc[c][1] = fmaf(mv, z.y, acc[c][1]);
                acc[c][2] = fmaf(mv, z.z, acc[c][2]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kTinyCols; ++c)
        if (c < k) a.x[__ldg(&rows[c])] = make_float4(acc[c][0], acc[c][1], acc[c][2], 0.f);
}

__global__ void __launch_bounds__(kSmallThreads) k_chol_fwd_tiny(CholArgs a, int t0, int n) {
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) tiny_prefetch(a, t0 + t);
    pdl_wait();
    if (a.done && *a.done) return;
    if (t < n) fwd_tiny_item(a, t0 + t);
}

__global__ void __launch_bounds__(kSmallThreads) k_chol_bwd_tiny(CholArgs a, int t0, int n) {
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) tiny_prefetch(a, t0 + t);
    pdl_wait();
    if (a.done && *a.done) return;
    if (t < n) bwd_tiny_item(a, t0 + t);
}

// A level's block items and a few warp items in one launch (128-thread
// CTAs: CTAs 0 .. nb-1 take the block items, the others four warp items
// each).  Items of one level are independent, so where the warp items are
// few (the upper levels of a batch, where only some bodies still have small
// supernodes) they run beside the block items instead of in a launch of a
// handful of CTAs that the next level's launch would wait for.
__global__ void __launch_bounds__(kBlockThreads) k_chol_fwd_mixed(CholArgs a, int b0, int nb, int w0, int nw) {
    __shared__ float4 rs[kFwdBlockCols];
    __shared__ float4 stage[kBlockThreads / 32][32];
    pdl_trigger();
    if ((int)blockIdx.x < nb) {
        FwdBlockPre p;
        fwd_block_load(a, b0 + blockIdx.x, p);  // static data before the wait
        pdl_wait();
        if (a.done && *a.done) return;
        fwd_block_run(a, p, rs);
    } else {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int it = ((int)blockIdx.x - nb) * (kBlockThreads / 32) + warp;
        if (it < nw) fwd_warp_prefetch(a, a.fwd_small + (size_t)kItemInts * (w0 + it), lane);
        pdl_wait();
        if (a.done && *a.done) return;
        if (it < nw) fwd_warp_item(a, a.fwd_small + (size_t)kItemInts * (w0 + it), stage[warp], lane);
    }
}

__global__ void __launch_bounds__(kBlockThreads) k_chol_bwd_mixed(CholArgs a, int b0, int nb, int w0, int nw) {
    pdl_trigger();
    if ((int)blockIdx.x < nb) {
        BwdBlockPre p;
        bwd_block_load(a, b0 + blockIdx.x, p);
        pdl_wait();
        if (a.done && *a.done) return;
        bwd_block_run(a, p);
    } else {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int it = ((int)blockIdx.x - nb) * (kBlockThreads / 32) + warp;
        bwd_warp_item_pre(a, a.bwd_small + (size_t)kItemInts * (w0 + min(it, nw - 1)), lane, it < nw);
    }
}

void launch_chol_solve_levels(const CholArgs& a, const std::vector<SolveLevel>& levels, cudaStream_t s) {
    constexpr int kWarps = kSmallThreads / 32;
    for (size_t L = 0; L < levels.size(); ++L) {
        const SolveLevel& v = levels[L];
        const int nb = v.fwdb_end - v.fwdb_begin, nw = v.fwdw_end - v.fwdw_begin, nt = v.tiny_end - v.tiny_begin;
        if (nt > 0) launch_pdl(k_chol_fwd_tiny, (nt + kSmallThreads - 1) / kSmallThreads, kSmallThreads, 0, s, a, v.tiny_begin, nt);
        if (mix_level(nb, nw)) {
            constexpr int kMixWarps = kBlockThreads / 32;
            launch_pdl(k_chol_fwd_mixed, nb + (nw + kMixWarps - 1) / kMixWarps, kBlockThreads, 0, s, a, v.fwdb_begin, nb,
                       v.fwdw_begin, nw);
            continue;
        }
        if (nw > 0) launch_pdl(k_chol_fwd_small, (nw + kWarps - 1) / kWarps, kSmallThreads, 0, s, a, v.fwdw_begin, nw);
        if (nb > 0) launch_pdl(k_chol_fwd_block, nb, kBlockThreads, 0, s, a, v.fwdb_begin);
    }
    for (size_t L = levels.size(); L-- > 0;) {
        const SolveLevel& v = levels[L];
        const int nb = v.bwdb_end - v.bwdb_begin, nw = v.bwdw_end - v.bwdw_begin, nt = v.tiny_end - v.tiny_begin;
        const int nz = v.zst_end - v.zst_begin;
        if (nz > 0) launch_pdl(k_chol_bwd_zstage, nz, kStageThreads, 0, s, a, v.zst_begin);
        if (mix_level(nb, nw)) {
            constexpr int kMixWarps = kBlockThreads / 32;
            launch_pdl(k_chol_bwd_mixed, nb + (nw + kMixWarps - 1) / kMixWarps, kBlockThreads, 0, s, a, v.bwdb_begin, nb,
                       v.bwdw_begin, nw);
        } else {
            if (nb > 0) launch_pdl(k_chol_bwd_block, nb, kBlockThreads, 0, s, a, v.bwdb_begin);
            if (nw > 0)
                launch_pdl(k_chol_bwd_small, (nw + kWarps - 1) / kWarps, kSmallThreads, 0, s, a, v.bwdw_begin, nw);
        }
        if (nt > 0) launch_pdl(k_chol_bwd_tiny, (nt + kSmallThreads - 1) / kSmallThreads, kSmallThreads, 0, s, a, v.tiny_begin, nt);
    }
}

// ---- the whole solve in one persistent launch over the GPU.
// All CTAs are resident (cooperative launch), 128 threads each.  Per
// forward level the CTAs stride over the level's units -- one block item,
// four warp items or 128 tiny supernodes per unit -- and meet at a
// grid-wide barrier; per backward level the z staging (when the level has
// block items) and the backward items are separated by barriers as well.
// The barrier spins for a bounded time: past the limit it sets a sticky
// timeout word and every CTA returns at its next barrier (the step's result
// is then invalid and the engine reports PDGB_ERR_TIMEOUT).
__device__ __forceinline__ bool grid_sync(GridSync* g, unsigned& gen, unsigned expect, long long spin_limit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = gen + 1;
        bool good = true;
        __threadfence();  // this CTA's writes before the arrival (cumulative over the CTA barrier)
        const unsigned prev = atomicAdd(&g->arrive, 1u);
        if (prev == expect - 1) {
            atomicExch(&g->arrive, 0u);
            __threadfence();
            atomicExch(&g->gen, target);
        } else {
            long long n = 0;
            for (;;) {
                if (*reinterpret_cast<volatile unsigned*>(&g->gen) == target) break;
                if (*reinterpret_cast<volatile int*>(&g->timeout)) {
                    good = false;
                    break;
                }
                if (++n > spin_limit) {
                    atomicExch(&g->timeout, 1);
                    good = false;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();  // the other CTAs' writes before any read after the barrier
        gen = target;
        ok = good && !*reinterpret_cast<volatile int*>(&g->timeout);
    }
    __syncthreads();
    return ok;
}

__global__ void __launch_bounds__(kBlockThreads) k_chol_solve_persistent(CholArgs a, const SolveLevel* __restrict__ lv,
                                                                         int nl, GridSync* bar, long long spin) {
    __shared__ float4 rs[kFwdBlockCols];
    __shared__ float4 stage[kBlockThreads / 32][32];
    if (a.done && *a.done) return;  // set before this launch: the same for every CTA
    constexpr int kWarps = kBlockThreads / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned expect = gridDim.x;
    unsigned gen = 0;
    for (int L = 0; L < nl; ++L) {
        const SolveLevel v = lv[L];
        const int nb = v.fwdb_end - v.fwdb_begin, nw = v.fwdw_end - v.fwdw_begin, nt = v.tiny_end - v.tiny_begin;
        const int nwu = (nw + kWarps - 1) / kWarps, ntu = (nt + kBlockThreads - 1) / kBlockThreads;
        for (int u = blockIdx.x; u < nb + nwu + ntu; u += gridDim.x) {
            if (u < nb) {
                __syncthreads();  // rs of the previous block item is read
                FwdBlockPre p;
                fwd_block_load(a, v.fwdb_begin + u, p);
                fwd_block_run(a, p, rs);
            } else if (u < nb + nwu) {
                const int it = (u - nb) * kWarps + warp;
                if (it < nw) fwd_warp_item(a, a.fwd_small + (size_t)kItemInts * (v.fwdw_begin + it), stage[warp], lane);
            } else {
                const int t = (u - nb - nwu) * kBlockThreads + threadIdx.x;
                if (t < nt) fwd_tiny_item(a, v.tiny_begin + t);
            }
        }
        if (!grid_sync(bar, gen, expect, spin)) return;
    }
    for (int L = nl - 1; L >= 0; --L) {
        const SolveLevel v = lv[L];
        const int nz = v.zst_end - v.zst_begin;
        if (nz > 0) {
            for (int u = blockIdx.x; u < nz; u += gridDim.x) zstage_item(a, v.zst_begin + u, false);
            if (!grid_sync(bar, gen, expect, spin)) return;
        }
        const int nb = v.bwdb_end - v.bwdb_begin, nw = v.bwdw_end - v.bwdw_begin, nt = v.tiny_end - v.tiny_begin;
        const int nwu = (nw + kWarps - 1) / kWarps, ntu = (nt + kBlockThreads - 1) / kBlockThreads;
        for (int u = blockIdx.x; u < nb + nwu + ntu; u += gridDim.x) {
            if (u < nb) {
                BwdBlockPre p;
                bwd_block_load(a, v.bwdb_begin + u, p);
                bwd_block_run(a, p);
            } else if (u < nb + nwu) {
                const int it = (u - nb) * kWarps + warp;
                if (it < nw) bwd_warp_item(a, a.bwd_small + (size_t)kItemInts * (v.bwdw_begin + it), stage[warp], lane);
            } else {
                const int t = (u - nb - nwu) * kBlockThreads + threadIdx.x;
                if (t < nt) bwd_tiny_item(a, v.tiny_begin + t);
            }
        }
        if (L > 0 && !grid_sync(bar, gen, expect, spin)) return;
    }
}

// CTAs of the persistent solve: the resident CTAs per SM (at most
// PDGB_PERSIST_CTAS_PER_SM, default 8) times the SMs.
int persistent_grid() {
    static int grid[64] = {0};
    int dev = 0;
    PDGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error{PDGB_ERR_CUDA, "device index out of range"};
    if (!grid[dev]) {
        int sms = 0, per = 0;
        PDGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PDGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_chol_solve_persistent, kBlockThreads, 0));
        int cap = 8;
        if (const char* e = std::getenv("PDGB_PERSIST_CTAS_PER_SM")) cap = std::max(1, std::atoi(e));
        grid[dev] = sms * std::max(1, std::min(per, cap));
    }
    return grid[dev];
}

void launch_chol_solve_persistent(const CholArgs& a, const SolveLevel* levels, int nl, GridSync* bar,
                                  long long spin_limit, cudaStream_t s) {
    if (nl <= 0) return;
    PDGB_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s));  // arrival count and generation
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(persistent_grid());
    cfg.blockDim = dim3(kBlockThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PDGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_chol_solve_persistent, a, levels, nl, bar, spin_limit));
}

// Check of the grid barrier on its own: `rounds` barriers of a cooperative
// launch of `ctas` CTAs that wait for `missing` more arrivals than there are
// CTAs (0: the barrier completes; > 0: it can only time out).
__global__ void k_grid_sync_check(GridSync* bar, int rounds, int missing, long long spin) {
    unsigned gen = 0;
    for (int r = 0; r < rounds; ++r)
        if (!grid_sync(bar, gen, gridDim.x + (unsigned)missing, spin)) return;
}

void launch_grid_sync_check(GridSync* bar, int ctas, int rounds, int missing, long long spin_limit, cudaStream_t s) {
    PDGB_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridSync), s));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kBlockThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PDGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_grid_sync_check, bar, rounds, missing, spin_limit));
}

// ---- one body per CTA: warps stride over the items of a level,
// __syncthreads between levels (global writes of the block become visible
// to the whole block at the barrier).  Bodies are independent, so CTAs
// never wait on each other.
__global__ void __launch_bounds__(kCtaSolveThreads) k_chol_solve_cta(CholArgs a) {
    __shared__ float4 stage[kCtaSolveThreads / 32][32];
    if (a.done && *a.done) return;
    constexpr int kWarps = kCtaSolveThreads / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int body = __ldg(&a.body_order[blockIdx.x]);
    const int L0 = __ldg(&a.body_level[body]), L1 = __ldg(&a.body_level[body + 1]);
    for (int L = L0; L < L1; ++L) {
        const int4 lv = __ldg(&a.levels[L]);
        for (int it = lv.x + warp; it < lv.y; it += kWarps)
            fwd_warp_item(a, a.fwd_items + (size_t)kItemInts * it, stage[warp], lane);
        __syncthreads();
    }
    for (int L = L1 - 1; L >= L0; --L) {
        const int4 lv = __ldg(&a.levels[L]);
        for (int it = lv.z + warp; it < lv.w; it += kWarps)
            bwd_warp_item(a, a.bwd_items + (size_t)kItemInts * it, stage[warp], lane);
        __syncthreads();
    }
}

void launch_chol_solve_cta(const CholArgs& a, int nbodies, cudaStream_t s) {
    if (nbodies > 0) k_chol_solve_cta<<<nbodies, kCtaSolveThreads, 0, s>>>(a);
}

// ---- one body per thread-block cluster: the cluster's warps stride over
// the items of a level, with a cluster barrier between levels.  The barrier
// (arrive with release, wait with acquire semantics at cluster scope) makes
// the level's global writes and atomics of every CTA of the cluster visible
// to all of them.  All CTAs of a cluster run the same level loops, so every
// thread arrives at every barrier; the hardware co-schedules the cluster.
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterSolveThreads)
    k_chol_solve_cluster(CholArgs a) {
    __shared__ float4 stage[kClusterSolveThreads / 32][32];
    if (a.done && *a.done) return;  // the flag is fixed for the kernel: uniform over the cluster
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    constexpr int kWarps = kClusterSolveThreads / 32;
    constexpr int kStride = kWarps * kClusterCtas;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gw = (int)cl.block_rank() * kWarps + warp;
    const int body = __ldg(&a.body_order[blockIdx.x / kClusterCtas]);
    const int L0 = __ldg(&a.body_level[body]), L1 = __ldg(&a.body_level[body + 1]);
    for (int L = L0; L < L1; ++L) {
        const int4 lv = __ldg(&a.levels[L]);
        for (int it = lv.x + gw; it < lv.y; it += kStride)
            fwd_warp_item(a, a.fwd_items + (size_t)kItemInts * it, stage[warp], lane);
        cl.sync();
    }
    for (int L = L1 - 1; L >= L0; --L) {
        const int4 lv = __ldg(&a.levels[L]);
        for (int it = lv.z + gw; it < lv.w; it += kStride)
            bwd_warp_item(a, a.bwd_items + (size_t)kItemInts * it, stage[warp], lane);
        cl.sync();
    }
}

void launch_chol_solve_cluster(const CholArgs& a, int nbodies, cudaStream_t s) {
    if (nbodies > 0) k_chol_solve_cluster<<<nbodies * kClusterCtas, kClusterSolveThreads, 0, s>>>(a);
}

// ---- one body per cluster, everything in the cluster's shared memory.
// Each CTA stages the M_s blocks and row lists of its supernodes (stored
// back to back per CTA by the plan: one float4-wide copy each), and
// holds the vector slots of vertices v with v % 8 == its rank.  The level
// loops run the warp items of the CTA's supernodes; right-hand side, y and x
// are read and updated in whichever CTA holds the vertex (distributed shared
// memory, float atomics for the forward updates); a cluster barrier
// separates levels.  Nothing but the staging and the final x touches global
// memory.
namespace {
namespace cg = cooperative_groups;

__device__ __forceinline__ float4* dsm_slot(cg::cluster_group& cl, float4* local, int v) {
    return cl.map_shared_rank(local + (v >> 3), (unsigned)(v & (kClusterCtas - 1)));
}

__device__ __forceinline__ void dsm_add(float4* p, float x, float y, float z) {
    atomicAdd(&p->x, x);
    atomicAdd(&p->y, y);
    atomicAdd(&p->z, z);
}

// cnt4 16-byte words from global to shared memory, the whole CTA at once
__device__ __forceinline__ void dsm_copy16(void* dst, const void* src, int cnt4) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4* d4 = reinterpret_cast<float4*>(dst);
    for (int t = threadIdx.x; t < cnt4; t += blockDim.x) d4[t] = __ldg(s4 + t);
}
}  // namespace

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterSolveThreads)
    k_chol_solve_dsm(CholArgs a, DsmArgs d) {
    extern __shared__ float4 dsm_base[];
    if (a.done && *a.done) return;  // the flag is fixed for the kernel: uniform over the cluster
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kClusterSolveThreads / 32;
    const int S = d.slots;
    float4* vr = dsm_base;
    float4* vy = vr + S;
    float4* vx = vy + S;
    float4* stage = vx + S + warp * 32;
    float* Ms = reinterpret_cast<float*>(dsm_base) + d.m_area;
    int* Rs = reinterpret_cast<int*>(dsm_base) + d.r_area;
    const int m0 = d.mcopy_ptr[rank], r0c = d.rcopy_ptr[rank];
    dsm_copy16(Ms, d.mcopy + m0, (d.mcopy_ptr[rank + 1] - m0) >> 2);
    dsm_copy16(Rs, d.rcopy + r0c, (d.rcopy_ptr[rank + 1] - r0c) >> 2);
    for (int j = threadIdx.x; j < S; j += blockDim.x) {
        const int v = j * kClusterCtas + rank;
        vr[j] = v < d.n ? a.r[v] : make_float4(0.f, 0.f, 0.f, 0.f);
        vy[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        vx[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    cl.sync();
    // forward: y_s = L_ss^-1 r_s (pivot rows), r_O -= L_os L_ss^-1 r_s
    for (int L = 0; L < d.nlevels; ++L) {
        const int4 lv = d.lvl[rank * d.nlevels + L];
        for (int it = lv.x + warp; it < lv.y; it += kWarps) {
            const int* w = d.items + (size_t)kItemInts * it;
            const int moff = w[0], m = w[2], k = w[3], r0 = w[4], c0 = w[5], c1 = w[6];
            const int* rows = Rs + w[1];
            const int row = r0 + lane;
            const bool valid = row < m;
            const int cend = !valid ? c0 : (row < k ? min(c1, row + 1) : c1);
            const float* Mr = Ms + moff + row;
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (int cb = c0; cb < c1; cb += 32) {
                const int nc = min(32, c1 - cb);
                __syncwarp();
                if (lane < nc) stage[lane] = *dsm_slot(cl, vr, rows[cb + lane]);
                __syncwarp();
                for (int c = cb; c < cb + nc; ++c) {
                    const float mv = c < cend ? Mr[(size_t)c * m] : 0.f;
                    const float4 v = stage[c - cb];
                    ax = fmaf(mv, v.x, ax);
                    ay = fmaf(mv, v.y, ay);
                    az = fmaf(mv, v.z, az);
                }
            }
            if (valid) {
                const int vid = rows[row];
                if (row < k) dsm_add(dsm_slot(cl, vy, vid), ax, ay, az);
                else dsm_add(dsm_slot(cl, vr, vid), -ax, -ay, -az);
            }
        }
        cl.sync();
    }
    // backward: x_s = sum_{i >= c} M_s[i, c] z_i, z = [y_pivots ; -x_offdiag]
    for (int L = d.nlevels - 1; L >= 0; --L) {
        const int4 lv = d.lvl[rank * d.nlevels + L];
        for (int it = lv.z + warp; it < lv.w; it += kWarps) {
            const int* w = d.items + (size_t)kItemInts * it;
            const int moff = w[0], m = w[2], k = w[3], c = w[4];
            const int* rows = Rs + w[1];
            const float* Mc = Ms + moff + (size_t)c * m;
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (int i = c + lane; i < m; i += 32) {
                const int vid = rows[i];
                const float mv = Mc[i];
                float4 z;
                if (i < k) {
                    z = *dsm_slot(cl, vy, vid);
                } else {
                    const float4 xv = *dsm_slot(cl, vx, vid);
                    z = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
                }
                ax = fmaf(mv, z.x, ax);
                ay = fmaf(mv, z.y, ay);
                az = fmaf(mv, z.z, az);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                ax += __shfl_xor_sync(0xffffffffu, ax, off);
                ay += __shfl_xor_sync(0xffffffffu, ay, off);
                az += __shfl_xor_sync(0xffffffffu, az, off);
            }
            if (lane == 0) *dsm_slot(cl, vx, rows[c]) = make_float4(ax, ay, az, 0.f);
        }
        cl.sync();
    }
    for (int j = threadIdx.x; j < S; j += blockDim.x) {
        const int v = j * kClusterCtas + rank;
        if (v < d.n) a.x[v] = vx[j];
    }
}

void launch_chol_solve_dsm(const CholArgs& a, const DsmArgs& d, size_t smem_bytes, cudaStream_t s) {
    static size_t allowed = 0;
    if (smem_bytes > allowed) {
        PDGB_CUDA_TRY(cudaFuncSetAttribute(k_chol_solve_dsm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes));
        allowed = smem_bytes;
    }
    k_chol_solve_dsm<<<kClusterCtas, kClusterSolveThreads, smem_bytes, s>>>(a, d);
}

// Cholesky-path vertex kernel after each solve (new positions in sn, written
// by the backward pass): resets b for the next local step (pinned vertices
// get the pin RHS: computeDBCLocal overwrites b, pdUtil.cu:153-158), clears
// y, and with tol > 0 runs the reference's convergence test
// (computeError, pdSolver.cu:186-191, 243-253): err = mean over the 3n
// coordinates of (sn - prev)^2, prev = sn, stop when sqrt(err) < tol.  The
// last block to finish evaluates the test and sets st->done, which makes
// every later kernel of the step return at entry.
__global__ void __launch_bounds__(256) k_chol_vertex(CholVertexArgs a) {
    __shared__ float red[8];
    __shared__ bool last;
    if (a.st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (i < a.nv) {
        const float4 s = a.sn[i];
        a.y[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 cf = __ldg(&a.coef[i]);
        a.b[i] = cf.z != 0.f ? __ldg(&a.pin_rhs[i]) : __ldg(&a.base[i]);
        if (a.tol > 0.f) {
            const float4 p = a.prev[i];
            const float dx = p.x - s.x, dy = p.y - s.y, dz = p.z - s.z;
            e = dx * dx + dy * dy + dz * dz;
            a.prev[i] = s;
        }
    }
    if (a.tol <= 0.f) return;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) e += __shfl_xor_sync(0xffffffffu, e, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        float blk = 0.f;
        for (int w = 0; w < 8; ++w) blk += red[w];
        atomicAdd(&a.st->err_acc, blk);
        __threadfence();
        last = atomicAdd(&a.st->count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const float total = atomicAdd(&a.st->err_acc, 0.0f);
        const float err = (float)((double)total / (3.0 * (double)a.nv));
        if (!(sqrtf(err) >= a.tol)) {
            a.st->done = 1;
            a.st->iterations = a.iteration + 1;
        }
        a.st->err_acc = 0.f;
        a.st->count = 0u;
    }
}

// Multi-request forms (serving, fixed iteration count): CTA i takes 256
// vertices of request list[i].x from list[i].y.
__global__ void __launch_bounds__(256) k_chol_vertex_multi(const CholVertexArgs* __restrict__ req,
                                                           const int2* __restrict__ list,
                                                           const int* __restrict__ count) {
    if ((int)blockIdx.x >= *count) return;
    const int2 w = list[blockIdx.x];
    const CholVertexArgs& a = req[w.x];
    const int i = w.y + threadIdx.x;
    if (i >= a.nv) return;
    a.y[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 cf = __ldg(&a.coef[i]);
    a.b[i] = cf.z != 0.f ? __ldg(&a.pin_rhs[i]) : __ldg(&a.base[i]);
}

__global__ void __launch_bounds__(256) k_chol_finish_multi(const CholVertexArgs* __restrict__ req,
                                                           const int2* __restrict__ list,
                                                           const int* __restrict__ count) {
    if ((int)blockIdx.x >= *count) return;
    const int2 w = list[blockIdx.x];
    const CholVertexArgs& a = req[w.x];
    const int i = w.y + threadIdx.x;
    if (i >= a.nv) return;
    finish_vertex(a.sc, i, a.sn[i], a.dt_inv, a.x, a.v);
    a.y[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

void launch_chol_vertex_multi(const CholVertexArgs* req, const int2* list, const int* count, int grid,
                              cudaStream_t s) {
    if (grid > 0) k_chol_vertex_multi<<<grid, 256, 0, s>>>(req, list, count);
}

void launch_chol_finish_multi(const CholVertexArgs* req, const int2* list, const int* count, int grid,
                              cudaStream_t s) {
    if (grid > 0) k_chol_finish_multi<<<grid, 256, 0, s>>>(req, list, count);
}

// After the iterations: velocity / position update (updateVelPos,
// pdUtil.cu:180-193), X <- XTilde (pdSolver.cu:227) and the fixed-body
// correction of XTilde and V (pdSolver.cu:228-231).
__global__ void __launch_bounds__(256) k_chol_finish(CholVertexArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nv) return;
    finish_vertex(a.sc, i, a.sn[i], a.dt_inv, a.x, a.v);
    a.y[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---- iterative refinement
__global__ void __launch_bounds__(256) k_copy_rhs(int nv, const float4* __restrict__ b, float4* bsave,
                                                  const int* done) {
    if (done && *done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) bsave[i] = b[i];
}

// One warp per row: r = bsave - K x0 accumulated in double over the row's
// nonzeros (lanes stride the row, then a warp reduction).
__global__ void __launch_bounds__(256) k_refine_residual(RefineArgs a) {
    if (a.done && *a.done) return;
    const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= a.nv) return;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int e = __ldg(&a.rowptr[row]) + lane; e < __ldg(&a.rowptr[row + 1]); e += 32) {
        const double kv = __ldg(&a.val[e]);
        const float4 xv = a.x0[__ldg(&a.colind[e])];
        sx = fma(kv, (double)xv.x, sx);
        sy = fma(kv, (double)xv.y, sy);
        sz = fma(kv, (double)xv.z, sz);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
        sz += __shfl_xor_sync(0xffffffffu, sz, off);
    }
    if (lane == 0) {
        const float4 b = a.bsave[row];
        a.b[row] = make_float4((float)((double)b.x - sx), (float)((double)b.y - sy), (float)((double)b.z - sz), 0.f);
        a.y[row] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void __launch_bounds__(256) k_refine_update(RefineArgs a) {
    if (a.done && *a.done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nv) return;
    const float4 x = a.x[i], d = a.dx[i];
    a.x[i] = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, 0.f);
}

void launch_copy_rhs(int nv, const float4* b, float4* bsave, const int* done, cudaStream_t s) {
    if (nv > 0) k_copy_rhs<<<(nv + 255) / 256, 256, 0, s>>>(nv, b, bsave, done);
}
void launch_refine_residual(const RefineArgs& a, cudaStream_t s) {
    if (a.nv > 0) k_refine_residual<<<(a.nv + 7) / 8, 256, 0, s>>>(a);
}
void launch_refine_update(const RefineArgs& a, cudaStream_t s) {
    if (a.nv > 0) k_refine_update<<<(a.nv + 255) / 256, 256, 0, s>>>(a);
}

void launch_chol_vertex(const CholVertexArgs& a, cudaStream_t s) {
    const int blocks = (a.nv + 255) / 256;
    if (blocks) k_chol_vertex<<<blocks, 256, 0, s>>>(a);
}

void launch_chol_finish(const CholVertexArgs& a, cudaStream_t s) {
    const int blocks = (a.nv + 255) / 256;
    if (blocks) k_chol_finish<<<blocks, 256, 0, s>>>(a);
}

}  // namespace pdgb
