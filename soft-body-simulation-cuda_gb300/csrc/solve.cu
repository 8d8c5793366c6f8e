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

namespace pdgb {

// Forward item (s, r0, r1, c0 | c1 << 16): rows r0..r1 of M_s times the
// right-hand side of the pivot columns c0..c1.  Pivot rows accumulate into y,
// off-diagonal rows subtract from r (ancestor columns, solved at a later level).
__global__ void __launch_bounds__(kFwdThreads) k_chol_forward(CholArgs a, int item0) {
    __shared__ float4 rs[kFwdCols];
    if (a.done && *a.done) return;
    const int4 it = __ldg(reinterpret_cast<const int4*>(a.fwd_items) + item0 + blockIdx.x);
    const int s = it.x, r0 = it.y, r1 = it.z, c0 = it.w & 0xffff, c1 = it.w >> 16;
    const int k = __ldg(&a.sk[s]), m = __ldg(&a.sm[s]);
    const int* rows = a.rows + __ldg(&a.roff[s]);
    const float* M = a.mval + __ldg(&a.moff[s]);
    for (int c = c0 + threadIdx.x; c < c1; c += kFwdThreads) rs[c - c0] = a.r[__ldg(&rows[c])];
    __syncthreads();
    const int row = r0 + threadIdx.x;
    if (row >= r1) return;
    // inverse of the lower-triangular pivot block is lower triangular
    const int cend = row < k ? min(c1, row + 1) : c1;
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float* Mr = M + row;
#pragma unroll 4
    for (int c = c0; c < cend; ++c) {
        const float mv = __ldg(Mr + (size_t)c * m);
        const float4 v = rs[c - c0];
        ax = fmaf(mv, v.x, ax);
        ay = fmaf(mv, v.y, ay);
        az = fmaf(mv, v.z, az);
    }
    const int vid = __ldg(&rows[row]);
    if (row < k) atomicAdd(&a.y[vid], make_float4(ax, ay, az, 0.f));
    else atomicAdd(&a.r[vid], make_float4(-ax, -ay, -az, 0.f));
}

// Backward item (s, c0, c1): x[pivot c] = sum_i M_s[i, c] z_i with
// z = [y_pivots ; -x_offdiag], one warp per column, z staged in shared
// memory in chunks of kBwdChunk rows.
__global__ void __launch_bounds__(kBwdThreads) k_chol_backward(CholArgs a, int item0) {
    __shared__ float4 zs[kBwdChunk];
    if (a.done && *a.done) return;
    const int4 it = __ldg(reinterpret_cast<const int4*>(a.bwd_items) + item0 + blockIdx.x);
    const int s = it.x, c0 = it.y, c1 = it.z;
    const int k = __ldg(&a.sk[s]), m = __ldg(&a.sm[s]);
    const int* rows = a.rows + __ldg(&a.roff[s]);
    const float* M = a.mval + __ldg(&a.moff[s]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kBwdThreads / 32;
    constexpr int kPer = (kBwdColsPerItem + kWarps - 1) / kWarps;
    float acc[kPer][3];
#pragma unroll
    for (int q = 0; q < kPer; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.f;
    // rows below c0 are zero in every column of this item (lower triangle)
    for (int base = c0; base < m; base += kBwdChunk) {
        const int nrow = min(kBwdChunk, m - base);
        __syncthreads();
        for (int i = threadIdx.x; i < nrow; i += kBwdThreads) {
            const int g = base + i;
            const int vid = __ldg(&rows[g]);
            if (g < k) zs[i] = a.y[vid];
            else {
                const float4 xv = a.x[vid];
                zs[i] = make_float4(-xv.x, -xv.y, -xv.z, 0.f);
            }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int c = c0 + warp + q * kWarps;
            if (c >= c1) continue;
            const float* Mc = M + (size_t)c * m;
            const int i0 = max(c, base);
            for (int g = i0 + lane; g < base + nrow; g += 32) {
                const float mv = __ldg(Mc + g);
                const float4 z = zs[g - base];
                acc[q][0] = fmaf(mv, z.x, acc[q][0]);
                acc[q][1] = fmaf(mv, z.y, acc[q][1]);
                acc[q][2] = fmaf(mv, z.z, acc[q][2]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int c = c0 + warp + q * kWarps;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            acc[q][0] += __shfl_xor_sync(0xffffffffu, acc[q][0], off);
            acc[q][1] += __shfl_xor_sync(0xffffffffu, acc[q][1], off);
            acc[q][2] += __shfl_xor_sync(0xffffffffu, acc[q][2], off);
        }
        if (lane == 0 && c < c1) a.x[__ldg(&rows[c])] = make_float4(acc[q][0], acc[q][1], acc[q][2], 0.f);
    }
}

void launch_chol_solve(const CholArgs& a, const std::vector<SolveLevel>& levels, cudaStream_t s) {
    for (size_t L = 0; L < levels.size(); ++L) {
        const int n = levels[L].fwd_end - levels[L].fwd_begin;
        if (n > 0) k_chol_forward<<<n, kFwdThreads, 0, s>>>(a, levels[L].fwd_begin);
    }
    for (size_t L = levels.size(); L-- > 0;) {
        const int n = levels[L].bwd_end - levels[L].bwd_begin;
        if (n > 0) k_chol_backward<<<n, kBwdThreads, 0, s>>>(a, levels[L].bwd_begin);
    }
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

// After the iterations: velocity / position update (updateVelPos,
// pdUtil.cu:180-193) and X <- XTilde (pdSolver.cu:227).
__global__ void __launch_bounds__(256) k_chol_finish(CholVertexArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nv) return;
    const float4 s = a.sn[i];
    const float4 xo = a.x[i];
    a.v[i] = make_float4((s.x - xo.x) * a.dt_inv, (s.y - xo.y) * a.dt_inv, (s.z - xo.z) * a.dt_inv, 0.f);
    a.x[i] = s;
    a.y[i] = make_float4(0.f, 0.f, 0.f, 0.f);
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
