// FP64 numeric factorisation of the PD system on the GPU (supernodal,
// multifrontal), run once per system matrix.
//
// The reference factors A = K (x) I_3 on the GPU with cuSOLVER's low-level
// sparse Cholesky in FP32 (cusolverSpScsrcholFactor, cholesky.cu:152-157).
// Here the scalar K is factored in FP64 with the engine's own dense kernels,
// level by level of the supernodal elimination tree (leaves first; all
// bodies of a batch together), and the result is stored as the FP32 blocks
// M_s = [L_ss^-1 ; L_os L_ss^-1] that the triangular solves use (solve.cu).
//
// Per level:
//   k_fz     zero the level's fronts (memory of finished fronts is reused)
//   k_fk     entries of K in the pivot columns of each front
//   k_fea    extend-add: the children's Schur complements into the front
//   per panel of 32 pivot columns:
//     k_fdiag  Cholesky of the 32 x 32 diagonal block (one warp per front)
//     k_fpanel the panel rows below it: L_i = A_i L_jj^-T
//     k_ftrail trailing update of the lower triangle, 32 x 32 tiles
//   k_fm     M_s = [I ; L_os] L_ss^-1, rows independent, by column blocks
//            from the right; FP64 in the pool, FP32 into mval
// A non-positive pivot is recorded in a status word; the host raises
// PDGB_ERR_NOT_SPD after the last level.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "cholesky.h"
#include "engine.h"

namespace pdgb {
namespace {

constexpr int kNB = 32;           // panel width and tile size
constexpr int kRowChunk = 256;    // panel rows per CTA
constexpr int kZeroChunk = 1 << 16;

struct FDev {
    double* pool;
    const int64_t* foff;
    const int* sk;
    const int* sm;
    const int64_t* moff;
    float* mval;
    const int* child_ptr;
    const int* child;
    const int* rel_ptr;
    const int* rel;
    const int* kptr;
    const int* kpos;
    const double* kval;
    int* status;
};

__device__ __forceinline__ int lower_bound_dev(const int* a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Zeroes the front and M_s block of list[blockIdx.x], kZeroChunk doubles per CTA.
__global__ void __launch_bounds__(256) k_fz(FDev d, const int* __restrict__ list) {
    const int s = list[blockIdx.x];
    const int64_t m = d.sm[s], k = d.sk[s];
    const int64_t tot = m * m + m * k;
    const int64_t b0 = (int64_t)blockIdx.y * kZeroChunk;
    if (b0 >= tot) return;
    const int64_t b1 = b0 + kZeroChunk < tot ? b0 + kZeroChunk : tot;
    double* F = d.pool + d.foff[s];
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) F[i] = 0.0;
}

// Entries of K in the pivot columns (positions are distinct within a front).
__global__ void __launch_bounds__(256) k_fk(FDev d, const int* __restrict__ list) {
    const int s = list[blockIdx.x];
    double* F = d.pool + d.foff[s];
    for (int i = d.kptr[s] + threadIdx.x; i < d.kptr[s + 1]; i += blockDim.x) F[d.kpos[i]] += d.kval[i];
}

// Extend-add of the children's Schur complements (lower triangles) into the
// front, parent columns [32 y, 32 y + 32) per CTA, children one after the
// other: no two threads ever add into the same entry at once.
__global__ void __launch_bounds__(256) k_fea(FDev d, const int* __restrict__ list) {
    const int s = list[blockIdx.x];
    const int mp = d.sm[s];
    const int j0 = blockIdx.y * kNB;
    if (j0 >= mp) return;
    const int j1 = min(mp, j0 + kNB);
    double* Fp = d.pool + d.foff[s];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int ci = d.child_ptr[s]; ci < d.child_ptr[s + 1]; ++ci) {
        const int c = d.child[ci];
        const int kc = d.sk[c], mc = d.sm[c], uc = mc - kc;
        const int* rc = d.rel + d.rel_ptr[c];  // ascending positions in the parent's rows
        const double* Fc = d.pool + d.foff[c];
        const int b0 = lower_bound_dev(rc, uc, j0), b1 = lower_bound_dev(rc, uc, j1);
        for (int b = b0 + warp; b < b1; b += nw) {
            double* dst = Fp + (int64_t)rc[b] * mp;
            const double* src = Fc + (int64_t)(kc + b) * mc + kc;
            for (int a = b + lane; a < uc; a += 32) dst[rc[a]] += src[a];
        }
        __syncthreads();
    }
}

// Cholesky of the diagonal block [j0, j0 + nb) of each front with more than
// j0 pivots: one warp per front, lane = row, the block in shared memory.
__global__ void __launch_bounds__(32) k_fdiag(FDev d, const int* __restrict__ list, int j0) {
    const int s = list[blockIdx.x];
    const int k = d.sk[s], m = d.sm[s];
    if (j0 >= k) return;
    const int nb = min(kNB, k - j0);
    double* F = d.pool + d.foff[s] + (int64_t)j0 * m + j0;  // F[c m + r] = A[j0 + r][j0 + c]
    __shared__ double D[kNB][kNB + 1];
    const int lane = threadIdx.x;
    for (int c = 0; c < kNB; ++c) D[lane][c] = (lane < nb && c <= lane) ? F[(int64_t)c * m + lane] : 0.0;
    __syncwarp();
    bool bad = false;
    for (int j = 0; j < nb; ++j) {
        double l = D[j][j];
        if (!(l > 0.0) || !isfinite(l)) {
            bad = true;
            l = 1.0;
        } else {
            l = sqrt(l);
        }
        __syncwarp();
        if (lane == j) D[j][j] = l;
        if (lane > j && lane < nb) D[lane][j] /= l;
        __syncwarp();
        if (lane > j && lane < nb) {
            const double a = D[lane][j];
            for (int c = j + 1; c <= lane; ++c) D[lane][c] = fma(-a, D[c][j], D[lane][c]);
        }
        __syncwarp();
    }
    if (bad && lane == 0) atomicCAS(d.status, 0, s + 1);
    if (lane < nb)
        for (int c = 0; c <= lane; ++c) F[(int64_t)c * m + lane] = D[lane][c];
}

// Panel rows below the diagonal block: row i of L over columns
// [j0, j0 + nb) solves x L_jj^T = A[i, j0 : j0 + nb]; items {s, first row}.
__global__ void __launch_bounds__(kRowChunk) k_fpanel(FDev d, const int2* __restrict__ items, int j0) {
    const int2 it = items[blockIdx.x];
    const int s = it.x;
    const int k = d.sk[s], m = d.sm[s];
    const int nb = min(kNB, k - j0);
    double* F = d.pool + d.foff[s];
    __shared__ double D[kNB][kNB + 1];
    for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
        const int r = e % kNB, c = e / kNB;
        D[r][c] = (r < nb && c <= r) ? F[(int64_t)(j0 + c) * m + j0 + r] : 0.0;
    }
    __syncthreads();
    const int i = it.y + threadIdx.x;
    if (i >= m) return;
    double x[kNB];
#pragma unroll
    for (int j = 0; j < kNB; ++j) {
        if (j < nb) {
            double v = F[(int64_t)(j0 + j) * m + i];
#pragma unroll
            for (int q = 0; q < j; ++q) v = fma(-x[q], D[j][q], v);
            x[j] = v / D[j][j];
            F[(int64_t)(j0 + j) * m + i] = x[j];
        }
    }
}

// Trailing update of the panel over the lower triangle past it:
// A[r][c] -= sum_q L[r][j0 + q] L[c][j0 + q] for r >= c >= j0 + nb, one
// 32 x 32 tile per CTA; items {s, tile}, tile t = ti (ti + 1) / 2 + tj.
__global__ void __launch_bounds__(256) k_ftrail(FDev d, const int2* __restrict__ items, int j0) {
    const int2 it = items[blockIdx.x];
    const int s = it.x;
    const int k = d.sk[s], m = d.sm[s];
    const int nb = min(kNB, k - j0);
    const int j1 = j0 + nb;
    int ti = (int)((sqrt(8.0 * (double)it.y + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= it.y) ++ti;
    while (ti * (ti + 1) / 2 > it.y) --ti;
    const int tj = it.y - ti * (ti + 1) / 2;
    const int r0 = j1 + kNB * ti, c0 = j1 + kNB * tj;
    double* F = d.pool + d.foff[s];
    __shared__ double Lr[kNB][kNB + 1], Lc[kNB][kNB + 1];
    for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
        const int r = e % kNB, q = e / kNB;
        const bool okq = q < nb;
        Lr[r][q] = (okq && r0 + r < m) ? F[(int64_t)(j0 + q) * m + r0 + r] : 0.0;
        Lc[r][q] = (okq && c0 + r < m) ? F[(int64_t)(j0 + q) * m + c0 + r] : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x & 31, cb = threadIdx.x >> 5;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < nb; ++q) {
        const double a = Lr[r][q];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fma(a, Lc[cb + 8 * u][q], acc[u]);
    }
    const int gr = r0 + r;
    if (gr >= m) return;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int gc = c0 + cb + 8 * u;
        if (gc < m && gc <= gr) F[(int64_t)gc * m + gr] -= acc[u];
    }
}

// M_s = B L_ss^-1 with B = [I_k ; L_os] (m x k): each row x of M_s solves
// x L_ss = b, by blocks of 32 columns from the right,
//   X[:, J] = (B[:, J] - X[:, J+1:] L[J+1:, J]) L_JJ^-1,
// for the 32 rows {s, r0} of the item.  X is kept in FP64 in the block
// after the front (zeroed with it) and written to mval in FP32.  Rows below
// k are rows of L_ss^-1, which vanish right of the diagonal: those blocks
// are skipped.
__global__ void __launch_bounds__(256) k_fm(FDev d, const int2* __restrict__ items) {
    const int2 it = items[blockIdx.x];
    const int s = it.x, r0 = it.y;
    const int k = d.sk[s], m = d.sm[s];
    const double* F = d.pool + d.foff[s];
    double* X = d.pool + d.foff[s] + (int64_t)m * m;
    float* M = d.mval + d.moff[s];
    __shared__ double Xs[kNB][kNB + 1];
    __shared__ double Xq[kNB][kNB + 1];
    __shared__ double Lq[kNB][kNB + 1];
    const int nbk = (k + kNB - 1) / kNB;
    // last column that can be nonzero in these rows
    const int cmax = r0 + kNB <= k ? r0 + kNB - 1 : k - 1;
    const int jtop = cmax / kNB;
    const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
    const int row = r0 + tr;
    for (int J = min(nbk - 1, jtop); J >= 0; --J) {
        const int c0 = J * kNB, cn = min(kNB, k - c0);
        double acc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int col = c0 + tc + 8 * u;
            double b = 0.0;
            if (col < k && row < m) b = row < k ? (row == col ? 1.0 : 0.0) : F[(int64_t)col * m + row];
            acc[u] = b;
        }
        for (int Q = J + 1; Q <= min(nbk - 1, jtop); ++Q) {
            const int q0 = Q * kNB, qn = min(kNB, k - q0);
            __syncthreads();
            for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
                const int rr = e % kNB, cc = e / kNB;
                Xq[rr][cc] = (r0 + rr < m && cc < qn) ? X[(int64_t)(q0 + cc) * m + r0 + rr] : 0.0;
                Lq[rr][cc] = (rr < qn && cc < cn) ? F[(int64_t)(c0 + cc) * m + q0 + rr] : 0.0;  // L[q0 + rr][c0 + cc]
            }
            __syncthreads();
            for (int q = 0; q < qn; ++q) {
                const double xv = Xq[tr][q];
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[u] = fma(-xv, Lq[q][tc + 8 * u], acc[u]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 4; ++u) Xs[tr][tc + 8 * u] = acc[u];
        for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
            const int rr = e % kNB, cc = e / kNB;
            Lq[rr][cc] = (rr < cn && cc <= rr) ? F[(int64_t)(c0 + cc) * m + c0 + rr] : 0.0;  // L_JJ
        }
        __syncthreads();
        if (threadIdx.x < kNB) {
            for (int j = cn - 1; j >= 0; --j) {
                double v = Xs[tr][j];
                for (int q = j + 1; q < cn; ++q) v = fma(-Xs[tr][q], Lq[q][j], v);
                Xs[tr][j] = v / Lq[j][j];
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int col = c0 + tc + 8 * u;
            if (col < k && row < m) {
                const double v = Xs[tr][tc + 8 * u];
                X[(int64_t)col * m + row] = v;
                M[(int64_t)col * m + row] = (float)v;
            }
        }
    }
}

template <class T> void put(DBuf<T>& b, const std::vector<T>& h, cudaStream_t s) {
    b.alloc(std::max<size_t>(h.size(), 1));
    if (!h.empty()) PDGB_CUDA_TRY(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

double gpu_factor(const CholFactor& f, float* mval, void* stream) {
    const FrontPlan& P = f.fp;
    if (!P.on) throw Error{PDGB_ERR_INVALID_ARGUMENT, "gpu_factor: no front plan"};
    cudaStream_t s = (cudaStream_t)stream;
    const int ns = f.nsuper;
    const int nl = (int)P.lvl_ptr.size() - 1;
    // ---- launch lists, built on the host and uploaded at once
    struct Launch {
        int kind;        // 0 level start (zero / K / extend-add), 1 panel, 2 M_s
        int level;
        int j0;
        size_t i0, n0;   // panel rows items, or M_s items
        size_t i1, n1;   // trailing tiles
        int ychunks, ycols;
    };
    std::vector<Launch> plan;
    std::vector<int2> items;
    for (int L = 0; L < nl; ++L) {
        const int a = P.lvl_ptr[L], b = P.lvl_ptr[L + 1];
        int64_t max_tot = 0;
        int max_m = 0, max_k = 0;
        for (int q = a; q < b; ++q) {
            const int sn = P.lvl_sn[q];
            max_tot = std::max<int64_t>(max_tot, front_doubles(f, sn));
            max_m = std::max(max_m, f.sm[sn]);
            max_k = std::max(max_k, f.sk[sn]);
        }
        Launch st{0, L, 0, 0, 0, 0, 0, (int)((max_tot + kZeroChunk - 1) / kZeroChunk), (max_m + kNB - 1) / kNB};
        plan.push_back(st);
        for (int j0 = 0; j0 < max_k; j0 += kNB) {
            Launch pl{1, L, j0, items.size(), 0, 0, 0, 0, 0};
            for (int q = a; q < b; ++q) {
                const int sn = P.lvl_sn[q], k = f.sk[sn], m = f.sm[sn];
                if (k <= j0) continue;
                const int j1 = j0 + std::min(kNB, k - j0);
                for (int r = j1; r < m; r += kRowChunk) items.push_back(make_int2(sn, r));
            }
            pl.n0 = items.size() - pl.i0;
            pl.i1 = items.size();
            for (int q = a; q < b; ++q) {
                const int sn = P.lvl_sn[q], k = f.sk[sn], m = f.sm[sn];
                if (k <= j0) continue;
                const int j1 = j0 + std::min(kNB, k - j0);
                if (m <= j1) continue;
                const int64_t T = (m - j1 + kNB - 1) / kNB;
                for (int64_t t = 0; t < T * (T + 1) / 2; ++t) items.push_back(make_int2(sn, (int)t));
            }
            pl.n1 = items.size() - pl.i1;
            plan.push_back(pl);
        }
        Launch mm{2, L, 0, items.size(), 0, 0, 0, 0, 0};
        for (int q = a; q < b; ++q) {
            const int sn = P.lvl_sn[q];
            for (int r = 0; r < f.sm[sn]; r += kNB) items.push_back(make_int2(sn, r));
        }
        mm.n0 = items.size() - mm.i0;
        plan.push_back(mm);
    }
    // ---- device data
    DBuf<double> pool, kval;
    DBuf<int64_t> foff, moff;
    DBuf<int> sk, sm, cptr, child, rptr, rel, kptr, kpos, lvl, status;
    DBuf<int2> ditems;
    pool.alloc((size_t)std::max<int64_t>(P.pool, 1));
    put(foff, P.foff, s);
    put(moff, std::vector<int64_t>(f.moff.begin(), f.moff.begin() + ns), s);
    put(sk, f.sk, s);
    put(sm, f.sm, s);
    put(cptr, P.child_ptr, s);
    put(child, P.child, s);
    put(rptr, P.rel_ptr, s);
    put(rel, P.rel, s);
    put(kptr, P.kptr, s);
    put(kpos, P.kpos, s);
    put(kval, P.kval, s);
    put(lvl, P.lvl_sn, s);
    put(ditems, items, s);
    status.alloc(1);
    PDGB_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    PDGB_CUDA_TRY(cudaMemsetAsync(mval, 0, (size_t)f.mval_size * sizeof(float), s));
    FDev d{pool.p, foff.p, sk.p, sm.p, moff.p, mval, cptr.p, child.p, rptr.p, rel.p, kptr.p, kpos.p, kval.p, status.p};
    cudaEvent_t ev[2];
    PDGB_CUDA_TRY(cudaEventCreate(&ev[0]));
    PDGB_CUDA_TRY(cudaEventCreate(&ev[1]));
    float ms = 0.f;
    cudaError_t err = cudaEventRecord(ev[0], s);
    for (const Launch& l : plan) {
        if (err != cudaSuccess) break;
        const int a = P.lvl_ptr[l.level], nf = P.lvl_ptr[l.level + 1] - a;
        const int* list = lvl.p + a;
        if (l.kind == 0) {
            k_fz<<<dim3(nf, l.ychunks), 256, 0, s>>>(d, list);
            k_fk<<<nf, 256, 0, s>>>(d, list);
            k_fea<<<dim3(nf, l.ycols), 256, 0, s>>>(d, list);
        } else if (l.kind == 1) {
            k_fdiag<<<nf, 32, 0, s>>>(d, list, l.j0);
            if (l.n0) k_fpanel<<<(unsigned)l.n0, kRowChunk, 0, s>>>(d, ditems.p + l.i0, l.j0);
            if (l.n1) k_ftrail<<<(unsigned)l.n1, 256, 0, s>>>(d, ditems.p + l.i1, l.j0);
        } else {
            if (l.n0) k_fm<<<(unsigned)l.n0, 256, 0, s>>>(d, ditems.p + l.i0);
        }
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaEventRecord(ev[1], s);
    if (err == cudaSuccess) err = cudaEventSynchronize(ev[1]);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    PDGB_CUDA_TRY(err);
    int bad = 0;
    PDGB_CUDA_TRY(cudaMemcpy(&bad, status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad)
        throw Error{PDGB_ERR_NOT_SPD, "system matrix is not positive definite (supernode " + std::to_string(bad - 1) + ")"};
    return (double)ms;
}

}  // namespace pdgb
