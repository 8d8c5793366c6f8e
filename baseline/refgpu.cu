// The reference's float PD step on the GPU, restated kernel for kernel so
// that it can be timed on the same GPU as the engine.  It is a baseline, not
// part of the engine: nothing in libpdgb.so calls it.
//
// The reference's own sources are not present where the GPU runs, so this
// file restates its GPU path (PdSolver::SolverStep + Update,
// src/simulation/solver/projective/pdSolver.cu:141-232) with the same
// structure and the same libraries:
//   - one thread per vertex or per tet, 128 threads per block
//     (src/context.cpp:331), the legacy default stream, synchronous copies;
//   - computeLocal: per-tet gather of 4 vertices from the interleaved
//     float[3n] iterate, F = Ds DmInv, R from a 4-sweep McAdams SVD, 12
//     scalar float atomics into b (pdUtil.cu:97-145);
//   - the global solve either as getErrorKern + chebyshevKern with the
//     host-side omega schedule (pdUtil.cu:195-226, pdSolver.cu:193-200), or
//     as cuSOLVER's low-level sparse Cholesky on the 3n x 3n FP32 system:
//     csrsymamd ordering and csrperm on the host, csrcholAnalysis /
//     BufferInfo / Factor on the GPU once, then per iteration permute,
//     cusolverSpScsrcholSolve, inverse permute (cholesky.cu:72-192);
//   - computeError after every Cholesky solve: a reduction whose result is
//     read on the host, which synchronises every iteration
//     (pdSolver.cu:186-191,243-253).
// The system matrix is assembled on the host (in double, stored as float)
// with the entries computeSiTSi and setMDt_2 emit (pdUtil.cu:9-54),
// duplicates summed as sort_coo does (linear.cu:6-40); set-up is not timed.
#include <cuda_runtime.h>
#include <cusolverSp.h>
#include <cusolverSp_LOWLEVEL_PREVIEW.h>
#include <cusparse.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "rotation.cuh"

namespace {

constexpr int kThreads = 128;
thread_local std::string g_err;

int fail(const std::string& what) {
    g_err = what;
    return 1;
}

#define RG_CUDA(x)                                                                   \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define RG_SOLVER(x)                                                                  \
    do {                                                                              \
        cusolverStatus_t s_ = (x);                                                    \
        if (s_ != CUSOLVER_STATUS_SUCCESS) return fail(std::string(#x) + ": status " + std::to_string((int)s_)); \
    } while (0)

struct RefGpu {
    int nv = 0, nt = 0, n3 = 0, ndbc = 0;
    bool cholesky = false;
    float dt = 0, gravity = 0, tol = 0, rho = 0, pw = 0;
    int iters = 0;
    // SolverData (def.h:21-56): vec3 arrays as float[3n]
    float *X = nullptr, *V = nullptr, *XTilde = nullptr, *DBCX = nullptr, *OffsetX = nullptr, *force = nullptr;
    float *mass = nullptr, *dbc = nullptr, *more = nullptr, *V0 = nullptr, *w = nullptr, *DmInv = nullptr;
    uint32_t* tet = nullptr;
    // PdSolver scratch (pdSolver.cu:29-38)
    float *sn = nullptr, *sn_old = nullptr, *b = nullptr, *next_x = nullptr, *prev_x = nullptr, *mdt2 = nullptr,
          *diag = nullptr, *err = nullptr;
    // CholeskySpLinearSolver (cholesky.cu:72-192)
    cusolverSpHandle_t sp = nullptr;
    cusparseMatDescr_t descr = nullptr;
    csrcholInfo_t info = nullptr;
    int *rowptr = nullptr, *col = nullptr, *perm = nullptr;
    float *val = nullptr, *bp = nullptr, *xp = nullptr;
    void* buf = nullptr;
    int nnz = 0;
    long long last_iterations = 0;
};

// ---- per-step kernels (pdUtil.cu), one thread per vertex / tet / dof
__global__ void k_gravity(int nv, const float* mass, float g, float* f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) {
        f[3 * i] = 0.f;
        f[3 * i + 1] = -g * mass[i];
        f[3 * i + 2] = 0.f;
    }
}

__global__ void k_set_mdt2_more(int nv, const float* mass, float dt2, float* mdt2, const float* more, const float* dbc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv && dbc[i] == 0.f) {
        const float wi = more[i];
        mdt2[i] = wi > 0.f ? (mass[i] + wi) / dt2 : mass[i] / dt2;
    }
}

__global__ void k_compute_sn(int nv, float* sn, float dt, const float* mdt2, const float* X, const float* V,
                             const float* f, const float* more, const float* offset, float* DBCX) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    if (more[i] > 0.f) {
        // drag target = offset (the mouse target is the origin here)
        for (int k = 0; k < 3; ++k) {
            sn[3 * i + k] = offset[3 * i + k];
            DBCX[3 * i + k] = offset[3 * i + k];
        }
    } else {
        const float r = 1.0f / mdt2[i];
        for (int k = 0; k < 3; ++k) sn[3 * i + k] = X[3 * i + k] + dt * V[3 * i + k] + r * f[3 * i + k];
    }
}

__global__ void k_add_mh2_sn(float* b, const float* sn, const float* mdt2, int nv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) {
        const float m = mdt2[i];
        b[3 * i] = m * sn[3 * i];
        b[3 * i + 1] = m * sn[3 * i + 1];
        b[3 * i + 2] = m * sn[3 * i + 2];
    }
}

// computeLocal: DmInv is glm mat3 (column-major: DmInv[3 c + r] = entry (r, c)).
__global__ void k_compute_local(const float* V0, const float* w, float* b, const float* DmInv, const float* q,
                                const uint32_t* tet, int nt, bool jacobi) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int i0 = 3 * (int)tet[4 * t], i1 = 3 * (int)tet[4 * t + 1], i2 = 3 * (int)tet[4 * t + 2],
              i3 = 3 * (int)tet[4 * t + 3];
    float Ds[9];  // row-major
    for (int r = 0; r < 3; ++r) {
        Ds[3 * r] = q[i1 + r] - q[i0 + r];
        Ds[3 * r + 1] = q[i2 + r] - q[i0 + r];
        Ds[3 * r + 2] = q[i3 + r] - q[i0 + r];
    }
    float D[9];  // row-major DmInv
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) D[3 * r + c] = DmInv[9 * (size_t)t + 3 * c + r];
    float F[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) F[3 * r + c] = Ds[3 * r] * D[c] + Ds[3 * r + 1] * D[3 + c] + Ds[3 * r + 2] * D[6 + c];
    float R[9];
    pdgb::closest_rotation<4>(F, R);  // U V^T of the 4-sweep SVD, proper
    if (jacobi)
        for (int k = 0; k < 9; ++k) R[k] -= F[k];
    const float c = fabsf(V0[t]) * w[t];
    // M = c R DmInv^T; corner 0 gets -(M e0 + M e1 + M e2), corner j M e_{j-1}
    float M[9];
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k)
            M[3 * r + k] = c * (R[3 * r] * D[3 * k] + R[3 * r + 1] * D[3 * k + 1] + R[3 * r + 2] * D[3 * k + 2]);
    for (int r = 0; r < 3; ++r) {
        atomicAdd(&b[i0 + r], -M[3 * r] - M[3 * r + 1] - M[3 * r + 2]);
        atomicAdd(&b[i1 + r], M[3 * r]);
        atomicAdd(&b[i2 + r], M[3 * r + 1]);
        atomicAdd(&b[i3 + r], M[3 * r + 2]);
    }
}

__global__ void k_dbc_local(int nv, const float* dbc, const float* more, const float* x0, float wi, float* b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float mw = more[i];
    if (dbc[i] > 0.f) {
        for (int k = 0; k < 3; ++k) b[3 * i + k] = x0[3 * i + k] * wi;
    } else if (mw > 0.f) {
        for (int k = 0; k < 3; ++k) b[3 * i + k] = x0[3 * i + k] * mw;
    }
}

__global__ void k_update_vel_pos(const float* q, float dt_1, float* pos, float* vel, int nv, const float* more) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    for (int k = 0; k < 3; ++k) {
        const float x = q[3 * i + k];
        vel[3 * i + k] = more[i] > 0.f ? 0.f : (x - pos[3 * i + k]) * dt_1;
        pos[3 * i + k] = x;
    }
}

__global__ void k_jacobi(int nv, float* next_x, const float* b, const float* mdt2, const float* sn, const float* diag,
                         const float* more) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    if (more[i] > 0.f) {
        for (int k = 0; k < 3; ++k) next_x[3 * i + k] = sn[3 * i + k];
        return;
    }
    const float c = mdt2[i], md = diag[i];
    for (int k = 0; k < 3; ++k) next_x[3 * i + k] = (b[3 * i + k] - c * sn[3 * i + k]) / (c + md) + sn[3 * i + k];
}

__global__ void k_chebyshev(int n3, float* next_x, float* prev_x, float* sn, float omega) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    float nx = (float)(0.9 * (double)(next_x[i] - sn[i]) + (double)sn[i]);  // double literal, as in the reference
    nx = (nx - prev_x[i]) * omega + prev_x[i];
    next_x[i] = nx;
    prev_x[i] = sn[i];
    sn[i] = nx;
}

__global__ void k_permute(const float* b, float* bp, const int* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) bp[i] = b[p[i]];
}

__global__ void k_permute_inv(const float* xp, float* x, const int* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[p[i]] = xp[i];
}

// sum of (a - b)^2 over n entries into *out (float, like plus<float>)
__global__ void k_sq_diff(const float* a, const float* b, int n, float* out) {
    __shared__ float part[kThreads / 32];
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float d = b[i] - a[i];
        s += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int k = 0; k < kThreads / 32; ++k) t += part[k];
        atomicAdd(out, t);
    }
}

inline int blocks(int n) { return (n + kThreads - 1) / kThreads; }

template <class T>
int dalloc(T** p, size_t n) {
    RG_CUDA(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
    return 0;
}

template <class T>
int upload(T** p, const T* h, size_t n) {
    if (dalloc(p, n)) return 1;
    RG_CUDA(cudaMemcpy(*p, h, n * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

void destroy(RefGpu* r) {
    if (!r) return;
    float* fs[] = {r->X, r->V, r->XTilde, r->DBCX, r->OffsetX, r->force, r->mass, r->dbc, r->more, r->V0, r->w,
                   r->DmInv, r->sn, r->sn_old, r->b, r->next_x, r->prev_x, r->mdt2, r->diag, r->err, r->val, r->bp,
                   r->xp};
    for (float* p : fs) cudaFree(p);
    cudaFree(r->tet);
    cudaFree(r->rowptr);
    cudaFree(r->col);
    cudaFree(r->perm);
    cudaFree(r->buf);
    if (r->info) cusolverSpDestroyCsrcholInfo(r->info);
    if (r->descr) cusparseDestroyMatDescr(r->descr);
    if (r->sp) cusolverSpDestroy(r->sp);
    delete r;
}

// Host assembly of the PD system (computeSiTSi + setMDt_2) and of the
// Jacobi diagonal; CSR with duplicates summed, rows sorted.
void assemble(const RefGpu& r, const std::vector<float>& X, const std::vector<uint32_t>& T,
              const std::vector<float>& mass, const std::vector<float>& w, const std::vector<float>& dbc,
              const std::vector<double>& DmInv, const std::vector<double>& V0, std::vector<int>& rowptr,
              std::vector<int>& col, std::vector<float>& val, std::vector<float>& diag, std::vector<float>& mdt2) {
    const int nv = r.nv, n3 = 3 * nv;
    const double dt2 = (double)r.dt * r.dt;
    diag.assign(nv, 0.f);
    mdt2.assign(nv, 0.f);
    std::vector<std::vector<std::pair<int, double>>> rows(n3);
    std::vector<double> diagd(nv, 0.0);
    for (int t = 0; t < r.nt; ++t) {
        const double* Dm = &DmInv[9 * (size_t)t];  // row-major
        // A = DmInv^T G, G = [-1 -1 -1; I] as 3x4 columns (-1,-1,-1), e0, e1, e2
        double A[3][4];
        for (int i = 0; i < 3; ++i) {
            // row i of DmInv^T = column i of DmInv
            const double c0 = Dm[0 * 3 + i], c1 = Dm[1 * 3 + i], c2 = Dm[2 * 3 + i];
            A[i][0] = -(c0 + c1 + c2);
            A[i][1] = c0;
            A[i][2] = c1;
            A[i][3] = c2;
        }
        const double coef = V0[t] * (double)w[t];
        for (int i = 0; i < 4; ++i) {
            for (int j = 0; j < 4; ++j) {
                const double s = (A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j]) * coef;
                const int vi = (int)T[4 * t + i], vj = (int)T[4 * t + j];
                for (int k = 0; k < 3; ++k) rows[3 * vi + k].push_back({3 * vj + k, s});
                if (i == j) diagd[vi] += s;
            }
        }
    }
    for (int v = 0; v < nv; ++v) {
        const double m = ((double)mass[v] + (double)dbc[v] * r.pw) / dt2;
        mdt2[v] = (float)(((float)mass[v] + dbc[v] * r.pw) / (r.dt * r.dt));
        diag[v] = (float)diagd[v];
        for (int k = 0; k < 3; ++k) rows[3 * v + k].push_back({3 * v + k, m});
    }
    rowptr.assign(n3 + 1, 0);
    col.clear();
    val.clear();
    for (int i = 0; i < n3; ++i) {
        auto& rw = rows[i];
        std::sort(rw.begin(), rw.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (size_t k = 0; k < rw.size();) {
            double s = 0.0;
            const int c = rw[k].first;
            for (; k < rw.size() && rw[k].first == c; ++k) s += rw[k].second;
            col.push_back(c);
            val.push_back((float)s);
        }
        rowptr[i + 1] = (int)col.size();
        std::vector<std::pair<int, double>>().swap(rw);
    }
}

int setup_cholesky(RefGpu* r, std::vector<int>& rowptr, std::vector<int>& col, std::vector<float>& val) {
    const int n = r->n3, nnz = (int)col.size();
    r->nnz = nnz;
    RG_SOLVER(cusolverSpCreate(&r->sp));
    if (cusparseCreateMatDescr(&r->descr) != CUSPARSE_STATUS_SUCCESS) return fail("cusparseCreateMatDescr");
    cusparseSetMatType(r->descr, CUSPARSE_MATRIX_TYPE_GENERAL);
    cusparseSetMatIndexBase(r->descr, CUSPARSE_INDEX_BASE_ZERO);
    // ComputeAMD (cholesky.cu:72-130): symamd on the host, B = Q A Q^T
    std::vector<int> Q(n);
    RG_SOLVER(cusolverSpXcsrsymamdHost(r->sp, n, nnz, r->descr, rowptr.data(), col.data(), Q.data()));
    size_t perm_bytes = 0;
    RG_SOLVER(cusolverSpXcsrperm_bufferSizeHost(r->sp, n, n, nnz, r->descr, rowptr.data(), col.data(), Q.data(),
                                                Q.data(), &perm_bytes));
    std::vector<char> pbuf(perm_bytes + 1);
    std::vector<int> map(nnz);
    for (int j = 0; j < nnz; ++j) map[j] = j;
    RG_SOLVER(cusolverSpXcsrpermHost(r->sp, n, n, nnz, r->descr, rowptr.data(), col.data(), Q.data(), Q.data(),
                                     map.data(), pbuf.data()));
    std::vector<float> valB(nnz);
    for (int j = 0; j < nnz; ++j) valB[j] = val[map[j]];
    if (upload(&r->rowptr, rowptr.data(), rowptr.size()) || upload(&r->col, col.data(), col.size()) ||
        upload(&r->val, valB.data(), valB.size()) || upload(&r->perm, Q.data(), Q.size()) || dalloc(&r->bp, n) ||
        dalloc(&r->xp, n))
        return 1;
    RG_SOLVER(cusolverSpCreateCsrcholInfo(&r->info));
    RG_SOLVER(cusolverSpXcsrcholAnalysis(r->sp, n, nnz, r->descr, r->rowptr, r->col, r->info));
    size_t internal = 0, work = 0;
    RG_SOLVER(cusolverSpScsrcholBufferInfo(r->sp, n, nnz, r->descr, r->val, r->rowptr, r->col, r->info, &internal,
                                           &work));
    RG_CUDA(cudaMalloc(&r->buf, std::max<size_t>(work, 1)));
    RG_SOLVER(cusolverSpScsrcholFactor(r->sp, n, nnz, r->descr, r->val, r->rowptr, r->col, r->info, r->buf));
    int pos = -1;
    RG_SOLVER(cusolverSpScsrcholZeroPivot(r->sp, r->info, 0.f, &pos));
    if (pos >= 0) return fail("cusolverSpScsrcholFactor: zero pivot at row " + std::to_string(pos));
    RG_CUDA(cudaDeviceSynchronize());
    return 0;
}

// One SolverStep + the Update tail without collision or fixed bodies.
int step_once(RefGpu* r) {
    const int nv = r->nv, n3 = r->n3;
    const float dt = r->dt, dt2 = dt * dt, dtInv = 1.0f / dt, dt2Inv = dtInv * dtInv;
    k_gravity<<<blocks(nv), kThreads>>>(nv, r->mass, r->gravity, r->force);
    k_set_mdt2_more<<<blocks(nv), kThreads>>>(nv, r->mass, dt2, r->mdt2, r->more, r->dbc);
    k_compute_sn<<<blocks(nv), kThreads>>>(nv, r->sn, dt, r->mdt2, r->X, r->V, r->force, r->more, r->OffsetX,
                                           r->DBCX);
    RG_CUDA(cudaMemcpy(r->sn_old, r->sn, sizeof(float) * n3, cudaMemcpyDeviceToDevice));
    if (!r->cholesky)
        RG_CUDA(cudaMemcpy(r->prev_x, r->sn, sizeof(float) * n3, cudaMemcpyDeviceToDevice));
    else
        RG_CUDA(cudaMemset(r->prev_x, 0, n3));  // bytes, as pdSolver.cu:162
    float err = 1.f, omega = 1.f;
    for (int i = 0; i < r->iters && std::sqrt(err) >= r->tol; ++i) {
        k_add_mh2_sn<<<blocks(nv), kThreads>>>(r->b, r->sn_old, r->mdt2, nv);
        k_compute_local<<<blocks(r->nt), kThreads>>>(r->V0, r->w, r->b, r->DmInv, r->sn, r->tet, r->nt, !r->cholesky);
        if (r->ndbc > 0) k_dbc_local<<<blocks(nv), kThreads>>>(nv, r->dbc, r->more, r->DBCX, r->pw * dt2Inv, r->b);
        if (r->cholesky) {
            k_permute<<<blocks(n3), kThreads>>>(r->b, r->bp, r->perm, n3);
            RG_SOLVER(cusolverSpScsrcholSolve(r->sp, n3, r->bp, r->xp, r->info, r->buf));
            k_permute_inv<<<blocks(n3), kThreads>>>(r->xp, r->sn, r->perm, n3);
            RG_CUDA(cudaMemset(r->err, 0, sizeof(float)));
            k_sq_diff<<<std::min(blocks(n3), 1024), kThreads>>>(r->sn, r->prev_x, n3, r->err);
            float s = 0.f;
            RG_CUDA(cudaMemcpy(&s, r->err, sizeof(float), cudaMemcpyDeviceToHost));
            err = s / n3;
            RG_CUDA(cudaMemcpy(r->prev_x, r->sn, sizeof(float) * n3, cudaMemcpyDeviceToDevice));
        } else {
            k_jacobi<<<blocks(nv), kThreads>>>(nv, r->next_x, r->b, r->mdt2, r->sn, r->diag, r->more);
            if (i <= 10) omega = 1.f;
            else if (i == 11) omega = 2.f / (2.f - r->rho * r->rho);
            else omega = 4.f / (4.f - r->rho * r->rho * omega);
            k_chebyshev<<<blocks(n3), kThreads>>>(n3, r->next_x, r->prev_x, r->sn, omega);
        }
        ++r->last_iterations;
    }
    k_update_vel_pos<<<blocks(nv), kThreads>>>(r->sn, dtInv, r->XTilde, r->V, nv, r->more);
    RG_CUDA(cudaMemcpy(r->X, r->XTilde, sizeof(float) * n3, cudaMemcpyDeviceToDevice));
    RG_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" {

const char* rg_last_error(void) { return g_err.c_str(); }

// Creates the reference-path baseline for one body (host arrays: X float[3 nv],
// tets u32[4 nt], mass float[nv], weight float[nt] (the PD weight mu), dbc
// float[nv] pin mask), prepares it (DmInv/V0, system, factor) and uploads
// the rest state.  cholesky = 0 runs Jacobi + Chebyshev.
int rg_create(int nv, int nt, const float* X, const uint32_t* tets, const float* mass, const float* weight,
              const float* dbc, float dt, float gravity, int iterations, float tol, float rho,
              float positional_weight, int cholesky, void** out) {
    if (!out || nv <= 0 || nt <= 0 || !X || !tets || !mass || !weight || !dbc) return fail("rg_create: bad arguments");
    *out = nullptr;
    RefGpu* r = new RefGpu();
    r->nv = nv;
    r->nt = nt;
    r->n3 = 3 * nv;
    r->cholesky = cholesky != 0;
    r->dt = dt;
    r->gravity = gravity;
    r->iters = iterations;
    r->tol = tol;
    r->rho = rho;
    r->pw = positional_weight;
    std::vector<float> hX(X, X + 3 * (size_t)nv), hm(mass, mass + nv), hw(weight, weight + nt), hd(dbc, dbc + nv);
    std::vector<uint32_t> hT(tets, tets + 4 * (size_t)nt);
    for (uint32_t v : hT)
        if (v >= (uint32_t)nv) {
            destroy(r);
            return fail("rg_create: tet vertex index out of range");
        }
    for (float d : hd) r->ndbc += d > 0.f;
    // computeInvDmV0 (solverUtil.cuh:108-138), in double, stored as float
    std::vector<double> DmInv(9 * (size_t)nt), V0(nt);
    std::vector<float> DmInvF(9 * (size_t)nt), V0F(nt);
    for (int t = 0; t < nt; ++t) {
        double Dm[3][3];  // columns = edges
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) Dm[k][c] = (double)hX[3 * hT[4 * t + c + 1] + k] - hX[3 * hT[4 * t] + k];
        const double det = Dm[0][0] * (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) -
                           Dm[0][1] * (Dm[1][0] * Dm[2][2] - Dm[1][2] * Dm[2][0]) +
                           Dm[0][2] * (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]);
        if (det == 0.0) {
            destroy(r);
            return fail("rg_create: degenerate tet " + std::to_string(t));
        }
        double inv[3][3];
        inv[0][0] = (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) / det;
        inv[0][1] = (Dm[0][2] * Dm[2][1] - Dm[0][1] * Dm[2][2]) / det;
        inv[0][2] = (Dm[0][1] * Dm[1][2] - Dm[0][2] * Dm[1][1]) / det;
        inv[1][0] = (Dm[1][2] * Dm[2][0] - Dm[1][0] * Dm[2][2]) / det;
        inv[1][1] = (Dm[0][0] * Dm[2][2] - Dm[0][2] * Dm[2][0]) / det;
        inv[1][2] = (Dm[0][2] * Dm[1][0] - Dm[0][0] * Dm[1][2]) / det;
        inv[2][0] = (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]) / det;
        inv[2][1] = (Dm[0][1] * Dm[2][0] - Dm[0][0] * Dm[2][1]) / det;
        inv[2][2] = (Dm[0][0] * Dm[1][1] - Dm[0][1] * Dm[1][0]) / det;
        for (int rr = 0; rr < 3; ++rr)
            for (int c = 0; c < 3; ++c) {
                DmInv[9 * (size_t)t + 3 * rr + c] = inv[rr][c];      // row-major (host assembly)
                DmInvF[9 * (size_t)t + 3 * c + rr] = (float)inv[rr][c];  // glm column-major (device)
            }
        V0[t] = std::fabs(det) / 6.0;
        V0F[t] = (float)V0[t];
    }
    std::vector<int> rowptr, col;
    std::vector<float> val, diag, mdt2;
    assemble(*r, hX, hT, hm, hw, hd, DmInv, V0, rowptr, col, val, diag, mdt2);
    const size_t n3 = (size_t)r->n3;
    std::vector<float> zeros(n3, 0.f);
    int rc = upload(&r->X, hX.data(), n3) || upload(&r->XTilde, hX.data(), n3) || upload(&r->DBCX, hX.data(), n3) ||
             upload(&r->V, zeros.data(), n3) || upload(&r->OffsetX, zeros.data(), n3) || dalloc(&r->force, n3) ||
             upload(&r->mass, hm.data(), nv) || upload(&r->dbc, hd.data(), nv) ||
             upload(&r->more, zeros.data(), nv) || upload(&r->V0, V0F.data(), nt) || upload(&r->w, hw.data(), nt) ||
             upload(&r->DmInv, DmInvF.data(), 9 * (size_t)nt) || upload(&r->tet, hT.data(), hT.size()) ||
             dalloc(&r->sn, n3) || dalloc(&r->sn_old, n3) || dalloc(&r->b, n3) || dalloc(&r->next_x, n3) ||
             dalloc(&r->prev_x, n3) || upload(&r->mdt2, mdt2.data(), nv) || upload(&r->diag, diag.data(), nv) ||
             dalloc(&r->err, 1);
    if (!rc) {
        cudaError_t e = cudaMemset(r->prev_x, 0, n3 * sizeof(float));
        if (e != cudaSuccess) rc = fail(std::string("cudaMemset: ") + cudaGetErrorString(e));
    }
    if (!rc && r->cholesky) rc = setup_cholesky(r, rowptr, col, val);
    if (rc) {
        destroy(r);
        return rc;
    }
    *out = r;
    return 0;
}

// Runs nsteps PD steps; *ms = elapsed time between CUDA events on the legacy
// default stream around them, *iterations = local/global iterations run.
int rg_step(void* h, int nsteps, float* ms, long long* iterations) {
    RefGpu* r = static_cast<RefGpu*>(h);
    if (!r || nsteps < 0) return fail("rg_step: bad arguments");
    cudaEvent_t e0, e1;
    RG_CUDA(cudaEventCreate(&e0));
    RG_CUDA(cudaEventCreate(&e1));
    r->last_iterations = 0;
    RG_CUDA(cudaEventRecord(e0, 0));
    int rc = 0;
    for (int s = 0; s < nsteps && !rc; ++s) rc = step_once(r);
    if (!rc) {
        cudaEventRecord(e1, 0);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (ms) *ms = t;
        if (iterations) *iterations = r->last_iterations;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// Uploads positions and velocities (host float[3 nv] each; V may be null for
// rest) and sets XTilde = X.
int rg_upload(void* h, const float* X, const float* V) {
    RefGpu* r = static_cast<RefGpu*>(h);
    if (!r || !X) return fail("rg_upload: bad arguments");
    const size_t n = sizeof(float) * r->n3;
    RG_CUDA(cudaMemcpy(r->X, X, n, cudaMemcpyHostToDevice));
    RG_CUDA(cudaMemcpy(r->XTilde, X, n, cudaMemcpyHostToDevice));
    if (V) RG_CUDA(cudaMemcpy(r->V, V, n, cudaMemcpyHostToDevice));
    else RG_CUDA(cudaMemset(r->V, 0, n));
    return 0;
}

int rg_read(void* h, float* X, float* V) {
    RefGpu* r = static_cast<RefGpu*>(h);
    if (!r) return fail("rg_read: bad arguments");
    const size_t n = sizeof(float) * r->n3;
    if (X) RG_CUDA(cudaMemcpy(X, r->X, n, cudaMemcpyDeviceToHost));
    if (V) RG_CUDA(cudaMemcpy(V, r->V, n, cudaMemcpyDeviceToHost));
    return 0;
}

// nnz of the 3n x 3n system matrix (0 on the Jacobi path).
long long rg_system_nnz(void* h) { return h ? static_cast<RefGpu*>(h)->nnz : 0; }

void rg_destroy(void* h) { destroy(static_cast<RefGpu*>(h)); }

}  // extern "C"
