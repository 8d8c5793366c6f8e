// pdgb_step_noalloc: PD time steps (Jacobi + Chebyshev global solve) that
// allocate no memory at all.
//
// Who needs this.  Some callers cannot call cudaMalloc (or any allocating
// routine) at the point where they want to advance a soft body:
//   - a host application whose device-memory allocator owns the GPU's memory
//     (a game engine or renderer with its own pools) and forbids plugins to
//     allocate behind its back;
//   - code running inside a frame loop with a hard latency budget, where a
//     cudaMalloc/cudaFree can synchronise the whole device;
//   - plugins that receive only device pointers to the simulation arrays
//     (the way the reference's SolverData is handed to its solvers) and have
//     no place to keep per-body allocations between calls.
// pdgb_create/pdgb_step allocate the engine's buffers once; this entry point
// instead keeps its scratch in one fixed, file-scope device array that every
// GPU loading the library holds until the process exits.
//
// Limits and sharing rules (also stated in include/pdgb.h):
//   - at most kNaMaxVerts vertices and kNaMaxTets tets per call;
//   - every call uses the same scratch array, so calls that overlap on the
//     GPU (on different streams, or from several host threads) race and
//     corrupt each other's results; serialise them;
//   - the scratch keeps the previous call's contents; everything a call
//     needs is recomputed or cleared by that call;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) once for that device.  The address is kept for
//     the life of the process, so a cudaDeviceReset between calls is not
//     supported;
//   - every call waits for its stream (after the mesh check and before it
//     returns), so no call can be captured into a CUDA graph;
//   - the mesh is checked on the device (tet indices, rest volumes, weights)
//     before any step: a bad mesh returns PDGB_ERR_BAD_MESH with X and V
//     untouched.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/pdgb.h"
#include "relax.cuh"
#include "rotation.cuh"

namespace pdgb {
namespace {

constexpr int kNaMaxVerts = 32768;
constexpr int kNaMaxTets = 131072;
constexpr int kNaMaxDevices = 64;

// Scratch layout (bytes):
//   tet part   : per tet 10 floats (DmInv row-major, V0 * mu)       [kNaMaxTets]
//   vertex part: float4 sn, prev, b, base, coef {M/h^2, diag, pin, m} [kNaMaxVerts]
//                float  diag accumulator                            [kNaMaxVerts]
//   flags      : int bad-mesh flag (256 bytes reserved)
// 5.2 MB + 2.6 MB + 0.1 MB = about 8 MB in total.
constexpr size_t kNaTetBytes = (size_t)kNaMaxTets * 10 * sizeof(float);
constexpr size_t kNaVecBytes = (size_t)kNaMaxVerts * sizeof(float4);
constexpr size_t kNaDiagBytes = (size_t)kNaMaxVerts * sizeof(float);
constexpr size_t kNaScratchBytes = kNaTetBytes + 5 * kNaVecBytes + kNaDiagBytes + 256;

static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

struct NaScratch {
    float* geo;     // [10][kNaMaxTets] SoA
    float4* sn;
    float4* prev;
    float4* b;
    float4* base;
    float4* coef;
    float* diag;
    int* bad;       // set when a tet has an out-of-range index, no float-representable
                    // DmInv (zero or nearly zero rest volume) or a negative or
                    // non-finite weight
};

NaScratch carve(unsigned char* base) {
    NaScratch s;
    s.geo = reinterpret_cast<float*>(base);
    unsigned char* p = base + kNaTetBytes;
    s.sn = reinterpret_cast<float4*>(p);
    s.prev = reinterpret_cast<float4*>(p + kNaVecBytes);
    s.b = reinterpret_cast<float4*>(p + 2 * kNaVecBytes);
    s.base = reinterpret_cast<float4*>(p + 3 * kNaVecBytes);
    s.coef = reinterpret_cast<float4*>(p + 4 * kNaVecBytes);
    s.diag = reinterpret_cast<float*>(p + 5 * kNaVecBytes);
    s.bad = reinterpret_cast<int*>(p + 5 * kNaVecBytes + kNaDiagBytes);
    return s;
}

// Per-tet DmInv and V0 * mu from the rest shape (solverUtil.cuh:108-138) and
// the stiffness diagonal sum_t c_t (B_t^T B_t)_jj (pdUtil.cu:21-24).
__global__ void na_tets(int nv, int nt, const uint32_t* __restrict__ tets, const float* __restrict__ X0,
                        const float* __restrict__ mu, NaScratch s) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const uint32_t i0 = tets[4 * t], i1 = tets[4 * t + 1], i2 = tets[4 * t + 2], i3 = tets[4 * t + 3];
    if (i0 >= (uint32_t)nv || i1 >= (uint32_t)nv || i2 >= (uint32_t)nv || i3 >= (uint32_t)nv) {
        atomicExch(s.bad, 1);
        return;
    }
    double D[3][3];
    const uint32_t id[3] = {i1, i2, i3};
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) D[r][c] = (double)X0[3 * id[c] + r] - (double)X0[3 * i0 + r];
    const double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) - D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                       D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
    const float w = mu[t];
    if (!(det != 0.0) || !isfinite(det) || !(w >= 0.f) || !isfinite(w)) {
        atomicExch(s.bad, 1);
        return;
    }
    double inv[9];
    inv[0] = (D[1][1] * D[2][2] - D[1][2] * D[2][1]) / det;
    inv[1] = (D[0][2] * D[2][1] - D[0][1] * D[2][2]) / det;
    inv[2] = (D[0][1] * D[1][2] - D[0][2] * D[1][1]) / det;
    inv[3] = (D[1][2] * D[2][0] - D[1][0] * D[2][2]) / det;
    inv[4] = (D[0][0] * D[2][2] - D[0][2] * D[2][0]) / det;
    inv[5] = (D[0][2] * D[1][0] - D[0][0] * D[1][2]) / det;
    inv[6] = (D[1][0] * D[2][1] - D[1][1] * D[2][0]) / det;
    inv[7] = (D[0][1] * D[2][0] - D[0][0] * D[2][1]) / det;
    inv[8] = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) / det;
    const double coef = fabs(det) / 6.0 * (double)w;
    // a nearly flat tet has a finite double inverse that overflows float:
    // rejected like a flat one (the layout of pdgb_create does the same)
    bool finite = isfinite((float)coef);
    for (int k = 0; k < 9; ++k) finite = finite && isfinite((float)inv[k]);
    if (!finite) {
        atomicExch(s.bad, 1);
        return;
    }
    for (int k = 0; k < 9; ++k) s.geo[(size_t)k * kNaMaxTets + t] = (float)inv[k];
    s.geo[(size_t)9 * kNaMaxTets + t] = (float)coef;
    const uint32_t corner[4] = {i0, i1, i2, i3};
    for (int j = 0; j < 4; ++j) {
        double bx, by, bz;  // column j of B = DmInv^T G
        if (j == 0) {
            bx = -(inv[0] + inv[3] + inv[6]);
            by = -(inv[1] + inv[4] + inv[7]);
            bz = -(inv[2] + inv[5] + inv[8]);
        } else {
            bx = inv[3 * (j - 1)];
            by = inv[3 * (j - 1) + 1];
            bz = inv[3 * (j - 1) + 2];
        }
        atomicAdd(&s.diag[corner[j]], (float)(coef * (bx * bx + by * by + bz * bz)));
    }
}

__global__ void na_clear(int nv, NaScratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) s.diag[i] = 0.f;
}

__global__ void na_vertex_coef(int nv, const float* __restrict__ mass, const float* __restrict__ dbc, float dt,
                               float pw, NaScratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float pin = dbc ? dbc[i] : 0.f;
    const float mdt2 = (mass[i] + pin * pw) / (dt * dt);
    s.coef[i] = make_float4(mdt2, s.diag[i], pin > 0.f ? 1.f : 0.f, mass[i]);
}

// s = x + h v + f / (M/h^2); base = b = (M/h^2) s.
__global__ void na_begin(int nv, const float* __restrict__ X, const float* __restrict__ V, float dt, float g,
                         NaScratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 cf = s.coef[i];
    const float dt2_m_1 = 1.0f / cf.x;
    const float fy = -g * cf.w;
    const float4 sn = make_float4(X[3 * i] + dt * V[3 * i], X[3 * i + 1] + dt * V[3 * i + 1] + dt2_m_1 * fy,
                                  X[3 * i + 2] + dt * V[3 * i + 2], 0.f);
    s.sn[i] = sn;
    const float4 bs = make_float4(cf.x * sn.x, cf.x * sn.y, cf.x * sn.z, 0.f);
    s.base[i] = bs;
    s.b[i] = bs;
}

// Local step, one thread per tet, residual form c (R - F) B, float4 atomics
// into the scratch b (pinned vertices ignore b).
__global__ void na_local(int nv, int nt, const uint32_t* __restrict__ tets, NaScratch s) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt || *s.bad) return;
    const uint32_t i0 = tets[4 * t], i1 = tets[4 * t + 1], i2 = tets[4 * t + 2], i3 = tets[4 * t + 3];
    if (i0 >= (uint32_t)nv || i1 >= (uint32_t)nv || i2 >= (uint32_t)nv || i3 >= (uint32_t)nv) return;
    float D[9];
    for (int k = 0; k < 9; ++k) D[k] = s.geo[(size_t)k * kNaMaxTets + t];
    const float c = s.geo[(size_t)9 * kNaMaxTets + t];
    const float4 p0 = s.sn[i0], p1 = s.sn[i1], p2 = s.sn[i2], p3 = s.sn[i3];
    const float e[3][3] = {{p1.x - p0.x, p2.x - p0.x, p3.x - p0.x},
                           {p1.y - p0.y, p2.y - p0.y, p3.y - p0.y},
                           {p1.z - p0.z, p2.z - p0.z, p3.z - p0.z}};
    float F[9];
    for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) F[3 * r + cc] = e[r][0] * D[cc] + e[r][1] * D[3 + cc] + e[r][2] * D[6 + cc];
    float R[9];
    closest_rotation_horn(F, R);
    for (int k = 0; k < 9; ++k) R[k] -= F[k];
    float M[9];
    for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc)
            M[3 * r + cc] = c * (R[3 * r] * D[3 * cc] + R[3 * r + 1] * D[3 * cc + 1] + R[3 * r + 2] * D[3 * cc + 2]);
    atomicAdd(&s.b[i0], make_float4(-(M[0] + M[1] + M[2]), -(M[3] + M[4] + M[5]), -(M[6] + M[7] + M[8]), 0.f));
    atomicAdd(&s.b[i1], make_float4(M[0], M[3], M[6], 0.f));
    atomicAdd(&s.b[i2], make_float4(M[1], M[4], M[7], 0.f));
    atomicAdd(&s.b[i3], make_float4(M[2], M[5], M[8], 0.f));
}

// Jacobi update + 0.9 relaxation + Chebyshev blend (pdUtil.cu:195-226) with
// the pin RHS x0 * w / h^2 (pdUtil.cu:147-166); the last iteration writes
// V and X (pdUtil.cu:180-193).
__global__ void na_vertex(int nv, const float* __restrict__ X0, float wpin, float omega, int read_prev,
                          int write_prev, int final_iter, float dt_inv, float* X, float* V, NaScratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 sn = s.sn[i];
    const float4 cf = s.coef[i];
    float4 bb;
    if (cf.z != 0.f) bb = make_float4(X0[3 * i] * wpin, X0[3 * i + 1] * wpin, X0[3 * i + 2] * wpin, 0.f);
    else bb = s.b[i];
    const float den = cf.x + cf.y;
    float n[3];
    const float sv[3] = {sn.x, sn.y, sn.z}, bv[3] = {bb.x, bb.y, bb.z};
    for (int d = 0; d < 3; ++d) n[d] = relax09((bv[d] - cf.x * sv[d]) / den + sv[d], sv[d]);
    if (read_prev) {
        const float4 p = s.prev[i];
        n[0] = (n[0] - p.x) * omega + p.x;
        n[1] = (n[1] - p.y) * omega + p.y;
        n[2] = (n[2] - p.z) * omega + p.z;
    }
    if (write_prev) s.prev[i] = sn;
    if (final_iter) {
        for (int d = 0; d < 3; ++d) {
            V[3 * i + d] = (n[d] - X[3 * i + d]) * dt_inv;
            X[3 * i + d] = n[d];
        }
    } else {
        s.sn[i] = make_float4(n[0], n[1], n[2], 0.f);
        s.b[i] = s.base[i];
    }
}

std::mutex g_na_mutex;
unsigned char* g_na_ptr[kNaMaxDevices] = {};

}  // namespace
}  // namespace pdgb

using namespace pdgb;

extern "C" int pdgb_step_noalloc(const pdgb_noalloc_mesh* mesh, const pdgb_params* p, float* X, float* V,
                                 int nsteps, void* stream) {
    if (!mesh || !p || !X || !V || !mesh->tets || !mesh->X0 || !mesh->mass || !mesh->mu || nsteps < 0)
        return PDGB_ERR_INVALID_ARGUMENT;
    if (mesh->num_verts <= 0 || mesh->num_tets <= 0) return PDGB_ERR_INVALID_ARGUMENT;
    if (mesh->num_verts > kNaMaxVerts || mesh->num_tets > kNaMaxTets) return PDGB_ERR_UNSUPPORTED;
    if (!(p->dt > 0.f) || p->num_iterations < 1 || p->num_iterations > 4096) return PDGB_ERR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return PDGB_ERR_CUDA;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[dev]) {
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_na_scratch) != cudaSuccess || !ptr) return PDGB_ERR_CUDA;
            g_na_ptr[dev] = static_cast<unsigned char*>(ptr);
        }
        base = g_na_ptr[dev];
    }
    const NaScratch s = carve(base);
    cudaStream_t st = (cudaStream_t)stream;
    const int nv = mesh->num_verts, nt = mesh->num_tets;
    const int vb = (nv + 255) / 256, tb = (nt + 255) / 256;
    if (cudaMemsetAsync(s.bad, 0, sizeof(int), st) != cudaSuccess) return PDGB_ERR_CUDA;
    na_clear<<<vb, 256, 0, st>>>(nv, s);
    na_tets<<<tb, 256, 0, st>>>(nv, nt, mesh->tets, mesh->X0, mesh->mu, s);
    na_vertex_coef<<<vb, 256, 0, st>>>(nv, mesh->mass, mesh->dbc, p->dt, p->positional_weight, s);
    // The mesh check is read back before the first step, so that a bad mesh
    // leaves the caller's X and V untouched.
    int hbad = 0;
    if (cudaGetLastError() != cudaSuccess) return PDGB_ERR_CUDA;
    if (cudaMemcpyAsync(&hbad, s.bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PDGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PDGB_ERR_CUDA;
    if (hbad) return PDGB_ERR_BAD_MESH;
    const float dt_inv = 1.0f / p->dt;
    const float wpin = p->positional_weight * (dt_inv * dt_inv);
    const int n = p->num_iterations;
    for (int k = 0; k < nsteps; ++k) {
        na_begin<<<vb, 256, 0, st>>>(nv, X, V, p->dt, p->gravity, s);
        float omega = 1.f;
        for (int i = 0; i < n; ++i) {
            if (i <= 10) omega = 1;
            else if (i == 11) omega = 2 / (2 - p->rho * p->rho);
            else omega = 4 / (4 - p->rho * p->rho * omega);
            na_local<<<tb, 256, 0, st>>>(nv, nt, mesh->tets, s);
            na_vertex<<<vb, 256, 0, st>>>(nv, mesh->X0, wpin, omega, i >= 11, i >= 10 && i + 1 < n, i + 1 == n,
                                          dt_inv, X, V, s);
        }
    }
    if (cudaGetLastError() != cudaSuccess) return PDGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PDGB_ERR_CUDA;
    return PDGB_OK;
}
