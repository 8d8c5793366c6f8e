// Internal definitions of the pdgb engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pdgb.h"

namespace pdgb {

// ----------------------------------------------------------------- errors
struct Error {
    int status;
    std::string msg;
};
void set_last_error(int status, const std::string& msg);

#define PDGB_CUDA_TRY(call)                                                                       \
    do {                                                                                          \
        cudaError_t err__ = (call);                                                               \
        if (err__ != cudaSuccess)                                                                 \
            throw ::pdgb::Error{PDGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err__)}; \
    } while (0)

// ------------------------------------------------------- tiling constants
// Local-step tiles: a CTA owns a run of Morton-ordered tets and the patch of
// vertices they touch.  kMaxPatch bounds the patch so that its positions and
// accumulators fit in shared memory (16 + 12 bytes per vertex).
constexpr int kMaxPatch = 1024;
// A tet corner is recorded as patch index k (kPatchBits) | rank r of the
// corner within k's run of slots (the remaining bits of a uint16), so a
// vertex has at most kMaxRun corners in one tile.
constexpr int kPatchBits = 10;
constexpr int kMaxRun = 1 << (16 - kPatchBits);
static_assert(kMaxPatch <= (1 << kPatchBits), "patch index field");
constexpr int kLocalThreads = 256;
constexpr int kTileTets = 2 * kLocalThreads;
constexpr int kLayoutTailPad = 8;

// Device buffer with RAII.
template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error{PDGB_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed"};
        }
        n = count;
    }
    void upload(const std::vector<T>& h, cudaStream_t s) {
        if (h.size() > n) alloc(h.size());
        if (!h.empty()) PDGB_CUDA_TRY(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
};

// Host-side product of prepare: everything the kernels need, in the
// engine's internal (Morton) vertex and tet order.
struct HostLayout {
    int nv = 0, nt = 0, nt_pad = 0, ntiles = 0;
    int tile_cap = 0;         // most tets per tile of the current cut
    int max_patch = 0;        // largest tile patch of the current cut
    std::vector<int> vperm;   // internal vertex -> caller vertex
    std::vector<int> viperm;  // caller vertex -> internal vertex
    std::vector<int> tperm;   // internal tet -> caller tet
    int nbodies = 1;
    std::vector<int> body_ivstart;  // [nbodies+1] internal vertex range of each body
    std::vector<int> body_itstart;  // [nbodies+1] internal tet range of each body
    // tiles
    std::vector<int> tile_tet_ptr;   // [ntiles+1]
    std::vector<int> tile_vptr;      // [ntiles+1]
    std::vector<uint32_t> tile_verts;  // internal vertex ids of each patch (longest run first) | kPinnedBit [+ kLayoutTailPad]
    // Slots of a tile: one per tet corner, ordered by patch vertex (then tet,
    // then corner), so patch vertex k owns the slots inc_end[k-1] ..
    // inc_end[k] (inc_end[-1] = 0).  inc_ent[4 t + c] = k | r << kPatchBits
    // for corner c of tet t: its patch vertex k and its rank r in k's run
    // (slot inc_end[k-1] + r).
    // The arrays the pipelined local step bulk-copies are padded so that
    // 16-byte-rounded copy ranges stay inside them: inc_ent to 4 nt_pad
    // entries, tile_verts and inc_end by kLayoutTailPad zero entries.
    std::vector<uint16_t> inc_ent;   // [4 nt_pad]
    std::vector<uint16_t> inc_end;   // [sum of patch sizes + kLayoutTailPad]
    std::vector<float> geo;          // planes float4 [nt_pad] x2 + float2 [nt_pad]: g DmInv (row major), g = sqrt(V0 w)
    std::vector<uint32_t> tets_int;  // [4*nt] internal vertex ids (Cholesky assembly, checks)
    std::vector<double> dminv_d;     // [9*nt] double DmInv (system assembly)
    std::vector<double> coef_d;      // [nt]   double V0*w
    // per vertex, internal order
    std::vector<float4> coef;        // {mdt2, stiffness diag, pin flag, mass}
    std::vector<float4> pin_rhs;     // x0 * (pin weight / h^2) for pinned vertices
    std::vector<float4> x0;          // rest positions
};

// Builds the layout from caller arrays (host memory).  Throws Error.
// body_vstart (nullable, nbodies + 1 entries): vertex ranges of independent
// bodies; vertices and tets are then ordered body-major (Morton within a
// body), so tiles never mix bodies and each body's internal vertices are
// contiguous.
void build_layout(int nv, int nt, const float* X0, const uint32_t* tets, const float* mass, const float* mu,
                  const float* dbc, const pdgb_params& prm, HostLayout& L, int nbodies = 1,
                  const int* body_vstart = nullptr, int max_tile_tets = kTileTets);

// Re-cuts the tiles of a built layout with at most max_tile_tets tets each
// (vertex and tet orders unchanged).  dbc: caller-order pin flags or null.
void build_tiles(HostLayout& L, const float* dbc, int max_tile_tets);

// Recomputes the per-vertex coefficients that depend on dt / pin weight.
void build_vertex_coefficients(const float* mass, const float* dbc, const pdgb_params& prm, HostLayout& L);

// Jacobi-Chebyshev relaxation weights of iterations 0..n-1, computed in float
// exactly as the reference's host loop does (pdSolver.cu:196-199).
std::vector<float> chebyshev_omegas(int n, float rho);

// --------------------------------------------------------------- kernels
// Patch entries: vertex id in the low 31 bits; bit 31 marks a pinned vertex,
// whose RHS is overwritten by the pin term, so the tile adds nothing to it.
constexpr uint32_t kPinnedBit = 0x80000000u;

struct LocalArgs {
    const float4* sn;
    float4* b;
    const uint16_t* inc_ent;
    const uint16_t* inc_end;
    const float* geo;
    const int* tile_tet_ptr;
    const int* tile_vptr;
    const uint32_t* tile_verts;
    int nt_pad;
    const int* done;  // step early-exit flag (Cholesky tol rule), may be null
    // Pipelined local step (k_local_pipe): resident CTAs (0: the one-tile-
    // per-CTA kernel runs instead) and the word set when one of its bounded
    // waits for a bulk copy runs out.
    int pipe_grid;
    int* timeout;
};

// Vertex-kernel mode flags.
enum : int {
    kReadPrev = 1,    // Chebyshev blend with prev (omega != 1)
    kWritePrev = 2,   // store sn as prev for the next iteration
    kFinal = 4,       // last iteration: velocity/position update, no b reset
};

// ---- interactive drag and fixed rigid bodies (optional per engine)
enum : int { kFixedSphere = 0, kFixedPlane = 1, kFixedCylinder = 2 };

// One fixed rigid body: p.xyz = sphere/cylinder centre or a point of the
// plane, p.w = radius; n.xyz = plane normal or cylinder axis (unit),
// n.w = type.  Bodies are stored spheres first, then planes, then cylinders
// (the order FixedBodyData::HandleCollisions applies them).
struct FixedBodyDev {
    float4 p;
    float4 n;
};

struct SceneArgs {
    const float* drag_w;      // per-vertex drag weight (moreDBC); null: no drag
    const float4* drag_off;   // per-vertex offset from the grabbed vertex
    const float4* target;     // drag target, one float4 in device memory
    int drag_rhs;             // the system has pinned vertices, so dragged rows of b are overwritten
    float dt2;                // dt * dt
    float4* xt;               // XTilde (position after collision handling); null: X serves as XTilde
    const FixedBodyDev* fixed;
    int nfixed;
    float mu_t, mu_n;
    int ccd;                  // collision handling on: the step writes XTilde only; X and the
                              // fixed-body correction follow the collision response
    int* nonfinite;           // set to 1 when a vertex ends a step with a non-finite position or
                              // velocity (sticky until the state is set again); may be null
};

struct VertexArgs {
    int nv;
    float4* sn;
    float4* prev;
    float4* b;
    const float4* base;
    const float4* coef;
    const float4* pin_rhs;
    float4* x;
    float4* v;
    float omega;
    float dt_inv;
    SceneArgs sc;
};

struct BeginArgs {
    int nv;
    const float4* x;
    const float4* v;
    const float4* coef;
    const float4* pin_rhs;
    float4* sn;
    float4* base;
    float4* b;
    float dt;
    float gravity;
    // Cholesky path with tol > 0: reproduce the reference's
    // cudaMemset(prev_x, 0, 3 n) (a byte count, pdSolver.cu:162) on the
    // interleaved caller-order vector; null otherwise.
    float4* prev;
    const int* vperm;
    int* done;          // reset to 0 at step start (may be null)
    int* iterations;    // reset to the full count (may be null)
    int num_iterations;
    SceneArgs sc;
};

void launch_begin(const BeginArgs& a, cudaStream_t s);
// Multi-request forms (serving): one launch covers the work lists of all
// active requests; entries are {request index, tile or first vertex}.
void launch_begin_multi(const BeginArgs* req, const int2* list, const int* count, int grid, cudaStream_t s);
void launch_local_multi(const LocalArgs* req, const int2* list, const int* count, int grid, cudaStream_t s,
                        bool jacobi_form = true);
void launch_jacobi_vertex_multi(const VertexArgs* req, const int2* list, const int* count, int grid, int mode,
                                float omega, cudaStream_t s);
void launch_local(const LocalArgs& a, int ntiles, int max_patch, bool jacobi_form, int rotation, cudaStream_t s);
// Resident CTAs of the pipelined local step for this mesh's largest patch
// (2 per SM when its shared memory allows), capped at ntiles; 0 when it
// cannot run (the one-tile-per-CTA kernel is used).
int local_pipe_grid(int ntiles, int max_patch);
// Check of the bounded bulk-copy wait (pdgb_bulk_wait_check): src holds 64
// words 0..63; out[0] = timed out, out[1] = data intact.
void launch_bulk_wait_check(const void* src, int extra, unsigned long long limit_ns, int* out, cudaStream_t s);
void launch_jacobi_vertex(const VertexArgs& a, int mode, cudaStream_t s);
void launch_gather_state(int nv, const int* vperm, const float* X, const float* V, float4* x, float4* v,
                         cudaStream_t s);
void launch_scatter_state(int nv, const int* vperm, const float4* x, const float4* v, float* X, float* V,
                          cudaStream_t s);
void launch_copy_x0(int nv, const float4* x0, float4* x, float4* v, cudaStream_t s);

// Drag: per-vertex weights and offsets from caller order (gather); the
// selection kernel of the reference's mouse drag; the Cholesky-path RHS
// overwrite of dragged rows after the local step.
void launch_gather_drag(int nv, const int* vperm, const float* w, const float* off, float* drag_w, float4* drag_off,
                        cudaStream_t s);
void launch_drag_select(int nv, const float4* x, const float4* coef, int select_v, float control_mag,
                        double radius_sq, float* drag_w, float4* drag_off, cudaStream_t s);
void launch_drag_rhs(int nv, const SceneArgs& sc, const float4* base, float4* b, const int* done, cudaStream_t s);
void launch_copy_state(int nv, const float4* src, float4* dst, cudaStream_t s);
// The local step's rotation on n row-major 3x3 matrices (device arrays).
void launch_rotations(int n, const float* F, float* R, int rotation, cudaStream_t s);
// Surface positions / normals for rendering (tri_nor as float4 per corner).
void launch_render_surface(int n, const uint32_t* tris, const int* viperm, int nv, const float4* x, float* pos,
                           float* nor, cudaStream_t s);

}  // namespace pdgb
