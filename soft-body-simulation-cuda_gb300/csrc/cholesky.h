// Sparse Cholesky of the scalar PD system K (host side).
//
// The reference assembles A = K (x) I_3 (3n x 3n) from per-tet triplets
// (pdUtil.cu:9-54), orders it with cuSOLVER's host AMD and factors it in
// FP32 with cuSOLVER's low-level sparse Cholesky (cholesky.cu:72-158).  The
// engine factors the n x n scalar K once, in FP64 on the host (approximate
// minimum degree ordering, supernodal multifrontal LL^T), and solves the
// three coordinates together on the GPU.
//
// Solve representation.  For every supernode s with pivot columns C_s
// (k_s of them) and off-diagonal rows O_s (m_s - k_s), the GPU stores the
// m_s x k_s matrix
//     M_s = [ L_ss^-1 ; L_os L_ss^-1 ]       (column major, FP32)
// so that the forward step of s is y_s = L_ss^-1 r_s plus the update
// r_O -= (L_os L_ss^-1) r_s, and the backward step is
// x_s = (L_ss^-1)^T y_s - (L_os L_ss^-1)^T x_O: both are dense
// matrix-vector products with M_s.  Supernodes on the same level of the
// supernodal elimination tree are independent.
#pragma once

#include <cstdint>
#include <vector>

namespace pdgb {

struct SparseSym {
    int n = 0;
    std::vector<int64_t> p;  // CSR row pointers (full symmetric pattern, diagonal included)
    std::vector<int> i;
    std::vector<double> x;
};

// Approximate minimum degree ordering (Amestoy, Davis & Duff, SIAM J. Matrix
// Anal. Appl. 17(4), 1996): quotient graph with element absorption,
// approximate external degrees, mass elimination and supervariable
// detection.  Returns perm (perm[k] = row eliminated k-th).
std::vector<int> amd_order(const SparseSym& A);

// Geometric nested dissection (recursive coordinate bisection), an
// alternative ordering for meshes.  xyz: 3 floats per row.
std::vector<int> nd_order(const SparseSym& A, const float* xyz);

struct SolveLevel {
    int fwd_begin, fwd_end;  // warp work items of the forward pass for this level
    int bwd_begin, bwd_end;  // warp work items of the backward pass
    int fwdb_begin, fwdb_end;  // per-level launches: CTA block items (large supernodes)
    int bwdb_begin, bwdb_end;
    int fwdw_begin, fwdw_end;  // per-level launches: warp items of the small supernodes
    int bwdw_begin, bwdw_end;
    int tiny_begin, tiny_end;  // per-level launches: tiny supernodes, one thread each
    int zst_begin, zst_end;    // per-level launches: backward z staging of the block supernodes
};

// Warp work items, 8 ints each (two int4 loads, no dependent metadata loads):
//   forward : {moff_lo, moff_hi, roff, m, k, r0, c0, c1}: rows r0 .. min(r0+32, m)
//             of M_s (column major) times the right-hand side of pivot
//             columns c0 .. c1
//   backward: {moff_lo, moff_hi, roff, m, k, c, 0, 0}: pivot column c
constexpr int kItemInts = 8;
constexpr int kFwdItemRows = 32;
constexpr int kFwdItemCols = 64;
// CTA block items (same 8-int layout) of the per-level launches:
//   forward : {moff_lo, moff_hi, roff, m, k, r0, c0, c1}: rows r0 .. r0+128,
//             pivot columns c0 .. c1 (at most 256, staged in shared memory)
//   backward: {moff_lo, moff_hi, roff, m, r0, c0 | (c1 - c0) << 27, r1,
//             zoff}: pivot columns c0 .. c1 against rows r0 .. r1 of
//             z = [y_pivots ; -x_offdiag] of the supernode, staged once per
//             level at zbuf[zoff ..] by z-staging items
//             {moff_lo, moff_hi, roff, m, k, r0, split, zoff} of kStageRows
//             rows; when split != 0 the columns are split into row chunks
//             that add their partial sums into x, and staging clears x at
//             the pivot rows first
// Supernodes with at least kBlockMinRows rows use block items in the
// per-level launches; smaller ones keep warp items (packed 4 per CTA).
// Columns per forward block item and per warp of a backward block item.
// With the amalgamated supernodes, 32 forward columns (against 16) solve the
// 512-body batch in 677 instead of 703 us and the 40^3 cube in 182 instead
// of 188 us (same box).
#ifndef PDGB_FWDB_COLS
#define PDGB_FWDB_COLS 32
#endif
#ifndef PDGB_BWD_WARP_COLS
#define PDGB_BWD_WARP_COLS 2
#endif
// Rows of one backward block item of a single-body factor: a column's rows
// are split into chunks so that no warp walks a long column alone.  (A
// batch's levels hold many bodies' supernodes, enough parallelism without
// the split, which would only add items and atomics: there a column is one
// item.)
#ifndef PDGB_BWD_CHUNK_ROWS
#define PDGB_BWD_CHUNK_ROWS 256
#endif
constexpr int kBwdColShift = 27;  // backward block: c1 - c0 above c0 in one int
#ifndef PDGB_BLOCK_MIN_ROWS
#define PDGB_BLOCK_MIN_ROWS 64
#endif
// Tiny supernodes (at most kTinyCols pivots and kTinyRows rows -- most of
// them are leaves with one pivot) are solved one per thread in the per-level
// launches: descriptor {moff_lo, moff_hi, roff, m, k, 0, 0, 0}.
#ifndef PDGB_TINY_COLS
#define PDGB_TINY_COLS 1
#endif
#ifndef PDGB_TINY_ROWS
#define PDGB_TINY_ROWS 32
#endif
constexpr int kTinyCols = PDGB_TINY_COLS;
constexpr int kTinyRows = PDGB_TINY_ROWS;
constexpr int kFwdBlockRows = 128;
constexpr int kFwdBlockCols = PDGB_FWDB_COLS;
constexpr int kBwdWarpCols = PDGB_BWD_WARP_COLS;   // backward block: columns per warp (4 warps)
constexpr int kBwdBlockCols = 4 * kBwdWarpCols;
static_assert(kBwdBlockCols < (1 << (32 - kBwdColShift)), "backward block: column count field");
static_assert(kFwdBlockCols <= 128, "forward block: pivot right-hand sides staged by the first threads");
constexpr int kStageRows = 128;
constexpr int kBwdChunkRows = PDGB_BWD_CHUNK_ROWS;
constexpr int kBlockMinRows = PDGB_BLOCK_MIN_ROWS;

// Numeric factorisation on the GPU (factor.cu): everything the device needs
// beyond the symbolic structure of CholFactor.  Each supernode s has a dense
// front F_s (m_s x m_s, column major, FP64) in one pool, followed by an
// m_s x k_s FP64 block for M_s; F_s receives the entries of K in its pivot
// columns and the Schur complements of its children (extend-add), is
// factored over its first k_s columns, and its own Schur complement
// F_s[k_s:, k_s:] is then added into its parent's front.  Fronts live from
// their level until their parent's level is assembled, and the pool reuses
// the memory of the fronts that are done.
struct FrontPlan {
    bool on = false;                   // mval is left to the GPU
    int64_t pool = 0;                  // doubles in the front pool
    int max_m = 0;                     // largest front
    std::vector<int64_t> foff;         // [nsuper] front offset in the pool
    std::vector<int> parent;           // [nsuper] parent supernode, -1 for a root
    std::vector<int> child_ptr, child; // children of each supernode ([nsuper + 1] / [nsuper])
    std::vector<int> rel_ptr, rel;     // rows of s past its pivots, as positions in its parent's row list
    std::vector<int> kptr;             // [nsuper + 1] entries of K in the pivot columns of s
    std::vector<int> kpos;             // position of the entry in F_s (column * m_s + row)
    std::vector<double> kval;
    std::vector<int> lvl_ptr, lvl_sn;  // supernodes by level (from the leaves, all bodies together)
};

struct CholFactor {
    int n = 0;
    long long nnz_L = 0;             // nnz of the scalar factor (incl. diagonal)
    int nsuper = 0;
    double flops = 0.0;
    // per supernode
    std::vector<int> sk, sm;         // pivot count k_s, row count m_s
    std::vector<int64_t> moff;       // offset of M_s in mval (column major m x k)
    std::vector<int> roff;           // offset of the row list in rows
    std::vector<int> rows;           // row lists (vertex ids; first k = pivots)
    std::vector<float> mval;         // FP32 M_s blocks, column major
    std::vector<int> level;          // level of each supernode (leaves = 0)
    int nlevels = 0;
    // GPU warp work items grouped by level (see kItemInts).
    std::vector<int> fwd_items;
    std::vector<int> bwd_items;
    std::vector<int> fwd_blocks;     // CTA block items (see kFwdBlockRows)
    std::vector<int> bwd_blocks;
    std::vector<int> fwd_small;      // warp items of the small supernodes (per-level launches)
    std::vector<int> bwd_small;
    std::vector<int> tiny;           // tiny supernode descriptors (per-level launches)
    std::vector<int> zstage;         // backward z-staging items of the block supernodes
    int64_t zrows = 0;               // rows of the z staging buffer
    std::vector<SolveLevel> levels;  // body-major: body b owns levels[body_level[b] .. body_level[b+1])
    // Per-level launches (block and small items): level L of every body in
    // one launch, levels counted from the leaves.  Equal to `levels` for a
    // single body.
    std::vector<SolveLevel> step_levels;
    std::vector<int> body_level;     // [nbodies + 1]
    std::vector<int> body_order;     // bodies by decreasing stored factor size (batch solve order)
    long long zeros = 0;             // explicit zeros stored by amalgamated supernodes
    // FP64 copy of K for refinement residuals (CSR over vertex ids)
    SparseSym K;
    int64_t mval_size = 0;           // FP32 entries of the M_s blocks (= mval.size() when factored on the host)
    FrontPlan fp;                    // numeric factorisation left to the GPU (fp.on)
};

// Plan of the distributed-shared-memory solve of a single body: an 8-CTA
// cluster, each CTA owning a set of supernodes whose M_s blocks and row
// lists it stages into its shared memory once per solve; the right-hand
// side, y and x live in the cluster's shared memory, vertex v in CTA v % 8
// at slot v / 8.  Items use the warp-item layout with shared-memory offsets:
//   forward : {m_off, r_off, m, k, r0, c0, c1, 0}; backward: {m_off, r_off, m, k, c, 0, 0, 0}.
struct DsmPlan {
    bool ok = false;
    int ctas = 0;                 // cluster size
    int n = 0;                    // vertices
    int slots = 0;                // vector slots per CTA (ceil(n / ctas))
    int nlevels = 0;
    int m_area = 0;               // float index of the staged M area in shared memory
    int r_area = 0;               // int index of the staged row area
    size_t smem_bytes = 0;        // dynamic shared memory per CTA
    // Each CTA's staged areas, laid out as in its shared memory and stored
    // contiguously per CTA, so that staging is one wide copy per CTA.
    std::vector<float> mcopy;     // M_s blocks of CTA c at [mcopy_ptr[c], mcopy_ptr[c+1])
    std::vector<int> mcopy_ptr;   // [ctas + 1], multiples of 4
    std::vector<int> rcopy;       // row lists of CTA c at [rcopy_ptr[c], rcopy_ptr[c+1])
    std::vector<int> rcopy_ptr;   // [ctas + 1], multiples of 4
    std::vector<int> items;       // kItemInts per item, each CTA's items grouped by level
    std::vector<int> lvl;         // [ctas][nlevels] x {fwd_begin, fwd_end, bwd_begin, bwd_end}
};
// Fills the plan for a single-body factor when the busiest CTA's share fits
// max_smem bytes of shared memory; plan.ok tells whether it does.
void build_dsm_plan(const CholFactor& f, int ctas, int warps_per_cta, size_t max_smem, DsmPlan& plan);

// Factors K (vertex-indexed, n x n SPD).  ordering: 0 = AMD, 1 = nested
// dissection (xyz required), 2 = AMD order stored as one dense supernode.  Throws Error(PDGB_ERR_NOT_SPD) if a pivot is
// not positive.  bwd_chunk_rows: rows per backward block item (0: whole
// columns).
// gpu_numeric: stop after the symbolic analysis and fill out.fp for the
// GPU factorisation (factor.cu) instead of computing mval on the host;
// finish_plan: complete it (finish_front_plan) -- a batch completes the
// combined plan of its bodies instead.
// amalgamation: how many explicit zeros a supernode may take on when it is
// merged into its parent (kAmalgChain for the engine's solves, bound by
// their chain of levels; kAmalgBytes for the serving step, bound by the
// factor's bytes).
enum : int { kAmalgChain = 0, kAmalgBytes = 1 };
void cholesky_factor(const SparseSym& K, int ordering, const float* xyz, CholFactor& out,
                     int bwd_chunk_rows = kBwdChunkRows, bool gpu_numeric = false, bool finish_plan = true,
                     int amalgamation = kAmalgChain);

// Factors the block-diagonal system of independent bodies, one block per
// body (vertex range vstart[b]..vstart[b+1], tets tstart[b]..tstart[b+1] in
// the engine's order), in parallel over bodies, and concatenates the
// factors: rows keep engine vertex ids, work items and levels are grouped
// per body.
void cholesky_factor_bodies(int nbodies, const std::vector<int>& vstart, const std::vector<int>& tstart,
                            const uint32_t* tets4, const double* dminv, const double* coef,
                            const std::vector<double>& mdt2, int ordering, const float* xyz, CholFactor& out,
                            bool gpu_numeric = false);

// Doubles of the pool that supernode s takes: its front and its M_s block.
int64_t front_doubles(const CholFactor& f, int s);

// Numeric factorisation of the plan f.fp on the GPU (factor.cu): writes the
// FP32 M_s blocks (f.mval_size floats, device memory) and returns the device
// time in ms.  Waits for the stream.  Throws Error(PDGB_ERR_NOT_SPD) when a
// pivot is not positive.
double gpu_factor(const CholFactor& f, float* mval, void* stream);

// Completes out.fp once the supernodes of all bodies are in place: children
// lists, supernodes by level, and the front pool (best-fit reuse of the
// fronts whose parents are assembled).
void finish_front_plan(CholFactor& out);

// Applies the factor on the host exactly as the GPU work items do
// (forward by levels with M_s, backward by levels), in double: x = K^-1 b
// for 3 interleaved right-hand sides indexed by vertex id.
void cholesky_solve_host(const CholFactor& f, const double* b3, double* x3);

// Assembles K = diag(mdt2) + sum_t c_t B_t^T B_t for tets given by internal
// vertex ids (tets4), DmInv (9 doubles per tet, row major) and c_t.
SparseSym assemble_system(int nv, int nt, const uint32_t* tets4, const double* dminv, const double* coef,
                          const std::vector<double>& mdt2);

// The scalar system K of a single body's layout, in its internal vertex
// order: M/h^2 from the float coefficients the kernels use (pin weight
// included) and the double geometry.
struct HostLayout;
SparseSym layout_system(const HostLayout& L);

// Rest positions of a layout as 3 floats per vertex (the nested-dissection
// ordering's coordinates).
std::vector<float> layout_xyz(const HostLayout& L);

}  // namespace pdgb
