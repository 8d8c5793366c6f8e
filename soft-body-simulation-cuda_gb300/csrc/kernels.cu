// Hot-path kernels of the pdgb PD engine (sm_103a).
//
//   k_local        per-tet corotational projection + RHS scatter
//                  (reference: PdUtil::computeLocal, pdUtil.cu:97-145)
//   k_jacobi_vertex Jacobi update + Chebyshev blend + pinned-RHS overwrite
//                  + b reset, fused; last iteration also does the velocity /
//                  position update (reference: getErrorKern, chebyshevKern,
//                  computeDBCLocal, addM_h2Sn, updateVelPos; pdUtil.cu:147-226)
//   k_begin        step prologue: gravity, s_n, M/h^2 s_n (reference:
//                  pdSolver.cu:154-163, computeSn pdUtil.cu:73-95)
#include <algorithm>
#include <mutex>

#include "engine.h"
#include "pdl.cuh"
#include "scene.cuh"
#include "relax.cuh"
#include "rotation.cuh"
#include "bulk.cuh"

namespace pdgb {

// ------------------------------------------------------------ local step
// One tet: corner positions from the patch, F' = Ds D', its closest
// rotation R, and the 4 corner contributions of (g R [- F']) D'^T G written
// to their slots (run start of the corner's patch vertex + its rank).
// ga, gb, gc: the tet's geometry planes (D' = g DmInv row major, g);
// rec: its 4 corner records k | r << kPatchBits.
template <bool kJacobiForm, int kRotation>
__device__ __forceinline__ void tet_contrib(const float4 ga, const float4 gb, const float2 gc, const uint2 rec,
                                            const float4* __restrict__ pos, float4* __restrict__ slot) {
    constexpr uint32_t kPatchMask = (1u << kPatchBits) - 1u;
    // D' = g DmInv (row major) and g = sqrt(V0 w)
    const float D[9] = {ga.x, ga.y, ga.z, ga.w, gb.x, gb.y, gb.z, gb.w, gc.x};
    const float g = gc.y;
    const uint32_t w0 = rec.x & 0xffffu, w1 = rec.x >> 16, w2 = rec.y & 0xffffu, w3 = rec.y >> 16;
    const float4 p0 = pos[w0 & kPatchMask], p1 = pos[w1 & kPatchMask], p2 = pos[w2 & kPatchMask],
                 p3 = pos[w3 & kPatchMask];
    // slots of the 4 corners, two 16-bit slot numbers per register
    const uint32_t s01 = (uint32_t)(__float_as_int(p0.w) + (int)(w0 >> kPatchBits)) |
                         ((uint32_t)(__float_as_int(p1.w) + (int)(w1 >> kPatchBits)) << 16);
    const uint32_t s23 = (uint32_t)(__float_as_int(p2.w) + (int)(w2 >> kPatchBits)) |
                         ((uint32_t)(__float_as_int(p3.w) + (int)(w3 >> kPatchBits)) << 16);
    // Ds columns = edges; F' = Ds * D' = g F (row-major F[r][c])
    const float e[3][3] = {{p1.x - p0.x, p2.x - p0.x, p3.x - p0.x},
                           {p1.y - p0.y, p2.y - p0.y, p3.y - p0.y},
                           {p1.z - p0.z, p2.z - p0.z, p3.z - p0.z}};
    float F[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            F[3 * r + cc] = fmaf(e[r][0], D[cc], fmaf(e[r][1], D[3 + cc], e[r][2] * D[6 + cc]));
    // closest rotation of F' (that of F: g > 0 scales the singular values)
    float R[9];
    if (kRotation == PDGB_ROTATION_SVD) closest_rotation(F, R);
    else closest_rotation_horn(F, R);
    // c (R - F) DmInv^T = (g R - F') D'^T ; c R DmInv^T = (g R) D'^T
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = kJacobiForm ? fmaf(g, R[k], -F[k]) : g * R[k];
    // M = R D'^T ; contributions: corner 0 = -(M0+M1+M2), corner j = M_{j-1}
    float M[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            M[3 * r + cc] = fmaf(R[3 * r], D[3 * cc], fmaf(R[3 * r + 1], D[3 * cc + 1], R[3 * r + 2] * D[3 * cc + 2]));
    }
    const int s0 = s01 & 0xffff, s1 = s01 >> 16, s2 = s23 & 0xffff, s3 = s23 >> 16;
    slot[s0] = make_float4(-(M[0] + M[1] + M[2]), -(M[3] + M[4] + M[5]), -(M[6] + M[7] + M[8]), 0.f);
    slot[s1] = make_float4(M[0], M[3], M[6], 0.f);
    slot[s2] = make_float4(M[1], M[4], M[7], 0.f);
    slot[s3] = make_float4(M[2], M[5], M[8], 0.f);
}

// Sum of patch vertex k's run of slots e0 .. e1, added to b[v] with one
// float4 atomic.  The run is summed from a lane-dependent start (then
// wrapping), so that the 8 lanes of a quarter-warp read 8 different 16-byte
// bank groups while their runs last, instead of colliding at random.
__device__ __forceinline__ void add_run(const float4* __restrict__ slot, int k, int e0, int e1, float4* b,
                                        uint32_t v) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    const int len = e1 - e0;
    int off = (k - e0) & 7;
    if (off >= len) off = 0;
    int e = e0 + off;
    for (int j = 0; j < len; ++j) {
        const float4 q = slot[e];
        sx += q.x;
        sy += q.y;
        sz += q.z;
        if (++e == e1) e = e0;
    }
    atomicAdd(&b[v], make_float4(sx, sy, sz, 0.f));
}

// One CTA per tile of Morton-ordered tets.  (1) Every patch vertex k is
// loaded once (coalesced over the patch list) into pos[k], with the start of
// its run of slots in the w lane.  (2) Every tet reads its 4 corner
// positions (corner records k | r << kPatchBits, loaded with its geometry),
// computes F = Ds DmInv, the closest rotation R (minus F in the Jacobi
// residual form) and the corner contributions c R DmInv^T G, and writes each
// to its slot: run start of k + rank r.  The slots of a tile are ordered by
// patch vertex, so patch vertex k owns the contiguous slots inc_end[k-1] ..
// inc_end[k].  (3) Every patch vertex sums its run of slots and adds the sum
// to b with one float4 atomic (pinned vertices are skipped: their RHS is the
// pin term).  No shared-memory atomics; within a tile the sums are
// deterministic.
template <bool kJacobiForm, int kRotation>
__device__ __forceinline__ void local_tile(const LocalArgs& a, int tile, float4* slot, float4* pos) {
    pdl_trigger();
    const int vb = a.tile_vptr[tile];
    const int np = a.tile_vptr[tile + 1] - vb;
    const int t0 = a.tile_tet_ptr[tile], t1 = a.tile_tet_ptr[tile + 1];
    const int ntile = t1 - t0;
    const uint16_t* iend = a.inc_end + vb;
    // The first tet's geometry and corner records are issued before the
    // patch positions are gathered (in flight meanwhile); the second tet's
    // after the barrier, so that phase 1 holds one tet's registers, not two.
    constexpr int kPer = kTileTets / kLocalThreads;
    const int ntp = a.nt_pad;
    const float4* geo0 = reinterpret_cast<const float4*>(a.geo);
    const float2* geo2 = reinterpret_cast<const float2*>(a.geo + 8 * (size_t)ntp);
    float4 GA[kPer], GB[kPer];
    float2 GC[kPer];
    uint2 S[kPer];
    {
        const int lt = threadIdx.x;
        const int t = t0 + (lt < ntile ? lt : 0);
        GA[0] = __ldg(geo0 + t);
        GB[0] = __ldg(geo0 + ntp + t);
        GC[0] = __ldg(geo2 + t);
        S[0] = __ldg(reinterpret_cast<const uint2*>(a.inc_ent) + t);
    }
    // the tile's layout and first geometry are in flight; positions, b and
    // the early-exit flag come from earlier kernels of the step
    pdl_wait();
    if (a.done && *a.done) return;
    // the first patch vertex of each thread keeps its id and slot run in
    // registers for the reduction phase
    uint32_t v_first = kPinnedBit;
    int e0_first = 0, e1_first = 0;
    for (int k = threadIdx.x; k < np; k += kLocalThreads) {
        const uint32_t v = __ldg(&a.tile_verts[vb + k]);
        const float4 p = __ldg(&a.sn[v & ~kPinnedBit]);
        const int e0 = k ? __ldg(&iend[k - 1]) : 0;
        pos[k] = make_float4(p.x, p.y, p.z, __int_as_float(e0));
        if (k == (int)threadIdx.x) {
            v_first = v;
            e0_first = e0;
            e1_first = __ldg(&iend[k]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 1; j < kPer; ++j) {
        const int lt = threadIdx.x + j * kLocalThreads;
        const int t = t0 + (lt < ntile ? lt : 0);
        GA[j] = __ldg(geo0 + t);
        GB[j] = __ldg(geo0 + ntp + t);
        GC[j] = __ldg(geo2 + t);
        S[j] = __ldg(reinterpret_cast<const uint2*>(a.inc_ent) + t);
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int lt = threadIdx.x + j * kLocalThreads;
        if (lt >= ntile) break;
        tet_contrib<kJacobiForm, kRotation>(GA[j], GB[j], GC[j], S[j], pos, slot);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < np; k += kLocalThreads) {
        const bool first = k == (int)threadIdx.x;
        const uint32_t v = first ? v_first : __ldg(&a.tile_verts[vb + k]);
        if (v & kPinnedBit) continue;
        const int e0 = first ? e0_first : __ldg(&iend[k - 1]);
        const int e1 = first ? e1_first : __ldg(&iend[k]);
        add_run(slot, k, e0, e1, a.b, v);
    }
}

// Resident CTAs per SM the register allocation of the local step aims for.
#ifndef PDGB_LOCAL_MIN_BLOCKS
#define PDGB_LOCAL_MIN_BLOCKS 4
#endif

// Shared memory: the tile's slots (static) and its patch positions
// (dynamic, 16 bytes per patch vertex of the largest tile).
template <bool kJacobiForm, int kRotation>
__global__ void __launch_bounds__(kLocalThreads, PDGB_LOCAL_MIN_BLOCKS) k_local(LocalArgs a) {
    __shared__ float4 slot[4 * kTileTets];
    extern __shared__ float4 pos[];
    local_tile<kJacobiForm, kRotation>(a, blockIdx.x, slot, pos);
}

// Multi-request form (serving): CTA i runs tile list[i] of request
// descriptor req[list[i].x]; CTAs beyond *count exit.
template <bool kJacobiForm>
__global__ void __launch_bounds__(kLocalThreads) k_local_multi(const LocalArgs* __restrict__ req,
                                                               const int2* __restrict__ list,
                                                               const int* __restrict__ count) {
    __shared__ float4 slot[4 * kTileTets];
    extern __shared__ float4 pos[];
    if ((int)blockIdx.x >= *count) return;
    const int2 w = list[blockIdx.x];
    local_tile<kJacobiForm, PDGB_ROTATION_QUAT>(req[w.x], w.y, slot, pos);
}

void launch_local_multi(const LocalArgs* req, const int2* list, const int* count, int grid, cudaStream_t s,
                        bool jacobi_form) {
    if (grid <= 0) return;
    if (jacobi_form) k_local_multi<true><<<grid, kLocalThreads, kMaxPatch * sizeof(float4), s>>>(req, list, count);
    else k_local_multi<false><<<grid, kLocalThreads, kMaxPatch * sizeof(float4), s>>>(req, list, count);
}

// ------------------------------------------------ pipelined local step
// Persistent form of the same tile computation, with the tile form's shape
// (kLocalThreads threads, two tets each, 4 CTAs per SM): the CTAs of the grid
// walk the tiles blockIdx.x, blockIdx.x + gridDim.x, ...  What a tile needs
// at its start -- its patch list and run ends (double-buffered) and the
// geometry planes and corner records of its first kLocalThreads tets (single
// buffer) -- is bulk-copied into shared memory (cp.async.bulk on mbarriers)
// during the previous tile, so a tile no longer starts with a chain of
// waits for its bounds, its patch list and its geometry.  The second half's
// geometry is loaded into registers after barrier A, as in the tile form.
// Per tile:
//   gather pos from the copied patch list (sn stays in L2); barrier A (pos
//   complete; the previous tile's run sums are done, so the other patch
//   buffer is free): thread 0 issues the next tile's patch copy; wait for
//   this tile's geometry copy; tet contributions -> slots; barrier B (the
//   geometry buffer has been read): thread 0 issues the next tile's geometry
//   copy; run sums -> b.
// A bounded wait that runs out sets *a.timeout and the CTA stops after its
// copies in flight have landed (or a second bound has passed).
constexpr uint64_t kPipeWaitNs = 1000000000ull;  // 1 s

// Shared-memory carve of the pipelined kernel for patches of up to P
// vertices (P rounded up to a multiple of 8): byte offsets, 128-aligned.
struct PipeCarve {
    uint32_t ga, gb, gc, ent, slot, pos, tv, ie, bar, info, total;
    int pstride;  // entries per buffer of tv / ie beyond P
};
__host__ __device__ inline PipeCarve pipe_carve(int max_patch) {
    PipeCarve c;
    const uint32_t P = (uint32_t)((max_patch + 7) & ~7);
    uint32_t o = 0;
    auto take = [&o](uint32_t bytes) {
        const uint32_t r = o;
        o = (o + bytes + 127u) & ~127u;
        return r;
    };
    c.ga = take(kLocalThreads * 16u);
    c.gb = take(kLocalThreads * 16u);
    c.gc = take((kLocalThreads + 8u) * 8u);
    c.ent = take((kLocalThreads + 8u) * 8u);
    c.slot = take(4u * kTileTets * 16u);
    c.pos = take(P * 16u);
    c.tv = take(2u * (P + 8u) * 4u);
    c.ie = take(2u * (P + 16u) * 2u);
    c.bar = take(3u * 8u);
    c.info = take(2u * 16u);
    c.total = o;
    c.pstride = (int)P;
    return c;
}

// Tile bounds as the copy issuer keeps them: tets t0..t1, patch vb..ve.
struct TileBounds {
    int t0, t1, vb, ve;
};
__device__ __forceinline__ TileBounds tile_bounds(const LocalArgs& a, int tile) {
    return TileBounds{__ldg(&a.tile_tet_ptr[tile]), __ldg(&a.tile_tet_ptr[tile + 1]), __ldg(&a.tile_vptr[tile]),
                      __ldg(&a.tile_vptr[tile + 1])};
}

template <bool kJacobiForm, int kRotation>
__global__ void __launch_bounds__(kLocalThreads, PDGB_LOCAL_MIN_BLOCKS) k_local_pipe(LocalArgs a, int ntiles,
                                                                                     int max_patch) {
    extern __shared__ __align__(128) unsigned char smem[];
    const PipeCarve C = pipe_carve(max_patch);
    float4* ga = reinterpret_cast<float4*>(smem + C.ga);
    float4* gb = reinterpret_cast<float4*>(smem + C.gb);
    float2* gc = reinterpret_cast<float2*>(smem + C.gc);
    uint2* ent = reinterpret_cast<uint2*>(smem + C.ent);
    float4* slot = reinterpret_cast<float4*>(smem + C.slot);
    float4* pos = reinterpret_cast<float4*>(smem + C.pos);
    uint32_t* tv = reinterpret_cast<uint32_t*>(smem + C.tv);
    uint16_t* ie = reinterpret_cast<uint16_t*>(smem + C.ie);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C.bar);  // [0], [1]: patch buffers; [2]: geometry
    int4* info = reinterpret_cast<int4*>(smem + C.info);
    const int tvs = C.pstride + 8, ies = C.pstride + 16;  // per-buffer strides (entries)
    const int tid = threadIdx.x;
    const int ntp = a.nt_pad;
    const float4* geo_a = reinterpret_cast<const float4*>(a.geo);
    const float4* geo_b = geo_a + ntp;
    const float2* geo_c = reinterpret_cast<const float2*>(a.geo + 8 * (size_t)ntp);
    const uint2* recs = reinterpret_cast<const uint2*>(a.inc_ent);

    // Thread 0: copies of a tile's patch list and run ends into patch buffer
    // pbuf (ranges rounded out to 16 bytes; the arrays are padded for that),
    // info[pbuf] = {t0, tets, vb, patch size}.
    auto issue_patch = [&](const TileBounds& tb, int pbuf) {
        const int v0 = tb.vb & ~3, v1 = (tb.ve + 3) & ~3;
        const int i0 = tb.vb & ~7, i1 = (tb.ve + 7) & ~7;
        const uint32_t bytes_v = (uint32_t)(v1 - v0) * 4u, bytes_i = (uint32_t)(i1 - i0) * 2u;
        mbar_expect_tx(&bar[pbuf], bytes_v + bytes_i);
        bulk_load(tv + pbuf * tvs, a.tile_verts + v0, bytes_v, &bar[pbuf]);
        bulk_load(ie + pbuf * ies, a.inc_end + i0, bytes_i, &bar[pbuf]);
        info[pbuf] = make_int4(tb.t0, tb.t1 - tb.t0, tb.vb, tb.ve - tb.vb);
    };
    // Thread 0: copies of the geometry and corner records of a tile's first
    // kLocalThreads tets into the geometry buffer.
    auto issue_geo = [&](const TileBounds& tb) {
        const int n = min(tb.t1 - tb.t0, kLocalThreads);
        const int c0 = tb.t0 & ~1, c1 = (tb.t0 + n + 1) & ~1;
        const uint32_t bytes_g = (uint32_t)n * 16u, bytes_c = (uint32_t)(c1 - c0) * 8u;
        mbar_expect_tx(&bar[2], 2u * bytes_g + 2u * bytes_c);
        bulk_load(ga, geo_a + tb.t0, bytes_g, &bar[2]);
        bulk_load(gb, geo_b + tb.t0, bytes_g, &bar[2]);
        bulk_load(gc, geo_c + c0, bytes_c, &bar[2]);
        bulk_load(ent, recs + c0, bytes_c, &bar[2]);
    };
    // Gathers the positions of the tile in patch buffer pbuf into pos (w
    // lane: the start of the vertex's run of slots).
    auto gather = [&](int pbuf) {
        const int4 in = info[pbuf];
        const uint32_t* tvb = tv + pbuf * tvs + (in.z & 3);
        const uint16_t* ieb = ie + pbuf * ies + (in.z & 7);
        for (int k = tid; k < in.w; k += kLocalThreads) {
            const float4 p = __ldg(&a.sn[tvb[k] & ~kPinnedBit]);
            pos[k] = make_float4(p.x, p.y, p.z, __int_as_float(k ? (int)ieb[k - 1] : 0));
        }
    };

    TileBounds next{};  // thread 0: bounds of the next tile
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        mbar_init_fence();
        const TileBounds first = tile_bounds(a, blockIdx.x);  // the layout is not written by earlier kernels
        issue_patch(first, 0);
        issue_geo(first);
        if ((int)(blockIdx.x + gridDim.x) < ntiles) next = tile_bounds(a, blockIdx.x + gridDim.x);
    }
    __syncthreads();
    pdl_trigger();
    pdl_wait();
    if (a.done && *a.done) {
        // the first copies may still be landing in shared memory
        mbar_wait_bounded(&bar[0], 0, kPipeWaitNs);
        mbar_wait_bounded(&bar[2], 0, kPipeWaitNs);
        return;
    }
    bool ok = mbar_wait_bounded(&bar[0], 0, kPipeWaitNs);
    if (ok) gather(0);
    for (int it = 0;; ++it) {
        const int tile = blockIdx.x + it * gridDim.x;
        const int pb = it & 1;
        const bool more = tile + (int)gridDim.x < ntiles;
        // barrier A: pos is complete; the previous tile's run sums are done
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(a.timeout, 1);
            mbar_wait_bounded(&bar[pb], (it >> 1) & 1, kPipeWaitNs);
            mbar_wait_bounded(&bar[2], it & 1, kPipeWaitNs);
            break;
        }
        if (tid == 0 && more) {
            fence_proxy_async_smem();
            issue_patch(next, pb ^ 1);
        }
        const int4 in = info[pb];
        const int t0 = in.x, ntile = in.y, oc = t0 & 1;
        // the second half's geometry, into registers (in flight during the first tet)
        const int lt1 = tid + kLocalThreads;
        const int t1i = t0 + (lt1 < ntile ? lt1 : 0);
        const float4 ga1 = __ldg(geo_a + t1i), gb1 = __ldg(geo_b + t1i);
        const float2 gc1 = __ldg(geo_c + t1i);
        const uint2 s1 = __ldg(recs + t1i);
        ok = mbar_wait_bounded(&bar[2], it & 1, kPipeWaitNs);
        if (ok && tid < ntile)
            tet_contrib<kJacobiForm, kRotation>(ga[tid], gb[tid], gc[oc + tid], ent[oc + tid], pos, slot);
        if (ok && lt1 < ntile) tet_contrib<kJacobiForm, kRotation>(ga1, gb1, gc1, s1, pos, slot);
        // barrier B: the slots are complete; the geometry buffer has been read
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(a.timeout, 1);
            mbar_wait_bounded(&bar[2], it & 1, kPipeWaitNs);
            if (more) mbar_wait_bounded(&bar[pb ^ 1], ((it + 1) >> 1) & 1, kPipeWaitNs);
            break;
        }
        if (tid == 0 && more) {
            fence_proxy_async_smem();
            issue_geo(next);
            const int after = tile + 2 * (int)gridDim.x;
            if (after < ntiles) next = tile_bounds(a, after);
        }
        const uint32_t* tvb = tv + pb * tvs + (in.z & 3);
        const uint16_t* ieb = ie + pb * ies + (in.z & 7);
        for (int k = tid; k < in.w; k += kLocalThreads) {
            const uint32_t v = tvb[k];
            if (v & kPinnedBit) continue;
            add_run(slot, k, k ? (int)ieb[k - 1] : 0, (int)ieb[k], a.b, v);
        }
        if (!more) break;
        // the next tile's positions, as soon as this thread has no more runs
        ok = mbar_wait_bounded(&bar[pb ^ 1], ((it + 1) >> 1) & 1, kPipeWaitNs);
        if (ok) gather(pb ^ 1);
    }
}

// Raises the kernel's dynamic shared-memory limit once per device (function
// attributes are per device), then asks for its resident CTAs per SM.
template <bool kJacobiForm>
static int pipe_occupancy(size_t smem) {
    constexpr int kDevices = 64;
    static std::mutex mu;
    static signed char set[kDevices] = {};  // 0: not yet, 1: done, -1: refused
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) return 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!set[dev])
            set[dev] = cudaFuncSetAttribute(k_local_pipe<kJacobiForm, PDGB_ROTATION_QUAT>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)pipe_carve(kMaxPatch).total) == cudaSuccess
                           ? 1
                           : -1;
        if (set[dev] < 0) return 0;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_local_pipe<kJacobiForm, PDGB_ROTATION_QUAT>,
                                                      kLocalThreads, smem) != cudaSuccess)
        return 0;
    return nb;
}

int local_pipe_grid(int ntiles, int max_patch) {
    if (ntiles <= 0 || max_patch < 1 || max_patch > kMaxPatch) return 0;
    const size_t smem = pipe_carve(max_patch).total;
    const int nb = std::min(pipe_occupancy<true>(smem), pipe_occupancy<false>(smem));
    int dev = 0, sms = 0;
    if (nb <= 0 || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    cudaGetLastError();
    return std::min(ntiles, nb * sms);
}

// Check kernel of the bounded bulk-copy wait (one CTA of 32 threads):
// thread 0 registers 256 + extra bytes on an mbarrier and copies 256; every
// thread waits with the given bound.  out[0] = 1 if the wait timed out in
// any thread, out[1] = 1 if the copied words arrived intact (checked only
// when the phase completed).
__global__ void k_bulk_wait_check(const uint4* __restrict__ src, int extra, unsigned long long limit_ns, int* out) {
    __shared__ __align__(128) uint4 buf[16];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, 256u + (uint32_t)extra);
        bulk_load(buf, src, 256u, &bar);
    }
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    const bool any_late = __syncthreads_or(!ok);
    if (any_late) {
        // the phase cannot complete, so its copy's arrival is not observable
        // on the barrier: give the copy (microseconds, against a bound of at
        // least 1 ms) a further 100 us before the CTA's shared memory is freed
        const uint64_t t0 = global_ns();
        while (global_ns() - t0 < 100000ull) __nanosleep(1000);
    }
    if (threadIdx.x == 0) {
        out[0] = any_late ? 1 : 0;
        int good = 0;
        if (!any_late) {
            good = 1;
            for (int k = 0; k < 16; ++k)
                good &= buf[k].x == 4u * k && buf[k].y == 4u * k + 1 && buf[k].z == 4u * k + 2 && buf[k].w == 4u * k + 3;
        }
        out[1] = good;
    }
}

void launch_bulk_wait_check(const void* src, int extra, unsigned long long limit_ns, int* out, cudaStream_t s) {
    k_bulk_wait_check<<<1, 32, 0, s>>>(reinterpret_cast<const uint4*>(src), extra, limit_ns, out);
}

// The plain form (Cholesky path) is launched with programmatic dependent
// launch: its CTAs load their tile layout and first geometry while the
// preceding kernel drains.  On the Jacobi path, local step and vertex update
// alternate 20 times per step and plain launches measured faster.
void launch_local(const LocalArgs& a, int ntiles, int max_patch, bool jacobi_form, int rotation, cudaStream_t s) {
    if (ntiles <= 0) return;
    if (max_patch < 1 || max_patch > kMaxPatch)
        throw Error{PDGB_ERR_INVALID_ARGUMENT, "local step: tile patch size out of range"};
    if (a.pipe_grid > 0 && rotation == PDGB_ROTATION_QUAT) {
        if (!a.timeout) throw Error{PDGB_ERR_INVALID_ARGUMENT, "local step: pipelined form without a status word"};
        const size_t smp = pipe_carve(max_patch).total;
        if (jacobi_form) k_local_pipe<true, PDGB_ROTATION_QUAT><<<a.pipe_grid, kLocalThreads, smp, s>>>(a, ntiles, max_patch);
        else launch_pdl(k_local_pipe<false, PDGB_ROTATION_QUAT>, a.pipe_grid, kLocalThreads, smp, s, a, ntiles, max_patch);
        return;
    }
    const size_t sm = (size_t)max_patch * sizeof(float4);
    if (rotation == PDGB_ROTATION_SVD) {
        if (jacobi_form) k_local<true, PDGB_ROTATION_SVD><<<ntiles, kLocalThreads, sm, s>>>(a);
        else launch_pdl(k_local<false, PDGB_ROTATION_SVD>, ntiles, kLocalThreads, sm, s, a);
    } else {
        if (jacobi_form) k_local<true, PDGB_ROTATION_QUAT><<<ntiles, kLocalThreads, sm, s>>>(a);
        else launch_pdl(k_local<false, PDGB_ROTATION_QUAT>, ntiles, kLocalThreads, sm, s, a);
    }
}

// ------------------------------------------------------- vertex kernels
// (relax09: the 0.9 under-relaxation of pdUtil.cu:221, relax.cuh)

template <int kMode>
__device__ __forceinline__ void jacobi_vertex(const VertexArgs& a, int i, float omega) {
    const float4 s = a.sn[i];
    const float4 cf = __ldg(&a.coef[i]);
    const float cm = cf.x, md = cf.y;
    const float4 bb = (cf.z != 0.f) ? __ldg(&a.pin_rhs[i]) : a.b[i];
    const float den = cm + md;
    float4 nx;
    if (drag_weight(a.sc, i) > 0.f) {
        nx = s;  // dragged vertices keep the current iterate (getErrorKern, pdUtil.cu:200-205)
    } else {
        nx.x = (bb.x - cm * s.x) / den + s.x;
        nx.y = (bb.y - cm * s.y) / den + s.y;
        nx.z = (bb.z - cm * s.z) / den + s.z;
    }
    nx.x = relax09(nx.x, s.x);
    nx.y = relax09(nx.y, s.y);
    nx.z = relax09(nx.z, s.z);
    nx.w = 0.f;
    if (kMode & kReadPrev) {
        const float4 p = a.prev[i];
        nx.x = (nx.x - p.x) * omega + p.x;
        nx.y = (nx.y - p.y) * omega + p.y;
        nx.z = (nx.z - p.z) * omega + p.z;
    }
    if (kMode & kWritePrev) a.prev[i] = s;
    if (kMode & kFinal) {
        finish_vertex(a.sc, i, nx, a.dt_inv, a.x, a.v);
    } else {
        a.sn[i] = nx;
        a.b[i] = __ldg(&a.base[i]);
    }
}

template <int kMode>
__global__ void __launch_bounds__(256) k_jacobi_vertex(VertexArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.nv) jacobi_vertex<kMode>(a, i, a.omega);
}

// Multi-request form: CTA i updates 256 vertices of request list[i].x
// starting at list[i].y.
template <int kMode>
__global__ void __launch_bounds__(256) k_jacobi_vertex_multi(const VertexArgs* __restrict__ req,
                                                             const int2* __restrict__ list,
                                                             const int* __restrict__ count, float omega) {
    if ((int)blockIdx.x >= *count) return;
    const int2 w = list[blockIdx.x];
    const VertexArgs& a = req[w.x];
    const int i = w.y + threadIdx.x;
    if (i < a.nv) jacobi_vertex<kMode>(a, i, omega);
}

void launch_jacobi_vertex_multi(const VertexArgs* req, const int2* list, const int* count, int grid, int mode,
                                float omega, cudaStream_t s) {
    if (grid <= 0) return;
    switch (mode & 7) {
        case 0: k_jacobi_vertex_multi<0><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 1: k_jacobi_vertex_multi<1><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 2: k_jacobi_vertex_multi<2><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 3: k_jacobi_vertex_multi<3><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 4: k_jacobi_vertex_multi<4><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 5: k_jacobi_vertex_multi<5><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        case 6: k_jacobi_vertex_multi<6><<<grid, 256, 0, s>>>(req, list, count, omega); break;
        default: k_jacobi_vertex_multi<7><<<grid, 256, 0, s>>>(req, list, count, omega); break;
    }
}

void launch_jacobi_vertex(const VertexArgs& a, int mode, cudaStream_t s) {
    const int blocks = (a.nv + 255) / 256;
    if (blocks == 0) return;
    switch (mode & 7) {
        case 0: k_jacobi_vertex<0><<<blocks, 256, 0, s>>>(a); break;
        case 1: k_jacobi_vertex<1><<<blocks, 256, 0, s>>>(a); break;
        case 2: k_jacobi_vertex<2><<<blocks, 256, 0, s>>>(a); break;
        case 3: k_jacobi_vertex<3><<<blocks, 256, 0, s>>>(a); break;
        case 4: k_jacobi_vertex<4><<<blocks, 256, 0, s>>>(a); break;
        case 5: k_jacobi_vertex<5><<<blocks, 256, 0, s>>>(a); break;
        case 6: k_jacobi_vertex<6><<<blocks, 256, 0, s>>>(a); break;
        default: k_jacobi_vertex<7><<<blocks, 256, 0, s>>>(a); break;
    }
}

// Step prologue: f = (0, -g m, 0); s = x + h v + f / (M/h^2); base = (M/h^2) s;
// b = base (pinned vertices: the pin RHS).  A dragged vertex (weight w > 0)
// starts at its drag target, its M/h^2 becomes (m + w)/h^2
// (setMDt_2MoreDBC, pdUtil.cu:56-69), and when the system has pinned
// vertices its RHS row is target * w (computeDBCLocal, pdUtil.cu:159-164).
__device__ __forceinline__ void begin_vertex(const BeginArgs& a, int i) {
    const float4 x = a.x[i], v = a.v[i], cf = __ldg(&a.coef[i]);
    const float w = drag_weight(a.sc, i);
    float4 s;
    float mdt2 = cf.x;
    if (w > 0.f) {
        s = drag_target(a.sc, i);
        if (cf.z == 0.f) mdt2 = (cf.w + w) / a.sc.dt2;
    } else {
        const float dt2_m_1 = 1.0f / cf.x;
        const float fy = -a.gravity * cf.w;
        s.x = x.x + a.dt * v.x + dt2_m_1 * 0.0f;
        s.y = x.y + a.dt * v.y + dt2_m_1 * fy;
        s.z = x.z + a.dt * v.z + dt2_m_1 * 0.0f;
        s.w = 0.f;
    }
    a.sn[i] = s;
    float4 bs = make_float4(mdt2 * s.x, mdt2 * s.y, mdt2 * s.z, 0.f);
    if (w > 0.f && a.sc.drag_rhs && cf.z == 0.f) bs = make_float4(s.x * w, s.y * w, s.z * w, 0.f);
    a.base[i] = bs;
    a.b[i] = cf.z != 0.f ? __ldg(&a.pin_rhs[i]) : bs;
    if (a.prev) {
        // bytes [0, 3 nv) of the caller-order float[3 nv] vector are zeroed
        const long long zero_bytes = 3LL * a.nv;
        const long long o = a.vperm[i];
        float4 p = a.prev[i];
        float* pc = &p.x;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const long long b0 = 4 * (3 * o + d);
            if (b0 + 4 <= zero_bytes) pc[d] = 0.f;
            else if (b0 < zero_bytes) {
                const int nz = (int)(zero_bytes - b0);  // low-order bytes cleared (little endian)
                const unsigned mask = ~((1u << (8 * nz)) - 1u);
                pc[d] = __uint_as_float(__float_as_uint(pc[d]) & mask);
            }
        }
        a.prev[i] = p;
    }
}

__global__ void __launch_bounds__(256) k_begin(BeginArgs a) {
    pdl_trigger();  // the step's first local step may be scheduled meanwhile (Cholesky path)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        if (a.done) *a.done = 0;
        if (a.iterations) *a.iterations = a.num_iterations;
    }
    if (i < a.nv) begin_vertex(a, i);
}

__global__ void __launch_bounds__(256) k_begin_multi(const BeginArgs* __restrict__ req, const int2* __restrict__ list,
                                                     const int* __restrict__ count) {
    if ((int)blockIdx.x >= *count) return;
    const int2 w = list[blockIdx.x];
    const BeginArgs& a = req[w.x];
    const int i = w.y + threadIdx.x;
    if (i < a.nv) begin_vertex(a, i);
}

void launch_begin_multi(const BeginArgs* req, const int2* list, const int* count, int grid, cudaStream_t s) {
    if (grid > 0) k_begin_multi<<<grid, 256, 0, s>>>(req, list, count);
}

void launch_begin(const BeginArgs& a, cudaStream_t s) {
    const int blocks = (a.nv + 255) / 256;
    if (blocks) k_begin<<<blocks, 256, 0, s>>>(a);
}

// ------------------------------------------------------- rotation check
// The local step's rotation on n row-major 3x3 matrices (checking and
// benchmarking the rotation on its own).
__global__ void k_rotations(int n, const float* __restrict__ F, float* R, int rotation) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[9], r[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = F[9 * (size_t)i + k];
    if (rotation == PDGB_ROTATION_SVD) closest_rotation(f, r);
    else closest_rotation_horn(f, r);
#pragma unroll
    for (int k = 0; k < 9; ++k) R[9 * (size_t)i + k] = r[k];
}

void launch_rotations(int n, const float* F, float* R, int rotation, cudaStream_t s) {
    if (n > 0) k_rotations<<<(n + 255) / 256, 256, 0, s>>>(n, F, R, rotation);
}

// ------------------------------------------------------- state transfer
__global__ void k_gather_state(int nv, const int* __restrict__ vperm, const float* __restrict__ X,
                               const float* __restrict__ V, float4* x, float4* v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int o = vperm[i];
    x[i] = make_float4(X[3 * o], X[3 * o + 1], X[3 * o + 2], 0.f);
    if (V) v[i] = make_float4(V[3 * o], V[3 * o + 1], V[3 * o + 2], 0.f);
    else v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_scatter_state(int nv, const int* __restrict__ vperm, const float4* __restrict__ x,
                                const float4* __restrict__ v, float* X, float* V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int o = vperm[i];
    if (X) {
        const float4 p = x[i];
        X[3 * o] = p.x; X[3 * o + 1] = p.y; X[3 * o + 2] = p.z;
    }
    if (V) {
        const float4 q = v[i];
        V[3 * o] = q.x; V[3 * o + 1] = q.y; V[3 * o + 2] = q.z;
    }
}

__global__ void k_copy_x0(int nv, const float4* __restrict__ x0, float4* x, float4* v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    x[i] = x0[i];
    v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

void launch_gather_state(int nv, const int* vperm, const float* X, const float* V, float4* x, float4* v,
                         cudaStream_t s) {
    if (nv > 0) k_gather_state<<<(nv + 255) / 256, 256, 0, s>>>(nv, vperm, X, V, x, v);
}
void launch_scatter_state(int nv, const int* vperm, const float4* x, const float4* v, float* X, float* V,
                          cudaStream_t s) {
    if (nv > 0) k_scatter_state<<<(nv + 255) / 256, 256, 0, s>>>(nv, vperm, x, v, X, V);
}
void launch_copy_x0(int nv, const float4* x0, float4* x, float4* v, cudaStream_t s) {
    if (nv > 0) k_copy_x0<<<(nv + 255) / 256, 256, 0, s>>>(nv, x0, x, v);
}

}  // namespace pdgb
