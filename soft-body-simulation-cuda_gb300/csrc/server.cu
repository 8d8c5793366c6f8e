// Serving loop: continuous batching of PD simulation requests on one GPU.
//
// Requests (a soft body and a number of steps) are submitted at any time.
// Host worker threads build each request's layout (the same Morton tiles and
// coefficients as a single engine) and, on the Cholesky path, the ordering
// and symbolic analysis of its system.  pdgb_server_tick then
//   1. admits ready requests in arrival order while their device bytes fit
//      the HBM budget (and the slot limit).  Each gets one block from a
//      stream-ordered pool (cudaMallocAsync, no device-wide synchronisation)
//      for its tile layout and state; on the Cholesky path its factor is
//      computed on the GPU in FP64 (factor.cu) straight into the server's
//      factor arena and stays resident until the request finishes;
//   2. runs ONE PD step for every active request with one set of launches:
//      prologue, num_iterations x (local step, global solve), epilogue, each
//      covering the work lists of all active requests (tiles, 256-vertex
//      chunks and, for the Cholesky solve, level L of every request's
//      elimination tree in the same per-level launches, as a batch engine
//      does for its bodies), captured as a CUDA graph and replayed every tick
//      while the set of requests stays the same;
//   3. retires the requests that reached their step count: state copied to
//      host memory, memory returned to the pool and arenas.
// Requests join and leave between steps, their work shares every launch,
// and a request's arithmetic is the single engine's (same kernels, own
// arrays), so its result does not depend on the mix.
//
// Memory.  Jacobi requests keep everything in their block.  Cholesky
// requests keep the vectors the solve reaches through its row lists (the
// iterate, the right-hand side and the forward result) in arenas shared by
// all requests, so that one set of solve launches addresses every request:
// a request owns a vertex range of the vector arena (row ids are shifted by
// its start), a range of the factor arena (its M_s blocks), of the row-list
// arena and of the backward staging arena.  Arenas grow by doubling; a
// growth copies them (offsets are kept) and rebuilds the work lists.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <thread>
#include <unordered_map>

#include "cholesky.h"
#include "engine.h"
#include "solve.h"

using namespace pdgb;

namespace {

using Clock = std::chrono::steady_clock;

enum : int { kQueued = 0, kPreparing = 1, kReady = 2, kRunning = 3, kDone = 4, kFailed = 5 };

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// What the workers prepare for a mesh, shared by the requests that submit
// the same mesh (cache by content).
struct MeshEntry {
    std::shared_ptr<const HostLayout> L;
    std::shared_ptr<CholFactor> f;  // symbolic factor + front plan (Cholesky servers)
    // numeric factor: host copy of the M_s blocks once the GPU has computed
    // them (written and read by the tick thread only)
    std::vector<float> mval;
    bool numeric = false;
};

// Best-fit allocator of element ranges [offset, offset + n) in an arena.
struct RangeAlloc {
    int64_t top = 0;
    std::set<std::pair<int64_t, int64_t>> by_size;  // (size, offset)
    std::map<int64_t, int64_t> by_off;              // offset -> size
    int64_t take(int64_t n) {
        auto it = by_size.lower_bound({n, INT64_MIN});
        if (it == by_size.end()) {
            const int64_t o = top;
            top += n;
            return o;
        }
        const int64_t size = it->first, o = it->second;
        by_size.erase(it);
        by_off.erase(o);
        if (size > n) {
            by_size.emplace(size - n, o + n);
            by_off.emplace(o + n, size - n);
        }
        return o;
    }
    void give(int64_t o, int64_t n) {
        auto next = by_off.lower_bound(o);
        if (next != by_off.end() && next->first == o + n) {
            by_size.erase({next->second, next->first});
            n += next->second;
            next = by_off.erase(next);
        }
        if (next != by_off.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == o) {
                by_size.erase({prev->second, prev->first});
                o = prev->first;
                n += prev->second;
                by_off.erase(prev);
            }
        }
        if (o + n == top) {
            top = o;
            return;
        }
        by_off.emplace(o, n);
        by_size.emplace(n, o);
    }
};

// A growable device array whose element ranges are handed out by a RangeAlloc.
template <class T> struct Arena {
    T* p = nullptr;
    int64_t cap = 0;
    RangeAlloc ra;
    ~Arena() {
        if (p) cudaFree(p);
    }
    // Takes n elements; grows (copying the contents) when the range does
    // not fit.  Returns true when the array moved.
    bool take(int64_t n, int64_t& off, cudaStream_t s) {
        off = ra.take(std::max<int64_t>(n, 1));
        if (ra.top <= cap) return false;
        const int64_t ncap = std::max<int64_t>(ra.top, 2 * cap + 4096);
        T* q = nullptr;
        PDGB_CUDA_TRY(cudaStreamSynchronize(s));
        PDGB_CUDA_TRY(cudaMalloc(&q, (size_t)ncap * sizeof(T)));
        if (p) {
            PDGB_CUDA_TRY(cudaMemcpyAsync(q, p, (size_t)cap * sizeof(T), cudaMemcpyDeviceToDevice, s));
            PDGB_CUDA_TRY(cudaStreamSynchronize(s));
            cudaFree(p);
        }
        p = q;
        cap = ncap;
        return true;
    }
    void give(int64_t off, int64_t n) { ra.give(off, std::max<int64_t>(n, 1)); }
};

struct Request {
    long long id = 0;
    int state = kQueued;
    int nsteps = 0, steps_done = 0;
    int nv = 0, nt = 0;
    std::vector<float> X, V, mass, mu, dbc;
    std::vector<uint32_t> tets;
    std::shared_ptr<MeshEntry> me;        // layout (and symbolic factor) of its mesh
    const HostLayout* L = nullptr;
    std::string error;
    // device block and carved arrays
    unsigned char* block = nullptr;
    size_t bytes = 0;
    LocalArgs la{};
    VertexArgs va{};
    BeginArgs ba{};
    CholVertexArgs cv{};
    float* staging = nullptr;
    int* vperm = nullptr;
    int* flag = nullptr;                  // non-finite state (device)
    int flag_host = 0;
    // arena ranges of a Cholesky request
    int64_t v0 = 0, m0 = 0, r0 = 0, z0 = 0;
    float4 *x = nullptr, *v = nullptr, *prev = nullptr, *base = nullptr;
    const float4 *coef = nullptr, *pin = nullptr;
    std::vector<float> X_out, V_out;
    Clock::time_point t_submit, t_admit, t_done;
};

template <class T> size_t bytes_of(const std::vector<T>& v) { return align256(v.size() * sizeof(T)); }

// Device bytes of a prepared request: its block (layout arrays, the state
// vectors it owns, staging for the state transfers, the status word) and,
// on the Cholesky path, its arena ranges (3 vectors, rows, M_s, staging).
size_t request_bytes(const Request& r, bool chol) {
    const HostLayout& L = *r.L;
    size_t b = bytes_of(L.inc_ent) + bytes_of(L.inc_end) + bytes_of(L.geo) + bytes_of(L.tile_tet_ptr) +
               bytes_of(L.tile_vptr) + bytes_of(L.tile_verts) + bytes_of(L.vperm) + bytes_of(L.coef) +
               bytes_of(L.pin_rhs);
    b += (chol ? 4 : 6) * align256((size_t)r.nv * sizeof(float4));  // x, v, prev, base (+ sn, b)
    b += align256(6 * (size_t)r.nv * sizeof(float));                // staging
    b += 256;                                                         // status word
    if (chol) {
        const CholFactor& f = *r.me->f;
        b += 3 * (size_t)r.nv * sizeof(float4) + f.rows.size() * sizeof(int) + (size_t)f.mval_size * sizeof(float) +
             (size_t)f.zrows * sizeof(float4);
    }
    return b;
}

}  // namespace

struct pdgb_server {
    pdgb_server_config cfg{};
    bool chol = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaMemPool_t pool = nullptr;  // the server's own stream-ordered pool
    std::mutex mu;
    std::condition_variable cv;
    std::vector<std::thread> workers;
    bool stop = false;
    long long next_id = 1;
    std::unordered_map<long long, std::unique_ptr<Request>> reqs;
    std::deque<long long> prep_queue, ready_queue;
    std::vector<Request*> active;
    size_t bytes_in_use = 0;
    bool lists_dirty = true;
    bool graph_dirty = true;
    // work lists (device + pinned host mirrors)
    int cap_req = 0, cap_tiles = 0, cap_chunks = 0;
    LocalArgs* d_la = nullptr;
    VertexArgs* d_va = nullptr;
    BeginArgs* d_ba = nullptr;
    CholVertexArgs* d_cv = nullptr;
    int2 *d_tiles = nullptr, *d_chunks = nullptr;
    int* d_counts = nullptr;  // {tiles, chunks}
    LocalArgs* h_la = nullptr;
    VertexArgs* h_va = nullptr;
    BeginArgs* h_ba = nullptr;
    CholVertexArgs* h_cv = nullptr;
    int2 *h_tiles = nullptr, *h_chunks = nullptr;
    int* h_counts = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    // Cholesky path: arenas and the combined per-level solve lists
    Arena<float4> va_sn, va_b, va_y;  // one vertex range per request, same offset in all three
    Arena<float> ar_mval;
    Arena<int> ar_rows;
    Arena<float4> ar_zbuf;
    DBuf<int> d_fwdb, d_bwdb, d_fwds, d_bwds, d_tiny, d_zst;
    std::vector<SolveLevel> step_levels;
    // stats
    long long completed = 0, failed = 0, nonfinite = 0;
    double tet_iterations = 0.0;
    std::vector<double> latencies_ms;
    double busy_ms = 0.0, admit_ms = 0.0, step_ms = 0.0, factor_ms = 0.0;
    long long ticks = 0, factors = 0, factor_hits = 0;
    // mesh cache: requests for a mesh seen before reuse its host layout (and
    // its factor, symbolic and numeric)
    std::mutex cache_mu;
    std::unordered_map<uint64_t, std::pair<uint64_t, std::shared_ptr<MeshEntry>>> cache;
    std::deque<uint64_t> cache_order;  // insertion order, for eviction
    size_t cache_cap = 256;
    long long cache_hits = 0;

    ~pdgb_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        for (auto& t : workers) t.join();
        if (stream) cudaStreamSynchronize(stream);
        for (auto& kv : reqs)
            if (kv.second->block) cudaFreeAsync(kv.second->block, stream);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        cudaFree(d_la);
        cudaFree(d_va);
        cudaFree(d_ba);
        cudaFree(d_cv);
        cudaFree(d_tiles);
        cudaFree(d_chunks);
        cudaFree(d_counts);
        cudaFreeHost(h_la);
        cudaFreeHost(h_va);
        cudaFreeHost(h_ba);
        cudaFreeHost(h_cv);
        cudaFreeHost(h_tiles);
        cudaFreeHost(h_chunks);
        cudaFreeHost(h_counts);
        if (stream) cudaStreamSynchronize(stream);
        if (pool) cudaMemPoolDestroy(pool);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace {

template <class F> int guarded_s(F&& f) {
    try {
        f();
        return PDGB_OK;
    } catch (const Error& e) {
        set_last_error(e.status, e.msg);
        return e.status;
    } catch (const std::bad_alloc&) {
        set_last_error(PDGB_ERR_OUT_OF_MEMORY, "host allocation failed");
        return PDGB_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, e.what());
        return PDGB_ERR_INVALID_ARGUMENT;
    }
}

// Two independent 64-bit hashes of a request's mesh (the layout and the
// factor depend on nothing else for a given server).
struct MeshKey {
    uint64_t a, b;
};

MeshKey mesh_key(const Request& r) {
    uint64_t a = 0x9e3779b97f4a7c15ull ^ ((uint64_t)r.nv << 32 | (uint32_t)r.nt);
    uint64_t b = 0xc2b2ae3d27d4eb4full + (uint64_t)r.nv * 31 + (uint64_t)r.nt;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, c + i, 8);
            a = (a ^ w) * 0x100000001b3ull;
            a ^= a >> 29;
            b = (b + w) * 0x9fb21c651e98df25ull;
            b ^= b >> 31;
        }
        for (; i < n; ++i) {
            a = (a ^ c[i]) * 0x100000001b3ull;
            b = (b + c[i]) * 0x9fb21c651e98df25ull;
        }
        a ^= n;
        b += n;
    };
    mix(r.X.data(), r.X.size() * sizeof(float));
    mix(r.tets.data(), r.tets.size() * sizeof(uint32_t));
    mix(r.mass.data(), r.mass.size() * sizeof(float));
    mix(r.mu.data(), r.mu.size() * sizeof(float));
    mix(r.dbc.data(), r.dbc.size() * sizeof(float));
    return {a, b};
}

void worker_loop(pdgb_server* S) {
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait(lk, [&] { return S->stop || !S->prep_queue.empty(); });
            if (S->stop) return;
            const long long id = S->prep_queue.front();
            S->prep_queue.pop_front();
            auto it = S->reqs.find(id);
            if (it == S->reqs.end()) continue;
            r = it->second.get();
            r->state = kPreparing;
        }
        bool ok = true;
        try {
            const MeshKey key = mesh_key(*r);
            if (S->cache_cap > 0) {
                std::lock_guard<std::mutex> ck(S->cache_mu);
                auto it = S->cache.find(key.a);
                if (it != S->cache.end() && it->second.first == key.b) {
                    r->me = it->second.second;
                    S->cache_hits++;
                }
            }
            if (!r->me) {
                auto me = std::make_shared<MeshEntry>();
                auto L = std::make_shared<HostLayout>();
                build_layout(r->nv, r->nt, r->X.data(), r->tets.data(), r->mass.data(), r->mu.data(),
                             r->dbc.empty() ? nullptr : r->dbc.data(), S->cfg.params, *L);
                if (S->chol) {
                    // ordering and symbolic analysis here; the numeric
                    // factorisation runs on the GPU at admission.  Whole
                    // columns per backward item, as the bodies of a batch.
                    auto f = std::make_shared<CholFactor>();
                    const std::vector<float> xyz = layout_xyz(*L);
                    cholesky_factor(layout_system(*L), PDGB_ORDER_AMD, xyz.data(), *f, 0, true);
                    f->K = SparseSym();  // no refinement residuals in the server
                    me->f = f;
                }
                me->L = L;
                r->me = me;
                if (S->cache_cap > 0) {
                    std::lock_guard<std::mutex> ck(S->cache_mu);
                    if (S->cache.emplace(key.a, std::make_pair(key.b, r->me)).second) {
                        S->cache_order.push_back(key.a);
                        if (S->cache_order.size() > S->cache_cap) {
                            S->cache.erase(S->cache_order.front());
                            S->cache_order.pop_front();
                        }
                    }
                }
            }
            r->L = r->me->L.get();
            r->bytes = request_bytes(*r, S->chol);
        } catch (const Error& e) {
            ok = false;
            r->error = e.msg;
        } catch (const std::exception& e) {
            ok = false;
            r->error = e.what();
        }
        std::lock_guard<std::mutex> lk(S->mu);
        if (ok) {
            r->state = kReady;
            S->ready_queue.push_back(r->id);
        } else {
            r->state = kFailed;
            S->failed++;
        }
    }
}

template <class T> T* carve(unsigned char*& p, size_t n) {
    T* q = reinterpret_cast<T*>(p);
    p += align256(n * sizeof(T));
    return q;
}

template <class T> void put(cudaStream_t s, T* dst, const std::vector<T>& src) {
    if (!src.empty()) PDGB_CUDA_TRY(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

SceneArgs request_scene(const pdgb_server* S, Request* r) {
    SceneArgs sc{};
    sc.dt2 = S->cfg.params.dt * S->cfg.params.dt;
    sc.nonfinite = r->flag;
    return sc;
}

// Kernel arguments of a request from its block and (Cholesky) its arena
// ranges at the arenas' current addresses.
void set_args(pdgb_server* S, Request* r) {
    const int nv = r->nv;
    float4* sn = S->chol ? S->va_sn.p + r->v0 : r->la.sn ? const_cast<float4*>(r->la.sn) : nullptr;
    float4* b = S->chol ? S->va_b.p + r->v0 : r->la.b;
    const HostLayout& L = *r->L;
    r->la.sn = sn;
    r->la.b = b;
    r->la.nt_pad = L.nt_pad;
    r->la.done = nullptr;
    const SceneArgs sc = request_scene(S, r);
    r->va = VertexArgs{nv, sn, r->prev, b, r->base, r->coef, r->pin, r->x, r->v, 1.f, 1.0f / S->cfg.params.dt, sc};
    BeginArgs ba{};
    ba.nv = nv;
    ba.x = r->x;
    ba.v = r->v;
    ba.coef = r->coef;
    ba.pin_rhs = r->pin;
    ba.sn = sn;
    ba.base = r->base;
    ba.b = b;
    ba.dt = S->cfg.params.dt;
    ba.gravity = S->cfg.params.gravity;
    ba.vperm = r->vperm;
    ba.num_iterations = S->cfg.params.num_iterations;
    ba.sc = sc;
    r->ba = ba;
    if (S->chol) {
        CholVertexArgs cv{};
        cv.nv = nv;
        cv.sn = sn;
        cv.y = S->va_y.p + r->v0;
        cv.b = b;
        cv.base = r->base;
        cv.coef = r->coef;
        cv.pin_rhs = r->pin;
        cv.x = r->x;
        cv.v = r->v;
        cv.prev = r->prev;
        cv.dt_inv = 1.0f / S->cfg.params.dt;
        cv.sc = sc;
        r->cv = cv;
    }
}

// Uploads a prepared request into its device block (and arenas).
void admit(pdgb_server* S, Request* r) {
    cudaStream_t s = S->stream;
    const HostLayout& L = *r->L;
    const int nv = r->nv;
    const bool chol = S->chol;
    size_t block_bytes = r->bytes;
    if (chol) {  // the arena part of r->bytes is not in the block
        const CholFactor& f = *r->me->f;
        block_bytes -= 3 * (size_t)nv * sizeof(float4) + f.rows.size() * sizeof(int) +
                       (size_t)f.mval_size * sizeof(float) + (size_t)f.zrows * sizeof(float4);
    }
    PDGB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r->block), block_bytes, S->pool, s));
    unsigned char* p = r->block;
    uint16_t* inc_ent = carve<uint16_t>(p, L.inc_ent.size());
    uint16_t* inc_end = carve<uint16_t>(p, L.inc_end.size());
    float* geo = carve<float>(p, L.geo.size());
    int* ttp = carve<int>(p, L.tile_tet_ptr.size());
    int* tvp = carve<int>(p, L.tile_vptr.size());
    uint32_t* tv = carve<uint32_t>(p, L.tile_verts.size());
    r->vperm = carve<int>(p, L.vperm.size());
    float4* coef = carve<float4>(p, L.coef.size());
    float4* pin = carve<float4>(p, L.pin_rhs.size());
    r->coef = coef;
    r->pin = pin;
    r->x = carve<float4>(p, nv);
    r->v = carve<float4>(p, nv);
    r->prev = carve<float4>(p, nv);
    r->base = carve<float4>(p, nv);
    float4* sn = nullptr;
    float4* b = nullptr;
    if (!chol) {
        sn = carve<float4>(p, nv);
        b = carve<float4>(p, nv);
    }
    r->staging = carve<float>(p, 6 * (size_t)nv);
    r->flag = carve<int>(p, 1);
    put(s, inc_ent, L.inc_ent);
    put(s, inc_end, L.inc_end);
    put(s, geo, L.geo);
    put(s, ttp, L.tile_tet_ptr);
    put(s, tvp, L.tile_vptr);
    put(s, tv, L.tile_verts);
    put(s, r->vperm, L.vperm);
    put(s, coef, L.coef);
    put(s, pin, L.pin_rhs);
    PDGB_CUDA_TRY(cudaMemsetAsync(r->flag, 0, sizeof(int), s));
    PDGB_CUDA_TRY(cudaMemsetAsync(r->prev, 0, (size_t)nv * sizeof(float4), s));
    PDGB_CUDA_TRY(cudaMemcpyAsync(r->staging, r->X.data(), 3 * (size_t)nv * sizeof(float), cudaMemcpyHostToDevice, s));
    const bool hasV = !r->V.empty();
    if (hasV)
        PDGB_CUDA_TRY(cudaMemcpyAsync(r->staging + 3 * (size_t)nv, r->V.data(), 3 * (size_t)nv * sizeof(float),
                                      cudaMemcpyHostToDevice, s));
    launch_gather_state(nv, r->vperm, r->staging, hasV ? r->staging + 3 * (size_t)nv : nullptr, r->x, r->v, s);
    PDGB_CUDA_TRY(cudaGetLastError());
    r->la = LocalArgs{sn, b, inc_ent, inc_end, geo, ttp, tvp, tv, L.nt_pad, nullptr};
    if (chol) {
        MeshEntry& me = *r->me;
        const CholFactor& f = *me.f;
        int64_t v0, m0, r0, z0, tmp;
        bool moved = S->va_sn.take(nv, v0, s);
        moved |= S->va_b.take(nv, tmp, s);
        moved |= S->va_y.take(nv, tmp, s);
        moved |= S->ar_mval.take(f.mval_size, m0, s);
        moved |= S->ar_rows.take((int64_t)f.rows.size(), r0, s);
        moved |= S->ar_zbuf.take(f.zrows, z0, s);
        if (moved) S->graph_dirty = true;  // every request's arena pointers change
        r->v0 = v0;
        r->m0 = m0;
        r->r0 = r0;
        r->z0 = z0;
        // row lists as arena vertex ids
        std::vector<int> rows(f.rows.size());
        for (size_t i = 0; i < rows.size(); ++i) rows[i] = f.rows[i] + (int)v0;
        if (!rows.empty())
            PDGB_CUDA_TRY(cudaMemcpyAsync(S->ar_rows.p + r0, rows.data(), rows.size() * sizeof(int),
                                          cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemsetAsync(S->va_y.p + v0, 0, (size_t)nv * sizeof(float4), s));
        // the numeric factor: computed on the GPU the first time the mesh is
        // seen, uploaded from the host copy after that
        if (me.numeric) {
            if (!me.mval.empty())
                PDGB_CUDA_TRY(cudaMemcpyAsync(S->ar_mval.p + m0, me.mval.data(), me.mval.size() * sizeof(float),
                                              cudaMemcpyHostToDevice, s));
            S->factor_hits++;
        } else {
            S->factor_ms += gpu_factor(f, S->ar_mval.p + m0, s);
            S->factors++;
            if (S->cache_cap > 0) {
                me.mval.resize((size_t)f.mval_size);
                if (!me.mval.empty())
                    PDGB_CUDA_TRY(cudaMemcpy(me.mval.data(), S->ar_mval.p + m0, me.mval.size() * sizeof(float),
                                             cudaMemcpyDeviceToHost));
                me.numeric = true;
                me.f->fp = FrontPlan();  // the front plan is not needed again
            }
        }
    }
    set_args(S, r);
    r->state = kRunning;
    r->t_admit = Clock::now();
    S->bytes_in_use += r->bytes;
}

// Releases a finished request's arena ranges.
void release_arenas(pdgb_server* S, Request* r) {
    if (!S->chol) return;
    const CholFactor& f = *r->me->f;
    S->va_sn.give(r->v0, r->nv);
    S->va_b.give(r->v0, r->nv);
    S->va_y.give(r->v0, r->nv);
    S->ar_mval.give(r->m0, f.mval_size);
    S->ar_rows.give(r->r0, (int64_t)f.rows.size());
    S->ar_zbuf.give(r->z0, f.zrows);
}

void ensure_capacity(pdgb_server* S, int nreq, int ntiles, int nchunks) {
    auto grow = [](int need, int cap) { return need <= cap ? cap : std::max(need, 2 * cap + 64); };
    const int creq = grow(nreq, S->cap_req), ctile = grow(ntiles, S->cap_tiles), cchunk = grow(nchunks, S->cap_chunks);
    if (creq == S->cap_req && ctile == S->cap_tiles && cchunk == S->cap_chunks && S->d_counts) return;
    PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));
    cudaFree(S->d_la);
    cudaFree(S->d_va);
    cudaFree(S->d_ba);
    cudaFree(S->d_cv);
    cudaFree(S->d_tiles);
    cudaFree(S->d_chunks);
    cudaFreeHost(S->h_la);
    cudaFreeHost(S->h_va);
    cudaFreeHost(S->h_ba);
    cudaFreeHost(S->h_cv);
    cudaFreeHost(S->h_tiles);
    cudaFreeHost(S->h_chunks);
    PDGB_CUDA_TRY(cudaMalloc(&S->d_la, creq * sizeof(LocalArgs)));
    PDGB_CUDA_TRY(cudaMalloc(&S->d_va, creq * sizeof(VertexArgs)));
    PDGB_CUDA_TRY(cudaMalloc(&S->d_ba, creq * sizeof(BeginArgs)));
    PDGB_CUDA_TRY(cudaMalloc(&S->d_cv, creq * sizeof(CholVertexArgs)));
    PDGB_CUDA_TRY(cudaMalloc(&S->d_tiles, ctile * sizeof(int2)));
    PDGB_CUDA_TRY(cudaMalloc(&S->d_chunks, cchunk * sizeof(int2)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_la, creq * sizeof(LocalArgs)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_va, creq * sizeof(VertexArgs)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_ba, creq * sizeof(BeginArgs)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_cv, creq * sizeof(CholVertexArgs)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_tiles, ctile * sizeof(int2)));
    PDGB_CUDA_TRY(cudaMallocHost(&S->h_chunks, cchunk * sizeof(int2)));
    if (!S->d_counts) {
        PDGB_CUDA_TRY(cudaMalloc(&S->d_counts, 2 * sizeof(int)));
        PDGB_CUDA_TRY(cudaMallocHost(&S->h_counts, 2 * sizeof(int)));
    }
    S->cap_req = creq;
    S->cap_tiles = ctile;
    S->cap_chunks = cchunk;
    S->graph_dirty = true;  // the step graph bakes the list pointers and grid sizes
}

// The step graph.  Jacobi: grids sized by the list capacities (CTAs past the
// current counts exit), so it survives changes of the active set.  Cholesky:
// the per-level solve launches follow the active requests' trees, so it is
// captured again whenever the set changes.
void capture_step(pdgb_server* S) {
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    if (S->graph) cudaGraphDestroy(S->graph);
    S->gexec = nullptr;
    S->graph = nullptr;
    cudaStream_t s = S->stream;
    const int n = S->cfg.params.num_iterations;
    PDGB_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        launch_begin_multi(S->d_ba, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
        if (!S->chol) {
            const std::vector<float> omega = chebyshev_omegas(n, S->cfg.params.rho);
            for (int i = 0; i < n; ++i) {
                launch_local_multi(S->d_la, S->d_tiles, S->d_counts, S->cap_tiles, s, true);
                int mode = 0;
                if (i >= 11) mode |= kReadPrev;
                if (i >= 10 && i + 1 < n) mode |= kWritePrev;
                if (i + 1 == n) mode |= kFinal;
                launch_jacobi_vertex_multi(S->d_va, S->d_chunks, S->d_counts + 1, S->cap_chunks, mode, omega[i], s);
            }
        } else {
            CholArgs ca{};
            ca.rows = S->ar_rows.p;
            ca.mval = S->ar_mval.p;
            ca.r = S->va_b.p;
            ca.y = S->va_y.p;
            ca.x = S->va_sn.p;
            ca.done = nullptr;
            ca.fwd_blocks = S->d_fwdb.p;
            ca.bwd_blocks = S->d_bwdb.p;
            ca.fwd_small = S->d_fwds.p;
            ca.bwd_small = S->d_bwds.p;
            ca.tiny = S->d_tiny.p;
            ca.zstage = S->d_zst.p;
            ca.zbuf = S->ar_zbuf.p;
            for (int i = 0; i < n; ++i) {
                launch_local_multi(S->d_la, S->d_tiles, S->d_counts, S->cap_tiles, s, false);
                launch_chol_solve_levels(ca, S->step_levels, s);
                launch_chol_vertex_multi(S->d_cv, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
            }
            launch_chol_finish_multi(S->d_cv, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
        }
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cudaError_t err = cudaStreamEndCapture(s, &S->graph);
    if (err != cudaSuccess) throw Error{PDGB_ERR_CUDA, std::string("server graph capture: ") + cudaGetErrorString(err)};
    PDGB_CUDA_TRY(cudaGraphInstantiate(&S->gexec, S->graph, 0));
    S->graph_dirty = false;
}

// Per-level solve items of all active Cholesky requests: level L of every
// request's tree in the same lists (levels counted from the leaves), with
// each request's offsets into the arenas (factor, rows, staging) added.
void build_solve_lists(pdgb_server* S) {
    std::vector<int> fwdb, bwdb, fwds, bwds, tiny, zst;
    int nl = 0;
    for (Request* r : S->active) nl = std::max(nl, (int)r->me->f->step_levels.size());
    S->step_levels.assign(nl, SolveLevel{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0});
    auto append = [](std::vector<int>& dst, const std::vector<int>& src, int b0, int b1, int64_t m0, int64_t r0,
                     int64_t z0, bool zfield) {
        for (int it = b0; it < b1; ++it) {
            const int* w = &src[(size_t)kItemInts * it];
            const int64_t mo = ((int64_t)(uint32_t)w[0] | ((int64_t)w[1] << 32)) + m0;
            dst.push_back((int)(mo & 0xffffffff));
            dst.push_back((int)(mo >> 32));
            dst.push_back(w[2] + (int)r0);
            for (int j = 3; j < kItemInts - 1; ++j) dst.push_back(w[j]);
            dst.push_back(w[kItemInts - 1] + (zfield ? (int)z0 : 0));
        }
    };
    for (int L = 0; L < nl; ++L) {
        SolveLevel& lv = S->step_levels[L];
        lv.fwdb_begin = (int)(fwdb.size() / kItemInts);
        lv.bwdb_begin = (int)(bwdb.size() / kItemInts);
        lv.fwdw_begin = (int)(fwds.size() / kItemInts);
        lv.bwdw_begin = (int)(bwds.size() / kItemInts);
        lv.tiny_begin = (int)(tiny.size() / kItemInts);
        lv.zst_begin = (int)(zst.size() / kItemInts);
        for (Request* r : S->active) {
            const CholFactor& f = *r->me->f;
            if (L >= (int)f.step_levels.size()) continue;
            const SolveLevel& q = f.step_levels[L];
            append(fwdb, f.fwd_blocks, q.fwdb_begin, q.fwdb_end, r->m0, r->r0, r->z0, false);
            append(bwdb, f.bwd_blocks, q.bwdb_begin, q.bwdb_end, r->m0, r->r0, r->z0, true);
            append(fwds, f.fwd_small, q.fwdw_begin, q.fwdw_end, r->m0, r->r0, r->z0, false);
            append(bwds, f.bwd_small, q.bwdw_begin, q.bwdw_end, r->m0, r->r0, r->z0, false);
            append(tiny, f.tiny, q.tiny_begin, q.tiny_end, r->m0, r->r0, r->z0, false);
            append(zst, f.zstage, q.zst_begin, q.zst_end, r->m0, r->r0, r->z0, true);
        }
        lv.fwdb_end = (int)(fwdb.size() / kItemInts);
        lv.bwdb_end = (int)(bwdb.size() / kItemInts);
        lv.fwdw_end = (int)(fwds.size() / kItemInts);
        lv.bwdw_end = (int)(bwds.size() / kItemInts);
        lv.tiny_end = (int)(tiny.size() / kItemInts);
        lv.zst_end = (int)(zst.size() / kItemInts);
    }
    cudaStream_t s = S->stream;
    S->d_fwdb.upload(fwdb, s);
    S->d_bwdb.upload(bwdb, s);
    S->d_fwds.upload(fwds, s);
    S->d_bwds.upload(bwds, s);
    S->d_tiny.upload(tiny, s);
    S->d_zst.upload(zst, s);
    S->graph_dirty = true;
}

void rebuild_lists(pdgb_server* S) {
    int ntiles = 0, nchunks = 0;
    for (Request* r : S->active) {
        ntiles += r->L->ntiles;
        nchunks += (r->nv + 255) / 256;
    }
    ensure_capacity(S, (int)S->active.size(), ntiles, nchunks);
    PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));  // host mirrors and lists may still be in flight
    if (S->chol) {
        for (Request* r : S->active) set_args(S, r);  // arenas may have moved
        build_solve_lists(S);
    }
    int t = 0, c = 0;
    for (int q = 0; q < (int)S->active.size(); ++q) {
        Request* r = S->active[q];
        S->h_la[q] = r->la;
        S->h_va[q] = r->va;
        S->h_ba[q] = r->ba;
        S->h_cv[q] = r->cv;
        for (int k = 0; k < r->L->ntiles; ++k) S->h_tiles[t++] = make_int2(q, k);
        for (int v0 = 0; v0 < r->nv; v0 += 256) S->h_chunks[c++] = make_int2(q, v0);
    }
    S->h_counts[0] = t;
    S->h_counts[1] = c;
    const size_t nq = S->active.size();
    cudaStream_t s = S->stream;
    if (nq) {
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_la, S->h_la, nq * sizeof(LocalArgs), cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_va, S->h_va, nq * sizeof(VertexArgs), cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_ba, S->h_ba, nq * sizeof(BeginArgs), cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_cv, S->h_cv, nq * sizeof(CholVertexArgs), cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_tiles, S->h_tiles, t * sizeof(int2), cudaMemcpyHostToDevice, s));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_chunks, S->h_chunks, c * sizeof(int2), cudaMemcpyHostToDevice, s));
    }
    PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_counts, S->h_counts, 2 * sizeof(int), cudaMemcpyHostToDevice, s));
    if (S->graph_dirty) capture_step(S);
    S->lists_dirty = false;
}

}  // namespace

extern "C" {

void pdgb_server_default_config(pdgb_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    pdgb_default_params(&c->params);
    c->params.solver = PDGB_SOLVER_JACOBI;
    c->hbm_budget_bytes = (size_t)8 << 30;
    c->max_active = 0;
    c->host_threads = 0;
    c->cache_entries = 0;
}

int pdgb_server_create(const pdgb_server_config* cfg, void* stream, pdgb_server** out) {
    if (!cfg || !out) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "null config or out");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    pdgb_server* S = nullptr;
    const int st = guarded_s([&] {
        if (cfg->params.solver != PDGB_SOLVER_JACOBI && cfg->params.solver != PDGB_SOLVER_CHOLESKY)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "unknown solver"};
        if (!(cfg->params.dt > 0.f) || cfg->params.num_iterations < 1 || cfg->params.num_iterations > 4096)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "bad solver parameters"};
        if (cfg->hbm_budget_bytes == 0) throw Error{PDGB_ERR_INVALID_ARGUMENT, "zero HBM budget"};
        S = new pdgb_server();
        S->cfg = *cfg;
        S->chol = cfg->params.solver == PDGB_SOLVER_CHOLESKY;
        S->cache_cap = cfg->cache_entries < 0 ? 0 : cfg->cache_entries == 0 ? 256 : (size_t)cfg->cache_entries;
        if (stream) S->stream = (cudaStream_t)stream;
        else {
            PDGB_CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
            S->own_stream = true;
        }
        int dev = 0;
        PDGB_CUDA_TRY(cudaGetDevice(&dev));
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        PDGB_CUDA_TRY(cudaMemPoolCreate(&S->pool, &props));
        uint64_t keep = UINT64_MAX;  // keep freed blocks for the next admissions
        PDGB_CUDA_TRY(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        int nthr = cfg->host_threads > 0 ? cfg->host_threads : (int)std::max(1u, std::thread::hardware_concurrency() / 2);
        for (int i = 0; i < nthr; ++i) S->workers.emplace_back(worker_loop, S);
    });
    if (st != PDGB_OK) {
        delete S;
        return st;
    }
    *out = S;
    return PDGB_OK;
}

int pdgb_server_submit(pdgb_server* S, const pdgb_mesh_desc* mesh, int nsteps, long long* request_id) {
    if (!S || !mesh || !request_id || nsteps < 1 || mesh->memory != PDGB_MEM_HOST || !mesh->X || !mesh->tets ||
        !mesh->mass || !mesh->mu || mesh->num_verts <= 0 || mesh->num_tets <= 0) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad request (host mesh, nsteps >= 1 required)");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded_s([&] {
        auto r = std::make_unique<Request>();
        r->nsteps = nsteps;
        r->nv = mesh->num_verts;
        r->nt = mesh->num_tets;
        r->X.assign(mesh->X, mesh->X + 3 * (size_t)r->nv);
        if (mesh->V) r->V.assign(mesh->V, mesh->V + 3 * (size_t)r->nv);
        r->tets.assign(mesh->tets, mesh->tets + 4 * (size_t)r->nt);
        r->mass.assign(mesh->mass, mesh->mass + r->nv);
        r->mu.assign(mesh->mu, mesh->mu + r->nt);
        if (mesh->dbc) r->dbc.assign(mesh->dbc, mesh->dbc + r->nv);
        r->t_submit = Clock::now();
        std::lock_guard<std::mutex> lk(S->mu);
        r->id = S->next_id++;
        *request_id = r->id;
        S->prep_queue.push_back(r->id);
        S->reqs.emplace(r->id, std::move(r));
        S->cv.notify_one();
    });
}

int pdgb_server_tick(pdgb_server* S, int* active, int* completed) {
    if (!S) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded_s([&] {
        // The server lock is held for admission and bookkeeping only, not
        // while the step runs: the layout workers and the submitting threads
        // need it to make progress.  Only pdgb_server_tick changes the active
        // set, the arenas and the step graph, so they need no lock of their own.
        const auto t0 = Clock::now();
        std::unique_lock<std::mutex> lk(S->mu);
        // 1. admission in arrival order, by HBM budget and slot limit
        while (!S->ready_queue.empty()) {
            if (S->cfg.max_active > 0 && (int)S->active.size() >= S->cfg.max_active) break;
            auto it = S->reqs.find(S->ready_queue.front());
            if (it == S->reqs.end()) {
                S->ready_queue.pop_front();
                continue;
            }
            Request* r = it->second.get();
            if (S->bytes_in_use + r->bytes > S->cfg.hbm_budget_bytes) {
                if (S->active.empty() && r->bytes > S->cfg.hbm_budget_bytes) {  // can never fit
                    r->state = kFailed;
                    r->error = "request larger than the HBM budget";
                    S->failed++;
                    S->ready_queue.pop_front();
                    continue;
                }
                break;
            }
            S->ready_queue.pop_front();
            try {
                admit(S, r);
            } catch (const Error& e) {
                // a factor that is not positive definite fails the request
                // alone; anything else fails the tick
                if (e.status != PDGB_ERR_NOT_SPD) throw;
                if (r->block) PDGB_CUDA_TRY(cudaFreeAsync(r->block, S->stream));
                r->block = nullptr;
                release_arenas(S, r);
                r->state = kFailed;
                r->error = e.msg;
                S->failed++;
                continue;
            }
            S->active.push_back(r);
            S->lists_dirty = true;
        }
        const auto t1 = Clock::now();
        S->admit_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        int done_now = 0;
        if (!S->active.empty()) {
            S->ticks++;
            if (S->lists_dirty || S->graph_dirty) rebuild_lists(S);
            // 2. one PD step for every active request
            PDGB_CUDA_TRY(cudaGraphLaunch(S->gexec, S->stream));
            // 3. retire finished requests (copies ordered after the step)
            std::vector<Request*> keep, retired;
            for (Request* r : S->active) {
                r->steps_done++;
                S->tet_iterations += (double)r->nt * S->cfg.params.num_iterations;
                if (r->steps_done >= r->nsteps) {
                    const size_t n3 = 3 * (size_t)r->nv;
                    r->X_out.resize(n3);
                    r->V_out.resize(n3);
                    launch_scatter_state(r->nv, r->vperm, r->x, r->v, r->staging, r->staging + n3, S->stream);
                    PDGB_CUDA_TRY(cudaMemcpyAsync(r->X_out.data(), r->staging, n3 * sizeof(float),
                                                  cudaMemcpyDeviceToHost, S->stream));
                    PDGB_CUDA_TRY(cudaMemcpyAsync(r->V_out.data(), r->staging + n3, n3 * sizeof(float),
                                                  cudaMemcpyDeviceToHost, S->stream));
                    PDGB_CUDA_TRY(cudaMemcpyAsync(&r->flag_host, r->flag, sizeof(int), cudaMemcpyDeviceToHost,
                                                  S->stream));
                    PDGB_CUDA_TRY(cudaFreeAsync(r->block, S->stream));
                    r->block = nullptr;
                    release_arenas(S, r);  // reused only by later ticks, after this step
                    S->bytes_in_use -= r->bytes;
                    S->lists_dirty = true;
                    retired.push_back(r);
                    done_now++;
                } else {
                    keep.push_back(r);
                }
            }
            S->active.swap(keep);
            lk.unlock();
            PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));
            const auto now = Clock::now();
            lk.lock();
            S->step_ms += std::chrono::duration<double, std::milli>(now - t1).count();
            for (Request* r : retired) {  // results are on the host now
                r->t_done = now;
                S->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
                if (r->flag_host) {
                    // the iteration left the finite range: a failed request,
                    // not a silent NaN result
                    r->state = kFailed;
                    r->error = "the state became non-finite";
                    S->failed++;
                    S->nonfinite++;
                } else {
                    r->state = kDone;
                    S->completed++;
                }
            }
            PDGB_CUDA_TRY(cudaGetLastError());
        }
        S->busy_ms += std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
        if (active) *active = (int)S->active.size();
        if (completed) *completed = done_now;
    });
}

int pdgb_server_poll(pdgb_server* S, long long id, int* state, int* steps_done) {
    if (!S || !state) return PDGB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
        set_last_error(PDGB_ERR_NOT_FOUND, "unknown request id");
        return PDGB_ERR_NOT_FOUND;
    }
    *state = it->second->state;
    if (steps_done) *steps_done = it->second->steps_done;
    return PDGB_OK;
}

int pdgb_server_result(pdgb_server* S, long long id, float* X, float* V) {
    if (!S || (!X && !V)) return PDGB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
        set_last_error(PDGB_ERR_NOT_FOUND, "unknown request id");
        return PDGB_ERR_NOT_FOUND;
    }
    Request* r = it->second.get();
    if (r->state == kFailed) {
        const int st = r->flag_host ? PDGB_ERR_NONFINITE : PDGB_ERR_INVALID_ARGUMENT;
        set_last_error(st, "request failed: " + r->error);
        S->reqs.erase(it);
        return st;
    }
    if (r->state != kDone) {
        set_last_error(PDGB_ERR_BUSY, "request not finished");
        return PDGB_ERR_BUSY;
    }
    if (X) std::memcpy(X, r->X_out.data(), r->X_out.size() * sizeof(float));
    if (V) std::memcpy(V, r->V_out.data(), r->V_out.size() * sizeof(float));
    S->reqs.erase(it);
    return PDGB_OK;
}

int pdgb_server_get_stats(pdgb_server* S, pdgb_server_stats* out) {
    if (!S || !out) return PDGB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->completed = S->completed;
    out->failed = S->failed;
    out->active = (int)S->active.size();
    out->waiting = (int)(S->prep_queue.size() + S->ready_queue.size());
    out->bytes_in_use = S->bytes_in_use;
    out->tet_iterations = S->tet_iterations;
    out->busy_ms = S->busy_ms;
    out->admit_ms = S->admit_ms;
    out->step_ms = S->step_ms;
    out->ticks = S->ticks;
    out->ready = (int)S->ready_queue.size();
    {
        std::lock_guard<std::mutex> ck(S->cache_mu);
        out->layout_cache_hits = (int)std::min<long long>(S->cache_hits, INT32_MAX);
    }
    out->nonfinite = S->nonfinite;
    out->factors = S->factors;
    out->factor_cache_hits = S->factor_hits;
    out->factor_ms = S->factor_ms;
    return PDGB_OK;
}

int pdgb_server_latencies(pdgb_server* S, double* out_ms, int capacity, int* count) {
    if (!S || !count) return PDGB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    *count = (int)S->latencies_ms.size();
    if (out_ms)
        for (int i = 0; i < std::min(capacity, *count); ++i) out_ms[i] = S->latencies_ms[i];
    return PDGB_OK;
}

int pdgb_server_destroy(pdgb_server* S) {
    if (!S) return PDGB_ERR_INVALID_ARGUMENT;
    delete S;
    return PDGB_OK;
}

}  // extern "C"
