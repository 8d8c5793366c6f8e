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
// The tick does not wait for its step: while the step runs, it admits the
// next requests and prepares the next step's work lists (their uploads are
// ordered after the step on the stream), and the next tick waits for the
// step before it hands out the results of the requests it finished.
// Requests join and leave between steps, their work shares every launch,
// and a request's arithmetic is the single engine's (same kernels, own
// arrays), so its result does not depend on the mix.
//
// Uploads come from page-locked images kept with the cached mesh: the tile
// layout as laid out in a request's block, and (Cholesky) the row lists,
// the solve's work items and, once computed, the numeric factor.  A
// request's work items stay in a device arena with its offsets applied on
// the device; the combined per-level lists of a step are gathered from them
// by a kernel, so the host only writes a table of segments per step.
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

// Page-locked host buffer (asynchronous uploads).
template <class T> struct Pinned {
    T* p = nullptr;
    size_t n = 0;
    Pinned() = default;
    Pinned(const Pinned&) = delete;
    Pinned& operator=(const Pinned&) = delete;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
    void reserve(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        PDGB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T)));
        n = std::max<size_t>(count, 1);
    }
};

constexpr int kItemKinds = 6;  // fwd blocks, bwd blocks, fwd small, bwd small, tiny, z staging

// What the workers prepare for a mesh, shared by the requests that submit
// the same mesh (cache by content).  The images are built by the tick
// thread at the mesh's first admission and used by it only.
struct MeshEntry {
    std::shared_ptr<const HostLayout> L;
    std::shared_ptr<CholFactor> f;  // symbolic factor + front plan (Cholesky servers)
    bool images = false;
    size_t layout_bytes = 0;        // tile layout part of a request's block
    Pinned<unsigned char> layout;   // that part, as laid out in the block
    Pinned<int> rows;               // row lists (mesh vertex ids)
    Pinned<int> items;              // work items of the 6 kinds, back to back (mesh offsets)
    int64_t kbase[kItemKinds + 1] = {0};  // ints: start of each kind in items
    Pinned<float> mval;             // numeric factor once computed
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
    int64_t hin = -1, hout = -1;          // page-locked staging ranges (input state, results)
    // arena ranges of a Cholesky request
    int64_t v0 = 0, m0 = 0, r0 = 0, z0 = 0, io = 0;
    float4 *x = nullptr, *v = nullptr, *prev = nullptr, *base = nullptr;
    const float4 *coef = nullptr, *pin = nullptr;
    std::vector<float> X_out, V_out;
    Clock::time_point t_submit, t_admit, t_done;
};

template <class T> size_t bytes_of(const std::vector<T>& v) { return align256(v.size() * sizeof(T)); }

int64_t item_ints(const CholFactor& f) {
    return (int64_t)(f.fwd_blocks.size() + f.bwd_blocks.size() + f.fwd_small.size() + f.bwd_small.size() +
                     f.tiny.size() + f.zstage.size());
}

// Arena bytes of a Cholesky request: 3 solve vectors, rows, M_s, backward
// staging and work items.
size_t arena_bytes(const Request& r) {
    const CholFactor& f = *r.me->f;
    return 3 * (size_t)r.nv * sizeof(float4) + f.rows.size() * sizeof(int) + (size_t)f.mval_size * sizeof(float) +
           (size_t)f.zrows * sizeof(float4) + (size_t)item_ints(f) * sizeof(int);
}

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
    if (chol) b += arena_bytes(r);
    return b;
}

// A run of work items copied into a step's combined list: cnt ints from
// items[src] to comb[kind][dst].
struct ItemSeg {
    long long src;
    int cnt;
    int dst;
    int kind;
    int pad;
};

struct CombPtrs {
    int* p[kItemKinds];
};

__global__ void __launch_bounds__(256) k_gather_items(const int* __restrict__ items,
                                                      const ItemSeg* __restrict__ seg, CombPtrs comb) {
    const ItemSeg g = seg[blockIdx.x];
    int* dst = comb.p[g.kind] + g.dst;
    const int* src = items + g.src;
    for (int i = threadIdx.x; i < g.cnt; i += blockDim.x) dst[i] = __ldg(src + i);
}

__global__ void k_add_offset(int* a, int64_t n, int off) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += off;
}

// A request's work items (kinds back to back, kb[k] = first item of kind k)
// moved to its arena ranges: factor offset m0 into the 64-bit field of
// ints 0-1, row-list offset r0 into int 2, backward staging offset z0 into
// int 7 of the backward blocks (kind 1) and staging items (kind 5).
struct ItemShift {
    long long m0;
    int r0, z0;
    long long kb[kItemKinds + 1];
};

__global__ void k_shift_items(int* items, ItemShift sh) {
    const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= sh.kb[kItemKinds]) return;
    int kind = 0;
    while (kind + 1 < kItemKinds && it >= sh.kb[kind + 1]) ++kind;
    int* w = items + it * kItemInts;
    const long long mo = ((long long)(uint32_t)w[0] | ((long long)w[1] << 32)) + sh.m0;
    w[0] = (int)(mo & 0xffffffff);
    w[1] = (int)(mo >> 32);
    w[2] += sh.r0;
    if (kind == 1 || kind == 5) w[7] += sh.z0;
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
    Arena<int> ar_items;               // every request's work items, its offsets applied
    DBuf<int> d_comb[kItemKinds];       // the step's combined per-level lists, by kind
    Pinned<ItemSeg> h_seg;              // segments gathered into them
    // page-locked staging of the requests' states: inputs at admission,
    // results at retirement (copies to and from pageable memory would make
    // the host wait for the step in flight)
    Pinned<float> hst;
    RangeAlloc hst_ra;
    std::vector<std::pair<int64_t, int64_t>> hst_free_after_wait;
    DBuf<ItemSeg> d_seg;
    std::vector<SolveLevel> step_levels;
    // pipelining: the step launched by the last tick and the requests it finishes
    bool inflight = false;
    bool rebuilt = false;               // lists rebuilt since the last wait for the stream
    std::vector<Request*> retiring;
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
                    cholesky_factor(layout_system(*L), PDGB_ORDER_AMD, xyz.data(), *f, 0, true, true, kAmalgBytes);
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

// A range of the page-locked staging buffer (floats).  Growing it waits for
// the stream (no copy may be reading or writing the old buffer) and keeps
// its contents.
float* host_stage(pdgb_server* S, int64_t n, int64_t& off) {
    off = S->hst_ra.take(std::max<int64_t>(n, 1));
    if ((size_t)S->hst_ra.top > S->hst.n || !S->hst.p) {
        PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));
        const size_t ncap = std::max<size_t>((size_t)S->hst_ra.top, 2 * S->hst.n + (1u << 20));
        float* q = nullptr;
        PDGB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&q), ncap * sizeof(float)));
        if (S->hst.p) {
            std::memcpy(q, S->hst.p, S->hst.n * sizeof(float));
            cudaFreeHost(S->hst.p);
        }
        S->hst.p = q;
        S->hst.n = ncap;
    }
    return S->hst.p + off;
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

// The page-locked images of a mesh, built at its first admission: the tile
// layout as carved into a block, and (Cholesky) row lists and work items.
void build_images(pdgb_server* S, MeshEntry& me) {
    if (me.images) return;
    const HostLayout& L = *me.L;
    auto sz = [](size_t bytes) { return align256(bytes); };
    const size_t lb = sz(L.inc_ent.size() * 2) + sz(L.inc_end.size() * 2) + sz(L.geo.size() * 4) +
                      sz(L.tile_tet_ptr.size() * 4) + sz(L.tile_vptr.size() * 4) + sz(L.tile_verts.size() * 4) +
                      sz(L.vperm.size() * 4) + sz(L.coef.size() * 16) + sz(L.pin_rhs.size() * 16);
    me.layout.reserve(lb);
    std::memset(me.layout.p, 0, lb);
    unsigned char* q = me.layout.p;
    auto copy = [&](const void* src, size_t bytes) {
        if (bytes) std::memcpy(q, src, bytes);
        q += sz(bytes);
    };
    copy(L.inc_ent.data(), L.inc_ent.size() * 2);
    copy(L.inc_end.data(), L.inc_end.size() * 2);
    copy(L.geo.data(), L.geo.size() * 4);
    copy(L.tile_tet_ptr.data(), L.tile_tet_ptr.size() * 4);
    copy(L.tile_vptr.data(), L.tile_vptr.size() * 4);
    copy(L.tile_verts.data(), L.tile_verts.size() * 4);
    copy(L.vperm.data(), L.vperm.size() * 4);
    copy(L.coef.data(), L.coef.size() * 16);
    copy(L.pin_rhs.data(), L.pin_rhs.size() * 16);
    me.layout_bytes = lb;
    if (S->chol) {
        const CholFactor& f = *me.f;
        me.rows.reserve(f.rows.size());
        if (!f.rows.empty()) std::memcpy(me.rows.p, f.rows.data(), f.rows.size() * sizeof(int));
        const std::vector<int>* kinds[kItemKinds] = {&f.fwd_blocks, &f.bwd_blocks, &f.fwd_small,
                                                     &f.bwd_small,  &f.tiny,       &f.zstage};
        me.kbase[0] = 0;
        for (int k = 0; k < kItemKinds; ++k) me.kbase[k + 1] = me.kbase[k] + (int64_t)kinds[k]->size();
        me.items.reserve((size_t)me.kbase[kItemKinds]);
        for (int k = 0; k < kItemKinds; ++k)
            if (!kinds[k]->empty())
                std::memcpy(me.items.p + me.kbase[k], kinds[k]->data(), kinds[k]->size() * sizeof(int));
    }
    me.images = true;
}

// Uploads a prepared request into its device block (and arenas).  The
// copies are ordered on the stream after any step in flight.
void admit(pdgb_server* S, Request* r) {
    cudaStream_t s = S->stream;
    MeshEntry& me = *r->me;
    build_images(S, me);
    const HostLayout& L = *r->L;
    const int nv = r->nv;
    const bool chol = S->chol;
    const size_t block_bytes = r->bytes - (chol ? arena_bytes(*r) : 0);
    PDGB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r->block), block_bytes, S->pool, s));
    PDGB_CUDA_TRY(cudaMemcpyAsync(r->block, me.layout.p, me.layout_bytes, cudaMemcpyHostToDevice, s));
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
    if ((size_t)(p - r->block) != me.layout_bytes) throw Error{PDGB_ERR_CUDA, "server: layout image mismatch"};
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
    PDGB_CUDA_TRY(cudaMemsetAsync(r->flag, 0, sizeof(int), s));
    PDGB_CUDA_TRY(cudaMemsetAsync(r->prev, 0, (size_t)nv * sizeof(float4), s));
    const bool hasV = !r->V.empty();
    {
        const int64_t n = (hasV ? 6 : 3) * (int64_t)nv;
        float* h = host_stage(S, n, r->hin);
        std::memcpy(h, r->X.data(), 3 * (size_t)nv * sizeof(float));
        if (hasV) std::memcpy(h + 3 * (size_t)nv, r->V.data(), 3 * (size_t)nv * sizeof(float));
        PDGB_CUDA_TRY(cudaMemcpyAsync(r->staging, h, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s));
        S->hst_free_after_wait.emplace_back(r->hin, n);  // read by the copy: free once the stream is waited for
    }
    launch_gather_state(nv, r->vperm, r->staging, hasV ? r->staging + 3 * (size_t)nv : nullptr, r->x, r->v, s);
    PDGB_CUDA_TRY(cudaGetLastError());
    r->la = LocalArgs{sn, b, inc_ent, inc_end, geo, ttp, tvp, tv, L.nt_pad, nullptr};
    if (chol) {
        const CholFactor& f = *me.f;
        int64_t v0, m0, r0, z0, io, tmp;
        const int64_t nitems = me.kbase[kItemKinds];
        bool moved = S->va_sn.take(nv, v0, s);
        moved |= S->va_b.take(nv, tmp, s);
        moved |= S->va_y.take(nv, tmp, s);
        moved |= S->ar_mval.take(f.mval_size, m0, s);
        moved |= S->ar_rows.take((int64_t)f.rows.size(), r0, s);
        moved |= S->ar_zbuf.take(f.zrows, z0, s);
        moved |= S->ar_items.take(nitems, io, s);
        if (moved) S->lists_dirty = true;  // every request's arena pointers change
        r->v0 = v0;
        r->m0 = m0;
        r->r0 = r0;
        r->z0 = z0;
        r->io = io;
        const int64_t nrows = (int64_t)f.rows.size();
        if (nrows) {
            PDGB_CUDA_TRY(cudaMemcpyAsync(S->ar_rows.p + r0, me.rows.p, (size_t)nrows * sizeof(int),
                                          cudaMemcpyHostToDevice, s));
            k_add_offset<<<(unsigned)((nrows + 255) / 256), 256, 0, s>>>(S->ar_rows.p + r0, nrows, (int)v0);
        }
        if (nitems) {
            PDGB_CUDA_TRY(cudaMemcpyAsync(S->ar_items.p + io, me.items.p, (size_t)nitems * sizeof(int),
                                          cudaMemcpyHostToDevice, s));
            ItemShift sh{};
            sh.m0 = m0;
            sh.r0 = (int)r0;
            sh.z0 = (int)z0;
            for (int k = 0; k <= kItemKinds; ++k) sh.kb[k] = me.kbase[k] / kItemInts;
            const long long n = sh.kb[kItemKinds];
            if (n) k_shift_items<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(S->ar_items.p + io, sh);
        }
        PDGB_CUDA_TRY(cudaMemsetAsync(S->va_y.p + v0, 0, (size_t)nv * sizeof(float4), s));
        // the numeric factor: computed on the GPU the first time the mesh is
        // seen, uploaded from the page-locked copy after that
        if (me.numeric) {
            if (f.mval_size)
                PDGB_CUDA_TRY(cudaMemcpyAsync(S->ar_mval.p + m0, me.mval.p, (size_t)f.mval_size * sizeof(float),
                                              cudaMemcpyHostToDevice, s));
            S->factor_hits++;
        } else {
            S->factor_ms += gpu_factor(f, S->ar_mval.p + m0, s);
            S->factors++;
            if (S->cache_cap > 0) {
                me.mval.reserve((size_t)f.mval_size);
                if (f.mval_size)
                    PDGB_CUDA_TRY(cudaMemcpyAsync(me.mval.p, S->ar_mval.p + m0, (size_t)f.mval_size * sizeof(float),
                                                  cudaMemcpyDeviceToHost, s));
                PDGB_CUDA_TRY(cudaStreamSynchronize(s));
                me.numeric = true;
                me.f->fp = FrontPlan();  // the front plan is not needed again
            }
        }
        PDGB_CUDA_TRY(cudaGetLastError());
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
    S->ar_items.give(r->io, r->me->kbase[kItemKinds]);
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

// Jacobi: the step as a CUDA graph, grids sized by the list capacities
// (CTAs past the current counts exit), so it survives changes of the active
// set; captured again only when the capacities grow.
void capture_step(pdgb_server* S) {
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    if (S->graph) cudaGraphDestroy(S->graph);
    S->gexec = nullptr;
    S->graph = nullptr;
    cudaStream_t s = S->stream;
    const int n = S->cfg.params.num_iterations;
    const std::vector<float> omega = chebyshev_omegas(n, S->cfg.params.rho);
    PDGB_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        launch_begin_multi(S->d_ba, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
        for (int i = 0; i < n; ++i) {
            launch_local_multi(S->d_la, S->d_tiles, S->d_counts, S->cap_tiles, s, true);
            int mode = 0;
            if (i >= 11) mode |= kReadPrev;
            if (i >= 10 && i + 1 < n) mode |= kWritePrev;
            if (i + 1 == n) mode |= kFinal;
            launch_jacobi_vertex_multi(S->d_va, S->d_chunks, S->d_counts + 1, S->cap_chunks, mode, omega[i], s);
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

// One PD step for every active request.  Cholesky: direct launches, since
// the per-level solve launches follow the active requests' trees and the
// set changes from one step to the next (the host issues them while the GPU
// works through them).
void launch_step(pdgb_server* S) {
    cudaStream_t s = S->stream;
    if (!S->chol) {
        PDGB_CUDA_TRY(cudaGraphLaunch(S->gexec, s));
        return;
    }
    const int n = S->cfg.params.num_iterations;
    CholArgs ca{};
    ca.rows = S->ar_rows.p;
    ca.mval = S->ar_mval.p;
    ca.r = S->va_b.p;
    ca.y = S->va_y.p;
    ca.x = S->va_sn.p;
    ca.done = nullptr;
    ca.fwd_blocks = S->d_comb[0].p;
    ca.bwd_blocks = S->d_comb[1].p;
    ca.fwd_small = S->d_comb[2].p;
    ca.bwd_small = S->d_comb[3].p;
    ca.tiny = S->d_comb[4].p;
    ca.zstage = S->d_comb[5].p;
    ca.zbuf = S->ar_zbuf.p;
    launch_begin_multi(S->d_ba, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
    for (int i = 0; i < n; ++i) {
        launch_local_multi(S->d_la, S->d_tiles, S->d_counts, S->cap_tiles, s, false);
        launch_chol_solve_levels(ca, S->step_levels, s);
        launch_chol_vertex_multi(S->d_cv, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
    }
    launch_chol_finish_multi(S->d_cv, S->d_chunks, S->d_counts + 1, S->cap_chunks, s);
    PDGB_CUDA_TRY(cudaGetLastError());
}

// Per-level solve lists of all active Cholesky requests: level L of every
// request's tree in the same lists (levels counted from the leaves).  The
// host writes one segment per (level, request, kind) -- where the request's
// items of that level lie in the items arena (its offsets already applied)
// and where they go -- and a kernel gathers the items on the device.
void build_solve_lists(pdgb_server* S) {
    int nl = 0;
    for (Request* r : S->active) nl = std::max(nl, (int)r->me->f->step_levels.size());
    S->step_levels.assign(nl, SolveLevel{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0});
    std::vector<ItemSeg> seg;
    seg.reserve((size_t)nl * S->active.size() * 2);
    int64_t tot[kItemKinds] = {0};
    auto range = [](const SolveLevel& q, int k, int& b, int& e) {
        switch (k) {
            case 0: b = q.fwdb_begin; e = q.fwdb_end; break;
            case 1: b = q.bwdb_begin; e = q.bwdb_end; break;
            case 2: b = q.fwdw_begin; e = q.fwdw_end; break;
            case 3: b = q.bwdw_begin; e = q.bwdw_end; break;
            case 4: b = q.tiny_begin; e = q.tiny_end; break;
            default: b = q.zst_begin; e = q.zst_end; break;
        }
    };
    for (int L = 0; L < nl; ++L) {
        int begin[kItemKinds];
        for (int k = 0; k < kItemKinds; ++k) begin[k] = (int)(tot[k] / kItemInts);
        for (Request* r : S->active) {
            const CholFactor& f = *r->me->f;
            if (L >= (int)f.step_levels.size()) continue;
            const SolveLevel& q = f.step_levels[L];
            for (int k = 0; k < kItemKinds; ++k) {
                int b, e;
                range(q, k, b, e);
                if (e <= b) continue;
                const int cnt = (e - b) * kItemInts;
                seg.push_back(ItemSeg{(long long)(r->io + r->me->kbase[k] + (int64_t)b * kItemInts), cnt,
                                      (int)tot[k], k, 0});
                tot[k] += cnt;
            }
        }
        SolveLevel& lv = S->step_levels[L];
        int end[kItemKinds];
        for (int k = 0; k < kItemKinds; ++k) end[k] = (int)(tot[k] / kItemInts);
        lv.fwdb_begin = begin[0]; lv.fwdb_end = end[0];
        lv.bwdb_begin = begin[1]; lv.bwdb_end = end[1];
        lv.fwdw_begin = begin[2]; lv.fwdw_end = end[2];
        lv.bwdw_begin = begin[3]; lv.bwdw_end = end[3];
        lv.tiny_begin = begin[4]; lv.tiny_end = end[4];
        lv.zst_begin = begin[5]; lv.zst_end = end[5];
    }
    cudaStream_t s = S->stream;
    bool grow = seg.size() > S->h_seg.n || seg.size() > S->d_seg.n;
    for (int k = 0; k < kItemKinds; ++k) grow |= (size_t)tot[k] > S->d_comb[k].n;
    if (grow) {
        // the buffers may be in use by the step in flight
        PDGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (seg.size() > S->h_seg.n) S->h_seg.reserve(seg.size() * 2);
        if (seg.size() > S->d_seg.n) S->d_seg.alloc(seg.size() * 2);
        for (int k = 0; k < kItemKinds; ++k)
            if ((size_t)tot[k] > S->d_comb[k].n) S->d_comb[k].alloc((size_t)tot[k] * 2);
    }
    if (!seg.empty()) {
        std::memcpy(S->h_seg.p, seg.data(), seg.size() * sizeof(ItemSeg));
        PDGB_CUDA_TRY(cudaMemcpyAsync(S->d_seg.p, S->h_seg.p, seg.size() * sizeof(ItemSeg), cudaMemcpyHostToDevice, s));
        CombPtrs cp;
        for (int k = 0; k < kItemKinds; ++k) cp.p[k] = S->d_comb[k].p;
        k_gather_items<<<(unsigned)seg.size(), 256, 0, s>>>(S->ar_items.p, S->d_seg.p, cp);
        PDGB_CUDA_TRY(cudaGetLastError());
    }
}

// Work lists of the next step.  Uploads are ordered on the stream after any
// step in flight; the page-locked mirrors they read were last read by the
// uploads of an earlier tick, which the wait at the start of this tick has
// completed -- unless the lists were already rebuilt since that wait, in
// which case their uploads may be pending and the stream is waited for.
void rebuild_lists(pdgb_server* S) {
    if (S->rebuilt) PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));
    S->rebuilt = true;
    int ntiles = 0, nchunks = 0;
    for (Request* r : S->active) {
        ntiles += r->L->ntiles;
        nchunks += (r->nv + 255) / 256;
    }
    ensure_capacity(S, (int)S->active.size(), ntiles, nchunks);
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
    if (!S->chol && S->graph_dirty) capture_step(S);
    if (S->chol) S->graph_dirty = false;  // no graph: the step is launched directly
    S->lists_dirty = false;
}

// Admission in arrival order, by HBM budget and slot limit (server lock held).
void admit_ready(pdgb_server* S) {
    while (!S->ready_queue.empty()) {
        if (S->cfg.max_active > 0 && (int)S->active.size() >= S->cfg.max_active) break;
        auto it = S->reqs.find(S->ready_queue.front());
        if (it == S->reqs.end()) {
            S->ready_queue.pop_front();
            continue;
        }
        Request* r = it->second.get();
        if (S->bytes_in_use + r->bytes > S->cfg.hbm_budget_bytes) {
            if (S->active.empty() && S->retiring.empty() && r->bytes > S->cfg.hbm_budget_bytes) {
                r->state = kFailed;  // can never fit
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
}

// Requests that reached their step count with the step just launched: their
// state is copied to the host and their memory released, ordered after the
// step; they are handed out once the next tick has waited for it.
void retire_finished(pdgb_server* S) {
    std::vector<Request*> keep;
    for (Request* r : S->active) {
        r->steps_done++;
        S->tet_iterations += (double)r->nt * S->cfg.params.num_iterations;
        if (r->steps_done < r->nsteps) {
            keep.push_back(r);
            continue;
        }
        const size_t n3 = 3 * (size_t)r->nv;
        launch_scatter_state(r->nv, r->vperm, r->x, r->v, r->staging, r->staging + n3, S->stream);
        float* h = host_stage(S, 2 * (int64_t)n3 + 1, r->hout);
        PDGB_CUDA_TRY(cudaMemcpyAsync(h, r->staging, 2 * n3 * sizeof(float), cudaMemcpyDeviceToHost, S->stream));
        PDGB_CUDA_TRY(cudaMemcpyAsync(h + 2 * n3, r->flag, sizeof(int), cudaMemcpyDeviceToHost, S->stream));
        PDGB_CUDA_TRY(cudaFreeAsync(r->block, S->stream));
        r->block = nullptr;
        release_arenas(S, r);  // reused only by uploads ordered after this step
        S->bytes_in_use -= r->bytes;
        S->lists_dirty = true;
        S->retiring.push_back(r);
    }
    S->active.swap(keep);
}

// After the wait for the step: the retired requests' results are on the host.
int hand_out(pdgb_server* S, Clock::time_point now) {
    int n = 0;
    for (auto& fr : S->hst_free_after_wait) S->hst_ra.give(fr.first, fr.second);
    S->hst_free_after_wait.clear();
    for (Request* r : S->retiring) {
        const size_t n3 = 3 * (size_t)r->nv;
        const float* h = S->hst.p + r->hout;
        r->X_out.assign(h, h + n3);
        r->V_out.assign(h + n3, h + 2 * n3);
        std::memcpy(&r->flag_host, h + 2 * n3, sizeof(int));
        S->hst_ra.give(r->hout, 2 * (int64_t)n3 + 1);
        r->t_done = now;
        S->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
        if (r->flag_host) {
            // the iteration left the finite range: a failed request, not a
            // silent NaN result
            r->state = kFailed;
            r->error = "the state became non-finite";
            S->failed++;
            S->nonfinite++;
        } else {
            r->state = kDone;
            S->completed++;
        }
        ++n;
    }
    S->retiring.clear();
    return n;
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
        // while waiting for the GPU: the layout workers and the submitting
        // threads need it to make progress.  Only pdgb_server_tick changes
        // the active set, the arenas and the step lists, so they need no
        // lock of their own.
        const auto t0 = Clock::now();
        std::unique_lock<std::mutex> lk(S->mu);
        int done_now = 0;
        // 1. wait for the step launched by the previous tick; hand out the
        //    results of the requests it finished
        if (S->inflight) {
            lk.unlock();
            PDGB_CUDA_TRY(cudaStreamSynchronize(S->stream));
            const auto now = Clock::now();
            lk.lock();
            S->step_ms += std::chrono::duration<double, std::milli>(now - t0).count();
            done_now = hand_out(S, now);
            S->inflight = false;
        }
        S->rebuilt = false;
        // 2. admission when the server is idle (otherwise requests are
        //    admitted while the step runs, step 4)
        const auto t1 = Clock::now();
        if (S->active.empty()) admit_ready(S);
        double admit = std::chrono::duration<double, std::milli>(Clock::now() - t1).count();
        if (!S->active.empty()) {
            S->ticks++;
            // 3. one PD step for every active request
            if (S->lists_dirty || S->graph_dirty) rebuild_lists(S);
            launch_step(S);
            retire_finished(S);
            S->inflight = true;
            // 4. while it runs: the next admissions and the next step's lists
            const auto t2 = Clock::now();
            admit_ready(S);
            if (!S->active.empty() && (S->lists_dirty || S->graph_dirty)) rebuild_lists(S);
            admit += std::chrono::duration<double, std::milli>(Clock::now() - t2).count();
        }
        S->admit_ms += admit;
        PDGB_CUDA_TRY(cudaGetLastError());
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
    out->finishing = (int)S->retiring.size();
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
