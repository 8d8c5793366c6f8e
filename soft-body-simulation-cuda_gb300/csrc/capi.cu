// C ABI of the pdgb engine (include/pdgb.h).
//
// An engine is the GB300 counterpart of one PdSolver bound to one
// SolverData<float> (pdSolver.h:12-44): it owns a device copy of the mesh in
// its own layout, the solver scratch, and a CUDA graph holding one full time
// step (prologue, num_iterations x (local kernel, global solve), velocity /
// position update), replayed by pdgb_step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "ccd.h"
#include "cholesky.h"
#include "engine.h"
#include "solve.h"

namespace pdgb {

static thread_local std::string g_last_error;

void set_last_error(int status, const std::string& msg) {
    (void)status;
    g_last_error = msg;
}

}  // namespace pdgb

using namespace pdgb;

struct pdgb_engine {
    pdgb_params prm{};
    int ordering = PDGB_ORDER_AMD;
    int rotation = PDGB_ROTATION_QUAT;
    int local_kernel = PDGB_LOCAL_TILE;
    int pipe_grid = 0;  // resident CTAs of the pipelined local step (0: tile form)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int nv = 0, nt = 0;
    int nbodies = 1;
    std::vector<int> body_vstart, body_tstart;  // caller order, [nbodies + 1]
    // caller data (host copies, caller order)
    std::vector<float> X0, mass, mu, dbc;
    std::vector<uint32_t> tets;
    bool has_dbc = false;
    HostLayout L;
    bool prepared = false;
    // device: mesh
    DBuf<uint16_t> inc_ent, inc_end;
    DBuf<float> geo;
    DBuf<int> tile_tet_ptr, tile_vptr, vperm;
    DBuf<int> viperm;  // caller -> internal vertex, uploaded on first render
    DBuf<uint32_t> tile_verts;
    DBuf<float4> coef, pin_rhs, x0;
    // device: state + scratch
    DBuf<float4> x, v, sn, prev, base, b, y;
    DBuf<float> staging;  // [6 nv] host <-> device transfers
    DBuf<StepState> st;   // convergence state of the Cholesky path
    // Cholesky factor
    CholFactor chol;
    int chol_ordering = -1;
    float chol_dt = 0.f, chol_pw = -1.f;
    DBuf<int> ch_fwd, ch_bwd, ch_rows, ch_body_level, ch_body_order, ch_fwdb, ch_bwdb, ch_fwds, ch_bwds, ch_tiny,
        ch_zstage;
    DBuf<float4> ch_zbuf;
    DBuf<int4> ch_levels;
    DBuf<SolveLevel> ch_step_lv;  // per-level item ranges on the device (persistent solve)
    // distributed-shared-memory solve of a single body (when it fits)
    DsmPlan dsm;
    DBuf<float> dsm_mcopy;
    DBuf<int> dsm_mcopy_ptr, dsm_rcopy, dsm_rcopy_ptr, dsm_items, dsm_lvl;
    DBuf<float> ch_mval;
    DBuf<int> k_rowptr, k_colind;  // FP64 K for refinement residuals
    DBuf<double> k_val;
    DBuf<float4> bsave, dx;
    int solve_req = PDGB_SOLVE_AUTO;  // requested solve schedule
    int solve_mode = PDGB_SOLVE_LEVELS;  // schedule in use (decided at prepare)
    int factor_req = PDGB_FACTOR_GPU;    // where the numeric factorisation runs
    int factor_dev = PDGB_FACTOR_GPU;    // where it ran for the current factor
    double factor_ms = 0.0, numeric_ms = 0.0;
    long long pool_bytes = 0;
    // scene terms: drag and fixed rigid bodies
    bool drag_on = false;
    DBuf<float> drag_w;
    DBuf<float4> drag_off, drag_target;
    DBuf<float4> xt;                  // XTilde, allocated when fixed bodies are first set
    DBuf<FixedBodyDev> fixed;
    int nfixed = 0;
    float mu_t = 0.5f, mu_n = 0.5f;
    // continuous collision between bodies
    std::unique_ptr<CcdContext> ccd;
    bool ccd_on = false;
    int num_pinned = 0;
    // step graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // timing: PDGB_TIMING_STEPS records a pair of events around every step
    // graph launch; PDGB_TIMING_KERNELS also brackets every local-step launch
    // inside the graph and waits for each step
    int timing_mode = PDGB_TIMING_OFF;
    bool timing = false;              // graph carries the per-local events
    std::vector<cudaEvent_t> events;  // 2 per local launch
    cudaEvent_t step_ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> step_pairs;  // 2 per step, PDGB_TIMING_STEPS
    size_t step_pairs_used = 0;
    std::vector<cudaEvent_t> solve_events;  // 2 per global solve (Cholesky path)
    double local_ms_acc = 0.0, step_ms_acc = 0.0, solve_ms_acc = 0.0;
    long long local_launches = 0, steps_timed = 0, solves = 0;
    // perf
    double prepare_ms = 0.0;
    double steps_run = 0, iters_run = 0;

    ~pdgb_engine() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        for (auto ev : events) cudaEventDestroy(ev);
        for (auto ev : step_ev)
            if (ev) cudaEventDestroy(ev);
        for (auto ev : step_pairs) cudaEventDestroy(ev);
        for (auto ev : solve_events) cudaEventDestroy(ev);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace {

// Single bodies up to this many vertices: the autotuner also tries the
// factor as one dense supernode.
constexpr int kDenseTuneMaxVerts = 4096;

// Factors up to this many stored entries use the single-CTA solve.
constexpr size_t kCtaSolveMaxEntries = 1u << 15;

template <class F> int guarded(F&& f) {
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

void check_params(const pdgb_params& p) {
    if (!(p.dt > 0.f) || !std::isfinite(p.dt)) throw Error{PDGB_ERR_INVALID_ARGUMENT, "dt must be > 0"};
    if (p.num_iterations < 1 || p.num_iterations > 4096)
        throw Error{PDGB_ERR_INVALID_ARGUMENT, "num_iterations must be in [1, 4096]"};
    if (p.solver != PDGB_SOLVER_JACOBI && p.solver != PDGB_SOLVER_CHOLESKY)
        throw Error{PDGB_ERR_INVALID_ARGUMENT, "unknown solver"};
    if (p.refine_steps < 0 || p.refine_steps > 3) throw Error{PDGB_ERR_INVALID_ARGUMENT, "refine_steps must be 0..3"};
    // refinement applies to the Cholesky path of single-body engines
    if (!(p.positional_weight >= 0.f)) throw Error{PDGB_ERR_INVALID_ARGUMENT, "positional_weight must be >= 0"};
    if (!(p.tol >= 0.f)) throw Error{PDGB_ERR_INVALID_ARGUMENT, "tol must be >= 0"};
}

template <class T> void copy_in(std::vector<T>& dst, const T* src, size_t n, int memory) {
    dst.resize(n);
    if (n == 0) return;
    if (memory == PDGB_MEM_DEVICE) PDGB_CUDA_TRY(cudaMemcpy(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost));
    else std::memcpy(dst.data(), src, n * sizeof(T));
}

void destroy_graph(pdgb_engine* e) {
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->gexec = nullptr;
    e->graph = nullptr;
}

LocalArgs local_args(pdgb_engine* e, const int* done) {
    LocalArgs a;
    a.sn = e->sn.p;
    a.b = e->b.p;
    a.inc_ent = e->inc_ent.p;
    a.inc_end = e->inc_end.p;
    a.geo = e->geo.p;
    a.tile_tet_ptr = e->tile_tet_ptr.p;
    a.tile_vptr = e->tile_vptr.p;
    a.tile_verts = e->tile_verts.p;
    a.nt_pad = e->L.nt_pad;
    a.done = done;
    a.pipe_grid = e->local_kernel == PDGB_LOCAL_PIPELINED ? e->pipe_grid : 0;
    a.timeout = &e->st.p->local_timeout;
    return a;
}

SceneArgs scene_args(pdgb_engine* e) {
    SceneArgs sc{};
    if (e->drag_on) {
        sc.drag_w = e->drag_w.p;
        sc.drag_off = e->drag_off.p;
        sc.target = e->drag_target.p;
        sc.drag_rhs = e->num_pinned > 0;
    }
    sc.dt2 = e->prm.dt * e->prm.dt;
    sc.xt = e->xt.p;
    sc.fixed = e->fixed.p;
    sc.nfixed = e->nfixed;
    sc.mu_t = e->mu_t;
    sc.mu_n = e->mu_n;
    sc.ccd = e->ccd_on ? 1 : 0;
    sc.nonfinite = e->st.p ? &e->st.p->nonfinite : nullptr;
    return sc;
}

// Clears the sticky step status words (the state was set again): the
// non-finite flag and the persistent solve's barrier state.
void clear_nonfinite(pdgb_engine* e) {
    PDGB_CUDA_TRY(cudaMemsetAsync(&e->st.p->nonfinite, 0, 2 * sizeof(int), e->stream));  // + local_timeout
    PDGB_CUDA_TRY(cudaMemsetAsync(&e->st.p->bar, 0, sizeof(GridSync), e->stream));
}

// Collision detection + response after a step (PdSolver::Update,
// pdSolver.cu:218-231).
void run_collision(pdgb_engine* e) {
    e->ccd->detect(e->x.p, e->xt.p);
    e->ccd->respond(e->x.p, e->xt.p, e->v.p, scene_args(e));
}

BeginArgs begin_args(pdgb_engine* e) {
    BeginArgs ba{};
    ba.nv = e->nv;
    ba.x = e->x.p;
    ba.v = e->v.p;
    ba.coef = e->coef.p;
    ba.pin_rhs = e->pin_rhs.p;
    ba.sn = e->sn.p;
    ba.base = e->base.p;
    ba.b = e->b.p;
    ba.dt = e->prm.dt;
    ba.gravity = e->prm.gravity;
    ba.vperm = e->vperm.p;
    ba.num_iterations = e->prm.num_iterations;
    ba.sc = scene_args(e);
    return ba;
}

DsmArgs dsm_args(const pdgb_engine* e) {
    DsmArgs d{};
    d.mcopy = e->dsm_mcopy.p;
    d.mcopy_ptr = e->dsm_mcopy_ptr.p;
    d.rcopy = e->dsm_rcopy.p;
    d.rcopy_ptr = e->dsm_rcopy_ptr.p;
    d.items = e->dsm_items.p;
    d.lvl = reinterpret_cast<const int4*>(e->dsm_lvl.p);
    d.nlevels = e->dsm.nlevels;
    d.n = e->dsm.n;
    d.slots = e->dsm.slots;
    d.m_area = e->dsm.m_area;
    d.r_area = e->dsm.r_area;
    return d;
}

void record_local(pdgb_engine* e, const LocalArgs& la, bool jacobi_form, int i) {
    cudaStream_t s = e->stream;
    if (e->timing) PDGB_CUDA_TRY(cudaEventRecordWithFlags(e->events[2 * i], s, cudaEventRecordExternal));
    launch_local(la, e->L.ntiles, e->L.max_patch, jacobi_form, e->rotation, s);
    if (e->timing) PDGB_CUDA_TRY(cudaEventRecordWithFlags(e->events[2 * i + 1], s, cudaEventRecordExternal));
}

// One time step of the Jacobi-Chebyshev path (pdSolver.cu:141-208, Jacobi).
void record_jacobi_step(pdgb_engine* e) {
    cudaStream_t s = e->stream;
    const int n = e->prm.num_iterations;
    launch_begin(begin_args(e), s);
    const std::vector<float> omega = chebyshev_omegas(n, e->prm.rho);
    const LocalArgs la = local_args(e, nullptr);
    VertexArgs va{e->nv, e->sn.p, e->prev.p, e->b.p, e->base.p, e->coef.p, e->pin_rhs.p, e->x.p, e->v.p, 1.f,
                  1.0f / e->prm.dt};
    va.sc = scene_args(e);
    for (int i = 0; i < n; ++i) {
        record_local(e, la, true, i);
        int mode = 0;
        if (i >= 11) mode |= kReadPrev;                // omega != 1 from iteration 11 on
        if (i >= 10 && i + 1 < n) mode |= kWritePrev;  // prev is read from iteration 11 on
        if (i + 1 == n) mode |= kFinal;
        va.omega = omega[i];
        launch_jacobi_vertex(va, mode, s);
    }
}

// One time step of the Cholesky path (pdSolver.cu:141-208, cuSOLVER branch).
void record_chol_step(pdgb_engine* e) {
    cudaStream_t s = e->stream;
    const int n = e->prm.num_iterations;
    const bool use_tol = e->prm.tol > 0.f && e->nbodies == 1;  // batches: fixed iteration count
    StepState* st = e->st.p;
    BeginArgs ba = begin_args(e);
    ba.done = &st->done;
    ba.iterations = &st->iterations;
    ba.prev = use_tol ? e->prev.p : nullptr;
    launch_begin(ba, s);
    const LocalArgs la = local_args(e, &st->done);
    CholArgs ca{e->ch_fwd.p, e->ch_bwd.p, e->ch_rows.p, e->ch_mval.p, e->ch_levels.p, e->ch_body_level.p,
                e->ch_body_order.p, e->b.p, e->y.p, e->sn.p, &st->done, e->ch_fwdb.p, e->ch_bwdb.p,
                e->ch_fwds.p, e->ch_bwds.p, e->ch_tiny.p, e->ch_zstage.p, e->ch_zbuf.p};
    CholVertexArgs cv{};
    cv.nv = e->nv;
    cv.tol = use_tol ? e->prm.tol : 0.f;
    cv.st = st;
    cv.prev = e->prev.p;
    cv.sn = e->sn.p;
    cv.y = e->y.p;
    cv.b = e->b.p;
    cv.base = e->base.p;
    cv.coef = e->coef.p;
    cv.pin_rhs = e->pin_rhs.p;
    cv.x = e->x.p;
    cv.v = e->v.p;
    cv.dt_inv = 1.0f / e->prm.dt;
    cv.sc = scene_args(e);
    const bool drag_rhs = cv.sc.drag_w && cv.sc.drag_rhs;
    const int refine = e->nbodies == 1 ? e->prm.refine_steps : 0;
    CholArgs cd = ca;  // refinement solves write the correction into dx
    cd.x = e->dx.p;
    RefineArgs ra{e->nv, e->k_rowptr.p, e->k_colind.p, e->k_val.p, e->bsave.p, e->sn.p, e->b.p, e->y.p,
                  e->dx.p, e->sn.p, &st->done};
    auto solve = [&](const CholArgs& args) {
        if (e->solve_mode == PDGB_SOLVE_CTA) launch_chol_solve_cta(args, e->nbodies, s);
        else if (e->solve_mode == PDGB_SOLVE_CLUSTER) launch_chol_solve_cluster(args, e->nbodies, s);
        else if (e->solve_mode == PDGB_SOLVE_DSM) launch_chol_solve_dsm(args, dsm_args(e), e->dsm.smem_bytes, s);
        else if (e->solve_mode == PDGB_SOLVE_PERSISTENT)
            launch_chol_solve_persistent(args, e->ch_step_lv.p, (int)e->chol.step_levels.size(), &st->bar,
                                         kPersistSpinLimit, s);
        else launch_chol_solve_levels(args, e->chol.step_levels, s);
    };
    for (int i = 0; i < n; ++i) {
        record_local(e, la, false, i);
        if (drag_rhs) launch_drag_rhs(e->nv, cv.sc, e->base.p, e->b.p, &st->done, s);
        if (refine > 0) launch_copy_rhs(e->nv, e->b.p, e->bsave.p, &st->done, s);
        if (e->timing) PDGB_CUDA_TRY(cudaEventRecordWithFlags(e->solve_events[2 * i], s, cudaEventRecordExternal));
        solve(ca);
        if (e->timing) PDGB_CUDA_TRY(cudaEventRecordWithFlags(e->solve_events[2 * i + 1], s, cudaEventRecordExternal));
        for (int r = 0; r < refine; ++r) {
            launch_refine_residual(ra, s);
            solve(cd);
            launch_refine_update(ra, s);
        }
        cv.iteration = i;
        launch_chol_vertex(cv, s);
    }
    launch_chol_finish(cv, s);
}

void build_graph(pdgb_engine* e) {
    destroy_graph(e);
    if (e->timing) {
        const size_t need = 2 * (size_t)e->prm.num_iterations;
        for (auto* vec : {&e->events, &e->solve_events})
            while (vec->size() < need) {
                cudaEvent_t ev;
                PDGB_CUDA_TRY(cudaEventCreate(&ev));
                vec->push_back(ev);
            }
    }
    PDGB_CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    try {
        if (e->prm.solver == PDGB_SOLVER_JACOBI) record_jacobi_step(e);
        else record_chol_step(e);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(e->stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    PDGB_CUDA_TRY(cudaStreamEndCapture(e->stream, &e->graph));
    PDGB_CUDA_TRY(cudaGraphInstantiate(&e->gexec, e->graph, 0));
}

void upload_mesh(pdgb_engine* e) {
    const HostLayout& L = e->L;
    cudaStream_t s = e->stream;
    e->inc_ent.upload(L.inc_ent, s);
    e->inc_end.upload(L.inc_end, s);
    e->geo.upload(L.geo, s);
    e->tile_tet_ptr.upload(L.tile_tet_ptr, s);
    e->tile_vptr.upload(L.tile_vptr, s);
    e->tile_verts.upload(L.tile_verts, s);
    e->vperm.upload(L.vperm, s);
    e->x0.upload(L.x0, s);
    const size_t nv = e->nv;
    e->x.alloc(nv);
    e->v.alloc(nv);
    e->sn.alloc(nv);
    e->prev.alloc(nv);
    e->base.alloc(nv);
    e->b.alloc(nv);
    e->y.alloc(nv);
    e->coef.upload(L.coef, s);  // valid before the first prepare (pin flags)
    e->pin_rhs.upload(L.pin_rhs, s);
    e->staging.alloc(6 * nv);
    e->st.alloc(1);
    PDGB_CUDA_TRY(cudaMemsetAsync(e->prev.p, 0, nv * sizeof(float4), s));
    PDGB_CUDA_TRY(cudaMemsetAsync(e->y.p, 0, nv * sizeof(float4), s));
    PDGB_CUDA_TRY(cudaMemsetAsync(e->st.p, 0, sizeof(StepState), s));
}

// Scalar system K of the engine's vertex order, from the float coefficients
// the kernels use (M/h^2 incl. the pin weight) and the double geometry.
SparseSym engine_system(const HostLayout& L) { return layout_system(L); }

// Solve schedule: the requested one, or by size.  The per-level launches
// (programmatic dependent launch, factor blocks loaded before each wait)
// are fastest from a single 10^3 body up (48 K stored entries: 59 us per
// solve against 68 us for one cluster; 512 bodies: 0.82 ms against 2.4 ms
// for one CTA per body); below 2^15 stored entries the chain of launches
// dominates and one cluster (a single body) or one CTA per body (a batch)
// walks the whole tree instead.
int choose_solve_mode(const pdgb_engine* e) {
    const bool small = (size_t)e->chol.mval_size <= kCtaSolveMaxEntries;
    const int m = e->solve_req;
    if (m == PDGB_SOLVE_DSM && !e->dsm.ok)
        throw Error{PDGB_ERR_UNSUPPORTED, "the factor does not fit the shared memory of one cluster (DSM solve)"};
    if (m != PDGB_SOLVE_AUTO) return m;
    if (!small) return PDGB_SOLVE_LEVELS;
    return e->nbodies > 1 ? PDGB_SOLVE_CTA : PDGB_SOLVE_CLUSTER;
}

void prepare_cholesky(pdgb_engine* e) {
    // the distributed-shared-memory solve stages the factor from host memory
    const int dev = e->solve_req == PDGB_SOLVE_DSM ? PDGB_FACTOR_HOST : e->factor_req;
    if (e->chol_ordering == e->ordering && e->chol_dt == e->prm.dt && e->chol_pw == e->prm.positional_weight &&
        e->chol.n == e->nv && e->factor_dev == dev) {
        e->solve_mode = choose_solve_mode(e);
        return;  // the system matrix depends only on the mesh, dt and the pin weight
    }
    const bool gpu = dev == PDGB_FACTOR_GPU;
    auto t0 = std::chrono::steady_clock::now();
    SparseSym K;
    if (e->nbodies == 1) K = engine_system(e->L);
    std::vector<float> xyz(3 * (size_t)e->nv);
    for (int i = 0; i < e->nv; ++i) {
        xyz[3 * i] = e->L.x0[i].x;
        xyz[3 * i + 1] = e->L.x0[i].y;
        xyz[3 * i + 2] = e->L.x0[i].z;
    }
    if (e->nbodies > 1) {
        std::vector<double> mdt2(e->nv);
        for (int i = 0; i < e->nv; ++i) mdt2[i] = (double)e->L.coef[i].x;
        cholesky_factor_bodies(e->nbodies, e->L.body_ivstart, e->L.body_itstart, e->L.tets_int.data(),
                               e->L.dminv_d.data(), e->L.coef_d.data(), mdt2, e->ordering, xyz.data(), e->chol,
                               gpu);
    } else {
        cholesky_factor(K, e->ordering, xyz.data(), e->chol, kBwdChunkRows, gpu);
    }
    cudaStream_t s = e->stream;
    const CholFactor& f = e->chol;
    e->numeric_ms = 0.0;
    e->pool_bytes = 0;
    if (gpu) {
        // FP64 numeric factorisation on the GPU, straight into the M_s blocks
        e->ch_mval.alloc((size_t)std::max<int64_t>(f.mval_size, 1));
        e->numeric_ms = gpu_factor(f, e->ch_mval.p, s);
        e->pool_bytes = (long long)f.fp.pool * (long long)sizeof(double);
        e->chol.fp = FrontPlan();  // the plan is not needed after the factorisation
    } else {
        e->ch_mval.upload(f.mval, s);
    }
    e->factor_dev = dev;
    e->factor_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    e->ch_fwd.upload(f.fwd_items, s);
    e->ch_bwd.upload(f.bwd_items, s);
    e->ch_fwdb.upload(f.fwd_blocks, s);
    e->ch_bwdb.upload(f.bwd_blocks, s);
    e->ch_fwds.upload(f.fwd_small, s);
    e->ch_bwds.upload(f.bwd_small, s);
    e->ch_tiny.upload(f.tiny, s);
    e->ch_zstage.upload(f.zstage, s);
    e->ch_zbuf.alloc((size_t)std::max<int64_t>(f.zrows, 1));
    e->ch_rows.upload(f.rows, s);
    std::vector<int4> lv(f.levels.size());
    for (size_t i = 0; i < lv.size(); ++i)
        lv[i] = make_int4(f.levels[i].fwd_begin, f.levels[i].fwd_end, f.levels[i].bwd_begin, f.levels[i].bwd_end);
    e->ch_levels.upload(lv, s);
    e->ch_step_lv.upload(f.step_levels, s);
    if (f.K.n == e->nv) {  // FP64 copy of K for refinement residuals (single body)
        std::vector<int> rp(f.K.p.begin(), f.K.p.end());
        e->k_rowptr.upload(rp, s);
        e->k_colind.upload(f.K.i, s);
        e->k_val.upload(f.K.x, s);
        e->bsave.alloc(e->nv);
        e->dx.alloc(e->nv);
    }
    e->ch_body_level.upload(f.body_level, s);
    e->ch_body_order.upload(f.body_order, s);
    e->dsm = DsmPlan{};
    if (e->solve_req == PDGB_SOLVE_DSM) {
        int dev = 0, optin = 0;
        PDGB_CUDA_TRY(cudaGetDevice(&dev));
        PDGB_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        build_dsm_plan(f, kClusterCtas, kClusterSolveThreads / 32, (size_t)optin, e->dsm);
        if (e->dsm.ok) {
            e->dsm_mcopy.upload(e->dsm.mcopy, s);
            e->dsm_mcopy_ptr.upload(e->dsm.mcopy_ptr, s);
            e->dsm_rcopy.upload(e->dsm.rcopy, s);
            e->dsm_rcopy_ptr.upload(e->dsm.rcopy_ptr, s);
            e->dsm_items.upload(e->dsm.items, s);
            e->dsm_lvl.upload(e->dsm.lvl, s);
        }
    }
    e->solve_mode = choose_solve_mode(e);
    e->chol_ordering = e->ordering;
    e->chol_dt = e->prm.dt;
    e->chol_pw = e->prm.positional_weight;
}

void prepare(pdgb_engine* e) {
    auto t0 = std::chrono::steady_clock::now();
    build_vertex_coefficients(e->mass.data(), e->has_dbc ? e->dbc.data() : nullptr, e->prm, e->L);
    e->coef.upload(e->L.coef, e->stream);
    e->pin_rhs.upload(e->L.pin_rhs, e->stream);
    if (e->prm.solver == PDGB_SOLVER_CHOLESKY) prepare_cholesky(e);
    PDGB_CUDA_TRY(cudaMemsetAsync(e->y.p, 0, (size_t)e->nv * sizeof(float4), e->stream));
    // resident CTAs of the pipelined local step for the current tile cut
    // (queried here, not while the step graph is being captured)
    e->pipe_grid = e->local_kernel == PDGB_LOCAL_PIPELINED ? local_pipe_grid(e->L.ntiles, e->L.max_patch) : 0;
    build_graph(e);
    PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->prepared = true;
    e->prepare_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

void pdgb_default_params(pdgb_params* p) {
    if (!p) return;
    p->dt = 1.0f / 120.0f;
    p->gravity = 9.8f;
    p->num_iterations = 10;
    p->tol = 0.0f;
    p->rho = 0.9992f;
    p->positional_weight = 1e6f;
    p->solver = PDGB_SOLVER_JACOBI;
    p->refine_steps = 0;
}

}  // extern "C"

namespace {

int create_impl(const pdgb_mesh_desc* mesh, const pdgb_params* params, void* stream, pdgb_engine** out,
                const std::vector<int>* body_vstart) {
    if (!out) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "out is null");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    pdgb_engine* e = nullptr;
    int st = guarded([&] {
        if (!mesh || !params) throw Error{PDGB_ERR_INVALID_ARGUMENT, "mesh or params is null"};
        if (!mesh->X || !mesh->tets || !mesh->mass || !mesh->mu)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "mesh X, tets, mass and mu are required"};
        if (mesh->memory != PDGB_MEM_HOST && mesh->memory != PDGB_MEM_DEVICE)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "mesh memory must be PDGB_MEM_HOST or PDGB_MEM_DEVICE"};
        if (mesh->num_verts <= 0 || mesh->num_tets <= 0)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "num_verts and num_tets must be positive"};
        if (mesh->num_verts > (1 << 28) || mesh->num_tets > (1 << 28))
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "mesh too large (limit 2^28 vertices / tets)"};
        check_params(*params);
        e = new pdgb_engine();
        e->prm = *params;
        e->nv = mesh->num_verts;
        e->nt = mesh->num_tets;
        if (stream) e->stream = (cudaStream_t)stream;
        else {
            PDGB_CUDA_TRY(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
            e->own_stream = true;
        }
        copy_in(e->X0, mesh->X, 3 * (size_t)e->nv, mesh->memory);
        copy_in(e->tets, mesh->tets, 4 * (size_t)e->nt, mesh->memory);
        copy_in(e->mass, mesh->mass, (size_t)e->nv, mesh->memory);
        copy_in(e->mu, mesh->mu, (size_t)e->nt, mesh->memory);
        e->has_dbc = mesh->dbc != nullptr;
        if (e->has_dbc) copy_in(e->dbc, mesh->dbc, (size_t)e->nv, mesh->memory);
        if (e->has_dbc)
            for (float d : e->dbc) e->num_pinned += d > 0.f;
        if (body_vstart) {
            e->nbodies = (int)body_vstart->size() - 1;
            e->body_vstart = *body_vstart;
        } else {
            e->body_vstart = {0, e->nv};
        }
        build_layout(e->nv, e->nt, e->X0.data(), e->tets.data(), e->mass.data(), e->mu.data(),
                     e->has_dbc ? e->dbc.data() : nullptr, e->prm, e->L, e->nbodies,
                     e->nbodies > 1 ? e->body_vstart.data() : nullptr);
        upload_mesh(e);
        // initial state X (and V) from the descriptor
        std::vector<float> Vh;
        if (mesh->V) copy_in(Vh, mesh->V, 3 * (size_t)e->nv, mesh->memory);
        PDGB_CUDA_TRY(cudaMemcpyAsync(e->staging.p, e->X0.data(), 3 * (size_t)e->nv * sizeof(float),
                                      cudaMemcpyHostToDevice, e->stream));
        if (mesh->V)
            PDGB_CUDA_TRY(cudaMemcpyAsync(e->staging.p + 3 * (size_t)e->nv, Vh.data(),
                                          3 * (size_t)e->nv * sizeof(float), cudaMemcpyHostToDevice, e->stream));
        launch_gather_state(e->nv, e->vperm.p, e->staging.p, mesh->V ? e->staging.p + 3 * (size_t)e->nv : nullptr,
                            e->x.p, e->v.p, e->stream);
        PDGB_CUDA_TRY(cudaGetLastError());
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    });
    if (st != PDGB_OK) {
        delete e;
        return st;
    }
    *out = e;
    return PDGB_OK;
}

}  // namespace

extern "C" {

int pdgb_create(const pdgb_mesh_desc* mesh, const pdgb_params* params, void* stream, pdgb_engine** out) {
    return create_impl(mesh, params, stream, out, nullptr);
}

int pdgb_create_batch(int nbodies, const pdgb_mesh_desc* bodies, const pdgb_params* params, void* stream,
                      pdgb_engine** out) {
    if (!out || !bodies || !params || nbodies < 1) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad batch arguments");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    // concatenate the bodies (host copies), vertex ids offset per body
    std::vector<float> X, V, mass, mu, dbc;
    std::vector<uint32_t> tets;
    std::vector<int> vstart(1, 0);
    bool anyV = false;
    int st = guarded([&] {
        long long nv_tot = 0, nt_tot = 0;
        for (int b = 0; b < nbodies; ++b) {
            const pdgb_mesh_desc& d = bodies[b];
            if (!d.X || !d.tets || !d.mass || !d.mu || d.num_verts <= 0 || d.num_tets <= 0 ||
                (d.memory != PDGB_MEM_HOST && d.memory != PDGB_MEM_DEVICE))
                throw Error{PDGB_ERR_INVALID_ARGUMENT, "body " + std::to_string(b) + ": bad descriptor"};
            nv_tot += d.num_verts;
            nt_tot += d.num_tets;
            anyV = anyV || d.V;
        }
        if (nv_tot > (1 << 28) || nt_tot > (1 << 28)) throw Error{PDGB_ERR_INVALID_ARGUMENT, "batch too large"};
        X.reserve(3 * nv_tot);
        for (int b = 0; b < nbodies; ++b) {
            const pdgb_mesh_desc& d = bodies[b];
            std::vector<float> tmp;
            std::vector<uint32_t> tt;
            copy_in(tmp, d.X, 3 * (size_t)d.num_verts, d.memory);
            X.insert(X.end(), tmp.begin(), tmp.end());
            if (anyV) {
                if (d.V) copy_in(tmp, d.V, 3 * (size_t)d.num_verts, d.memory);
                else tmp.assign(3 * (size_t)d.num_verts, 0.f);
                V.insert(V.end(), tmp.begin(), tmp.end());
            }
            copy_in(tmp, d.mass, (size_t)d.num_verts, d.memory);
            mass.insert(mass.end(), tmp.begin(), tmp.end());
            copy_in(tmp, d.mu, (size_t)d.num_tets, d.memory);
            mu.insert(mu.end(), tmp.begin(), tmp.end());
            if (d.dbc) copy_in(tmp, d.dbc, (size_t)d.num_verts, d.memory);
            else tmp.assign((size_t)d.num_verts, 0.f);
            dbc.insert(dbc.end(), tmp.begin(), tmp.end());
            copy_in(tt, d.tets, 4 * (size_t)d.num_tets, d.memory);
            for (uint32_t& t : tt) {
                if (t >= (uint32_t)d.num_verts)
                    throw Error{PDGB_ERR_BAD_MESH, "body " + std::to_string(b) + ": tet index out of range"};
                t += (uint32_t)vstart.back();
            }
            tets.insert(tets.end(), tt.begin(), tt.end());
            vstart.push_back(vstart.back() + d.num_verts);
        }
    });
    if (st != PDGB_OK) return st;
    pdgb_mesh_desc all{vstart.back(), (int)(tets.size() / 4), X.data(), anyV ? V.data() : nullptr, tets.data(),
                       mass.data(), mu.data(), dbc.data(), PDGB_MEM_HOST};
    return create_impl(&all, params, stream, out, &vstart);
}

int pdgb_num_bodies(pdgb_engine* e) { return e ? e->nbodies : 0; }

int pdgb_download_body(pdgb_engine* e, int body, float* X, float* V, int memory) {
    if (!e || body < 0 || body >= e->nbodies || (!X && !V)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, body or outputs");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        const size_t n3 = 3 * (size_t)e->nv;
        const size_t o = 3 * (size_t)e->body_vstart[body];
        const size_t c = 3 * (size_t)(e->body_vstart[body + 1] - e->body_vstart[body]);
        launch_scatter_state(e->nv, e->vperm.p, e->x.p, e->v.p, e->staging.p, e->staging.p + n3, e->stream);
        const cudaMemcpyKind kind = memory == PDGB_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
        if (X) PDGB_CUDA_TRY(cudaMemcpyAsync(X, e->staging.p + o, c * sizeof(float), kind, e->stream));
        if (V) PDGB_CUDA_TRY(cudaMemcpyAsync(V, e->staging.p + n3 + o, c * sizeof(float), kind, e->stream));
        if (memory == PDGB_MEM_HOST) PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        PDGB_CUDA_TRY(cudaGetLastError());
    });
}

int pdgb_prepare(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] { prepare(e); });
}

int pdgb_step(pdgb_engine* e, int nsteps) {
    if (!e || nsteps < 0) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or nsteps");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        if (!e->prepared) prepare(e);
        if (e->timing && !e->step_ev[0]) {
            PDGB_CUDA_TRY(cudaEventCreate(&e->step_ev[0]));
            PDGB_CUDA_TRY(cudaEventCreate(&e->step_ev[1]));
        }
        for (int k = 0; k < nsteps; ++k) {
            if (e->timing_mode == PDGB_TIMING_STEPS) {
                // events only, no wait: pdgb_read_timing sums the pairs
                while (e->step_pairs.size() < 2 * (e->step_pairs_used + 1)) {
                    cudaEvent_t ev;
                    PDGB_CUDA_TRY(cudaEventCreate(&ev));
                    e->step_pairs.push_back(ev);
                }
                cudaEvent_t* pr = &e->step_pairs[2 * e->step_pairs_used++];
                PDGB_CUDA_TRY(cudaEventRecord(pr[0], e->stream));
                PDGB_CUDA_TRY(cudaGraphLaunch(e->gexec, e->stream));
                if (e->ccd_on) run_collision(e);
                PDGB_CUDA_TRY(cudaEventRecord(pr[1], e->stream));
                continue;
            }
            if (e->timing) PDGB_CUDA_TRY(cudaEventRecord(e->step_ev[0], e->stream));
            PDGB_CUDA_TRY(cudaGraphLaunch(e->gexec, e->stream));
            if (e->ccd_on) run_collision(e);
            if (e->timing) {
                PDGB_CUDA_TRY(cudaEventRecord(e->step_ev[1], e->stream));
                PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
                float ms = 0.f;
                PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, e->step_ev[0], e->step_ev[1]));
                e->step_ms_acc += ms;
                e->steps_timed++;
                for (int i = 0; i < e->prm.num_iterations; ++i) {
                    PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, e->events[2 * i], e->events[2 * i + 1]));
                    e->local_ms_acc += ms;
                    e->local_launches++;
                    if (e->prm.solver == PDGB_SOLVER_CHOLESKY) {
                        PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, e->solve_events[2 * i], e->solve_events[2 * i + 1]));
                        e->solve_ms_acc += ms;
                        e->solves++;
                    }
                }
            }
        }
        e->steps_run += nsteps;
        e->iters_run += (double)nsteps * e->prm.num_iterations;
    });
}

int pdgb_set_solver(pdgb_engine* e, int solver) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        pdgb_params p = e->prm;
        p.solver = solver;
        check_params(p);
        if (p.solver != e->prm.solver) e->prepared = false;
        e->prm = p;
    });
}

int pdgb_set_params(pdgb_engine* e, const pdgb_params* params) {
    if (!e || !params) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        check_params(*params);
        e->prm = *params;
        e->prepared = false;  // coefficients, omegas and the graph depend on them
    });
}

int pdgb_set_ordering(pdgb_engine* e, int ordering) {
    if (!e || (ordering != PDGB_ORDER_AMD && ordering != PDGB_ORDER_ND && ordering != PDGB_ORDER_DENSE)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or ordering");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (ordering != e->ordering) {
        e->ordering = ordering;
        e->prepared = false;
    }
    return PDGB_OK;
}

int pdgb_set_local_kernel(pdgb_engine* e, int kind) {
    if (!e || (kind != PDGB_LOCAL_TILE && kind != PDGB_LOCAL_PIPELINED)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or local-step kind");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (kind != e->local_kernel) {
        e->local_kernel = kind;
        e->prepared = false;  // the step graph holds the local-step launches
    }
    return PDGB_OK;
}

int pdgb_get_local_kernel(pdgb_engine* e, int* kind) {
    if (!e || !kind) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or output");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    *kind = e->local_kernel;
    return PDGB_OK;
}

int pdgb_set_rotation(pdgb_engine* e, int rotation) {
    if (!e || (rotation != PDGB_ROTATION_QUAT && rotation != PDGB_ROTATION_SVD)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or rotation mode");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (rotation != e->rotation) {
        e->rotation = rotation;
        e->prepared = false;
    }
    return PDGB_OK;
}

namespace {
void upload_tiles(pdgb_engine* e) {
    const HostLayout& L = e->L;
    cudaStream_t s = e->stream;
    e->inc_ent.upload(L.inc_ent, s);
    e->inc_end.upload(L.inc_end, s);
    e->tile_tet_ptr.upload(L.tile_tet_ptr, s);
    e->tile_vptr.upload(L.tile_vptr, s);
    e->tile_verts.upload(L.tile_verts, s);
}

void set_tile_cap(pdgb_engine* e, int cap) {
    if (cap == e->L.tile_cap) return;
    PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));  // no step in flight reads the old tiles
    build_tiles(e->L, e->has_dbc ? e->dbc.data() : nullptr, cap);
    upload_tiles(e);
    PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->prepared = false;
}

// Device time of `steps` steps of the current configuration (prepared),
// one warm-up step first.
double time_steps(pdgb_engine* e, int steps) {
    if (!e->prepared) prepare(e);
    cudaEvent_t ev[2];
    PDGB_CUDA_TRY(cudaEventCreate(&ev[0]));
    PDGB_CUDA_TRY(cudaEventCreate(&ev[1]));
    float ms = 0.f;
    try {
        PDGB_CUDA_TRY(cudaGraphLaunch(e->gexec, e->stream));
        PDGB_CUDA_TRY(cudaEventRecord(ev[0], e->stream));
        for (int k = 0; k < steps; ++k) PDGB_CUDA_TRY(cudaGraphLaunch(e->gexec, e->stream));
        PDGB_CUDA_TRY(cudaEventRecord(ev[1], e->stream));
        PDGB_CUDA_TRY(cudaEventSynchronize(ev[1]));
        PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    } catch (...) {
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
        throw;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    return (double)ms / std::max(steps, 1);
}
}  // namespace

int pdgb_time_local(pdgb_engine* e, int launches, double* ms_per_launch) {
    if (!e || launches < 1 || launches > 100000 || !ms_per_launch) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, launch count or output");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        if (!e->prepared) prepare(e);
        // the step prologue fills sn and b from the current state; the local
        // steps then read the same sn every launch (b only accumulates)
        BeginArgs ba = begin_args(e);
        launch_begin(ba, e->stream);
        const LocalArgs la = local_args(e, nullptr);
        const bool jf = e->prm.solver == PDGB_SOLVER_JACOBI;
        launch_local(la, e->L.ntiles, e->L.max_patch, jf, e->rotation, e->stream);  // warm-up
        cudaEvent_t ev[2];
        PDGB_CUDA_TRY(cudaEventCreate(&ev[0]));
        PDGB_CUDA_TRY(cudaEventCreate(&ev[1]));
        float ms = 0.f;
        cudaError_t err = cudaEventRecord(ev[0], e->stream);
        for (int k = 0; k < launches && err == cudaSuccess; ++k) {
            launch_local(la, e->L.ntiles, e->L.max_patch, jf, e->rotation, e->stream);
            err = cudaGetLastError();
        }
        if (err == cudaSuccess) err = cudaEventRecord(ev[1], e->stream);
        if (err == cudaSuccess) err = cudaEventSynchronize(ev[1]);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
        PDGB_CUDA_TRY(err);
        *ms_per_launch = (double)ms / launches;
    });
}

int pdgb_set_tile_size(pdgb_engine* e, int max_tets) {
    if (!e || max_tets < 0 || (max_tets > 0 && (max_tets < 32 || max_tets > kTileTets))) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or tile size (32..512, 0 = default)");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] { set_tile_cap(e, max_tets ? max_tets : kTileTets); });
}

int pdgb_autotune(pdgb_engine* e, int steps, pdgb_tune_report* rep) {
    if (!e || steps < 1 || steps > 1000) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or step count (1..1000)");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        if (!e->prepared) prepare(e);
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        // the simulation state is saved and restored around every trial
        const size_t nv = (size_t)e->nv;
        DBuf<float4> save;
        save.alloc(4 * nv);
        float4* keep[4] = {e->x.p, e->v.p, e->prev.p, e->xt.p};
        auto copy_state = [&](bool restore) {
            for (int k = 0; k < 4; ++k) {
                if (!keep[k]) continue;
                float4* a = save.p + k * nv;
                PDGB_CUDA_TRY(cudaMemcpyAsync(restore ? keep[k] : a, restore ? a : keep[k], nv * sizeof(float4),
                                              cudaMemcpyDeviceToDevice, e->stream));
            }
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        };
        copy_state(false);
        const int cap0 = e->L.tile_cap, req0 = e->solve_req;
        const double t0 = time_steps(e, steps);
        copy_state(true);
        std::vector<int> caps = {kTileTets, kTileTets / 2, kTileTets / 4, kTileTets / 8};
        std::vector<int> modes = {e->solve_req};
        if (e->prm.solver == PDGB_SOLVER_CHOLESKY) {
            modes = {PDGB_SOLVE_CTA, PDGB_SOLVE_CLUSTER, PDGB_SOLVE_LEVELS, PDGB_SOLVE_PERSISTENT};
        }
        // orderings: the current one, and for a small single body on the
        // Cholesky path the one dense supernode (a few wide solve launches)
        std::vector<int> ords = {e->ordering};
        if (e->prm.solver == PDGB_SOLVER_CHOLESKY && e->nbodies == 1 && e->nv <= kDenseTuneMaxVerts &&
            e->ordering != PDGB_ORDER_DENSE)
            ords.push_back(PDGB_ORDER_DENSE);
        const int ord0 = e->ordering;
        double best = t0;
        int best_cap = cap0, best_mode = req0, best_ord = ord0, tried = 1;
        for (int ord : ords) {
            if (ord != e->ordering) {
                e->ordering = ord;
                e->prepared = false;
            }
            for (int cap : caps)
                for (int mode : modes) {
                    set_tile_cap(e, cap);
                    if (mode != e->solve_req) {
                        e->solve_req = mode;
                        e->prepared = false;
                    }
                    const double t = time_steps(e, steps);
                    copy_state(true);
                    ++tried;
                    if (t < best) {
                        best = t;
                        best_cap = cap;
                        best_mode = mode;
                        best_ord = ord;
                    }
                }
        }
        // the pipelined local step at the chosen configuration (and at its
        // natural 512-tet tiles)
        const int lk0 = e->local_kernel;
        int best_lk = lk0;
        if (e->rotation == PDGB_ROTATION_QUAT) {
            e->solve_req = best_mode;
            e->ordering = best_ord;
            const int other = lk0 == PDGB_LOCAL_TILE ? PDGB_LOCAL_PIPELINED : PDGB_LOCAL_TILE;
            std::vector<int> lk_caps = {best_cap};
            if (best_cap != kTileTets) lk_caps.push_back(kTileTets);
            for (int cap : lk_caps) {
                set_tile_cap(e, cap);
                e->local_kernel = other;
                e->prepared = false;
                const double t = time_steps(e, steps);
                copy_state(true);
                ++tried;
                if (t < best) {
                    best = t;
                    best_cap = cap;
                    best_lk = other;
                }
            }
        }
        set_tile_cap(e, best_cap);
        e->solve_req = best_mode;
        e->ordering = best_ord;
        e->local_kernel = best_lk;
        e->prepared = false;
        prepare(e);
        copy_state(true);
        if (rep) {
            rep->tile_tets = best_cap;
            rep->solve_mode = e->prm.solver == PDGB_SOLVER_CHOLESKY ? e->solve_mode : PDGB_SOLVE_AUTO;
            rep->candidates = tried;
            rep->ordering = e->ordering;
            rep->best_ms = best;
            rep->default_ms = t0;
        }
    });
}

int pdgb_set_solve_mode(pdgb_engine* e, int mode) {
    if (!e || mode < PDGB_SOLVE_AUTO || mode > PDGB_SOLVE_PERSISTENT) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or solve mode");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (mode != e->solve_req) {
        e->solve_req = mode;
        e->prepared = false;
    }
    return PDGB_OK;
}

int pdgb_get_solve_mode(pdgb_engine* e, int* mode) {
    if (!e || !mode) return PDGB_ERR_INVALID_ARGUMENT;
    *mode = e->prm.solver == PDGB_SOLVER_CHOLESKY && e->prepared ? e->solve_mode : PDGB_SOLVE_AUTO;
    return PDGB_OK;
}

int pdgb_upload_state(pdgb_engine* e, const float* X, const float* V, int memory) {
    if (!e || !X) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        const size_t n3 = 3 * (size_t)e->nv;
        if (memory == PDGB_MEM_HOST) {
            PDGB_CUDA_TRY(cudaMemcpyAsync(e->staging.p, X, n3 * sizeof(float), cudaMemcpyHostToDevice, e->stream));
            if (V)
                PDGB_CUDA_TRY(
                    cudaMemcpyAsync(e->staging.p + n3, V, n3 * sizeof(float), cudaMemcpyHostToDevice, e->stream));
            launch_gather_state(e->nv, e->vperm.p, e->staging.p, V ? e->staging.p + n3 : nullptr, e->x.p, e->v.p,
                                e->stream);
        } else if (memory == PDGB_MEM_DEVICE) {
            launch_gather_state(e->nv, e->vperm.p, X, V, e->x.p, e->v.p, e->stream);
        } else {
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "bad memory kind"};
        }
        if (e->xt.p) launch_copy_state(e->nv, e->x.p, e->xt.p, e->stream);  // XTilde = X
        clear_nonfinite(e);
        PDGB_CUDA_TRY(cudaGetLastError());
    });
}

int pdgb_download_state(pdgb_engine* e, float* X, float* V, int memory) {
    if (!e || (!X && !V)) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        const size_t n3 = 3 * (size_t)e->nv;
        if (memory == PDGB_MEM_HOST) {
            launch_scatter_state(e->nv, e->vperm.p, e->x.p, e->v.p, X ? e->staging.p : nullptr,
                                 V ? e->staging.p + n3 : nullptr, e->stream);
            if (X) PDGB_CUDA_TRY(cudaMemcpyAsync(X, e->staging.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
            if (V)
                PDGB_CUDA_TRY(
                    cudaMemcpyAsync(V, e->staging.p + n3, n3 * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        } else if (memory == PDGB_MEM_DEVICE) {
            launch_scatter_state(e->nv, e->vperm.p, e->x.p, e->v.p, X, V, e->stream);
        } else {
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "bad memory kind"};
        }
        PDGB_CUDA_TRY(cudaGetLastError());
    });
}

int pdgb_reset(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        launch_copy_x0(e->nv, e->x0.p, e->x.p, e->v.p, e->stream);
        if (e->xt.p) launch_copy_state(e->nv, e->x0.p, e->xt.p, e->stream);
        if (e->drag_w.p) PDGB_CUDA_TRY(cudaMemsetAsync(e->drag_w.p, 0, (size_t)e->nv * sizeof(float), e->stream));
        e->drag_on = false;
        PDGB_CUDA_TRY(cudaMemsetAsync(e->prev.p, 0, (size_t)e->nv * sizeof(float4), e->stream));
        clear_nonfinite(e);
        PDGB_CUDA_TRY(cudaGetLastError());
        e->prepared = false;
        e->steps_run = 0;
        e->iters_run = 0;
    });
}

// ---- drag
namespace {
void ensure_drag(pdgb_engine* e) {
    if (e->drag_w.p) return;
    e->drag_w.alloc(e->nv);
    e->drag_off.alloc(e->nv);
    e->drag_target.alloc(1);
    PDGB_CUDA_TRY(cudaMemsetAsync(e->drag_w.p, 0, (size_t)e->nv * sizeof(float), e->stream));
    PDGB_CUDA_TRY(cudaMemsetAsync(e->drag_off.p, 0, (size_t)e->nv * sizeof(float4), e->stream));
    PDGB_CUDA_TRY(cudaMemsetAsync(e->drag_target.p, 0, sizeof(float4), e->stream));
}

void enable_drag(pdgb_engine* e) {
    if (!e->drag_on) {
        e->drag_on = true;
        e->prepared = false;  // the step graph gains the drag terms
    }
}
}  // namespace

int pdgb_set_drag(pdgb_engine* e, const float* weights, const float* offsets, int memory) {
    if (!e || !weights || (memory != PDGB_MEM_HOST && memory != PDGB_MEM_DEVICE)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, weights or memory kind");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        const size_t nv = (size_t)e->nv;
        std::vector<float> w, off;
        copy_in(w, weights, nv, memory);
        if (offsets) copy_in(off, offsets, 3 * nv, memory);
        for (size_t i = 0; i < nv; ++i) {
            if (!std::isfinite(w[i])) throw Error{PDGB_ERR_NONFINITE, "drag weight is not finite"};
            if (w[i] > 0.f && e->has_dbc && e->dbc[i] > 0.f)
                throw Error{PDGB_ERR_INVALID_ARGUMENT, "drag weight on pinned vertex " + std::to_string(i)};
        }
        ensure_drag(e);
        // host copies are staged through the engine's transfer buffer
        PDGB_CUDA_TRY(cudaMemcpyAsync(e->staging.p, w.data(), nv * sizeof(float), cudaMemcpyHostToDevice, e->stream));
        if (offsets)
            PDGB_CUDA_TRY(cudaMemcpyAsync(e->staging.p + nv, off.data(), 3 * nv * sizeof(float), cudaMemcpyHostToDevice,
                                          e->stream));
        launch_gather_drag(e->nv, e->vperm.p, e->staging.p, offsets ? e->staging.p + nv : nullptr, e->drag_w.p,
                           e->drag_off.p, e->stream);
        PDGB_CUDA_TRY(cudaGetLastError());
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));  // w / off leave scope
        enable_drag(e);
    });
}

int pdgb_drag_select(pdgb_engine* e, int select_v, float control_mag, double radius_sq) {
    if (!e || select_v < -1 || select_v >= (e ? e->nv : 0) || !(control_mag >= 0.f)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, vertex or control magnitude");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        ensure_drag(e);
        const int sel = select_v < 0 ? -1 : e->L.viperm[select_v];
        launch_drag_select(e->nv, e->x.p, e->coef.p, sel, control_mag, radius_sq, e->drag_w.p, e->drag_off.p,
                           e->stream);
        PDGB_CUDA_TRY(cudaGetLastError());
        enable_drag(e);
    });
}

int pdgb_set_drag_target(pdgb_engine* e, const float target[3]) {
    if (!e || !target) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        ensure_drag(e);
        const float4 t = make_float4(target[0], target[1], target[2], 0.f);
        // pageable source: the call returns once the 16 bytes are staged
        PDGB_CUDA_TRY(cudaMemcpyAsync(e->drag_target.p, &t, sizeof(t), cudaMemcpyHostToDevice, e->stream));
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    });
}

int pdgb_clear_drag(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        if (e->drag_w.p) PDGB_CUDA_TRY(cudaMemsetAsync(e->drag_w.p, 0, (size_t)e->nv * sizeof(float), e->stream));
        if (e->drag_on) {
            e->drag_on = false;
            e->prepared = false;
        }
    });
}

// ---- fixed rigid bodies
int pdgb_set_fixed_bodies(pdgb_engine* e, const pdgb_fixed_body* bodies, int n, float mu_t, float mu_n) {
    if (!e || n < 0 || (n > 0 && !bodies) || n > 4096 || !std::isfinite(mu_t) || !std::isfinite(mu_n)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, body list or friction coefficients");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        std::vector<FixedBodyDev> dev;
        for (int kind : {PDGB_FIXED_SPHERE, PDGB_FIXED_PLANE, PDGB_FIXED_CYLINDER})
            for (int j = 0; j < n; ++j) {
                const pdgb_fixed_body& fb = bodies[j];
                if (fb.type < PDGB_FIXED_SPHERE || fb.type > PDGB_FIXED_CYLINDER)
                    throw Error{PDGB_ERR_INVALID_ARGUMENT, "unknown fixed body type"};
                for (float m : fb.model)
                    if (!std::isfinite(m)) throw Error{PDGB_ERR_NONFINITE, "fixed body model is not finite"};
                if (fb.type != kind) continue;
                FixedBodyDev d{};
                d.p = make_float4(fb.model[12], fb.model[13], fb.model[14], fb.radius);
                if (kind == PDGB_FIXED_PLANE) {
                    d.n = make_float4(fb.up[0], fb.up[1], fb.up[2], (float)kFixedPlane);
                } else if (kind == PDGB_FIXED_CYLINDER) {
                    // normalize(vec3(model * vec4(0, 1, 0, 0))), fixedBodyData.cu:116
                    const float ax = fb.model[4], ay = fb.model[5], az = fb.model[6];
                    const float inv = 1.0f / std::sqrt(ax * ax + ay * ay + az * az);
                    d.n = make_float4(ax * inv, ay * inv, az * inv, (float)kFixedCylinder);
                } else {
                    d.n = make_float4(0.f, 0.f, 0.f, (float)kFixedSphere);
                }
                dev.push_back(d);
            }
        if (n > 0 && !e->xt.p) {  // XTilde starts as X
            e->xt.alloc(e->nv);
            launch_copy_state(e->nv, e->x.p, e->xt.p, e->stream);
            PDGB_CUDA_TRY(cudaGetLastError());
        }
        if (!dev.empty()) e->fixed.upload(dev, e->stream);
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        e->nfixed = (int)dev.size();
        e->mu_t = mu_t;
        e->mu_n = mu_n;
        e->prepared = false;  // body count and friction are graph parameters
    });
}

int pdgb_download_xtilde(pdgb_engine* e, float* XT, int memory) {
    if (!e || !XT) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        const float4* src = e->xt.p ? e->xt.p : e->x.p;
        const size_t n3 = 3 * (size_t)e->nv;
        if (memory == PDGB_MEM_HOST) {
            launch_scatter_state(e->nv, e->vperm.p, src, nullptr, e->staging.p, nullptr, e->stream);
            PDGB_CUDA_TRY(cudaMemcpyAsync(XT, e->staging.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        } else if (memory == PDGB_MEM_DEVICE) {
            launch_scatter_state(e->nv, e->vperm.p, src, nullptr, XT, nullptr, e->stream);
        } else {
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "bad memory kind"};
        }
        PDGB_CUDA_TRY(cudaGetLastError());
    });
}

int pdgb_set_collision_surface(pdgb_engine* e, const uint32_t* tris, const int* tri_body, int num_tris) {
    if (!e || num_tris < 0 || (num_tris > 0 && !tris)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or triangle list");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        std::vector<int> body(num_tris, 0);
        for (int t = 0; t < num_tris; ++t) {
            if (tri_body) {
                body[t] = tri_body[t];
            } else {
                const uint32_t v = tris[3 * (size_t)t];
                if (v < (uint32_t)e->nv && e->nbodies > 1)
                    body[t] = (int)(std::upper_bound(e->body_vstart.begin(), e->body_vstart.end(), (int)v) -
                                    e->body_vstart.begin()) - 1;
            }
        }
        const CcdSurface surf = build_ccd_surface(e->nv, num_tris, tris, body.data(), e->L.viperm.data());
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        e->ccd.reset(new CcdContext(surf, e->vperm.p, e->stream));
    });
}

int pdgb_enable_collision(pdgb_engine* e, int on) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        if (on && !e->ccd) throw Error{PDGB_ERR_INVALID_ARGUMENT, "no collision surface set"};
        if (on && !e->xt.p) {  // XTilde starts as X
            e->xt.alloc(e->nv);
            launch_copy_state(e->nv, e->x.p, e->xt.p, e->stream);
            PDGB_CUDA_TRY(cudaGetLastError());
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        }
        if ((on != 0) != e->ccd_on) {
            e->ccd_on = on != 0;
            e->prepared = false;  // the step epilogue changes
        }
    });
}

int pdgb_get_collision(pdgb_engine* e, float* tI, float* normals, pdgb_collision_info* info) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        if (!e->ccd) throw Error{PDGB_ERR_INVALID_ARGUMENT, "no collision surface set"};
        const size_t nv = e->nv;
        if (tI || normals) {
            std::vector<float> t(nv);
            std::vector<float4> n(nv);
            PDGB_CUDA_TRY(cudaMemcpyAsync(t.data(), e->ccd->tI(), nv * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
            PDGB_CUDA_TRY(cudaMemcpyAsync(n.data(), e->ccd->normals(), nv * sizeof(float4), cudaMemcpyDeviceToHost,
                                          e->stream));
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
            for (size_t i = 0; i < nv; ++i) {
                const size_t o = (size_t)e->L.vperm[i];
                if (tI) tI[o] = t[i];
                if (normals) {
                    normals[3 * o] = n[i].x;
                    normals[3 * o + 1] = n[i].y;
                    normals[3 * o + 2] = n[i].z;
                }
            }
        }
        if (info) {
            const CcdStats& st = e->ccd->stats();
            info->candidate_pairs = st.pairs;
            info->vertices_hit = st.marked;
            info->regrows = st.regrows;
            info->detect_ms = st.ms;
        }
    });
}

int pdgb_ccd_detect(int num_verts, int num_tris, const uint32_t* tris, const int* tri_body, const float* X,
                    const float* XT, float* tI, float* normals, pdgb_collision_info* info) {
    if (num_verts <= 0 || num_tris < 0 || !X || !XT || !tI || !normals || (num_tris > 0 && (!tris || !tri_body))) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad sizes or null arrays");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        const size_t nv = num_verts;
        for (size_t i = 0; i < 3 * nv; ++i)
            if (!std::isfinite(X[i]) || !std::isfinite(XT[i])) throw Error{PDGB_ERR_NONFINITE, "non-finite position"};
        const CcdSurface surf = build_ccd_surface(num_verts, num_tris, tris, tri_body, nullptr);
        std::vector<float4> h(2 * nv);
        for (size_t i = 0; i < nv; ++i) {
            h[i] = make_float4(X[3 * i], X[3 * i + 1], X[3 * i + 2], 0.f);
            h[nv + i] = make_float4(XT[3 * i], XT[3 * i + 1], XT[3 * i + 2], 0.f);
        }
        DBuf<float4> d;
        d.upload(h, nullptr);
        CcdContext ctx(surf, nullptr, nullptr);
        ctx.detect(d.p, d.p + nv);
        std::vector<float4> n(nv);
        PDGB_CUDA_TRY(cudaMemcpyAsync(tI, ctx.tI(), nv * sizeof(float), cudaMemcpyDeviceToHost, nullptr));
        PDGB_CUDA_TRY(cudaMemcpyAsync(n.data(), ctx.normals(), nv * sizeof(float4), cudaMemcpyDeviceToHost, nullptr));
        PDGB_CUDA_TRY(cudaStreamSynchronize(nullptr));
        for (size_t i = 0; i < nv; ++i) {
            normals[3 * i] = n[i].x;
            normals[3 * i + 1] = n[i].y;
            normals[3 * i + 2] = n[i].z;
        }
        if (info) {
            info->candidate_pairs = ctx.stats().pairs;
            info->vertices_hit = ctx.stats().marked;
            info->regrows = ctx.stats().regrows;
            info->detect_ms = ctx.stats().ms;
        }
    });
}

int pdgb_render_surface(pdgb_engine* e, const uint32_t* tris, int num_tris, float* tri_pos, float* tri_nor) {
    if (!e || num_tris < 0 || (num_tris > 0 && (!tris || !tri_pos || !tri_nor))) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine, triangles or output buffers");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        if (!e->viperm.p) e->viperm.upload(e->L.viperm, e->stream);
        launch_render_surface(num_tris, tris, e->viperm.p, e->nv, e->x.p, tri_pos, tri_nor, e->stream);
        PDGB_CUDA_TRY(cudaGetLastError());
    });
}

int pdgb_get_perf(pdgb_engine* e, pdgb_perf* out) {
    if (!e || !out) return PDGB_ERR_INVALID_ARGUMENT;
    out->prepare_ms = e->prepare_ms;
    out->steps = e->steps_run;
    out->iterations = e->iters_run;
    out->factor_nnz = e->prm.solver == PDGB_SOLVER_CHOLESKY ? e->chol.nnz_L : 0;
    out->tiles = e->L.ntiles;
    out->patch_verts = (long long)e->L.tile_vptr.back();
    return PDGB_OK;
}

int pdgb_last_step_iterations(pdgb_engine* e, int* iterations) {
    if (!e || !iterations) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        if (e->prm.solver != PDGB_SOLVER_CHOLESKY) {
            *iterations = e->prm.num_iterations;
            return;
        }
        StepState h{};
        PDGB_CUDA_TRY(cudaMemcpyAsync(&h, e->st.p, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
        *iterations = h.iterations;
    });
}

int pdgb_synchronize(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] { PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream)); });
}

int pdgb_last_step_status(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    int flag[2] = {0, 0};  // nonfinite, local_timeout
    GridSync bar{};
    const int st = guarded([&] {
        PDGB_CUDA_TRY(cudaMemcpyAsync(flag, &e->st.p->nonfinite, 2 * sizeof(int), cudaMemcpyDeviceToHost, e->stream));
        PDGB_CUDA_TRY(cudaMemcpyAsync(&bar, &e->st.p->bar, sizeof(GridSync), cudaMemcpyDeviceToHost, e->stream));
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    });
    if (st != PDGB_OK) return st;
    if (bar.timeout) {
        set_last_error(PDGB_ERR_TIMEOUT, "a grid-barrier wait of the persistent solve ran out of its bound");
        return PDGB_ERR_TIMEOUT;
    }
    if (flag[1]) {
        set_last_error(PDGB_ERR_TIMEOUT, "a bulk-copy wait of the pipelined local step ran out of its bound");
        return PDGB_ERR_TIMEOUT;
    }
    if (flag[0]) {
        set_last_error(PDGB_ERR_NONFINITE, "a step ended with a non-finite position or velocity");
        return PDGB_ERR_NONFINITE;
    }
    return PDGB_OK;
}

int pdgb_enable_kernel_timing(pdgb_engine* e, int mode) {
    if (!e || mode < PDGB_TIMING_OFF || mode > PDGB_TIMING_KERNELS) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or timing mode");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    const bool kernels = mode == PDGB_TIMING_KERNELS;
    if (kernels != e->timing) {
        e->timing = kernels;
        e->prepared = false;  // the graph gains or loses the per-local events
    }
    e->timing_mode = mode;
    e->local_ms_acc = e->step_ms_acc = e->solve_ms_acc = 0.0;
    e->local_launches = e->steps_timed = e->solves = 0;
    e->step_pairs_used = 0;
    return PDGB_OK;
}

int pdgb_read_timing(pdgb_engine* e, pdgb_timing* out) {
    if (!e || !out) return PDGB_ERR_INVALID_ARGUMENT;
    if (e->step_pairs_used) {
        int st = guarded([&] {
            PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
            for (size_t k = 0; k < e->step_pairs_used; ++k) {
                float ms = 0.f;
                PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, e->step_pairs[2 * k], e->step_pairs[2 * k + 1]));
                e->step_ms_acc += ms;
            }
            e->steps_timed += (long long)e->step_pairs_used;
        });
        e->step_pairs_used = 0;
        if (st != PDGB_OK) return st;
    }
    out->step_ms = e->step_ms_acc;
    out->steps = e->steps_timed;
    out->local_ms = e->local_ms_acc;
    out->local_launches = e->local_launches;
    out->solve_ms = e->solve_ms_acc;
    out->solves = e->solves;
    e->local_ms_acc = e->step_ms_acc = e->solve_ms_acc = 0.0;
    e->local_launches = e->steps_timed = e->solves = 0;
    return PDGB_OK;
}

int pdgb_local_step_bytes(pdgb_engine* e, double* bytes) {
    if (!e || !bytes) return PDGB_ERR_INVALID_ARGUMENT;
    // per tet: 4 x u32 corner ids + 9 x f32 DmInv + 1 x f32 V0*w = 56 B;
    // per vertex: read q (12 B), read (M/h^2) s (12 B), write b (12 B) = 36 B.
    *bytes = 56.0 * e->nt + 36.0 * e->nv;
    return PDGB_OK;
}

int pdgb_solve_bytes(pdgb_engine* e, double* bytes) {
    if (!e || !bytes) return PDGB_ERR_INVALID_ARGUMENT;
    *bytes = 0.0;
    if (e->prm.solver != PDGB_SOLVER_CHOLESKY || e->chol.n != e->nv) return PDGB_OK;
    // forward + backward: factor values and row indices (4 B + 4 B per
    // nonzero of the scalar L) and column pointers, plus the 3-column
    // right-hand sides: read b 12 n, write and read y 24 n, write x 12 n
    const double n = (double)e->nv, nnz = (double)e->chol.nnz_L;
    *bytes = 2.0 * (8.0 * nnz + 4.0 * (n + 1.0)) + 48.0 * n;
    return PDGB_OK;
}

int pdgb_destroy(pdgb_engine* e) {
    if (!e) return PDGB_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(e->stream);
    delete e;
    return PDGB_OK;
}

void* pdgb_stream(pdgb_engine* e) { return e ? (void*)e->stream : nullptr; }

const char* pdgb_status_string(int status) {
    switch (status) {
        case PDGB_OK: return "ok";
        case PDGB_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PDGB_ERR_BAD_MESH: return "bad mesh";
        case PDGB_ERR_NOT_SPD: return "system matrix not positive definite";
        case PDGB_ERR_CUDA: return "CUDA error";
        case PDGB_ERR_OUT_OF_MEMORY: return "out of memory";
        case PDGB_ERR_NONFINITE: return "non-finite value";
        case PDGB_ERR_UNSUPPORTED: return "unsupported";
        case PDGB_ERR_TIMEOUT: return "device wait timed out";
        case PDGB_ERR_NOT_FOUND: return "not found";
        case PDGB_ERR_BUSY: return "busy";
        default: return "unknown status";
    }
}

const char* pdgb_last_error(void) { return g_last_error.c_str(); }

int pdgb_inspect_layout(const pdgb_mesh_desc* mesh, pdgb_layout_info* info, int* vperm, int* tperm) {
    if (!mesh || !info || mesh->memory != PDGB_MEM_HOST || !mesh->X || !mesh->tets || !mesh->mass || !mesh->mu) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "host mesh with X, tets, mass, mu required");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        pdgb_params p;
        pdgb_default_params(&p);
        HostLayout L;
        build_layout(mesh->num_verts, mesh->num_tets, mesh->X, mesh->tets, mesh->mass, mesh->mu, mesh->dbc, p, L);
        info->num_tiles = L.ntiles;
        info->patch_verts = (long long)L.tile_vptr.back();
        info->max_patch = 0;
        info->max_tile_tets = 0;
        info->reserved = 0;
        for (int t = 0; t < L.ntiles; ++t) {
            info->max_patch = std::max(info->max_patch, L.tile_vptr[t + 1] - L.tile_vptr[t]);
            info->max_tile_tets = std::max(info->max_tile_tets, L.tile_tet_ptr[t + 1] - L.tile_tet_ptr[t]);
        }
        if (vperm) std::copy(L.vperm.begin(), L.vperm.end(), vperm);
        if (tperm) std::copy(L.tperm.begin(), L.tperm.end(), tperm);
    });
}

namespace {
// Kernel launches of one solve in the schedule in use.
int solve_launches(const pdgb_engine* e) {
    if (e->solve_mode != PDGB_SOLVE_LEVELS) return 1;  // PERSISTENT: one launch (and a barrier reset)
    int n = 0;
    for (const SolveLevel& v : e->chol.step_levels) {
        const int fb = v.fwdb_end - v.fwdb_begin, fw = v.fwdw_end - v.fwdw_begin;
        const int bb = v.bwdb_end - v.bwdb_begin, bw = v.bwdw_end - v.bwdw_begin;
        n += mix_level(fb, fw) ? 1 : (fb > 0) + (fw > 0);
        n += mix_level(bb, bw) ? 1 : (bb > 0) + (bw > 0);
        n += 2 * (v.tiny_end > v.tiny_begin) + (v.zst_end > v.zst_begin);
    }
    return n;
}
}  // namespace

int pdgb_get_factor_info(pdgb_engine* e, pdgb_factor_info* info) {
    if (!e || !info) return PDGB_ERR_INVALID_ARGUMENT;
    std::memset(info, 0, sizeof(*info));
    if (e->prm.solver != PDGB_SOLVER_CHOLESKY || e->chol.n != e->nv) return PDGB_OK;
    const CholFactor& f = e->chol;
    info->nnz_L = f.nnz_L;
    info->m_entries = (long long)f.mval_size;
    info->num_supernodes = f.nsuper;
    info->num_levels = f.nlevels;
    info->fwd_items = (int)(f.fwd_items.size() / kItemInts);
    info->bwd_items = (int)(f.bwd_items.size() / kItemInts);
    info->flops = f.flops;
    info->factor_ms = e->factor_ms;
    info->solve_launches = solve_launches(e);
    info->numeric_device = e->factor_dev;
    info->numeric_ms = e->numeric_ms;
    info->pool_bytes = e->pool_bytes;
    return PDGB_OK;
}

int pdgb_set_factor_device(pdgb_engine* e, int device) {
    if (!e || (device != PDGB_FACTOR_GPU && device != PDGB_FACTOR_HOST)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad engine or factor device");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (device != e->factor_req) {
        e->factor_req = device;
        e->prepared = false;
    }
    return PDGB_OK;
}

int pdgb_get_factor_blocks(pdgb_engine* e, float* out, long long capacity) {
    if (!e || !out || capacity < 0) return PDGB_ERR_INVALID_ARGUMENT;
    return guarded([&] {
        if (e->prm.solver != PDGB_SOLVER_CHOLESKY || e->chol.n != e->nv || !e->ch_mval.p)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "no prepared Cholesky factor"};
        const long long n = (long long)e->chol.mval_size;
        if (capacity < n) throw Error{PDGB_ERR_INVALID_ARGUMENT, "capacity below the factor's m_entries"};
        PDGB_CUDA_TRY(cudaMemcpyAsync(out, e->ch_mval.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
        PDGB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    });
}

int pdgb_host_factor_check(const pdgb_mesh_desc* mesh, const pdgb_params* params, int ordering, const double* b,
                           double* x, pdgb_factor_info* info) {
    if (!mesh || !params || mesh->memory != PDGB_MEM_HOST || !mesh->X || !mesh->tets || !mesh->mass || !mesh->mu) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "host mesh with X, tets, mass, mu and params required");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        check_params(*params);
        HostLayout L;
        build_layout(mesh->num_verts, mesh->num_tets, mesh->X, mesh->tets, mesh->mass, mesh->mu, mesh->dbc, *params,
                     L);
        auto t0 = std::chrono::steady_clock::now();
        SparseSym K = engine_system(L);
        std::vector<float> xyz(3 * (size_t)L.nv);
        for (int i = 0; i < L.nv; ++i) {
            xyz[3 * i] = L.x0[i].x;
            xyz[3 * i + 1] = L.x0[i].y;
            xyz[3 * i + 2] = L.x0[i].z;
        }
        CholFactor f;
        cholesky_factor(K, ordering, xyz.data(), f);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (info) {
            info->nnz_L = f.nnz_L;
            info->m_entries = (long long)f.mval_size;
            info->num_supernodes = f.nsuper;
            info->num_levels = f.nlevels;
            info->fwd_items = (int)(f.fwd_items.size() / kItemInts);
            info->bwd_items = (int)(f.bwd_items.size() / kItemInts);
            info->flops = f.flops;
            info->factor_ms = ms;
            info->solve_launches = 0;
            info->numeric_device = PDGB_FACTOR_HOST;
            info->numeric_ms = 0.0;
            info->pool_bytes = 0;
        }
        if (b && x) {
            const int nv = L.nv;
            std::vector<double> bi(3 * (size_t)nv), xi(3 * (size_t)nv);
            for (int i = 0; i < nv; ++i)
                for (int d = 0; d < 3; ++d) bi[3 * (size_t)i + d] = b[3 * (size_t)L.vperm[i] + d];
            cholesky_solve_host(f, bi.data(), xi.data());
            for (int i = 0; i < nv; ++i)
                for (int d = 0; d < 3; ++d) x[3 * (size_t)L.vperm[i] + d] = xi[3 * (size_t)i + d];
        }
    });
}

int pdgb_closest_rotations(int n, const float* F, float* R, int rotation) {
    if (n < 0 || (n > 0 && (!F || !R)) || (rotation != PDGB_ROTATION_QUAT && rotation != PDGB_ROTATION_SVD)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad count, arrays or rotation mode");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PDGB_OK;
    return guarded([&] {
        DBuf<float> dF, dR;
        dF.alloc(9 * (size_t)n);
        dR.alloc(9 * (size_t)n);
        PDGB_CUDA_TRY(cudaMemcpy(dF.p, F, 9 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
        launch_rotations(n, dF.p, dR.p, rotation, nullptr);
        PDGB_CUDA_TRY(cudaGetLastError());
        PDGB_CUDA_TRY(cudaMemcpy(R, dR.p, 9 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

int pdgb_grid_sync_check(int ctas, int rounds, int missing, long long spin_limit) {
    if (ctas < 0 || rounds < 1 || rounds > 1000 || missing < 0 || spin_limit < 1) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad barrier check arguments");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    GridSync h{};
    const int st = guarded([&] {
        DBuf<GridSync> bar;
        bar.alloc(1);
        launch_grid_sync_check(bar.p, ctas ? ctas : persistent_grid(), rounds, missing, spin_limit, nullptr);
        PDGB_CUDA_TRY(cudaGetLastError());
        PDGB_CUDA_TRY(cudaMemcpy(&h, bar.p, sizeof(GridSync), cudaMemcpyDeviceToHost));
    });
    if (st != PDGB_OK) return st;
    if (h.timeout) {
        set_last_error(PDGB_ERR_TIMEOUT, "grid barrier wait ran out of its bound");
        return PDGB_ERR_TIMEOUT;
    }
    return PDGB_OK;
}

int pdgb_bulk_wait_check(int extra_bytes, long long limit_ns) {
    if (extra_bytes < 0 || extra_bytes % 16 || extra_bytes > 4096 || limit_ns < 1000000 || limit_ns > 2000000000ll) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad bulk-wait check arguments");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    int h[2] = {0, 0};
    const int st = guarded([&] {
        std::vector<uint32_t> words(64);
        for (int k = 0; k < 64; ++k) words[k] = (uint32_t)k;
        DBuf<uint32_t> src;
        DBuf<int> out;
        src.alloc(64);
        out.alloc(2);
        PDGB_CUDA_TRY(cudaMemcpy(src.p, words.data(), 64 * sizeof(uint32_t), cudaMemcpyHostToDevice));
        PDGB_CUDA_TRY(cudaMemset(out.p, 0, 2 * sizeof(int)));
        launch_bulk_wait_check(src.p, extra_bytes, (unsigned long long)limit_ns, out.p, nullptr);
        PDGB_CUDA_TRY(cudaGetLastError());
        PDGB_CUDA_TRY(cudaMemcpy(h, out.p, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    });
    if (st != PDGB_OK) return st;
    if (h[0]) {
        set_last_error(PDGB_ERR_TIMEOUT, "bulk-copy wait ran out of its bound");
        return PDGB_ERR_TIMEOUT;
    }
    if (!h[1]) {
        set_last_error(PDGB_ERR_CUDA, "bulk copy completed with wrong data");
        return PDGB_ERR_CUDA;
    }
    return PDGB_OK;
}

const char* pdgb_version(void) { return "pdgb 0.2 (sm_103a)"; }

}  // extern "C"
