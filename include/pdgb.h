/*
 * pdgb — GB300-native projective-dynamics (PD) step engine, C ABI.
 *
 * Drop-in replacement for the float PD path of the reference simulator
 * (GrahamZen/Soft-Body-Simulation-CUDA).  Each entry point names the
 * reference interface it replaces (paths inside the reference project):
 *
 *   Solver<float> / FEMSolver<float>   src/simulation/solver/solver.h:11-28,
 *                                      src/simulation/solver/femSolver.h:5-15
 *   PdSolver                           src/simulation/solver/projective/pdSolver.h:12-44
 *   SolverData<float>, SolverParams    src/def.h:21-56, 82-100
 *
 * Conventions
 *   - Every function returns an int status (PDGB_OK = 0 on success); no C++
 *     exception crosses this boundary.  pdgb_last_error() gives a message
 *     for the most recent failure on the calling host thread.
 *   - Vertex vectors are float[3*num_verts], xyz interleaved (the layout of
 *     glm::vec3 arrays in SolverData).  Tets are uint32[4*num_tets].
 *   - `memory` arguments say whether a pointer is host (PDGB_MEM_HOST) or
 *     device (PDGB_MEM_DEVICE) memory.
 *   - Work is ordered on the engine's CUDA stream.  pdgb_step() does not
 *     synchronise the host; pdgb_download_state() to host memory does.
 *   - One engine per host thread at a time; engines are independent.
 */
#ifndef PDGB_H_
#define PDGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define PDGB_OK 0
#define PDGB_ERR_INVALID_ARGUMENT 1 /* null pointer, bad size, bad enum        */
#define PDGB_ERR_BAD_MESH 2         /* tet index out of range, degenerate tet  */
#define PDGB_ERR_NOT_SPD 3          /* system matrix not positive definite     */
#define PDGB_ERR_CUDA 4             /* a CUDA runtime call failed              */
#define PDGB_ERR_OUT_OF_MEMORY 5    /* device allocation or HBM budget failed  */
#define PDGB_ERR_NONFINITE 6        /* NaN/Inf detected in the state           */
#define PDGB_ERR_UNSUPPORTED 7      /* feature not available for this config   */
#define PDGB_ERR_TIMEOUT 8          /* a bounded device-side wait gave up      */
#define PDGB_ERR_NOT_FOUND 9        /* unknown request / body id               */
#define PDGB_ERR_BUSY 10            /* admission refused (capacity), retry     */

#define PDGB_MEM_HOST 0
#define PDGB_MEM_DEVICE 1

/* Global solver choice.  Mirrors PdSolver::SolverType {Jacobi,
 * CuSolverCholesky, EigenCholesky} (pdSolver.h:14-17); both Cholesky forms
 * map to the engine's own prefactored sparse Cholesky. */
#define PDGB_SOLVER_JACOBI 0
#define PDGB_SOLVER_CHOLESKY 1

/* Mirrors SolverParams<float> (def.h:82-100) for the fields PD reads, plus the
 * pin weight (PdSolver::positional_weight, pdSolver.h:31) and the engine's
 * refinement count. */
typedef struct pdgb_params {
    float dt;                /* time step h (SolverParams::dt)                  */
    float gravity;           /* g > 0, along -y (SolverParams::gravity)         */
    int num_iterations;      /* local/global iterations per step                */
    float tol;               /* Cholesky early exit: stop when sqrt(mean squared
                                change) < tol (pdSolver.cu:164); 0 = never    */
    float rho;               /* Chebyshev spectral radius (SolverParams::rho)   */
    float positional_weight; /* pin weight, reference value 1e6                  */
    int solver;              /* PDGB_SOLVER_*                                    */
    int refine_steps;        /* Cholesky: FP64-residual refinement steps 0..3   */
} pdgb_params;

/* Fills *p with the reference defaults (SolverParams<float> defaults with
 * positional_weight 1e6, Jacobi, 10 iterations, dt 1/120). */
void pdgb_default_params(pdgb_params* p);

/* One soft-body system: the arrays SolverData<float> holds for PD. */
typedef struct pdgb_mesh_desc {
    int num_verts;
    int num_tets;
    const float* X;       /* [3*nv] positions; also the rest shape X0/DBCX    */
    const float* V;       /* [3*nv] velocities or NULL (zero)                 */
    const uint32_t* tets; /* [4*nt] vertex indices (SolverData::Tet)          */
    const float* mass;    /* [nv] per-vertex mass (SolverData::mass)          */
    const float* mu;      /* [nt] per-tet PD weight (SolverData::mu)          */
    const float* dbc;     /* [nv] pin flags 0/1 or NULL (SolverData::DBC)      */
    int memory;           /* PDGB_MEM_HOST or PDGB_MEM_DEVICE, for all above   */
} pdgb_mesh_desc;

typedef struct pdgb_engine pdgb_engine;

/* Per-phase timing, mirrors Solver::GetPerformanceData() (solver.h:19). */
typedef struct pdgb_perf {
    double prepare_ms;       /* last SolverPrepare equivalent (host + device)   */
    double steps;            /* steps run since create/reset                    */
    double iterations;       /* local/global iterations run                     */
    long long factor_nnz;    /* nnz of the scalar Cholesky factor (0: Jacobi)   */
    long long tiles;         /* tet tiles of the local-step kernel              */
    long long patch_verts;   /* sum of tile patch sizes                         */
} pdgb_perf;

/* Replaces PdSolver(int threadsPerBlock, const SolverData<float>&)
 * (pdSolver.cu:22-27, femSolver.cu:7-17).  Copies the mesh; the caller's
 * arrays may be freed afterwards.  stream: a cudaStream_t or NULL for a
 * stream the engine creates. */
int pdgb_create(const pdgb_mesh_desc* mesh, const pdgb_params* params, void* stream, pdgb_engine** out);

/* Batch of independent soft bodies advanced together (the reference's own
 * multi-body mode concatenates bodies into one system,
 * dataLoader.cu:291-378).  Vertices of body b are caller ids
 * sum_{i<b} nv_i .. + nv_b in pdgb_upload_state / pdgb_download_state.  Per
 * step: one local-step launch over the tiles of all bodies and, on the
 * Cholesky path, one solve launch with one CTA per body (each body has its own
 * factor, largest first).  The early-exit tolerance applies to single-body
 * engines only; batches run num_iterations iterations. */
int pdgb_create_batch(int nbodies, const pdgb_mesh_desc* bodies, const pdgb_params* params, void* stream,
                      pdgb_engine** out);
int pdgb_num_bodies(pdgb_engine* e);
/* State of one body of a batch (caller layout, nv_b x 3 floats each). */
int pdgb_download_body(pdgb_engine* e, int body, float* X, float* V, int memory);

/* ---------------------------------------------------------------------
 * Serving: a request loop with continuous batching (no counterpart in the
 * reference, which advances one scene per frame).  Requests are soft bodies
 * with a step count, submitted at any time.  Host threads prepare each
 * request's layout (and, on the Cholesky path, the ordering and symbolic
 * analysis of its system); pdgb_server_tick admits ready requests in
 * arrival order while their device memory fits hbm_budget_bytes (and
 * max_active), runs ONE PD step (the shared params: Jacobi + Chebyshev, or
 * the prefactored Cholesky solve with num_iterations iterations) for every
 * active request with one set of launches, and retires finished requests
 * (state copied to host memory, device memory returned to the server).  On
 * the Cholesky path every request's FP64 factor is computed on the GPU at
 * admission and stays resident with its mesh and state; the per-level solve
 * launches cover level L of every active request's elimination tree.  A
 * request's arithmetic is that of a single engine, so its result does not
 * depend on the other requests in the mix.  A request whose state leaves the
 * finite range fails (PDGB_ERR_NONFINITE from pdgb_server_result). */
typedef struct pdgb_server_config {
    pdgb_params params;       /* shared solver parameters                     */
    size_t hbm_budget_bytes;  /* device bytes of resident requests           */
    int max_active;           /* slot limit, 0 = budget only                  */
    int host_threads;         /* layout workers, 0 = half the host cores      */
    int cache_entries;        /* meshes whose layout (and factor) are kept    */
                              /* for resubmission: 0 = 256, < 0 = no cache    */
    int reserved;
} pdgb_server_config;

#define PDGB_REQ_QUEUED 0
#define PDGB_REQ_PREPARING 1
#define PDGB_REQ_READY 2
#define PDGB_REQ_RUNNING 3
#define PDGB_REQ_DONE 4
#define PDGB_REQ_FAILED 5

typedef struct pdgb_server_stats {
    long long completed;
    long long failed;
    int active;               /* requests resident and stepping              */
    int waiting;              /* submitted, not yet admitted                  */
    size_t bytes_in_use;
    double tet_iterations;    /* sum over steps run of tets x iterations      */
    double busy_ms;           /* host time spent inside pdgb_server_tick      */
    double admit_ms;          /* of which admission (allocation, uploads)     */
    double step_ms;           /* of which stepping: launch to step complete   */
    long long ticks;          /* ticks that ran a step                        */
    int ready;                /* prepared, waiting for admission              */
    int layout_cache_hits;    /* requests that reused a cached host layout    */
    long long nonfinite;      /* failed requests whose state became non-finite */
    long long factors;        /* numeric factorisations run on the GPU         */
    long long factor_cache_hits; /* admissions that reused a cached factor     */
    double factor_ms;         /* device time of those factorisations           */
    int finishing;            /* stepped to their count, results handed out   */
                              /* by the next tick                              */
    int reserved;
} pdgb_server_stats;

typedef struct pdgb_server pdgb_server;
void pdgb_server_default_config(pdgb_server_config* cfg);
int pdgb_server_create(const pdgb_server_config* cfg, void* stream, pdgb_server** out);
/* Copies the host mesh; returns the request id.  Host layouts (and, on the
 * Cholesky path, the symbolic and numeric factors) are cached by mesh
 * content (the last cache_entries distinct meshes): a mesh submitted again
 * skips the layout build and the factorisation. */
int pdgb_server_submit(pdgb_server* s, const pdgb_mesh_desc* mesh, int nsteps, long long* request_id);
/* One tick: waits for the step launched by the previous tick and hands out
 * the requests it finished, admits ready requests, launches one step of
 * every active request and, while it runs, admits more and prepares the
 * next step's work lists; it returns without waiting for its step.  active
 * / completed (nullable): requests resident after the tick, requests handed
 * out by it.  Keep calling it while requests are active, waiting or
 * finishing (pdgb_server_stats). */
int pdgb_server_tick(pdgb_server* s, int* active, int* completed);
int pdgb_server_poll(pdgb_server* s, long long request_id, int* state, int* steps_done);
/* Final state of a finished request (caller layout); releases the request. */
int pdgb_server_result(pdgb_server* s, long long request_id, float* X, float* V);
int pdgb_server_get_stats(pdgb_server* s, pdgb_server_stats* out);
/* Submit-to-finish latencies of all completed requests, in ms. */
int pdgb_server_latencies(pdgb_server* s, double* out_ms, int capacity, int* count);
int pdgb_server_destroy(pdgb_server* s);

/* Replaces PdSolver::SolverPrepare (pdSolver.cu:40-139): per-tet DmInv/V0,
 * system assembly, ordering and factorisation, step graph.  pdgb_step calls
 * it on first use, as PdSolver::Update does (pdSolver.cu:212-216). */
int pdgb_prepare(pdgb_engine* e);

/* Replaces nsteps calls of PdSolver::Update (pdSolver.cu:210-232) without
 * collision handling: s_n, local/global iterations, velocity/position update,
 * X <- XTilde. */
int pdgb_step(pdgb_engine* e, int nsteps);

/* Replaces PdSolver::SetGlobalSolver (pdSolver.h:20).  Takes effect at the
 * next prepare (a changed solver forces one). */
int pdgb_set_solver(pdgb_engine* e, int solver);

/* Updates dt/gravity/iterations/tol/rho/pin weight/refinement.  A change of
 * dt, pin weight or solver re-prepares on the next step. */
int pdgb_set_params(pdgb_engine* e, const pdgb_params* params);

/* State transfer in the reference layout (SolverData::X / V). */
int pdgb_upload_state(pdgb_engine* e, const float* X, const float* V, int memory);
int pdgb_download_state(pdgb_engine* e, float* X, float* V, int memory);

/* Replaces SimulationCUDAContext::Reset + Solver::Reset
 * (simulationContext.cu:233-243, solver.h:40-43): X = X0, V = 0, re-prepare. */
int pdgb_reset(pdgb_engine* e);

int pdgb_get_perf(pdgb_engine* e, pdgb_perf* out);

/* Per-iteration convergence record of the last step (Cholesky path): the
 * number of iterations run (early exit on tol).  Synchronises. */
int pdgb_last_step_iterations(pdgb_engine* e, int* iterations);

/* Waits for the engine's stream. */
int pdgb_synchronize(pdgb_engine* e);

/* Status of the steps run since the state was last set (pdgb_create,
 * pdgb_upload_state, pdgb_reset): PDGB_ERR_NONFINITE once any step has ended
 * with a non-finite position or velocity (the iteration left the finite
 * range), else PDGB_OK.  The step epilogue sets a device word; this call
 * waits for the stream and reads it.  The reference reports nothing here
 * (SolverStep returns true unconditionally, pdSolver.cu:207).  With the
 * PERSISTENT solve schedule or the PIPELINED local step, PDGB_ERR_TIMEOUT
 * when a grid-barrier or bulk-copy wait ran out of its bound (the steps
 * since then are invalid). */
int pdgb_last_step_status(pdgb_engine* e);

/* Check of the persistent solve's grid barrier on its own (no counterpart
 * in the reference): one cooperative launch of `ctas` CTAs (0: the solve's
 * grid) passes `rounds` barriers, each waiting for `missing` more arrivals
 * than there are CTAs.  With missing = 0 every barrier completes (PDGB_OK);
 * with missing > 0 no barrier can complete and every wait gives up after
 * spin_limit polls (PDGB_ERR_TIMEOUT) -- the kernel returns, the context
 * stays usable.  Waits for the GPU. */
int pdgb_grid_sync_check(int ctas, int rounds, int missing, long long spin_limit);

/* Check of the pipelined local step's bounded bulk-copy wait on its own (no
 * counterpart in the reference): one CTA bulk-copies 256 bytes into shared
 * memory on an mbarrier that expects 256 + extra_bytes (a multiple of 16).
 * With extra_bytes = 0 the copy completes the phase and the wait returns
 * (PDGB_OK, data checked); with extra_bytes > 0 the phase cannot complete and
 * the wait gives up after limit_ns nanoseconds, 1e6..2e9 (PDGB_ERR_TIMEOUT) --
 * the copy itself has landed, the kernel returns, the context stays usable.
 * Waits for the GPU. */
int pdgb_bulk_wait_check(int extra_bytes, long long limit_ns);

/* Device timing for benchmarks (mode, default OFF):
 *   PDGB_TIMING_STEPS: pdgb_step brackets every step-graph launch with a
 *     pair of CUDA events on the engine's stream and does not wait;
 *     pdgb_read_timing waits for the stream and sums the pairs.
 *   PDGB_TIMING_KERNELS: additionally brackets every local-step kernel
 *     inside the graph (event nodes, which add a little time to the step)
 *     and waits for each step.
 * pdgb_read_timing returns the sums since the last read and clears them.
 * With timing off pdgb_step never waits. */
#define PDGB_TIMING_OFF 0
#define PDGB_TIMING_STEPS 1
#define PDGB_TIMING_KERNELS 2
typedef struct pdgb_timing {
    double step_ms;          /* summed device time of the step graphs          */
    long long steps;         /* steps timed                                     */
    double local_ms;         /* summed device time of the local-step launches   */
    long long local_launches;
    double solve_ms;         /* Cholesky path: summed device time of the solves */
    long long solves;
} pdgb_timing;
int pdgb_enable_kernel_timing(pdgb_engine* e, int mode);
int pdgb_read_timing(pdgb_engine* e, pdgb_timing* out);

/* Algorithmic bytes of one local-step launch (inputs read once, outputs
 * written once; see the roofline section of the design notes). */
int pdgb_local_step_bytes(pdgb_engine* e, double* bytes);
/* Algorithmic bytes of one Cholesky solve (forward + backward): factor
 * values and row indices of the scalar L (8 B per nonzero), column pointers,
 * and the 3-column right-hand sides; 0 on the Jacobi path or before the
 * first prepare. */
int pdgb_solve_bytes(pdgb_engine* e, double* bytes);

int pdgb_destroy(pdgb_engine* e);

/* Returns the CUDA stream (cudaStream_t) the engine orders its work on. */
void* pdgb_stream(pdgb_engine* e);

const char* pdgb_status_string(int status);
const char* pdgb_last_error(void);

/* Host-only inspection of the engine's data layout for a mesh (no GPU
 * needed): the Morton vertex/tet renumbering and the local-step tiles.
 * vperm/tperm (nullable) receive internal -> caller maps of length nv / nt. */
typedef struct pdgb_layout_info {
    int num_tiles;          /* CTAs of one local-step launch                   */
    int max_patch;          /* largest tile vertex patch (<= 1024)             */
    int max_tile_tets;      /* largest tile                                    */
    int reserved;
    long long patch_verts;  /* sum of patch sizes (vertex reuse = nv*4/this)   */
} pdgb_layout_info;
int pdgb_inspect_layout(const pdgb_mesh_desc* mesh, pdgb_layout_info* info, int* vperm, int* tperm);

/* Ordering of the Cholesky factor (default AMD, as the reference's
 * cusolverSpXcsrsymamdHost, cholesky.cu:88-91).  PDGB_ORDER_DENSE keeps
 * the AMD order but stores the factor as one dense supernode (all n pivots,
 * n^2 FP32 entries of L^-1): the solve is then a few wide dense launches
 * instead of one launch per tree level, which pays off for small single
 * bodies (the autotuner tries it up to 4096 vertices).  Takes effect at the
 * next prepare. */
#define PDGB_ORDER_AMD 0
#define PDGB_ORDER_ND 1 /* geometric nested dissection */
#define PDGB_ORDER_DENSE 2
int pdgb_set_ordering(pdgb_engine* e, int ordering);

/* Rotation of the local step.  QUAT (default): the closest proper rotation
 * from the dominant eigenvector of Horn's 4x4 quaternion matrix, converged to
 * float precision.  SVD: the reference's scheme -- 4 approximate-Givens
 * Jacobi sweeps of a McAdams-style 3x3 SVD, R = U V^T (svd.cuh:7-14,
 * pdUtil.cu:113-122) -- which is not fully converged on stretched elements. */
#define PDGB_ROTATION_QUAT 0
#define PDGB_ROTATION_SVD 1
int pdgb_set_rotation(pdgb_engine* e, int rotation);

/* Form of the local step (reference: PdUtil::computeLocal, pdUtil.cu:97-145;
 * same arithmetic and result in both).  TILE (default): one CTA per tile of
 * up to 512 tets, four CTAs per SM, the tile's geometry loaded at its start.
 * PIPELINED: four persistent CTAs per SM walk the tiles; while one tile is
 * computed, the next tile's patch list and the geometry of its first 256
 * tets are bulk-copied into shared memory (on the 64^3 cube it measures
 * slower than TILE, whose independent CTAs already overlap one another's
 * loads); pdgb_autotune tries it.  A bulk-copy wait that runs out of its
 * bound (1 s) makes pdgb_last_step_status return PDGB_ERR_TIMEOUT.  The SVD
 * rotation always uses TILE.  Takes effect at the next step. */
#define PDGB_LOCAL_TILE 0
#define PDGB_LOCAL_PIPELINED 1
int pdgb_set_local_kernel(pdgb_engine* e, int kind);
int pdgb_get_local_kernel(pdgb_engine* e, int* kind);

/* Schedule of the Cholesky solve.  CTA: one CTA per body walks the body's
 * whole elimination tree (levels separated by block barriers); CLUSTER: one
 * cluster of 8 CTAs per body (cluster barriers); LEVELS: one launch per
 * level and direction over the whole GPU, level L of every body of a batch
 * in the same launch (levels counted from the leaves); DSM: a single body
 * whose factor fits the shared memory of an 8-CTA cluster is solved by that
 * cluster with the factor blocks, row lists and vectors on chip
 * (distributed shared memory between the CTAs; PDGB_ERR_UNSUPPORTED at
 * prepare when it does not fit; on request only: with whole supernodes
 * per CTA and remote float atomics it measures slower than CLUSTER on the
 * bodies that fit); PERSISTENT: the whole solve (every body of a batch) in
 * one cooperative launch over the GPU, the levels of LEVELS separated by a
 * grid-wide barrier whose waits are bounded (a wait that runs out sets a
 * status word: pdgb_last_step_status then returns PDGB_ERR_TIMEOUT).  AUTO
 * picks by size: LEVELS from 2^15 stored factor entries up, below that
 * CLUSTER for a single system and CTA for a batch; pdgb_autotune times CTA,
 * CLUSTER, LEVELS and PERSISTENT.  Takes
 * effect at the next prepare; pdgb_get_solve_mode returns the schedule in
 * use (AUTO before the first prepare or on the Jacobi path). */
#define PDGB_SOLVE_AUTO 0
#define PDGB_SOLVE_CTA 1
#define PDGB_SOLVE_CLUSTER 2
#define PDGB_SOLVE_LEVELS 3
#define PDGB_SOLVE_DSM 4
#define PDGB_SOLVE_PERSISTENT 5
int pdgb_set_solve_mode(pdgb_engine* e, int mode);
int pdgb_get_solve_mode(pdgb_engine* e, int* mode);

/* Average device time of `launches` back-to-back local-step launches on
 * the current state (the step prologue runs first; the state X, V is not
 * changed).  For benchmarking the local step alone.  Waits for the GPU. */
int pdgb_time_local(pdgb_engine* e, int launches, double* ms_per_launch);

/* Tiles of the local step: at most max_tets tets each (32..512; 0 = 512).
 * Smaller tiles give small meshes more CTAs; vertex and tet order are
 * unchanged, so the state carries over.  Takes effect at the next step. */
int pdgb_set_tile_size(pdgb_engine* e, int max_tets);

/* Autotuner: times `steps` steps (after one warm-up step) of every
 * candidate configuration on the engine's own mesh -- tile sizes 512, 256,
 * 128, 64 and, on the Cholesky path, the solve schedules CTA and CLUSTER
 * (and LEVELS for a single system) -- keeps the fastest and leaves the
 * engine prepared with it.  The simulation state is restored after every
 * trial, so tuning does not advance the simulation.  Waits for the GPU. */
typedef struct pdgb_tune_report {
    int tile_tets;       /* chosen most tets per tile                        */
    int solve_mode;      /* chosen PDGB_SOLVE_* (AUTO on the Jacobi path)    */
    int candidates;      /* configurations timed                             */
    int ordering;        /* chosen PDGB_ORDER_* (Cholesky path)              */
    double best_ms;      /* device time per step, chosen configuration       */
    double default_ms;   /* device time per step before tuning               */
} pdgb_tune_report;
int pdgb_autotune(pdgb_engine* e, int steps, pdgb_tune_report* report);

/* Host-only check of the Cholesky factor for a mesh (no GPU needed): builds
 * the system for params (dt, pin weight), orders and factors it, and applies
 * the factor on the host exactly as the GPU solve does (double):
 * x = K^-1 b for 3 interleaved right-hand sides in caller vertex order. */
typedef struct pdgb_factor_info {
    long long nnz_L;        /* nonzeros of the scalar factor                  */
    long long m_entries;    /* stored FP32 entries of the M_s blocks          */
    int num_supernodes;
    int num_levels;         /* levels of the supernodal elimination tree     */
    int fwd_items;          /* GPU work items, forward pass                   */
    int bwd_items;          /* GPU work items, backward pass                  */
    double flops;           /* factorisation flops (approx.)                  */
    double factor_ms;       /* wall time of ordering + symbolic analysis +    */
                            /* numeric factorisation                          */
    int solve_launches;     /* kernel launches of one solve, current schedule */
    int numeric_device;     /* where the numeric factorisation ran:           */
                            /* PDGB_FACTOR_GPU or PDGB_FACTOR_HOST            */
    double numeric_ms;      /* device time of the GPU numeric factorisation   */
    long long pool_bytes;   /* FP64 front pool of the GPU factorisation       */
} pdgb_factor_info;
/* Factor statistics of a prepared engine on the Cholesky path (zeros
 * otherwise). */
int pdgb_get_factor_info(pdgb_engine* e, pdgb_factor_info* info);

/* Where the one-time numeric factorisation of the system runs.  The
 * reference factors on the GPU in FP32 (cusolverSpScsrcholFactor,
 * cholesky.cu:152-157).  PDGB_FACTOR_GPU (default): FP64 supernodal
 * multifrontal factorisation with the engine's own kernels, level by level
 * of the elimination tree; PDGB_FACTOR_HOST: the same factorisation in FP64
 * on the host (OpenMP).  The ordering and symbolic analysis run on the host
 * in both.  The distributed-shared-memory solve (PDGB_SOLVE_DSM) stages the
 * factor from host memory and always uses the host factorisation.  Takes
 * effect at the next prepare. */
#define PDGB_FACTOR_GPU 0
#define PDGB_FACTOR_HOST 1
int pdgb_set_factor_device(pdgb_engine* e, int device);

/* Copies the FP32 M_s blocks of the prepared factor (m_entries floats, see
 * pdgb_factor_info) to host memory; capacity in floats.  Waits for the
 * stream. */
int pdgb_get_factor_blocks(pdgb_engine* e, float* out, long long capacity);

int pdgb_host_factor_check(const pdgb_mesh_desc* mesh, const pdgb_params* params, int ordering, const double* b,
                           double* x, pdgb_factor_info* info);

/* ---------------------------------------------------------------------
 * Interactive drag (soft positional constraints).  The reference keeps a
 * per-vertex weight moreDBC, an offset OffsetX and one mouse target in
 * SolverData (def.h:16-18, 30-33) and applies them inside
 * PdSolver::SolverStep (pdUtil.cu:56-95, 147-166, 180-205): a dragged vertex
 * (weight w > 0) starts each step at target + offset, its mass term becomes
 * (m + w)/h^2, it keeps that position through the Jacobi iterations, its
 * RHS row becomes (target + offset) * w when the system has pinned vertices
 * (the reference runs that overwrite only then), and its velocity is set to
 * 0 at the end of the step.  The system matrix is not refactored.
 *
 * pdgb_set_drag: weights (float[nv]) and offsets (float[3 nv], nullable:
 * keep the current ones), caller vertex order.  A weight > 0 on a pinned
 * vertex is rejected (PDGB_ERR_INVALID_ARGUMENT): the reference's selection
 * never sets one.
 * pdgb_drag_select: the reference's selection (Control_Kernel,
 * simulationContext.cu:201-231) on the current positions: every free vertex
 * gets offset X_i - X_select, and weight control_mag if |offset|^2 <
 * radius_sq (the reference uses 10 and 0.002); select_v = -1 clears the
 * weights.  select_v is a caller vertex index.
 * pdgb_set_drag_target: the mouse target (mouseSelection.target).
 * pdgb_clear_drag: all weights 0 and the drag terms leave the step graph
 * (ResetMoreDBC(true), simulationContext.cu:220-226; pdgb_reset does it
 * too). */
int pdgb_set_drag(pdgb_engine* e, const float* weights, const float* offsets, int memory);
int pdgb_drag_select(pdgb_engine* e, int select_v, float control_mag, double radius_sq);
int pdgb_set_drag_target(pdgb_engine* e, const float target[3]);
int pdgb_clear_drag(pdgb_engine* e);

/* ---------------------------------------------------------------------
 * Fixed rigid bodies (FixedBodyData, fixedBodyData.cu:8-148).  After every
 * step the engine projects XTilde out of each body and resolves the
 * velocity with friction muT and restitution muN, spheres first, then
 * planes, then cylinders, as FixedBodyData::HandleCollisions does, fused
 * into the step's last kernel.  As in PdSolver::Update (pdSolver.cu:
 * 218-232) X is copied from XTilde before the correction: X (what
 * pdgb_download_state returns) holds the uncorrected positions and the next
 * step starts from it, while the velocity update uses XTilde.
 *
 * A body is given as the reference's FixedBody fields: model is m_model
 * (glm::mat4, column-major, 16 floats), radius is m_radius (sphere,
 * cylinder), up is Plane::m_floorUp (plane only).  The cylinder axis is the
 * normalised second column of model.  n = 0 removes all bodies.  The
 * bodies and muT / muN apply from the next step. */
#define PDGB_FIXED_SPHERE 0
#define PDGB_FIXED_PLANE 1
#define PDGB_FIXED_CYLINDER 2
typedef struct pdgb_fixed_body {
    int type;         /* PDGB_FIXED_*                                      */
    float model[16];  /* column-major 4x4 model matrix                     */
    float radius;
    float up[3];
} pdgb_fixed_body;
int pdgb_set_fixed_bodies(pdgb_engine* e, const pdgb_fixed_body* bodies, int n, float mu_t, float mu_n);
/* SolverData::XTilde after the last step (equals X without fixed bodies). */
int pdgb_download_xtilde(pdgb_engine* e, float* XT, int memory);

/* ---------------------------------------------------------------------
 * Continuous collision between bodies.  Replaces the reference's
 * CollisionDetection::DetectCollision(..., ignoreSelfCollision = true) +
 * CCDKernel that PdSolver::Update runs after each step when collision
 * handling is on (src/simulation/solver/projective/pdSolver.cu:218-224;
 * src/collision/bvh.cu:153-165, broadphase.cu, narrowphase.cu,
 * intersections.cu:286-334; src/simulation/collisionUtil.cu:50-70):
 *   - candidates: surface triangles of different bodies that share no
 *     vertex and whose swept boxes (X -> XTilde) overlap (GPU LBVH);
 *   - per pair, both ways: 3 point-face and 9 edge-edge continuous tests
 *     (coplanarity cubic, proximity 1e-6, barycentric slack 1e-3);
 *   - per vertex / per edge the earliest contact; every vertex of such a
 *     contact before t = 1 gets tI = 0.5 and the normal of the earliest
 *     contact touching it (the reference lets these writes race);
 *   - response: tI < 1 -> X is kept and V = -(d . n) n with
 *     d = XTilde - X (a displacement, as in the reference); else X = XTilde.
 *     The fixed-body correction of XTilde and V follows (pdSolver.cu:228).
 * Triangles are caller vertex ids (3 per triangle); tri_body gives each
 * triangle's body (NULL: the body of its first vertex, from the engine's
 * body ranges).  Detection waits for the stream once per step (the
 * candidate count sizes the narrow phase, as in the reference). */
typedef struct pdgb_collision_info {
    long long candidate_pairs;  /* triangle pairs tested by the last detection */
    int vertices_hit;           /* vertices with tI < 1 after it               */
    int regrows;                /* candidate-buffer enlargements so far        */
    double detect_ms;           /* device time of the last detection           */
} pdgb_collision_info;
int pdgb_set_collision_surface(pdgb_engine* e, const uint32_t* tris, const int* tri_body, int num_tris);
/* on != 0: every step runs detection + response (needs a surface). */
int pdgb_enable_collision(pdgb_engine* e, int on);
/* tI [nv], normals [3 nv] (host, caller order, nullable) and statistics of
 * the last detection. */
int pdgb_get_collision(pdgb_engine* e, float* tI, float* normals, pdgb_collision_info* info);
/* One detection on host arrays, no engine: X (start) and XT (end) [3 nv];
 * outputs tI [nv] and normals [3 nv] (zero where tI = 1).  Uses the current
 * CUDA device and its default stream. */
int pdgb_ccd_detect(int num_verts, int num_tris, const uint32_t* tris, const int* tri_body, const float* X,
                    const float* XT, float* tI, float* normals, pdgb_collision_info* info);

/* ---------------------------------------------------------------------
 * Tet-mesh files (host only, no GPU needed).  Replaces the reference's
 * DataLoader::CollectData for one soft body (src/simulation/dataLoader.cu:
 * 38-290; Gmsh reader src/simulation/MshLoader.cpp):
 *   - TetGen: node_file + ele_file (+ optional face_file).  The .node's
 *     first line holds the vertex count, each following "id x y z ..." line
 *     the next vertex; .ele / .face lines "id a b c [d] ..." hold corner ids
 *     minus start_index (the scene file's "start index"; -1 = the first
 *     .node id).  centralize subtracts the centroid and swaps y and z.
 *     Without faces the surface is extracted from the tets (faces used by
 *     exactly one tet, ascending by sorted corners, oriented as the tet
 *     lists them).  '#' comments and blank lines are skipped.
 *   - Gmsh 2.0-2.2, ASCII or binary: msh_file (used when node_file is NULL
 *     or empty); its tetrahedra (type 4, corner nodes of type 11); no
 *     centring and no surface, as in the reference.
 *   - placement: X <- translate(pos) * scale(scale) * rotX * rotY * rotZ * X,
 *     angles in degrees (dataLoader.cu:209-217).
 * The result owns its arrays (malloc); free it with pdgb_free_tet_mesh.
 * Edges are the distinct surface-triangle edges, ascending. */
typedef struct pdgb_body_file {
    const char* node_file;
    const char* ele_file;
    const char* face_file;
    const char* msh_file;
    float pos[3];
    float scale[3];
    float rot[3];
    int centralize;
    int start_index;
} pdgb_body_file;

typedef struct pdgb_tet_mesh {
    int num_verts;
    int num_tets;
    int num_tris;
    int num_edges;
    float* X;          /* [3 num_verts], placed                          */
    uint32_t* tets;    /* [4 num_tets]                                   */
    uint32_t* tris;    /* [3 num_tris] surface triangles                 */
    uint32_t* edges;   /* [2 num_edges]                                  */
} pdgb_tet_mesh;
int pdgb_load_body_file(const pdgb_body_file* file, pdgb_tet_mesh** out);
void pdgb_free_tet_mesh(pdgb_tet_mesh* mesh);
/* Surface triangles of a tet list (the extraction above); capacity in
 * triangles.  num_tris receives the count even when capacity is short
 * (then PDGB_ERR_INVALID_ARGUMENT). */
int pdgb_surface_triangles(int num_tets, const uint32_t* tets, uint32_t* tris, long long capacity, int* num_tris);

/* Render-side positions and normals of a triangle surface, written to
 * device buffers in place of the reference's OpenGL vertex buffers
 * (PopulateTriPos + RecalculateNormals, utilities.cu:93-107, 147-183, run
 * by SimulationCUDAContext::PrepareRenderData, simulationContext.cu:
 * 245-257).  tris (device, uint32[3 n], caller vertex ids) index the
 * engine's current X.  tri_pos (device, float[9 n]) receives per triangle
 * X[t0], X[t2], X[t1]; tri_nor (device, float[12 n]) the face normal
 * cross(p1 - p0, p2 - p0), normalised when its squared length exceeds
 * 1e-12, w = 0, once per corner.  Stream-ordered, no synchronisation. */
int pdgb_render_surface(pdgb_engine* e, const uint32_t* tris, int num_tris, float* tri_pos, float* tri_nor);

/* ---------------------------------------------------------------------
 * Allocation-free PD steps.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory when they advance a body -- a
 * host application whose own allocator owns the GPU's memory, a frame loop
 * where cudaMalloc/cudaFree would stall the device, or a plugin that is only
 * handed device pointers to the simulation arrays.
 *
 * pdgb_step_noalloc runs nsteps Jacobi + Chebyshev PD steps (the same
 * iteration as pdgb_step with PDGB_SOLVER_JACOBI) on caller-owned device
 * arrays, updating X and V (device, float[3 nv], in place).  It calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch is one
 * fixed device array of about 8 MB inside this library, held by every GPU
 * that loads it until the process exits.
 *   - Limits: num_verts <= 32768 and num_tets <= 131072, else
 *     PDGB_ERR_UNSUPPORTED.  The mesh is checked on the device before the
 *     first step: a tet with an out-of-range index, a zero or nearly zero
 *     rest volume (a DmInv that float cannot hold) or a negative or
 *     non-finite weight gives PDGB_ERR_BAD_MESH, and X and V are left as
 *     they were.
 *   - All calls share that scratch array: calls that overlap on the GPU
 *     (other streams, other host threads) race; serialise them.  Each call
 *     recomputes or clears everything it reads from the scratch.
 *   - The first call on a device looks up the scratch's device address for
 *     that device.  The address is kept until the process exits: a
 *     cudaDeviceReset between calls is not supported.
 *   - The call waits for its stream twice: after the mesh check and before
 *     returning.  So no call can be captured into a CUDA graph: call it on
 *     a stream that is not capturing. */
typedef struct pdgb_noalloc_mesh {
    int num_verts;
    int num_tets;
    const uint32_t* tets; /* device [4 nt]                                 */
    const float* X0;      /* device [3 nv] rest shape and pin targets      */
    const float* mass;    /* device [nv]                                   */
    const float* mu;      /* device [nt] PD weight                         */
    const float* dbc;     /* device [nv] pin flags, or NULL                */
} pdgb_noalloc_mesh;
int pdgb_step_noalloc(const pdgb_noalloc_mesh* mesh, const pdgb_params* params, float* X, float* V, int nsteps,
                      void* stream);

/* The local step's rotation on n row-major 3x3 matrices F (host arrays,
 * 9 floats each): R = the closest proper rotation as the engine computes it
 * (PDGB_ROTATION_QUAT or _SVD), for checking the rotation on its own.
 * Waits for the GPU. */
int pdgb_closest_rotations(int n, const float* F, float* R, int rotation);

/* Library version string. */
const char* pdgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PDGB_H_ */
