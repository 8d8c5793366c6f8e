/*
 * CPU oracle for the projective-dynamics (PD) step: TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker for the GPU engine.  Only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py load it.
 * The engine never links, calls or falls back to it.
 *
 * It restates, in plain C++, the float PD step of the reference solver:
 *   - per-tet precompute          src/simulation/solver/solverUtil.cuh:108-138
 *   - system assembly K, diag     src/simulation/solver/projective/pdUtil.cu:9-54
 *   - step prologue (s_n, b)      pdUtil.cu:56-95, 168-179; pdSolver.cu:154-163
 *   - local projection + scatter  pdUtil.cu:97-145 (rotation via SVD, svd.cuh:7-14)
 *   - pinned-vertex RHS overwrite pdUtil.cu:147-166
 *   - global solve, Jacobi +
 *     Chebyshev                    pdUtil.cu:195-226, pdSolver.cu:193-200
 *   - global solve, Cholesky +
 *     error-based early exit       pdSolver.cu:186-191, 243-253
 *   - velocity/position update     pdUtil.cu:180-193, pdSolver.cu:218-227
 * (line numbers refer to files of the reference project).
 *
 * Two arithmetic modes:
 *   64: every quantity in double, rotation = exact closest proper rotation
 *       (cyclic Jacobi on F^T F to convergence), global solve exact (sparse
 *       LL^T in double).  This is the accuracy reference ("FP64 oracle").
 *   32: float arithmetic in the reference's operation order, rotation by a
 *       McAdams-style approximate-Givens SVD (4 sweeps), Cholesky factor in
 *       double stored and applied in float.  This is the CPU baseline.
 *
 * The sparse factor orders unknowns by geometric nested dissection (its own
 * ordering, independent of the engine's AMD) and factors with an up-looking
 * simplicial LL^T.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    float dt;                 /* time step h */
    float gravity;            /* g > 0, acts along -y */
    int num_iterations;       /* local/global iterations per step */
    float tol;                /* Cholesky early-exit tolerance on sqrt(mean sq change) */
    float rho;                /* Chebyshev spectral radius estimate */
    float positional_weight;  /* pin weight (reference: 1e6) */
    int solver;               /* 0 = Jacobi + Chebyshev, 1 = Cholesky */
    int reserved;
} orc_params;

/* Runs nsteps PD steps.  X0 = rest/pin positions, X/V = state (in/out).
 * precision: 32 or 64.  nthreads: OpenMP threads (0 = default).  iters_out
 * (nullable) receives the iteration count of every step; step_seconds
 * (nullable) the wall time of the steps, set-up excluded.  Returns 0 on
 * success, <0 on bad input / non-SPD system. */
int orc_simulate(int nv, int nt, const float* X0, float* X, float* V,
                 const uint32_t* tets, const float* mass, const float* mu,
                 const float* dbc, const orc_params* p, int precision,
                 int nsteps, int nthreads, int* iters_out, double* step_seconds);

/* Scene terms of a step: interactive drag (SolverData moreDBC / OffsetX /
 * mouseSelection.target, def.h:16-33; applied in pdUtil.cu:56-95, 147-205)
 * and fixed rigid bodies (fixedBodyData.cu:66-148, applied after each step
 * to XTilde and V, pdSolver.cu:218-232).  Body fields are the reference's
 * FixedBody members: model = m_model (glm column-major), radius = m_radius,
 * up = Plane::m_floorUp.  type: 0 sphere, 1 plane, 2 cylinder. */
typedef struct orc_fixed_body {
    int type;
    float model[16];
    float radius;
    float up[3];
} orc_fixed_body;

typedef struct orc_scene {
    const float* drag_w;    /* [nv] drag weights (moreDBC) or NULL         */
    const float* drag_off;  /* [3 nv] offsets (OffsetX), with drag_w       */
    float target[3];        /* mouse target                                */
    int nfixed;
    const orc_fixed_body* fixed;
    float mu_t, mu_n;
    float* XT;              /* [3 nv] XTilde in/out, or NULL (XTilde = X)  */
} orc_scene;

/* orc_simulate with scene terms (scene may be NULL). */
int orc_simulate_scene(int nv, int nt, const float* X0, float* X, float* V,
                       const uint32_t* tets, const float* mass, const float* mu,
                       const float* dbc, const orc_params* p, int precision,
                       int nsteps, int nthreads, int* iters_out, double* step_seconds,
                       const orc_scene* scene);

/* A persistent simulation for timing: set-up (geometry, system, factor)
 * once, then steps on demand; the state carries over between runs.
 * num_iterations > 0 overrides the parameters' count for that run. */
typedef struct orc_runner orc_runner;
orc_runner* orc_runner_create(int nv, int nt, const float* X0, const float* X, const float* V,
                              const uint32_t* tets, const float* mass, const float* mu,
                              const float* dbc, const orc_params* p, int precision, int nthreads);
int orc_runner_run(orc_runner* r, int nsteps, int num_iterations, int* iters_out, double* step_seconds);
int orc_runner_state(const orc_runner* r, float* X, float* V);
void orc_runner_destroy(orc_runner* r);

/* Closest proper rotation of each 3x3 matrix F (row-major, 9 per item).
 * precision 64: exact; 32: the float McAdams-style SVD.  R row-major. */
void orc_rotations(int n, const double* F, double* R, int precision);

/* One local step (reference pdUtil.cu:97-145 + 168-179): b = mdt2*s_old +
 * sum_t c_t (R_t [- F_t]) B_t, in double.  q, s_old: [3nv]. b: [3nv] out.
 * jacobi_form != 0 subtracts F (residual form used by the Jacobi path). */
int orc_local_rhs(int nv, int nt, const float* X0, const uint32_t* tets,
                  const float* mass, const float* mu, const float* dbc,
                  float dt, float positional_weight, const double* q,
                  const double* s_old, int jacobi_form, double* b);

/* Scalar system K (nv x nv, CSR, full symmetric) of the PD step:
 * K = diag((m + pin*w)/h^2) + sum_t c_t B_t^T B_t.  Returns nnz, fills the
 * arrays when they are non-null (call once with nulls to size them). */
long orc_system_csr(int nv, int nt, const float* X0, const uint32_t* tets,
                    const float* mass, const float* mu, const float* dbc,
                    float dt, float positional_weight, int64_t* rowptr,
                    int32_t* colind, double* val);

/* Exact solve K x = b for 3 interleaved right-hand sides (double). */
int orc_solve3(int nv, int nt, const float* X0, const uint32_t* tets,
               const float* mass, const float* mu, const float* dbc,
               float dt, float positional_weight, const double* b, double* x);

/* Generic sparse SPD factor (geometric nested dissection + up-looking LL^T,
 * double).  xyz: 3 coordinates per unknown for the ordering.  Returns an
 * opaque handle or NULL (not SPD / bad input). */
void* orc_factor_csr(int n, const int64_t* rowptr, const int32_t* colind, const double* val, const float* xyz);
/* x = A^-1 b (one right-hand side, double). */
void orc_solve_factored(const void* h, const double* b, double* x);
long orc_factor_nnz(const void* h);
void orc_free_factor(void* h);

#ifdef __cplusplus
}
#endif
