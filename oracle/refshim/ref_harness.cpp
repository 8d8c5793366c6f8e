// CPU driver of the reference's own PD kernels — TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/build_ref.sh together with the reference's
// src/simulation/solver/projective/pdUtil.cu (compiled as C++ through
// shim.h) into oracle/_ref/libref_pd.so.  It replays, serially and in host
// memory, what the reference's PdSolver does on the GPU:
//   FEMSolver ctor      femSolver.cu:7-17  (computeInvDmV0)
//   SolverPrepare       pdSolver.cu:40-139 (computeSiTSi, setMDt_2, DBCX = X0)
//   SolverStep          pdSolver.cu:141-208
//   Update (no CCD collision; fixed bodies)  pdSolver.cu:210-232
// The only piece that is not the reference's code is the Cholesky global
// solve: the reference calls cuSOLVER's sparse Cholesky (a GPU library);
// here the same 3n x 3n system (the COO the kernels emit, duplicates summed
// as sort_coo does, linear.cu:6-40) is solved exactly in double.
#include <def.h>
#include <simulation/solver/projective/pdUtil.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../pd_oracle.h"
#include "ref_scene.h"

thread_local refshim_dim3 blockIdx, threadIdx, blockDim, gridDim;

// Scene terms (nullable): select_v >= 0 runs the drag selection (the
// reference's ResetMoreDBC while dragging) before the first step, or before
// every step with reselect != 0 (as a mouse-move callback does); target is
// the mouse target; the fixed bodies are built from their scene-file
// description and applied after every step as PdSolver::Update does;
// XTout (nullable) receives XTilde.
extern "C" int ref_simulate_scene(int nv, int nt, const float* X0in, float* Xio, float* Vio, const uint32_t* tetsin,
                                  const float* massin, const float* muin, const float* dbcin, float dt, float gravity,
                                  int numIterations, float tol, float rho, int solver, int nsteps, int* iters_out,
                                  int select_v, int reselect, const float* target_in, int nfixed,
                                  const RefFixedSpec* fixed_specs, float muT, float muN, float* XTout) {
    const int tpb = 128;  // context.json "threads per block"
    const float positional_weight = 1e6f;
    const int vertBlocks = (nv + tpb - 1) / tpb;
    const int vert3Blocks = (3 * nv + tpb - 1) / tpb;
    const int tetBlocks = (nt + tpb - 1) / tpb;
    const bool jacobi = solver == 0;
    // ---- SolverData<float>
    std::vector<glm::vec3> X(nv), X0(nv), XTilde(nv), V(nv), DBCX(nv), OffsetX(nv, glm::vec3(0.f)),
        ExtForce(nv, glm::vec3(0.f));
    std::vector<float> DBC(nv, 0.f), moreDBC(nv, 0.f), mass(nv), mu(nt), V0(nt, 0.f), contact_area(nv, 0.f),
        degree(nv, 0.f);
    std::vector<indexType> Tet(4 * (size_t)nt);
    std::vector<glm::mat3> DmInv(nt);
    int numDBC = 0;
    for (int v = 0; v < nv; ++v) {
        X0[v] = glm::vec3(X0in[3 * v], X0in[3 * v + 1], X0in[3 * v + 2]);
        X[v] = glm::vec3(Xio[3 * v], Xio[3 * v + 1], Xio[3 * v + 2]);
        V[v] = glm::vec3(Vio[3 * v], Vio[3 * v + 1], Vio[3 * v + 2]);
        mass[v] = massin[v];
        DBC[v] = dbcin ? dbcin[v] : 0.f;
        numDBC += DBC[v] > 0.f;
    }
    XTilde = X;
    for (int t = 0; t < nt; ++t) mu[t] = muin[t];
    for (size_t i = 0; i < 4 * (size_t)nt; ++i) {
        if (tetsin[i] >= (uint32_t)nv) return -1;
        Tet[i] = tetsin[i];
    }
    // ---- FEMSolver ctor: DmInv, V0 from the rest shape
    refshim_launch(tetBlocks, tpb, [&] {
        computeInvDmV0<float>(V0.data(), DmInv.data(), nt, X0.data(), Tet.data(), contact_area.data(), degree.data());
    });
    // ---- SolverPrepare
    const int len = nv * 3 + 48 * nt;
    const int ASize = 3 * nv;
    std::vector<int> ARow(len, 0), ACol(len, 0);
    std::vector<float> AVal(len, 0.f), massDt_2s(nv, 0.f), matrix_diag(nv, 0.f);
    refshim_launch(tetBlocks, tpb, [&] {
        PdUtil::computeSiTSi(ARow.data(), ACol.data(), AVal.data(), matrix_diag.data(), V0.data(), DmInv.data(),
                             Tet.data(), mu.data(), nt, nv);
    });
    refshim_launch(vertBlocks, tpb, [&] {
        PdUtil::setMDt_2(nv, ARow.data(), ACol.data(), AVal.data(), 48 * nt, mass.data(), dt * dt, massDt_2s.data(),
                         DBC.data(), positional_weight);
    });
    DBCX = X0;
    void* factor = nullptr;
    if (!jacobi) {
        std::vector<std::map<int, double>> rows(ASize);
        for (int k = 0; k < len; ++k) {
            if (ARow[k] < 0 || ARow[k] >= ASize || ACol[k] < 0 || ACol[k] >= ASize) return -1;
            rows[ARow[k]][ACol[k]] += (double)AVal[k];
        }
        std::vector<int64_t> rp(ASize + 1, 0);
        std::vector<int32_t> ci;
        std::vector<double> cv;
        for (int r = 0; r < ASize; ++r) {
            for (auto& kv : rows[r]) {
                ci.push_back(kv.first);
                cv.push_back(kv.second);
            }
            rp[r + 1] = (int64_t)ci.size();
        }
        std::vector<float> xyz(3 * (size_t)ASize);
        for (int d = 0; d < ASize; ++d)
            for (int k = 0; k < 3; ++k) xyz[3 * (size_t)d + k] = X0in[3 * (d / 3) + k];
        factor = orc_factor_csr(ASize, rp.data(), ci.data(), cv.data(), xyz.data());
        if (!factor) return -2;
    }
    // ---- solver scratch (pdSolver.cu:99-106)
    std::vector<float> sn(ASize), sn_old(ASize), next_x(ASize), prev_x(ASize, 0.f), b(ASize);
    std::vector<double> bd(ASize), xd(ASize);
    float omega = 1.f;
    const float dtInv = 1.0f / dt;
    const float dt2Inv = dtInv * dtInv;
    const glm::vec3 target = target_in ? glm::vec3(target_in[0], target_in[1], target_in[2]) : glm::vec3(0.f);
    if (select_v >= nv) return -1;
    void* fixed = nfixed > 0 ? ref_make_fixed(nfixed, fixed_specs) : nullptr;
    if (select_v >= 0) ref_control(X.data(), DBC.data(), moreDBC.data(), OffsetX.data(), nv, select_v);
    for (int step = 0; step < nsteps; ++step) {
        if (select_v >= 0 && reselect && step > 0)
            ref_control(X.data(), DBC.data(), moreDBC.data(), OffsetX.data(), nv, select_v);
        // ---- SolverStep (pdSolver.cu:141-208)
        for (int v = 0; v < nv; ++v) ExtForce[v] = glm::vec3(0.0f, -gravity * mass[v], 0.0f);
        refshim_launch(vertBlocks, tpb, [&] {
            PdUtil::setMDt_2MoreDBC(nv, mass.data(), dt * dt, massDt_2s.data(), moreDBC.data(), DBC.data());
        });
        refshim_launch(vertBlocks, tpb, [&] {
            PdUtil::computeSn(nv, sn.data(), dt, massDt_2s.data(), X.data(), V.data(), ExtForce.data(),
                              moreDBC.data(), OffsetX.data(), DBCX.data(), target);
        });
        sn_old = sn;
        if (jacobi) prev_x = sn;
        else std::memset(prev_x.data(), 0, (size_t)nv * 3);  // byte count, as in pdSolver.cu:162
        float err = 1.f;
        int it = 0;
        for (int i = 0; i < numIterations && std::sqrt(err) >= tol; i++, it++) {
            refshim_launch(vertBlocks, tpb, [&] { PdUtil::addM_h2Sn(b.data(), sn_old.data(), massDt_2s.data(), nv); });
            refshim_launch(tetBlocks, tpb, [&] {
                PdUtil::computeLocal(V0.data(), mu.data(), b.data(), DmInv.data(), sn.data(), Tet.data(), nt, jacobi);
            });
            if (numDBC > 0)
                refshim_launch(vertBlocks, tpb, [&] {
                    PdUtil::computeDBCLocal(nv, DBC.data(), moreDBC.data(), DBCX.data(), positional_weight * dt2Inv,
                                            b.data());
                });
            if (!jacobi) {
                for (int k = 0; k < ASize; ++k) bd[k] = b[k];
                orc_solve_factored(factor, bd.data(), xd.data());
                for (int k = 0; k < ASize; ++k) sn[k] = (float)xd[k];
                float acc = 0.f;  // computeError: plus<float> reduction (pdSolver.cu:243-253)
                for (int k = 0; k < ASize; ++k) acc = acc + (prev_x[k] - sn[k]) * (prev_x[k] - sn[k]);
                err = (float)((double)acc / ASize);
                prev_x = sn;
            } else {
                refshim_launch(vertBlocks, tpb, [&] {
                    PdUtil::getErrorKern(nv, next_x.data(), b.data(), massDt_2s.data(), sn.data(), matrix_diag.data(),
                                         moreDBC.data());
                });
                if (i <= 10) omega = 1;
                else if (i == 11) omega = 2 / (2 - rho * rho);
                else omega = 4 / (4 - rho * rho * omega);
                refshim_launch(vert3Blocks, tpb, [&] {
                    PdUtil::chebyshevKern(3 * nv, next_x.data(), prev_x.data(), sn.data(), omega);
                });
            }
        }
        if (iters_out) iters_out[step] = it;
        refshim_launch(vertBlocks, tpb, [&] {
            PdUtil::updateVelPos(sn.data(), dtInv, XTilde.data(), V.data(), nv, moreDBC.data());
        });
        X = XTilde;  // Update tail without collision handling (pdSolver.cu:227)
        if (fixed) ref_handle_collisions(fixed, XTilde.data(), V.data(), nv, muT, muN);  // pdSolver.cu:228-231
    }
    if (factor) orc_free_factor(factor);
    if (fixed) ref_free_fixed(fixed);
    for (int v = 0; v < nv; ++v) {
        Xio[3 * v] = X[v].x; Xio[3 * v + 1] = X[v].y; Xio[3 * v + 2] = X[v].z;
        Vio[3 * v] = V[v].x; Vio[3 * v + 1] = V[v].y; Vio[3 * v + 2] = V[v].z;
        if (XTout) {
            XTout[3 * v] = XTilde[v].x; XTout[3 * v + 1] = XTilde[v].y; XTout[3 * v + 2] = XTilde[v].z;
        }
    }
    return 0;
}

extern "C" int ref_simulate(int nv, int nt, const float* X0in, float* Xio, float* Vio, const uint32_t* tetsin,
                            const float* massin, const float* muin, const float* dbcin, float dt, float gravity,
                            int numIterations, float tol, float rho, int solver, int nsteps, int* iters_out) {
    return ref_simulate_scene(nv, nt, X0in, Xio, Vio, tetsin, massin, muin, dbcin, dt, gravity, numIterations, tol,
                              rho, solver, nsteps, iters_out, -1, 0, nullptr, 0, nullptr, 0.5f, 0.5f, nullptr);
}

// The reference's rotation for one deformation gradient: svdGLM + R = U V^T
// with the det < 0 column flip (pdUtil.cu:113-122).  F, R row-major.
#include <svd.cuh>
extern "C" void ref_rotation(const float* F, float* R) {
    glm::mat3 f;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) f[c][r] = F[3 * r + c];  // glm: f[column][row]
    glm::mat3 U, S, Vm;
    svdGLM(f, U, S, Vm);
    glm::mat3 Rm = U * glm::transpose(Vm);
    if (glm::determinant(Rm) < 0) Rm[2] = -Rm[2];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[3 * r + c] = Rm[c][r];
}
