// CPU oracle for the PD step — TEST INFRASTRUCTURE ONLY (see pd_oracle.h).
// Restates the reference's float PD path (src/simulation/solver/projective/)
// in plain C++, in double ("FP64 oracle") or in float (CPU baseline).
#include "pd_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

double now_seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- 3x3 math
// Row-major 3x3: a[r][c].
template <class T> struct Mat3 { T a[3][3]; };

template <class T> inline T dot3(const T* x, const T* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; }

// ---- FP64 rotation: exact cyclic Jacobi on S = F^T F, then U by
// Gram-Schmidt on B = F V (columns sorted by norm), third column = u1 x u2.
// Returns the closest proper rotation of F (signed smallest singular value).
void polar_rotation_f64(const double F[3][3], double R[3][3]) {
    double S[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
    static const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][2] * S[1][2];
        double dia = S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2];
        if (off == 0.0 || off <= 1e-36 * dia) break;
        for (auto& pq : P) {
            int p = pq[0], q = pq[1];
            if (S[p][q] == 0.0) continue;
            double theta = (S[q][q] - S[p][p]) / (2.0 * S[p][q]);
            double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
            double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
            double J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
            J[p][p] = c; J[q][q] = c; J[p][q] = s; J[q][p] = -s;
            double T1[3][3], T2[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) T1[i][j] = S[i][0] * J[0][j] + S[i][1] * J[1][j] + S[i][2] * J[2][j];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) T2[i][j] = J[0][i] * T1[0][j] + J[1][i] * T1[1][j] + J[2][i] * T1[2][j];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) S[i][j] = T2[i][j];
            S[p][q] = S[q][p] = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) T1[i][j] = V[i][0] * J[0][j] + V[i][1] * J[1][j] + V[i][2] * J[2][j];
            std::memcpy(V, T1, sizeof(V));
        }
    }
    // B = F V; columns b_j.
    double b[3][3];  // b[j] = column j
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) b[j][i] = F[i][0] * V[0][j] + F[i][1] * V[1][j] + F[i][2] * V[2][j];
    double v[3][3];  // v[j] = column j of V
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) v[j][i] = V[i][j];
    int ord[3] = {0, 1, 2};
    double nrm[3] = {dot3(b[0], b[0]), dot3(b[1], b[1]), dot3(b[2], b[2])};
    std::sort(ord, ord + 3, [&](int x, int y) { return nrm[x] > nrm[y]; });
    double bs[3][3], vs[3][3];
    for (int j = 0; j < 3; ++j) {
        std::memcpy(bs[j], b[ord[j]], sizeof(bs[j]));
        std::memcpy(vs[j], v[ord[j]], sizeof(vs[j]));
    }
    // det(V) must be +1 so that U V^T is proper.
    double cr[3] = {vs[0][1] * vs[1][2] - vs[0][2] * vs[1][1], vs[0][2] * vs[1][0] - vs[0][0] * vs[1][2],
                    vs[0][0] * vs[1][1] - vs[0][1] * vs[1][0]};
    if (dot3(cr, vs[2]) < 0)
        for (int i = 0; i < 3; ++i) { vs[2][i] = -vs[2][i]; bs[2][i] = -bs[2][i]; }
    double scale = std::sqrt(nrm[ord[0]]);
    double u[3][3];
    if (!(scale > 1e-300)) {
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) u[j][i] = (i == j);
    } else {
        for (int i = 0; i < 3; ++i) u[0][i] = bs[0][i] / scale;
        double d = dot3(u[0], bs[1]);
        double w[3] = {bs[1][0] - d * u[0][0], bs[1][1] - d * u[0][1], bs[1][2] - d * u[0][2]};
        double wn = std::sqrt(dot3(w, w));
        if (!(wn > 1e-13 * scale)) {
            // rank-1 F: any unit vector orthogonal to u1.
            int k = 0;
            for (int i = 1; i < 3; ++i) if (std::fabs(u[0][i]) < std::fabs(u[0][k])) k = i;
            double e[3] = {0, 0, 0}; e[k] = 1;
            double dd = dot3(u[0], e);
            for (int i = 0; i < 3; ++i) w[i] = e[i] - dd * u[0][i];
            wn = std::sqrt(dot3(w, w));
        }
        for (int i = 0; i < 3; ++i) u[1][i] = w[i] / wn;
        u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
        u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
        u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = u[0][i] * vs[0][j] + u[1][i] * vs[1][j] + u[2][i] * vs[2][j];
}

// ---- FP32 rotation: McAdams et al. (UW-Madison TR1690, 2011) scheme:
// 4 sweeps of approximate-Givens Jacobi on F^T F accumulated as a quaternion,
// columns of F V sorted by norm, then U by Gram-Schmidt + cross product.
inline void quat_mul_axis(float q[4], float ch, float sh, int axis) {
    // q <- q * (ch, sh e_axis); quaternion (w, x, y, z).
    float w = q[0], x = q[1], y = q[2], z = q[3];
    if (axis == 0) { q[0] = w * ch - x * sh; q[1] = x * ch + w * sh; q[2] = y * ch + z * sh; q[3] = z * ch - y * sh; }
    else if (axis == 1) { q[0] = w * ch - y * sh; q[1] = x * ch - z * sh; q[2] = y * ch + w * sh; q[3] = z * ch + x * sh; }
    else { q[0] = w * ch - z * sh; q[1] = x * ch + y * sh; q[2] = y * ch - x * sh; q[3] = z * ch + w * sh; }
}

void polar_rotation_f32(const float F[3][3], float R[3][3]) {
    const float kGamma = 5.828427124746190f;        // (1 + sqrt 2)^2
    const float kCos8 = 0.9238795325112867f, kSin8 = 0.3826834323650898f;  // cos, sin of pi/8
    float S[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
    float q[4] = {1, 0, 0, 0};
    // rotation planes (p, q) and the quaternion axis of the rotation.
    static const int PL[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    for (int sweep = 0; sweep < 4; ++sweep) {
        for (auto& pl : PL) {
            int p = pl[0], qq = pl[1], r = pl[2];
            float ch = 2.0f * (S[p][p] - S[qq][qq]);
            float sh = S[p][qq];
            bool ok = kGamma * sh * sh < ch * ch;
            float w = 1.0f / std::sqrt(ch * ch + sh * sh);
            ch = ok ? w * ch : kCos8;
            sh = ok ? w * sh : kSin8;
            float c = ch * ch - sh * sh, s = 2.0f * sh * ch;
            // S <- Q^T S Q, Q rotating e_p toward e_q by the angle (c, s).
            float spp = S[p][p], sqq = S[qq][qq], spq = S[p][qq], srp = S[r][p], srq = S[r][qq];
            float npp = c * c * spp + 2.0f * c * s * spq + s * s * sqq;
            float nqq = s * s * spp - 2.0f * c * s * spq + c * c * sqq;
            float npq = c * s * (sqq - spp) + (c * c - s * s) * spq;
            float nrp = c * srp + s * srq;
            float nrq = -s * srp + c * srq;
            S[p][p] = npp; S[qq][qq] = nqq; S[p][qq] = S[qq][p] = npq;
            S[r][p] = S[p][r] = nrp; S[r][qq] = S[qq][r] = nrq;
            quat_mul_axis(q, ch, sh, r);
        }
    }
    float qn = 1.0f / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    float w = q[0] * qn, x = q[1] * qn, y = q[2] * qn, z = q[3] * qn;
    float V[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                     {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                     {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    float b[3][3], v[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            b[j][i] = F[i][0] * V[0][j] + F[i][1] * V[1][j] + F[i][2] * V[2][j];
            v[j][i] = V[i][j];
        }
    // sort by column norm, swapping with a sign flip so det(V) stays +1.
    auto swapneg = [&](int i, int j) {
        for (int k = 0; k < 3; ++k) {
            float t = b[i][k]; b[i][k] = b[j][k]; b[j][k] = -t;
            t = v[i][k]; v[i][k] = v[j][k]; v[j][k] = -t;
        }
    };
    float n0 = dot3(b[0], b[0]), n1 = dot3(b[1], b[1]), n2 = dot3(b[2], b[2]);
    if (n0 < n1) { swapneg(0, 1); std::swap(n0, n1); }
    if (n0 < n2) { swapneg(0, 2); std::swap(n0, n2); }
    if (n1 < n2) { swapneg(1, 2); std::swap(n1, n2); }
    float u[3][3];
    if (!(n0 > 1e-30f)) {
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) u[j][i] = (i == j);
    } else {
        float in0 = 1.0f / std::sqrt(n0);
        for (int i = 0; i < 3; ++i) u[0][i] = b[0][i] * in0;
        float d = dot3(u[0], b[1]);
        float t[3] = {b[1][0] - d * u[0][0], b[1][1] - d * u[0][1], b[1][2] - d * u[0][2]};
        float tn = dot3(t, t);
        if (!(tn > 1e-12f * n0)) {
            int k = 0;
            for (int i = 1; i < 3; ++i) if (std::fabs(u[0][i]) < std::fabs(u[0][k])) k = i;
            float e[3] = {0, 0, 0}; e[k] = 1;
            float dd = dot3(u[0], e);
            for (int i = 0; i < 3; ++i) t[i] = e[i] - dd * u[0][i];
            tn = dot3(t, t);
        }
        float itn = 1.0f / std::sqrt(tn);
        for (int i = 0; i < 3; ++i) u[1][i] = t[i] * itn;
        u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
        u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
        u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = u[0][i] * v[0][j] + u[1][i] * v[1][j] + u[2][i] * v[2][j];
}

template <class T> void polar_rotation(const T F[3][3], T R[3][3]);
template <> void polar_rotation<double>(const double F[3][3], double R[3][3]) { polar_rotation_f64(F, R); }
template <> void polar_rotation<float>(const float F[3][3], float R[3][3]) { polar_rotation_f32(F, R); }

// ------------------------------------------------------------- mesh model
// Per-tet precompute (reference solverUtil.cuh:98-138): Dm = [X1-X0, X2-X0,
// X3-X0] (columns), DmInv = Dm^-1, V0 = |det Dm| / 6.  Computed in double.
struct TetGeom {
    std::vector<double> dminv;  // 9 per tet, row-major DmInv
    std::vector<double> coef;   // V0 * w
};

bool tet_geometry(int nv, int nt, const float* X0, const uint32_t* tets, const float* mu, TetGeom& g) {
    g.dminv.resize((size_t)nt * 9);
    g.coef.resize(nt);
    for (int t = 0; t < nt; ++t) {
        uint32_t id[4];
        for (int k = 0; k < 4; ++k) {
            id[k] = tets[4 * (size_t)t + k];
            if (id[k] >= (uint32_t)nv) return false;
        }
        double D[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) D[r][c] = (double)X0[3 * id[c + 1] + r] - (double)X0[3 * id[0] + r];
        double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) - D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                     D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
        if (det == 0.0) return false;
        double inv[3][3];
        inv[0][0] = (D[1][1] * D[2][2] - D[1][2] * D[2][1]) / det;
        inv[0][1] = (D[0][2] * D[2][1] - D[0][1] * D[2][2]) / det;
        inv[0][2] = (D[0][1] * D[1][2] - D[0][2] * D[1][1]) / det;
        inv[1][0] = (D[1][2] * D[2][0] - D[1][0] * D[2][2]) / det;
        inv[1][1] = (D[0][0] * D[2][2] - D[0][2] * D[2][0]) / det;
        inv[1][2] = (D[0][2] * D[1][0] - D[0][0] * D[1][2]) / det;
        inv[2][0] = (D[1][0] * D[2][1] - D[1][1] * D[2][0]) / det;
        inv[2][1] = (D[0][1] * D[2][0] - D[0][0] * D[2][1]) / det;
        inv[2][2] = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) / det;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) g.dminv[9 * (size_t)t + 3 * r + c] = inv[r][c];
        g.coef[t] = std::fabs(det) / 6.0 * (double)mu[t];
    }
    return true;
}

// B = DmInv^T G (3x4) with G = [[-1,1,0,0],[-1,0,1,0],[-1,0,0,1]]
// (reference pdUtil.cu:16, 126-127).  Column j of B belongs to tet corner j.
template <class T> inline void make_B(const T* Dinv, T B[3][4]) {
    for (int i = 0; i < 3; ++i) {
        // (D^T)_{i,k} = D_{k,i}
        B[i][1] = Dinv[3 * 0 + i];
        B[i][2] = Dinv[3 * 1 + i];
        B[i][3] = Dinv[3 * 2 + i];
        B[i][0] = -(B[i][1] + B[i][2] + B[i][3]);
    }
}

// vertex -> (tet, corner) incidence, sorted by tet, for deterministic gathers.
struct Incidence {
    std::vector<int> ptr, ent;  // ent = 4*tet + corner
};
Incidence build_incidence(int nv, int nt, const uint32_t* tets) {
    Incidence inc;
    inc.ptr.assign(nv + 1, 0);
    for (size_t i = 0; i < (size_t)nt * 4; ++i) inc.ptr[tets[i] + 1]++;
    for (int v = 0; v < nv; ++v) inc.ptr[v + 1] += inc.ptr[v];
    inc.ent.resize((size_t)nt * 4);
    std::vector<int> fill(inc.ptr.begin(), inc.ptr.end() - 1);
    for (size_t i = 0; i < (size_t)nt * 4; ++i) inc.ent[fill[tets[i]]++] = (int)i;
    return inc;
}

// ------------------------------------------------------ sparse LL^T oracle
struct CSR {
    int n = 0;
    std::vector<int64_t> p;
    std::vector<int> i;
    std::vector<double> x;
};

// K = diag(mdt2) + sum_t c_t B_t^T B_t  (reference pdUtil.cu:9-54; the
// reference's 3n x 3n matrix is K (x) I_3 in interleaved order).
CSR assemble_K(int nv, int nt, const uint32_t* tets, const TetGeom& g, const std::vector<double>& mdt2,
               std::vector<double>* stiff_diag) {
    std::vector<std::vector<std::pair<int, double>>> rows(nv);
    if (stiff_diag) stiff_diag->assign(nv, 0.0);
    for (int t = 0; t < nt; ++t) {
        double B[3][4];
        make_B(&g.dminv[9 * (size_t)t], B);
        for (int a = 0; a < 4; ++a)
            for (int bb = 0; bb < 4; ++bb) {
                double s = g.coef[t] * (B[0][a] * B[0][bb] + B[1][a] * B[1][bb] + B[2][a] * B[2][bb]);
                rows[tets[4 * (size_t)t + a]].push_back({(int)tets[4 * (size_t)t + bb], s});
                if (a == bb && stiff_diag) (*stiff_diag)[tets[4 * (size_t)t + a]] += s;
            }
    }
    CSR K;
    K.n = nv;
    K.p.assign(nv + 1, 0);
    for (int v = 0; v < nv; ++v) {
        rows[v].push_back({v, mdt2[v]});
        std::sort(rows[v].begin(), rows[v].end(), [](auto& x, auto& y) { return x.first < y.first; });
        int last = -1;
        for (auto& e : rows[v]) {
            if (e.first == last) K.x.back() += e.second;
            else { K.i.push_back(e.first); K.x.push_back(e.second); last = e.first; }
        }
        K.p[v + 1] = (int64_t)K.i.size();
    }
    return K;
}

// Geometric nested dissection: recursive median bisection along the longest
// bounding-box axis; separator = vertices of the upper half adjacent to the
// lower half; order = lower, upper\sep, sep.
void nd_recurse(std::vector<int>& vs, const CSR& K, const float* X0, std::vector<int>& order,
                std::vector<int>& mark, int& stamp) {
    if (vs.size() <= 48) {
        order.insert(order.end(), vs.begin(), vs.end());
        return;
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v : vs)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], (double)X0[3 * v + d]);
            hi[d] = std::max(hi[d], (double)X0[3 * v + d]);
        }
    int ax = 0;
    for (int d = 1; d < 3; ++d) if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    size_t half = vs.size() / 2;
    std::nth_element(vs.begin(), vs.begin() + half, vs.end(), [&](int a, int b) {
        float xa = X0[3 * a + ax], xb = X0[3 * b + ax];
        return xa < xb || (xa == xb && a < b);
    });
    int my = ++stamp;
    for (size_t k = 0; k < half; ++k) mark[vs[k]] = my;
    std::vector<int> A(vs.begin(), vs.begin() + half), B, S;
    for (size_t k = half; k < vs.size(); ++k) {
        int v = vs[k];
        bool sep = false;
        for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e)
            if (mark[K.i[e]] == my) { sep = true; break; }
        (sep ? S : B).push_back(v);
    }
    std::vector<int>().swap(vs);
    nd_recurse(A, K, X0, order, mark, stamp);
    nd_recurse(B, K, X0, order, mark, stamp);
    order.insert(order.end(), S.begin(), S.end());
}

struct SpChol {
    int n = 0;
    std::vector<int> perm;  // perm[k] = original index of pivot k
    std::vector<int64_t> Lp;
    std::vector<int> Li;
    std::vector<double> Lx;
    std::vector<float> Lxf;

    // Up-looking simplicial LL^T of C = P K P^T.
    bool factor(const CSR& K, const float* X0) {
        n = K.n;
        {
            std::vector<int> vs(n), mark(n, 0);
            std::iota(vs.begin(), vs.end(), 0);
            int stamp = 0;
            perm.clear();
            perm.reserve(n);
            nd_recurse(vs, K, X0, perm, mark, stamp);
        }
        std::vector<int> iperm(n);
        for (int k = 0; k < n; ++k) iperm[perm[k]] = k;
        // upper part of column k of C: entries (j, k) with j <= k
        std::vector<int64_t> Cp(n + 1, 0);
        std::vector<int> Ci;
        std::vector<double> Cx;
        for (int k = 0; k < n; ++k) {
            int v = perm[k];
            for (int64_t e = K.p[v]; e < K.p[v + 1]; ++e) {
                int j = iperm[K.i[e]];
                if (j <= k) { Ci.push_back(j); Cx.push_back(K.x[e]); }
            }
            Cp[k + 1] = (int64_t)Ci.size();
        }
        // elimination tree
        std::vector<int> parent(n, -1), anc(n, -1);
        for (int k = 0; k < n; ++k)
            for (int64_t e = Cp[k]; e < Cp[k + 1]; ++e) {
                int i = Ci[e];
                while (i != -1 && i < k) {
                    int nxt = anc[i];
                    anc[i] = k;
                    if (nxt == -1) { parent[i] = k; break; }
                    i = nxt;
                }
            }
        // row patterns via ereach -> column counts
        std::vector<int> w(n, -1), s(n), cnt(n, 1);
        auto ereach = [&](int k) {
            int top = n;
            w[k] = k;
            for (int64_t e = Cp[k]; e < Cp[k + 1]; ++e) {
                int i = Ci[e];
                if (i > k) continue;
                int len = 0;
                for (; w[i] != k; i = parent[i]) { s[len++] = i; w[i] = k; }
                while (len > 0) s[--top] = s[--len];
            }
            return top;
        };
        for (int k = 0; k < n; ++k) {
            int top = ereach(k);
            for (int p = top; p < n; ++p) cnt[s[p]]++;
        }
        Lp.assign(n + 1, 0);
        for (int k = 0; k < n; ++k) Lp[k + 1] = Lp[k] + cnt[k];
        Li.assign(Lp[n], 0);
        Lx.assign(Lp[n], 0.0);
        std::vector<int64_t> c(Lp.begin(), Lp.end() - 1);
        std::vector<double> x(n, 0.0);
        std::fill(w.begin(), w.end(), -1);
        for (int k = 0; k < n; ++k) {
            int top = ereach(k);
            for (int64_t e = Cp[k]; e < Cp[k + 1]; ++e) x[Ci[e]] += Cx[e];
            double d = x[k];
            x[k] = 0.0;
            for (int p = top; p < n; ++p) {
                int i = s[p];
                double lki = x[i] / Lx[Lp[i]];
                x[i] = 0.0;
                for (int64_t q = Lp[i] + 1; q < c[i]; ++q) x[Li[q]] -= Lx[q] * lki;
                d -= lki * lki;
                Li[c[i]] = k;
                Lx[c[i]] = lki;
                c[i]++;
            }
            if (!(d > 0.0)) return false;
            Li[c[k]] = k;
            Lx[c[k]] = std::sqrt(d);
            c[k]++;
        }
        Lxf.assign(Lx.begin(), Lx.end());
        return true;
    }

    // Solve K x = b for 3 interleaved right-hand sides, in T.
    template <class T> void solve3(const T* b, T* x) const {
        std::vector<T> y((size_t)3 * n);
        const auto& L = lx<T>();
        for (int k = 0; k < n; ++k)
            for (int d = 0; d < 3; ++d) y[3 * k + d] = b[3 * (size_t)perm[k] + d];
        for (int j = 0; j < n; ++j) {
            T dj = L[Lp[j]];
            T y0 = y[3 * j] / dj, y1 = y[3 * j + 1] / dj, y2 = y[3 * j + 2] / dj;
            y[3 * j] = y0; y[3 * j + 1] = y1; y[3 * j + 2] = y2;
            for (int64_t q = Lp[j] + 1; q < Lp[j + 1]; ++q) {
                size_t r = 3 * (size_t)Li[q];
                y[r] -= L[q] * y0; y[r + 1] -= L[q] * y1; y[r + 2] -= L[q] * y2;
            }
        }
        for (int j = n - 1; j >= 0; --j) {
            T a0 = y[3 * j], a1 = y[3 * j + 1], a2 = y[3 * j + 2];
            for (int64_t q = Lp[j] + 1; q < Lp[j + 1]; ++q) {
                size_t r = 3 * (size_t)Li[q];
                a0 -= L[q] * y[r]; a1 -= L[q] * y[r + 1]; a2 -= L[q] * y[r + 2];
            }
            T dj = L[Lp[j]];
            y[3 * j] = a0 / dj; y[3 * j + 1] = a1 / dj; y[3 * j + 2] = a2 / dj;
        }
        for (int k = 0; k < n; ++k)
            for (int d = 0; d < 3; ++d) x[3 * (size_t)perm[k] + d] = y[3 * k + d];
    }
    template <class T> const std::vector<T>& lx() const;
};
template <> const std::vector<double>& SpChol::lx<double>() const { return Lx; }
template <> const std::vector<float>& SpChol::lx<float>() const { return Lxf; }

// ---------------------------------------------------------------- PD loop
template <class T> struct Sim {
    int nv, nt;
    const uint32_t* tets;
    std::vector<T> dminv, coef;       // per tet
    std::vector<T> mass, mdt2, stiff_diag, dbc, x0;
    Incidence inc;
    SpChol chol;
    bool has_chol = false;
    std::vector<T> P;                 // per-tet 12 contributions
    std::vector<T> prev;              // persists across steps (Cholesky path)
};

template <class T>
void local_rhs(Sim<T>& S, const T* q, const T* s_old, bool jacobi_form, T* b, const T* mdt2) {
    const int nt = S.nt;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
        const uint32_t* id = S.tets + 4 * (size_t)t;
        const T* D = &S.dminv[9 * (size_t)t];
        T Ds[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) Ds[r][c] = q[3 * id[c + 1] + r] - q[3 * id[0] + r];
        T F[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) F[r][c] = Ds[r][0] * D[3 * 0 + c] + Ds[r][1] * D[3 * 1 + c] + Ds[r][2] * D[3 * 2 + c];
        T R[3][3];
        polar_rotation<T>(F, R);
        if (jacobi_form)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) R[r][c] -= F[r][c];
        // M = (c R) DmInv^T ; P = M G
        T cf = S.coef[t];
        T M[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                T cr0 = cf * R[r][0], cr1 = cf * R[r][1], cr2 = cf * R[r][2];
                M[r][c] = cr0 * D[3 * c + 0] + cr1 * D[3 * c + 1] + cr2 * D[3 * c + 2];
            }
        T* out = &S.P[12 * (size_t)t];
        for (int r = 0; r < 3; ++r) {
            out[0 * 3 + r] = -M[r][0] - M[r][1] - M[r][2];
            out[1 * 3 + r] = M[r][0];
            out[2 * 3 + r] = M[r][1];
            out[3 * 3 + r] = M[r][2];
        }
    }
#pragma omp parallel for schedule(static)
    for (int v = 0; v < S.nv; ++v) {
        T acc[3] = {mdt2[v] * s_old[3 * v], mdt2[v] * s_old[3 * v + 1], mdt2[v] * s_old[3 * v + 2]};
        for (int e = S.inc.ptr[v]; e < S.inc.ptr[v + 1]; ++e) {
            int ent = S.inc.ent[e];
            const T* o = &S.P[12 * (size_t)(ent >> 2) + 3 * (ent & 3)];
            acc[0] += o[0]; acc[1] += o[1]; acc[2] += o[2];
        }
        b[3 * v] = acc[0]; b[3 * v + 1] = acc[1]; b[3 * v + 2] = acc[2];
    }
}

// ---- fixed rigid bodies (fixedBodyData.cu:66-148)
template <class T> struct Fixed {
    int type;
    T p[3], n[3], r;
};

template <class T> std::vector<Fixed<T>> fixed_bodies(const orc_scene* sc) {
    std::vector<Fixed<T>> out;
    if (!sc) return out;
    for (int kind = 0; kind < 3; ++kind)  // HandleCollisions: spheres, planes, cylinders
        for (int j = 0; j < sc->nfixed; ++j) {
            const orc_fixed_body& fb = sc->fixed[j];
            if (fb.type != kind) continue;
            Fixed<T> f{};
            f.type = kind;
            for (int d = 0; d < 3; ++d) f.p[d] = (T)fb.model[12 + d];
            f.r = (T)fb.radius;
            if (kind == 1) {
                for (int d = 0; d < 3; ++d) f.n[d] = (T)fb.up[d];
            } else if (kind == 2) {  // axis = normalize(vec3(model * (0,1,0,0)))
                T a[3] = {(T)fb.model[4], (T)fb.model[5], (T)fb.model[6]};
                T inv = (T)1 / std::sqrt(dot3(a, a));
                for (int d = 0; d < 3; ++d) f.n[d] = a[d] * inv;
            }
            out.push_back(f);
        }
    return out;
}

template <class T> void contact_response(const T* nrm, T mu_t, T mu_n, T* V) {
    T vn = dot3(V, nrm);
    T vN[3], vT[3];
    for (int d = 0; d < 3; ++d) {
        vN[d] = vn * nrm[d];
        vT[d] = V[d] - vN[d];
    }
    T mag_vT = std::sqrt(dot3(vT, vT));
    T a = mag_vT == (T)0 ? (T)0 : std::max((T)1 - mu_t * ((T)1 + mu_n) * std::sqrt(dot3(vN, vN)) / mag_vT, (T)0);
    for (int d = 0; d < 3; ++d) V[d] = -mu_n * vN[d] + a * vT[d];
}

template <class T> void collide(const std::vector<Fixed<T>>& fb, T mu_t, T mu_n, T* X, T* V) {
    for (const Fixed<T>& f : fb) {
        if (f.type == 1) {
            T rel[3] = {X[0] - f.p[0], X[1] - f.p[1], X[2] - f.p[2]};
            T sd = dot3(rel, f.n);
            if (sd < (T)0 && dot3(V, f.n) < (T)0) {
                for (int d = 0; d < 3; ++d) X[d] -= sd * f.n[d];
                contact_response(f.n, mu_t, mu_n, V);
            }
            continue;
        }
        T dv[3] = {X[0] - f.p[0], X[1] - f.p[1], X[2] - f.p[2]};
        if (f.type == 2) {  // (I - a a^T) d
            T q[3] = {dv[0], dv[1], dv[2]};
            for (int r = 0; r < 3; ++r) {
                T acc = 0;
                for (int c = 0; c < 3; ++c) acc += ((r == c ? (T)1 : (T)0) - f.n[r] * f.n[c]) * q[c];
                dv[r] = acc;
            }
        }
        T len = std::sqrt(dot3(dv, dv));
        if (len < f.r) {
            T inv = (T)1 / len;
            T nrm[3] = {dv[0] * inv, dv[1] * inv, dv[2] * inv};
            for (int d = 0; d < 3; ++d) X[d] += (f.r - len) * nrm[d];
            contact_response(nrm, mu_t, mu_n, V);
        }
    }
}

// One simulation: set-up (geometry, system, factor) once, then steps.  The
// state X, V, XTilde and the Cholesky path's prev vector persist across
// calls of run().
struct RunnerBase {
    virtual ~RunnerBase() {}
    virtual void run(int nsteps, int iters, int* iters_out, double* step_seconds) = 0;
    virtual void state(float* X, float* V, float* XT) const = 0;
};

template <class T> struct Runner : RunnerBase {
    int nv = 0, nt = 0;
    Sim<T> S;
    orc_params prm{};
    bool chol = false;
    T dt = 0, dt2 = 0, dtInv = 0, dt2Inv = 0, pw = 0;
    int num_pinned = 0;
    std::vector<T> X, V, XT, sn, sn_old, b, mdt2s, dragw, dbcx, drag_off;
    T target[3] = {0, 0, 0};
    std::vector<Fixed<T>> fixed;
    T mu_t = 0, mu_n = 0;

    // Returns 0, or -1 (bad mesh) / -2 (factor failed).
    int setup(int nv_, int nt_, const float* X0, const float* Xin, const float* Vin, const uint32_t* tets,
              const float* mass, const float* mu, const float* dbc, const orc_params* p, const orc_scene* sc) {
        nv = nv_;
        nt = nt_;
        prm = *p;
        S.nv = nv; S.nt = nt; S.tets = tets;
        TetGeom g;
        if (!tet_geometry(nv, nt, X0, tets, mu, g)) return -1;
        S.dminv.assign(g.dminv.begin(), g.dminv.end());
        S.coef.assign(g.coef.begin(), g.coef.end());
        S.inc = build_incidence(nv, nt, tets);
        S.P.resize((size_t)nt * 12);
        dt = (T)p->dt;
        dt2 = dt * dt;
        dtInv = (T)1 / dt;
        dt2Inv = dtInv * dtInv;
        pw = (T)p->positional_weight;
        S.mass.resize(nv); S.mdt2.resize(nv); S.dbc.resize(nv); S.x0.resize((size_t)3 * nv);
        std::vector<double> mdt2d(nv);
        for (int v = 0; v < nv; ++v) {
            S.mass[v] = mass[v];
            S.dbc[v] = dbc ? (T)dbc[v] : (T)0;
            S.mdt2[v] = (S.mass[v] + S.dbc[v] * pw) / dt2;  // setMDt_2, pdUtil.cu:48
            mdt2d[v] = (double)S.mdt2[v];
            for (int d = 0; d < 3; ++d) S.x0[3 * v + d] = X0[3 * v + d];
        }
        chol = p->solver == 1;
        if (chol) {
            CSR K = assemble_K(nv, nt, tets, g, mdt2d, nullptr);
            if (!S.chol.factor(K, X0)) return -2;
        } else {
            // Jacobi needs only diag(sum_t c_t B_t^T B_t) (pdUtil.cu:21-24)
            std::vector<double> sd(nv, 0.0);
            for (int t = 0; t < nt; ++t) {
                double B[3][4];
                make_B(&g.dminv[9 * (size_t)t], B);
                for (int a = 0; a < 4; ++a)
                    sd[tets[4 * (size_t)t + a]] +=
                        g.coef[t] * (B[0][a] * B[0][a] + B[1][a] * B[1][a] + B[2][a] * B[2][a]);
            }
            S.stiff_diag.assign(sd.begin(), sd.end());
        }
        const size_t n3 = (size_t)3 * nv;
        X.resize(n3); V.resize(n3); XT.resize(n3); sn.resize(n3); sn_old.resize(n3); b.resize(n3);
        mdt2s.resize(nv); dragw.assign(nv, (T)0); dbcx.assign(n3, (T)0); drag_off.assign(n3, (T)0);
        S.prev.assign(n3, (T)0);
        for (size_t i = 0; i < n3; ++i) {
            X[i] = Xin[i];
            V[i] = Vin[i];
            XT[i] = (sc && sc->XT) ? (T)sc->XT[i] : X[i];
        }
        for (int v = 0; v < nv; ++v) num_pinned += S.dbc[v] > 0;
        if (sc && sc->drag_w) {
            for (int v = 0; v < nv; ++v) dragw[v] = (T)sc->drag_w[v];
            for (size_t i = 0; i < n3; ++i) drag_off[i] = (T)sc->drag_off[i];
        }
        if (sc)
            for (int d = 0; d < 3; ++d) target[d] = (T)sc->target[d];
        fixed = fixed_bodies<T>(sc);
        mu_t = sc ? (T)sc->mu_t : (T)0;
        mu_n = sc ? (T)sc->mu_n : (T)0;
        return 0;
    }

    // nsteps PD steps of `iters` iterations (0: the parameters' count).
    void run(int nsteps, int iters, int* iters_out, double* step_seconds) override {
        const int n_it = iters > 0 ? iters : prm.num_iterations;
        const T g_acc = (T)prm.gravity;
        const double t_start = now_seconds();
        for (int step = 0; step < nsteps; ++step) {
            // prologue: pdSolver.cu:154-163 (gravity, setMDt_2MoreDBC, computeSn)
            for (int v = 0; v < nv; ++v) {
                T md = dragw[v];
                mdt2s[v] = S.dbc[v] == (T)0 ? (md > (T)0 ? (S.mass[v] + md) / dt2 : S.mass[v] / dt2) : S.mdt2[v];
                if (md > (T)0) {  // dragged: target + offset, also the DBC position
                    for (int d = 0; d < 3; ++d) {
                        sn[3 * v + d] = target[d] + drag_off[3 * v + d];
                        dbcx[3 * v + d] = sn[3 * v + d];
                    }
                    continue;
                }
                T f1 = -g_acc * S.mass[v];
                T dt2_m_1 = (T)1 / mdt2s[v];
                sn[3 * v + 0] = X[3 * v + 0] + dt * V[3 * v + 0] + dt2_m_1 * (T)0;
                sn[3 * v + 1] = X[3 * v + 1] + dt * V[3 * v + 1] + dt2_m_1 * f1;
                sn[3 * v + 2] = X[3 * v + 2] + dt * V[3 * v + 2] + dt2_m_1 * (T)0;
            }
            sn_old = sn;
            if (!chol) S.prev = sn;
            else std::memset(S.prev.data(), 0, std::min((size_t)3 * nv, S.prev.size() * sizeof(T)));  // bytes (pdSolver.cu:162)
            T err = 1;
            T omega = 1;
            int it = 0;
            for (int i = 0; i < n_it && std::sqrt(err) >= (T)prm.tol; ++i, ++it) {
                local_rhs<T>(S, sn.data(), sn_old.data(), !chol, b.data(), mdt2s.data());
                // pinned / dragged RHS overwrite (pdUtil.cu:147-166), run only
                // when the system has pinned vertices (pdSolver.cu:170)
                if (num_pinned > 0)
                    for (int v = 0; v < nv; ++v) {
                        if (S.dbc[v] > 0)
                            for (int d = 0; d < 3; ++d) b[3 * v + d] = S.x0[3 * v + d] * (pw * dt2Inv);
                        else if (dragw[v] > (T)0)
                            for (int d = 0; d < 3; ++d) b[3 * v + d] = dbcx[3 * v + d] * dragw[v];
                    }
                if (chol) {
                    S.chol.template solve3<T>(b.data(), sn.data());
                    T acc = 0;
                    for (size_t k = 0; k < (size_t)3 * nv; ++k) {
                        T dlt = S.prev[k] - sn[k];
                        acc += dlt * dlt;
                    }
                    err = acc / (T)(3 * nv);
                    S.prev = sn;
                } else {
                    const T rho = (T)prm.rho;
                    if (i <= 10) omega = 1;
                    else if (i == 11) omega = (T)2 / ((T)2 - rho * rho);
                    else omega = (T)4 / ((T)4 - rho * rho * omega);
#pragma omp parallel for schedule(static)
                    for (int v = 0; v < nv; ++v) {
                        T c = mdt2s[v], md = S.stiff_diag[v];
                        for (int d = 0; d < 3; ++d) {
                            size_t k = 3 * (size_t)v + d;
                            // dragged vertices keep the iterate (getErrorKern, pdUtil.cu:200-205)
                            T nx = dragw[v] > (T)0 ? sn[k] : (b[k] - c * sn[k]) / (c + md) + sn[k];
                            // 0.9 is a double literal in the reference (pdUtil.cu:221)
                            nx = (T)(0.9 * (double)(nx - sn[k]) + (double)sn[k]);
                            nx = (nx - S.prev[k]) * omega + S.prev[k];
                            S.prev[k] = sn[k];
                            sn[k] = nx;
                        }
                    }
                }
            }
            if (iters_out) iters_out[step] = it;
            // updateVelPos (pdUtil.cu:180-193), X <- XTilde (pdSolver.cu:227),
            // fixed-body correction of XTilde and V (pdSolver.cu:228-231)
            for (int v = 0; v < nv; ++v) {
                for (int d = 0; d < 3; ++d) {
                    size_t k = 3 * (size_t)v + d;
                    V[k] = dragw[v] > (T)0 ? (T)0 : (sn[k] - XT[k]) * dtInv;
                    XT[k] = sn[k];
                    X[k] = sn[k];
                }
                if (!fixed.empty()) collide<T>(fixed, mu_t, mu_n, &XT[3 * (size_t)v], &V[3 * (size_t)v]);
            }
        }
        if (step_seconds) *step_seconds = now_seconds() - t_start;
    }

    void state(float* Xo, float* Vo, float* XTo) const override {
        for (size_t i = 0; i < (size_t)3 * nv; ++i) {
            if (Xo) Xo[i] = (float)X[i];
            if (Vo) Vo[i] = (float)V[i];
            if (XTo) XTo[i] = (float)XT[i];
        }
    }
};

template <class T>
int simulate(int nv, int nt, const float* X0, float* Xio, float* Vio, const uint32_t* tets, const float* mass,
             const float* mu, const float* dbc, const orc_params* p, int nsteps, int* iters_out, double* step_seconds,
             const orc_scene* sc) {
    Runner<T> r;
    const int st = r.setup(nv, nt, X0, Xio, Vio, tets, mass, mu, dbc, p, sc);
    if (st != 0) return st;
    r.run(nsteps, 0, iters_out, step_seconds);
    r.state(Xio, Vio, (sc && sc->XT) ? sc->XT : nullptr);
    return 0;
}

}  // namespace

extern "C" {

int orc_simulate(int nv, int nt, const float* X0, float* X, float* V, const uint32_t* tets, const float* mass,
                 const float* mu, const float* dbc, const orc_params* p, int precision, int nsteps, int nthreads,
                 int* iters_out, double* step_seconds) {
    if (nv <= 0 || nt <= 0 || !X0 || !X || !V || !tets || !mass || !mu || !p) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (precision == 64)
        return simulate<double>(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nsteps, iters_out, step_seconds, nullptr);
    return simulate<float>(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nsteps, iters_out, step_seconds, nullptr);
}

int orc_simulate_scene(int nv, int nt, const float* X0, float* X, float* V, const uint32_t* tets, const float* mass,
                       const float* mu, const float* dbc, const orc_params* p, int precision, int nsteps,
                       int nthreads, int* iters_out, double* step_seconds, const orc_scene* scene) {
    if (nv <= 0 || nt <= 0 || !X0 || !X || !V || !tets || !mass || !mu || !p) return -1;
    if (scene && ((scene->drag_w && !scene->drag_off) || (scene->nfixed > 0 && !scene->fixed) || scene->nfixed < 0))
        return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (precision == 64)
        return simulate<double>(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nsteps, iters_out, step_seconds, scene);
    return simulate<float>(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nsteps, iters_out, step_seconds, scene);
}

orc_runner* orc_runner_create(int nv, int nt, const float* X0, const float* X, const float* V, const uint32_t* tets,
                              const float* mass, const float* mu, const float* dbc, const orc_params* p,
                              int precision, int nthreads) {
    if (nv <= 0 || nt <= 0 || !X0 || !X || !V || !tets || !mass || !mu || !p) return nullptr;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    RunnerBase* r = nullptr;
    int st = 0;
    if (precision == 64) {
        auto* q = new Runner<double>();
        st = q->setup(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nullptr);
        r = q;
    } else {
        auto* q = new Runner<float>();
        st = q->setup(nv, nt, X0, X, V, tets, mass, mu, dbc, p, nullptr);
        r = q;
    }
    if (st != 0) {
        delete r;
        return nullptr;
    }
    return reinterpret_cast<orc_runner*>(r);
}

int orc_runner_run(orc_runner* r, int nsteps, int num_iterations, int* iters_out, double* step_seconds) {
    if (!r || nsteps < 0) return -1;
    reinterpret_cast<RunnerBase*>(r)->run(nsteps, num_iterations, iters_out, step_seconds);
    return 0;
}

int orc_runner_state(const orc_runner* r, float* X, float* V) {
    if (!r) return -1;
    reinterpret_cast<const RunnerBase*>(r)->state(X, V, nullptr);
    return 0;
}

void orc_runner_destroy(orc_runner* r) { delete reinterpret_cast<RunnerBase*>(r); }

void orc_rotations(int n, const double* F, double* R, int precision) {
    for (int k = 0; k < n; ++k) {
        if (precision == 64) {
            double f[3][3], r[3][3];
            std::memcpy(f, F + 9 * (size_t)k, sizeof(f));
            polar_rotation_f64(f, r);
            std::memcpy(R + 9 * (size_t)k, r, sizeof(r));
        } else {
            float f[3][3], r[3][3];
            for (int i = 0; i < 9; ++i) f[i / 3][i % 3] = (float)F[9 * (size_t)k + i];
            polar_rotation_f32(f, r);
            for (int i = 0; i < 9; ++i) R[9 * (size_t)k + i] = r[i / 3][i % 3];
        }
    }
}

int orc_local_rhs(int nv, int nt, const float* X0, const uint32_t* tets, const float* mass, const float* mu,
                  const float* dbc, float dt, float positional_weight, const double* q, const double* s_old,
                  int jacobi_form, double* b) {
    Sim<double> S;
    S.nv = nv; S.nt = nt; S.tets = tets;
    TetGeom g;
    if (!tet_geometry(nv, nt, X0, tets, mu, g)) return -1;
    S.dminv = g.dminv;
    S.coef = g.coef;
    S.inc = build_incidence(nv, nt, tets);
    S.P.resize((size_t)nt * 12);
    S.mdt2.resize(nv);
    double dt2 = (double)dt * (double)dt;
    for (int v = 0; v < nv; ++v) S.mdt2[v] = ((double)mass[v] + (dbc ? (double)dbc[v] : 0.0) * positional_weight) / dt2;
    local_rhs<double>(S, q, s_old, jacobi_form != 0, b, S.mdt2.data());
    return 0;
}

long orc_system_csr(int nv, int nt, const float* X0, const uint32_t* tets, const float* mass, const float* mu,
                    const float* dbc, float dt, float positional_weight, int64_t* rowptr, int32_t* colind,
                    double* val) {
    TetGeom g;
    if (!tet_geometry(nv, nt, X0, tets, mu, g)) return -1;
    std::vector<double> mdt2(nv);
    double dt2 = (double)dt * (double)dt;
    for (int v = 0; v < nv; ++v) mdt2[v] = ((double)mass[v] + (dbc ? (double)dbc[v] : 0.0) * positional_weight) / dt2;
    CSR K = assemble_K(nv, nt, tets, g, mdt2, nullptr);
    if (rowptr) std::copy(K.p.begin(), K.p.end(), rowptr);
    if (colind) std::copy(K.i.begin(), K.i.end(), colind);
    if (val) std::copy(K.x.begin(), K.x.end(), val);
    return (long)K.i.size();
}

int orc_solve3(int nv, int nt, const float* X0, const uint32_t* tets, const float* mass, const float* mu,
               const float* dbc, float dt, float positional_weight, const double* b, double* x) {
    TetGeom g;
    if (!tet_geometry(nv, nt, X0, tets, mu, g)) return -1;
    std::vector<double> mdt2(nv);
    double dt2 = (double)dt * (double)dt;
    for (int v = 0; v < nv; ++v) mdt2[v] = ((double)mass[v] + (dbc ? (double)dbc[v] : 0.0) * positional_weight) / dt2;
    CSR K = assemble_K(nv, nt, tets, g, mdt2, nullptr);
    SpChol c;
    if (!c.factor(K, X0)) return -2;
    c.solve3<double>(b, x);
    return 0;
}

void* orc_factor_csr(int n, const int64_t* rowptr, const int32_t* colind, const double* val, const float* xyz) {
    if (n <= 0 || !rowptr || !colind || !val || !xyz) return nullptr;
    CSR K;
    K.n = n;
    K.p.assign(rowptr, rowptr + n + 1);
    K.i.assign(colind, colind + rowptr[n]);
    K.x.assign(val, val + rowptr[n]);
    SpChol* c = new SpChol();
    if (!c->factor(K, xyz)) {
        delete c;
        return nullptr;
    }
    return c;
}

void orc_solve_factored(const void* h, const double* b, double* x) {
    const SpChol* c = (const SpChol*)h;
    const int n = c->n;
    std::vector<double> y(n);
    for (int k = 0; k < n; ++k) y[k] = b[c->perm[k]];
    for (int j = 0; j < n; ++j) {
        y[j] /= c->Lx[c->Lp[j]];
        for (int64_t q = c->Lp[j] + 1; q < c->Lp[j + 1]; ++q) y[c->Li[q]] -= c->Lx[q] * y[j];
    }
    for (int j = n - 1; j >= 0; --j) {
        double a = y[j];
        for (int64_t q = c->Lp[j] + 1; q < c->Lp[j + 1]; ++q) a -= c->Lx[q] * y[c->Li[q]];
        y[j] = a / c->Lx[c->Lp[j]];
    }
    for (int k = 0; k < n; ++k) x[c->perm[k]] = y[k];
}

long orc_factor_nnz(const void* h) { return h ? (long)((const SpChol*)h)->Lp.back() : 0; }

void orc_free_factor(void* h) { delete (SpChol*)h; }

}  // extern "C"
