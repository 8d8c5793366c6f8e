// Host-side layout of a PD system for the engine's kernels.
//
// Reference counterparts: the per-tet precompute of FEMSolver's constructor
// (femSolver.cu:7-17 -> computeInvDmV0, solverUtil.cuh:108-138) and the
// per-vertex coefficients of PdSolver::SolverPrepare (pdUtil.cu:9-54).
// What is new here is the data layout: vertices and tets are renumbered
// along a Morton curve, tets are cut into tiles whose vertex "patch" fits in
// shared memory, and each tet stores 16-bit patch-local corner ids.
#include <algorithm>
#include <cmath>
#include <tuple>
#include <cstring>
#include <numeric>

#include "engine.h"

namespace pdgb {

namespace {

inline uint64_t spread_bits21(uint64_t x) {
    x &= 0x1fffffULL;
    x = (x | (x << 32)) & 0x1f00000000ffffULL;
    x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}

struct Quantizer {
    double lo[3], scale[3];
    Quantizer(int nv, const float* X) {
        double hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = 1e300; hi[d] = -1e300; }
        for (int v = 0; v < nv; ++v)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], (double)X[3 * v + d]);
                hi[d] = std::max(hi[d], (double)X[3 * v + d]);
            }
        double ext = 0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, hi[d] - lo[d]);
        if (!(ext > 0)) ext = 1;
        for (int d = 0; d < 3; ++d) scale[d] = 2097151.0 / ext;
    }
    uint64_t key(double x, double y, double z) const {
        auto q = [&](double v, int d) {
            double t = (v - lo[d]) * scale[d];
            if (!(t > 0)) t = 0;
            if (t > 2097151.0) t = 2097151.0;
            return (uint64_t)t;
        };
        return spread_bits21(q(x, 0)) | (spread_bits21(q(y, 1)) << 1) | (spread_bits21(q(z, 2)) << 2);
    }
};

}  // namespace

std::vector<float> chebyshev_omegas(int n, float rho) {
    std::vector<float> w(std::max(n, 0));
    float omega = 1.0f;
    for (int i = 0; i < n; ++i) {
        if (i <= 10) omega = 1;
        else if (i == 11) omega = 2 / (2 - rho * rho);
        else omega = 4 / (4 - rho * rho * omega);
        w[i] = omega;
    }
    return w;
}

// Tiles: greedy runs of the Morton-ordered tets, cut at max_tile_tets tets
// (at most kTileTets), when the patch would exceed kMaxPatch vertices, or
// at a body boundary.  Each tile gets its vertex patch (pinned bit from the
// caller-order pin flags) and its incidence lists.  The patch is ordered by
// run length (the vertex's corners in the tile), longest first, then by
// vertex id: the local step sums one patch vertex's run per thread, and a warp
// loops as long as its longest run, so neighbouring threads should have runs
// of nearly the same length (in id order a warp mixes interior vertices, ~20
// corners, with patch-boundary vertices of 1 to 5).
void build_tiles(HostLayout& L, const float* dbc, int max_tile_tets) {
    const int nv = L.nv, nt = L.nt, nbodies = L.nbodies;
    const int cap = max_tile_tets > 0 ? std::min(max_tile_tets, kTileTets) : kTileTets;
    L.tile_cap = cap;
    L.tile_tet_ptr.assign(1, 0);
    L.tile_vptr.assign(1, 0);
    L.tile_verts.clear();
    L.inc_end.clear();
    L.inc_ent.assign((size_t)4 * ((nt + 31) & ~31), 0);  // padded to 4 nt_pad
    std::vector<int> mark(nv, -1), loc(nv, 0), cnt, run(nv, 0);
    std::vector<int> patch;
    patch.reserve(kMaxPatch);
    std::vector<int> vcount(nv, 0);  // corners of each patch vertex in the open tile
    L.max_patch = 0;
    int tile = 0, start = 0;
    int body_cursor = 0, next_body_start = nbodies > 1 ? L.body_itstart[1] : nt;
    auto close_tile = [&](int end) {
        std::sort(patch.begin(), patch.end(),
                  [&](int a, int b) { return vcount[a] != vcount[b] ? vcount[a] > vcount[b] : a < b; });
        const int np = (int)patch.size();
        for (int k = 0; k < np; ++k) loc[patch[k]] = k;
        // incidence lists in patch order
        cnt.assign(np + 1, 0);
        for (int i = start; i < end; ++i)
            for (int c = 0; c < 4; ++c) cnt[loc[L.tets_int[4 * (size_t)i + c]] + 1]++;
        for (int k = 0; k < np; ++k) cnt[k + 1] += cnt[k];
        for (int k = 0; k < np; ++k) L.inc_end.push_back((uint16_t)cnt[k + 1]);
        // corner record: patch index k and the corner's rank r within k's
        // run of slots (tile order), so that a patch vertex's corners are one
        // contiguous run of slots and the slot is inc_end[k-1] + r
        for (int i = start; i < end; ++i)
            for (int c = 0; c < 4; ++c) {
                const int k = loc[L.tets_int[4 * (size_t)i + c]];
                const int r = run[k]++;
                L.inc_ent[4 * (size_t)i + c] = (uint16_t)(k | (r << kPatchBits));
            }
        for (int k = 0; k < np; ++k) run[k] = 0;
        L.max_patch = std::max(L.max_patch, np);
        for (int v : patch) {
            const int o = L.vperm[v];
            const bool pinned = dbc && dbc[o] > 0.f;
            L.tile_verts.push_back((uint32_t)v | (pinned ? kPinnedBit : 0u));
        }
        L.tile_vptr.push_back((int)L.tile_verts.size());
        L.tile_tet_ptr.push_back(end);
        patch.clear();
        ++tile;
        start = end;
    };
    for (int i = 0; i < nt; ++i) {
        const uint32_t* id = &L.tets_int[4 * (size_t)i];
        int fresh = 0;
        for (int k = 0; k < 4; ++k) {
            bool dup = mark[id[k]] == tile;
            for (int j = 0; j < k; ++j) dup = dup || id[j] == id[k];
            fresh += !dup;
        }
        const bool new_body = i > start && i == next_body_start;
        bool run_full = false;  // a corner run would outgrow the rank field
        for (int k = 0; k < 4; ++k) {
            int extra = 0;
            for (int j = 0; j < 4; ++j) extra += id[j] == id[k];
            run_full = run_full || (mark[id[k]] == tile && vcount[id[k]] + extra > kMaxRun);
        }
        if (i - start == cap || (int)patch.size() + fresh > kMaxPatch || new_body || run_full) close_tile(i);
        while (i >= next_body_start && body_cursor < nbodies) next_body_start = L.body_itstart[++body_cursor];
        for (int k = 0; k < 4; ++k)
            if (mark[id[k]] != tile) {
                mark[id[k]] = tile;
                vcount[id[k]] = 0;
                patch.push_back((int)id[k]);
            }
        for (int k = 0; k < 4; ++k) vcount[id[k]]++;
    }
    close_tile(nt);
    L.ntiles = tile;
    L.tile_verts.insert(L.tile_verts.end(), kLayoutTailPad, 0u);
    L.inc_end.insert(L.inc_end.end(), kLayoutTailPad, (uint16_t)0);
}

void build_layout(int nv, int nt, const float* X0, const uint32_t* tets, const float* mass, const float* mu,
                  const float* dbc, const pdgb_params& prm, HostLayout& L, int nbodies, const int* body_vstart,
                  int max_tile_tets) {
    if (nv <= 0 || nt <= 0) throw Error{PDGB_ERR_INVALID_ARGUMENT, "num_verts and num_tets must be positive"};
    for (size_t i = 0; i < (size_t)4 * nt; ++i)
        if (tets[i] >= (uint32_t)nv)
            throw Error{PDGB_ERR_BAD_MESH, "tet " + std::to_string(i / 4) + " references vertex " +
                                               std::to_string(tets[i]) + " >= num_verts"};
    for (size_t i = 0; i < (size_t)3 * nv; ++i)
        if (!std::isfinite(X0[i])) throw Error{PDGB_ERR_NONFINITE, "non-finite rest position"};
    L.nv = nv;
    L.nt = nt;
    Quantizer qz(nv, X0);
    // body of every caller vertex (all 0 for a single body)
    if (nbodies < 1) throw Error{PDGB_ERR_INVALID_ARGUMENT, "nbodies must be >= 1"};
    std::vector<int> vbody(nv, 0);
    if (body_vstart) {
        if (body_vstart[0] != 0 || body_vstart[nbodies] != nv)
            throw Error{PDGB_ERR_INVALID_ARGUMENT, "body vertex ranges must cover all vertices"};
        for (int b = 0; b < nbodies; ++b) {
            if (body_vstart[b + 1] <= body_vstart[b]) throw Error{PDGB_ERR_INVALID_ARGUMENT, "empty body"};
            for (int v = body_vstart[b]; v < body_vstart[b + 1]; ++v) vbody[v] = b;
        }
    }
    L.nbodies = nbodies;
    // ---- vertex order (body, Morton)
    {
        std::vector<std::tuple<int, uint64_t, int>> key(nv);
        for (int v = 0; v < nv; ++v) key[v] = {vbody[v], qz.key(X0[3 * v], X0[3 * v + 1], X0[3 * v + 2]), v};
        std::sort(key.begin(), key.end());
        L.vperm.resize(nv);
        L.viperm.resize(nv);
        for (int i = 0; i < nv; ++i) {
            L.vperm[i] = std::get<2>(key[i]);
            L.viperm[std::get<2>(key[i])] = i;
        }
        L.body_ivstart.assign(nbodies + 1, 0);
        for (int v = 0; v < nv; ++v) L.body_ivstart[vbody[v] + 1]++;
        for (int b = 0; b < nbodies; ++b) L.body_ivstart[b + 1] += L.body_ivstart[b];
    }
    // ---- tet order (body, centroid Morton); a tet must not span bodies
    {
        std::vector<std::tuple<int, uint64_t, int>> key(nt);
        for (int t = 0; t < nt; ++t) {
            double c[3] = {0, 0, 0};
            const int b = vbody[tets[4 * (size_t)t]];
            for (int k = 0; k < 4; ++k) {
                const uint32_t v = tets[4 * (size_t)t + k];
                if (vbody[v] != b) throw Error{PDGB_ERR_BAD_MESH, "tet " + std::to_string(t) + " spans two bodies"};
                for (int d = 0; d < 3; ++d) c[d] += 0.25 * X0[3 * (size_t)v + d];
            }
            key[t] = {b, qz.key(c[0], c[1], c[2]), t};
        }
        std::sort(key.begin(), key.end());
        L.tperm.resize(nt);
        L.body_itstart.assign(nbodies + 1, 0);
        for (int i = 0; i < nt; ++i) {
            L.tperm[i] = std::get<2>(key[i]);
            L.body_itstart[std::get<0>(key[i]) + 1]++;
        }
        for (int b = 0; b < nbodies; ++b) L.body_itstart[b + 1] += L.body_itstart[b];
    }
    L.tets_int.resize((size_t)4 * nt);
    for (int i = 0; i < nt; ++i)
        for (int k = 0; k < 4; ++k) L.tets_int[4 * (size_t)i + k] = (uint32_t)L.viperm[tets[4 * (size_t)L.tperm[i] + k]];
    // ---- geometry: DmInv and V0 * w (solverUtil.cuh:98-138, pdUtil.cu:19).
    // The local step reads g = sqrt(V0 w) and D' = g DmInv: F' = Ds D' = g F
    // has the same closest rotation R as F, and c (R - F) DmInv^T =
    // (g R - F') D'^T, c R DmInv^T = g R D'^T.  Planes: D'[0..3] (float4),
    // D'[4..7] (float4), {D'[8], g} (float2).
    L.nt_pad = (nt + 31) & ~31;
    L.geo.assign((size_t)10 * L.nt_pad, 0.f);
    L.dminv_d.resize((size_t)9 * nt);
    L.coef_d.resize(nt);
    for (int i = 0; i < nt; ++i) {
        const int t = L.tperm[i];
        const uint32_t* id = tets + 4 * (size_t)t;
        double D[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) D[r][c] = (double)X0[3 * (size_t)id[c + 1] + r] - (double)X0[3 * (size_t)id[0] + r];
        const double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) -
                           D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                           D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
        if (!(det != 0.0) || !std::isfinite(det))
            throw Error{PDGB_ERR_BAD_MESH, "tet " + std::to_string(t) + " has zero rest volume"};
        double inv[9];
        inv[0] = (D[1][1] * D[2][2] - D[1][2] * D[2][1]) / det;
        inv[1] = (D[0][2] * D[2][1] - D[0][1] * D[2][2]) / det;
        inv[2] = (D[0][1] * D[1][2] - D[0][2] * D[1][1]) / det;
        inv[3] = (D[1][2] * D[2][0] - D[1][0] * D[2][2]) / det;
        inv[4] = (D[0][0] * D[2][2] - D[0][2] * D[2][0]) / det;
        inv[5] = (D[0][2] * D[1][0] - D[0][0] * D[1][2]) / det;
        inv[6] = (D[1][0] * D[2][1] - D[1][1] * D[2][0]) / det;
        inv[7] = (D[0][1] * D[2][0] - D[0][0] * D[2][1]) / det;
        inv[8] = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) / det;
        if (!(mu[t] >= 0.f) || !std::isfinite(mu[t]))
            throw Error{PDGB_ERR_BAD_MESH, "tet " + std::to_string(t) + " has a negative or non-finite weight"};
        const double coef = std::fabs(det) / 6.0 * (double)mu[t];
        const double g = std::sqrt(coef);
        const size_t np4 = (size_t)4 * L.nt_pad;
        for (int k = 0; k < 9; ++k) {
            L.dminv_d[9 * (size_t)i + k] = inv[k];
            const float v = (float)(g * inv[k]);
            // a nearly flat tet has a finite double inverse that overflows float
            if (!std::isfinite(inv[k]) || !std::isfinite(v))
                throw Error{PDGB_ERR_BAD_MESH, "tet " + std::to_string(t) + " is too flat (its DmInv overflows float)"};
            if (k < 4) L.geo[4 * (size_t)i + k] = v;
            else if (k < 8) L.geo[np4 + 4 * (size_t)i + (k - 4)] = v;
            else L.geo[2 * np4 + 2 * (size_t)i] = v;
        }
        L.coef_d[i] = coef;
        L.geo[2 * np4 + 2 * (size_t)i + 1] = (float)g;
    }
    build_tiles(L, dbc, max_tile_tets);
    // ---- rest positions (internal order)
    L.x0.resize(nv);
    for (int i = 0; i < nv; ++i) {
        const int o = L.vperm[i];
        L.x0[i] = make_float4(X0[3 * o], X0[3 * o + 1], X0[3 * o + 2], 0.f);
    }
    build_vertex_coefficients(mass, dbc, prm, L);
}

void build_vertex_coefficients(const float* mass, const float* dbc, const pdgb_params& prm, HostLayout& L) {
    const int nv = L.nv, nt = L.nt;
    // stiffness diagonal: sum_t c_t (B_t^T B_t)_jj  (pdUtil.cu:21-24)
    std::vector<double> md(nv, 0.0);
    for (int i = 0; i < nt; ++i) {
        const double* D = &L.dminv_d[9 * (size_t)i];
        double B[3][4];
        for (int r = 0; r < 3; ++r) {
            B[r][1] = D[0 * 3 + r];
            B[r][2] = D[1 * 3 + r];
            B[r][3] = D[2 * 3 + r];
            B[r][0] = -(B[r][1] + B[r][2] + B[r][3]);
        }
        for (int j = 0; j < 4; ++j)
            md[L.tets_int[4 * (size_t)i + j]] += L.coef_d[i] * (B[0][j] * B[0][j] + B[1][j] * B[1][j] + B[2][j] * B[2][j]);
    }
    const float dt = prm.dt;
    const float dt2 = dt * dt;
    const float dtInv = 1.0f / dt;
    const float dt2Inv = dtInv * dtInv;
    const float wpin = prm.positional_weight * dt2Inv;
    L.coef.resize(nv);
    L.pin_rhs.resize(nv);
    for (int i = 0; i < nv; ++i) {
        const int o = L.vperm[i];
        const float m = mass[o];
        const float pin = dbc ? dbc[o] : 0.f;
        const float mdt2 = (m + pin * prm.positional_weight) / dt2;  // setMDt_2, pdUtil.cu:48
        L.coef[i] = make_float4(mdt2, (float)md[i], pin > 0.f ? 1.f : 0.f, m);
        const float4 x0 = L.x0[i];
        L.pin_rhs[i] = make_float4(x0.x * wpin, x0.y * wpin, x0.z * wpin, 0.f);  // computeDBCLocal, pdUtil.cu:155-157
    }
}

}  // namespace pdgb
