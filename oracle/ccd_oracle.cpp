/*
 * CPU oracle for continuous collision between bodies: TEST INFRASTRUCTURE
 * ONLY (loaded by tests/ through oracle.py; the engine never calls it).
 *
 * Restates, in plain float C++, what the reference runs after a PD step when
 * collision handling is on (PdSolver::Update, pdSolver.cu:218-224):
 *   - candidates: every pair of surface triangles of different bodies that
 *     share no vertex and whose swept boxes (X -> XTilde) overlap
 *     (BVH traversal, broadphase.cu:331-407 with ignoreSelfCollision; the
 *     oracle enumerates the pairs directly, which gives the same set);
 *   - queries: for a pair (A, B), each vertex of A against face B and each
 *     edge of A against each edge of B, and the same with A and B swapped
 *     (fillQuery, broadphase.cu:272-305), each edge's ends ordered by id
 *     (sortEachQuery, broadphase.cu:440-461);
 *   - narrow phase: coplanarity times from the cubic in t of
 *     det[x1-x0, x2-x0, x3-x0](t), then a proximity + barycentric test at
 *     each root in [0, 1] (ccdCollisionTest, intersections.cu:286-334);
 *     the formulation is Bridson, Fedkiw and Anderson, "Robust treatment of
 *     collisions, contact and friction for cloth animation" (2002);
 *   - reduction: per vertex (face queries) and per edge (edge queries) the
 *     earliest contact (narrowphase.cu:8-56, 118-127); a vertex touched by
 *     an earliest contact before t = 1 gets tI = 0.5 and that contact's
 *     normal (storeTi, narrowphase.cu:72-113);
 *   - response: tI < 1 -> V = -(d . n) n with d = XTilde - X and X kept,
 *     else X = XTilde (CCDKernel, collisionUtil.cu:50-70).
 *
 * Thresholds are double constants compared against float values, as in the
 * reference (its literals are doubles); the arithmetic itself is float.
 *
 * Deterministic where the reference is not: the reference picks among equal
 * contact times by an unstable sort and lets concurrent writes of a
 * vertex's normal race; here ties go to the smaller face / edge index, and
 * a vertex touched by several contacts takes the normal of the earliest one
 * (then the smaller source key).  The GPU engine uses the same rule.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
};
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float len2(V3 a) { return dot(a, a); }
inline float len(V3 a) { return std::sqrt(len2(a)); }
inline V3 unit(V3 a) { return (1.0f / len(a)) * a; }
inline float triple(V3 u, V3 v, V3 w) { return dot(u, cross(v, w)); }

// Real roots of a x^2 + b x + c (numerically stable form); returns the count
// (0 when the discriminant is negative, x[0] then holds the vertex -b/2a).
int quad_roots(float a, float b, float c, float* x) {
    const float d = b * b - 4 * a * c;
    if (d < 0) {
        x[0] = -b / (2 * a);
        return 0;
    }
    const float sgn = (b > 0) ? 1.0f : (b < 0 ? -1.0f : 0.0f);
    const float q = -(b + sgn * std::sqrt(d)) / 2;
    int n = 0;
    if (std::fabs(a) > 1e-12 * std::fabs(q)) x[n++] = q / a;
    if (std::fabs(q) > 1e-12 * std::fabs(c)) x[n++] = c / q;
    if (n == 2 && x[0] > x[1]) std::swap(x[0], x[1]);
    return n;
}

// Newton iteration on the cubic from x0; with dir != 0 the start is first
// moved off the critical point by the local quadratic model.
float cubic_newton(float a, float b, float c, float d, float x0, int dir) {
    if (dir != 0) {
        const float y0 = d + x0 * (c + x0 * (b + x0 * a));
        const float ddy0 = 2 * b + x0 * (6 * a);
        if (ddy0 != 0) x0 += dir * std::sqrt(std::fabs(2 * y0 / ddy0));
    }
    for (int it = 0; it < 100; ++it) {
        const float y = d + x0 * (c + x0 * (b + x0 * a));
        const float dy = c + x0 * (2 * b + x0 * 3 * a);
        if (dy == 0) return x0;
        const float x1 = x0 - y / dy;
        if (std::fabs(x0 - x1) < 1e-6) return x0;
        x0 = x1;
    }
    return x0;
}

// Real roots of a x^3 + b x^2 + c x + d, bracketed by the critical points.
int cubic_roots(float a, float b, float c, float d, float* x) {
    float xc[2];
    const int ncrit = quad_roots(3 * a, 2 * b, c, xc);
    if (ncrit == 0) {
        x[0] = cubic_newton(a, b, c, d, xc[0], 0);
        return 1;
    }
    if (ncrit == 1) return quad_roots(b, c, d, x);
    const float yc[2] = {d + xc[0] * (c + xc[0] * (b + xc[0] * a)), d + xc[1] * (c + xc[1] * (b + xc[1] * a))};
    int n = 0;
    if (yc[0] * a >= 0) x[n++] = cubic_newton(a, b, c, d, xc[0], -1);
    if (yc[0] * yc[1] <= 0) {
        const int closer = std::fabs(yc[0]) < std::fabs(yc[1]) ? 0 : 1;
        x[n++] = cubic_newton(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
    }
    if (yc[1] * a <= 0) x[n++] = cubic_newton(a, b, c, d, xc[1], 1);
    return n;
}

// Signed distance of point p to the plane of face (y0, y1, y2), normal n and
// barycentric weights w (w0 = 1, w1..3 = minus the face coordinates).
float face_distance(V3 p, V3 y0, V3 y1, V3 y2, V3& n, float w[4]) {
    n = cross(unit(y1 - y0), unit(y2 - y0));
    if (len2(n) < 1e-6) return FLT_MAX;
    n = unit(n);
    const float h = dot(p - y0, n);
    const float b0 = triple(y1 - p, y2 - p, n), b1 = triple(y2 - p, y0 - p, n), b2 = triple(y0 - p, y1 - p, n);
    const float s = b0 + b1 + b2;
    w[0] = 1;
    w[1] = -b0 / s;
    w[2] = -b1 / s;
    w[3] = -b2 / s;
    return h;
}

// Signed distance between the lines of edges (x0, x1) and (y0, y1), normal n
// and weights (w0, w1 on the first edge, -w2, -w3 on the second).
float edge_distance(V3 x0, V3 x1, V3 y0, V3 y1, V3& n, float w[4]) {
    n = cross(unit(x1 - x0), unit(y1 - y0));
    if (len2(n) < 1e-6) return FLT_MAX;
    n = unit(n);
    const float h = dot(x0 - y0, n);
    const float a0 = triple(y1 - x1, y0 - x1, n), a1 = triple(y0 - x0, y1 - x0, n);
    const float b0 = triple(x0 - y1, x1 - y1, n), b1 = triple(x1 - y0, x0 - y0, n);
    w[0] = a0 / (a0 + a1);
    w[1] = a1 / (a0 + a1);
    w[2] = -b0 / (b0 + b1);
    w[3] = -b1 / (b0 + b1);
    return h;
}

// Earliest contact time in [0, 1] of a point-face (face = true: point q0,
// face q1..q3) or edge-edge (q0q1 against q2q3) query; 1 when none.
float contact_time(bool face, const V3 x[4], const V3 v[4], V3& n) {
    const V3 x01 = x[1] - x[0], x02 = x[2] - x[0], x03 = x[3] - x[0];
    const V3 v01 = v[1] - v[0], v02 = v[2] - v[0], v03 = v[3] - v[0];
    const float a0 = triple(x01, x02, x03);
    const float a1 = triple(v01, x02, x03) + triple(x01, v02, x03) + triple(x01, x02, v03);
    const float a2 = triple(x01, v02, v03) + triple(v01, x02, v03) + triple(v01, v02, x03);
    const float a3 = triple(v01, v02, v03);
    n = {0, 0, 0};
    if (std::fabs(a0) < 1e-12 * len(x01) * len(x02) * len(x03)) return 1.0f;  // coplanar at t = 0
    float t[3];
    const int nr = cubic_roots(a3, a2, a1, a0, t);
    for (int i = 0; i < nr; ++i) {
        if (t[i] < -1e-12 || t[i] > 1) continue;
        V3 xt[4];
        for (int k = 0; k < 4; ++k) xt[k] = x[k] + t[i] * v[k];
        float w[4] = {0, 0, 0, 0};
        float d;
        bool inside;
        if (face) {
            d = face_distance(xt[0], xt[1], xt[2], xt[3], n, w);
            inside = std::min(-w[1], std::min(-w[2], -w[3])) >= -1e-3;
        } else {
            d = edge_distance(xt[0], xt[1], xt[2], xt[3], n, w);
            inside = std::min(w[0], std::min(w[1], std::min(-w[2], -w[3]))) >= -1e-3;
        }
        if (dot(n, w[1] * v[1] + w[2] * v[2] + w[3] * v[3]) > 0) n = -1.0f * n;
        if (std::fabs(d) < 1e-6 && inside) return t[i];
    }
    return 1.0f;
}

inline uint64_t time_key(float t, uint32_t tag) {
    const float tk = t > 0.f ? t : 0.f;
    uint32_t bits;
    std::memcpy(&bits, &tk, 4);
    return ((uint64_t)bits << 32) | tag;
}

}  // namespace

extern "C" {

/* Contact time and normal of one query, float, as the reference evaluates
 * it: face != 0 -> vertex ids[0] against face ids[1..3], else edge
 * ids[0]ids[1] against edge ids[2]ids[3].  X, XT: [3 nv]. */
float orc_ccd_query(int face, const uint32_t* ids, const float* X, const float* XT, float* normal) {
    V3 x[4], v[4];
    for (int k = 0; k < 4; ++k) {
        const float* p = X + 3 * (size_t)ids[k];
        const float* q = XT + 3 * (size_t)ids[k];
        x[k] = {p[0], p[1], p[2]};
        v[k] = V3{q[0], q[1], q[2]} - x[k];
    }
    V3 n;
    const float t = contact_time(face != 0, x, v, n);
    if (normal) {
        normal[0] = n.x;
        normal[1] = n.y;
        normal[2] = n.z;
    }
    return t;
}

/* Collision detection between bodies.  tris: [3 ntris] vertex ids;
 * tri_body: [ntris] body of each triangle.  Outputs tI [nv] (1 or 0.5) and
 * normals [3 nv] (zero where tI = 1).  stats (nullable): {candidate pairs,
 * face queries before contact, vertices marked}.  Returns 0. */
int orc_ccd_detect(int nv, int ntris, const uint32_t* tris, const int* tri_body, const float* X, const float* XT,
                   float* tI, float* normals, long long* stats) {
    auto P = [&](const float* a, uint32_t i) { return V3{a[3 * i], a[3 * i + 1], a[3 * i + 2]}; };
    // swept boxes
    std::vector<V3> lo(ntris), hi(ntris);
    for (int t = 0; t < ntris; ++t) {
        V3 mn{FLT_MAX, FLT_MAX, FLT_MAX}, mx{-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < 3; ++k)
            for (const float* a : {X, XT}) {
                const V3 p = P(a, tris[3 * t + k]);
                mn = {std::min(mn.x, p.x), std::min(mn.y, p.y), std::min(mn.z, p.z)};
                mx = {std::max(mx.x, p.x), std::max(mx.y, p.y), std::max(mx.z, p.z)};
            }
        lo[t] = mn;
        hi[t] = mx;
    }
    // edge ids: unique (min, max) pairs in lexicographic order
    std::vector<std::pair<uint32_t, uint32_t>> edges;
    for (int t = 0; t < ntris; ++t)
        for (int k = 0; k < 3; ++k) {
            uint32_t a = tris[3 * t + k], b = tris[3 * t + (k + 1) % 3];
            if (a > b) std::swap(a, b);
            edges.push_back({a, b});
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    auto edge_id = [&](uint32_t a, uint32_t b) {
        if (a > b) std::swap(a, b);
        return (uint32_t)(std::lower_bound(edges.begin(), edges.end(), std::make_pair(a, b)) - edges.begin());
    };
    const uint64_t kNone = ~0ull;
    std::vector<uint64_t> vf_best(nv, kNone), ee_best(edges.size(), kNone);
    long long pairs = 0;
    for (int A = 0; A < ntris; ++A)
        for (int B = A + 1; B < ntris; ++B) {
            if (tri_body[A] == tri_body[B]) continue;
            const uint32_t* ta = tris + 3 * A;
            const uint32_t* tb = tris + 3 * B;
            bool adj = false;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) adj = adj || ta[i] == tb[j];
            if (adj) continue;
            if (hi[A].x < lo[B].x || lo[A].x > hi[B].x || hi[A].y < lo[B].y || lo[A].y > hi[B].y ||
                hi[A].z < lo[B].z || lo[A].z > hi[B].z)
                continue;
            ++pairs;
            for (int dir = 0; dir < 2; ++dir) {
                const uint32_t* p = dir ? tb : ta;  // the "first" triangle of the query order
                const uint32_t* f = dir ? ta : tb;
                const uint32_t face = (uint32_t)(dir ? A : B);
                uint32_t fs[3] = {f[0], f[1], f[2]};
                std::sort(fs, fs + 3);
                for (int i = 0; i < 3; ++i) {
                    const uint32_t ids[4] = {p[i], fs[0], fs[1], fs[2]};
                    const float t = orc_ccd_query(1, ids, X, XT, nullptr);
                    if (t < 1.0f) vf_best[p[i]] = std::min(vf_best[p[i]], time_key(t, face));
                }
                static const int ek[3][2] = {{0, 1}, {0, 2}, {1, 2}};
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        uint32_t a0 = p[ek[i][0]], a1 = p[ek[i][1]], b0 = f[ek[j][0]], b1 = f[ek[j][1]];
                        if (a0 > a1) std::swap(a0, a1);
                        if (b0 > b1) std::swap(b0, b1);
                        const uint32_t ids[4] = {a0, a1, b0, b1};
                        const float t = orc_ccd_query(0, ids, X, XT, nullptr);
                        if (t < 1.0f) {
                            const uint32_t ea = edge_id(a0, a1);
                            ee_best[ea] = std::min(ee_best[ea], time_key(t, edge_id(b0, b1)));
                        }
                    }
            }
        }
    // normal of each marked vertex: the earliest contact touching it
    std::vector<uint64_t> win(nv, kNone);
    std::vector<float> wn(3 * (size_t)nv, 0.f);
    auto offer = [&](uint32_t u, uint64_t key, V3 n) {
        if (key < win[u]) {
            win[u] = key;
            wn[3 * u] = n.x;
            wn[3 * u + 1] = n.y;
            wn[3 * u + 2] = n.z;
        }
    };
    long long marked_src = 0;
    for (int p = 0; p < nv; ++p) {
        if (vf_best[p] == kNone) continue;
        ++marked_src;
        const uint32_t face = (uint32_t)(vf_best[p] & 0xffffffffu);
        uint32_t fs[3] = {tris[3 * face], tris[3 * face + 1], tris[3 * face + 2]};
        std::sort(fs, fs + 3);
        const uint32_t ids[4] = {(uint32_t)p, fs[0], fs[1], fs[2]};
        float n[3];
        orc_ccd_query(1, ids, X, XT, n);
        const uint64_t key = (vf_best[p] & 0xffffffff00000000ull) | (uint32_t)p;
        offer((uint32_t)p, key, V3{n[0], n[1], n[2]});
        for (int k = 0; k < 3; ++k) offer(fs[k], key, V3{-n[0], -n[1], -n[2]});
    }
    for (size_t e = 0; e < edges.size(); ++e) {
        if (ee_best[e] == kNone) continue;
        const uint32_t o = (uint32_t)(ee_best[e] & 0xffffffffu);
        const uint32_t ids[4] = {edges[e].first, edges[e].second, edges[o].first, edges[o].second};
        float n[3];
        orc_ccd_query(0, ids, X, XT, n);
        const uint64_t key = (ee_best[e] & 0xffffffff00000000ull) | (uint32_t)(nv + e);
        offer(edges[e].first, key, V3{n[0], n[1], n[2]});
        offer(edges[e].second, key, V3{n[0], n[1], n[2]});
    }
    long long marked = 0;
    for (int u = 0; u < nv; ++u) {
        const bool hit = win[u] != kNone;
        marked += hit;
        tI[u] = hit ? 0.5f : 1.0f;
        for (int d = 0; d < 3; ++d) normals[3 * u + d] = hit ? wn[3 * u + d] : 0.f;
    }
    if (stats) {
        stats[0] = pairs;
        stats[1] = marked_src;
        stats[2] = marked;
    }
    return 0;
}

/* Response of the reference's CCDKernel: tI < 1 -> V = -(d . n) n with
 * d = XTilde - X (X kept), else X = XTilde.  All [3 nv] except tI. */
void orc_ccd_response(int nv, const float* tI, const float* normals, float* X, const float* XT, float* V) {
    for (int i = 0; i < nv; ++i) {
        if (tI[i] < 1.0f) {
            const V3 n{normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]};
            const V3 d = V3{XT[3 * i], XT[3 * i + 1], XT[3 * i + 2]} - V3{X[3 * i], X[3 * i + 1], X[3 * i + 2]};
            const V3 vn = dot(d, n) * n;
            V[3 * i] = -vn.x;
            V[3 * i + 1] = -vn.y;
            V[3 * i + 2] = -vn.z;
        } else {
            for (int dd = 0; dd < 3; ++dd) X[3 * i + dd] = XT[3 * i + dd];
        }
    }
}

}  // extern "C"
