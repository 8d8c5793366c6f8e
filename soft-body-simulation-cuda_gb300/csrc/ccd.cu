// Continuous collision between bodies on the GPU (see ccd.h).
//
// Per detection:
//   1. swept box of every surface triangle (X -> XTilde) and the scene box;
//   2. 30-bit Morton code of each box centre, radix sort (CUB);
//   3. LBVH over the sorted codes (Karras, "Maximizing parallelism in the
//      construction of BVHs, octrees, and k-d trees", HPG 2012), the code
//      extended by the sorted position so that keys are unique;
//   4. bottom-up box refit: every leaf walks to the root, and at each
//      internal node the second of its two children to arrive (an atomic
//      arrival count, nobody waits) merges the children's boxes;
//   5. traversal: each triangle collects the triangles of other bodies
//      sharing no vertex whose boxes overlap its own (pairs kept once, by
//      the larger triangle index);
//   6. narrow phase: per pair and direction 3 point-face and 9 edge-edge
//      continuous tests; per vertex (point-face) and per edge (edge-edge)
//      the earliest contact before t = 1 by a 64-bit atomic minimum of
//      (contact time bits, face / other edge index);
//   7. marking: tI = 0.5 and the earliest touching contact's normal for the
//      vertices of every such contact (the reference's storeTi rule with its
//      write race replaced by the earliest-contact choice).
// The reference's candidate set is the same (its BVH traversal is exact);
// its query and reduction semantics are restated in narrow_test() below
// (intersections.cu:286-334, narrowphase.cu:8-127).
//
// This unit is compiled without floating-point contraction, so the narrow
// phase performs the same IEEE single-precision operations as the CPU
// oracle and the reference's code compiled for the host.
#include "ccd.h"

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <utility>

#include "scene.cuh"

namespace pdgb {

namespace {

constexpr unsigned long long kNone = ~0ull;
constexpr int kStack = 64;
constexpr int kThreads = 256;

inline int blocks_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

// ------------------------------------------------------------ geometry
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 scl(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float len(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 unit(F3 a) { return scl(1.0f / len(a), a); }
__device__ __forceinline__ float triple(F3 u, F3 v, F3 w) { return dot(u, cross(v, w)); }

// Real roots of a x^2 + b x + c in the numerically stable form; 0 with the
// vertex -b / 2a in x[0] when the discriminant is negative.
__device__ int quad_roots(float a, float b, float c, float* x) {
    const float d = b * b - 4 * a * c;
    if (d < 0) {
        x[0] = -b / (2 * a);
        return 0;
    }
    const float sgn = (b > 0) ? 1.0f : (b < 0 ? -1.0f : 0.0f);
    const float q = -(b + sgn * sqrtf(d)) / 2;
    int n = 0;
    if (fabsf(a) > 1e-12 * fabsf(q)) x[n++] = q / a;
    if (fabsf(q) > 1e-12 * fabsf(c)) x[n++] = c / q;
    if (n == 2 && x[0] > x[1]) {
        const float t = x[0];
        x[0] = x[1];
        x[1] = t;
    }
    return n;
}

// Newton iteration on the cubic from x0 (at most 100 steps); with dir != 0
// the start is first moved off the critical point by the quadratic model.
__device__ float cubic_newton(float a, float b, float c, float d, float x0, int dir) {
    if (dir != 0) {
        const float y0 = d + x0 * (c + x0 * (b + x0 * a));
        const float ddy0 = 2 * b + x0 * (6 * a);
        if (ddy0 != 0) x0 += dir * sqrtf(fabsf(2 * y0 / ddy0));
    }
    for (int it = 0; it < 100; ++it) {
        const float y = d + x0 * (c + x0 * (b + x0 * a));
        const float dy = c + x0 * (2 * b + x0 * 3 * a);
        if (dy == 0) return x0;
        const float x1 = x0 - y / dy;
        if (fabsf(x0 - x1) < 1e-6) return x0;
        x0 = x1;
    }
    return x0;
}

// Real roots of a x^3 + b x^2 + c x + d, bracketed by the critical points.
__device__ int cubic_roots(float a, float b, float c, float d, float* x) {
    float xc[2];
    const int ncrit = quad_roots(3 * a, 2 * b, c, xc);
    if (ncrit == 0) {
        x[0] = cubic_newton(a, b, c, d, xc[0], 0);
        return 1;
    }
    if (ncrit == 1) return quad_roots(b, c, d, x);
    const float yc0 = d + xc[0] * (c + xc[0] * (b + xc[0] * a));
    const float yc1 = d + xc[1] * (c + xc[1] * (b + xc[1] * a));
    int n = 0;
    if (yc0 * a >= 0) x[n++] = cubic_newton(a, b, c, d, xc[0], -1);
    if (yc0 * yc1 <= 0) {
        const int closer = fabsf(yc0) < fabsf(yc1) ? 0 : 1;
        x[n++] = cubic_newton(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
    }
    if (yc1 * a <= 0) x[n++] = cubic_newton(a, b, c, d, xc[1], 1);
    return n;
}

// Signed distance of p to the plane of face (y0, y1, y2), its normal and
// the barycentric weights (w0 = 1, w1..3 = minus the face coordinates).
__device__ float face_distance(F3 p, F3 y0, F3 y1, F3 y2, F3& n, float w[4]) {
    n = cross(unit(sub(y1, y0)), unit(sub(y2, y0)));
    if (dot(n, n) < 1e-6) return FLT_MAX;
    n = unit(n);
    const float h = dot(sub(p, y0), n);
    const float b0 = triple(sub(y1, p), sub(y2, p), n), b1 = triple(sub(y2, p), sub(y0, p), n),
                b2 = triple(sub(y0, p), sub(y1, p), n);
    const float s = b0 + b1 + b2;
    w[0] = 1;
    w[1] = -b0 / s;
    w[2] = -b1 / s;
    w[3] = -b2 / s;
    return h;
}

// Signed distance between the lines of edges (x0, x1) and (y0, y1), their
// common normal and the weights (w0, w1 on the first, -w2, -w3 on the second).
__device__ float edge_distance(F3 x0, F3 x1, F3 y0, F3 y1, F3& n, float w[4]) {
    n = cross(unit(sub(x1, x0)), unit(sub(y1, y0)));
    if (dot(n, n) < 1e-6) return FLT_MAX;
    n = unit(n);
    const float h = dot(sub(x0, y0), n);
    const float a0 = triple(sub(y1, x1), sub(y0, x1), n), a1 = triple(sub(y0, x0), sub(y1, x0), n);
    const float b0 = triple(sub(x0, y1), sub(x1, y1), n), b1 = triple(sub(x1, y0), sub(x0, y0), n);
    w[0] = a0 / (a0 + a1);
    w[1] = a1 / (a0 + a1);
    w[2] = -b0 / (b0 + b1);
    w[3] = -b1 / (b0 + b1);
    return h;
}

// Earliest contact time in [0, 1] of a point-face (face: point q0, face
// q1..q3) or edge-edge (q0q1 against q2q3) query, 1 when none; n is the
// contact normal (pointing against the relative motion of the face side).
// Contact: the four points coplanar at a root of the cubic, within 1e-6 of
// each other's plane / line and inside by the barycentric test.
__device__ float narrow_test(bool face, const F3 x[4], const F3 v[4], F3& n) {
    const F3 x01 = sub(x[1], x[0]), x02 = sub(x[2], x[0]), x03 = sub(x[3], x[0]);
    const F3 v01 = sub(v[1], v[0]), v02 = sub(v[2], v[0]), v03 = sub(v[3], v[0]);
    const float a0 = triple(x01, x02, x03);
    const float a1 = triple(v01, x02, x03) + triple(x01, v02, x03) + triple(x01, x02, v03);
    const float a2 = triple(x01, v02, v03) + triple(v01, x02, v03) + triple(v01, v02, x03);
    const float a3 = triple(v01, v02, v03);
    n = {0.f, 0.f, 0.f};
    if (fabsf(a0) < 1e-12 * len(x01) * len(x02) * len(x03)) return 1.0f;  // coplanar at t = 0
    float t[3];
    const int nr = cubic_roots(a3, a2, a1, a0, t);
    for (int i = 0; i < nr; ++i) {
        if (t[i] < -1e-12 || t[i] > 1) continue;
        F3 xt[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) xt[k] = add(x[k], scl(t[i], v[k]));
        float w[4] = {0.f, 0.f, 0.f, 0.f};
        float d;
        bool inside;
        if (face) {
            d = face_distance(xt[0], xt[1], xt[2], xt[3], n, w);
            inside = fminf(-w[1], fminf(-w[2], -w[3])) >= -1e-3;
        } else {
            d = edge_distance(xt[0], xt[1], xt[2], xt[3], n, w);
            inside = fminf(w[0], fminf(w[1], fminf(-w[2], -w[3]))) >= -1e-3;
        }
        const F3 rel = add(add(scl(w[1], v[1]), scl(w[2], v[2])), scl(w[3], v[3]));
        if (dot(n, rel) > 0) n = scl(-1.0f, n);
        if (fabsf(d) < 1e-6 && inside) return t[i];
    }
    return 1.0f;
}

__device__ __forceinline__ float query(bool face, const uint32_t ids[4], const float4* x, const float4* xt, F3& n) {
    F3 p[4], v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        p[k] = f3(x[ids[k]]);
        v[k] = sub(f3(xt[ids[k]]), p[k]);
    }
    return narrow_test(face, p, v, n);
}

__device__ __forceinline__ unsigned long long time_key(float t, uint32_t tag) {
    const float tk = t > 0.f ? t : 0.f;
    return ((unsigned long long)__float_as_uint(tk) << 32) | tag;
}

// Order-preserving map of floats to signed ints (for atomic min / max).
__device__ __forceinline__ int ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ unsigned int spread10(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ bool overlap(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    return !(ahi.x < blo.x || alo.x > bhi.x || ahi.y < blo.y || alo.y > bhi.y || ahi.z < blo.z || alo.z > bhi.z);
}

// ------------------------------------------------------------ kernels
struct Dev {
    int nv, ntris, nedges;
    const float4* x;
    const float4* xt;
    const uint4* tri;
    const uint4* tri_edges;
    const uint2* edges;
    const int* vcaller;
    float4* tri_lo;   // [ntris] swept boxes, triangle order
    float4* tri_hi;
    float4* node_lo;  // [2 ntris - 1]: internal nodes, then leaves in sorted order
    float4* node_hi;
    int* scene;       // [6] ordered min xyz, max xyz
    unsigned int* code;
    unsigned int* code_sorted;
    int* order;
    int* order_sorted;
    int2* child;      // [ntris - 1]
    int* parent;      // [2 ntris - 1]
    int* visit;       // [ntris - 1]
    int2* pairs;
    int* counters;    // [0] pairs found, [1] traversal stack overflow
    int pair_cap;
    unsigned long long* vf_best;  // [nv]
    unsigned long long* ee_best;  // [nedges]
    unsigned long long* vwin;     // [nv]
    float4* vf_n;                 // [nv] normal of each vertex's earliest face contact
    float4* ee_n;                 // [nedges]
    float* tI;
    float4* nrm;
};

__global__ void k_init(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3) {
        d.scene[i] = ord(FLT_MAX);
        d.scene[3 + i] = ord(-FLT_MAX);
    }
    if (i < 2) d.counters[i] = 0;
    if (i < d.nv) {
        d.vf_best[i] = kNone;
        d.vwin[i] = kNone;
    }
    if (i < d.nedges) d.ee_best[i] = kNone;
    if (i < d.ntris - 1) d.visit[i] = 0;
}

__global__ void k_boxes(Dev d) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntris) return;
    const uint4 tr = d.tri[t];
    const uint32_t id[3] = {tr.x, tr.y, tr.z};
    float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const float4 p = s ? d.xt[id[k]] : d.x[id[k]];
            lo.x = fminf(lo.x, p.x);
            lo.y = fminf(lo.y, p.y);
            lo.z = fminf(lo.z, p.z);
            hi.x = fmaxf(hi.x, p.x);
            hi.y = fmaxf(hi.y, p.y);
            hi.z = fmaxf(hi.z, p.z);
        }
    d.tri_lo[t] = lo;
    d.tri_hi[t] = hi;
    atomicMin(&d.scene[0], ord(lo.x));
    atomicMin(&d.scene[1], ord(lo.y));
    atomicMin(&d.scene[2], ord(lo.z));
    atomicMax(&d.scene[3], ord(hi.x));
    atomicMax(&d.scene[4], ord(hi.y));
    atomicMax(&d.scene[5], ord(hi.z));
}

__global__ void k_morton(Dev d) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntris) return;
    const float lo[3] = {unord(d.scene[0]), unord(d.scene[1]), unord(d.scene[2])};
    const float hi[3] = {unord(d.scene[3]), unord(d.scene[4]), unord(d.scene[5])};
    const float4 a = d.tri_lo[t], b = d.tri_hi[t];
    const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned int q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ext = hi[k] - lo[k];
        const float u = ext > 0.f ? (c[k] - lo[k]) / ext : 0.f;
        q[k] = (unsigned int)fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
    }
    d.code[t] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    d.order[t] = t;
}

// Length of the common prefix of the keys (code, position) at sorted
// positions i and j; -1 outside [0, n).
__device__ __forceinline__ int prefix(const Dev& d, int i, int j) {
    if (j < 0 || j >= d.ntris) return -1;
    const unsigned long long ki = ((unsigned long long)d.code_sorted[i] << 32) | (unsigned int)i;
    const unsigned long long kj = ((unsigned long long)d.code_sorted[j] << 32) | (unsigned int)j;
    return __clzll(ki ^ kj);
}

// Internal node i of the radix tree over n sorted keys: its key range and
// split decide the two children (Karras 2012).  Nodes 0 .. n-2 are internal
// (0 is the root), n-1 .. 2n-2 the leaves in sorted order.
__global__ void k_build(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = d.ntris;
    if (i >= n - 1) return;
    const int dir = (prefix(d, i, i + 1) - prefix(d, i, i - 1)) > 0 ? 1 : -1;
    const int dmin = prefix(d, i, i - dir);
    int lmax = 2;
    while (lmax < 2 * n && prefix(d, i, i + lmax * dir) > dmin) lmax *= 2;  // keys are unique: lmax <= 2n
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (prefix(d, i, i + (l + t) * dir) > dmin) l += t;
    const int j = i + l * dir;
    const int dnode = prefix(d, i, j);
    int s = 0;
    int step = l;
    do {
        step = (step + 1) / 2;
        if (prefix(d, i, i + (s + step) * dir) > dnode) s += step;
    } while (step > 1);
    const int split = i + s * dir + (dir < 0 ? -1 : 0);
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const int left = (lo == split) ? (n - 1 + split) : split;
    const int right = (hi == split + 1) ? (n - 1 + split + 1) : split + 1;
    d.child[i] = make_int2(left, right);
    d.parent[left] = i;
    d.parent[right] = i;
}

// Leaf boxes, then the bottom-up merge: the second child to arrive at a node
// computes the node's box and goes on; the first stops.  No thread waits.
__global__ void k_refit(Dev d) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = d.ntris;
    if (j >= n) return;
    const int t = d.order_sorted[j];
    int node = n - 1 + j;
    d.node_lo[node] = d.tri_lo[t];
    d.node_hi[node] = d.tri_hi[t];
    if (n == 1) return;
    for (int guard = 0; guard < n; ++guard) {
        node = d.parent[node];
        __threadfence();
        if (atomicAdd(&d.visit[node], 1) == 0) return;
        const int2 c = d.child[node];
        const float4 al = __ldcg(&d.node_lo[c.x]), ah = __ldcg(&d.node_hi[c.x]);
        const float4 bl = __ldcg(&d.node_lo[c.y]), bh = __ldcg(&d.node_hi[c.y]);
        d.node_lo[node] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f);
        d.node_hi[node] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f);
        if (node == 0) return;
    }
}

__device__ __forceinline__ bool share_vertex(uint4 a, uint4 b) {
    return a.x == b.x || a.x == b.y || a.x == b.z || a.y == b.x || a.y == b.y || a.y == b.z || a.z == b.x ||
           a.z == b.y || a.z == b.z;
}

__global__ void k_traverse(Dev d) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = d.ntris;
    if (j >= n || n < 2) return;
    const int A = d.order_sorted[j];
    const uint4 ta = d.tri[A];
    const float4 lo = d.tri_lo[A], hi = d.tri_hi[A];
    int stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int2 c = d.child[node];
        const int kids[2] = {c.x, c.y};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int ch = kids[k];
            if (!overlap(lo, hi, d.node_lo[ch], d.node_hi[ch])) continue;
            if (ch >= n - 1) {
                const int B = d.order_sorted[ch - (n - 1)];
                if (B <= A) continue;  // each unordered pair once
                const uint4 tb = d.tri[B];
                if (tb.w == ta.w || share_vertex(ta, tb)) continue;
                const int slot = atomicAdd(&d.counters[0], 1);
                if (slot < d.pair_cap) d.pairs[slot] = make_int2(A, B);
            } else if (sp < kStack) {
                stack[sp++] = ch;
            } else {
                d.counters[1] = 1;  // deeper than the stack: result incomplete, reported
            }
        }
    }
}

// One thread per (pair, direction, query): q < 3 point-face, else edge-edge.
__global__ void k_narrow(Dev d, int npairs) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= 24LL * npairs) return;
    const int pi = (int)(g / 24), r = (int)(g % 24);
    const int dirn = r / 12, q = r % 12;
    const int2 pr = d.pairs[pi];
    const int P = dirn ? pr.y : pr.x, Fc = dirn ? pr.x : pr.y;
    const uint4 tp = d.tri[P], tf = d.tri[Fc];
    const uint32_t pv[3] = {tp.x, tp.y, tp.z};
    F3 nn;
    if (q < 3) {
        const uint32_t ids[4] = {pv[q], tf.x, tf.y, tf.z};
        const float t = query(true, ids, d.x, d.xt, nn);
        if (t < 1.0f) atomicMin(&d.vf_best[pv[q]], time_key(t, (uint32_t)Fc));
    } else {
        const uint4 ep = d.tri_edges[P], ef = d.tri_edges[Fc];
        const uint32_t pe[3] = {ep.x, ep.y, ep.z}, fe[3] = {ef.x, ef.y, ef.z};
        const uint32_t ea = pe[(q - 3) / 3], eb = fe[(q - 3) % 3];
        const uint2 a = d.edges[ea], b = d.edges[eb];
        const uint32_t ids[4] = {a.x, a.y, b.x, b.y};
        const float t = query(false, ids, d.x, d.xt, nn);
        if (t < 1.0f) atomicMin(&d.ee_best[ea], time_key(t, eb));
    }
}

// Winning contact per touched vertex: smallest (time, source) key, the
// source being the caller id of a point-face contact's point or nv + edge.
__global__ void k_mark(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nv && d.vf_best[i] != kNone) {
        const unsigned long long best = d.vf_best[i];
        const uint4 tf = d.tri[(uint32_t)(best & 0xffffffffu)];
        const uint32_t ids[4] = {(uint32_t)i, tf.x, tf.y, tf.z};
        F3 nn;
        query(true, ids, d.x, d.xt, nn);
        d.vf_n[i] = make_float4(nn.x, nn.y, nn.z, 0.f);
        const uint32_t src = d.vcaller ? (uint32_t)d.vcaller[i] : (uint32_t)i;
        const unsigned long long key = (best & 0xffffffff00000000ull) | src;
        atomicMin(&d.vwin[i], key);
        atomicMin(&d.vwin[tf.x], key);
        atomicMin(&d.vwin[tf.y], key);
        atomicMin(&d.vwin[tf.z], key);
    }
    if (i < d.nedges && d.ee_best[i] != kNone) {
        const unsigned long long best = d.ee_best[i];
        const uint2 a = d.edges[i], b = d.edges[(uint32_t)(best & 0xffffffffu)];
        const uint32_t ids[4] = {a.x, a.y, b.x, b.y};
        F3 nn;
        query(false, ids, d.x, d.xt, nn);
        d.ee_n[i] = make_float4(nn.x, nn.y, nn.z, 0.f);
        const unsigned long long key = (best & 0xffffffff00000000ull) | (uint32_t)(d.nv + i);
        atomicMin(&d.vwin[a.x], key);
        atomicMin(&d.vwin[a.y], key);
    }
}

// Normals from the winning contacts (each vertex has exactly one writer).
__global__ void k_normals(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nv && d.vf_best[i] != kNone) {
        const unsigned long long best = d.vf_best[i];
        const uint4 tf = d.tri[(uint32_t)(best & 0xffffffffu)];
        const uint32_t src = d.vcaller ? (uint32_t)d.vcaller[i] : (uint32_t)i;
        const unsigned long long key = (best & 0xffffffff00000000ull) | src;
        const float4 n = d.vf_n[i];
        const float4 m = make_float4(-n.x, -n.y, -n.z, 0.f);
        if (d.vwin[i] == key) d.nrm[i] = n;
        if (d.vwin[tf.x] == key) d.nrm[tf.x] = m;
        if (d.vwin[tf.y] == key) d.nrm[tf.y] = m;
        if (d.vwin[tf.z] == key) d.nrm[tf.z] = m;
    }
    if (i < d.nedges && d.ee_best[i] != kNone) {
        const unsigned long long key = (d.ee_best[i] & 0xffffffff00000000ull) | (uint32_t)(d.nv + i);
        const uint2 a = d.edges[i];
        if (d.vwin[a.x] == key) d.nrm[a.x] = d.ee_n[i];
        if (d.vwin[a.y] == key) d.nrm[a.y] = d.ee_n[i];
    }
}

__global__ void k_finish(Dev d, int* marked) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nv) return;
    const bool hit = d.vwin[i] != kNone;
    d.tI[i] = hit ? 0.5f : 1.0f;
    if (!hit) d.nrm[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (hit) atomicAdd(marked, 1);
}

// CCDKernel (collisionUtil.cu:50-70): a vertex with tI < 1 keeps X and gets
// v = -(d . n) n with d = XTilde - X; the others move to XTilde.  Then the
// fixed-body correction of XTilde and v.
__global__ void k_respond(int nv, const float* tI, const float4* nrm, float4* x, const float4* xt, float4* v,
                          SceneArgs sc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 p = x[i], q = xt[i];
    float4 vel = v[i];
    if (tI[i] < 1.0f) {
        const F3 n = f3(nrm[i]);
        const F3 dd = sub(f3(q), f3(p));
        const F3 vn = scl(dot(dd, n), n);
        vel = make_float4(-vn.x, -vn.y, -vn.z, 0.f);
    } else {
        x[i] = q;
    }
    if (sc.nfixed > 0 && sc.xt) {
        float3 X = make_float3(q.x, q.y, q.z), V = make_float3(vel.x, vel.y, vel.z);
        collide_fixed(sc, X, V);
        sc.xt[i] = make_float4(X.x, X.y, X.z, 0.f);
        vel = make_float4(V.x, V.y, V.z, 0.f);
    }
    v[i] = vel;
}

}  // namespace

// ------------------------------------------------------------ host side
CcdSurface build_ccd_surface(int nv, int ntris, const uint32_t* tris, const int* tri_body, const int* viperm) {
    if (nv <= 0 || ntris < 0 || (ntris > 0 && (!tris || !tri_body)))
        throw Error{PDGB_ERR_INVALID_ARGUMENT, "collision surface: bad sizes or null arrays"};
    CcdSurface s;
    s.nv = nv;
    s.ntris = ntris;
    auto iv = [&](uint32_t c) { return viperm ? (uint32_t)viperm[c] : c; };
    std::vector<std::pair<uint32_t, uint32_t>> edges;  // caller ids, ascending
    edges.reserve(3 * (size_t)ntris);
    for (int t = 0; t < ntris; ++t) {
        uint32_t c[3] = {tris[3 * (size_t)t], tris[3 * (size_t)t + 1], tris[3 * (size_t)t + 2]};
        for (uint32_t v : c)
            if (v >= (uint32_t)nv)
                throw Error{PDGB_ERR_BAD_MESH, "collision triangle " + std::to_string(t) + " references vertex " +
                                                   std::to_string(v) + " >= num_verts"};
        for (int k = 0; k < 3; ++k) {
            uint32_t a = c[k], b = c[(k + 1) % 3];
            if (a > b) std::swap(a, b);
            edges.push_back({a, b});
        }
    }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    if (edges.size() + (size_t)nv >= 0xffffffffull || ntris > 0x7fffffff)
        throw Error{PDGB_ERR_UNSUPPORTED, "collision surface too large"};
    auto edge_id = [&](uint32_t a, uint32_t b) {
        if (a > b) std::swap(a, b);
        return (uint32_t)(std::lower_bound(edges.begin(), edges.end(), std::make_pair(a, b)) - edges.begin());
    };
    s.nedges = (int)edges.size();
    s.tri.resize(ntris);
    s.tri_edges.resize(ntris);
    for (int t = 0; t < ntris; ++t) {
        uint32_t c[3] = {tris[3 * (size_t)t], tris[3 * (size_t)t + 1], tris[3 * (size_t)t + 2]};
        s.tri_edges[t] = make_uint4(edge_id(c[0], c[1]), edge_id(c[0], c[2]), edge_id(c[1], c[2]), 0u);
        std::sort(c, c + 3);
        s.tri[t] = make_uint4(iv(c[0]), iv(c[1]), iv(c[2]), (uint32_t)tri_body[t]);
    }
    s.edges.resize(edges.size());
    for (size_t e = 0; e < edges.size(); ++e) s.edges[e] = make_uint2(iv(edges[e].first), iv(edges[e].second));
    return s;
}

struct CcdContext::Buffers {
    DBuf<uint4> tri, tri_edges;
    DBuf<uint2> edges;
    DBuf<float4> tri_lo, tri_hi, node_lo, node_hi, vf_n, ee_n, nrm;
    DBuf<int> scene, order, order_sorted, parent, visit, counters, marked;
    DBuf<unsigned int> code, code_sorted;
    DBuf<int2> child, pairs;
    DBuf<unsigned long long> vf_best, ee_best, vwin;
    DBuf<float> tI;
    DBuf<unsigned char> sort_tmp;
    size_t sort_bytes = 0;
    int pair_cap = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

CcdContext::CcdContext(const CcdSurface& s, const int* vcaller, cudaStream_t stream)
    : b_(new Buffers), nv_(s.nv), ntris_(s.ntris), nedges_(s.nedges), vcaller_(vcaller), stream_(stream) {
    Buffers& b = *b_;
    const size_t n = (size_t)std::max(ntris_, 1);
    b.tri.upload(s.tri, stream);
    b.tri_edges.upload(s.tri_edges, stream);
    b.edges.upload(s.edges, stream);
    b.tri_lo.alloc(n);
    b.tri_hi.alloc(n);
    b.node_lo.alloc(2 * n);
    b.node_hi.alloc(2 * n);
    b.scene.alloc(6);
    b.code.alloc(n);
    b.code_sorted.alloc(n);
    b.order.alloc(n);
    b.order_sorted.alloc(n);
    b.child.alloc(n);
    b.parent.alloc(2 * n);
    b.visit.alloc(n);
    b.counters.alloc(2);
    b.marked.alloc(1);
    b.pair_cap = (int)std::min<size_t>(std::max<size_t>(16 * n, 4096), 1u << 30);
    b.pairs.alloc(b.pair_cap);
    b.vf_best.alloc(nv_);
    b.vwin.alloc(nv_);
    b.vf_n.alloc(nv_);
    b.ee_best.alloc(std::max(nedges_, 1));
    b.ee_n.alloc(std::max(nedges_, 1));
    b.tI.alloc(nv_);
    b.nrm.alloc(nv_);
    PDGB_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, b.sort_bytes, b.code.p, b.code_sorted.p, b.order.p,
                                                  b.order_sorted.p, (int)n, 0, 30, stream));
    b.sort_tmp.alloc(std::max<size_t>(b.sort_bytes, 1));
    PDGB_CUDA_TRY(cudaEventCreate(&b.ev[0]));
    PDGB_CUDA_TRY(cudaEventCreate(&b.ev[1]));
    // no contact until the first detection
    std::vector<float> ones(nv_, 1.0f);
    PDGB_CUDA_TRY(cudaMemcpyAsync(b.tI.p, ones.data(), nv_ * sizeof(float), cudaMemcpyHostToDevice, stream));
    PDGB_CUDA_TRY(cudaMemsetAsync(b.nrm.p, 0, nv_ * sizeof(float4), stream));
    PDGB_CUDA_TRY(cudaStreamSynchronize(stream));
}

CcdContext::~CcdContext() {
    if (b_) {
        if (b_->ev[0]) cudaEventDestroy(b_->ev[0]);
        if (b_->ev[1]) cudaEventDestroy(b_->ev[1]);
    }
}

const float* CcdContext::tI() const { return b_->tI.p; }
const float4* CcdContext::normals() const { return b_->nrm.p; }

void CcdContext::detect(const float4* x, const float4* xt) {
    Buffers& b = *b_;
    cudaStream_t s = stream_;
    PDGB_CUDA_TRY(cudaEventRecord(b.ev[0], s));
    Dev d{};
    d.nv = nv_;
    d.ntris = ntris_;
    d.nedges = nedges_;
    d.x = x;
    d.xt = xt;
    d.tri = b.tri.p;
    d.tri_edges = b.tri_edges.p;
    d.edges = b.edges.p;
    d.vcaller = vcaller_;
    d.tri_lo = b.tri_lo.p;
    d.tri_hi = b.tri_hi.p;
    d.node_lo = b.node_lo.p;
    d.node_hi = b.node_hi.p;
    d.scene = b.scene.p;
    d.code = b.code.p;
    d.code_sorted = b.code_sorted.p;
    d.order = b.order.p;
    d.order_sorted = b.order_sorted.p;
    d.child = b.child.p;
    d.parent = b.parent.p;
    d.visit = b.visit.p;
    d.pairs = b.pairs.p;
    d.counters = b.counters.p;
    d.pair_cap = b.pair_cap;
    d.vf_best = b.vf_best.p;
    d.ee_best = b.ee_best.p;
    d.vwin = b.vwin.p;
    d.vf_n = b.vf_n.p;
    d.ee_n = b.ee_n.p;
    d.tI = b.tI.p;
    d.nrm = b.nrm.p;
    const long long init_n = std::max<long long>({(long long)nv_, (long long)nedges_, (long long)ntris_, 6});
    k_init<<<blocks_for(init_n), kThreads, 0, s>>>(d);
    int npairs = 0;
    if (ntris_ >= 2) {
        k_boxes<<<blocks_for(ntris_), kThreads, 0, s>>>(d);
        k_morton<<<blocks_for(ntris_), kThreads, 0, s>>>(d);
        size_t bytes = b.sort_bytes;
        PDGB_CUDA_TRY(cub::DeviceRadixSort::SortPairs(b.sort_tmp.p, bytes, b.code.p, b.code_sorted.p, b.order.p,
                                                      b.order_sorted.p, ntris_, 0, 30, s));
        k_build<<<blocks_for(ntris_ - 1), kThreads, 0, s>>>(d);
        k_refit<<<blocks_for(ntris_), kThreads, 0, s>>>(d);
        for (int attempt = 0;; ++attempt) {
            k_traverse<<<blocks_for(ntris_), kThreads, 0, s>>>(d);
            int cnt[2] = {0, 0};
            PDGB_CUDA_TRY(cudaMemcpyAsync(cnt, b.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s));
            PDGB_CUDA_TRY(cudaStreamSynchronize(s));
            if (cnt[1]) throw Error{PDGB_ERR_UNSUPPORTED, "collision BVH deeper than the traversal stack"};
            if (cnt[0] <= b.pair_cap) {
                npairs = cnt[0];
                break;
            }
            if (attempt > 0 || cnt[0] > (1 << 30)) throw Error{PDGB_ERR_OUT_OF_MEMORY, "too many collision candidates"};
            b.pair_cap = cnt[0] + cnt[0] / 4;  // grow once to the count found, then rerun
            b.pairs.alloc(b.pair_cap);
            d.pairs = b.pairs.p;
            d.pair_cap = b.pair_cap;
            stats_.regrows++;
            PDGB_CUDA_TRY(cudaMemsetAsync(b.counters.p, 0, 2 * sizeof(int), s));
        }
        if (npairs > 0) k_narrow<<<blocks_for(24LL * npairs), kThreads, 0, s>>>(d, npairs);
    }
    PDGB_CUDA_TRY(cudaMemsetAsync(b.marked.p, 0, sizeof(int), s));
    k_mark<<<blocks_for(std::max(nv_, nedges_)), kThreads, 0, s>>>(d);
    k_normals<<<blocks_for(std::max(nv_, nedges_)), kThreads, 0, s>>>(d);
    k_finish<<<blocks_for(nv_), kThreads, 0, s>>>(d, b.marked.p);
    PDGB_CUDA_TRY(cudaGetLastError());
    PDGB_CUDA_TRY(cudaEventRecord(b.ev[1], s));
    int marked = 0;
    PDGB_CUDA_TRY(cudaMemcpyAsync(&marked, b.marked.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PDGB_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    PDGB_CUDA_TRY(cudaEventElapsedTime(&ms, b.ev[0], b.ev[1]));
    stats_.pairs = npairs;
    stats_.marked = marked;
    stats_.ms = ms;
}

void CcdContext::respond(float4* x, const float4* xt, float4* v, const SceneArgs& sc) {
    Buffers& b = *b_;
    k_respond<<<blocks_for(nv_), kThreads, 0, stream_>>>(nv_, b.tI.p, b.nrm.p, x, xt, v, sc);
    PDGB_CUDA_TRY(cudaGetLastError());
}

}  // namespace pdgb
