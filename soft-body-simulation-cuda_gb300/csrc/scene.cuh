// Device helpers for the optional per-step scene terms: interactive drag
// (the reference's moreDBC soft constraints) and fixed rigid bodies (plane,
// sphere, cylinder) resolved in the step epilogue.
#pragma once
#include "engine.h"

namespace pdgb {

__device__ __forceinline__ float dot3f(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Drag weight of vertex i (0 when no drag is set).
__device__ __forceinline__ float drag_weight(const SceneArgs& sc, int i) {
    return sc.drag_w ? __ldg(&sc.drag_w[i]) : 0.f;
}

// Target position of a dragged vertex: mouse target + the vertex's offset
// from the grabbed vertex (computeSn, pdUtil.cu:80-86).
__device__ __forceinline__ float4 drag_target(const SceneArgs& sc, int i) {
    const float4 t = *sc.target, o = __ldg(&sc.drag_off[i]);
    return make_float4(t.x + o.x, t.y + o.y, t.z + o.z, 0.f);
}

// Contact velocity response shared by the three fixed-body kinds
// (fixedBodyData.cu:66-144): the normal part is reflected and scaled by
// -muN, the tangential part shrinks by Coulomb friction, clamped at zero.
__device__ __forceinline__ void contact_velocity(float3 nrm, float mu_t, float mu_n, float3& V) {
    const float vn = dot3f(V, nrm);
    const float3 vN = make_float3(vn * nrm.x, vn * nrm.y, vn * nrm.z);
    const float3 vT = make_float3(V.x - vN.x, V.y - vN.y, V.z - vN.z);
    const float mag_vT = sqrtf(dot3f(vT, vT));
    const float a = mag_vT == 0.f ? 0.f : fmaxf(1.f - mu_t * (1.f + mu_n) * sqrtf(dot3f(vN, vN)) / mag_vT, 0.f);
    V = make_float3(-mu_n * vN.x + a * vT.x, -mu_n * vN.y + a * vT.y, -mu_n * vN.z + a * vT.z);
}

// Projects one vertex out of every fixed body, in the stored order
// (spheres, planes, cylinders), updating position and velocity.
__device__ __forceinline__ void collide_fixed(const SceneArgs& sc, float3& X, float3& V) {
    for (int j = 0; j < sc.nfixed; ++j) {
        const float4 p = sc.fixed[j].p, n = sc.fixed[j].n;
        const int type = (int)n.w;
        if (type == kFixedPlane) {
            const float3 up = make_float3(n.x, n.y, n.z);
            const float sd = dot3f(make_float3(X.x - p.x, X.y - p.y, X.z - p.z), up);
            if (sd < 0.f && dot3f(V, up) < 0.f) {
                X = make_float3(X.x - sd * up.x, X.y - sd * up.y, X.z - sd * up.z);
                contact_velocity(up, sc.mu_t, sc.mu_n, V);
            }
            continue;
        }
        float3 d = make_float3(X.x - p.x, X.y - p.y, X.z - p.z);
        if (type == kFixedCylinder) {
            // radial part (I - a a^T) d, element (r, c) = delta_rc - a_r a_c
            const float ax = n.x, ay = n.y, az = n.z;
            const float3 q = d;
            d.x = (1.f - ax * ax) * q.x + (0.f - ax * ay) * q.y + (0.f - ax * az) * q.z;
            d.y = (0.f - ay * ax) * q.x + (1.f - ay * ay) * q.y + (0.f - ay * az) * q.z;
            d.z = (0.f - az * ax) * q.x + (0.f - az * ay) * q.y + (1.f - az * az) * q.z;
        }
        const float len = sqrtf(dot3f(d, d));
        if (len < p.w) {
            const float inv = 1.f / sqrtf(dot3f(d, d));
            const float3 nrm = make_float3(d.x * inv, d.y * inv, d.z * inv);
            const float push = p.w - len;
            X = make_float3(X.x + push * nrm.x, X.y + push * nrm.y, X.z + push * nrm.z);
            contact_velocity(nrm, sc.mu_t, sc.mu_n, V);
        }
    }
}

// Step epilogue for one vertex: v = (q - XTilde) / h (0 for dragged
// vertices), X = XTilde = q, then the fixed-body correction of XTilde and v
// (updateVelPos pdUtil.cu:180-193; Update tail pdSolver.cu:218-232: X is
// copied before the correction, so X keeps the uncorrected position).  With
// collision handling on, only XTilde and v are written here: the collision
// response decides X, then corrects for the fixed bodies.
__device__ __forceinline__ void finish_vertex(const SceneArgs& sc, int i, float4 q, float dt_inv, float4* x,
                                              float4* v) {
    const float4 xo = sc.xt ? sc.xt[i] : x[i];
    float3 V = make_float3((q.x - xo.x) * dt_inv, (q.y - xo.y) * dt_inv, (q.z - xo.z) * dt_inv);
    if (drag_weight(sc, i) > 0.f) V = make_float3(0.f, 0.f, 0.f);
    // The reference has no such check (SolverStep returns true, pdSolver.cu:207);
    // a diverged step is reported through the engine's status word instead of
    // leaving the caller with silent NaN / inf positions.
    if (sc.nonfinite && !(isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && isfinite(V.x) && isfinite(V.y) &&
                          isfinite(V.z)))
        *sc.nonfinite = 1;
    if (sc.ccd) {
        sc.xt[i] = make_float4(q.x, q.y, q.z, 0.f);
        v[i] = make_float4(V.x, V.y, V.z, 0.f);
        return;
    }
    x[i] = make_float4(q.x, q.y, q.z, 0.f);
    if (sc.xt) {
        float3 X = make_float3(q.x, q.y, q.z);
        collide_fixed(sc, X, V);
        sc.xt[i] = make_float4(X.x, X.y, X.z, 0.f);
    }
    v[i] = make_float4(V.x, V.y, V.z, 0.f);
}

}  // namespace pdgb
