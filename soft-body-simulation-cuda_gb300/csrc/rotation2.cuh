// Paired form of the closest-rotation kernel: two independent 3x3 problems
// in the x and y lanes of float2 values, so that every multiply-add is one
// packed FP32x2 instruction (__ffma2_rn and friends, sm_100 and later).
// Same method as closest_rotation_horn in rotation.cuh (Horn's quaternion
// matrix, shifted and squared), each lane converged to float precision.
#pragma once
#include <cuda_runtime.h>

namespace pdgb {

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b, exact as one rounding: fma(b, -1, a)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }

// a <- a * a for symmetric 4x4 matrices stored as
// {ww, xx, yy, zz, wx, wy, wz, xy, xz, yz}, both lanes.
__device__ __forceinline__ void sym4_square2(float2 a[10]) {
    const float2 ww = a[0], xx = a[1], yy = a[2], zz = a[3], wx = a[4], wy = a[5], wz = a[6], xy = a[7],
                 xz = a[8], yz = a[9];
    a[0] = fma2(ww, ww, fma2(wx, wx, fma2(wy, wy, mul2(wz, wz))));
    a[1] = fma2(wx, wx, fma2(xx, xx, fma2(xy, xy, mul2(xz, xz))));
    a[2] = fma2(wy, wy, fma2(xy, xy, fma2(yy, yy, mul2(yz, yz))));
    a[3] = fma2(wz, wz, fma2(xz, xz, fma2(yz, yz, mul2(zz, zz))));
    a[4] = fma2(ww, wx, fma2(wx, xx, fma2(wy, xy, mul2(wz, xz))));
    a[5] = fma2(ww, wy, fma2(wx, xy, fma2(wy, yy, mul2(wz, yz))));
    a[6] = fma2(ww, wz, fma2(wx, xz, fma2(wy, yz, mul2(wz, zz))));
    a[7] = fma2(wx, wy, fma2(xx, xy, fma2(xy, yy, mul2(xz, yz))));
    a[8] = fma2(wx, wz, fma2(xx, xz, fma2(xy, yz, mul2(xz, zz))));
    a[9] = fma2(wy, wz, fma2(xy, xz, fma2(yy, yz, mul2(yz, zz))));
}

// Quaternion (w, x, y, z) of one lane: the column of the rank-one P with
// the largest diagonal entry, multiplied once more by P (a power step that
// squares the remaining error), normalised.
__device__ __forceinline__ void dominant_column(const float a[10], float q[4]) {
    // P as a full symmetric matrix, index (r, c) over (w, x, y, z)
    float c0 = a[0], c1 = a[4], c2 = a[5], c3 = a[6], best = a[0];
    if (a[1] > best) { best = a[1]; c0 = a[4]; c1 = a[1]; c2 = a[7]; c3 = a[8]; }
    if (a[2] > best) { best = a[2]; c0 = a[5]; c1 = a[7]; c2 = a[2]; c3 = a[9]; }
    if (a[3] > best) { c0 = a[6]; c1 = a[8]; c2 = a[9]; c3 = a[3]; }
    q[0] = fmaf(a[0], c0, fmaf(a[4], c1, fmaf(a[5], c2, a[6] * c3)));
    q[1] = fmaf(a[4], c0, fmaf(a[1], c1, fmaf(a[7], c2, a[8] * c3)));
    q[2] = fmaf(a[5], c0, fmaf(a[7], c1, fmaf(a[2], c2, a[9] * c3)));
    q[3] = fmaf(a[6], c0, fmaf(a[8], c1, fmaf(a[9], c2, a[3] * c3)));
    const float n = rsqrtf(fmaxf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3], 1e-37f));
    q[0] *= n; q[1] *= n; q[2] *= n; q[3] *= n;
}

// Closest proper rotations of F (row-major, lanes = two problems): R in the
// same layout.  Shift c = 0.6 |F|_F keeps the top eigenvalue of N(F) + c I
// dominant; 3 squarings, then -- per lane, only where P = A^8 is not yet
// rank one to float precision (trace(P^2) < (1 - 4e-7) trace(P)^2) --
// normalised squarings (at most kTail); then one power step on the dominant
// column.
template <int kTail = 6>
__device__ __forceinline__ void closest_rotation_horn2(const float2 F[9], float2 R[9]) {
    float2 f2s = mul2(F[0], F[0]);
#pragma unroll
    for (int i = 1; i < 9; ++i) f2s = fma2(F[i], F[i], f2s);
    f2s.x = fmaxf(f2s.x, 1e-30f);
    f2s.y = fmaxf(f2s.y, 1e-30f);
    const float2 c = make_float2(0.6f * f2s.x * rsqrtf(f2s.x), 0.6f * f2s.y * rsqrtf(f2s.y));
    const float2 sc = make_float2(__fdividef(0.25f, c.x), __fdividef(0.25f, c.y));
    const float2 tr = add2(add2(F[0], F[4]), F[8]);
    float2 a[10];
    a[0] = mul2(add2(tr, c), sc);
    a[1] = mul2(add2(sub2(sub2(F[0], F[4]), F[8]), c), sc);
    a[2] = mul2(add2(sub2(sub2(F[4], F[0]), F[8]), c), sc);
    a[3] = mul2(add2(sub2(sub2(F[8], F[0]), F[4]), c), sc);
    a[4] = mul2(sub2(F[7], F[5]), sc);
    a[5] = mul2(sub2(F[2], F[6]), sc);
    a[6] = mul2(sub2(F[3], F[1]), sc);
    a[7] = mul2(add2(F[1], F[3]), sc);
    a[8] = mul2(add2(F[2], F[6]), sc);
    a[9] = mul2(add2(F[5], F[7]), sc);
    sym4_square2(a);
    sym4_square2(a);
    sym4_square2(a);
    // rank-one test on P: trace(P^2) = |P|_F^2 against trace(P)^2
    float2 t = add2(add2(a[0], a[1]), add2(a[2], a[3]));
    float2 fro = mul2(a[0], a[0]);
#pragma unroll
    for (int i = 1; i < 4; ++i) fro = fma2(a[i], a[i], fro);
    float2 off = mul2(a[4], a[4]);
#pragma unroll
    for (int i = 5; i < 10; ++i) off = fma2(a[i], a[i], off);
    fro = fma2(f2(2.f), off, fro);
    bool todo_x = fro.x < (1.0f - 4e-7f) * t.x * t.x;
    bool todo_y = fro.y < (1.0f - 4e-7f) * t.y * t.y;
    if (todo_x || todo_y) {
        // slow convergence (strongly stretched or inverted F): normalised
        // squarings of the unconverged lanes until P is rank one
        float2 tt = t;  // trace of the current P
        for (int k = 0; k < kTail && (todo_x || todo_y); ++k) {
            const float2 it = make_float2(__fdividef(1.0f, tt.x), __fdividef(1.0f, tt.y));
            float2 b[10];
#pragma unroll
            for (int i = 0; i < 10; ++i) b[i] = mul2(a[i], it);
            sym4_square2(b);
            const float2 tn = add2(add2(b[0], b[1]), add2(b[2], b[3]));
#pragma unroll
            for (int i = 0; i < 10; ++i) {
                if (todo_x) a[i].x = b[i].x;
                if (todo_y) a[i].y = b[i].y;
            }
            if (todo_x) { tt.x = tn.x; todo_x = !(tn.x >= 1.0f - 4e-7f); }
            if (todo_y) { tt.y = tn.y; todo_y = !(tn.y >= 1.0f - 4e-7f); }
        }
    }
    float ax[10], ay[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) { ax[i] = a[i].x; ay[i] = a[i].y; }
    float qa[4], qb[4];
    dominant_column(ax, qa);
    dominant_column(ay, qb);
    const float2 qw = make_float2(qa[0], qb[0]), qx = make_float2(qa[1], qb[1]), qy = make_float2(qa[2], qb[2]),
                 qz = make_float2(qa[3], qb[3]);
    const float2 xx = mul2(qx, qx), yy = mul2(qy, qy), zz = mul2(qz, qz);
    const float2 xy = mul2(qx, qy), xz = mul2(qx, qz), yz = mul2(qy, qz);
    const float2 wx = mul2(qw, qx), wy = mul2(qw, qy), wz = mul2(qw, qz);
    const float2 one = f2(1.f), m2 = f2(-2.f), p2 = f2(2.f);
    R[0] = fma2(m2, add2(yy, zz), one); R[1] = mul2(p2, sub2(xy, wz)); R[2] = mul2(p2, add2(xz, wy));
    R[3] = mul2(p2, add2(xy, wz)); R[4] = fma2(m2, add2(xx, zz), one); R[5] = mul2(p2, sub2(yz, wx));
    R[6] = mul2(p2, sub2(xz, wy)); R[7] = mul2(p2, add2(yz, wx)); R[8] = fma2(m2, add2(xx, yy), one);
}

}  // namespace pdgb
