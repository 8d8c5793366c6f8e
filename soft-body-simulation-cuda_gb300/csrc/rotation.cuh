// Register-resident closest proper rotation of a 3x3 matrix (device code).
//
// The reference extracts R from an SVD, R = U V^T with U, V proper
// rotations and the smallest singular value carrying the sign of det F
// (svd.cuh:7-14, pdUtil.cu:113-122).  The scheme here follows McAdams et al.,
// "Computing the Singular Value Decomposition of 3x3 matrices with minimal
// branching and elementary floating point operations" (UW-Madison TR1690,
// 2011): approximate-Givens Jacobi sweeps on S = F^T F with the rotation kept
// as a quaternion, sort of the columns of F V by norm, then U.  U is formed
// by Gram-Schmidt on the two largest columns and a cross product for the
// third, which keeps U proper and gives det F's sign to the smallest
// singular value, as the reference's SVD does.
#pragma once

namespace pdgb {

// One approximate Jacobi conjugation in the (p, q) plane, r the third index:
// chooses the half-angle (ch, sh) that approximately zeroes s_pq, applies
// S <- Q^T S Q and returns (ch, sh) for the quaternion update.
__device__ __forceinline__ void jacobi_conjugate(float& spp, float& sqq, float& spq, float& srp, float& srq,
                                                 float& ch, float& sh) {
    constexpr float kGamma = 5.828427124746190f;  // (1 + sqrt 2)^2
    constexpr float kCos8 = 0.9238795325112867f;  // cos(pi/8)
    constexpr float kSin8 = 0.3826834323650898f;  // sin(pi/8)
    float a = 2.0f * (spp - sqq);
    float b = spq;
    const bool ok = kGamma * b * b < a * a;
    const float w = rsqrtf(fmaf(a, a, b * b));
    ch = ok ? w * a : kCos8;
    sh = ok ? w * b : kSin8;
    const float c = fmaf(ch, ch, -sh * sh);
    const float s = 2.0f * sh * ch;
    const float c2 = c * c, s2 = s * s, cs = c * s;
    const float npp = fmaf(c2, spp, fmaf(2.0f * cs, spq, s2 * sqq));
    const float nqq = fmaf(s2, spp, fmaf(-2.0f * cs, spq, c2 * sqq));
    const float npq = fmaf(cs, sqq - spp, (c2 - s2) * spq);
    const float nrp = fmaf(c, srp, s * srq);
    const float nrq = fmaf(-s, srp, c * srq);
    spp = npp;
    sqq = nqq;
    spq = npq;
    srp = nrp;
    srq = nrq;
}

// Quaternion (w, x, y, z) right-multiplied by (ch, sh * e_axis).
__device__ __forceinline__ void quat_axis_x(float& w, float& x, float& y, float& z, float ch, float sh) {
    const float nw = fmaf(w, ch, -x * sh), nx = fmaf(x, ch, w * sh), ny = fmaf(y, ch, z * sh), nz = fmaf(z, ch, -y * sh);
    w = nw; x = nx; y = ny; z = nz;
}
__device__ __forceinline__ void quat_axis_y(float& w, float& x, float& y, float& z, float ch, float sh) {
    const float nw = fmaf(w, ch, -y * sh), nx = fmaf(x, ch, -z * sh), ny = fmaf(y, ch, w * sh), nz = fmaf(z, ch, x * sh);
    w = nw; x = nx; y = ny; z = nz;
}
__device__ __forceinline__ void quat_axis_z(float& w, float& x, float& y, float& z, float ch, float sh) {
    const float nw = fmaf(w, ch, -z * sh), nx = fmaf(x, ch, y * sh), ny = fmaf(y, ch, -x * sh), nz = fmaf(z, ch, w * sh);
    w = nw; x = nx; y = ny; z = nz;
}

template <int kSweeps = 4>
__device__ __forceinline__ void closest_rotation(const float F[9], float R[9]) {
    // S = F^T F (symmetric)
    float s00 = F[0] * F[0] + F[3] * F[3] + F[6] * F[6];
    float s11 = F[1] * F[1] + F[4] * F[4] + F[7] * F[7];
    float s22 = F[2] * F[2] + F[5] * F[5] + F[8] * F[8];
    float s01 = F[0] * F[1] + F[3] * F[4] + F[6] * F[7];
    float s02 = F[0] * F[2] + F[3] * F[5] + F[6] * F[8];
    float s12 = F[1] * F[2] + F[4] * F[5] + F[7] * F[8];
    float qw = 1.f, qx = 0.f, qy = 0.f, qz = 0.f;
#pragma unroll
    for (int sweep = 0; sweep < kSweeps; ++sweep) {
        float ch, sh;
        // plane (0,1), rotation about z
        jacobi_conjugate(s00, s11, s01, s02, s12, ch, sh);
        quat_axis_z(qw, qx, qy, qz, ch, sh);
        // plane (1,2), rotation about x
        jacobi_conjugate(s11, s22, s12, s01, s02, ch, sh);
        quat_axis_x(qw, qx, qy, qz, ch, sh);
        // plane (2,0), rotation about y
        jacobi_conjugate(s22, s00, s02, s12, s01, ch, sh);
        quat_axis_y(qw, qx, qy, qz, ch, sh);
    }
    const float qn = rsqrtf(qw * qw + qx * qx + qy * qy + qz * qz);
    qw *= qn; qx *= qn; qy *= qn; qz *= qn;
    // V (row-major) from the quaternion; v_j = column j.
    float v0x = 1.f - 2.f * (qy * qy + qz * qz), v1x = 2.f * (qx * qy - qw * qz), v2x = 2.f * (qx * qz + qw * qy);
    float v0y = 2.f * (qx * qy + qw * qz), v1y = 1.f - 2.f * (qx * qx + qz * qz), v2y = 2.f * (qy * qz - qw * qx);
    float v0z = 2.f * (qx * qz - qw * qy), v1z = 2.f * (qy * qz + qw * qx), v2z = 1.f - 2.f * (qx * qx + qy * qy);
    // columns of B = F V
    float b0x = F[0] * v0x + F[1] * v0y + F[2] * v0z;
    float b0y = F[3] * v0x + F[4] * v0y + F[5] * v0z;
    float b0z = F[6] * v0x + F[7] * v0y + F[8] * v0z;
    float b1x = F[0] * v1x + F[1] * v1y + F[2] * v1z;
    float b1y = F[3] * v1x + F[4] * v1y + F[5] * v1z;
    float b1z = F[6] * v1x + F[7] * v1y + F[8] * v1z;
    float b2x = F[0] * v2x + F[1] * v2y + F[2] * v2z;
    float b2y = F[3] * v2x + F[4] * v2y + F[5] * v2z;
    float b2z = F[6] * v2x + F[7] * v2y + F[8] * v2z;
    float n0 = b0x * b0x + b0y * b0y + b0z * b0z;
    float n1 = b1x * b1x + b1y * b1y + b1z * b1z;
    float n2 = b2x * b2x + b2y * b2y + b2z * b2z;
    // sort columns by decreasing norm; a swap negates one column so that
    // det V stays +1.
#define PDGB_SWAPNEG(a, b)      \
    {                           \
        const float t_ = a;     \
        a = b;                  \
        b = -t_;                \
    }
    if (n0 < n1) {
        PDGB_SWAPNEG(b0x, b1x) PDGB_SWAPNEG(b0y, b1y) PDGB_SWAPNEG(b0z, b1z)
        PDGB_SWAPNEG(v0x, v1x) PDGB_SWAPNEG(v0y, v1y) PDGB_SWAPNEG(v0z, v1z)
        const float t = n0; n0 = n1; n1 = t;
    }
    if (n0 < n2) {
        PDGB_SWAPNEG(b0x, b2x) PDGB_SWAPNEG(b0y, b2y) PDGB_SWAPNEG(b0z, b2z)
        PDGB_SWAPNEG(v0x, v2x) PDGB_SWAPNEG(v0y, v2y) PDGB_SWAPNEG(v0z, v2z)
        const float t = n0; n0 = n2; n2 = t;
    }
    if (n1 < n2) {
        PDGB_SWAPNEG(b1x, b2x) PDGB_SWAPNEG(b1y, b2y) PDGB_SWAPNEG(b1z, b2z)
        PDGB_SWAPNEG(v1x, v2x) PDGB_SWAPNEG(v1y, v2y) PDGB_SWAPNEG(v1z, v2z)
        const float t = n1; n1 = n2; n2 = t;
    }
#undef PDGB_SWAPNEG
    float u0x, u0y, u0z, u1x, u1y, u1z;
    if (n0 > 1e-30f) {
        const float i0 = rsqrtf(n0);
        u0x = b0x * i0; u0y = b0y * i0; u0z = b0z * i0;
        const float d = u0x * b1x + u0y * b1y + u0z * b1z;
        float tx = b1x - d * u0x, ty = b1y - d * u0y, tz = b1z - d * u0z;
        float tn = tx * tx + ty * ty + tz * tz;
        if (!(tn > 1e-12f * n0)) {
            // rank-1 F: any unit vector orthogonal to u0 (from the axis u0 is
            // least aligned with).
            const float ax = fabsf(u0x), ay = fabsf(u0y), az = fabsf(u0z);
            float ex = 0.f, ey = 0.f, ez = 0.f;
            if (ax <= ay && ax <= az) ex = 1.f; else if (ay <= az) ey = 1.f; else ez = 1.f;
            const float dd = u0x * ex + u0y * ey + u0z * ez;
            tx = ex - dd * u0x; ty = ey - dd * u0y; tz = ez - dd * u0z;
            tn = tx * tx + ty * ty + tz * tz;
        }
        const float it = rsqrtf(tn);
        u1x = tx * it; u1y = ty * it; u1z = tz * it;
    } else {
        u0x = 1.f; u0y = 0.f; u0z = 0.f;
        u1x = 0.f; u1y = 1.f; u1z = 0.f;
    }
    const float u2x = u0y * u1z - u0z * u1y;
    const float u2y = u0z * u1x - u0x * u1z;
    const float u2z = u0x * u1y - u0y * u1x;
    // R = U V^T = sum_j u_j v_j^T
    R[0] = u0x * v0x + u1x * v1x + u2x * v2x;
    R[1] = u0x * v0y + u1x * v1y + u2x * v2y;
    R[2] = u0x * v0z + u1x * v1z + u2x * v2z;
    R[3] = u0y * v0x + u1y * v1x + u2y * v2x;
    R[4] = u0y * v0y + u1y * v1y + u2y * v2y;
    R[5] = u0y * v0z + u1y * v1z + u2y * v2z;
    R[6] = u0z * v0x + u1z * v1x + u2z * v2x;
    R[7] = u0z * v0y + u1z * v1y + u2z * v2y;
    R[8] = u0z * v0z + u1z * v1z + u2z * v2z;
}

// Closest proper rotation by Horn's quaternion form: for unit q,
// tr(R(q)^T F) = q^T N(F) q with N the symmetric 4x4 matrix below, so the
// rotation maximising tr(R^T F) -- the closest proper rotation, the same R as
// the reference's U V^T with a signed smallest singular value -- is the
// eigenvector of N's largest eigenvalue.  It is found as the dominant
// eigenvector of A = N + c I (c = 0.6 |F|_F > |sigma_3| keeps the top
// eigenvalue dominant even for inverted F) by repeated squaring: P = A^4
// after 2 squarings, then, while P is not close to rank one, up to kTail
// normalised squarings.  For eigenvalues 1 >= r_2, r_3, r_4 of the scaled P,
// trace(P^2) / trace(P)^2 = 1 - 2 sum r_i + O(r^2); P counts as rank one when
// that ratio is at least 1 - 5e-4 (sum r_i <~ 2.5e-4).  The column of P with
// the largest diagonal entry, multiplied once more by P (which squares the
// remaining error, to ~1e-7), is q.  Elements within a few percent of a
// rotation stop at A^4.  A test at float resolution (1 - 4e-7) gave the same
// rotations to ~6e-7 but, being decided by the rounding of trace(P^2), sent
// ~7 % of the elements at 1 % strain into an extra squaring -- and a warp
// pays for one when any of its lanes does.
__device__ __forceinline__ void sym4_square(float a[10]) {
    // a = {ww, xx, yy, zz, wx, wy, wz, xy, xz, yz}
    const float ww = a[0], xx = a[1], yy = a[2], zz = a[3], wx = a[4], wy = a[5], wz = a[6], xy = a[7], xz = a[8],
                yz = a[9];
    a[0] = fmaf(ww, ww, fmaf(wx, wx, fmaf(wy, wy, wz * wz)));
    a[1] = fmaf(wx, wx, fmaf(xx, xx, fmaf(xy, xy, xz * xz)));
    a[2] = fmaf(wy, wy, fmaf(xy, xy, fmaf(yy, yy, yz * yz)));
    a[3] = fmaf(wz, wz, fmaf(xz, xz, fmaf(yz, yz, zz * zz)));
    a[4] = fmaf(ww, wx, fmaf(wx, xx, fmaf(wy, xy, wz * xz)));
    a[5] = fmaf(ww, wy, fmaf(wx, xy, fmaf(wy, yy, wz * yz)));
    a[6] = fmaf(ww, wz, fmaf(wx, xz, fmaf(wy, yz, wz * zz)));
    a[7] = fmaf(wx, wy, fmaf(xx, xy, fmaf(xy, yy, xz * yz)));
    a[8] = fmaf(wx, wz, fmaf(xx, xz, fmaf(xy, yz, xz * zz)));
    a[9] = fmaf(wy, wz, fmaf(xy, xz, fmaf(yy, yz, yz * zz)));
}

// |P|_F^2 = trace(P^2) of a symmetric 4x4 in the packed layout above.
__device__ __forceinline__ float sym4_frob2(const float a[10]) {
    const float d = fmaf(a[0], a[0], fmaf(a[1], a[1], fmaf(a[2], a[2], a[3] * a[3])));
    const float o = fmaf(a[4], a[4], fmaf(a[5], a[5], fmaf(a[6], a[6], fmaf(a[7], a[7], fmaf(a[8], a[8], a[9] * a[9])))));
    return fmaf(2.f, o, d);
}

template <int kTail = 8>
__device__ __forceinline__ void closest_rotation_horn(const float F[9], float R[9]) {
    float f2 = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) f2 = fmaf(F[i], F[i], f2);
    f2 = fmaxf(f2, 1e-30f);
    const float c = 0.6f * f2 * rsqrtf(f2);      // shift; precision irrelevant
    const float sc = __fdividef(0.25f, c);       // eigenvalues of A / (4c) <= 1
    float a[10];
    a[0] = (F[0] + F[4] + F[8] + c) * sc;
    a[1] = (F[0] - F[4] - F[8] + c) * sc;
    a[2] = (-F[0] + F[4] - F[8] + c) * sc;
    a[3] = (-F[0] - F[4] + F[8] + c) * sc;
    a[4] = (F[7] - F[5]) * sc;
    a[5] = (F[2] - F[6]) * sc;
    a[6] = (F[3] - F[1]) * sc;
    a[7] = (F[1] + F[3]) * sc;
    a[8] = (F[2] + F[6]) * sc;
    a[9] = (F[5] + F[7]) * sc;
    // A^4: the top eigenvalue of A/(4c) is >= 1/4, so no underflow.
    sym4_square(a);
    sym4_square(a);
    float t = a[0] + a[1] + a[2] + a[3];
    for (int k = 0; k < kTail && sym4_frob2(a) < (1.0f - 5e-4f) * t * t; ++k) {
        const float it = __fdividef(1.0f, t);
#pragma unroll
        for (int i = 0; i < 10; ++i) a[i] *= it;
        sym4_square(a);
        t = a[0] + a[1] + a[2] + a[3];
    }
    // dominant column, one more power step, normalised
    float c0 = a[0], c1 = a[4], c2 = a[5], c3 = a[6], best = a[0];
    if (a[1] > best) { best = a[1]; c0 = a[4]; c1 = a[1]; c2 = a[7]; c3 = a[8]; }
    if (a[2] > best) { best = a[2]; c0 = a[5]; c1 = a[7]; c2 = a[2]; c3 = a[9]; }
    if (a[3] > best) { c0 = a[6]; c1 = a[8]; c2 = a[9]; c3 = a[3]; }
    float qw = fmaf(a[0], c0, fmaf(a[4], c1, fmaf(a[5], c2, a[6] * c3)));
    float qx = fmaf(a[4], c0, fmaf(a[1], c1, fmaf(a[7], c2, a[8] * c3)));
    float qy = fmaf(a[5], c0, fmaf(a[7], c1, fmaf(a[2], c2, a[9] * c3)));
    float qz = fmaf(a[6], c0, fmaf(a[8], c1, fmaf(a[9], c2, a[3] * c3)));
    const float n = rsqrtf(fmaxf(qw * qw + qx * qx + qy * qy + qz * qz, 1e-37f));
    qw *= n; qx *= n; qy *= n; qz *= n;
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
    const float xy = qx * qy, xz = qx * qz, yz = qy * qz, wx = qw * qx, wy = qw * qy, wz = qw * qz;
    R[0] = 1.f - 2.f * (yy + zz); R[1] = 2.f * (xy - wz);       R[2] = 2.f * (xz + wy);
    R[3] = 2.f * (xy + wz);       R[4] = 1.f - 2.f * (xx + zz); R[5] = 2.f * (yz - wx);
    R[6] = 2.f * (xz - wy);       R[7] = 2.f * (yz + wx);       R[8] = 1.f - 2.f * (xx + yy);
}

}  // namespace pdgb
