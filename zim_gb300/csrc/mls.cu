// mls.cu -- organised-window moving-least-squares smoothing.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_MLS_Filter.cpp:11-441 (CPU) and
// JSLAB_MLS_Filter.cu:14-466 (GPU).  Per valid pixel, over the (2hw+1)^2
// window of valid neighbours within the 3-D cut-off: weights
// w = exp(-d^2 / 2 sigma^2), weighted centroid, weighted covariance, its
// smallest eigenvector in closed form (the normal), then an order-0/1/2
// polynomial fit f(u, v) in a tangent frame about the normal by Cholesky with
// the 2 -> 1 -> 0 fallback, and projection of the point onto the fitted
// surface.
// Order selection follows the CPU reference: order drops to 0 when fewer than
// {3, 5, 8}[order] neighbours.  Coordinates are accumulated relative to the
// query point, which keeps FP32 sums at millimetre scale.
#include <cmath>

#include "zim_tiles.cuh"

namespace {

constexpr int MX = 16, MY = 16;

// Unit eigenvector of the smallest eigenvalue of a symmetric 3x3 matrix (the
// surface normal of a weighted covariance): the eigenvalue in closed form by
// the published trigonometric solution of the characteristic cubic (O. K.
// Smith, "Eigenvalues of a symmetric 3x3 matrix", Communications of the ACM
// 4(4):168, 1961: shift by q = tr/3, scale by p, phi = acos(det(B)/2)/3), the
// same method the reference's symmetricEigen3x3 uses
// (JSLAB_MLS_Filter.cpp:11-106), which is why the variable names and the
// diagonal/degenerate thresholds read alike; the vector is the longest cross
// product of two rows of C - lambda I.  Zero when that eigenvalue is not
// simple enough to give a direction.
__device__ void sym_normal3(const float C[3][3], float n[3]) {
    const float p1 = C[0][1] * C[0][1] + C[0][2] * C[0][2] + C[1][2] * C[1][2];
    if (p1 < 1e-20f) {  // diagonal: the axis of the smallest entry
        int m = 0;
        if (C[1][1] < C[m][m]) m = 1;
        if (C[2][2] < C[m][m]) m = 2;
        n[0] = m == 0 ? 1.f : 0.f; n[1] = m == 1 ? 1.f : 0.f; n[2] = m == 2 ? 1.f : 0.f;
        return;
    }
    const float tr = C[0][0] + C[1][1] + C[2][2];
    const float q = tr / 3.0f;
    float B[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] = C[i][j] - (i == j ? q : 0.f);
    float p2 = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2] + 2.0f * p1;
    float p = sqrtf(p2 / 6.0f);
    float ip = p > 1e-15f ? 1.0f / p : 0.f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] *= ip;
    float det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
    float r = fminf(1.f, fmaxf(-1.f, det * 0.5f));
    float phi = acosf(r) / 3.0f;
    const float ev = q + 2.0f * p * cosf(phi + 2.0f * ZIM_PI_F / 3.0f);
    float A[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = C[i][j] - (i == j ? ev : 0.f);
    float c01[3] = {A[0][1] * A[1][2] - A[0][2] * A[1][1], A[0][2] * A[1][0] - A[0][0] * A[1][2],
                    A[0][0] * A[1][1] - A[0][1] * A[1][0]};
    float c02[3] = {A[0][1] * A[2][2] - A[0][2] * A[2][1], A[0][2] * A[2][0] - A[0][0] * A[2][2],
                    A[0][0] * A[2][1] - A[0][1] * A[2][0]};
    float c12[3] = {A[1][1] * A[2][2] - A[1][2] * A[2][1], A[1][2] * A[2][0] - A[1][0] * A[2][2],
                    A[1][0] * A[2][1] - A[1][1] * A[2][0]};
    float l01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
    float l02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
    float l12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
    float b0 = c12[0], b1 = c12[1], b2 = c12[2], bl = l12;
    if (l01 > bl) { b0 = c01[0]; b1 = c01[1]; b2 = c01[2]; bl = l01; }
    if (l02 > bl) { b0 = c02[0]; b1 = c02[1]; b2 = c02[2]; bl = l02; }
    float il = bl > 1e-20f ? rsqrtf(bl) : 0.f;
    n[0] = b0 * il; n[1] = b1 * il; n[2] = b2 * il;
}

// Cholesky solve of an N x N system held in registers (every index is a
// compile-time constant after unrolling); thr[i] is the singular-pivot
// threshold of row i (the reference's 1e-12 expressed in the scaled basis).
template <int N>
__device__ __forceinline__ bool cholesky_fixed(const float (&A)[N][N], const float (&b)[N], float (&x)[N],
                                               const float (&thr)[6]) {
    float L[N][N], iL[N];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j <= i; j++) {
            float s = A[i][j];
#pragma unroll
            for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
            if (i == j) {
                ok = ok && s > thr[i];
                const float g = fmaxf(s, 1e-30f);
                iL[i] = rsqrtf(g);  // 1 / L[i][i]: the solves multiply
                L[i][j] = g * iL[i];
            } else {
                L[i][j] = s * iL[j];
            }
        }
    float y[N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        float s = b[i];
#pragma unroll
        for (int k = 0; k < i; k++) s -= L[i][k] * y[k];
        y[i] = s * iL[i];
    }
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
        float s = y[i];
#pragma unroll
        for (int k = i + 1; k < N; k++) s -= L[k][i] * x[k];
        x[i] = s * iL[i];
    }
    return ok;
}

// Gaussian weight exp(-d2 / (2 s^2)) = 2^(d2 * kw) with kw = -log2(e) / (2 s^2):
// one multiply and the hardware base-2 exponential (PTX ex2.approx).
__device__ __forceinline__ float mls_weight_arg(float a) {
    float w;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(w) : "f"(a));
    return w;
}
__device__ __forceinline__ float mls_weight(float d2, float kw) { return mls_weight_arg(d2 * kw); }

// The state of one query after the first sweep: centroid (relative to the
// query point), unit normal and orthonormal tangent frame, and the polynomial
// order the fit uses.
struct MlsFrame {
    float cx, cy, cz;
    float nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z;
    int cur;
};

// From the first sweep's weighted sums about the query point (weight sum ws,
// in-radius count nv, sum w d, sum w d d^T): the centroid, the weighted
// covariance about it, its smallest eigenvector (the normal) and the tangent
// frame.  False when the point keeps its position (fewer than 3 neighbours or
// no weight).  Order selection follows the CPU reference: order drops to 0
// with fewer than {3, 5, 8}[order] neighbours.
__device__ __forceinline__ bool mls_frame(float ws, int nv, float cx, float cy, float cz, float m00, float m01,
                                          float m02, float m11, float m12, float m22, int order, MlsFrame& F,
                                          float (*Cout)[3] = nullptr) {
    if (nv < 3 || ws < 1e-12f) return false;
    const float iw = 1.0f / ws;
    cx *= iw; cy *= iw; cz *= iw;
    // weighted covariance about the centroid: sum w d d^T - ws c c^T
    float C[3][3];
    C[0][0] = fmaf(-ws * cx, cx, m00); C[0][1] = fmaf(-ws * cx, cy, m01); C[0][2] = fmaf(-ws * cx, cz, m02);
    C[1][1] = fmaf(-ws * cy, cy, m11); C[1][2] = fmaf(-ws * cy, cz, m12); C[2][2] = fmaf(-ws * cz, cz, m22);
    C[1][0] = C[0][1]; C[2][0] = C[0][2]; C[2][1] = C[1][2];
    if (Cout)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Cout[i][j] = C[i][j];
    float nv3[3];
    sym_normal3(C, nv3);
    // Orthonormal tangent frame about the normal: the polynomial spaces of
    // orders 0-2 are unchanged by a rotation of (u, v), so any orthonormal pair
    // fits the same surface; t1 is the coordinate axis least aligned with the
    // normal, orthogonalised against it, and t2 = n x t1.  (A zero normal gives
    // a zero frame: the fit fails and the point stays.)
    float nx = nv3[0], ny = nv3[1], nz = nv3[2];
    float t1x = 0.f, t1y = 0.f, t1z = 0.f, t2x = 0.f, t2y = 0.f, t2z = 0.f;
    {
        float nn = nx * nx + ny * ny + nz * nz;
        if (nn > 1e-30f) {
            float in = rsqrtf(nn);
            nx *= in; ny *= in; nz *= in;
            const float ux = fabsf(nx), uy = fabsf(ny), uz = fabsf(nz);
            const int a = ux <= uy && ux <= uz ? 0 : (uy <= uz ? 1 : 2);
            const float d = a == 0 ? nx : (a == 1 ? ny : nz);
            float ax = (a == 0 ? 1.f : 0.f) - d * nx, ay = (a == 1 ? 1.f : 0.f) - d * ny, az = (a == 2 ? 1.f : 0.f) - d * nz;
            float ia = rsqrtf(ax * ax + ay * ay + az * az);  // >= 2/3: the axis is at least 54.7 deg off the normal
            t1x = ax * ia; t1y = ay * ia; t1z = az * ia;
            t2x = ny * t1z - nz * t1y;
            t2y = nz * t1x - nx * t1z;
            t2z = nx * t1y - ny * t1x;
        } else {
            nx = ny = nz = 0.f;
        }
    }
    F.cx = cx; F.cy = cy; F.cz = cz;
    F.nx = nx; F.ny = ny; F.nz = nz;
    F.t1x = t1x; F.t1y = t1y; F.t1z = t1z; F.t2x = t2x; F.t2y = t2y; F.t2z = t2z;
    const int min_nb = order == 2 ? 8 : (order == 1 ? 5 : 3);
    F.cur = nv >= min_nb ? order : 0;
    return true;
}

// Normal equations of the order-N polynomial fit (N = 3: 1, u, v; N = 6: also
// u^2, uv, v^2) in tangent coordinates u, v (scaled by is) and height f about
// the centroid.  Entry (a, b) is the weighted moment of u^i v^j whose exponents
// are those of basis terms a and b added.  The moments of degree <= 2 and the
// right-hand sides sum w f, sum w f u, sum w f v follow from the first sweep:
// about the centroid sum w u = sum w v = sum w f = 0, and sum w (u, v, f)
// (u, v, f)^T is the weighted covariance C expressed in the frame
// (t1 is, t2 is, n).  So the second sweep (N = 6 only) sums just the nine
// moments of degree 3 and 4 and sum w f (u^2, uv, v^2).
template <int N, typename Visit>
__device__ __forceinline__ void fit_normal_equations(Visit& visit, float kw, float r2c, float is, float ws,
                                                     const float (&C)[3][3], const MlsFrame& F, float (&A)[N][N],
                                                     float (&bv)[N]) {
    float Ct1[3], Ct2[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        Ct1[a] = fmaf(C[a][0], F.t1x, fmaf(C[a][1], F.t1y, C[a][2] * F.t1z));
        Ct2[a] = fmaf(C[a][0], F.t2x, fmaf(C[a][1], F.t2y, C[a][2] * F.t2z));
    }
    const float is2 = is * is;
    const float m20 = is2 * fmaf(F.t1x, Ct1[0], fmaf(F.t1y, Ct1[1], F.t1z * Ct1[2]));
    const float m11 = is2 * fmaf(F.t1x, Ct2[0], fmaf(F.t1y, Ct2[1], F.t1z * Ct2[2]));
    const float m02 = is2 * fmaf(F.t2x, Ct2[0], fmaf(F.t2y, Ct2[1], F.t2z * Ct2[2]));
    A[0][0] = ws; A[0][1] = 0.f; A[0][2] = 0.f;
    A[1][1] = m20; A[1][2] = m11; A[2][2] = m02;
    bv[0] = 0.f;
    bv[1] = is * fmaf(F.nx, Ct1[0], fmaf(F.ny, Ct1[1], F.nz * Ct1[2]));
    bv[2] = is * fmaf(F.nx, Ct2[0], fmaf(F.ny, Ct2[1], F.nz * Ct2[2]));
    if constexpr (N == 6) {
        // u = (d - c) . t1 is as one FMA chain on d (likewise v, f)
        const float ax = F.t1x * is, ay = F.t1y * is, az = F.t1z * is;
        const float bx = F.t2x * is, by = F.t2y * is, bz = F.t2z * is;
        const float nx = F.nx, ny = F.ny, nz = F.nz;
        const float uc = fmaf(F.cx, ax, fmaf(F.cy, ay, F.cz * az));
        const float vc = fmaf(F.cx, bx, fmaf(F.cy, by, F.cz * bz));
        const float fc = fmaf(F.cx, nx, fmaf(F.cy, ny, F.cz * nz));
        // u and v as the two lanes of paired FP32 instructions (each lane
        // rounded as the scalar instruction, so every sum below is the scalar
        // sequence's): (u, v) = d . (t1, t2) is - (uc, vc) as one chain
        const float2 axy = make_float2(ax, bx), ayy = make_float2(ay, by), azz = make_float2(az, bz);
        const float2 c_uv = make_float2(-uc, -vc);
        float2 m30_21 = make_float2(0.f, 0.f), m12_03 = m30_21, m40_31 = m30_21, m22_04 = m30_21, b3_4 = m30_21;
        float m13 = 0.f, b5 = 0.f;
        visit([&](float2 dxy, float dz) {
            const float d2 = fmaf(dz, dz, fmaf(dxy.y, dxy.y, dxy.x * dxy.x));
            if (!(d2 <= r2c)) return;
            const float w = mls_weight(d2, kw);
            const float2 uv = __ffma2_rn(make_float2(dxy.x, dxy.x), axy,
                                         __ffma2_rn(make_float2(dxy.y, dxy.y), ayy,
                                                    __ffma2_rn(make_float2(dz, dz), azz, c_uv)));
            const float f = fmaf(dxy.x, nx, fmaf(dxy.y, ny, fmaf(dz, nz, -fc)));
            const float2 wuv = __fmul2_rn(make_float2(w, w), uv);                // (w u, w v)
            const float wf = w * f;
            const float2 uu_uv = __fmul2_rn(make_float2(uv.x, uv.x), uv);        // (u u, u v)
            const float vv = uv.y * uv.y;
            const float2 vv2 = make_float2(vv, vv);
            m30_21 = __ffma2_rn(make_float2(wuv.x, wuv.x), uu_uv, m30_21);        // w u (uu, uv)
            m12_03 = __ffma2_rn(wuv, vv2, m12_03);                                // (w u, w v) vv
            const float2 wuu_vv = __fmul2_rn(wuv, uv);                            // (w u u, w v v)
            m40_31 = __ffma2_rn(make_float2(wuu_vv.x, wuu_vv.x), uu_uv, m40_31);  // w u u (uu, uv)
            m22_04 = __ffma2_rn(wuu_vv, vv2, m22_04);                             // (w u u, w v v) vv
            m13 = fmaf(wuu_vv.y, uu_uv.y, m13);                                   // w v v uv
            b3_4 = __ffma2_rn(make_float2(wf, wf), uu_uv, b3_4);                  // w f (uu, uv)
            b5 = fmaf(wf, vv, b5);
        });
        const float m30 = m30_21.x, m21 = m30_21.y, m12 = m12_03.x, m03 = m12_03.y;
        const float m40 = m40_31.x, m31 = m40_31.y, m22 = m22_04.x, m04 = m22_04.y;
        // basis exponents: 1 (0,0), u (1,0), v (0,1), u^2 (2,0), uv (1,1), v^2 (0,2)
        A[0][3] = m20; A[0][4] = m11; A[0][5] = m02;
        A[1][3] = m30; A[1][4] = m21; A[1][5] = m12;
        A[2][3] = m21; A[2][4] = m12; A[2][5] = m03;
        A[3][3] = m40; A[3][4] = m31; A[3][5] = m22;
        A[4][4] = m22; A[4][5] = m13; A[5][5] = m04;
        bv[3] = b3_4.x; bv[4] = b3_4.y; bv[5] = b5;
    }
#pragma unroll
    for (int a = 0; a < N; a++)
#pragma unroll
        for (int b = 0; b < a; b++) A[a][b] = A[b][a];
}

// Singular-pivot thresholds of the Cholesky solve (the reference's 1e-12) for
// a basis scaled by is = 1 / cut-off radius: the pivot of a degree-d row
// scales by is^(2d).
__device__ __forceinline__ void mls_thresholds(float is, float (&thr)[6]) {
    const float s2 = is * is, s4 = s2 * s2;
    thr[0] = 1e-12f; thr[1] = thr[2] = 1e-12f * s2; thr[3] = thr[4] = thr[5] = 1e-12f * s4;
}

// Solves the order-N normal equations (N = 6 falls back to order 1 on their
// leading block, as the reference's 2 -> 1 fallback does) and projects the
// query point onto the fitted surface (onto the tangent plane when no fit is
// solved).  cur: the frame's order, lowered to 1 by the fallback.  (ox, oy,
// oz) is the moved point relative to the query point.
template <int N>
__device__ __forceinline__ void mls_solve_project(const MlsFrame& F, int cur, const float (&A)[N][N],
                                                  const float (&bv)[N], float is, float& ox, float& oy, float& oz) {
    float thr[6];
    mls_thresholds(is, thr);
    bool solved = false;
    float co[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (cur == 2 && N == 6) {
        float x6[N];
        solved = cholesky_fixed<N>(A, bv, x6, thr);
        if (solved) {
#pragma unroll
            for (int a = 0; a < N; a++) co[a] = x6[a];
        }
    }
    if (cur >= 1 && !solved) {
        // order 1 on the leading 3 x 3 block of the same normal equations
        float A3[3][3], b3[3], x3[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            b3[a] = bv[a];
#pragma unroll
            for (int b = 0; b < 3; b++) A3[a][b] = A[a][b];
        }
        solved = cholesky_fixed<3>(A3, b3, x3, thr);
        if (solved) {
            cur = 1;
#pragma unroll
            for (int a = 0; a < 3; a++) co[a] = x3[a];
        }
    }
    // query point relative to the centroid: e0 = p - c = -c_rel
    const float ex0 = -F.cx, ey0 = -F.cy, ez0 = -F.cz;
    if (!solved) {
        float dot = ex0 * F.nx + ey0 * F.ny + ez0 * F.nz;
        ox = -dot * F.nx; oy = -dot * F.ny; oz = -dot * F.nz;
    } else {
        float u0 = ex0 * F.t1x + ey0 * F.t1y + ez0 * F.t1z;
        float v0 = ex0 * F.t2x + ey0 * F.t2y + ez0 * F.t2z;
        float us = u0 * is, vs = v0 * is;
        float ff = co[0] + co[1] * us + co[2] * vs;
        if (cur == 2) ff += co[3] * us * us + co[4] * us * vs + co[5] * vs * vs;
        // out = c + u0 t1 + v0 t2 + f n = p + (c_rel + u0 t1 + v0 t2 + f n)
        ox = F.cx + u0 * F.t1x + v0 * F.t2x + ff * F.nx;
        oy = F.cy + u0 * F.t1y + v0 * F.t2y + ff * F.ny;
        oz = F.cz + u0 * F.t1z + v0 * F.t2z + ff * F.nz;
    }
}

// MLS of one valid point.  visit(fn) calls fn((dx, dy), dz) with the offset from
// the query point of every valid neighbour of its window (in a fixed order);
// the distance test against the cut-off is made here.
template <typename Visit>
__device__ __forceinline__ void mls_point(float inv_2s2, int order, float r2c, Visit visit, float& ox, float& oy,
                                          float& oz, bool& moved) {
    moved = false;
    const float kw = -1.44269504088896341f * inv_2s2;  // -log2(e) / (2 s^2)
    // 1. weighted centroid and covariance in one sweep, from the moments about
    // the query point (offsets of at most the cut-off radius, so the FP32
    // moments lose ~1e-7 of |offset|^2 to cancellation: the frame turns by
    // ~1e-7 rad, far below the 1e-5 mm the points are held to)
    // (x, y) pairs as the two lanes of paired FP32 instructions
    float2 cxy = make_float2(0.f, 0.f), m00_11 = cxy;
    float cz = 0.f, ws = 0.f, m01 = 0.f, m02 = 0.f, m12 = 0.f, m22 = 0.f;
    int nv = 0;
    visit([&](float2 dxy, float dz) {
        const float d2 = fmaf(dz, dz, fmaf(dxy.y, dxy.y, dxy.x * dxy.x));
        if (!(d2 <= r2c)) return;
        const float w = mls_weight(d2, kw);
        const float2 wxy = __fmul2_rn(make_float2(w, w), dxy);            // (w dx, w dy)
        const float wz = w * dz;
        cxy = __fadd2_rn(cxy, wxy);
        cz += wz;
        m00_11 = __ffma2_rn(wxy, dxy, m00_11);
        m01 = fmaf(wxy.x, dxy.y, m01);
        m02 = fmaf(wxy.x, dz, m02);
        m12 = fmaf(wxy.y, dz, m12);
        m22 = fmaf(wz, dz, m22);
        ws += w;
        nv++;
    });
    MlsFrame F;
    float C[3][3];
    if (!mls_frame(ws, nv, cxy.x, cxy.y, cz, m00_11.x, m01, m02, m00_11.y, m12, m22, order, F, C)) return;
    // Polynomial basis in tangent coordinates scaled by 1/h (h = cut-off
    // radius): the fitted surface is the same, the normal equations are O(1).
    const float is = rsqrtf(r2c);
    if (F.cur == 2) {
        float A[6][6], bv[6];
        fit_normal_equations<6>(visit, kw, r2c, is, ws, C, F, A, bv);
        mls_solve_project<6>(F, 2, A, bv, is, ox, oy, oz);
    } else {
        float A[3][3], bv[3];
        fit_normal_equations<3>(visit, kw, r2c, is, ws, C, F, A, bv);
        mls_solve_project<3>(F, F.cur, A, bv, is, ox, oy, oz);
    }
    moved = true;
}

// Neighbours straight from global memory (windows too wide for shared memory).
__global__ void __launch_bounds__(MX* MY) mls_kernel(const float* __restrict__ src, const uint8_t* __restrict__ mask,
                                                     int rows, int cols, int hw, float inv_2s2, int order, float r2c,
                                                     float* __restrict__ dst) {
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= cols || y >= rows) return;
    const size_t o = (size_t)y * cols + x;
    const float px = src[3 * o], py = src[3 * o + 1], pz = src[3 * o + 2];
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool moved = false;
    if (mask[o]) {
        const int r0 = max(0, y - hw), r1 = min(rows, y + hw + 1), c0 = max(0, x - hw), c1 = min(cols, x + hw + 1);
        auto visit = [&](auto&& fn) {
            for (int i = r0; i < r1; i++)
                for (int j = c0; j < c1; j++) {
                    const size_t q = (size_t)i * cols + j;
                    if (!__ldg(mask + q)) continue;
                    fn(make_float2(__ldg(src + 3 * q) - px, __ldg(src + 3 * q + 1) - py), __ldg(src + 3 * q + 2) - pz);
                }
        };
        mls_point(inv_2s2, order, r2c, visit, ox, oy, oz, moved);
    }
    dst[3 * o] = moved ? px + ox : px;
    dst[3 * o + 1] = moved ? py + oy : py;
    dst[3 * o + 2] = moved ? pz + oz : pz;
}

// The tile and its hw halo staged in shared memory as float4, NaN for invalid
// and off-image pixels (their distance test fails).
inline size_t mls_smem_bytes(int hw) { return (size_t)(MX + 2 * hw) * (MY + 2 * hw) * sizeof(float4); }


// With pixel rays (rays != 0) each row of the window is cut to the disk beyond
// which the ray bound puts every point outside the cut-off: the pixels left out
// would fail the distance test, so the neighbours and their order are those
// of the full window.  The disk is the largest of the warp's (one loop bound).
// Every neighbour is a staged pixel, so the bound takes the largest distance of
// a staged point from its own ray (points smoothed across a depth edge lie far
// off their rays, but only near the edge).
// HW: the half-window at compile time (0: the hw argument), which makes the
// tile width and every neighbour offset constants.
template <int HW>
__global__ void __launch_bounds__(MX* MY) mls_smem_kernel(const float* __restrict__ src,
                                                          const uint8_t* __restrict__ mask, int rows, int cols, int hw_arg,
                                                          float inv_2s2, int order, float r2c, int rays,
                                                          zt::RayParams rp, float* __restrict__ dst) {
    extern __shared__ float4 mls_sp[];
    __shared__ unsigned warp_dev[MX * MY / 32];
    const int hw = HW ? HW : hw_arg;
    const int TW = MX + 2 * hw, TH = MY + 2 * hw;
    const int gx0 = blockIdx.x * MX - hw, gy0 = blockIdx.y * MY - hw;
    const int tid = threadIdx.y * MX + threadIdx.x;
    unsigned tdev = 0u;  // largest ray distance of this thread's staged points (float bits, >= 0)
    for (int t = tid; t < TW * TH; t += MX * MY) {
        const int ty = t / TW, tx = t - ty * TW;
        const int gx = gx0 + tx, gy = gy0 + ty;
        float4 v = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
        if (gx >= 0 && gy >= 0 && gx < cols && gy < rows) {
            const size_t q = (size_t)gy * cols + gx;
            if (__ldg(mask + q)) {
                v = make_float4(__ldg(src + 3 * q), __ldg(src + 3 * q + 1), __ldg(src + 3 * q + 2), 1.f);
                if (rays) {
                    float ax, ay, az;
                    zt::ray_dir(rp, gx, gy, ax, ay, az);
                    const float d = zt::ray_dev(v.x, v.y, v.z, ax, ay, az);
                    tdev = max(tdev, __float_as_uint(d == d ? d : INFINITY));  // NaN counts as unbounded
                }
            }
        }
        mls_sp[t] = v;
    }
    tdev = __reduce_max_sync(0xffffffffu, tdev);
    if ((tid & 31) == 0) warp_dev[tid >> 5] = tdev;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < MX * MY / 32; j++) tdev = max(tdev, warp_dev[j]);
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    const bool inside = x < cols && y < rows;
    const int cc = (threadIdx.y + hw) * TW + threadIdx.x + hw;
    const float4 c = mls_sp[cc];
    float wr2 = INFINITY;  // squared pixel radius of the warp's disk
    if (rays) {
        float rs2 = 0.f;
        if (inside && c.w != 0.f) {
            float ax, ay, az;
            zt::ray_dir(rp, x, y, ax, ay, az);
            const float an = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
            const float qn = sqrtf(fmaf(c.x, c.x, fmaf(c.y, c.y, c.z * c.z)));
            const float C = qn * rp.f / an;
            const float sd = sqrtf(r2c) + zt::ray_dev(c.x, c.y, c.z, ax, ay, az) + __uint_as_float(tdev) + 1e-5f * qn;
            rs2 = INFINITY;
            if (C > sd) {
                const float r = sd * an / (C - sd);
                rs2 = r * r;
            }
        }
        wr2 = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(rs2)));
    }
    if (!inside) return;
    const size_t o = (size_t)y * cols + x;
    const float px = src[3 * o], py = src[3 * o + 1], pz = src[3 * o + 2];
    const float2 npxy = make_float2(-px, -py);  // q - p as q + (-p): the same rounding
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool moved = false;
    if (c.w != 0.f) {
        // invalid and off-image neighbours are NaN and fail the distance test
        if constexpr (HW >= 1 && HW <= 7) {
            // half-width of window rows +-i, found once for both sweeps
            // (warp-uniform; 15 = row skipped)
            unsigned wpack = 0u;
#pragma unroll
            for (int ai = 0; ai <= HW; ai++) {
                const float rem = wr2 - (float)(ai * ai);
                const unsigned code =
                    rem < 0.f ? 15u : (rem < (float)(HW * HW) ? (unsigned)(int)sqrtf(rem) : (unsigned)HW);
                wpack |= code << (4 * ai);
            }
            auto visit = [&](auto&& fn) {
#pragma unroll 1
                for (int i = -HW; i <= HW; i++) {
                    const int w = (int)((wpack >> (4 * (i < 0 ? -i : i))) & 15u);
                    if (w == 15) continue;
                    for (int j = -w; j <= w; j++) {
                        const float4 q = mls_sp[cc + i * TW + j];
                        fn(__fadd2_rn(make_float2(q.x, q.y), npxy), q.z - pz);
                    }
                }
            };
            mls_point(inv_2s2, order, r2c, visit, ox, oy, oz, moved);
        } else {
            auto visit = [&](auto&& fn) {
                for (int i = -hw; i <= hw; i++) {
                    const float rem = wr2 - (float)(i * i);
                    if (rem < 0.f) continue;
                    const int w = rem < (float)(hw * hw) ? (int)sqrtf(rem) : hw;
                    for (int j = -w; j <= w; j++) {
                        const float4 q = mls_sp[cc + i * TW + j];
                        fn(__fadd2_rn(make_float2(q.x, q.y), npxy), q.z - pz);
                    }
                }
            };
            mls_point(inv_2s2, order, r2c, visit, ox, oy, oz, moved);
        }
    }
    dst[3 * o] = moved ? px + ox : px;
    dst[3 * o + 1] = moved ? py + oy : py;
    dst[3 * o + 2] = moved ? pz + oz : pz;
}

}  // namespace

size_t zim_mls_scratch_bytes(size_t n_points) { return zim_align256(n_points * 12); }

zim_status zim_mls_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, int window,
                          float sigma, int order, float max_radius, int iterations, float* out, float* tmp,
                          const zim_ray_model& rays, cudaStream_t st) {
    const float r2c = max_radius > 0.f ? max_radius * max_radius : 9.0f * sigma * sigma;
    const float inv_2s2 = 1.0f / (2.0f * sigma * sigma);
    const int ord = order < 0 ? 0 : (order > 2 ? 2 : order);
    const int n_iter = iterations < 1 ? 1 : iterations;
    dim3 blk(MX, MY), grd((cols + MX - 1) / MX, (rows + MY - 1) / MY);
    const size_t smem = mls_smem_bytes(window);
    const bool use_smem = smem <= 96 * 1024;
    auto kern = window == 7 ? mls_smem_kernel<7> : mls_smem_kernel<0>;
    if (use_smem) ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int use_rays = use_smem && rays.valid;
    const zt::RayParams rp = zt::ray_params(rays);
    // ping-pong so that the last pass lands in `out`
    const float* in = xyz;
    for (int it = 0; it < n_iter; it++) {
        float* dst = ((n_iter - 1 - it) % 2 == 0) ? out : tmp;
        if (dst == in) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "MLS in-place not supported");
        if (use_smem)
            kern<<<grd, blk, smem, st>>>(in, mask, rows, cols, window, inv_2s2, ord, r2c, use_rays, rp, dst);
        else
            mls_kernel<<<grd, blk, 0, st>>>(in, mask, rows, cols, window, inv_2s2, ord, r2c, dst);
        ctx->launches += 1;
        ZIM_LAUNCH_CHECK(ctx);
        in = dst;
    }
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_filter_mls(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                             int window, float sigma, int order, float max_radius, int iterations,
                                             float* out, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!xyz || !mask || !out || rows <= 0 || cols <= 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    if (window < 0 || window > 64 || !(sigma > 0)) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad MLS parameter");
    if (out == xyz) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "MLS in-place not supported");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    float* tmp = nullptr;
    zim_status s = zim_scratch_reserve(ctx, zim_mls_scratch_bytes((size_t)rows * cols) + 512);
    if (s) return s;
    zim_scratch_reset(ctx);
    if (iterations > 1) tmp = (float*)zim_scratch_take(ctx, (size_t)rows * cols * 12);
    // a cloud of the calibrated rectified size: its pixels' rays bound the window
    const zim_ray_model rays = rows == ctx->rect_h && cols == ctx->rect_w ? zim_rays_of(ctx, true, 0, 0)
                                                                          : zim_ray_model{};
    return zim_mls_launch(ctx, xyz, mask, rows, cols, window, sigma, order, max_radius, iterations, out, tmp, rays,
                          zim_stream(stream));
}
