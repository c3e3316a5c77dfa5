// diff.cu -- differentiable sub-pixel matching + reprojection: forward and
// hand-written adjoint w.r.t. the stereo calibration and the per-pixel phase.
//
// No counterpart in the reference (it has no gradients).  The forward follows
// its sub-pixel refinement and rectified-coordinate reprojection
// (PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:985-1000,
// :414-461) on rectified phase sampled with exact bilinear weights from the
// source phase through the undistort-rectify ray model of
// initUndistortRectifyMap (:329-337).  The match columns are inputs.
//
// Per rectified left pixel (j, i) with match column b:
//   phi_L = phase_L(map_L(j, i)),  phi_R,m = phase_R(map_R(b - 1 + m, i))
//   c_m = phi_R,m - phi_L;  delta = c1 (c0 - c2) / (2 (c0 - c1)(c1 - c2))
//   d = j - b - delta;  w = q32 d + q33;  P = (j + q03, i + q13, q23) / w
// Every parameter reaches P through the scalar w, so dP/dtheta = -P/w dw/dtheta:
// the kernel builds dw/dtheta (16 values) per point from the samples'
// position Jacobians and the phase slopes, then
//   dLoss/dtheta += -(g . P)/w * dw/dtheta   (g = upstream dLoss/dP)
//   J_r = -(n . P)/w * dw/dtheta             (plane distance, for J^T J).
// Reductions are FP64: per thread, per warp, per block in a fixed order, then
// a fixed-order sum of the block partials.
#include <cmath>
#include <cstring>
#include <vector>

#include "zim_internal.cuh"

namespace {

constexpr int DIFF_T = 256;   // threads per block
constexpr int DIFF_W = DIFF_T / 32;
constexpr int NP = ZIM_DIFF_NPARAMS;
constexpr int NJ = NP * (NP + 1) / 2;  // 136 upper-triangle entries of J^T J
constexpr int NACC = 2 + NP + NJ;       // loss, count, grad, jtj
constexpr int MAX_VIEWS = 4096;

struct DiffCam {
    float ir[9];  // rectified pixel -> camera ray
    float fx, fy, cx, cy, k1, k2, p1, p2, k3;
};

struct DiffDev {
    DiffCam cam[2];
    float q03, q13, q23, q32, q33;
    double q03d, q13d, q23d, q32d, q33d;  // the same in FP64, for w and the plane distance
    float dq32, dq33;  // d/d baseline
    int rw, rh, sw, sh;
    float zmin, zmax;
};

struct ViewDev {
    const int32_t* order[2];
    const float* res[2];
    const int32_t* best;
    double nd[3], pdd;  // plane
    float* xyz;
    uint8_t* mask;
    const float* gxyz;
    float* gphase[2];
};

// (a, b), a <= b, of upper-triangle entry e of J^T J in row-major order
__device__ __forceinline__ void jtj_pair(int e, int& a, int& b) {
    a = 0;
    while (e >= NP - a) {
        e -= NP - a;
        a++;
    }
    b = a + e;
}

// One phase sample of camera cam at rectified (col, row): position (u, v) in
// the source image, bilinear phase base + frac (phase = 2 pi base + frac), the
// phase slopes, and optionally d(u, v)/d(params of this camera): fx fy cx cy
// k1 k2 and, for the right camera, the three rotation components.
struct Sample {
    int base, x0, y0;
    float frac, a, b, gu, gv;
};

__device__ __forceinline__ bool take_sample(const DiffCam& c, float col, float row, const int32_t* __restrict__ ord,
                                            const float* __restrict__ res, int sw, int sh, Sample& s, float* ju,
                                            float* jv, bool rot) {
    const float X0 = fmaf(c.ir[0], col, fmaf(c.ir[1], row, c.ir[2]));
    const float X1 = fmaf(c.ir[3], col, fmaf(c.ir[4], row, c.ir[5]));
    const float X2 = fmaf(c.ir[6], col, fmaf(c.ir[7], row, c.ir[8]));
    const float x = X0 / X2, y = X1 / X2;
    const float r2 = fmaf(x, x, y * y);
    const float sd = fmaf(r2, fmaf(r2, fmaf(r2, c.k3, c.k2), c.k1), 1.0f);
    const float xd = fmaf(x, sd, fmaf(2.0f * c.p1, x * y, c.p2 * fmaf(2.0f * x, x, r2)));
    const float yd = fmaf(y, sd, fmaf(c.p1, fmaf(2.0f * y, y, r2), 2.0f * c.p2 * x * y));
    const float u = fmaf(c.fx, xd, c.cx), v = fmaf(c.fy, yd, c.cy);
    // all four taps inside the image (also rejects NaN)
    if (!(u >= 0.f && v >= 0.f && u < (float)(sw - 1) && v < (float)(sh - 1))) return false;
    const int x0 = (int)u, y0 = (int)v;
    if (x0 + 1 >= sw || y0 + 1 >= sh) return false;
    const size_t o = (size_t)y0 * sw + x0;
    const int k00 = __ldg(ord + o), k10 = __ldg(ord + o + 1), k01 = __ldg(ord + o + sw), k11 = __ldg(ord + o + sw + 1);
    if (k00 < 1 || k10 < 1 || k01 < 1 || k11 < 1) return false;
    const float r00 = __ldg(res + o), r10 = __ldg(res + o + 1), r01 = __ldg(res + o + sw), r11 = __ldg(res + o + sw + 1);
    // phases relative to tap 00, integer cycles subtracted exactly
    const float p10 = fmaf((float)(k10 - k00), ZIM_TWO_PI_F, r10 - r00);
    const float p01 = fmaf((float)(k01 - k00), ZIM_TWO_PI_F, r01 - r00);
    const float p11 = fmaf((float)(k11 - k00), ZIM_TWO_PI_F, r11 - r00);
    const float a = u - (float)x0, b = v - (float)y0;
    s.base = k00;
    s.frac = r00 + fmaf(a * (1.0f - b), p10, fmaf((1.0f - a) * b, p01, a * b * p11));
    s.gu = fmaf(1.0f - b, p10, b * (p11 - p01));
    s.gv = fmaf(1.0f - a, p01, a * (p11 - p10));
    s.x0 = x0;
    s.y0 = y0;
    s.a = a;
    s.b = b;
    if (ju) {
        const float r4 = r2 * r2;
        ju[0] = xd; ju[1] = 0.f; ju[2] = 1.f; ju[3] = 0.f; ju[4] = c.fx * x * r2; ju[5] = c.fx * x * r4;
        jv[0] = 0.f; jv[1] = yd; jv[2] = 0.f; jv[3] = 1.f; jv[4] = c.fy * y * r2; jv[5] = c.fy * y * r4;
        if (rot) {
            // ray X -> X + X x eps: d(x, y)/d eps_k for k = 0, 1, 2
            const float dx[3] = {x * y, -1.0f - x * x, y};
            const float dy[3] = {1.0f + y * y, -x * y, -x};
            const float s1 = fmaf(r2, fmaf(3.0f * c.k3, r2, 2.0f * c.k2), c.k1);  // d sd / d r2
            const float dxd_dx = sd + 2.0f * x * x * s1 + 2.0f * c.p1 * y + 6.0f * c.p2 * x;
            const float dxd_dy = 2.0f * x * y * s1 + 2.0f * c.p1 * x + 2.0f * c.p2 * y;
            const float dyd_dx = dxd_dy;
            const float dyd_dy = sd + 2.0f * y * y * s1 + 6.0f * c.p1 * y + 2.0f * c.p2 * x;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                ju[6 + k] = c.fx * fmaf(dxd_dx, dx[k], dxd_dy * dy[k]);
                jv[6 + k] = c.fy * fmaf(dyd_dx, dx[k], dyd_dy * dy[k]);
            }
        }
    }
    return true;
}

__global__ void diff_rectify_kernel(DiffDev P, int cam, const int32_t* __restrict__ ord, const float* __restrict__ res,
                                    int32_t* __restrict__ rbase, float* __restrict__ rres,
                                    int32_t* __restrict__ rorder) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= P.rw || i >= P.rh) return;
    Sample s;
    const size_t o = (size_t)i * P.rw + j;
    if (take_sample(P.cam[cam], (float)j, (float)i, ord, res, P.sw, P.sh, s, nullptr, nullptr, false)) {
        const int nx = s.a >= 0.5f ? s.x0 + 1 : s.x0, ny = s.b >= 0.5f ? s.y0 + 1 : s.y0;
        rbase[o] = s.base;
        rres[o] = s.frac;
        rorder[o] = __ldg(ord + (size_t)ny * P.sw + nx);
    } else {
        rbase[o] = 0;
        rres[o] = 0.f;
        rorder[o] = 0;
    }
}

__device__ __forceinline__ void scatter_phase(float* g, int sw, const Sample& s, float v) {
    if (!g || v == 0.f) return;
    const size_t o = (size_t)s.y0 * sw + s.x0;
    atomicAdd(g + o, v * (1.0f - s.a) * (1.0f - s.b));
    atomicAdd(g + o + 1, v * s.a * (1.0f - s.b));
    atomicAdd(g + o + sw, v * (1.0f - s.a) * s.b);
    atomicAdd(g + o + sw + 1, v * s.a * s.b);
}

template <bool BWD>
__global__ void __launch_bounds__(DIFF_T) diff_kernel(DiffDev P, const ViewDev* __restrict__ views, int n_views,
                                                       float loss_weight, double* __restrict__ part) {
    __shared__ float Js[DIFF_W][32][NP + 1];
    __shared__ double red[DIFF_W][NACC];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const size_t npx = (size_t)P.rw * P.rh, total = npx * (size_t)n_views;
    const size_t nwarps = (size_t)gridDim.x * DIFF_W;
    double loss = 0.0, cnt = 0.0;
    double g[NP];
    double jacc[(NJ + 31) / 32];
#pragma unroll
    for (int k = 0; k < NP; k++) g[k] = 0.0;
    int pa[(NJ + 31) / 32], pb[(NJ + 31) / 32];
#pragma unroll
    for (int q = 0; q < (NJ + 31) / 32; q++) {
        jacc[q] = 0.0;
        jtj_pair(min(lane + 32 * q, NJ - 1), pa[q], pb[q]);
    }

    // the loop bound depends on the warp only, so the lanes stay together for
    // the J^T J staging
    for (size_t base = ((size_t)blockIdx.x * DIFF_W + wib) * 32; base < total; base += nwarps * 32) {
        const size_t t = base + lane;
        float Jr[NP];
#pragma unroll
        for (int k = 0; k < NP; k++) Jr[k] = 0.f;
        if (t < total) {
            const int vi = (int)(t / npx);
            const size_t pix = t - (size_t)vi * npx;
            const ViewDev& V = views[vi];
            const int i = (int)(pix / P.rw), j = (int)(pix - (size_t)i * P.rw);
            const int b = V.best[pix];
            bool ok = b >= 1 && b + 1 < P.rw;
            Sample sL, sR[3];
            if (ok) ok = take_sample(P.cam[0], (float)j, (float)i, V.order[0], V.res[0], P.sw, P.sh, sL, nullptr,
                                     nullptr, false);
#pragma unroll
            for (int m = 0; m < 3; m++)
                if (ok) ok = take_sample(P.cam[1], (float)(b - 1 + m), (float)i, V.order[1], V.res[1], P.sw, P.sh,
                                         sR[m], nullptr, nullptr, false);
            float c[3] = {0.f, 0.f, 0.f};
            float delta = 0.f, dd[3] = {0.f, 0.f, 0.f};  // d delta / d c_m
            float X = 0.f, Y = 0.f, Z = 0.f, w = 0.f, d = 0.f;
            if (ok) {
#pragma unroll
                for (int m = 0; m < 3; m++) c[m] = fmaf((float)(sR[m].base - sL.base), ZIM_TWO_PI_F, sR[m].frac - sL.frac);
                const float num = c[1] * (c[0] - c[2]);
                const float den = 2.0f * (c[0] - c[1]) * (c[1] - c[2]);
                if (fabsf(den) > 1e-9f) {
                    delta = num / den;
                    const float inv = 1.0f / den;
                    dd[0] = (c[1] - delta * 2.0f * (c[1] - c[2])) * inv;
                    dd[1] = ((c[0] - c[2]) - delta * 2.0f * (c[0] - 2.0f * c[1] + c[2])) * inv;
                    dd[2] = (-c[1] + delta * 2.0f * (c[0] - c[1])) * inv;
                }
                d = (float)(j - b) - delta;
                ok = fabsf(d) >= 1e-5f;
            }
            // w from the exact integer part of the disparity and the FP32 sub-pixel
            // part: an FP32 disparity of ~1000 px would round at 6e-5 px
            double wd = 0.0;
            if (ok) {
                wd = fma(P.q32d, (double)(j - b) - (double)delta, P.q33d);
                w = (float)wd;
                if (fabsf(w) < 1e-2f * (fabsf(P.q32 * d) + fabsf(P.q33))) {
                    // near-zero disparity: the triangulation divide in FP64
                    X = (float)(((double)j + P.q03d) / wd);
                    Y = (float)(((double)i + P.q13d) / wd);
                    Z = (float)(P.q23d / wd);
                } else {
                    const float iw = 1.0f / w;
                    X = ((float)j + P.q03) * iw;
                    Y = ((float)i + P.q13) * iw;
                    Z = P.q23 * iw;
                }
                ok = Z > P.zmin && Z < P.zmax && isfinite(X) && isfinite(Y);
            }
            if (!BWD) {
                if (V.xyz) {
                    V.xyz[3 * pix] = ok ? X : 0.f;
                    V.xyz[3 * pix + 1] = ok ? Y : 0.f;
                    V.xyz[3 * pix + 2] = ok ? Z : 0.f;
                }
                if (V.mask) V.mask[pix] = ok ? 1 : 0;
            }
            if (ok) {
                // plane distance r = n . P + d = N / w, N = n . (j + q03, i + q13, q23) + d w
                // in FP64: the terms are ~1e3 times r, FP32 would lose three digits
                const double Nd = fma(V.nd[0], (double)j + P.q03d,
                                      fma(V.nd[1], (double)i + P.q13d, fma(V.nd[2], P.q23d, V.pdd * wd)));
                const float iw = 1.0f / w;
                const float r = (float)Nd * iw;
                loss += (double)r * (double)r;
                cnt += 1.0;
                if (BWD) {
                    // dLoss/dw = -(g . P)/w with g = lw 2 r n + grad_xyz, and n . P = r - d
                    const float nP = r - (float)V.pdd;
                    float gP = loss_weight * 2.0f * r * nP;
                    if (V.gxyz)
                        gP += fmaf(V.gxyz[3 * pix], X, fmaf(V.gxyz[3 * pix + 1], Y, V.gxyz[3 * pix + 2] * Z));
                    const float s_up = -gP * iw;
                    const float s_r = -nP * iw;  // dr/dw
                    // dw/dphi: d = j - b - delta, w = q32 d + q33
                    const float wR[3] = {-P.q32 * dd[0], -P.q32 * dd[1], -P.q32 * dd[2]};
                    const float wL = -(wR[0] + wR[1] + wR[2]);
                    float Jw[NP];
#pragma unroll
                    for (int k = 0; k < NP; k++) Jw[k] = 0.f;
                    Jw[12] = fmaf(d, P.dq32, P.dq33);
                    float ju[9], jv[9];
                    take_sample(P.cam[0], (float)j, (float)i, V.order[0], V.res[0], P.sw, P.sh, sL, ju, jv, false);
#pragma unroll
                    for (int k = 0; k < 6; k++) Jw[k] = wL * fmaf(sL.gu, ju[k], sL.gv * jv[k]);
                    scatter_phase(V.gphase[0], P.sw, sL, s_up * wL);
#pragma unroll
                    for (int m = 0; m < 3; m++) {
                        take_sample(P.cam[1], (float)(b - 1 + m), (float)i, V.order[1], V.res[1], P.sw, P.sh, sR[m], ju,
                                    jv, true);
#pragma unroll
                        for (int k = 0; k < 6; k++) Jw[6 + k] = fmaf(wR[m], fmaf(sR[m].gu, ju[k], sR[m].gv * jv[k]), Jw[6 + k]);
#pragma unroll
                        for (int k = 0; k < 3; k++)
                            Jw[13 + k] = fmaf(wR[m], fmaf(sR[m].gu, ju[6 + k], sR[m].gv * jv[6 + k]), Jw[13 + k]);
                        scatter_phase(V.gphase[1], P.sw, sR[m], s_up * wR[m]);
                    }
#pragma unroll
                    for (int k = 0; k < NP; k++) {
                        g[k] += (double)(s_up * Jw[k]);
                        Jr[k] = s_r * Jw[k];
                    }
                }
            }
        }
        if (BWD) {
#pragma unroll
            for (int k = 0; k < NP; k++) Js[wib][lane][k] = Jr[k];
            __syncwarp();
#pragma unroll
            for (int q = 0; q < (NJ + 31) / 32; q++) {
                const int e = lane + 32 * q;
                if (e < NJ) {
                    float acc = 0.f;
                    for (int rr = 0; rr < 32; rr++) acc = fmaf(Js[wib][rr][pa[q]], Js[wib][rr][pb[q]], acc);
                    jacc[q] += (double)acc;
                }
            }
            __syncwarp();
        }
    }
    // warp sums (fixed shuffle tree), then per-warp rows summed in warp order
    for (int off = 16; off; off >>= 1) {
        loss += __shfl_xor_sync(0xffffffffu, loss, off);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    if (BWD) {
#pragma unroll
        for (int k = 0; k < NP; k++)
            for (int off = 16; off; off >>= 1) g[k] += __shfl_xor_sync(0xffffffffu, g[k], off);
    }
    if (lane == 0) {
        red[wib][0] = loss;
        red[wib][1] = cnt;
#pragma unroll
        for (int k = 0; k < NP; k++) red[wib][2 + k] = BWD ? g[k] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < (NJ + 31) / 32; q++) {
        const int e = lane + 32 * q;
        if (e < NJ) red[wib][2 + NP + e] = BWD ? jacc[q] : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NACC; e += DIFF_T) {
        double s = 0.0;
        for (int ww = 0; ww < DIFF_W; ww++) s += red[ww][e];
        part[(size_t)blockIdx.x * NACC + e] = s;
    }
}

// Fixed-order sum of the block partials: one thread per accumulator.
__global__ void diff_total_kernel(const double* __restrict__ part, int nblk, double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= NACC) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += part[(size_t)b * NACC + e];
    out[e] = s;
}

// Rotation matrix of a rotation vector (Rodrigues' formula), row-major.
void rodrigues(const double v[3], double R[9]) {
    const double th = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double k[3] = {0, 0, 0}, c = 1.0, s = 0.0, cc = 0.0;
    if (th > 0) {
        for (int a = 0; a < 3; a++) k[a] = v[a] / th;
        c = std::cos(th);
        s = std::sin(th);
        cc = 1.0 - c;
    }
    R[0] = c + cc * k[0] * k[0];        R[1] = cc * k[0] * k[1] - s * k[2]; R[2] = cc * k[0] * k[2] + s * k[1];
    R[3] = cc * k[1] * k[0] + s * k[2]; R[4] = c + cc * k[1] * k[1];        R[5] = cc * k[1] * k[2] - s * k[0];
    R[6] = cc * k[2] * k[0] - s * k[1]; R[7] = cc * k[2] * k[1] + s * k[0]; R[8] = c + cc * k[2] * k[2];
}

zim_status make_dev(zim_ctx* ctx, const zim_diff_params* p, double zmin, double zmax, DiffDev& D) {
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    const double* t = ctx->calib.t;
    const double B0 = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    if (!(p->baseline > 0) || !(B0 > 0)) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "baseline must be > 0");
    for (int c = 0; c < 2; c++) {
        DiffCam& C = D.cam[c];
        double ir[9];
        if (c == 0) {
            std::memcpy(ir, ctx->ir[0], sizeof ir);
        } else {
            // (P2' R2 E)^-1 = E^T (P2' R2)^-1
            double E[9];
            rodrigues(p->rot, E);
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++) {
                    double s = 0;
                    for (int m = 0; m < 3; m++) s += E[m * 3 + r] * ctx->ir[1][m * 3 + q];
                    ir[r * 3 + q] = s;
                }
        }
        for (int a = 0; a < 9; a++) C.ir[a] = (float)ir[a];
        C.fx = (float)p->cam[c][0]; C.fy = (float)p->cam[c][1];
        C.cx = (float)p->cam[c][2]; C.cy = (float)p->cam[c][3];
        C.k1 = (float)p->cam[c][4]; C.k2 = (float)p->cam[c][5];
        const double* Dc = ctx->calib.dist_coeffs[c];
        C.p1 = (float)Dc[2]; C.p2 = (float)Dc[3]; C.k3 = (float)Dc[4];
    }
    const double* Q = ctx->Q;
    const double Tx0 = -1.0 / Q[14], dcx = Q[15] * Tx0;
    const double Tx = Tx0 * p->baseline / B0, dTx = Tx0 / B0;
    D.q03d = Q[3]; D.q13d = Q[7]; D.q23d = Q[11];
    D.q32d = -1.0 / Tx;
    D.q33d = dcx / Tx;
    D.q03 = (float)Q[3]; D.q13 = (float)Q[7]; D.q23 = (float)Q[11];
    D.q32 = (float)(-1.0 / Tx);
    D.q33 = (float)(dcx / Tx);
    D.dq32 = (float)(dTx / (Tx * Tx));
    D.dq33 = (float)(-dcx * dTx / (Tx * Tx));
    D.rw = ctx->rect_w; D.rh = ctx->rect_h; D.sw = ctx->src_w; D.sh = ctx->src_h;
    D.zmin = (float)zmin; D.zmax = (float)zmax;
    return ZIM_OK;
}

zim_status run(zim_ctx* ctx, const zim_diff_params* params, const zim_diff_view* views, int n_views, int rows,
               int cols, double zmin, double zmax, bool bwd, double loss_weight, zim_diff_result* out, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!params || !views || !out || n_views < 1 || n_views > MAX_VIEWS)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument (n_views must be in [1, %d])", MAX_VIEWS);
    DiffDev D;
    zim_status s = make_dev(ctx, params, zmin, zmax, D);
    if (s) return s;
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "phase size %dx%d differs from the calibration's %dx%d", cols, rows,
                        ctx->src_w, ctx->src_h);
    std::vector<ViewDev> hv((size_t)n_views);
    for (int v = 0; v < n_views; v++) {
        const zim_diff_view& V = views[v];
        if (!V.order[0] || !V.order[1] || !V.residual[0] || !V.residual[1] || !V.best_col)
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "view %d: missing phase or match columns", v);
        ViewDev& H = hv[(size_t)v];
        for (int c = 0; c < 2; c++) {
            H.order[c] = V.order[c];
            H.res[c] = V.residual[c];
            H.gphase[c] = bwd ? V.grad_phase[c] : nullptr;
        }
        H.best = V.best_col;
        for (int a = 0; a < 3; a++) H.nd[a] = V.plane[a];
        H.pdd = V.plane[3];
        H.xyz = bwd ? nullptr : V.xyz;
        H.mask = bwd ? nullptr : V.mask;
        H.gxyz = bwd ? V.grad_xyz : nullptr;
    }
    const int nblk = 4 * (ctx->sm_count > 0 ? ctx->sm_count : 152);
    zim_scratch_reset(ctx);
    s = zim_scratch_reserve(ctx, zim_align256(hv.size() * sizeof(ViewDev)) + zim_align256((size_t)nblk * NACC * 8) +
                                     zim_align256(NACC * 8) + 4096);
    if (s) return s;
    ViewDev* dv = (ViewDev*)zim_scratch_take(ctx, hv.size() * sizeof(ViewDev));
    double* part = (double*)zim_scratch_take(ctx, (size_t)nblk * NACC * 8);
    double* tot = (double*)zim_scratch_take(ctx, NACC * 8);
    cudaStream_t st = zim_stream(stream);
    static_assert(NACC * 8 <= 4096, "totals fit the pinned staging");
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(dv, hv.data(), hv.size() * sizeof(ViewDev), cudaMemcpyHostToDevice, st));
    if (bwd)
        diff_kernel<true><<<nblk, DIFF_T, 0, st>>>(D, dv, n_views, (float)loss_weight, part);
    else
        diff_kernel<false><<<nblk, DIFF_T, 0, st>>>(D, dv, n_views, (float)loss_weight, part);
    diff_total_kernel<<<1, 160, 0, st>>>(part, nblk, tot);
    ctx->launches += 2;
    ZIM_LAUNCH_CHECK(ctx);
    double* h = (double*)ctx->h_pinned;
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(h, tot, NACC * 8, cudaMemcpyDeviceToHost, st));
    ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    std::memset(out, 0, sizeof *out);
    out->loss = h[0];
    out->n_points = h[1];
    if (bwd) {
        for (int k = 0; k < NP; k++) out->grad[k] = h[2 + k];
        int e = 0;
        for (int a = 0; a < NP; a++)
            for (int b = a; b < NP; b++, e++) out->jtj[a * NP + b] = out->jtj[b * NP + a] = h[2 + NP + e];
    }
    return ZIM_OK;
}

}  // namespace

extern "C" ZIM_API zim_status zim_diff_params_nominal(const zim_ctx* ctx, zim_diff_params* out) {
    if (!ctx || !out) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return ZIM_ERR_NOT_CALIBRATED;
    for (int c = 0; c < 2; c++) {
        const double* K = ctx->calib.camera_matrix[c];
        const double* D = ctx->calib.dist_coeffs[c];
        out->cam[c][0] = K[0]; out->cam[c][1] = K[4]; out->cam[c][2] = K[2]; out->cam[c][3] = K[5];
        out->cam[c][4] = D[0]; out->cam[c][5] = D[1];
    }
    const double* t = ctx->calib.t;
    out->baseline = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    out->rot[0] = out->rot[1] = out->rot[2] = 0.0;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_diff_rectify(zim_ctx* ctx, const zim_diff_params* params, int cam,
                                               const int32_t* order, const float* residual, int rows, int cols,
                                               int32_t* rect_base, float* rect_res, int32_t* rect_order,
                                               void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!params || (cam != 0 && cam != 1) || !order || !residual || !rect_base || !rect_res || !rect_order)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    DiffDev D;
    zim_status s = make_dev(ctx, params, 0.0, 0.0, D);
    if (s) return s;
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "phase size %dx%d differs from the calibration's %dx%d", cols, rows,
                        ctx->src_w, ctx->src_h);
    dim3 grd((D.rw + 255) / 256, D.rh);
    diff_rectify_kernel<<<grd, 256, 0, zim_stream(stream)>>>(D, cam, order, residual, rect_base, rect_res,
                                                              rect_order);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_diff_forward(zim_ctx* ctx, const zim_diff_params* params,
                                               const zim_diff_view* views, int n_views, int rows, int cols,
                                               double z_min, double z_max, zim_diff_result* out, void* stream) {
    return run(ctx, params, views, n_views, rows, cols, z_min, z_max, false, 0.0, out, stream);
}

extern "C" ZIM_API zim_status zim_diff_backward(zim_ctx* ctx, const zim_diff_params* params,
                                                const zim_diff_view* views, int n_views, int rows, int cols,
                                                double z_min, double z_max, double loss_weight,
                                                zim_diff_result* out, void* stream) {
    return run(ctx, params, views, n_views, rows, cols, z_min, z_max, true, loss_weight, out, stream);
}
