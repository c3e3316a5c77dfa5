// zim_tiles.cuh -- per-tile / per-pixel device code shared by the plain
// per-pair kernels and the persistent batch kernels, so both paths run the
// same arithmetic (bit-identical results).  Every multiply-add that matters
// is an explicit fmaf, so the results do not depend on a translation unit's
// contraction flags.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseShiftDecoder_V2.cpp:18-182
// (pre-blur + decode body), JSLAB_PhaseEpipolarReconstructor_V2.cpp:368-395
// (setData remap), :933-1006 (stereoMatch), :405-461 (median + reprojection),
// :79-195 (pixel Gaussian, radius outlier filter).
#pragma once

#include <cmath>

#include "zim_internal.cuh"

namespace zt {

// ---------------------------------------------------------------- decode ----

constexpr int DX = 32, DY = 8;  // decode tile (threads of a block, as DX x DY)
constexpr int DHX = DX + 2, DHY = DY + 2;

struct DecodeParams {
    int rows, cols, enc, n_ps;
    int shift[4];
    int fbase[4];      // first frame of each phase-shift frequency
    float sinv[64];    // sin(2 pi k / N) per frame (reference LUT order)
    float cosv[64];
    float w2d[9];      // pre-blur weights k_a * k_b
    float thr;
    int avg3;
    // heterodyne (integer fringe counts)
    int f0, f1, f2, f12, f23, f1_gt_f2;
    float f0_f12, f1_f23, f2_f23, inv_f12, inv_f23, inv_f1, inv_f2;
    // hierarchical
    int iratio[4];
    float fratio[4];
    // Gray code
    int gray_bits, gray_base, complementary;
    // HDR least squares (JSLAB_HDRPhaseFit.h:10-61)
    int hdr;
    float hdr_sat, hdr_min_amp;
};

inline void decode_params(const zim_decode_config* c, int rows, int cols, DecodeParams& p) {
    p = DecodeParams{};
    p.rows = rows;
    p.cols = cols;
    p.enc = c->encoding;
    p.n_ps = c->encoding == ZIM_ENC_HETERODYNE3 ? 3 : (c->encoding == ZIM_ENC_HIERARCHICAL ? c->n_freq : 1);
    int f = 0;
    for (int i = 0; i < p.n_ps; i++) {
        p.shift[i] = c->shift_num[i];
        p.fbase[i] = f;
        for (int k = 0; k < c->shift_num[i]; k++, f++) {
            // sin(2.0 * PI * k / inum) in double, as the reference builds its LUT
            p.sinv[f] = (float)std::sin(2.0 * 3.14159265358979323846 * k / c->shift_num[i]);
            p.cosv[f] = (float)std::cos(2.0 * 3.14159265358979323846 * k / c->shift_num[i]);
        }
    }
    double kb[3];
    if (c->preblur_sigma <= 0) { kb[0] = 0.25; kb[1] = 0.5; kb[2] = 0.25; }
    else {
        double t = std::exp(-0.5 / (c->preblur_sigma * c->preblur_sigma));
        double mul = 1.0 / (2.0 * t + 1.0);
        kb[0] = t * mul; kb[1] = mul; kb[2] = t * mul;
    }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) p.w2d[a * 3 + b] = (float)(kb[a] * kb[b]);
    p.thr = (float)c->modulation_threshold;
    p.avg3 = c->avg_three_phase ? 1 : 0;
    if (c->encoding == ZIM_ENC_HETERODYNE3) {
        p.f0 = (int)c->freq[0]; p.f1 = (int)c->freq[1]; p.f2 = (int)c->freq[2];
        p.f12 = std::abs(p.f0 - p.f1); p.f23 = std::abs(p.f1 - p.f2);
        p.f1_gt_f2 = c->freq[1] > c->freq[2];
        p.f0_f12 = (float)((double)p.f0 / p.f12);
        p.f1_f23 = (float)((double)p.f1 / p.f23);
        p.f2_f23 = (float)((double)p.f2 / p.f23);
        p.inv_f12 = (float)(1.0 / p.f12);
        p.inv_f23 = (float)(1.0 / p.f23);
        p.inv_f1 = (float)(1.0 / p.f1);
        p.inv_f2 = (float)(1.0 / p.f2);
    } else if (c->encoding == ZIM_ENC_HIERARCHICAL) {
        for (int i = 1; i < c->n_freq; i++) {
            p.iratio[i] = (int)(c->freq[i] / c->freq[i - 1]);
            p.fratio[i] = (float)p.iratio[i];
        }
    } else {
        p.gray_bits = c->gray_bits;
        p.gray_base = c->shift_num[0];
        p.complementary = c->encoding == ZIM_ENC_GRAYCODE_COMPLEMENTARY;
    }
    p.hdr = c->enable_hdr ? 1 : 0;
    p.hdr_sat = (float)c->hdr_saturation_gray;
    p.hdr_min_amp = (float)c->hdr_min_amplitude;
}

// HDR fit of one frequency at one pixel (JSLAB_HDRPhaseFit.h:10-61 and
// JSLAB_PhaseShiftDecoder_V2.cpp:73-90): raw samples with 0 <= I < saturation
// enter an equal-variance least-squares fit of I = A + C cos d - S sin d
// (solved here from the 3x3 normal equations, the reference's cached
// pseudo-inverse of the same subset); fewer than three samples, amplitude
// hypot(C, S) <= min_amp or A <= 1e-3 reject the pixel.  Returns the sums the
// phase-shift path would have formed: sin_sum = S N/2, cos_sum = C N/2,
// sum = A N.
template <typename T>
__device__ __forceinline__ bool hdr_fit(const T* __restrict__ f0, size_t npx, int N, const float* sv, const float* cv,
                                        float sat, float min_amp, float& sin_sum, float& cos_sum, float& sum) {
    float m00 = 0.f, m01 = 0.f, m02 = 0.f, m11 = 0.f, m12 = 0.f, m22 = 0.f, r0 = 0.f, r1 = 0.f, r2 = 0.f;
    int n = 0;
    for (int k = 0; k < N; k++) {
        const float v = (float)__ldg(f0 + (size_t)k * npx);
        if (!(v >= 0.f && v < sat)) continue;
        const float c = cv[k], s = -sv[k];
        m00 += 1.f; m01 += c; m02 += s;
        m11 = fmaf(c, c, m11); m12 = fmaf(c, s, m12); m22 = fmaf(s, s, m22);
        r0 += v; r1 = fmaf(c, v, r1); r2 = fmaf(s, v, r2);
        n++;
    }
    if (n < 3) return false;
    // symmetric 3x3 inverse by cofactors
    const float c00 = fmaf(m11, m22, -m12 * m12), c01 = fmaf(m02, m12, -m01 * m22), c02 = fmaf(m01, m12, -m02 * m11);
    const float det = fmaf(m00, c00, fmaf(m01, c01, m02 * c02));
    if (!(fabsf(det) > 1e-6f * m00 * m00 * m00)) return false;
    const float c11 = fmaf(m00, m22, -m02 * m02), c12 = fmaf(m01, m02, -m00 * m12), c22 = fmaf(m00, m11, -m01 * m01);
    const float id = 1.0f / det;
    const float A = fmaf(c00, r0, fmaf(c01, r1, c02 * r2)) * id;
    const float C = fmaf(c01, r0, fmaf(c11, r1, c12 * r2)) * id;
    const float S = fmaf(c02, r0, fmaf(c12, r1, c22 * r2)) * id;
    if (!(hypotf(C, S) > min_amp) || !(A > 1e-3f)) return false;
    sin_sum = S * (float)N * 0.5f;
    cos_sum = C * (float)N * 0.5f;
    sum = A * (float)N;
    return true;
}

// floor(a / b) for b > 0 and |a / b| < 2^21, from the float reciprocal
// inv_b = 1 / b: the float quotient is within one of the true one, and one
// remainder check corrects it (an integer division costs ~40 instructions).
__device__ __forceinline__ int floor_div(int a, int b, float inv_b) {
    int q = __float2int_rd((float)a * inv_b);
    const int r = a - q * b;
    q += (r >= b) - (r < 0);
    return q;
}

// Shared memory of one decode tile: the raw per-pixel sums of the tile + halo,
// the phase-shift pair (S, C) as one float2 so that both are staged, loaded
// and blurred by paired FP32 instructions (__ffma2_rn: each lane rounded as
// the scalar fmaf, so the sums are those of the scalar sequence).
constexpr int DEC_MAX_PS = 4;  // phase-shift frequencies staged together
struct DecodeSmem {
    float2 SC[DEC_MAX_PS][DHY][DHX + 1];
    float M[DEC_MAX_PS][DHY][DHX + 1];
};

// sc += (-sin_k, cos_k) v: the S and C sums of one sample in one paired FMA
__device__ __forceinline__ float2 sc_add(float2 sc, float sn, float cs, float v) {
    return __ffma2_rn(make_float2(-sn, cs), make_float2(v, v), sc);
}

// Four-quadrant arctangent of the wrapped phase.  The octant ratio
// t = min(|y|, |x|) / max(|y|, |x|) in [0, 1] gives atan(t) = t P(t^2) with P of
// degree 7, fitted for this kernel by iteratively reweighted least squares on
// Chebyshev nodes (absolute error 3.7e-8 in exact arithmetic, 1.4e-7 evaluated
// by FP32 Horner FMAs); the octant and quadrant follow by symmetry, with atan2's
// signed zeros (the sign bits of y and x) and 0 for (0, 0).  __fdividef is
// exact to 2 ulp for the divisor range of these sums (far below 2^126).
__device__ __forceinline__ float phase_atan2(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float hi = fmaxf(ax, ay), lo = fminf(ax, ay);
    const float t = hi > 0.f ? __fdividef(lo, hi) : 0.f;
    const float s = t * t;
    float p = -0.004054566845297813f;
    p = fmaf(p, s, 0.021862957626581192f);
    p = fmaf(p, s, -0.0559123270213604f);
    p = fmaf(p, s, 0.0964219719171524f);
    p = fmaf(p, s, -0.1390862911939621f);
    p = fmaf(p, s, 0.19946566224098206f);
    p = fmaf(p, s, -0.33329859375953674f);
    p = fmaf(p, s, 0.9999993443489075f);
    float r = t * p;
    if (ay > ax) r = 0.5f * ZIM_PI_F - r;
    if (signbit(x)) r = ZIM_PI_F - r;
    return copysignf(r, y);
}

// Raw sums of one halo pixel over the N frames of one frequency, four frames'
// loads in flight at a time (the same accumulation order as one at a time).
template <typename T>
__device__ __forceinline__ void frame_sums(const T* __restrict__ src, size_t npx, int N, const float* sv,
                                           const float* cv, float2& sc, float& m) {
    sc = make_float2(0.f, 0.f);
    m = 0.f;
    int k = 0;
    for (; k + 4 <= N; k += 4) {
        const float v0 = (float)__ldg(src + (size_t)k * npx), v1 = (float)__ldg(src + (size_t)(k + 1) * npx);
        const float v2 = (float)__ldg(src + (size_t)(k + 2) * npx), v3 = (float)__ldg(src + (size_t)(k + 3) * npx);
        sc = sc_add(sc, sv[k], cv[k], v0); m += v0;
        sc = sc_add(sc, sv[k + 1], cv[k + 1], v1); m += v1;
        sc = sc_add(sc, sv[k + 2], cv[k + 2], v2); m += v2;
        sc = sc_add(sc, sv[k + 3], cv[k + 3], v3); m += v3;
    }
    for (; k < N; k++) {
        float v = (float)__ldg(src + (size_t)k * npx);
        sc = sc_add(sc, sv[k], cv[k], v);
        m += v;
    }
}

// Raw per-pixel sums of the tile (bx, by) and its 1-pixel halo (clamped to the
// image) into shared memory, every frequency in one pass: all of a pixel's
// frame loads are issued before the tile waits.  Ends with a block barrier.
template <typename T>
__device__ __forceinline__ void decode_stage_sums(const T* __restrict__ frames, const DecodeParams& p, int bx, int by,
                                                  int tid, DecodeSmem& sm) {
    const int gx0 = bx * DX - 1, gy0 = by * DY - 1;
    const size_t npx = (size_t)p.rows * p.cols;
    for (int h = tid; h < DHX * DHY; h += DX * DY) {
        const int hy = h / DHX, hx = h - hy * DHX;
        const int gy = min(max(gy0 + hy, 0), p.rows - 1), gx = min(max(gx0 + hx, 0), p.cols - 1);
        const size_t pix = (size_t)gy * p.cols + gx;
#pragma unroll
        for (int i = 0; i < DEC_MAX_PS; i++) {
            if (i >= p.n_ps) break;
            float2 sc;
            float m;
            frame_sums(frames + (size_t)p.fbase[i] * npx + pix, npx, p.shift[i], p.sinv + p.fbase[i],
                       p.cosv + p.fbase[i], sc, m);
            sm.SC[i][hy][hx] = sc;
            sm.M[i][hy][hx] = m;
        }
    }
    __syncthreads();
}

// The validity test on the normalised modulation nm = (2 |S, C| / N) / (M / N)
// (0 when M <= 1e-3 N): nm < thr fails the pixel.  For M > 0 that is
// 4 (S^2 + C^2) < (thr M)^2 with thr > 0, which needs neither the square root
// nor the division; they are computed only where nm is written out
// (want_value: frequency 0 with a modulation map).  The two forms decide
// differently only where nm lies within float rounding of thr.
__device__ __forceinline__ bool modulation_ok(float S, float C, float M, int N, float thr, bool want_value,
                                              float& value) {
    const float q = fmaf(S, S, C * C);
    const bool has_m = M > 1e-3f * (float)N;
    if (want_value) value = has_m ? 2.0f * sqrtf(q) / M : 0.f;
    if (!(thr > 0.f)) return true;
    const float tm = thr * M;
    return has_m && !(4.0f * q < tm * tm);
}

// Decodes tile (bx, by) of DX x DY pixels with the DX * DY threads of a block
// (tid = ty * DX + tx).  The pre-blur is linear, so the blurred sums
// S = -sum sin_k I_k, C = sum cos_k I_k, sum I_k are the 3x3 blur of the raw
// per-pixel sums, staged over the tile's 1-pixel halo in shared memory (by
// decode_stage_sums or the caller, before this is called; not with HDR).
// Ends with every thread past its last shared read, so the caller may start
// the next tile at once.  NPS / NS: the frequency count and the frames per
// frequency when known at compile time (0: taken from p); the arithmetic is
// the same either way.
template <typename T, int NPS = 0, int NS = 0>
__device__ __forceinline__ void decode_finish(const T* __restrict__ frames, const DecodeParams& p, int bx, int by,
                                              int tid, DecodeSmem& sm, int32_t* __restrict__ order,
                                              float* __restrict__ residual, float* __restrict__ mod_out,
                                              uint8_t* __restrict__ valid_out) {
    const int tx = tid % DX, ty = tid / DX;
    const int x = bx * DX + tx, y = by * DY + ty;
    const size_t npx = (size_t)p.rows * p.cols;

    float wrap0 = 0.f, wrap1 = 0.f, wrap2 = 0.f, wrap3 = 0.f;  // named, so they stay in registers
    float mod0 = 0.f;
    bool ok = true;
    const bool inside = x < p.cols && y < p.rows;
    const int n_ps = NPS ? NPS : p.n_ps;
#pragma unroll
    for (int i = 0; i < (NPS ? NPS : DEC_MAX_PS); i++) {
        if (i >= n_ps) break;
        const int N = NS ? NS : p.shift[i];
        const T* fb = frames + (size_t)p.fbase[i] * npx;
        const float* sv = p.sinv + p.fbase[i];
        const float* cv = p.cosv + p.fbase[i];
        if (p.hdr) {
            // raw samples, no pre-blur: saturation is classified before any blur
            float S = 0.f, C = 0.f, M = 0.f;
            if (ok && inside && !hdr_fit(fb + (size_t)y * p.cols + x, npx, N, sv, cv, p.hdr_sat, p.hdr_min_amp, S, C, M))
                ok = false;
            if (ok) {
                const float wr = phase_atan2(S, C);
                if (i == 0) wrap0 = wr;
                else if (i == 1) wrap1 = wr;
                else if (i == 2) wrap2 = wr;
                else wrap3 = wr;
                if (!modulation_ok(S, C, M, N, p.thr, i == 0 && mod_out, mod0)) ok = false;
            }
            continue;
        }
        float2 SC = make_float2(0.f, 0.f);
        float M = 0.f;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                float w = p.w2d[a * 3 + b];
                SC = __ffma2_rn(make_float2(w, w), sm.SC[i][ty + a][tx + b], SC);
                M = fmaf(w, sm.M[i][ty + a][tx + b], M);
            }
        const float S = SC.x, C = SC.y;
        if (ok) {
            const float wr = phase_atan2(S, C);
            if (i == 0) wrap0 = wr;
            else if (i == 1) wrap1 = wr;
            else if (i == 2) wrap2 = wr;
            else wrap3 = wr;
            if (!modulation_ok(S, C, M, N, p.thr, i == 0 && mod_out, mod0)) ok = false;
        }
    }
    // every thread is past its last shared read before the block's next tile
    if (!p.hdr) __syncthreads();
    if (x >= p.cols || y >= p.rows) return;
    const size_t pix = (size_t)y * p.cols + x;
    if (mod_out) mod_out[pix] = mod0;
    int k = 0;
    float r = 0.f;
    if (ok) {
        if (p.enc == ZIM_ENC_HETERODYNE3) {
            const float w0 = wrap0, w1 = wrap1, w2 = wrap2;
            float p12 = w0 > w1 ? w0 - w1 : w0 - w1 + ZIM_TWO_PI_F;
            float p23;
            if (p.f1_gt_f2) p23 = w1 > w2 ? w1 - w2 : w1 - w2 + ZIM_TWO_PI_F;
            else p23 = w2 > w1 ? w2 - w1 : w2 - w1 + ZIM_TWO_PI_F;
            float p123 = p12 > p23 ? p12 - p23 : p12 - p23 + ZIM_TWO_PI_F;
            // uphase12 = p12 + 2 pi m12;  k = round(m12 f0 / f12 + (p12 f0 / f12 - w0) / 2 pi)
            int m12 = (int)roundf(fmaf(p123, (float)p.f12, -p12) * ZIM_INV_TWO_PI_F);
            int num = m12 * p.f0;
            int q = floor_div(num, p.f12, p.inv_f12);
            int rem = num - q * p.f12;
            k = q + (int)roundf(fmaf((float)rem, p.inv_f12, fmaf(p12, p.f0_f12, -w0) * ZIM_INV_TWO_PI_F));
            r = w0;
            if (p.avg3) {
                int m23 = (int)roundf(fmaf(p123, (float)p.f23, -p23) * ZIM_INV_TWO_PI_F);
                int n2 = m23 * p.f1, q2 = floor_div(n2, p.f23, p.inv_f23), r2i = n2 - q2 * p.f23;
                int k2 = q2 + (int)roundf(fmaf((float)r2i, p.inv_f23, fmaf(p23, p.f1_f23, -w1) * ZIM_INV_TWO_PI_F));
                int n3 = m23 * p.f2, q3 = floor_div(n3, p.f23, p.inv_f23), r3i = n3 - q3 * p.f23;
                int k3 = q3 + (int)roundf(fmaf((float)r3i, p.inv_f23, fmaf(p23, p.f2_f23, -w2) * ZIM_INV_TWO_PI_F));
                // (uphase2 f0 / f1 - 2 pi k) = (w1 f0 + 2 pi (k2 f0 - k f1)) / f1, same for 3
                float r2 = fmaf((float)(k2 * p.f0 - k * p.f1), ZIM_TWO_PI_F, w1 * (float)p.f0) * p.inv_f1;
                float r3 = fmaf((float)(k3 * p.f0 - k * p.f2), ZIM_TWO_PI_F, w2 * (float)p.f0) * p.inv_f2;
                r = (w0 + r2 + r3) * (1.0f / 3.0f);
            }
        } else if (p.enc == ZIM_ENC_HIERARCHICAL) {
            const float wr[4] = {wrap0, wrap1, wrap2, wrap3};
#pragma unroll
            for (int i = 1; i < 4; i++) {
                if (i < n_ps) {
                    float a = fmaf(p.fratio[i], wr[i - 1] + ZIM_PI_F, -(wr[i] + ZIM_PI_F)) * ZIM_INV_TWO_PI_F;
                    k = p.iratio[i] * k + (int)roundf(a);
                    r = wr[i];
                }
            }
            if (n_ps == 1) r = wrap0;
        } else {
            const int N = p.shift[0];
            int sum_raw = 0;
            for (int t = 0; t < N; t++) sum_raw += (int)__ldg(frames + (size_t)t * npx + pix);
            int bin = 0, v1 = 0;
            for (int b = 0; b < p.gray_bits; b++) {
                int g = N * (int)__ldg(frames + (size_t)(p.gray_base + b) * npx + pix) > sum_raw ? 1 : 0;
                bin ^= g;
                v1 = (v1 << 1) | bin;
            }
            k = v1;
            if (p.complementary) {
                int g = N * (int)__ldg(frames + (size_t)(p.gray_base + p.gray_bits) * npx + pix) > sum_raw ? 1 : 0;
                int v2 = (v1 << 1) | (bin ^ g);
                int k2 = (v2 + 1) >> 1;
                float w = wrap0;
                if (w <= -0.5f * ZIM_PI_F) k = k2;
                else if (w >= 0.5f * ZIM_PI_F) k = k2 - 1;
            }
            r = wrap0;
        }
    }
    order[pix] = ok ? k : (p.hdr ? -1 : 0);  // the HDR decoder marks invalid orders -1
    residual[pix] = r;
    if (valid_out) valid_out[pix] = ok ? 1 : 0;
}

// One decode tile with its sums staged from global memory.
template <typename T>
__device__ __forceinline__ void decode_tile(const T* __restrict__ frames, const DecodeParams& p, int bx, int by,
                                            int tid, DecodeSmem& sm, int32_t* __restrict__ order,
                                            float* __restrict__ residual, float* __restrict__ mod_out,
                                            uint8_t* __restrict__ valid_out) {
    if (!p.hdr) decode_stage_sums(frames, p, bx, by, tid, sm);
    decode_finish(frames, p, bx, by, tid, sm, order, residual, mod_out, valid_out);
}

// --------------------------------------------------------------- rectify ----

// Post-smoothed phase at a source pixel in exact integer + FP32 form:
// phase_s = 2*pi*K16/16 + R, K16 = sum (1 2 1)x(1 2 1) * order (BORDER_REPLICATE).
__device__ __forceinline__ void smoothed_tap(const int32_t* __restrict__ order, const float* __restrict__ res, int x,
                                             int y, int rows, int cols, int post_smooth, int& K16, float& R) {
    // post_smooth 0: the tap as decoded; 3: the same for HDR decodes, whose
    // invalid pixels (order -1) have phase 0
    if (post_smooth == 0 || post_smooth == 3) {
        size_t o = (size_t)y * cols + x;
        const int k = __ldg(order + o);
        const bool zero = post_smooth == 3 && k < 0;
        K16 = zero ? 0 : 16 * k;
        R = zero ? 0.f : __ldg(res + o);
        return;
    }
    int k = 0;
    float r = 0.f;
#pragma unroll
    for (int a = -1; a <= 1; a++) {
        int yy = min(max(y + a, 0), rows - 1);
        int ca = a == 0 ? 2 : 1;
#pragma unroll
        for (int b = -1; b <= 1; b++) {
            int xx = min(max(x + b, 0), cols - 1);
            int cw = ca * (b == 0 ? 2 : 1);
            size_t o = (size_t)yy * cols + xx;
            k += cw * __ldg(order + o);
            r = fmaf((float)cw * 0.0625f, __ldg(res + o), r);
        }
    }
    K16 = k;
    R = r;
}

// setData remap of one rectified pixel: INTER_LINEAR of the (post-smoothed)
// phase with OpenCV's 1/32-pixel quantised weights and BORDER_CONSTANT 0,
// INTER_NEAREST of the order.  The phase is kept as an integer cycle count
// (exact: every weight is a multiple of 1/16384) plus an FP32 residual.
__device__ __forceinline__ void rectify_pixel(const int32_t* __restrict__ order, const float* __restrict__ res,
                                              int srows, int scols, float mx, float my, int post_smooth,
                                              int32_t& rbase, float& rres, int32_t& rorder) {
    int nx = __float2int_rn(mx), ny = __float2int_rn(my);
    int ko = 0;
    if (nx >= 0 && ny >= 0 && nx < scols && ny < srows) ko = __ldg(order + (size_t)ny * scols + nx);
    int sx = __float2int_rn(mx * 32.0f), sy = __float2int_rn(my * 32.0f);
    int x0 = sx >> 5, y0 = sy >> 5;
    int fx = sx & 31, fy = sy & 31;
    long long I = 0;
    float Rs = 0.f;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        int xx = x0 + (t & 1), yy = y0 + (t >> 1);
        if (xx < 0 || yy < 0 || xx >= scols || yy >= srows) continue;
        int wq = ((t >> 1) ? fy : 32 - fy) * ((t & 1) ? fx : 32 - fx);
        if (wq == 0) continue;
        int K16;
        float R;
        smoothed_tap(order, res, xx, yy, srows, scols, post_smooth, K16, R);
        I += (long long)wq * K16;
        Rs = fmaf((float)wq * (1.0f / 1024.0f), R, Rs);
    }
    // phase = 2*pi*I/16384 + Rs; split I = 16384*base + frac, frac in [-8192, 8192)
    long long base = (I + 8192) >> 14;  // floor((I + 8192) / 16384)
    int frac = (int)(I - (base << 14));
    rbase = (int32_t)base;
    rres = fmaf((float)frac, ZIM_TWO_PI_F / 16384.0f, Rs);
    rorder = ko;
}

// The same remap from phase that was post-smoothed once per source pixel
// (smooth_pixel: K16 = 16 x smoothed cycles, R = smoothed residual), so a
// rectified pixel reads 4 taps instead of 4 x 9.  Identical results: the taps
// hold exactly what smoothed_tap computes.
__device__ __forceinline__ void smooth_pixel(const int32_t* __restrict__ order, const float* __restrict__ res, int rows,
                                             int cols, int x, int y, int32_t* __restrict__ K16,
                                             float* __restrict__ R) {
    int k;
    float r;
    smoothed_tap(order, res, x, y, rows, cols, 1, k, r);
    const size_t o = (size_t)y * cols + x;
    K16[o] = k;
    R[o] = r;
}

// HDR post-smooth (JSLAB_PhaseShiftDecoder_V2.cpp:280-291): the blurred phase
// divided by the blurred validity (invalid pixels, order < 0, count as phase
// 0 with weight 0), 0 at invalid pixels.  With W = sum of the valid [1 2 1]^2
// weights and Kw = sum w k: phase = 2 pi Kw / W + 16 (sum w r / 16) / W, and
// Kw / W splits exactly into an integer q and remainder, so the output keeps
// the (16 x cycles, residual) form: K16 = 16 q, R = (2 pi rem + 16 Rw) / W.
__device__ __forceinline__ void smooth_pixel_hdr(const int32_t* __restrict__ order, const float* __restrict__ res,
                                                 int rows, int cols, int x, int y, int32_t* __restrict__ K16,
                                                 float* __restrict__ R) {
    const size_t o = (size_t)y * cols + x;
    if (__ldg(order + o) < 0) {
        K16[o] = 0;
        R[o] = 0.f;
        return;
    }
    int kw = 0, wv = 0;
    float rw = 0.f;
#pragma unroll
    for (int a = -1; a <= 1; a++) {
        const int yy = min(max(y + a, 0), rows - 1);
        const int ca = a == 0 ? 2 : 1;
#pragma unroll
        for (int b = -1; b <= 1; b++) {
            const int xx = min(max(x + b, 0), cols - 1);
            const int cw = ca * (b == 0 ? 2 : 1);
            const size_t q = (size_t)yy * cols + xx;
            const int kq = __ldg(order + q);
            if (kq < 0) continue;
            kw += cw * kq;
            wv += cw;
            rw = fmaf((float)cw * 0.0625f, __ldg(res + q), rw);
        }
    }
    int qd = kw / wv;  // wv in [4, 16]
    int rem = kw - qd * wv;
    if (rem < 0) { qd--; rem += wv; }
    K16[o] = 16 * qd;
    R[o] = fmaf((float)rem, ZIM_TWO_PI_F, 16.0f * rw) / (float)wv;
}

__device__ __forceinline__ void rectify_pixel_smoothed(const int32_t* __restrict__ K16, const float* __restrict__ Rs_,
                                                       const int32_t* __restrict__ order, int srows, int scols,
                                                       float mx, float my, int32_t& rbase, float& rres,
                                                       int32_t& rorder) {
    int nx = __float2int_rn(mx), ny = __float2int_rn(my);
    int ko = 0;
    if (nx >= 0 && ny >= 0 && nx < scols && ny < srows) ko = __ldg(order + (size_t)ny * scols + nx);
    int sx = __float2int_rn(mx * 32.0f), sy = __float2int_rn(my * 32.0f);
    int x0 = sx >> 5, y0 = sy >> 5;
    int fx = sx & 31, fy = sy & 31;
    long long I = 0;
    float Rs = 0.f;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        int xx = x0 + (t & 1), yy = y0 + (t >> 1);
        if (xx < 0 || yy < 0 || xx >= scols || yy >= srows) continue;
        int wq = ((t >> 1) ? fy : 32 - fy) * ((t & 1) ? fx : 32 - fx);
        if (wq == 0) continue;
        const size_t o = (size_t)yy * scols + xx;
        I += (long long)wq * __ldg(K16 + o);
        Rs = fmaf((float)wq * (1.0f / 1024.0f), __ldg(Rs_ + o), Rs);
    }
    long long base = (I + 8192) >> 14;
    int frac = (int)(I - (base << 14));
    rbase = (int32_t)base;
    rres = fmaf((float)frac, ZIM_TWO_PI_F / 16384.0f, Rs);
    rorder = ko;
}

// ----------------------------------------------------------------- match ----

__device__ __forceinline__ float phase_diff(int bR, float rR, int bL, float rL) {
    // (2 pi bR + rR) - (2 pi bL + rL) with the integer cycles subtracted exactly
    return fmaf((float)(bR - bL), ZIM_TWO_PI_F, rR - rL);
}

// Monotone spans.  Within a right row the rectified phase of one fringe order
// normally rises column by column.  When the order's span [lo, hi] holds only
// pixels of that order and every step to the next column rises by more than
// MATCH_MONO_MARGIN (verified per row and order by match_spans_check), the
// float differences d(c) = phase_R(c) - phase_L computed by phase_diff are
// strictly increasing in c for any left pixel whose phase lies within 1024
// cycles of the span (the rounding of each d is below half the margin), so
// |d| falls, then rises, and its first minimum is at the sign change of d: a
// binary search finds the same column as the reference's scan over every
// candidate (ties keep the earlier column, as the scan's strict < does).
// Spans that fail the check are scanned in full.
constexpr float MATCH_MONO_MARGIN = 2e-3f;

// One left pixel against a right row staged in shared memory (s_ord, s_base,
// s_res; cols columns) with the per-order column spans [s_lo, s_hi] and the
// spans' failed-check flags s_bad (null: always the full scan): the first
// column of minimum |phase_R - phase_L| among right pixels of the same order
// (strict <), rejected if min >= grad_threshold or the column is < 2 or
// >= cols - 1, then the reference's three-point sub-pixel refinement.
// dx_off is (left window x) - (right window x) for the ROI path
// (startCalculate_v2_roi, V2.cpp:719-778: global left x - global right x - delta).
__device__ __forceinline__ void match_pixel(int j, int k, int bL, float rL, const int* s_ord, const int* s_base,
                                            const float* s_res, const int* s_lo, const int* s_hi, const int* s_bad,
                                            int cols, int pha_f, float grad_threshold, float& d, int& best,
                                            int dx_off = 0) {
    d = 0.f;
    best = -1;
    if (k < 1 || k > pha_f) return;
    const int lo = s_lo[k], hi = s_hi[k];
    if (lo > hi) return;
    float min_cost = 1e9f;
    int bj = -1;
    if (s_bad && !s_bad[k] && abs(s_base[lo] - bL) < 1024 && abs(s_base[hi] - bL) < 1024) {
        // first column with d >= 0 (hi + 1 if none)
        int a = lo, b = hi + 1;
        while (a < b) {
            const int m = (a + b) >> 1;
            if (phase_diff(s_base[m], s_res[m], bL, rL) < 0.f) a = m + 1;
            else b = m;
        }
        if (a > hi) {
            bj = hi;
            min_cost = fabsf(phase_diff(s_base[hi], s_res[hi], bL, rL));
        } else if (a == lo) {
            bj = lo;
            min_cost = fabsf(phase_diff(s_base[lo], s_res[lo], bL, rL));
        } else {
            const float dn = fabsf(phase_diff(s_base[a - 1], s_res[a - 1], bL, rL));
            const float dp = fabsf(phase_diff(s_base[a], s_res[a], bL, rL));
            bj = dp < dn ? a : a - 1;
            min_cost = dp < dn ? dp : dn;
        }
    } else {
        for (int c = lo; c <= hi; c++) {
            if (s_ord[c] != k) continue;
            float diff = fabsf(phase_diff(s_base[c], s_res[c], bL, rL));
            if (diff < min_cost) {
                min_cost = diff;
                bj = c;
            }
        }
    }
    if (bj >= 0 && min_cost < grad_threshold && bj >= 2 && bj < cols - 1) {
        float c0 = phase_diff(s_base[bj - 1], s_res[bj - 1], bL, rL);
        float c1 = phase_diff(s_base[bj], s_res[bj], bL, rL);
        float c2 = phase_diff(s_base[bj + 1], s_res[bj + 1], bL, rL);
        float num = c1 * (c0 - c2);
        float den = 2.0f * (c0 - c1) * (c1 - c2);
        float delta = fabsf(den) > 1e-9f ? num / den : 0.f;
        d = (float)(j - bj + dx_off) - delta;
        best = bj;
    }
}

// Per-order column spans of a staged right row (shared atomics).  Callers
// initialise s_lo = INT_MAX, s_hi = -1, s_bad = 0 and sync before, and sync
// after, then run match_spans_check (and sync again).  A span's first column
// is the first column of one of its order's runs and its last the last of
// one, so only run starts update s_lo and only run ends s_hi: about two
// atomics per run instead of one per pixel (a warp's lanes nearly always
// share an order, and same-address atomics serialise).
__device__ __forceinline__ void match_spans(const int* s_ord, int cols, int pha_f, int* s_lo, int* s_hi, int tid,
                                            int nthreads) {
    for (int j = tid; j < cols; j += nthreads) {
        int k = s_ord[j];
        if (k >= 0 && k <= pha_f) {
            if (j == 0 || s_ord[j - 1] != k) atomicMin(&s_lo[k], j);
            if (j == cols - 1 || s_ord[j + 1] != k) atomicMax(&s_hi[k], j);
        }
    }
}

// Marks in s_bad every order whose span holds a pixel of another order or a
// step that does not rise by MATCH_MONO_MARGIN (see match_pixel).  A foreign
// run inside a span always follows a pixel of the span's order, so checking
// each pixel against its right neighbour finds it.
__device__ __forceinline__ void match_spans_check(const int* s_ord, const int* s_base, const float* s_res, int cols,
                                                  int pha_f, const int* s_hi, int* s_bad, int tid, int nthreads) {
    for (int j = tid; j + 1 < cols; j += nthreads) {
        const int k = s_ord[j];
        if (k < 0 || k > pha_f || j >= s_hi[k]) continue;
        if (s_ord[j + 1] != k || !(phase_diff(s_base[j + 1], s_res[j + 1], s_base[j], s_res[j]) > MATCH_MONO_MARGIN))
            s_bad[k] = 1;
    }
}

// -------------------------------------------------------- pixel rays ----
// An organised cloud from one camera: cloud pixel (u, v) looks from the origin
// along R (u + ox - cx, v + oy - cy, f).  A point p seen along the ray of
// pixel b and a query q near the ray of pixel a satisfy
// |p - q| >= |q| sin(angle(a, b)) - dev(q) - dev(p) (dev: distance from the own
// ray), and with |a x b| >= f |b - a|, |b| <= |a| + |b - a|:
// sin(angle) >= f |b - a| / (|a| (|a| + |b - a|)), increasing in |b - a|.
// The window paths of the filters use this to stop scanning a pixel window.

struct RayParams {
    float cx, cy, f, R[9];
    int ox, oy;
};

__device__ __forceinline__ void ray_dir(const RayParams& r, int u, int v, float& ax, float& ay, float& az) {
    const float x = (float)(u + r.ox) - r.cx, y = (float)(v + r.oy) - r.cy;
    ax = fmaf(r.R[0], x, fmaf(r.R[1], y, r.R[2] * r.f));
    ay = fmaf(r.R[3], x, fmaf(r.R[4], y, r.R[5] * r.f));
    az = fmaf(r.R[6], x, fmaf(r.R[7], y, r.R[8] * r.f));
}

// Distance of p from the line through the origin along a: |p x a| / |a|.
__device__ __forceinline__ float ray_dev(float px, float py, float pz, float ax, float ay, float az) {
    const float cx = fmaf(py, az, -pz * ay), cy = fmaf(pz, ax, -px * az), cz = fmaf(px, ay, -py * ax);
    return sqrtf(fmaf(cx, cx, fmaf(cy, cy, cz * cz))) * rsqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
}

inline RayParams ray_params(const zim_ray_model& r) {
    RayParams p;
    p.cx = r.cx; p.cy = r.cy; p.f = r.f;
    for (int a = 0; a < 9; a++) p.R[a] = r.R[a];
    p.ox = r.ox; p.oy = r.oy;
    return p;
}

// half-size and offset count of the window-pass windows (the offsets
// themselves, ordered by length, then row, then column, are a compile-time
// table beside the kernels)
constexpr int SPIRAL_R = 7;
constexpr int SPIRAL_N = (2 * SPIRAL_R + 1) * (2 * SPIRAL_R + 1) - 1;

// -------------------------------------------------- median + reprojection ----

constexpr int RX = 32, RY = 8;  // median/reprojection tile

struct ReprojParams {
    float q03, q13, q23, q32, q33;
    double dq03, dq13, dq23, dq32, dq33;
    float r1[9];
    float min_depth, max_depth;
    double dmin_depth, dmax_depth;
    int use_rectified, use_median;
    int model;                 // 0: Q matrix; 1: per-pixel polynomial maps
    double dr1[9];
    const float4* poly[3];     // x, y, z coefficient maps (c0, c1, c2, c3) per rectified pixel
    // ROI tiles (startCalculate_v2_roi): the disparity tile starts at rectified
    // pixel (ox, oy); points are made only where roi_mask (rectified frame,
    // gstride pixels per row) is non-zero.  Whole frames: 0, 0, null.
    int ox, oy, gstride;
    const uint8_t* roi_mask;
};

inline void reproj_params(const double Q[16], const double R1[9], const zim_recon_config* cfg, ReprojParams& p) {
    p.q03 = (float)Q[3]; p.q13 = (float)Q[7]; p.q23 = (float)Q[11];
    p.q32 = (float)Q[14]; p.q33 = (float)Q[15];
    p.dq03 = Q[3]; p.dq13 = Q[7]; p.dq23 = Q[11]; p.dq32 = Q[14]; p.dq33 = Q[15];
    for (int i = 0; i < 9; i++) p.r1[i] = (float)R1[i];
    p.min_depth = (float)cfg->min_depth;
    p.max_depth = (float)cfg->max_depth;
    p.dmin_depth = cfg->min_depth;
    p.dmax_depth = cfg->max_depth;
    p.use_rectified = cfg->use_rectified_coords != 0;
    p.use_median = cfg->use_disp_median_filter != 0;
    p.model = cfg->reproject_model;
    for (int i = 0; i < 9; i++) p.dr1[i] = R1[i];
    p.poly[0] = p.poly[1] = p.poly[2] = nullptr;
    p.ox = p.oy = p.gstride = 0;
    p.roi_mask = nullptr;
}

// Per-pixel polynomial calibration, evaluateV2CalibPoint
// (JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76): the coefficient maps carry
// a model tag in c3 of the x map (-1 inverse depth, -2 fitted ray, -3 z-linear
// x/y) and of the z map (-1 inverse depth, -4 rational depth); untagged maps
// are cubics in d.  Evaluated in FP64 in the reference's operation order with
// every product and sum rounded separately (no contraction), so the result is
// the same bit pattern as a strict IEEE evaluation on the host.
__device__ __forceinline__ double pm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double pa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ bool poly_tag(float c, float tag) { return fabsf(c - tag) < 1e-6f; }

__device__ __forceinline__ bool poly_point(const float4& cx, const float4& cy, const float4& cz, double d, double& X,
                                           double& Y, double& Z) {
    if (fabsf(cz.x) <= 1e-9 && fabsf(cz.y) <= 1e-9 && fabsf(cz.z) <= 1e-9 && fabsf(cz.w) <= 1e-9) return false;
    const double z0 = cz.x, z1 = cz.y, z2 = cz.z, z3 = cz.w;
    if (poly_tag(cx.w, -1.0f) || poly_tag(cx.w, -2.0f)) {
        const double d2 = pm(d, d);
        if (poly_tag(cx.w, -1.0f) || poly_tag(cz.w, -1.0f)) {
            // inverse depth: cubic (x-map tag -1) or quadratic (x-map tag -2, z-map tag -1)
            double iz = pa(pa(z0, pm(z1, d)), pm(z2, d2));
            if (poly_tag(cx.w, -1.0f)) iz = pa(iz, pm(pm(z3, d2), d));
            if (!isfinite(iz) || fabs(iz) < 1e-12) return false;
            Z = 1.0 / iz;
        } else {
            Z = pa(pa(pa(z0, pm(z1, d)), pm(z2, d2)), pm(pm(z3, d2), d));
        }
        X = pm((double)cx.x, Z);
        Y = pm((double)cy.x, Z);
    } else if (poly_tag(cx.w, -3.0f)) {
        if (poly_tag(cz.w, -4.0f)) {
            const double den = pa(pm(z1, d), 1.0);
            if (!isfinite(den) || fabs(den) < 1e-12) return false;
            Z = z0 / den;
        } else {
            const double d2 = pm(d, d), d3 = pm(d2, d);
            Z = pa(pa(pa(z0, pm(z1, d)), pm(z2, d2)), pm(z3, d3));
        }
        X = pa(pm((double)cx.x, Z), (double)cx.y);
        Y = pa(pm((double)cy.x, Z), (double)cy.y);
    } else if (poly_tag(cz.w, -1.0f)) {
        const double iz = pa(pa(z0, pm(z1, d)), pm(pm(z2, d), d));
        if (!isfinite(iz) || fabs(iz) < 1e-12) return false;
        Z = 1.0 / iz;
        X = pm((double)cx.x, Z);
        Y = pm((double)cy.x, Z);
    } else {
        const double d2 = pm(d, d), d3 = pm(d2, d);
        X = pa(pa(pa((double)cx.x, pm((double)cx.y, d)), pm((double)cx.z, d2)), pm((double)cx.w, d3));
        Y = pa(pa(pa((double)cy.x, pm((double)cy.y, d)), pm((double)cy.z, d2)), pm((double)cy.w, d3));
        Z = pa(pa(pa(z0, pm(z1, d)), pm(z2, d2)), pm(z3, d3));
    }
    return isfinite(X) && isfinite(Y) && isfinite(Z);
}

// startCalculate_v2's per-pixel body (:505-547): polynomial point, optional
// R1^T rotation, depth gate on the reported z.
__device__ __forceinline__ void poly_reproject_point(const ReprojParams& p, size_t o, float d, float& ox, float& oy,
                                                     float& oz, uint8_t& m) {
    const float4 cz = __ldg(p.poly[2] + o);
    double X, Y, Z;
    if (!poly_point(__ldg(p.poly[0] + o), __ldg(p.poly[1] + o), cz, (double)d, X, Y, Z)) return;
    if (p.use_rectified) {
        if (Z > p.dmin_depth && Z < p.dmax_depth) { ox = (float)X; oy = (float)Y; oz = (float)Z; m = 1; }
        return;
    }
    const double rx = pa(pa(pm(p.dr1[0], X), pm(p.dr1[3], Y)), pm(p.dr1[6], Z));
    const double ry = pa(pa(pm(p.dr1[1], X), pm(p.dr1[4], Y)), pm(p.dr1[7], Z));
    const double rz = pa(pa(pm(p.dr1[2], X), pm(p.dr1[5], Y)), pm(p.dr1[8], Z));
    if (rz > p.dmin_depth && rz < p.dmax_depth) { ox = (float)rx; oy = (float)ry; oz = (float)rz; m = 1; }
}

__device__ __forceinline__ void cswap(float& a, float& b) {
    float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}

// Moves the minimum of w[0..n) to w[0] and the maximum to w[n-1].
template <int N>
__device__ __forceinline__ void minmax_ends(float* w) {
#pragma unroll
    for (int i = 1; i < N; i++) cswap(w[0], w[i]);
#pragma unroll
    for (int i = 1; i < N - 1; i++) cswap(w[i], w[N - 1]);
}

// Exact median of 25 values by forgetful selection: keep 14, drop min and max,
// add one, repeat; every dropped value provably has rank != 13.
__device__ __forceinline__ float median25(float* a) {
    minmax_ends<14>(a);            // a[1..12] live
    a[13] = a[14]; minmax_ends<13>(a + 1);  // live a[2..12]
    a[1] = a[15];  minmax_ends<12>(a + 1);  // live a[2..11]
    a[12] = a[16]; minmax_ends<11>(a + 2);  // live a[3..11]
    a[2] = a[17];  minmax_ends<10>(a + 2);  // live a[3..10]
    a[11] = a[18]; minmax_ends<9>(a + 3);   // live a[4..10]
    a[3] = a[19];  minmax_ends<8>(a + 3);   // live a[4..9]
    a[10] = a[20]; minmax_ends<7>(a + 4);   // live a[5..9]
    a[4] = a[21];  minmax_ends<6>(a + 4);   // live a[5..8]
    a[9] = a[22];  minmax_ends<5>(a + 5);   // live a[6..8]
    a[5] = a[23];  minmax_ends<4>(a + 5);   // live a[6..7]
    a[8] = a[24];  minmax_ends<3>(a + 6);   // live a[7]
    return a[7];
}

// Two horizontally adjacent 5x5 windows share 20 values.  A shared value of
// rank r among those 20 has rank r .. r + 5 in either window, so only ranks
// 8..13 can be a window's median (rank 13 of 25); with the 7 lower shared
// values below them and at most 5 own values among the rest, each window's
// median is the median (rank 6) of those 6 and its own 5-value column.
// mid6_of_20: forgetful selection on a[0..19] leaving ranks 8..13 in a[4..9]
// (each dropped min has rank <= 7, each dropped max rank >= 14).
__device__ __forceinline__ void mid6_of_20(float* a) {
    minmax_ends<14>(a);            // live a[1..12], unseen a[14..19]
    a[13] = a[14]; minmax_ends<13>(a + 1);  // live a[2..12]
    a[1] = a[15];  minmax_ends<12>(a + 1);  // live a[2..11]
    a[12] = a[16]; minmax_ends<11>(a + 2);  // live a[3..11]
    a[2] = a[17];  minmax_ends<10>(a + 2);  // live a[3..10]
    a[11] = a[18]; minmax_ends<9>(a + 3);   // live a[4..10]
    a[3] = a[19];  minmax_ends<8>(a + 3);   // live a[4..9]
    // ranks 8..13 of the 20 in a[4..9]
}

// Median (rank 6) of 11 values by forgetful selection.
__device__ __forceinline__ float median11(float* a) {
    minmax_ends<7>(a);            // live a[1..5], unseen a[7..10]
    a[6] = a[7];  minmax_ends<6>(a + 1);  // live a[2..5]
    a[1] = a[8];  minmax_ends<5>(a + 1);  // live a[2..4]
    a[5] = a[9];  minmax_ends<4>(a + 2);  // live a[3..4]
    a[2] = a[10]; minmax_ends<3>(a + 2);  // live a[3]
    return a[3];
}

// Median tiles are MTX x RY pixels for RX x RY threads: each thread takes two
// adjacent pixels (2 tx, 2 tx + 1) of a row.
constexpr int MTX = 2 * RX;

struct MedianSmem {
    __align__(8) float tile[RY + 4][MTX + 4];
};

// Q (or polynomial-map) reprojection of one pixel's disparity; (gx, gy) its
// rectified-frame pixel, go its index in the maps.
__device__ __forceinline__ void reproject_pixel(const ReprojParams& p, int gx, int gy, size_t go, float d, float& ox,
                                                float& oy, float& oz, uint8_t& m) {
    ox = oy = oz = 0.f;
    m = 0;
    // the reference gates |d| < 1e-5 on the disparity widened to double
    const bool has_d = fabs((double)d) >= 1e-5 && (!p.roi_mask || p.roi_mask[go]);
    if (p.model == 1) {
        if (has_d) poly_reproject_point(p, go, d, ox, oy, oz, m);
    } else if (has_d) {
        float X, Y, Z;
        float w = fmaf(p.q32, d, p.q33);
        if (fabsf(w) < 1e-2f * (fabsf(p.q32 * d) + fabsf(p.q33))) {
            // near-zero disparity denominator: FP64 divide
            double wd = fma(p.dq32, (double)d, p.dq33);
            double iw = 1.0 / wd;
            X = (float)(((double)gx + p.dq03) * iw);
            Y = (float)(((double)gy + p.dq13) * iw);
            Z = (float)(p.dq23 * iw);
            double zz = p.dq23 * iw;
            if (p.use_rectified) {
                if (zz > p.dmin_depth && zz < p.dmax_depth) { ox = X; oy = Y; oz = Z; m = 1; }
            } else {
                double xx = ((double)gx + p.dq03) * iw, yy = ((double)gy + p.dq13) * iw;
                double rx = fma((double)p.r1[0], xx, fma((double)p.r1[3], yy, (double)p.r1[6] * zz));
                double ry = fma((double)p.r1[1], xx, fma((double)p.r1[4], yy, (double)p.r1[7] * zz));
                double rz = fma((double)p.r1[2], xx, fma((double)p.r1[5], yy, (double)p.r1[8] * zz));
                if (rz > p.dmin_depth && rz < p.dmax_depth) { ox = (float)rx; oy = (float)ry; oz = (float)rz; m = 1; }
            }
        } else {
            float iw = 1.0f / w;
            X = ((float)gx + p.q03) * iw;
            Y = ((float)gy + p.q13) * iw;
            Z = p.q23 * iw;
            if (p.use_rectified) {
                if (Z > p.min_depth && Z < p.max_depth) { ox = X; oy = Y; oz = Z; m = 1; }
            } else {
                float rx = fmaf(p.r1[0], X, fmaf(p.r1[3], Y, p.r1[6] * Z));
                float ry = fmaf(p.r1[1], X, fmaf(p.r1[4], Y, p.r1[7] * Z));
                float rz = fmaf(p.r1[2], X, fmaf(p.r1[5], Y, p.r1[8] * Z));
                if (rz > p.min_depth && rz < p.max_depth) { ox = rx; oy = ry; oz = rz; m = 1; }
            }
        }
    }
}

// 5x5 median (replicate border) + Q reprojection of median tile (bx, by)
// (MTX x RY pixels) with the RX * RY threads of a block.  Ends past the last
// shared read.
__device__ __forceinline__ void median_reproject_tile(const float* __restrict__ disp, int rows, int cols,
                                                      const ReprojParams& p, int bx, int by, int tid, MedianSmem& sm,
                                                      float* __restrict__ disp_out, float* __restrict__ xyz,
                                                      uint8_t* __restrict__ mask) {
    const int tx = tid % RX, ty = tid / RX;
    const int x = bx * MTX + 2 * tx, y = by * RY + ty;  // the thread's pixels: x and x + 1
    float d0 = 0.f, d1 = 0.f;
    if (p.use_median) {
        const int gx0 = bx * MTX - 2, gy0 = by * RY - 2;
        for (int h = tid; h < (MTX + 4) * (RY + 4); h += RX * RY) {
            int hy = h / (MTX + 4), hx = h - hy * (MTX + 4);
            int gy = min(max(gy0 + hy, 0), rows - 1), gx = min(max(gx0 + hx, 0), cols - 1);
            sm.tile[hy][hx] = __ldg(disp + (size_t)gy * cols + gx);
        }
        __syncthreads();
        // columns x - 2 .. x + 3 of five rows as float2 pairs: c0 only in
        // pixel x's window, c5 only in pixel x + 1's, c1..c4 in both
        float sh[20], own0[5], own1[5];
#pragma unroll
        for (int dy = 0; dy < 5; dy++) {
            const float2* r2 = reinterpret_cast<const float2*>(&sm.tile[ty + dy][2 * tx]);
            const float2 a = r2[0], b = r2[1], c = r2[2];
            own0[dy] = a.x;
            sh[4 * dy] = a.y; sh[4 * dy + 1] = b.x; sh[4 * dy + 2] = b.y; sh[4 * dy + 3] = c.x;
            own1[dy] = c.y;
        }
        __syncthreads();
        mid6_of_20(sh);
        float m0[11], m1[11];
#pragma unroll
        for (int q = 0; q < 6; q++) m0[q] = m1[q] = sh[4 + q];
#pragma unroll
        for (int q = 0; q < 5; q++) { m0[6 + q] = own0[q]; m1[6 + q] = own1[q]; }
        d0 = median11(m0);
        d1 = median11(m1);
    } else if (y < rows) {
        if (x < cols) d0 = disp[(size_t)y * cols + x];
        if (x + 1 < cols) d1 = disp[(size_t)y * cols + x + 1];
    }
    if (y >= rows) return;
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const int xx = x + l;
        if (xx >= cols) break;
        const float d = l ? d1 : d0;
        const size_t o = (size_t)y * cols + xx;
        if (disp_out) disp_out[o] = d;
        // rectified-frame pixel (ROI tiles are offset) and its index in the maps
        const int gx = xx + p.ox, gy = y + p.oy;
        const size_t go = p.gstride ? (size_t)gy * p.gstride + gx : o;
        float ox, oy, oz;
        uint8_t m;
        reproject_pixel(p, gx, gy, go, d, ox, oy, oz, m);
        xyz[3 * o] = ox;
        xyz[3 * o + 1] = oy;
        xyz[3 * o + 2] = oz;
        mask[o] = m;
    }
}

// ------------------------------------------------- pixel-window filters ----

// getGaussianKernel(3, 0.7, CV_32F) outer-product weights: corner, edge, centre.
inline void px_gaussian_weights(float& w00, float& w01, float& w11) {
    double t = std::exp(-0.5 / (0.7 * 0.7));
    double mul = 1.0 / (2.0 * t + 1.0);
    float k0 = (float)(t * mul), k1 = (float)mul;
    w00 = k0 * k0;
    w01 = k0 * k1;
    w11 = k1 * k1;
}

// 3x3 point-cloud Gaussian (sigma 0.7 px) at (x, y): neighbour used if valid
// and |x_n - x_c| < 3; output sum(w p) / sum(w) if sum(w) > 0.8, else 0;
// borders 0.  The weighted mean is accumulated as p_c + sum(w (p_n - p_c)) /
// sum(w), the same value with millimetre-scale FP32 sums.
__device__ __forceinline__ void px_gaussian_pixel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask,
                                                  int rows, int cols, int x, int y, float w00, float w01, float w11,
                                                  float* __restrict__ out, uint8_t* __restrict__ mask_out) {
    size_t o = (size_t)y * cols + x;
    float sx = 0.f, sy = 0.f, sz = 0.f, cnt = 0.f;
    bool inner = x >= 1 && y >= 1 && x < cols - 1 && y < rows - 1 && mask[o];
    float cx = 0.f, cy = 0.f, cz = 0.f;
    if (inner) {
        cx = __ldg(xyz + 3 * o);
        cy = __ldg(xyz + 3 * o + 1);
        cz = __ldg(xyz + 3 * o + 2);
#pragma unroll
        for (int a = -1; a <= 1; a++)
#pragma unroll
            for (int b = -1; b <= 1; b++) {
                size_t q = o + (ptrdiff_t)a * cols + b;
                if (!__ldg(mask + q)) continue;
                float nx = __ldg(xyz + 3 * q);
                if (fabsf(nx - cx) < 3.0f) {
                    float w = (a == 0 && b == 0) ? w11 : ((a == 0 || b == 0) ? w01 : w00);
                    sx = fmaf(nx - cx, w, sx);
                    sy = fmaf(__ldg(xyz + 3 * q + 1) - cy, w, sy);
                    sz = fmaf(__ldg(xyz + 3 * q + 2) - cz, w, sz);
                    cnt += w;
                }
            }
    }
    bool keep = inner && cnt > 0.8f;
    out[3 * o] = keep ? cx + sx / cnt : 0.f;
    out[3 * o + 1] = keep ? cy + sy / cnt : 0.f;
    out[3 * o + 2] = keep ? cz + sz / cnt : 0.f;
    if (mask_out) mask_out[o] = keep ? 1 : 0;
}

// Radius outlier filter over tile (bx, by) of RX x RY pixels with the RX * RY
// threads of a block: keep a valid point if at least min_nb valid neighbours
// (not itself) of its (2 hw + 1)^2 window lie within sqrt(r2).  The tile and
// its hw halo are staged in shared memory (ror_smem_bytes) as float4 with
// invalid and off-image pixels NaN, so a neighbour test is one shared load
// and an FP32 distance that compares false for NaN.  The point itself passes
// its own test (distance 0), so the count including it must reach
// min_nb + 1.  Ends past the last shared read.
inline size_t ror_smem_bytes(int hw) { return (size_t)(RX + 2 * hw) * (RY + 2 * hw) * sizeof(float4); }

__device__ __forceinline__ void ror_tile(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows,
                                         int cols, int bx, int by, int tid, float r2, int min_nb, int hw, float4* sp,
                                         float* __restrict__ out, uint8_t* __restrict__ mask_out) {
    const int TW = RX + 2 * hw, TH = RY + 2 * hw;
    const int gx0 = bx * RX - hw, gy0 = by * RY - hw;
    for (int t = tid; t < TW * TH; t += RX * RY) {
        const int ty = t / TW, tx = t - ty * TW;
        const int gx = gx0 + tx, gy = gy0 + ty;
        float4 v = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
        if (gx >= 0 && gy >= 0 && gx < cols && gy < rows) {
            const size_t q = (size_t)gy * cols + gx;
            if (__ldg(mask + q)) v = make_float4(__ldg(xyz + 3 * q), __ldg(xyz + 3 * q + 1), __ldg(xyz + 3 * q + 2), 1.f);
        }
        sp[t] = v;
    }
    __syncthreads();
    const int tx = tid % RX, ty = tid / RX;
    const int x = bx * RX + tx, y = by * RY + ty;
    const float4 c = sp[(ty + hw) * TW + tx + hw];
    bool keep = false;
    if (x < cols && y < rows && c.w != 0.f) {
        keep = min_nb <= 0;
        int cnt = 0;
        for (int i = 0; i <= 2 * hw && !keep; i++) {
            const float4* row = sp + (ty + i) * TW + tx;
            for (int j = 0; j <= 2 * hw; j++) {
                const float4 p = row[j];
                const float dx = c.x - p.x, dy = c.y - p.y, dz = c.z - p.z;
                cnt += fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= r2 ? 1 : 0;
            }
            keep = cnt >= min_nb + 1;
        }
    }
    __syncthreads();
    if (x >= cols || y >= rows) return;
    const size_t o = (size_t)y * cols + x;
    out[3 * o] = keep ? c.x : 0.f;
    out[3 * o + 1] = keep ? c.y : 0.f;
    out[3 * o + 2] = keep ? c.z : 0.f;
    mask_out[o] = keep ? 1 : 0;
}

}  // namespace zt
