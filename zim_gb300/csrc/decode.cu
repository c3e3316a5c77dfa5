// decode.cu -- per-pixel N-step phase-shift decode: fused 3x3 pre-blur,
// wrapped phase (atan2) + normalised modulation with the validity threshold,
// then heterodyne (reference), hierarchical or Gray-code unwrapping.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseShiftDecoder_V2.cpp:18-28
// (pre-blur), :54-182 (decode body); GPU port JSLAB_PhaseShiftDecoder_V2_GPU.cu:44-146.
//
// Arithmetic is FP32.  The pre-blur is linear, so the blurred sums
// S = -sum sin_k I_k, C = sum cos_k I_k, sum I_k are the 3x3 blur of the raw
// per-pixel sums: a CTA computes the raw sums over its tile + 1-pixel halo into
// shared memory once per frequency and blurs 3 channels instead of N frames.
// Unwrapping keeps integer cycle counts exact and only small fractional parts
// in FP32, so an order differs from the FP64 restatement only when a decision
// argument sits within ~1e-6 of its threshold.
#include <cmath>

#include "zim_internal.cuh"

namespace {

constexpr int TX = 32, TY = 8;
constexpr int HX = TX + 2, HY = TY + 2;

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
};

__device__ __forceinline__ int floor_div(int a, int b) {  // b > 0
    int q = a / b;
    return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

template <typename T>
__global__ void __launch_bounds__(TX* TY) decode_kernel(const T* __restrict__ frames, DecodeParams p,
                                                         int32_t* __restrict__ order, float* __restrict__ residual,
                                                         float* __restrict__ mod_out, uint8_t* __restrict__ valid_out) {
    __shared__ float sS[HY][HX + 1], sC[HY][HX + 1], sM[HY][HX + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x = blockIdx.x * TX + tx, y = blockIdx.y * TY + ty;
    const int gx0 = blockIdx.x * TX - 1, gy0 = blockIdx.y * TY - 1;
    const size_t npx = (size_t)p.rows * p.cols;

    float wrap[4];
    float mod0 = 0.f;
    bool ok = true;
    for (int i = 0; i < p.n_ps; i++) {
        const int N = p.shift[i];
        const T* fb = frames + (size_t)p.fbase[i] * npx;
        const float* sv = p.sinv + p.fbase[i];
        const float* cv = p.cosv + p.fbase[i];
        for (int h = tid; h < HX * HY; h += TX * TY) {
            int hy = h / HX, hx = h - hy * HX;
            int gy = min(max(gy0 + hy, 0), p.rows - 1), gx = min(max(gx0 + hx, 0), p.cols - 1);
            const T* src = fb + (size_t)gy * p.cols + gx;
            float s = 0.f, c = 0.f, m = 0.f;
            for (int k = 0; k < N; k++) {
                float v = (float)__ldg(src + (size_t)k * npx);
                s = fmaf(-sv[k], v, s);
                c = fmaf(cv[k], v, c);
                m += v;
            }
            sS[hy][hx] = s;
            sC[hy][hx] = c;
            sM[hy][hx] = m;
        }
        __syncthreads();
        float S = 0.f, C = 0.f, M = 0.f;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                float w = p.w2d[a * 3 + b];
                S = fmaf(w, sS[ty + a][tx + b], S);
                C = fmaf(w, sC[ty + a][tx + b], C);
                M = fmaf(w, sM[ty + a][tx + b], M);
            }
        __syncthreads();
        if (ok) {
            wrap[i] = atan2f(S, C);
            float b = 2.0f * sqrtf(S * S + C * C) / (float)N;
            float mean = M / (float)N;
            float nm = mean > 1e-3f ? b / mean : 0.f;
            if (i == 0) mod0 = nm;
            if (nm < p.thr) ok = false;
        }
    }
    if (x >= p.cols || y >= p.rows) return;
    const size_t pix = (size_t)y * p.cols + x;
    if (mod_out) mod_out[pix] = mod0;
    int k = 0;
    float r = 0.f;
    if (ok) {
        if (p.enc == ZIM_ENC_HETERODYNE3) {
            const float w0 = wrap[0], w1 = wrap[1], w2 = wrap[2];
            float p12 = w0 > w1 ? w0 - w1 : w0 - w1 + ZIM_TWO_PI_F;
            float p23;
            if (p.f1_gt_f2) p23 = w1 > w2 ? w1 - w2 : w1 - w2 + ZIM_TWO_PI_F;
            else p23 = w2 > w1 ? w2 - w1 : w2 - w1 + ZIM_TWO_PI_F;
            float p123 = p12 > p23 ? p12 - p23 : p12 - p23 + ZIM_TWO_PI_F;
            // uphase12 = p12 + 2 pi m12;  k = round(m12 f0 / f12 + (p12 f0 / f12 - w0) / 2 pi)
            int m12 = (int)roundf((p123 * (float)p.f12 - p12) * ZIM_INV_TWO_PI_F);
            int num = m12 * p.f0;
            int q = floor_div(num, p.f12);
            int rem = num - q * p.f12;
            k = q + (int)roundf((float)rem * p.inv_f12 + (p12 * p.f0_f12 - w0) * ZIM_INV_TWO_PI_F);
            r = w0;
            if (p.avg3) {
                int m23 = (int)roundf((p123 * (float)p.f23 - p23) * ZIM_INV_TWO_PI_F);
                int n2 = m23 * p.f1, q2 = floor_div(n2, p.f23), r2i = n2 - q2 * p.f23;
                int k2 = q2 + (int)roundf((float)r2i * p.inv_f23 + (p23 * p.f1_f23 - w1) * ZIM_INV_TWO_PI_F);
                int n3 = m23 * p.f2, q3 = floor_div(n3, p.f23), r3i = n3 - q3 * p.f23;
                int k3 = q3 + (int)roundf((float)r3i * p.inv_f23 + (p23 * p.f2_f23 - w2) * ZIM_INV_TWO_PI_F);
                // (uphase2 f0 / f1 - 2 pi k) = (w1 f0 + 2 pi (k2 f0 - k f1)) / f1, same for 3
                float r2 = fmaf((float)(k2 * p.f0 - k * p.f1), ZIM_TWO_PI_F, w1 * (float)p.f0) * p.inv_f1;
                float r3 = fmaf((float)(k3 * p.f0 - k * p.f2), ZIM_TWO_PI_F, w2 * (float)p.f0) * p.inv_f2;
                r = (w0 + r2 + r3) * (1.0f / 3.0f);
            }
        } else if (p.enc == ZIM_ENC_HIERARCHICAL) {
            for (int i = 1; i < p.n_ps; i++) {
                float a = (p.fratio[i] * (wrap[i - 1] + ZIM_PI_F) - (wrap[i] + ZIM_PI_F)) * ZIM_INV_TWO_PI_F;
                k = p.iratio[i] * k + (int)roundf(a);
            }
            r = wrap[p.n_ps - 1];
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
                float w = wrap[0];
                if (w <= -0.5f * ZIM_PI_F) k = k2;
                else if (w >= 0.5f * ZIM_PI_F) k = k2 - 1;
            }
            r = wrap[0];
        }
    }
    order[pix] = k;
    residual[pix] = r;
    if (valid_out) valid_out[pix] = ok ? 1 : 0;
}

// Absolute phase as f64 (startCalculate's CV_64F map), optional 3x3 post-smooth
// (fixed [1/4 1/2 1/4] kernel, BORDER_REPLICATE).
__global__ void phase_f64_kernel(const int32_t* __restrict__ order, const float* __restrict__ res, int rows, int cols,
                                 int post_smooth, double* __restrict__ out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= cols || y >= rows) return;
    if (!post_smooth) {
        size_t o = (size_t)y * cols + x;
        out[o] = 6.283185307179586 * order[o] + (double)res[o];
        return;
    }
    int K = 0;
    double R = 0;
    for (int a = -1; a <= 1; a++) {
        int yy = min(max(y + a, 0), rows - 1);
        for (int b = -1; b <= 1; b++) {
            int xx = min(max(x + b, 0), cols - 1);
            int w = (a == 0 ? 2 : 1) * (b == 0 ? 2 : 1);
            size_t o = (size_t)yy * cols + xx;
            K += w * order[o];
            R += w * (double)res[o];
        }
    }
    out[(size_t)y * cols + x] = 6.283185307179586 * (K / 16.0) + R / 16.0;
}

}  // namespace

static bool build_params(const zim_decode_config* c, int rows, int cols, DecodeParams& p) {
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
    return true;
}

zim_status zim_decode_launch(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames, int sample_type, int rows,
                             int cols, int32_t* order, float* residual, float* mod, uint8_t* valid, cudaStream_t st) {
    DecodeParams p;
    build_params(cfg, rows, cols, p);
    dim3 blk(TX, TY), grd((cols + TX - 1) / TX, (rows + TY - 1) / TY);
    if (sample_type == ZIM_SAMPLE_U8)
        decode_kernel<uint8_t><<<grd, blk, 0, st>>>((const uint8_t*)frames, p, order, residual, mod, valid);
    else
        decode_kernel<uint16_t><<<grd, blk, 0, st>>>((const uint16_t*)frames, p, order, residual, mod, valid);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_decode(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames,
                                         int sample_type, int rows, int cols, int32_t* order, float* residual,
                                         float* mod, uint8_t* valid, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    zim_status s = zim_decode_validate(cfg);
    if (s != ZIM_OK) return zim_fail(ctx, s, "invalid decode config");
    if (!frames || !order || !residual) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows <= 0 || cols <= 0 || (size_t)rows * cols > ((size_t)1 << 31))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad image size %dx%d", cols, rows);
    if (sample_type != ZIM_SAMPLE_U8 && sample_type != ZIM_SAMPLE_U16)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad sample type");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return zim_decode_launch(ctx, cfg, frames, sample_type, rows, cols, order, residual, mod, valid, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_decode_phase_f64(zim_ctx* ctx, const int32_t* order, const float* residual, int rows,
                                                   int cols, int post_smooth, double* phase, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!order || !residual || !phase || rows <= 0 || cols <= 0)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    dim3 blk(256), grd((cols + 255) / 256, rows);
    phase_f64_kernel<<<grd, blk, 0, zim_stream(stream)>>>(order, residual, rows, cols, post_smooth, phase);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}
