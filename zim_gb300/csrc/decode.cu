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

#include "zim_tiles.cuh"

namespace {

using zt::DecodeParams;

template <typename T>
__global__ void __launch_bounds__(zt::DX* zt::DY) decode_kernel(const T* __restrict__ frames, DecodeParams p,
                                                                 int32_t* __restrict__ order,
                                                                 float* __restrict__ residual,
                                                                 float* __restrict__ mod_out,
                                                                 uint8_t* __restrict__ valid_out) {
    __shared__ zt::DecodeSmem sm;
    zt::decode_tile<T>(frames, p, blockIdx.x, blockIdx.y, threadIdx.y * zt::DX + threadIdx.x, sm, order, residual,
                       mod_out, valid_out);
}

// Absolute phase as f64 (startCalculate's CV_64F map; 0 where invalid), with
// the optional 3x3 post-smooth (fixed [1/4 1/2 1/4] kernel, BORDER_REPLICATE):
// post_smooth 1 blurs the phase map as is; 2 is the HDR form, the blur divided
// by the blurred validity, 0 at invalid pixels (JSLAB_PhaseShiftDecoder_V2.cpp:280-291);
// 3 is an HDR decode without smoothing.  An HDR decode marks invalid pixels
// with order -1 (a plain decode zeroes them, and Gray code can give a valid -1).
__global__ void phase_f64_kernel(const int32_t* __restrict__ order, const float* __restrict__ res, int rows, int cols,
                                 int post_smooth, double* __restrict__ out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= cols || y >= rows) return;
    const size_t oc = (size_t)y * cols + x;
    const bool hdr = post_smooth >= 2;
    if (post_smooth == 0 || post_smooth == 3) {
        out[oc] = hdr && order[oc] < 0 ? 0.0 : 6.283185307179586 * order[oc] + (double)res[oc];
        return;
    }
    if (hdr && order[oc] < 0) {
        out[oc] = 0.0;
        return;
    }
    double P = 0, W = 0;
    for (int a = -1; a <= 1; a++) {
        int yy = min(max(y + a, 0), rows - 1);
        for (int b = -1; b <= 1; b++) {
            int xx = min(max(x + b, 0), cols - 1);
            int w = (a == 0 ? 2 : 1) * (b == 0 ? 2 : 1);
            size_t o = (size_t)yy * cols + xx;
            if (hdr && order[o] < 0) continue;
            P += w * (6.283185307179586 * order[o] + (double)res[o]);
            W += w;
        }
    }
    out[oc] = hdr ? P / W : P / 16.0;
}

}  // namespace

zim_status zim_decode_launch(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames, int sample_type, int rows,
                             int cols, int32_t* order, float* residual, float* mod, uint8_t* valid, cudaStream_t st) {
    DecodeParams p;
    zt::decode_params(cfg, rows, cols, p);
    dim3 blk(zt::DX, zt::DY), grd((cols + zt::DX - 1) / zt::DX, (rows + zt::DY - 1) / zt::DY);
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
