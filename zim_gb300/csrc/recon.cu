// recon.cu -- disparity median + Q reprojection, the reference's pixel-window
// point-cloud filters (3x3 Gaussian, radius outlier) and PointXYZ compaction.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp
//   medianBlur(5) :405-410, reprojection :414-461, Gaussian :79-124, ROR :126-195;
//   GPU port JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:119-347.
#include <cmath>

#include "zim_tiles.cuh"

namespace {

using zt::ReprojParams;
using zt::RX;
using zt::RY;

__global__ void __launch_bounds__(RX* RY) median_reproject_kernel(const float* __restrict__ disp, int rows, int cols,
                                                                  ReprojParams p, float* __restrict__ disp_out,
                                                                  float* __restrict__ xyz, uint8_t* __restrict__ mask) {
    __shared__ zt::MedianSmem sm;
    zt::median_reproject_tile(disp, rows, cols, p, blockIdx.x, blockIdx.y, threadIdx.y * RX + threadIdx.x, sm,
                              disp_out, xyz, mask);
}

__global__ void px_gaussian_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                   float w00, float w01, float w11, float* __restrict__ out,
                                   uint8_t* __restrict__ mask_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= cols || y >= rows) return;
    zt::px_gaussian_pixel(xyz, mask, rows, cols, x, y, w00, w01, w11, out, mask_out);
}

__global__ void __launch_bounds__(RX* RY) ror_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask,
                                                     int rows, int cols, float r2, int min_nb, int hw,
                                                     float* __restrict__ out, uint8_t* __restrict__ mask_out) {
    extern __shared__ float4 ror_smem[];
    zt::ror_tile(xyz, mask, rows, cols, blockIdx.x, blockIdx.y, threadIdx.y * RX + threadIdx.x, r2, min_nb, hw,
                 ror_smem, out, mask_out);
}

constexpr int CB = 1024;  // compaction block

__global__ void compact_count_kernel(const uint8_t* __restrict__ mask, size_t n, uint32_t* __restrict__ counts) {
    __shared__ uint32_t warp_sums[CB / 32];
    size_t i = (size_t)blockIdx.x * CB + threadIdx.x;
    uint32_t v = (i < n && mask[i]) ? 1u : 0u;
    uint32_t b = __ballot_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = warp_sums[threadIdx.x];
        for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) counts[blockIdx.x] = s;
    }
}

// Single-CTA exclusive scan of the block counts; total goes to count_dev.
__global__ void compact_scan_kernel(uint32_t* __restrict__ counts, int nb, uint64_t* __restrict__ count_dev) {
    __shared__ uint32_t carry_s;
    __shared__ uint32_t wsum[32];
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        int i = base + threadIdx.x;
        uint32_t v = i < nb ? counts[i] : 0;
        uint32_t x = v;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += t;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t s = wsum[lane];
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, s, off);
                if (lane >= off) s += t;
            }
            wsum[lane] = s;
        }
        __syncthreads();
        uint32_t incl = x + (w > 0 ? wsum[w - 1] : 0);
        uint32_t carry = carry_s;
        if (i < nb) counts[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = carry + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count_dev = carry_s;
}

// Record layouts the compaction can emit for each valid point, in row order.
enum Emit { EMIT_POINTXYZ, EMIT_PLY_XYZ, EMIT_PLY_XYZ_GRAY };

// Binary little-endian PLY vertex bodies (savePointCloudToPlyBinary and
// savePointCloudToPlyBinaryWithGray, main.cpp:85-160): float x, y, z, then for
// the grey variant the grey value three times as uchar red, green, blue.
template <int E>
__device__ __forceinline__ void emit(const float* __restrict__ xyz, const uint8_t* __restrict__ gray, size_t i,
                                     uint32_t pos, void* __restrict__ out) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (E == EMIT_POINTXYZ) {
        zim_point_xyz p;
        p.x = x; p.y = y; p.z = z;
        p.pad = 1.0f;
        static_cast<zim_point_xyz*>(out)[pos] = p;
    } else if (E == EMIT_PLY_XYZ) {
        float* r = static_cast<float*>(out) + 3 * (size_t)pos;
        r[0] = x; r[1] = y; r[2] = z;
    } else {
        uint8_t* r = static_cast<uint8_t*>(out) + 15 * (size_t)pos;  // byte-aligned records
        const float v[3] = {x, y, z};
        const uint8_t* b = reinterpret_cast<const uint8_t*>(v);
#pragma unroll
        for (int k = 0; k < 12; k++) r[k] = b[k];
        const uint8_t g = gray ? gray[i] : (uint8_t)255;
        r[12] = g; r[13] = g; r[14] = g;
    }
}

template <int E>
__global__ void compact_write_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                     const uint32_t* __restrict__ offsets, const uint8_t* __restrict__ gray,
                                     void* __restrict__ out) {
    __shared__ uint32_t warp_off[CB / 32];
    size_t i = (size_t)blockIdx.x * CB + threadIdx.x;
    bool v = i < n && mask[i];
    uint32_t b = __ballot_sync(0xffffffffu, v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_off[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = warp_off[threadIdx.x], x = s;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, off);
            if (threadIdx.x >= off) x += t;
        }
        warp_off[threadIdx.x] = x - s;
    }
    __syncthreads();
    if (v) emit<E>(xyz, gray, i, offsets[blockIdx.x] + warp_off[w] + __popc(b & ((1u << lane) - 1u)), out);
}

}  // namespace

zim_status zim_median_reproject_launch(zim_ctx* ctx, const zim_recon_config* cfg, const float* disp, int rows,
                                       int cols, float* disp_out, float* xyz, uint8_t* mask, cudaStream_t st) {
    ReprojParams p;
    zt::reproj_params(ctx->Q, ctx->R1, cfg, p);
    for (int k = 0; k < 3; k++) p.poly[k] = ctx->d_poly[k];
    dim3 blk(RX, RY), grd((cols + zt::MTX - 1) / zt::MTX, (rows + RY - 1) / RY);
    median_reproject_kernel<<<grd, blk, 0, st>>>(disp, rows, cols, p, disp_out, xyz, mask);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_px_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float* out,
                                  uint8_t* mask_out, cudaStream_t st) {
    float w00, w01, w11;
    zt::px_gaussian_weights(w00, w01, w11);
    dim3 blk(32, 8), grd((cols + 31) / 32, (rows + 7) / 8);
    px_gaussian_kernel<<<grd, blk, 0, st>>>(xyz, mask, rows, cols, w00, w01, w11, out, mask_out);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_ror_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float radius,
                          int min_neighbors, int window_size, float* out, uint8_t* mask_out, cudaStream_t st) {
    const int hw = window_size / 2;
    const size_t smem = zt::ror_smem_bytes(hw);
    ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(ror_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 blk(RX, RY), grd((cols + RX - 1) / RX, (rows + RY - 1) / RY);
    ror_kernel<<<grd, blk, smem, st>>>(xyz, mask, rows, cols, radius * radius, min_neighbors, hw, out, mask_out);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_compact_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                              zim_point_xyz* points, uint64_t* count_dev, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    int nb = (int)((n + CB - 1) / CB);
    uint32_t* counts = (uint32_t*)zim_scratch_take(ctx, (size_t)nb * 4);
    if (!counts) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "compaction scratch");
    compact_count_kernel<<<nb, CB, 0, st>>>(mask, n, counts);
    compact_scan_kernel<<<1, 1024, 0, st>>>(counts, nb, count_dev);
    compact_write_kernel<EMIT_POINTXYZ><<<nb, CB, 0, st>>>(xyz, mask, n, counts, nullptr, points);
    ctx->launches += 3;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

static zim_status pack_ply_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, const uint8_t* gray,
                                  int with_gray, int rows, int cols, void* records, uint64_t* count_dev,
                                  cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    int nb = (int)((n + CB - 1) / CB);
    uint32_t* counts = (uint32_t*)zim_scratch_take(ctx, (size_t)nb * 4);
    if (!counts) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "compaction scratch");
    compact_count_kernel<<<nb, CB, 0, st>>>(mask, n, counts);
    compact_scan_kernel<<<1, 1024, 0, st>>>(counts, nb, count_dev);
    if (with_gray)
        compact_write_kernel<EMIT_PLY_XYZ_GRAY><<<nb, CB, 0, st>>>(xyz, mask, n, counts, gray, records);
    else
        compact_write_kernel<EMIT_PLY_XYZ><<<nb, CB, 0, st>>>(xyz, mask, n, counts, nullptr, records);
    ctx->launches += 3;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_ray_model zim_rays_of(const zim_ctx* ctx, bool rectified_coords, int ox, int oy) {
    if (!ctx->calibrated) return zim_ray_model{};
    return zim_rays_from(ctx->Q, ctx->R1, rectified_coords, ox, oy);
}

zim_ray_model zim_rays_from(const double* Q, const double* R1, bool rectified_coords, int ox, int oy) {
    zim_ray_model r;
    if (!(Q[11] != 0.0)) return r;
    // Q reprojects pixel (u, v) along (u + Q03, v + Q13, Q23)
    r.cx = (float)-Q[3];
    r.cy = (float)-Q[7];
    r.f = (float)Q[11];
    if (!rectified_coords)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) r.R[3 * a + b] = (float)R1[3 * b + a];  // R1^T
    r.ox = ox;
    r.oy = oy;
    r.valid = 1;
    return r;
}

zim_status zim_check_reproject(zim_ctx* ctx, const zim_recon_config* cfg) {
    if (cfg->reproject_model != 0 && cfg->reproject_model != 1)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "reproject_model must be 0 (Q) or 1 (polynomial maps)");
    // startCalculate_v2 writes no point without V2 coefficients (V2.cpp:505-548)
    if (cfg->reproject_model == 1 && !ctx->d_poly[0])
        return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "reproject_model 1 needs zim_set_poly_calib");
    return ZIM_OK;
}

static zim_status check_cloud(zim_ctx* ctx, const void* a, const void* b, const void* c, int rows, int cols) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!a || !b || !c) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows <= 0 || cols <= 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad size");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_median_reproject(zim_ctx* ctx, const zim_recon_config* cfg, const float* disp,
                                                   int rows, int cols, float* disp_out, float* xyz, uint8_t* mask,
                                                   void* stream) {
    zim_status s = check_cloud(ctx, disp, xyz, mask, rows, cols);
    if (s) return s;
    if (!cfg) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null config");
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    s = zim_check_reproject(ctx, cfg);
    if (s) return s;
    if (cfg->reproject_model == 1 && (rows != ctx->poly_h || cols != ctx->poly_w))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "disparity %dx%d differs from the coefficient maps %dx%d", cols, rows,
                        ctx->poly_w, ctx->poly_h);
    return zim_median_reproject_launch(ctx, cfg, disp, rows, cols, disp_out, xyz, mask, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_filter_px_gaussian(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                                     int cols, float* out, uint8_t* mask_out, void* stream) {
    zim_status s = check_cloud(ctx, xyz, mask, out, rows, cols);
    if (s) return s;
    return zim_px_gaussian_launch(ctx, xyz, mask, rows, cols, out, mask_out, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_filter_ror(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                             float radius, int min_neighbors, int window_size, float* out,
                                             uint8_t* mask_out, void* stream) {
    zim_status s = check_cloud(ctx, xyz, mask, out, rows, cols);
    if (s) return s;
    if (!mask_out || window_size < 0 || window_size > ZIM_MAX_ROR_WINDOW || min_neighbors < 0)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad ROR argument");
    return zim_ror_launch(ctx, xyz, mask, rows, cols, radius, min_neighbors, window_size, out, mask_out,
                          zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_compact_points(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                                 int cols, zim_point_xyz* points, uint64_t* count_dev, void* stream) {
    zim_status s = check_cloud(ctx, xyz, mask, points, rows, cols);
    if (s) return s;
    if (!count_dev) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null count");
    size_t nb = ((size_t)rows * cols + CB - 1) / CB;
    s = zim_scratch_reserve(ctx, nb * 4 + 256);
    if (s) return s;
    zim_scratch_reset(ctx);
    return zim_compact_launch(ctx, xyz, mask, rows, cols, points, count_dev, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_pack_ply(zim_ctx* ctx, const float* xyz, const uint8_t* mask, const uint8_t* gray,
                                           int with_gray, int rows, int cols, void* records, uint64_t* count_dev,
                                           void* stream) {
    zim_status s = check_cloud(ctx, xyz, mask, records, rows, cols);
    if (s) return s;
    if (!count_dev) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null count");
    size_t nb = ((size_t)rows * cols + CB - 1) / CB;
    s = zim_scratch_reserve(ctx, nb * 4 + 256);
    if (s) return s;
    zim_scratch_reset(ctx);
    return pack_ply_launch(ctx, xyz, mask, gray, with_gray, rows, cols, records, count_dev, zim_stream(stream));
}
