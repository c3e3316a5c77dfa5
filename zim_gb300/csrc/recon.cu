// recon.cu -- disparity median + Q reprojection, the reference's pixel-window
// point-cloud filters (3x3 Gaussian, radius outlier) and PointXYZ compaction.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp
//   medianBlur(5) :405-410, reprojection :414-461, Gaussian :79-124, ROR :126-195;
//   GPU port JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:119-347.
#include <cmath>

#include "zim_internal.cuh"

namespace {

constexpr int RX = 32, RY = 8;

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

struct ReprojParams {
    float q03, q13, q23, q32, q33;
    double dq03, dq13, dq23, dq32, dq33;
    float r1[9];
    float min_depth, max_depth;
    double dmin_depth, dmax_depth;
    int use_rectified, use_median;
};

__global__ void __launch_bounds__(RX* RY) median_reproject_kernel(const float* __restrict__ disp, int rows, int cols,
                                                                  ReprojParams p, float* __restrict__ disp_out,
                                                                  float* __restrict__ xyz, uint8_t* __restrict__ mask) {
    __shared__ float tile[RY + 4][RX + 5];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * RX + tx, y = blockIdx.y * RY + ty;
    float d;
    if (p.use_median) {
        const int gx0 = blockIdx.x * RX - 2, gy0 = blockIdx.y * RY - 2;
        for (int h = ty * RX + tx; h < (RX + 4) * (RY + 4); h += RX * RY) {
            int hy = h / (RX + 4), hx = h - hy * (RX + 4);
            int gy = min(max(gy0 + hy, 0), rows - 1), gx = min(max(gx0 + hx, 0), cols - 1);
            tile[hy][hx] = __ldg(disp + (size_t)gy * cols + gx);
        }
        __syncthreads();
        float a[25];
#pragma unroll
        for (int dy = 0; dy < 5; dy++)
#pragma unroll
            for (int dx = 0; dx < 5; dx++) a[dy * 5 + dx] = tile[ty + dy][tx + dx];
        d = median25(a);
    } else {
        if (x >= cols || y >= rows) return;
        d = disp[(size_t)y * cols + x];
    }
    if (x >= cols || y >= rows) return;
    const size_t o = (size_t)y * cols + x;
    if (disp_out) disp_out[o] = d;
    float ox = 0.f, oy = 0.f, oz = 0.f;
    uint8_t m = 0;
    if (fabsf(d) >= 1e-5f) {
        float X, Y, Z;
        float w = fmaf(p.q32, d, p.q33);
        if (fabsf(w) < 1e-2f * (fabsf(p.q32 * d) + fabsf(p.q33))) {
            // near-zero disparity denominator: FP64 divide
            double wd = p.dq32 * (double)d + p.dq33;
            double iw = 1.0 / wd;
            X = (float)(((double)x + p.dq03) * iw);
            Y = (float)(((double)y + p.dq13) * iw);
            Z = (float)(p.dq23 * iw);
            double zz = p.dq23 * iw;
            if (p.use_rectified) {
                if (zz > p.dmin_depth && zz < p.dmax_depth) { ox = X; oy = Y; oz = Z; m = 1; }
            } else {
                double xx = ((double)x + p.dq03) * iw, yy = ((double)y + p.dq13) * iw;
                double rx = p.r1[0] * xx + p.r1[3] * yy + p.r1[6] * zz;
                double ry = p.r1[1] * xx + p.r1[4] * yy + p.r1[7] * zz;
                double rz = p.r1[2] * xx + p.r1[5] * yy + p.r1[8] * zz;
                if (rz > p.dmin_depth && rz < p.dmax_depth) { ox = (float)rx; oy = (float)ry; oz = (float)rz; m = 1; }
            }
        } else {
            float iw = 1.0f / w;
            X = ((float)x + p.q03) * iw;
            Y = ((float)y + p.q13) * iw;
            Z = p.q23 * iw;
            if (p.use_rectified) {
                if (Z > p.min_depth && Z < p.max_depth) { ox = X; oy = Y; oz = Z; m = 1; }
            } else {
                float rx = p.r1[0] * X + p.r1[3] * Y + p.r1[6] * Z;
                float ry = p.r1[1] * X + p.r1[4] * Y + p.r1[7] * Z;
                float rz = p.r1[2] * X + p.r1[5] * Y + p.r1[8] * Z;
                if (rz > p.min_depth && rz < p.max_depth) { ox = rx; oy = ry; oz = rz; m = 1; }
            }
        }
    }
    xyz[3 * o] = ox;
    xyz[3 * o + 1] = oy;
    xyz[3 * o + 2] = oz;
    mask[o] = m;
}

// 3x3 point-cloud Gaussian (sigma 0.7 px): neighbour used if valid and
// |x_n - x_c| < 3; output sum(w p) / sum(w) if sum(w) > 0.8, else 0; borders 0.
// The weighted mean is accumulated as p_c + sum(w (p_n - p_c)) / sum(w), the
// same value with millimetre-scale FP32 sums.
__global__ void px_gaussian_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                   float w00, float w01, float w11, float* __restrict__ out,
                                   uint8_t* __restrict__ mask_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= cols || y >= rows) return;
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

__global__ void ror_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                           float r2, int min_nb, int hw, float* __restrict__ out, uint8_t* __restrict__ mask_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= cols || y >= rows) return;
    size_t o = (size_t)y * cols + x;
    bool keep = false;
    float px = 0.f, py = 0.f, pz = 0.f;
    if (mask[o]) {
        keep = min_nb <= 0;
        px = xyz[3 * o]; py = xyz[3 * o + 1]; pz = xyz[3 * o + 2];
        int cnt = 0;
        int r0 = max(0, y - hw), r1 = min(rows, y + hw + 1), c0 = max(0, x - hw), c1 = min(cols, x + hw + 1);
        for (int i = r0; i < r1 && !keep; i++)
            for (int j = c0; j < c1; j++) {
                size_t q = (size_t)i * cols + j;
                if (q == o || !__ldg(mask + q)) continue;
                float dx = px - __ldg(xyz + 3 * q), dy = py - __ldg(xyz + 3 * q + 1), dz = pz - __ldg(xyz + 3 * q + 2);
                if (dx * dx + dy * dy + dz * dz <= r2) {
                    if (++cnt >= min_nb) { keep = true; break; }
                }
            }
    }
    out[3 * o] = keep ? px : 0.f;
    out[3 * o + 1] = keep ? py : 0.f;
    out[3 * o + 2] = keep ? pz : 0.f;
    mask_out[o] = keep ? 1 : 0;
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

__global__ void compact_write_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                     const uint32_t* __restrict__ offsets, zim_point_xyz* __restrict__ pts) {
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
    if (v) {
        uint32_t pos = offsets[blockIdx.x] + warp_off[w] + __popc(b & ((1u << lane) - 1u));
        zim_point_xyz p;
        p.x = xyz[3 * i];
        p.y = xyz[3 * i + 1];
        p.z = xyz[3 * i + 2];
        p.pad = 1.0f;
        pts[pos] = p;
    }
}

}  // namespace

zim_status zim_median_reproject_launch(zim_ctx* ctx, const zim_recon_config* cfg, const float* disp, int rows,
                                       int cols, float* disp_out, float* xyz, uint8_t* mask, cudaStream_t st) {
    ReprojParams p;
    const double* Q = ctx->Q;
    p.dq03 = Q[3]; p.dq13 = Q[7]; p.dq23 = Q[11]; p.dq32 = Q[14]; p.dq33 = Q[15];
    p.q03 = (float)Q[3]; p.q13 = (float)Q[7]; p.q23 = (float)Q[11]; p.q32 = (float)Q[14]; p.q33 = (float)Q[15];
    for (int i = 0; i < 9; i++) p.r1[i] = (float)ctx->R1[i];
    p.min_depth = (float)cfg->min_depth; p.max_depth = (float)cfg->max_depth;
    p.dmin_depth = cfg->min_depth; p.dmax_depth = cfg->max_depth;
    p.use_rectified = cfg->use_rectified_coords ? 1 : 0;
    p.use_median = cfg->use_disp_median_filter ? 1 : 0;
    dim3 blk(RX, RY), grd((cols + RX - 1) / RX, (rows + RY - 1) / RY);
    median_reproject_kernel<<<grd, blk, 0, st>>>(disp, rows, cols, p, disp_out, xyz, mask);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_px_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float* out,
                                  uint8_t* mask_out, cudaStream_t st) {
    // getGaussianKernel(3, 0.7, CV_32F), outer product in float
    double t = std::exp(-0.5 / (0.7 * 0.7));
    double mul = 1.0 / (2.0 * t + 1.0);
    float k0 = (float)(t * mul), k1 = (float)mul;
    dim3 blk(32, 8), grd((cols + 31) / 32, (rows + 7) / 8);
    px_gaussian_kernel<<<grd, blk, 0, st>>>(xyz, mask, rows, cols, k0 * k0, k0 * k1, k1 * k1, out, mask_out);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_ror_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float radius,
                          int min_neighbors, int window_size, float* out, uint8_t* mask_out, cudaStream_t st) {
    dim3 blk(32, 8), grd((cols + 31) / 32, (rows + 7) / 8);
    ror_kernel<<<grd, blk, 0, st>>>(xyz, mask, rows, cols, radius * radius, min_neighbors, window_size / 2, out,
                                    mask_out);
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
    compact_write_kernel<<<nb, CB, 0, st>>>(xyz, mask, n, counts, points);
    ctx->launches += 3;
    ZIM_LAUNCH_CHECK(ctx);
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
    if (!mask_out || window_size < 0 || window_size > 128 || min_neighbors < 0)
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
