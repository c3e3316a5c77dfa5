// roi.cu -- ROI-restricted reconstruction: prepareRectifiedROI and
// startCalculate_v2_roi (PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:595-914).
//
// Prepare (host + four small kernels, synchronising):
//   1. the rotated rectangle's corners (cv::RotatedRect::points, rounded to
//      integers) are rasterised on the host into one column span per source
//      row: the closed convex polygon plus its 8-connected outline
//      (cv::fillConvexPoly);
//   2. roi_mask_kernel remaps that source mask into the rectified frame with
//      the fixed-point INTER_LINEAR of an 8-bit image and thresholds > 0;
//   3. dilate5_kernel applies the 5x5 rectangular dilation and reduces the
//      bounding box of the result;
//   4. needed_orders_kernel marks the orders 1..pha_f present in the left ROI,
//      right_window_kernel finds the first and last right column (over the
//      ROI's rows) holding one of them; the host pads the window by 32 columns.
// Reconstruct: matching of the left rectangle against the right window, 5x5
// median of the ROI disparity, reprojection of the masked pixels (global
// coordinates for the maps), then the filter chain, with the reference's rule
// that keeps the pre-ROR cloud when ROR leaves fewer than a tenth of it.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "zim_tiles.cuh"

zim_status zim_match_roi_launch(zim_ctx* ctx, const int32_t* l_base, const float* l_res, const int32_t* l_order,
                                const int32_t* r_base, const float* r_res, const int32_t* r_order,
                                const uint8_t* l_mask, int cols, int lx, int ly, int lw, int lh, int rx, int rw,
                                int pha_f, double grad_threshold, float* disp, int32_t* best_col, cudaStream_t st);

namespace {

constexpr int ROI_PAD = 32;  // order_search_pad, V2.cpp:657

// ---------------------------------------------------------------- host ----

struct Pt { long long x, y; };

// cv::RotatedRect::points: corners from the centre, size and angle (degrees),
// single-precision like OpenCV's Point2f arithmetic.
void rotated_rect_points(const zim_rotated_rect& r, float px[4], float py[4]) {
    const double ang = (double)r.angle * 3.14159265358979323846 / 180.0;
    const float b = (float)std::cos(ang) * 0.5f, a = (float)std::sin(ang) * 0.5f;
    // every product and sum rounded to float on its own (no contraction)
    volatile float ah = a * r.height, bw = b * r.width, bh = b * r.height, aw = a * r.width;
    volatile float t;
    t = r.center_x - ah; px[0] = t - bw;
    t = r.center_y + bh; py[0] = t - aw;
    t = r.center_x + ah; px[1] = t - bw;
    t = r.center_y - bh; py[1] = t - aw;
    px[2] = 2 * r.center_x - px[0];
    py[2] = 2 * r.center_y - py[0];
    px[3] = 2 * r.center_x - px[1];
    py[3] = 2 * r.center_y - py[1];
}

long long floor_div(long long a, long long b) {  // b > 0
    return a >= 0 ? a / b : -((-a + b - 1) / b);
}

// Column span per source row of the filled polygon: pixels (x, y) inside or on
// the closed convex polygon, united with the pixels of its 8-connected outline
// (Bresenham).  lo > hi marks an empty row.
void polygon_spans(const Pt* v, int n, int rows, int cols, std::vector<int2>& span) {
    span.assign(rows, make_int2(INT_MAX, INT_MIN));
    auto add = [&](long long x, long long y) {
        if (y < 0 || y >= rows) return;
        int2& s = span[(size_t)y];
        s.x = (int)std::min<long long>(s.x, x);
        s.y = (int)std::max<long long>(s.y, x);
    };
    // interior rows: the horizontal line y meets the boundary in [xa, xb]
    long long ymin = LLONG_MAX, ymax = LLONG_MIN;
    for (int i = 0; i < n; i++) {
        ymin = std::min(ymin, v[i].y);
        ymax = std::max(ymax, v[i].y);
    }
    for (long long y = std::max(ymin, 0LL); y <= std::min(ymax, (long long)rows - 1); y++) {
        // Each crossing x gives ceil(x) and floor(x); their midpoint orders
        // crossings like x itself, so the leftmost crossing's ceil and the
        // rightmost crossing's floor bound the closed interior span.
        bool any = false;
        long long lo = 0, hi = 0;  // ceil(min x), floor(max x)
        double xmin = 0, xmax = 0;
        for (int i = 0; i < n; i++) {
            const Pt p = v[i], q = v[(i + 1) % n];
            if (y < std::min(p.y, q.y) || y > std::max(p.y, q.y)) continue;
            long long xl, xh;  // ceil and floor of the crossing
            if (p.y == q.y) {
                xl = std::min(p.x, q.x);
                xh = std::max(p.x, q.x);
            } else {
                // x = p.x + (y - p.y) (q.x - p.x) / (q.y - p.y)
                long long num = (y - p.y) * (q.x - p.x), den = q.y - p.y;
                if (den < 0) { num = -num; den = -den; }
                long long f = floor_div(num, den);
                xh = p.x + f;
                xl = p.x + (f * den == num ? f : f + 1);
            }
            const double xc = 0.5 * ((double)xl + (double)xh);
            if (!any || xc < xmin) { xmin = xc; lo = xl; }
            if (!any || xc > xmax) { xmax = xc; hi = xh; }
            any = true;
        }
        if (any && lo <= hi && hi >= 0 && lo < cols) {
            add(std::max(lo, 0LL), y);
            add(std::min(hi, (long long)cols - 1), y);
        }
    }
    // outline
    for (int i = 0; i < n; i++) {
        long long x0 = v[i].x, y0 = v[i].y;
        const long long x1 = v[(i + 1) % n].x, y1 = v[(i + 1) % n].y;
        const long long dx = std::llabs(x1 - x0), dy = -std::llabs(y1 - y0);
        const int sx = x0 < x1 ? 1 : -1, sy = y0 < y1 ? 1 : -1;
        long long err = dx + dy;
        for (;;) {
            if (x0 >= 0 && x0 < cols) add(x0, y0);
            if (x0 == x1 && y0 == y1) break;
            const long long e2 = 2 * err;
            if (e2 >= dy) { err += dy; x0 += sx; }
            if (e2 <= dx) { err += dx; y0 += sy; }
        }
    }
}

// -------------------------------------------------------------- kernels ----

// Thresholded INTER_LINEAR remap (8-bit fixed point) of the 0/255 source mask
// given by the row spans: 255 where (sum of inside weights x 255 + 2^14) >> 15 > 0.
__global__ void roi_mask_kernel(const int2* __restrict__ span, int srows, int scols, const float* __restrict__ mapx,
                                const float* __restrict__ mapy, int drows, int dcols, uint8_t* __restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= dcols || i >= drows) return;
    const size_t o = (size_t)i * dcols + j;
    int sx = __float2int_rn(mapx[o] * 32.0f), sy = __float2int_rn(mapy[o] * 32.0f);
    int x0 = sx >> 5, y0 = sy >> 5, fx = sx & 31, fy = sy & 31;
    int acc = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        int xx = x0 + (t & 1), yy = y0 + (t >> 1);
        if (xx < 0 || yy < 0 || xx >= scols || yy >= srows) continue;
        const int2 s = __ldg(span + yy);
        if (xx < s.x || xx > s.y) continue;
        acc += ((t >> 1) ? fy : 32 - fy) * ((t & 1) ? fx : 32 - fx) * 32 * 255;
    }
    out[o] = ((acc + (1 << 14)) >> 15) > 0 ? 255 : 0;
}

// 5x5 rectangular dilation (pixels outside the image do not contribute) and
// the bounding box of the result: bbox = {min x, min y, -max x, -max y}.
__global__ void dilate5_kernel(const uint8_t* __restrict__ in, int rows, int cols, uint8_t* __restrict__ out,
                               int* __restrict__ bbox) {
    int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    bool on = false;
    if (j < cols && i < rows) {
        for (int dy = -2; dy <= 2 && !on; dy++) {
            const int y = i + dy;
            if (y < 0 || y >= rows) continue;
            for (int dx = -2; dx <= 2; dx++) {
                const int x = j + dx;
                if (x >= 0 && x < cols && in[(size_t)y * cols + x]) {
                    on = true;
                    break;
                }
            }
        }
        out[(size_t)i * cols + j] = on ? 255 : 0;
    }
    int v[4] = {on ? j : INT_MAX, on ? i : INT_MAX, on ? -j : INT_MAX, on ? -i : INT_MAX};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int m = __reduce_min_sync(0xffffffffu, v[k]);
        if ((threadIdx.y * blockDim.x + threadIdx.x) % 32 == 0 && m != INT_MAX) atomicMin(bbox + k, m);
    }
}

// Orders 1..pha_f of the left rectified order map inside the ROI mask.
__global__ void needed_orders_kernel(const uint8_t* __restrict__ mask, const int32_t* __restrict__ l_order, int cols,
                                     int lx, int ly, int lw, int lh, int pha_f, uint8_t* __restrict__ needed) {
    int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= lw || i >= lh) return;
    const size_t o = (size_t)(ly + i) * cols + lx + j;
    if (!mask[o]) return;
    const int k = l_order[o];
    if (k > 0 && k <= pha_f) needed[k] = 1;
}

// First and last right column, over rows [ly, ly + lh), whose order is needed:
// win = {min x, -max x}.
__global__ void right_window_kernel(const int32_t* __restrict__ r_order, int cols, int ly, int lh, int pha_f,
                                    const uint8_t* __restrict__ needed, int* __restrict__ win) {
    int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    bool hit = false;
    if (j < cols && i < lh) {
        const int k = r_order[(size_t)(ly + i) * cols + j];
        hit = k > 0 && k <= pha_f && needed[k];
    }
    int a = __reduce_min_sync(0xffffffffu, hit ? j : INT_MAX);
    int b = __reduce_min_sync(0xffffffffu, hit ? -j : INT_MAX);
    if ((threadIdx.y * blockDim.x + threadIdx.x) % 32 == 0) {
        if (a != INT_MAX) atomicMin(win, a);
        if (b != INT_MAX) atomicMin(win + 1, b);
    }
}

// Valid-point counts of two masks (cnt[0] += mask a, cnt[1] += mask b).
__global__ void count2_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, size_t n,
                              unsigned long long* __restrict__ cnt) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned ca = __popc(__ballot_sync(0xffffffffu, i < n && a[i]));
    unsigned cb = __popc(__ballot_sync(0xffffffffu, i < n && b[i]));
    if ((threadIdx.x & 31) == 0) {
        if (ca) atomicAdd(cnt, (unsigned long long)ca);
        if (cb) atomicAdd(cnt + 1, (unsigned long long)cb);
    }
}

// The reference keeps the pre-ROR cloud (Gaussian output, pre-ROR mask) when
// ROR leaves fewer than a tenth of the raw points (V2.cpp:873-882).
__global__ void ror_select_kernel(const unsigned long long* __restrict__ cnt, size_t n, const float* __restrict__ x_pre,
                                  const uint8_t* __restrict__ m_pre, const float* __restrict__ x_ror,
                                  const uint8_t* __restrict__ m_ror, float* __restrict__ x_out,
                                  uint8_t* __restrict__ m_out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long raw = cnt[0], kept = cnt[1];
    const bool pre = raw > 0 && (double)kept < (double)raw * 0.1;
    const float* x = pre ? x_pre : x_ror;
    x_out[3 * i] = x[3 * i];
    x_out[3 * i + 1] = x[3 * i + 1];
    x_out[3 * i + 2] = x[3 * i + 2];
    m_out[i] = pre ? m_pre[i] : m_ror[i];
}

__global__ void roi_reproject_kernel(const float* __restrict__ disp, int rows, int cols, zt::ReprojParams p,
                                     float* __restrict__ disp_out, float* __restrict__ xyz,
                                     uint8_t* __restrict__ mask) {
    __shared__ zt::MedianSmem sm;
    zt::median_reproject_tile(disp, rows, cols, p, blockIdx.x, blockIdx.y, threadIdx.y * zt::RX + threadIdx.x, sm,
                              disp_out, xyz, mask);
}

}  // namespace

extern "C" ZIM_API zim_status zim_prepare_roi(zim_ctx* ctx, const zim_rotated_rect* roi, const int32_t* l_order,
                                              const int32_t* r_order, int pha_f, zim_rectified_roi* out,
                                              uint8_t* roi_mask, int* valid, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!roi || !l_order || !r_order || !out || !roi_mask || !valid)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    if (pha_f < 0 || pha_f > ZIM_MAX_ORDER) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pha_f out of range");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    *valid = 0;
    *out = zim_rectified_roi{};
    const int SH = ctx->src_h, SW = ctx->src_w, RH = ctx->rect_h, RW = ctx->rect_w;
    cudaStream_t st = zim_stream(stream);

    float px[4], py[4];
    rotated_rect_points(*roi, px, py);
    Pt v[4];
    for (int i = 0; i < 4; i++) v[i] = Pt{(long long)std::nearbyint(px[i]), (long long)std::nearbyint(py[i])};
    std::vector<int2> span;
    polygon_spans(v, 4, SH, SW, span);

    const size_t n = (size_t)RH * RW;
    zim_status s = zim_scratch_reserve(ctx, zim_align256((size_t)SH * 8) + zim_align256(n) + 1024 +
                                                zim_align256((size_t)pha_f + 1) + 256);
    if (s) return s;
    zim_scratch_reset(ctx);
    int2* d_span = (int2*)zim_scratch_take(ctx, (size_t)SH * 8);
    uint8_t* lin = (uint8_t*)zim_scratch_take(ctx, n);
    int* d_box = (int*)zim_scratch_take(ctx, 64);
    uint8_t* needed = (uint8_t*)zim_scratch_take(ctx, (size_t)pha_f + 1);
    if (!d_span || !lin || !d_box || !needed) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "roi scratch");
    int* h = (int*)ctx->h_pinned;  // 6 ints: bbox + window
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(d_span, span.data(), (size_t)SH * 8, cudaMemcpyHostToDevice, st));
    const int init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX, INT_MAX, INT_MAX};
    std::memcpy(h, init, sizeof init);
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(d_box, h, sizeof init, cudaMemcpyHostToDevice, st));
    ZIM_CUDA_TRY(ctx, cudaMemsetAsync(needed, 0, (size_t)pha_f + 1, st));
    dim3 blk(32, 8), grd((RW + 31) / 32, (RH + 7) / 8);
    roi_mask_kernel<<<grd, blk, 0, st>>>(d_span, SH, SW, ctx->d_map[0][0], ctx->d_map[0][1], RH, RW, lin);
    dilate5_kernel<<<grd, blk, 0, st>>>(lin, RH, RW, roi_mask, d_box);
    ctx->launches += 2;
    ZIM_LAUNCH_CHECK(ctx);
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(h, d_box, 16, cudaMemcpyDeviceToHost, st));
    ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (h[0] == INT_MAX) return ZIM_OK;  // empty mask
    zim_rect L{h[0], h[1], -h[2] - h[0] + 1, -h[3] - h[1] + 1};
    dim3 lgrd((L.width + 31) / 32, (L.height + 7) / 8), rgrd((RW + 31) / 32, (L.height + 7) / 8);
    needed_orders_kernel<<<lgrd, blk, 0, st>>>(roi_mask, l_order, RW, L.x, L.y, L.width, L.height, pha_f, needed);
    right_window_kernel<<<rgrd, blk, 0, st>>>(r_order, RW, L.y, L.height, pha_f, needed, d_box + 4);
    ctx->launches += 2;
    ZIM_LAUNCH_CHECK(ctx);
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(h + 4, d_box + 4, 8, cudaMemcpyDeviceToHost, st));
    ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    zim_rect R;
    if (h[4] != INT_MAX) {
        const int x0 = std::max(0, h[4] - ROI_PAD), x1 = std::min(RW - 1, -h[5] + ROI_PAD);
        R = zim_rect{x0, L.y, x1 - x0 + 1, L.height};
    } else {
        R = zim_rect{0, L.y, RW, L.height};  // no needed order on the right: whole rows
    }
    out->left_rect = L;
    out->right_rect = R;
    *valid = 1;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_roi_source_spans(const zim_rotated_rect* roi, int rows, int cols, int* lo,
                                                   int* hi) {
    if (!roi || !lo || !hi || rows <= 0 || cols <= 0) return ZIM_ERR_INVALID_ARG;
    float px[4], py[4];
    rotated_rect_points(*roi, px, py);
    Pt v[4];
    for (int i = 0; i < 4; i++) v[i] = Pt{(long long)std::nearbyint(px[i]), (long long)std::nearbyint(py[i])};
    std::vector<int2> span;
    polygon_spans(v, 4, rows, cols, span);
    for (int y = 0; y < rows; y++) {
        lo[y] = span[y].x;
        hi[y] = span[y].y;
    }
    return ZIM_OK;
}

static bool rect_in(const zim_rect& r, int w, int h) {
    return r.width > 0 && r.height > 0 && r.x >= 0 && r.y >= 0 && r.x + r.width <= w && r.y + r.height <= h;
}

extern "C" ZIM_API zim_status zim_reconstruct_roi(zim_ctx* ctx, const zim_recon_config* r, const zim_rectified_roi* roi,
                                                  const uint8_t* roi_mask, const int32_t* l_base, const float* l_res,
                                                  const int32_t* l_order, const int32_t* r_base, const float* r_res,
                                                  const int32_t* r_order, int pha_f, float* xyz, uint8_t* mask,
                                                  float* disp, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!r || !roi || !roi_mask || !l_base || !l_res || !l_order || !r_base || !r_res || !r_order || !xyz || !mask)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    zim_status s = zim_check_reproject(ctx, r);
    if (s) return s;
    const int RH = ctx->rect_h, RW = ctx->rect_w;
    const zim_rect L = roi->left_rect, R = roi->right_rect;
    if (!rect_in(L, RW, RH) || !rect_in(R, RW, RH) || R.y != L.y || R.height != L.height)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "ROI rectangles outside the rectified frame or on other rows");
    if (R.width > ZIM_MAX_MATCH_COLS) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "right window too wide");
    if (pha_f < 0 || pha_f > ZIM_MAX_ORDER) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pha_f out of range");
    if (r->use_mls && (r->mls_window_size < 0 || r->mls_window_size > 64))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "mls_window_size out of range");
    if (r->use_ror && (r->radius_window_size < 0 || r->radius_window_size > ZIM_MAX_ROR_WINDOW))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "radius_window_size must be in [0, %d]", ZIM_MAX_ROR_WINDOW);
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = zim_stream(stream);
    const int H = L.height, W = L.width;
    const size_t n = (size_t)H * W;
    size_t need = 2 * zim_align256(n * 4) + 3 * (zim_align256(n * 12) + zim_align256(n)) + 512;
    if (r->use_mls) need += zim_align256(n * 12);
    if (r->use_sor || r->use_metric_gaussian) need += zim_grid_scratch_bytes(n);
    s = zim_scratch_reserve(ctx, need + 4096);
    if (s) return s;
    zim_scratch_reset(ctx);
    float* d_raw = (float*)zim_scratch_take(ctx, n * 4);
    float* d_med = disp ? disp : (float*)zim_scratch_take(ctx, n * 4);
    float* xb[3];
    uint8_t* mb[3];
    for (int k = 0; k < 3; k++) {
        xb[k] = (float*)zim_scratch_take(ctx, n * 12);
        mb[k] = (uint8_t*)zim_scratch_take(ctx, n);
    }
    unsigned long long* cnt = (unsigned long long*)zim_scratch_take(ctx, 16);
    float* mls_tmp = r->use_mls ? (float*)zim_scratch_take(ctx, n * 12) : nullptr;
    if (!d_raw || !d_med || !xb[2] || !mb[2] || !cnt || (r->use_mls && !mls_tmp))
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "roi scratch");
    const size_t grid_mark = ctx->scratch_used;

    s = zim_match_roi_launch(ctx, l_base, l_res, l_order, r_base, r_res, r_order, roi_mask, RW, L.x, L.y, W, H, R.x,
                             R.width, pha_f, r->grad_threshold, d_raw, nullptr, st);
    if (s) return s;

    zt::ReprojParams p;
    zt::reproj_params(ctx->Q, ctx->R1, r, p);
    for (int k = 0; k < 3; k++) p.poly[k] = ctx->d_poly[k];
    p.ox = L.x;
    p.oy = L.y;
    p.gstride = RW;
    p.roi_mask = roi_mask;
    dim3 blk(zt::RX, zt::RY), grd((W + zt::MTX - 1) / zt::MTX, (H + zt::RY - 1) / zt::RY);
    roi_reproject_kernel<<<grd, blk, 0, st>>>(d_raw, H, W, p, d_med, xb[0], mb[0]);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);

    // the chain on the ROI cloud: xb[0]/mb[0] raw, then ping-pong through xb[1..2]
    const float* cx = xb[0];
    const uint8_t* cm = mb[0];
    if (r->use_px_gaussian) {
        s = zim_px_gaussian_launch(ctx, cx, cm, H, W, xb[1], r->px_gaussian_updates_mask ? mb[1] : nullptr, st);
        if (s) return s;
        cx = xb[1];
        if (r->px_gaussian_updates_mask) cm = mb[1];
    }
    if (r->use_ror) {
        float* xr = cx == xb[1] ? xb[2] : xb[1];
        uint8_t* mr = cm == mb[1] ? mb[2] : mb[1];
        s = zim_ror_launch(ctx, cx, cm, H, W, r->radius_search, r->radius_min_neighbors, r->radius_window_size, xr, mr,
                           st);
        if (s) return s;
        // select into the buffers neither input uses
        float* xs = (xb[0] != cx && xb[0] != xr) ? xb[0] : (xb[1] != cx && xb[1] != xr) ? xb[1] : xb[2];
        uint8_t* ms = (mb[0] != cm && mb[0] != mr) ? mb[0] : (mb[1] != cm && mb[1] != mr) ? mb[1] : mb[2];
        ZIM_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, 16, st));
        // raw count: the reprojection mask (P_raw)
        count2_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(mb[0], mr, n, cnt);
        ror_select_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cnt, n, cx, cm, xr, mr, xs, ms);
        ctx->launches += 2;
        ZIM_LAUNCH_CHECK(ctx);
        cx = xs;
        cm = ms;
    }
    if (r->use_sor) {
        float* xo = (xb[0] != cx) ? xb[0] : xb[1];
        uint8_t* mo = (mb[0] != cm) ? mb[0] : mb[1];
        s = zim_sor_launch(ctx, cx, cm, H, W, r->sor_mean_k, r->sor_std_mul, xo, mo, nullptr,
                           zim_rays_of(ctx, r->use_rectified_coords != 0, L.x, L.y), st);
        if (s) return s;
        ctx->scratch_used = grid_mark;
        cx = xo;
        cm = mo;
    }
    if (r->use_mls) {
        float* xo = (xb[0] != cx) ? xb[0] : xb[1];
        s = zim_mls_launch(ctx, cx, cm, H, W, r->mls_window_size, r->mls_spatial_sigma, r->mls_polynomial_order,
                           r->mls_max_radius, r->mls_iterations, xo, mls_tmp,
                           zim_rays_of(ctx, r->use_rectified_coords != 0, L.x, L.y), st);
        if (s) return s;
        cx = xo;
    }
    if (r->use_metric_gaussian) {
        float* xo = (xb[0] != cx) ? xb[0] : xb[1];
        s = zim_metric_gaussian_launch(ctx, cx, cm, H, W, r->metric_gaussian_sigma, xo,
                                       zim_rays_of(ctx, r->use_rectified_coords != 0, L.x, L.y), st);
        if (s) return s;
        ctx->scratch_used = grid_mark;
        cx = xo;
    }
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(xyz, cx, n * 12, cudaMemcpyDeviceToDevice, st));
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(mask, cm, n, cudaMemcpyDeviceToDevice, st));
    return ZIM_OK;
}
