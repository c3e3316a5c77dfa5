// match.cu -- row-wise order-constrained absolute-phase matching with
// three-point sub-pixel refinement.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:933-1006
// (stereoMatch) and the GPU span-table variant
// JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:18-113.
//
// One CTA per rectified row.  The right row (order, phase base, residual) is
// staged in shared memory; the per-order column span [lo, hi] is built with
// shared-memory atomics and checked for a strictly rising phase; each left
// pixel of order k in [1, pha_f] finds the first column of minimum
// |phase_R - phase_L| among the right pixels of order k (strict <, so the
// smallest column wins ties) -- by binary search on a checked span, by a scan
// of the span otherwise, the same column either way -- rejects
// min >= grad_threshold and columns < 2 or >= cols - 1, then refines with the
// parabola through the costs of columns best-1, best, best+1.
#include <climits>

#include "zim_tiles.cuh"

namespace {

constexpr int MATCH_THREADS = 256;

// Left and right windows of one launch.  The whole-frame match uses the full
// rows of both images; the ROI match a left rectangle and a right column
// window over the same rectified rows, and an optional left mask.
struct MatchWin {
    const int32_t* l_base; const float* l_res; const int32_t* l_order;  // at the left window's origin
    const int32_t* r_base; const float* r_res; const int32_t* r_order;  // at the right window's origin
    const uint8_t* l_mask;  // at the left window's origin, or null
    size_t stride;          // elements per image row
    int l_cols, r_cols;     // window widths
    int dx_off;             // left window x - right window x
    float* disp;            // l_cols per row, row pitch out_stride
    int32_t* best_col;
    size_t out_stride;
};

__global__ void __launch_bounds__(MATCH_THREADS) match_kernel(MatchWin w, int pha_f, float grad_threshold) {
    extern __shared__ int4 smem_raw[];
    const int cols = w.r_cols;
    int* s_ord = reinterpret_cast<int*>(smem_raw);
    int* s_base = s_ord + cols;
    float* s_res = reinterpret_cast<float*>(s_base + cols);
    int* s_lo = reinterpret_cast<int*>(s_res + cols);
    int* s_hi = s_lo + (pha_f + 1);
    int* s_bad = s_hi + (pha_f + 1);

    const int row = blockIdx.x;
    const size_t ro = (size_t)row * w.stride;
    for (int k = threadIdx.x; k <= pha_f; k += blockDim.x) {
        s_lo[k] = INT_MAX;
        s_hi[k] = -1;
        s_bad[k] = 0;
    }
    for (int j = threadIdx.x; j < cols; j += blockDim.x) {
        s_ord[j] = w.r_order[ro + j];
        s_base[j] = w.r_base[ro + j];
        s_res[j] = w.r_res[ro + j];
    }
    __syncthreads();
    zt::match_spans(s_ord, cols, pha_f, s_lo, s_hi, threadIdx.x, blockDim.x);
    __syncthreads();
    zt::match_spans_check(s_ord, s_base, s_res, cols, pha_f, s_hi, s_bad, threadIdx.x, blockDim.x);
    __syncthreads();
    const size_t oo = (size_t)row * w.out_stride;
    for (int j = threadIdx.x; j < w.l_cols; j += blockDim.x) {
        float d = 0.f;
        int best = -1;
        if (!w.l_mask || w.l_mask[ro + j])
            zt::match_pixel(j, w.l_order[ro + j], w.l_base[ro + j], w.l_res[ro + j], s_ord, s_base, s_res, s_lo,
                            s_hi, s_bad, cols, pha_f, grad_threshold, d, best, w.dx_off);
        w.disp[oo + j] = d;
        if (w.best_col) w.best_col[oo + j] = best;
    }
}

zim_status launch_match(zim_ctx* ctx, const MatchWin& w, int rows, int pha_f, double grad_threshold,
                        cudaStream_t st) {
    size_t smem = (size_t)w.r_cols * 12 + (size_t)(pha_f + 1) * 12;
    // the attribute is per device and per function: set it on every call
    ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(match_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    match_kernel<<<rows, MATCH_THREADS, smem, st>>>(w, pha_f, (float)grad_threshold);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

// Rectification fused into matching (the plain whole-pair path): one CTA per
// rectified row rectifies the right row straight into shared memory and each
// left pixel in registers (the setData remap, zt::rectify_pixel[_smoothed], so
// the results are those of rectify + match), and the rectified maps never
// reach global memory.  post_smooth 1 / 2: sk / sr hold the post-smoothed taps
// of each camera (smooth_kernel); 0 / 3: the remap reads order / residual.
struct RectMatchArgs {
    const int32_t* order[2];
    const float* res[2];
    const int32_t* sk[2];
    const float* sr[2];
    const float* map[2][2];
    int srows, scols, rows, cols, post_smooth;
    float* disp;
};

__device__ __forceinline__ void rect_px(const RectMatchArgs& a, int cam, float mx, float my, int32_t& b, float& r,
                                        int32_t& k) {
    if (a.post_smooth == 1 || a.post_smooth == 2)
        zt::rectify_pixel_smoothed(a.sk[cam], a.sr[cam], a.order[cam], a.srows, a.scols, mx, my, b, r, k);
    else
        zt::rectify_pixel(a.order[cam], a.res[cam], a.srows, a.scols, mx, my, a.post_smooth, b, r, k);
}

__global__ void __launch_bounds__(MATCH_THREADS) rectify_match_kernel(RectMatchArgs a, int pha_f,
                                                                      float grad_threshold) {
    extern __shared__ int4 smem_raw[];
    const int cols = a.cols;
    int* s_ord = reinterpret_cast<int*>(smem_raw);
    int* s_base = s_ord + cols;
    float* s_res = reinterpret_cast<float*>(s_base + cols);
    int* s_lo = reinterpret_cast<int*>(s_res + cols);
    int* s_hi = s_lo + (pha_f + 1);
    int* s_bad = s_hi + (pha_f + 1);
    const int row = blockIdx.x;
    const size_t ro = (size_t)row * cols;
    for (int k = threadIdx.x; k <= pha_f; k += blockDim.x) {
        s_lo[k] = INT_MAX;
        s_hi[k] = -1;
        s_bad[k] = 0;
    }
    // each column's map entry is loaded one iteration ahead, so that its
    // latency overlaps the previous column's tap gathers
    const float* mxr = a.map[1][0] + ro;
    const float* myr = a.map[1][1] + ro;
    int j = threadIdx.x;
    float mx = 0.f, my = 0.f;
    if (j < cols) { mx = __ldg(mxr + j); my = __ldg(myr + j); }
    for (; j < cols; j += blockDim.x) {
        const int jn = j + blockDim.x;
        float nx = 0.f, ny = 0.f;
        if (jn < cols) { nx = __ldg(mxr + jn); ny = __ldg(myr + jn); }
        int32_t b, k;
        float r;
        rect_px(a, 1, mx, my, b, r, k);
        s_ord[j] = k;
        s_base[j] = b;
        s_res[j] = r;
        mx = nx;
        my = ny;
    }
    // the left row's first map entries, in flight across the barriers
    const float* mxl = a.map[0][0] + ro;
    const float* myl = a.map[0][1] + ro;
    j = threadIdx.x;
    if (j < cols) { mx = __ldg(mxl + j); my = __ldg(myl + j); }
    __syncthreads();
    zt::match_spans(s_ord, cols, pha_f, s_lo, s_hi, threadIdx.x, blockDim.x);
    __syncthreads();
    zt::match_spans_check(s_ord, s_base, s_res, cols, pha_f, s_hi, s_bad, threadIdx.x, blockDim.x);
    __syncthreads();
    for (; j < cols; j += blockDim.x) {
        const int jn = j + blockDim.x;
        float nx = 0.f, ny = 0.f;
        if (jn < cols) { nx = __ldg(mxl + jn); ny = __ldg(myl + jn); }
        int32_t bL, kL;
        float rL;
        rect_px(a, 0, mx, my, bL, rL, kL);
        mx = nx;
        my = ny;
        float d;
        int best;
        zt::match_pixel(j, kL, bL, rL, s_ord, s_base, s_res, s_lo, s_hi, s_bad, cols, pha_f, grad_threshold, d,
                        best);
        a.disp[ro + j] = d;
    }
}

}  // namespace

// The plain path's rectify + match of both cameras (see rectify_match_kernel);
// sk / sr: per camera the post-smoothed taps (post_smooth 1 or 2), else null.
zim_status zim_rectify_match_launch(zim_ctx* ctx, const int32_t* const order[2], const float* const res[2],
                                    int32_t* const sk[2], float* const sr[2], int srows, int scols, int post_smooth,
                                    int pha_f, double grad_threshold, float* disp, cudaStream_t st) {
    RectMatchArgs a{};
    for (int c = 0; c < 2; c++) {
        a.order[c] = order[c];
        a.res[c] = res[c];
        a.sk[c] = sk[c];
        a.sr[c] = sr[c];
        a.map[c][0] = ctx->d_map[c][0];
        a.map[c][1] = ctx->d_map[c][1];
    }
    a.srows = srows;
    a.scols = scols;
    a.rows = ctx->rect_h;
    a.cols = ctx->rect_w;
    a.post_smooth = post_smooth;
    a.disp = disp;
    if (a.cols > ZIM_MAX_MATCH_COLS)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "rectified width %d above %d", a.cols, ZIM_MAX_MATCH_COLS);
    const size_t smem = (size_t)a.cols * 12 + (size_t)(pha_f + 1) * 12;
    ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(rectify_match_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    rectify_match_kernel<<<a.rows, MATCH_THREADS, smem, st>>>(a, pha_f, (float)grad_threshold);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_match_launch(zim_ctx* ctx, const int32_t* l_base, const float* l_res, const int32_t* l_order,
                            const int32_t* r_base, const float* r_res, const int32_t* r_order, int rows, int cols,
                            int pha_f, double grad_threshold, float* disp, int32_t* best_col, cudaStream_t st) {
    MatchWin w{l_base, l_res, l_order, r_base, r_res, r_order, nullptr, (size_t)cols, cols, cols, 0, disp,
               best_col, (size_t)cols};
    return launch_match(ctx, w, rows, pha_f, grad_threshold, st);
}

// ROI matching (startCalculate_v2_roi, V2.cpp:719-778): left rectangle lx, ly,
// lw, lh with the left mask, right columns [rx, rx + rw) of the same rows;
// disp / best_col are lw x lh.
zim_status zim_match_roi_launch(zim_ctx* ctx, const int32_t* l_base, const float* l_res, const int32_t* l_order,
                                const int32_t* r_base, const float* r_res, const int32_t* r_order,
                                const uint8_t* l_mask, int cols, int lx, int ly, int lw, int lh, int rx, int rw,
                                int pha_f, double grad_threshold, float* disp, int32_t* best_col, cudaStream_t st) {
    const size_t lo = (size_t)ly * cols + lx, ro = (size_t)ly * cols + rx;
    MatchWin w{l_base + lo, l_res + lo, l_order + lo, r_base + ro, r_res + ro, r_order + ro,
               l_mask ? l_mask + lo : nullptr, (size_t)cols, lw, rw, lx - rx, disp, best_col, (size_t)lw};
    return launch_match(ctx, w, lh, pha_f, grad_threshold, st);
}

extern "C" ZIM_API zim_status zim_match(zim_ctx* ctx, const int32_t* l_base, const float* l_res,
                                        const int32_t* l_order, const int32_t* r_base, const float* r_res,
                                        const int32_t* r_order, int rows, int cols, int pha_f, double grad_threshold,
                                        float* disp, int32_t* best_col, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!l_base || !l_res || !l_order || !r_base || !r_res || !r_order || !disp)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows <= 0 || cols <= 0 || cols > ZIM_MAX_MATCH_COLS)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "cols must be in [1, %d]", ZIM_MAX_MATCH_COLS);
    if (pha_f < 0 || pha_f > ZIM_MAX_ORDER) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pha_f out of range");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return zim_match_launch(ctx, l_base, l_res, l_order, r_base, r_res, r_order, rows, cols, pha_f, grad_threshold,
                            disp, best_col, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_rectify_match(zim_ctx* ctx, const int32_t* l_order, const float* l_res,
                                                const int32_t* r_order, const float* r_res, int rows, int cols,
                                                int post_smooth, int pha_f, double grad_threshold, float* disp,
                                                void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    if (!l_order || !l_res || !r_order || !r_res || !disp) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "image size differs from calibration");
    if (post_smooth < 0 || post_smooth > 3) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "post_smooth must be 0..3");
    if (pha_f < 0 || pha_f > ZIM_MAX_ORDER) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pha_f out of range");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int32_t* sk[2] = {nullptr, nullptr};
    float* sr[2] = {nullptr, nullptr};
    cudaStream_t st = zim_stream(stream);
    const int32_t* ord[2] = {l_order, r_order};
    const float* res[2] = {l_res, r_res};
    if (post_smooth == 1 || post_smooth == 2) {
        const size_t src = (size_t)rows * cols;
        zim_status s = zim_scratch_reserve(ctx, 4 * zim_align256(src * 4) + 1024);
        if (s) return s;
        zim_scratch_reset(ctx);
        for (int c = 0; c < 2; c++) {
            sk[c] = (int32_t*)zim_scratch_take(ctx, src * 4);
            sr[c] = (float*)zim_scratch_take(ctx, src * 4);
            if (!sk[c] || !sr[c]) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "rectify scratch");
            s = zim_smooth_launch(ctx, ord[c], res[c], rows, cols, post_smooth, sk[c], sr[c], st);
            if (s) return s;
        }
    }
    return zim_rectify_match_launch(ctx, ord, res, sk, sr, rows, cols, post_smooth, pha_f, grad_threshold, disp, st);
}
