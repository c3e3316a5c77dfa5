// ctx.cu -- context, errors, configuration defaults and validation, scratch
// arena, and the whole-pair pipeline of the zim_gb300 C ABI.
#include <cmath>
#include <cstring>
#include <vector>

#include "zim_internal.cuh"

zim_status zim_fail(zim_ctx* ctx, zim_status st, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return st;
}

extern "C" ZIM_API const char* zim_version(void) { return "zim_gb300 0.1.0 (sm_103a)"; }

extern "C" ZIM_API void zim_decode_config_default(zim_decode_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->freq[0] = 121; c->freq[1] = 110; c->freq[2] = 120;
    c->shift_num[0] = c->shift_num[1] = c->shift_num[2] = 8;
    c->modulation_threshold = 1.0;
    c->preblur_sigma = 3.0;
    c->avg_three_phase = 1;
    c->post_smooth = 1;
    c->enable_hdr = 0;
    c->hdr_saturation_gray = 255.0;
    c->hdr_min_amplitude = 2.0;
    c->encoding = ZIM_ENC_HETERODYNE3;
    c->n_freq = 3;
    c->gray_bits = 0;
}

extern "C" ZIM_API void zim_recon_config_default(zim_recon_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->min_depth = 0; c->max_depth = 1000;
    c->min_phase_diff = 0.03; c->max_phase_diff = 0.4;
    c->grad_threshold = 1.0;
    c->use_rectified_coords = 1;
    c->use_disp_median_filter = 1;
    c->use_full_left_rectification = 1;
    c->use_px_gaussian = 1;
    c->px_gaussian_updates_mask = 0;
    c->use_ror = 1;
    c->radius_search = 0.7f; c->radius_min_neighbors = 10; c->radius_window_size = 10;
    c->use_mls = 0; c->mls_window_size = 30; c->mls_spatial_sigma = 0.6f;
    c->mls_polynomial_order = 1; c->mls_max_radius = 0.0f; c->mls_iterations = 3;
    c->use_sor = 0; c->sor_mean_k = 50; c->sor_std_mul = 1.0;
    c->use_metric_gaussian = 0; c->metric_gaussian_sigma = 0.5;
}

static bool is_int(double v) { return std::isfinite(v) && v == std::floor(v); }

extern "C" ZIM_API zim_status zim_decode_validate(const zim_decode_config* c) {
    if (!c) return ZIM_ERR_INVALID_ARG;
    if (!(c->modulation_threshold >= 0) || !std::isfinite(c->preblur_sigma)) return ZIM_ERR_INVALID_ARG;
    if (c->enable_hdr) {
        // the reference fits HDR phase for its phase-shift frequencies only; Gray bits would threshold saturated frames
        if (c->encoding != ZIM_ENC_HETERODYNE3 && c->encoding != ZIM_ENC_HIERARCHICAL) return ZIM_ERR_UNSUPPORTED;
        if (!(c->hdr_saturation_gray > 0) || !(c->hdr_min_amplitude >= 0)) return ZIM_ERR_INVALID_ARG;
        for (int i = 0; i < (c->encoding == ZIM_ENC_HETERODYNE3 ? 3 : c->n_freq) && i < 4; i++)
            if (c->shift_num[i] > 12) return ZIM_ERR_INVALID_ARG;  // JSLAB_HDRPhaseFit: 3..12 steps
    }
    auto steps_ok = [](int n) { return n >= 3 && n <= 32; };
    switch (c->encoding) {
    case ZIM_ENC_HETERODYNE3: {
        // JSLAB_PhaseShiftDecoder::create returns nullptr unless all three are non-zero.
        if (c->freq[0] == 0 || c->freq[1] == 0 || c->freq[2] == 0) return ZIM_ERR_INVALID_ARG;
        for (int i = 0; i < 3; i++)
            if (!steps_ok(c->shift_num[i]) || !is_int(c->freq[i]) || c->freq[i] < 1 || c->freq[i] > ZIM_MAX_ORDER)
                return ZIM_ERR_INVALID_ARG;
        int f12 = std::abs((int)(c->freq[0] - c->freq[1])), f23 = std::abs((int)(c->freq[1] - c->freq[2]));
        if (f12 == 0 || f23 == 0) return ZIM_ERR_INVALID_ARG;
        break;
    }
    case ZIM_ENC_HIERARCHICAL: {
        if (c->n_freq < 2 || c->n_freq > 4 || c->freq[0] != 1.0) return ZIM_ERR_INVALID_ARG;
        for (int i = 0; i < c->n_freq; i++) {
            if (!steps_ok(c->shift_num[i]) || !is_int(c->freq[i]) || c->freq[i] > ZIM_MAX_ORDER + 1)
                return ZIM_ERR_INVALID_ARG;
            if (i > 0) {
                double r = c->freq[i] / c->freq[i - 1];
                if (!is_int(r) || r < 2) return ZIM_ERR_INVALID_ARG;
            }
        }
        break;
    }
    case ZIM_ENC_GRAYCODE:
    case ZIM_ENC_GRAYCODE_COMPLEMENTARY:
        if (!steps_ok(c->shift_num[0]) || c->gray_bits < 1 || c->gray_bits > 12) return ZIM_ERR_INVALID_ARG;
        break;
    default:
        return ZIM_ERR_INVALID_ARG;
    }
    if (zim_decode_frame_count(c) > 64) return ZIM_ERR_INVALID_ARG;
    return ZIM_OK;
}

extern "C" ZIM_API int zim_decode_frame_count(const zim_decode_config* c) {
    if (!c) return -1;
    int f = 0;
    switch (c->encoding) {
    case ZIM_ENC_HETERODYNE3: for (int i = 0; i < 3; i++) f += c->shift_num[i]; break;
    case ZIM_ENC_HIERARCHICAL:
        if (c->n_freq < 1 || c->n_freq > 4) return -1;
        for (int i = 0; i < c->n_freq; i++) f += c->shift_num[i];
        break;
    case ZIM_ENC_GRAYCODE: f = c->shift_num[0] + c->gray_bits; break;
    case ZIM_ENC_GRAYCODE_COMPLEMENTARY: f = c->shift_num[0] + c->gray_bits + 1; break;
    default: return -1;
    }
    return f;
}

extern "C" ZIM_API int zim_decode_max_order(const zim_decode_config* c) {
    if (!c) return -1;
    switch (c->encoding) {
    case ZIM_ENC_HETERODYNE3: return (int)c->freq[0];
    case ZIM_ENC_HIERARCHICAL: return (int)c->freq[c->n_freq - 1] - 1;
    case ZIM_ENC_GRAYCODE:
    case ZIM_ENC_GRAYCODE_COMPLEMENTARY: return (1 << c->gray_bits) - 1;
    default: return -1;
    }
}

extern "C" ZIM_API zim_status zim_create(int device, zim_ctx** out) {
    if (!out) return ZIM_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return ZIM_ERR_CUDA;
    }
    if (device < 0 || device >= n) return ZIM_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return ZIM_ERR_CUDA;
    zim_ctx* ctx = new zim_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaFree(0) != cudaSuccess || cudaMalloc(&ctx->d_error, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_error, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->d_sor_stats, 256) != cudaSuccess ||
        cudaMallocHost(&ctx->h_pinned, 4096) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->aux_event, cudaEventDisableTiming) != cudaSuccess) {
        delete ctx;
        return ZIM_ERR_CUDA;
    }
    *out = ctx;
    return ZIM_OK;
}

extern "C" ZIM_API void zim_destroy(zim_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (int c = 0; c < 2; c++)
        for (int m = 0; m < 2; m++) cudaFree(ctx->d_map[c][m]);
    for (int k = 0; k < 3; k++) cudaFree(ctx->d_poly[k]);
    cudaFree(ctx->scratch);
    cudaFree(ctx->d_error);
    cudaFree(ctx->d_sor_stats);
    cudaFreeHost(ctx->h_pinned);
    if (ctx->aux_event) cudaEventDestroy(ctx->aux_event);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    delete ctx;
    cudaGetLastError();  // destruction cannot report: do not leave its errors to the thread's next call
}

extern "C" ZIM_API const char* zim_last_error(const zim_ctx* ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" ZIM_API zim_status zim_release_scratch(zim_ctx* ctx) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    ZIM_CUDA_TRY(ctx, cudaFree(ctx->scratch));
    ctx->scratch = nullptr;
    ctx->scratch_cap = ctx->scratch_used = 0;
    return ZIM_OK;
}

extern "C" ZIM_API size_t zim_scratch_bytes(const zim_ctx* ctx) { return ctx ? ctx->scratch_cap : 0; }

extern "C" ZIM_API unsigned long long zim_launch_count(const zim_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" ZIM_API zim_status zim_check_device(zim_ctx* ctx, uint32_t* error_word) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    uint32_t w = 0;
    ZIM_CUDA_TRY(ctx, cudaMemcpy(&w, ctx->d_error, sizeof w, cudaMemcpyDeviceToHost));
    ZIM_CUDA_TRY(ctx, cudaMemset(ctx->d_error, 0, sizeof(uint32_t)));
    if (error_word) *error_word = w;
    return w ? zim_fail(ctx, ZIM_ERR_DEVICE_CHECK, "device error word 0x%08x", w) : ZIM_OK;
}

zim_status zim_scratch_reserve(zim_ctx* ctx, size_t bytes) {
    bytes = zim_align256(bytes);
    if (bytes <= ctx->scratch_cap) return ZIM_OK;
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    if (ctx->scratch) cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_cap = 0;
    size_t grown = bytes + bytes / 8;
    if (cudaMalloc(&ctx->scratch, grown) != cudaSuccess) {
        cudaGetLastError();
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "cannot reserve %zu bytes of scratch", grown);
    }
    ctx->scratch_cap = grown;
    return ZIM_OK;
}

void* zim_scratch_take(zim_ctx* ctx, size_t bytes) {
    size_t b = zim_align256(bytes);
    if (ctx->scratch_used + b > ctx->scratch_cap) return nullptr;
    void* p = ctx->scratch + ctx->scratch_used;
    ctx->scratch_used += b;
    return p;
}

// ---------------------------------------------------------------------------
// Whole-pair pipeline.
// ---------------------------------------------------------------------------
namespace {
struct PairBuffers {
    int32_t* order[2];
    float* res[2];
    int32_t* sk[2];  // post-smoothed taps (16 x cycles, residual)
    float* sr[2];
    float* disp_raw;
    float* disp_med;
    float* xyz[2];
    uint8_t* mask[2];
    float* mls_tmp;
};

size_t pair_scratch_bytes(const zim_ctx* ctx, const zim_recon_config* r, int rows, int cols, bool need_disp,
                          int sample_bytes, int frames, bool host) {
    size_t src = (size_t)rows * cols, dst = (size_t)ctx->rect_h * ctx->rect_w;
    size_t b = 0;
    b += 2 * (zim_align256(src * 4) * 4);
    b += zim_align256(dst * 4);
    if (need_disp) b += zim_align256(dst * 4);
    b += 2 * (zim_align256(dst * 12) + zim_align256(dst));
    if (r->use_mls) b += zim_align256(dst * 12);
    if (r->use_sor || r->use_metric_gaussian) b += zim_grid_scratch_bytes(dst);
    if (host) b += 2 * zim_align256((size_t)frames * src * sample_bytes);
    return b + 4096;
}
}  // namespace

static zim_status check_pair_args(zim_ctx* ctx, const zim_decode_config* d, const zim_recon_config* r,
                                  const void* lf, const void* rf, int sample_type, int rows, int cols,
                                  float* xyz, uint8_t* mask) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!d || !r || !lf || !rf || !xyz || !mask)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    zim_status s = zim_decode_validate(d);
    if (s != ZIM_OK) return zim_fail(ctx, s, "invalid decode config");
    if (sample_type != ZIM_SAMPLE_U8 && sample_type != ZIM_SAMPLE_U16)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad sample type");
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "zim_set_calibration first");
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "image %dx%d differs from calibration %dx%d", cols, rows,
                        ctx->src_w, ctx->src_h);
    if (r->use_mls && (r->mls_window_size < 0 || r->mls_window_size > 64))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "mls_window_size out of range");
    if (r->use_ror && (r->radius_window_size < 0 || r->radius_window_size > ZIM_MAX_ROR_WINDOW))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "radius_window_size must be in [0, %d]", ZIM_MAX_ROR_WINDOW);
    return zim_check_reproject(ctx, r);
}

// right_ready (may be null): an event the right camera's frames wait for, so
// that their upload overlaps the left camera's decode.
static zim_status run_pair(zim_ctx* ctx, const zim_decode_config* d, const zim_recon_config* r, const void* lf,
                           const void* rf, int sample_type, int rows, int cols, int pha_f, float* xyz_out,
                           uint8_t* mask_out, float* disp_out, PairBuffers& B, cudaStream_t st,
                           cudaEvent_t right_ready = nullptr) {
    zim_status s;
    const void* frames[2] = {lf, rf};
    const int post = d->enable_hdr ? (d->post_smooth ? 2 : 3) : (d->post_smooth ? 1 : 0);
    for (int c = 0; c < 2; c++) {
        if (c == 1 && right_ready) ZIM_CUDA_TRY(ctx, cudaStreamWaitEvent(st, right_ready, 0));
        s = zim_decode_launch(ctx, d, frames[c], sample_type, rows, cols, B.order[c], B.res[c], nullptr, nullptr, st);
        if (s) return s;
        s = zim_smooth_launch(ctx, B.order[c], B.res[c], rows, cols, post, B.sk[c], B.sr[c], st);
        if (s) return s;
    }
    const int RH = ctx->rect_h, RW = ctx->rect_w;
    if (pha_f <= 0) pha_f = zim_decode_max_order(d);
    // setData's remap fused into the matching: the rectified maps stay on chip
    {
        const int32_t* ord[2] = {B.order[0], B.order[1]};
        const float* res[2] = {B.res[0], B.res[1]};
        s = zim_rectify_match_launch(ctx, ord, res, B.sk, B.sr, rows, cols, post, pha_f, r->grad_threshold,
                                     B.disp_raw, st);
        if (s) return s;
    }

    // Stage routing: the last writer of xyz / mask writes the caller's buffers.
    enum { ST_REPROJ, ST_PXG, ST_ROR, ST_SOR, ST_MLS, ST_MG };
    bool on[6] = {true, r->use_px_gaussian != 0, r->use_ror != 0, r->use_sor != 0, r->use_mls != 0,
                  r->use_metric_gaussian != 0};
    bool writes_mask[6] = {true, r->px_gaussian_updates_mask != 0, true, true, false, false};
    int last_x = ST_REPROJ, last_m = ST_REPROJ;
    for (int i = 0; i < 6; i++)
        if (on[i]) {
            last_x = i;
            if (writes_mask[i]) last_m = i;
        }
    const float* cx = nullptr;
    const uint8_t* cm = nullptr;
    int sx = 0, sm = 0;  // next scratch slot
    auto next_x = [&](int stage) -> float* {
        if (stage == last_x) return xyz_out;
        float* p = B.xyz[sx];
        if (p == cx) { sx ^= 1; p = B.xyz[sx]; }
        sx ^= 1;
        return p;
    };
    auto next_m = [&](int stage) -> uint8_t* {
        if (stage == last_m) return mask_out;
        uint8_t* p = B.mask[sm];
        if (p == cm) { sm ^= 1; p = B.mask[sm]; }
        sm ^= 1;
        return p;
    };
    {
        float* ox = next_x(ST_REPROJ);
        uint8_t* om = next_m(ST_REPROJ);
        s = zim_median_reproject_launch(ctx, r, B.disp_raw, RH, RW, B.disp_med, ox, om, st);
        if (s) return s;
        cx = ox; cm = om;
    }
    if (on[ST_PXG]) {
        float* ox = next_x(ST_PXG);
        uint8_t* om = writes_mask[ST_PXG] ? next_m(ST_PXG) : nullptr;
        s = zim_px_gaussian_launch(ctx, cx, cm, RH, RW, ox, om, st);
        if (s) return s;
        cx = ox;
        if (om) cm = om;
    }
    if (on[ST_ROR]) {
        float* ox = next_x(ST_ROR);
        uint8_t* om = next_m(ST_ROR);
        s = zim_ror_launch(ctx, cx, cm, RH, RW, r->radius_search, r->radius_min_neighbors, r->radius_window_size, ox,
                           om, st);
        if (s) return s;
        cx = ox; cm = om;
    }
    // the grid filters carve their hash tables from the same region in turn
    const size_t grid_mark = ctx->scratch_used;
    if (on[ST_SOR]) {
        uint8_t* om = next_m(ST_SOR);
        float* ox = next_x(ST_SOR);
        // removed points read as zero in the organised output
        s = zim_sor_launch(ctx, cx, cm, RH, RW, r->sor_mean_k, r->sor_std_mul, ox, om, nullptr,
                           zim_rays_of(ctx, r->use_rectified_coords != 0, 0, 0), st);
        if (s) return s;
        ctx->scratch_used = grid_mark;
        cx = ox; cm = om;
    }
    if (on[ST_MLS]) {
        float* ox = next_x(ST_MLS);
        s = zim_mls_launch(ctx, cx, cm, RH, RW, r->mls_window_size, r->mls_spatial_sigma, r->mls_polynomial_order,
                           r->mls_max_radius, r->mls_iterations, ox, B.mls_tmp,
                           zim_rays_of(ctx, r->use_rectified_coords != 0, 0, 0), st);
        if (s) return s;
        cx = ox;
    }
    if (on[ST_MG]) {
        float* ox = next_x(ST_MG);
        s = zim_metric_gaussian_launch(ctx, cx, cm, RH, RW, r->metric_gaussian_sigma, ox,
                                       zim_rays_of(ctx, r->use_rectified_coords != 0, 0, 0), st);
        if (s) return s;
        ctx->scratch_used = grid_mark;
        cx = ox;
    }
    if (cm != mask_out) ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(mask_out, cm, (size_t)RH * RW, cudaMemcpyDeviceToDevice, st));
    if (cx != xyz_out) ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(xyz_out, cx, (size_t)RH * RW * 12, cudaMemcpyDeviceToDevice, st));
    if (disp_out && disp_out != B.disp_med)
        ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(disp_out, B.disp_med, (size_t)RH * RW * 4, cudaMemcpyDeviceToDevice, st));
    return ZIM_OK;
}

static zim_status carve_pair(zim_ctx* ctx, const zim_recon_config* r, int rows, int cols, float* disp_out,
                             PairBuffers& B) {
    size_t src = (size_t)rows * cols, dst = (size_t)ctx->rect_h * ctx->rect_w;
    for (int c = 0; c < 2; c++) {
        B.order[c] = (int32_t*)zim_scratch_take(ctx, src * 4);
        B.res[c] = (float*)zim_scratch_take(ctx, src * 4);
        B.sk[c] = (int32_t*)zim_scratch_take(ctx, src * 4);
        B.sr[c] = (float*)zim_scratch_take(ctx, src * 4);
        B.xyz[c] = (float*)zim_scratch_take(ctx, dst * 12);
        B.mask[c] = (uint8_t*)zim_scratch_take(ctx, dst);
    }
    B.disp_raw = (float*)zim_scratch_take(ctx, dst * 4);
    B.disp_med = disp_out ? disp_out : (float*)zim_scratch_take(ctx, dst * 4);
    B.mls_tmp = r->use_mls ? (float*)zim_scratch_take(ctx, dst * 12) : nullptr;
    for (int c = 0; c < 2; c++)
        if (!B.order[c] || !B.res[c] || !B.sk[c] || !B.sr[c] || !B.xyz[c] || !B.mask[c])
            return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "scratch carve failed");
    if (!B.disp_raw || !B.disp_med || (r->use_mls && !B.mls_tmp))
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "scratch carve failed");
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_reconstruct_pair(zim_ctx* ctx, const zim_decode_config* d,
                                                   const zim_recon_config* r, const void* lf, const void* rf,
                                                   int sample_type, int rows, int cols, int pha_f, float* xyz,
                                                   uint8_t* mask, float* disp, void* stream) {
    zim_status s = check_pair_args(ctx, d, r, lf, rf, sample_type, rows, cols, xyz, mask);
    if (s) return s;
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    s = zim_scratch_reserve(ctx, pair_scratch_bytes(ctx, r, rows, cols, disp == nullptr, 0, 0, false));
    if (s) return s;
    zim_scratch_reset(ctx);
    PairBuffers B;
    s = carve_pair(ctx, r, rows, cols, disp, B);
    if (s) return s;
    return run_pair(ctx, d, r, lf, rf, sample_type, rows, cols, pha_f, xyz, mask, disp, B, zim_stream(stream));
}

// Body of the host entries: uploads both frame stacks, runs the pair and
// queues the downloads on `stream`.  sync: drains the stream before returning.
// Without sync the call returns once everything is queued; on an error after
// work was queued it drains the stream all the same, so that nothing it queued
// still writes the caller's host buffers once it has returned.
static zim_status host_pair(zim_ctx* ctx, const zim_decode_config* d, const zim_recon_config* r, const void* lf,
                            const void* rf, int sample_type, int rows, int cols, int pha_f, float* xyz,
                            uint8_t* mask, float* disp, void* stream, bool sync) {
    zim_status s = check_pair_args(ctx, d, r, lf, rf, sample_type, rows, cols, xyz, mask);
    if (s) return s;
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int F = zim_decode_frame_count(d);
    const int sb = sample_type == ZIM_SAMPLE_U8 ? 1 : 2;
    const size_t fbytes = (size_t)F * rows * cols * sb;
    const size_t dst = (size_t)ctx->rect_h * ctx->rect_w;
    size_t need = pair_scratch_bytes(ctx, r, rows, cols, true, sb, F, true) + zim_align256(dst * 12) +
                  zim_align256(dst) + zim_align256(dst * 4);
    s = zim_scratch_reserve(ctx, need);
    if (s) return s;
    zim_scratch_reset(ctx);
    void* dl = zim_scratch_take(ctx, fbytes);
    void* dr = zim_scratch_take(ctx, fbytes);
    float* dxyz = (float*)zim_scratch_take(ctx, dst * 12);
    uint8_t* dmask = (uint8_t*)zim_scratch_take(ctx, dst);
    float* ddisp = (float*)zim_scratch_take(ctx, dst * 4);
    if (!dl || !dr || !dxyz || !dmask || !ddisp) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "scratch carve failed");
    PairBuffers B;
    s = carve_pair(ctx, r, rows, cols, ddisp, B);
    if (s) return s;
    cudaStream_t st = zim_stream(stream);
    // the right frames travel on the second queue while the left camera decodes
    // (the second queue starts after everything already on st)
    cudaError_t e = cudaMemcpyAsync(dl, lf, fbytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->aux_event, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux_stream, ctx->aux_event, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dr, rf, fbytes, cudaMemcpyHostToDevice, ctx->aux_stream);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->aux_event, ctx->aux_stream);
    // Synchronous calls: a pinned (page-locked) cloud buffer takes the last
    // stage's writes directly through its device address, so the copy back
    // overlaps that stage.  Only the last stage writes it; the mask, which
    // later stages read, stays on the device and is copied.  MLS with three
    // or more passes ping-pongs through its output, so a pass would read its
    // neighbourhoods back across the host link: that case writes the device
    // scratch and copies instead.  Asynchronous calls always copy: with other
    // pairs' kernels waiting for the SMs, a kernel that stalls on writes across
    // the host link costs more than a copy engine moving the cloud (5 MP,
    // three pairs in flight: 1327 -> 1427 Mpoints/s end to end).
    const bool last_reads_out = r->use_mls && !r->use_metric_gaussian && r->mls_iterations >= 3;
    float* xyz_dev = nullptr;
    if (e == cudaSuccess && !last_reads_out && sync) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, xyz) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer != nullptr)
            xyz_dev = static_cast<float*>(a.devicePointer);
        else
            cudaGetLastError();  // pageable memory: clear the query's error, copy back below
    }
    if (e == cudaSuccess)
        s = run_pair(ctx, d, r, dl, dr, sample_type, rows, cols, pha_f, xyz_dev ? xyz_dev : dxyz, dmask, ddisp, B,
                     st, ctx->aux_event);
    if (e == cudaSuccess && s == ZIM_OK && !xyz_dev) e = cudaMemcpyAsync(xyz, dxyz, dst * 12, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && s == ZIM_OK) e = cudaMemcpyAsync(mask, dmask, dst, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && s == ZIM_OK && disp) e = cudaMemcpyAsync(disp, ddisp, dst * 4, cudaMemcpyDeviceToHost, st);
    const bool failed = s != ZIM_OK || e != cudaSuccess;
    // Whatever failed, nothing queued here may still be writing the caller's
    // host buffers when this returns: drain the stream first.
    cudaError_t es = cudaSuccess;
    if (sync || failed) {
        es = cudaStreamSynchronize(st);
        if (failed) cudaStreamSynchronize(ctx->aux_stream);
    }
    if (s) return s;
    if (e != cudaSuccess || es != cudaSuccess) {
        const cudaError_t err = e != cudaSuccess ? e : es;
        cudaGetLastError();
        return zim_fail(ctx, ZIM_ERR_CUDA, "%s", cudaGetErrorString(err));
    }
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_reconstruct_pair_host(zim_ctx* ctx, const zim_decode_config* d,
                                                        const zim_recon_config* r, const void* lf,
                                                        const void* rf, int sample_type, int rows, int cols,
                                                        int pha_f, float* xyz, uint8_t* mask, float* disp,
                                                        void* stream) {
    return host_pair(ctx, d, r, lf, rf, sample_type, rows, cols, pha_f, xyz, mask, disp, stream, true);
}

extern "C" ZIM_API zim_status zim_reconstruct_pair_host_async(zim_ctx* ctx, const zim_decode_config* d,
                                                              const zim_recon_config* r, const void* lf,
                                                              const void* rf, int sample_type, int rows, int cols,
                                                              int pha_f, float* xyz, uint8_t* mask, float* disp,
                                                              void* stream) {
    return host_pair(ctx, d, r, lf, rf, sample_type, rows, cols, pha_f, xyz, mask, disp, stream, false);
}
