// zim_internal.cuh -- shared declarations of the zim_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/zim.h"

#define ZIM_TWO_PI_F 6.28318530717958647692f
#define ZIM_PI_F 3.14159265358979323846f
#define ZIM_INV_TWO_PI_F 0.159154943091895335769f

// Maximum rectified width handled by the one-CTA-per-row matcher.
#define ZIM_MAX_MATCH_COLS 8192
#define ZIM_MAX_ORDER 4095
// Largest radius-filter window: its shared-memory tile must fit one CTA.
#define ZIM_MAX_ROR_WINDOW 96

struct zim_ctx {
    int device = 0;
    int sm_count = 0;
    std::string last_error;

    // calibration (setCalibrationParams)
    bool calibrated = false;
    zim_stereo_calib calib{};
    double R1[9], R2[9], P1[12], P2[12], Q[16];
    double ir[2][9];  // (P_c[:, :3] R_c)^-1: rectified pixel -> camera ray
    int src_w = 0, src_h = 0, rect_w = 0, rect_h = 0;
    float* d_map[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    // per-pixel polynomial calibration maps (setCalibrationParamsV2), rect size
    float4* d_poly[3] = {nullptr, nullptr, nullptr};
    int poly_w = 0, poly_h = 0;

    // persistent scratch arena (per context, grown on demand)
    char* scratch = nullptr;
    size_t scratch_cap = 0;
    size_t scratch_used = 0;

    uint32_t* d_error = nullptr;  // device error word
    void* h_pinned = nullptr;     // small pinned staging (counts)
    unsigned long long launches = 0;  // kernels this context has launched
    void* d_sor_stats = nullptr;      // device copy of the last SOR run's statistics (256 B)
    cudaStream_t aux_stream = nullptr; // second copy engine queue for the host entry points
    cudaEvent_t aux_event = nullptr;
    bool have_sor_stats = false;
    double last_sor_std_mul = 1.0;
};

// Records a formatted error on the context and returns the status.
zim_status zim_fail(zim_ctx* ctx, zim_status st, const char* fmt, ...);

#define ZIM_CUDA_TRY(ctx, call)                                                             \
    do {                                                                                    \
        cudaError_t _e = (call);                                                            \
        if (_e != cudaSuccess)                                                              \
            return zim_fail((ctx), ZIM_ERR_CUDA, "%s failed: %s (%s:%d)", #call,             \
                            cudaGetErrorString(_e), __FILE__, __LINE__);                    \
    } while (0)

#define ZIM_LAUNCH_CHECK(ctx)                                                               \
    do {                                                                                    \
        cudaError_t _e = cudaGetLastError();                                                \
        if (_e != cudaSuccess)                                                              \
            return zim_fail((ctx), ZIM_ERR_CUDA, "kernel launch failed: %s (%s:%d)",         \
                            cudaGetErrorString(_e), __FILE__, __LINE__);                    \
    } while (0)

// Scratch arena: reserve() grows it (synchronising the device first), take()
// carves 256-byte aligned slices; reset() starts a new call's carving.
zim_status zim_scratch_reserve(zim_ctx* ctx, size_t bytes);
void* zim_scratch_take(zim_ctx* ctx, size_t bytes);
inline void zim_scratch_reset(zim_ctx* ctx) { ctx->scratch_used = 0; }
inline size_t zim_align256(size_t b) { return (b + 255) & ~(size_t)255; }

inline cudaStream_t zim_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- internal launchers (no argument validation; callers validate) ----
struct zim_decode_params;  // decode.cu
namespace zt {
struct DecodeParams;
}
// The bulk-tensor-copy decode: whether it applies to these frames (HDR, row
// pitch, frame count), and its launch (false, and nothing launched, when not).
bool zim_decode_tma_applies(const void* frames, int sample_type, const zt::DecodeParams& p);
bool zim_decode_tma_launch(zim_ctx* ctx, const void* frames, int sample_type, const zt::DecodeParams& p,
                           int32_t* order, float* residual, cudaStream_t st);
zim_status zim_decode_launch(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames,
                             int sample_type, int rows, int cols, int32_t* order, float* residual,
                             float* mod, uint8_t* valid, cudaStream_t st);
// post_smooth: smooth_k16 / smooth_r are rows*cols scratch for the smoothed taps.
zim_status zim_rectify_launch(zim_ctx* ctx, int cam, const int32_t* order, const float* residual,
                              int rows, int cols, int post_smooth, int32_t* smooth_k16, float* smooth_r,
                              int32_t* rect_base, float* rect_res, int32_t* rect_order, cudaStream_t st);
zim_status zim_match_launch(zim_ctx* ctx, const int32_t* l_base, const float* l_res,
                            const int32_t* l_order, const int32_t* r_base, const float* r_res,
                            const int32_t* r_order, int rows, int cols, int pha_f,
                            double grad_threshold, float* disp, int32_t* best_col, cudaStream_t st);
// Pixel rays of an organised cloud: cloud pixel (u, v) looks from the origin
// along R (u + ox - cx, v + oy - cy, f).  The window fast paths of the grid
// filters use it only as a hint: they measure how far every point lies from
// its ray and fall back to the exact grid search where the bound does not hold.
struct zim_ray_model {
    float cx = 0.f, cy = 0.f, f = 0.f;
    float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    int ox = 0, oy = 0;
    int valid = 0;
};
// The rays of the context's rectified left camera (rotated by R1^T for clouds
// in camera coordinates); invalid when the context is not calibrated.
zim_ray_model zim_rays_of(const zim_ctx* ctx, bool rectified_coords, int ox, int oy);
// The same from a rectification's Q and R1 (row-major 4x4, 3x3).
zim_ray_model zim_rays_from(const double* Q, const double* R1, bool rectified_coords, int ox, int oy);

// Checks that a reconstruction config can run on this context (reprojection
// model and its maps).
zim_status zim_check_reproject(zim_ctx* ctx, const zim_recon_config* cfg);
zim_status zim_median_reproject_launch(zim_ctx* ctx, const zim_recon_config* cfg, const float* disp,
                                       int rows, int cols, float* disp_out, float* xyz,
                                       uint8_t* mask, cudaStream_t st);
zim_status zim_px_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                  int cols, float* out, uint8_t* mask_out, cudaStream_t st);
zim_status zim_ror_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                          float radius, int min_neighbors, int window_size, float* out,
                          uint8_t* mask_out, cudaStream_t st);
zim_status zim_smooth_launch(zim_ctx* ctx, const int32_t* order, const float* residual, int rows, int cols,
                             int post_smooth, int32_t* smooth_k16, float* smooth_r, cudaStream_t st);
zim_status zim_rectify_match_launch(zim_ctx* ctx, const int32_t* const order[2], const float* const res[2],
                                    int32_t* const sk[2], float* const sr[2], int srows, int scols, int post_smooth,
                                    int pha_f, double grad_threshold, float* disp, cudaStream_t st);
zim_status zim_mls_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                          int window, float sigma, int order, float max_radius, int iterations,
                          float* out, float* tmp, const zim_ray_model& rays, cudaStream_t st);
zim_status zim_sor_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                          int mean_k, double std_mul, float* xyz_out, uint8_t* mask_out,
                          float* mean_dist, const zim_ray_model& rays, cudaStream_t st);
zim_status zim_metric_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                      int cols, double sigma, float* out, const zim_ray_model& rays,
                                      cudaStream_t st);
zim_status zim_compact_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                              int cols, zim_point_xyz* points, uint64_t* count_dev, cudaStream_t st);

// Rectification of one calibration: stereoRectify (+ full-left canvas) and the
// two cameras' float maps on the device (calib.cu).
struct zim_rect_state {
    double R1[9], R2[9], P1[12], P2[12], Q[16];
    double ir[2][9];
    int src_w = 0, src_h = 0, rect_w = 0, rect_h = 0;
    float* d_map[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
};
zim_status zim_rect_build(zim_ctx* ctx, const zim_stereo_calib* c, int use_full_left, zim_rect_state& st);
void zim_rect_free(zim_rect_state& st);

// Scratch bytes needed by the grid filters for n points.
size_t zim_grid_scratch_bytes(size_t n_points);
size_t zim_mls_scratch_bytes(size_t n_points);
