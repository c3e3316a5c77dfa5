/*
 * zim.h -- C ABI of zim_gb300, the GB300 (sm_103a) structured-light stereo
 * reconstruction path: phase-shift decode + unwrap, rectification, order-
 * constrained matching, Q reprojection and point-cloud filters.
 *
 * Reference interfaces replaced (PhaseShiftGrayCode3D/src/):
 *   JSLAB_PhaseShiftDecoder::Config / create / setImages / startCalculate /
 *     getOrderMap / getModulationMap        JSLAB_PhaseShiftDecoder.h:10-92
 *   JSLAB_DecodePhase_GPU / _Warmup / _Release
 *                                           JSLAB_PhaseShiftDecoder_V2_GPU.h:50-60
 *   JSLAB_StereoCalibParams_V1              JSLAB_StereoCalibParams_V1.h:9-20
 *   JSLAB_PhaseEpipolarReconstructor_V2::Config / setCalibrationParams /
 *     setData / startCalculate / getDisparityMap
 *                                           JSLAB_PhaseEpipolarReconstructor_V2.h:11-171
 *   JSLAB_ReconstructPipeline_GPU           JSLAB_PhaseEpipolarReconstructor_V2_GPU.h:131-137
 *   applyMLSFilterToPointCloud              JSLAB_MLS_Filter.h:31-57
 *
 * Conventions: plain pointers and sizes only.  Unless a name ends in _host,
 * every array argument is DEVICE memory and work is enqueued on `stream`
 * (a cudaStream_t passed as void*, NULL = legacy default stream); calls are
 * asynchronous w.r.t. the host.  Images are row-major, tightly packed.
 * A decoded phase is carried as (order k, residual r): phase = 2*pi*k + r,
 * which keeps 1e-6 rad resolution at hundreds of fringe periods in FP32.
 * Errors: every call returns a zim_status; nothing throws across the ABI;
 * zim_last_error() describes the last failure on that context.
 * Threading: one context per host thread; a context is not re-entrant.
 */
#ifndef ZIM_H
#define ZIM_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define ZIM_API __declspec(dllexport)
#else
#define ZIM_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum zim_status {
    ZIM_OK = 0,
    ZIM_ERR_INVALID_ARG = 1,    /* bad pointer/size/config (reference: CV_Assert, nullptr factory) */
    ZIM_ERR_UNSUPPORTED = 2,    /* valid but not implemented on this path */
    ZIM_ERR_NOT_CALIBRATED = 3, /* reconstruction before zim_set_calibration */
    ZIM_ERR_CUDA = 4,           /* a CUDA runtime call failed */
    ZIM_ERR_OUT_OF_MEMORY = 5,  /* scratch allocation failed */
    ZIM_ERR_TIMEOUT = 6,        /* a bounded device wait gave up */
    ZIM_ERR_DEVICE_CHECK = 7    /* a kernel's own bounds check tripped (device error word) */
} zim_status;

typedef struct zim_ctx zim_ctx;

typedef enum zim_encoding {
    ZIM_ENC_HETERODYNE3 = 0,            /* reference: 3-frequency heterodyne, beat-to-one */
    ZIM_ENC_HIERARCHICAL = 1,           /* temporal unwrapping, f0 = 1, integer ratios */
    ZIM_ENC_GRAYCODE = 2,               /* N-step phase shift + Gray code */
    ZIM_ENC_GRAYCODE_COMPLEMENTARY = 3  /* ... + one complementary (half-period) Gray bit */
} zim_encoding;

typedef enum zim_sample_type { ZIM_SAMPLE_U8 = 0, ZIM_SAMPLE_U16 = 1 } zim_sample_type;

/* JSLAB_PhaseShiftDecoder::Config (JSLAB_PhaseShiftDecoder.h:22-54), plus the
 * encoding selector.  Frames are ordered frequency 0 steps, frequency 1 steps,
 * ... (JSLAB_PhaseShiftDecoder_V2.cpp:230-238); Gray encodings: the shift_num[0]
 * phase frames, then gray_bits Gray frames MSB first, then the complementary frame. */
typedef struct zim_decode_config {
    double freq[4];              /* fringe counts across the projector (integers) */
    int shift_num[4];            /* phase steps per frequency (3..32) */
    double modulation_threshold; /* default 1.0 */
    double preblur_sigma;        /* 3x3 pre-blur sigma, default 3.0 (<= 0: OpenCV default kernel) */
    int avg_three_phase;         /* default 1 (heterodyne only) */
    int post_smooth;             /* default 1: 3x3 Gaussian of the absolute phase */
    int enable_hdr;              /* default 0; 1: HDR least squares on raw samples (heterodyne,
                                    hierarchical; JSLAB_HDRPhaseFit.h), invalid orders -1 */
    double hdr_saturation_gray;
    double hdr_min_amplitude;
    int encoding;                /* zim_encoding, default ZIM_ENC_HETERODYNE3 */
    int n_freq;                  /* frequencies used (heterodyne 3, hierarchical 2..4, Gray 1) */
    int gray_bits;               /* Gray encodings: bits (1..12) */
} zim_decode_config;

/* JSLAB_StereoCalibParams_V1 (JSLAB_StereoCalibParams_V1.h:9-20): row-major
 * 3x3 K, (k1 k2 p1 p2 k3), left->right R and t, calibration image size. */
typedef struct zim_stereo_calib {
    double camera_matrix[2][9];
    double dist_coeffs[2][5];
    double R[9];
    double t[3];
    int width, height;
} zim_stereo_calib;

/* JSLAB_PhaseEpipolarReconstructor_V2::Config (JSLAB_PhaseEpipolarReconstructor_V2.h:18-55)
 * plus the PCL-style filters.  Filter chain order: pixel Gaussian, radius
 * outlier (ROR), statistical outlier (SOR), MLS, metric Gaussian. */
typedef struct zim_recon_config {
    double min_depth, max_depth;             /* 0, 1000 */
    double min_phase_diff, max_phase_diff;   /* unused by V2, kept for layout parity */
    double grad_threshold;                   /* 1.0 */
    int use_rectified_coords;                /* 1 */
    int use_disp_median_filter;              /* 1 */
    int use_full_left_rectification;         /* 1 */
    int use_px_gaussian;                     /* 1: applyGaussianFilterToPointCloudV2 */
    int px_gaussian_updates_mask;            /* 0: CPU semantics (ROR sees the pre-filter mask); 1: GPU semantics */
    int use_ror;                             /* 1 */
    float radius_search;                     /* 0.7 */
    int radius_min_neighbors;                /* 10 */
    int radius_window_size;                  /* 10 */
    int use_mls;                             /* 0 */
    int mls_window_size;                     /* 30 (half size) */
    float mls_spatial_sigma;                 /* 0.6 */
    int mls_polynomial_order;                /* 1 */
    float mls_max_radius;                    /* 0 = 3 sigma */
    int mls_iterations;                      /* 3 */
    int use_sor;                             /* 0: PCL StatisticalOutlierRemoval semantics */
    int sor_mean_k;                          /* 50 */
    double sor_std_mul;                      /* 1.0 */
    int use_metric_gaussian;                 /* 0: radius-3-sigma Gaussian in millimetres */
    double metric_gaussian_sigma;            /* 0.5 */
    /* 0: Q-matrix reprojection (startCalculate, V2.cpp:397-480).
     * 1: per-pixel polynomial maps set by zim_set_poly_calib (startCalculate_v2,
     *    V2.cpp:482-593 with evaluateV2CalibPoint :13-76); the rest of the
     *    chain is unchanged. */
    int reproject_model;                     /* 0 */
} zim_recon_config;

/* PCL PointXYZ memory layout: x, y, z, padding (16 bytes). */
typedef struct zim_point_xyz { float x, y, z, pad; } zim_point_xyz;

ZIM_API const char* zim_version(void);
ZIM_API void zim_decode_config_default(zim_decode_config* cfg);
ZIM_API void zim_recon_config_default(zim_recon_config* cfg);

/* Frames a config consumes; <= 0 if the config is invalid. */
ZIM_API int zim_decode_frame_count(const zim_decode_config* cfg);
/* JSLAB_PhaseShiftDecoder::create's validity test (JSLAB_PhaseShiftDecoder.cpp:9-29:
 * nullptr unless every frequency is non-zero) plus this path's own limits. */
ZIM_API zim_status zim_decode_validate(const zim_decode_config* cfg);
/* Highest fringe order a config produces (the reference passes freq[0] as pha_f). */
ZIM_API int zim_decode_max_order(const zim_decode_config* cfg);

/* Context (replaces the reference decoder's static device buffers,
 * JSLAB_PhaseShiftDecoder_V2_GPU.cu:153-185).  zim_create also warms the
 * CUDA context (JSLAB_DecodePhase_GPU_Warmup). */
ZIM_API zim_status zim_create(int device, zim_ctx** out);
ZIM_API void zim_destroy(zim_ctx* ctx);
ZIM_API const char* zim_last_error(const zim_ctx* ctx);
/* Frees the context's scratch (JSLAB_DecodePhase_GPU_Release). */
ZIM_API zim_status zim_release_scratch(zim_ctx* ctx);
/* Bytes of device scratch the context currently holds. */
ZIM_API size_t zim_scratch_bytes(const zim_ctx* ctx);
/* Number of CUDA kernels this context has launched so far (all entry points). */
ZIM_API unsigned long long zim_launch_count(const zim_ctx* ctx);
/* Synchronises the context's device and reads/clears the device error word. */
ZIM_API zim_status zim_check_device(zim_ctx* ctx, uint32_t* error_word);

/* ---- decoder: JSLAB_DecodePhase_GPU (JSLAB_PhaseShiftDecoder_V2_GPU.cu:192-291) ----
 * frames: zim_decode_frame_count(cfg) planes of rows*cols samples (u8 or u16).
 * Outputs (rows*cols each): order (getOrderMap), residual (phase - 2*pi*order,
 * unsmoothed; 0 where invalid), mod (getModulationMap: frequency-0 normalised
 * modulation), valid (1/0).  Any output pointer except order/residual may be NULL. */
ZIM_API zim_status zim_decode(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames,
                              int sample_type, int rows, int cols, int32_t* order, float* residual,
                              float* mod, uint8_t* valid, void* stream);

/* startCalculate(phase) as CV_64F: phase = 2*pi*order + residual, then the
 * optional 3x3 post-smooth (JSLAB_PhaseShiftDecoder_V2.cpp:274-295). */
ZIM_API zim_status zim_decode_phase_f64(zim_ctx* ctx, const int32_t* order, const float* residual,
                                        int rows, int cols, int post_smooth, double* phase,
                                        void* stream);

/* ---- reconstructor ----
 * setCalibrationParams (JSLAB_PhaseEpipolarReconstructor_V2.cpp:292-339):
 * stereoRectify(flags 0, alpha -1), optional full-left canvas, rectification
 * maps (built once, on the device, in FP64). */
ZIM_API zim_status zim_set_calibration(zim_ctx* ctx, const zim_stereo_calib* calib,
                                       int use_full_left_rectification);
ZIM_API zim_status zim_get_rectification(const zim_ctx* ctx, double R1[9], double R2[9],
                                         double P1[12], double P2[12], double Q[16], int* rect_w,
                                         int* rect_h);
/* Copies the float rectification maps (rect_h*rect_w each) into device buffers. */
ZIM_API zim_status zim_get_rectify_maps(zim_ctx* ctx, int cam, float* mapx, float* mapy,
                                        void* stream);

/* JSLAB_PhaseEpipolarReconstructor_V2::setCalibrationParamsV2 (V2.cpp:340-366):
 * the per-pixel coefficient maps xyz_calib_coeffs[0..2] (CV_32FC4, rows*cols
 * float4 (c0, c1, c2, c3), row-major, HOST memory) of
 * JSLAB_StereoCalibParams_V2, used when zim_recon_config.reproject_model = 1.
 * Call after zim_set_calibration; rows x cols must be its rectified size.
 * cx = cy = cz = NULL drops the maps.  A later zim_set_calibration keeps them
 * only while the rectified size is unchanged.  Synchronises. */
ZIM_API zim_status zim_set_poly_calib(zim_ctx* ctx, const float* cx, const float* cy,
                                      const float* cz, int rows, int cols);

/* ---- ROI-restricted reconstruction (prepareRectifiedROI / startCalculate_v2_roi,
 * JSLAB_PhaseEpipolarReconstructor_V2.cpp:595-914) ---- */
typedef struct zim_rotated_rect {            /* cv::RotatedRect in source pixels */
    float center_x, center_y, width, height;
    float angle;                             /* degrees */
} zim_rotated_rect;
typedef struct zim_rect { int x, y, width, height; } zim_rect;  /* cv::Rect */
typedef struct zim_rectified_roi {           /* RectifiedROI (V2.h:97-102) without its mask */
    zim_rect left_rect, right_rect;
} zim_rectified_roi;

/* prepareRectifiedROI: the rotated rectangle's corners rounded to integers and
 * filled (closed polygon + 8-connected outline) in the source image, remapped
 * INTER_LINEAR (8-bit fixed point) into the rectified frame, thresholded > 0
 * and dilated 5x5 into roi_mask (rect_h*rect_w device bytes, 255 inside).
 * left_rect = the bounding box of that mask; right_rect = the ROI's rows and
 * the right columns holding any order 1..pha_f that occurs in the left ROI,
 * padded by 32 (all columns if none).  l_order / r_order are the rectified
 * order maps (zim_rectify).  *valid = 0 for an empty ROI (the reference's
 * false).  Synchronises the stream. */
ZIM_API zim_status zim_prepare_roi(zim_ctx* ctx, const zim_rotated_rect* roi, const int32_t* l_order,
                                   const int32_t* r_order, int pha_f, zim_rectified_roi* out,
                                   uint8_t* roi_mask, int* valid, void* stream);

/* The source-image mask of a rotated rectangle that zim_prepare_roi starts
 * from, as one column span per row (host memory, rows entries each; lo > hi
 * for an empty row).  Host only, no context. */
ZIM_API zim_status zim_roi_source_spans(const zim_rotated_rect* roi, int rows, int cols, int* lo, int* hi);

/* startCalculate_v2_roi on rectified maps (zim_rectify outputs, rect_h*rect_w):
 * left_rect pixels inside roi_mask matched against right_rect's columns only
 * (edge rejection and disparity relative to that window), 5x5 median of the
 * ROI disparity, reprojection of masked pixels (cfg->reproject_model: 1 the
 * polynomial maps like the reference, 0 Q) at their rectified coordinates,
 * then the filter chain; the pre-ROR cloud is kept when ROR leaves fewer than
 * a tenth of the reprojected points.  xyz (x3), mask and disp (may be NULL)
 * are left_rect.height x left_rect.width. */
ZIM_API zim_status zim_reconstruct_roi(zim_ctx* ctx, const zim_recon_config* cfg,
                                       const zim_rectified_roi* roi, const uint8_t* roi_mask,
                                       const int32_t* l_base, const float* l_res, const int32_t* l_order,
                                       const int32_t* r_base, const float* r_res, const int32_t* r_order,
                                       int pha_f, float* xyz, uint8_t* mask, float* disp, void* stream);

/* JSLAB_StereoCalib_V2::computePixelwiseDepthCalibration (JSLAB_StereoCalib_V2.cpp:113-240):
 * n_planes reference planes (disps[k] / masks[k]: DEVICE rows*cols float
 * disparity and 8-bit mask, passed as a host array of device pointers; a
 * sample needs mask != 0 and d > 0), reprojected through Q (row-major 4x4, the
 * rectification the disparities were measured in).  Each plane is fitted by
 * PCA (plane_eqs[4k..4k+3] = A, B, C, D with unit normal; host, may be NULL);
 * each pixel with >= 4 samples gets least-squares cubics in d for X, Y and Z
 * of the samples projected onto their planes, written as float4
 * (c0, c1, c2, c3) into cx / cy / cz (DEVICE, rows*cols each; zeros where
 * fewer than 4 samples).  1 <= n_planes <= 64.  Synchronises the stream. */
ZIM_API zim_status zim_fit_poly_calib(zim_ctx* ctx, const double Q[16], const float* const* disps,
                                      const uint8_t* const* masks, int n_planes, int rows, int cols,
                                      float* cx, float* cy, float* cz, double* plane_eqs, void* stream);

/* rectifyLeftImage (V2.cpp:920-924) for either camera: cv::remap INTER_LINEAR
 * of an 8-bit image (src_h x src_w, device) through the camera's rectification
 * maps with OpenCV's fixed-point bilinear weights (1/32-pixel positions,
 * weights in 1/32768, rounded shift) and BORDER_CONSTANT 0, into a
 * rect_h x rect_w image. */
ZIM_API zim_status zim_rectify_image(zim_ctx* ctx, int cam, const uint8_t* src, int rows, int cols,
                                     uint8_t* dst, void* stream);

/* setData for one camera (JSLAB_PhaseEpipolarReconstructor_V2.cpp:368-395):
 * post-smooth (optional) + remap INTER_LINEAR of the phase, INTER_NEAREST of
 * the order.  Rectified phase = 2*pi*rect_base + rect_res (rect_h*rect_w).
 * post_smooth (also for zim_decode_phase_f64): 0 none, 1 the 3x3 Gaussian;
 * for an HDR decode (invalid pixels carry order -1 and phase 0) 2 the HDR
 * post-smooth (blur normalised by the blurred validity,
 * JSLAB_PhaseShiftDecoder_V2.cpp:280-291) and 3 none. */
ZIM_API zim_status zim_rectify(zim_ctx* ctx, int cam, const int32_t* order, const float* residual,
                               int rows, int cols, int post_smooth, int32_t* rect_base,
                               float* rect_res, int32_t* rect_order, void* stream);

/* stereoMatch (JSLAB_PhaseEpipolarReconstructor_V2.cpp:933-1006): disparity
 * (0 = no match) and the integer match column (-1 = none; may be NULL). */
ZIM_API zim_status zim_match(zim_ctx* ctx, const int32_t* l_base, const float* l_res,
                             const int32_t* l_order, const int32_t* r_base, const float* r_res,
                             const int32_t* r_order, int rows, int cols, int pha_f,
                             double grad_threshold, float* disp, int32_t* best_col, void* stream);

/* Optional 5x5 median (reference :405-410) + Q reprojection (:414-461). */
ZIM_API zim_status zim_median_reproject(zim_ctx* ctx, const zim_recon_config* cfg,
                                        const float* disp, int rows, int cols, float* disp_out,
                                        float* xyz, uint8_t* mask, void* stream);

/* Point-cloud filters on an organised cloud (rows*cols points, xyz float3). */
ZIM_API zim_status zim_filter_px_gaussian(zim_ctx* ctx, const float* xyz, const uint8_t* mask,
                                          int rows, int cols, float* out, uint8_t* mask_out,
                                          void* stream);
ZIM_API zim_status zim_filter_ror(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                  int cols, float radius, int min_neighbors, int window_size,
                                  float* out, uint8_t* mask_out, void* stream);
ZIM_API zim_status zim_filter_mls(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                  int cols, int window, float sigma, int order, float max_radius,
                                  int iterations, float* out, void* stream);
ZIM_API zim_status zim_filter_sor(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                  int cols, int mean_k, double std_mul, uint8_t* mask_out,
                                  float* mean_dist, void* stream);
/* Statistics of the last SOR run on this context (zim_filter_sor or the SOR
 * stage of zim_reconstruct_pair): valid points, mean and standard deviation of
 * the per-point mean k-NN distance, the threshold mean + std_mul * stddev, and
 * how many points needed the second (outlier) search phase.  Synchronises. */
typedef struct zim_sor_stats {
    double n_valid, mean, stddev, threshold;
    uint32_t n_far_search;
} zim_sor_stats;
ZIM_API zim_status zim_filter_sor_stats(zim_ctx* ctx, zim_sor_stats* out);
ZIM_API zim_status zim_filter_metric_gaussian(zim_ctx* ctx, const float* xyz, const uint8_t* mask,
                                              int rows, int cols, double sigma, float* out,
                                              void* stream);

/* setData + stereoMatch in one step (JSLAB_PhaseEpipolarReconstructor_V2.cpp:
 * 368-395 then :933-1006; the order zim_reconstruct_pair runs them in): the
 * optional post-smooth of both cameras' decoded maps (source size rows x cols,
 * as zim_rectify's post_smooth), then one launch that rectifies each right row
 * into on-chip memory and each left pixel in registers and matches them.
 * disp (rect_h x rect_w) is the raw disparity of zim_match; the rectified
 * maps are never written.  Equal to zim_rectify of both cameras followed by
 * zim_match, bit for bit. */
ZIM_API zim_status zim_rectify_match(zim_ctx* ctx, const int32_t* l_order, const float* l_res,
                                     const int32_t* r_order, const float* r_res, int rows, int cols,
                                     int post_smooth, int pha_f, double grad_threshold, float* disp,
                                     void* stream);

/* Compacts valid points into PCL PointXYZ layout; *count_dev (device) gets the
 * number written.  Row-major order is preserved. */
ZIM_API zim_status zim_compact_points(zim_ctx* ctx, const float* xyz, const uint8_t* mask,
                                      int rows, int cols, zim_point_xyz* points,
                                      uint64_t* count_dev, void* stream);

/* zim_compact_points without any device allocation, for callers that may not
 * call cudaMalloc (a host application that owns all device memory through its
 * own pool, or a capture loop that cannot take the implicit synchronisation of
 * cudaMalloc/cudaFree).  No counterpart in the reference.  Its scratch is a
 * 256 KiB array in the library's device image, which limits it to
 * rows * cols <= 64 Mi pixels (larger sizes return ZIM_ERR_INVALID_ARG) and is
 * held by every GPU that loads the library until exit.  No context: it runs
 * on the current device.  The first call on a device does a one-time set-up
 * (cudaGetSymbolAddress); make it before any stream capture.  The address it
 * finds is kept until exit, so do not call this on a device after a
 * cudaDeviceReset of it.  All calls share the array: calls that overlap on the
 * GPU race, so serialise them.  ZIM_ERR_CUDA reports only this call's own
 * launch failures; errors pending from other work are left in place. */
ZIM_API zim_status zim_compact_points_noalloc(const float* xyz, const uint8_t* mask, int rows,
                                              int cols, zim_point_xyz* points,
                                              uint64_t* count_dev, void* stream);

/* The vertex body of a binary little-endian PLY file, packed on the device:
 * for each valid point in row order float x, y, z (12 bytes;
 * savePointCloudToPlyBinary, main.cpp:85-127) or, with with_gray, float x, y,
 * z then uchar red = green = blue = gray[pixel] (15 bytes, unaligned; gray
 * NULL writes 255; savePointCloudToPlyBinaryWithGray, main.cpp:132-160).
 * records holds rows*cols records at most; *count_dev (device) gets the
 * number written.  The host writes the header and copies the body out. */
ZIM_API zim_status zim_pack_ply(zim_ctx* ctx, const float* xyz, const uint8_t* mask,
                                const uint8_t* gray, int with_gray, int rows, int cols,
                                void* records, uint64_t* count_dev, void* stream);

/* Whole plain per-pair path (decode L+R, rectify, match, median, reproject,
 * filters) on device buffers.  xyz/mask/disp are rect_h*rect_w.  pha_f <= 0
 * selects zim_decode_max_order(dcfg). */
ZIM_API zim_status zim_reconstruct_pair(zim_ctx* ctx, const zim_decode_config* dcfg,
                                        const zim_recon_config* rcfg, const void* left_frames,
                                        const void* right_frames, int sample_type, int rows,
                                        int cols, int pha_f, float* xyz, uint8_t* mask, float* disp,
                                        void* stream);

/* The same from HOST buffers (the reference's cv::Mat entry): uploads both frame
 * stacks, runs the pair, downloads xyz and mask (and disp if non-NULL), and
 * synchronises.  Host buffers may be pageable; pinned is faster.  A pinned
 * (page-locked) xyz buffer is written by the last stage through its device
 * address instead of by a copy afterwards: it must not be read or written by
 * the host until the call returns (as with any output). */
ZIM_API zim_status zim_reconstruct_pair_host(zim_ctx* ctx, const zim_decode_config* dcfg,
                                             const zim_recon_config* rcfg, const void* left_frames,
                                             const void* right_frames, int sample_type, int rows,
                                             int cols, int pha_f, float* xyz, uint8_t* mask,
                                             float* disp, void* stream);

/* The same without the final synchronisation: the uploads, the pair and the
 * downloads are queued on `stream` (the right frames on the context's second
 * copy queue) and the call returns; the outputs are complete, and the frame
 * buffers free for reuse, once `stream` has drained (cudaStreamSynchronize or
 * an event recorded after the call).  With page-locked frames and outputs the
 * copies overlap other work on the GPU, so a caller that keeps two pairs in
 * flight -- one context and one stream each, alternating -- hides the
 * transfers of one pair behind the kernels of the other.  Calls on one context
 * reuse its scratch: give them the same stream (or order them yourself), and
 * keep one context per pair in flight.  The cloud is always written to device
 * scratch and copied back (a pinned xyz buffer is not written directly, as the
 * synchronous entry does: a kernel stalled on writes across the host link
 * would hold SMs the other pairs in flight need).  On an error after work was
 * queued the call drains the stream before returning.  The reference's entry
 * (startCalculate, JSLAB_PhaseEpipolarReconstructor_V2.cpp:397-480) is
 * synchronous; this is its pipelined form. */
ZIM_API zim_status zim_reconstruct_pair_host_async(zim_ctx* ctx, const zim_decode_config* dcfg,
                                                   const zim_recon_config* rcfg, const void* left_frames,
                                                   const void* right_frames, int sample_type, int rows,
                                                   int cols, int pha_f, float* xyz, uint8_t* mask,
                                                   float* disp, void* stream);

/* ---- batched path: many stereo pairs of uneven size and encoding ----
 * No counterpart in the reference (it reconstructs one pair per call through
 * JSLAB_PhaseEpipolarReconstructor_V2 / JSLAB_ReconstructPipeline_GPU).  One
 * submission holds any number of pairs, each with its own decode config,
 * sample type and one of the batch's calibrations.  Per pair it computes what
 * zim_reconstruct_pair computes (bit-identical): decode, rectify, match, 5x5
 * median, reprojection, 3x3 Gaussian and radius outlier filter, then the grid
 * filters (SOR -> MLS -> metric Gaussian) that the pair's filter config turns
 * on (zim_batch_pair.filters, or the submission's config).
 * Execution: one persistent kernel per pixel-domain stage drains a device work
 * queue of (pair, row band) items over all pairs (decode; rectify fused into
 * match; median + reprojection; each pixel filter); then the pairs' grid
 * filters run on up to six lanes (streams, each with its own scratch) side by
 * side, the largest pairs first, each to the least-loaded lane, so one pair's
 * latency-bound searches overlap another's kernels.  The whole sequence is captured once as a CUDA
 * graph and zim_batch_run replays it.  Band heights and persistent CTAs per SM
 * are tunables, chosen by zim_batch_autotune. */
typedef struct zim_batch zim_batch;

typedef struct zim_batch_pair {
    zim_decode_config decode;
    int sample_type;         /* ZIM_SAMPLE_U8 / ZIM_SAMPLE_U16 */
    int rows, cols;          /* camera image size: must equal its calibration's */
    int calib;               /* index into the batch's calibrations */
    int pha_f;               /* <= 0: zim_decode_max_order(&decode) */
    const void* frames[2];   /* device frame stacks, left and right */
    float* xyz;              /* device outputs, rect_h*rect_w of the calibration */
    uint8_t* mask;
    float* disp;             /* optional: the (median-filtered) disparity */
    /* optional: the grid filters of this pair (use_sor, use_mls,
     * use_metric_gaussian and their parameters are read from it); NULL: those
     * of the submission's config.  The pixel-domain stages, the reprojection
     * frame (use_rectified_coords) and its rays come from the submission's
     * config for every pair. */
    const zim_recon_config* filters;
} zim_batch_pair;

typedef struct zim_batch_tuning {
    int decode_rows;   /* 8-pixel tile rows per decode work item */
    int match_rows;    /* rectified rows per rectify+match work item */
    int filter_rows;   /* 8-pixel tile rows per median/filter work item */
    int ctas_per_sm;   /* persistent CTAs per SM (capped by occupancy) */
} zim_batch_tuning;

/* Rectification of every calibration (as zim_set_calibration) into a batch
 * bound to ctx's device. */
ZIM_API zim_status zim_batch_create(zim_ctx* ctx, const zim_stereo_calib* calibs, int n_calibs,
                                    int use_full_left_rectification, zim_batch** out);
/* Destroys a batch; it reads nothing of its context, so it may run after
 * zim_destroy of that context (as a garbage-collected caller may order them). */
ZIM_API void zim_batch_destroy(zim_batch* batch);
ZIM_API zim_status zim_batch_rect_size(const zim_batch* batch, int calib, int* rect_w, int* rect_h);
/* Validates the pairs, allocates the intermediates, builds the work queues
 * and captures the CUDA graph.  rcfg: zim_recon_config with use_sor, use_mls
 * and use_metric_gaussian 0.  tuning NULL: the last autotuned (else default)
 * tuning.  Replaces any previous submission; synchronises the device. */
ZIM_API zim_status zim_batch_submit(zim_batch* batch, const zim_batch_pair* pairs, int n_pairs,
                                    const zim_recon_config* rcfg, const zim_batch_tuning* tuning);
/* Replays the submitted batch on `stream` (asynchronous). */
ZIM_API zim_status zim_batch_run(zim_batch* batch, void* stream);
/* Times candidate tunings on the submitted batch (each run several times),
 * resubmits with the fastest and returns it and its time per run. */
ZIM_API zim_status zim_batch_autotune(zim_batch* batch, void* stream, zim_batch_tuning* best,
                                      double* best_ms);
ZIM_API zim_status zim_batch_get_tuning(const zim_batch* batch, zim_batch_tuning* out);

/* ---- differentiable sub-pixel matching + reprojection ----
 * No counterpart in the reference (it has no gradients); the forward restates
 * its sub-pixel refinement (JSLAB_PhaseEpipolarReconstructor_V2.cpp:985-1000)
 * and reprojection (:414-461, rectified coordinates) on phase sampled with
 * exact bilinear weights.  The integer decisions (fringe orders, match
 * columns) are inputs and stay fixed; everything else is differentiated.
 *
 * Parameters (FP64 on the host).  Camera c (0 left, 1 right): fx, fy, cx, cy,
 * k1, k2 of its intrinsics and distortion (p1, p2, k3 stay at the calibrated
 * values); baseline = |t|; rot = rotation vector of a right-multiplied update
 * of the right camera's rectifying rotation, R2 <- R2 * exp([rot]x) (an error
 * of the relative rotation).  The rectified virtual cameras (their
 * intrinsics, canvas and the left rectifying rotation) stay those of
 * zim_set_calibration.  Gradient order: fx0 fy0 cx0 cy0 k1_0 k2_0 fx1 fy1 cx1
 * cy1 k1_1 k2_1 baseline rot0 rot1 rot2. */
#define ZIM_DIFF_NPARAMS 16
typedef struct zim_diff_params {
    double cam[2][6]; /* fx, fy, cx, cy, k1, k2 */
    double baseline;
    double rot[3];
} zim_diff_params;

/* The parameters of the calibration set by zim_set_calibration (rot = 0). */
ZIM_API zim_status zim_diff_params_nominal(const zim_ctx* ctx, zim_diff_params* out);

/* Rectifies one camera's decoded phase under `params`: bilinear sampling of
 * 2*pi*order + residual with exact weights (a sample needs its four source
 * taps inside the image and valid, order >= 1; else order 0), order by
 * nearest neighbour; no post-smooth.  Feed both cameras' outputs to zim_match
 * to fix the match columns for zim_diff_forward/backward. */
ZIM_API zim_status zim_diff_rectify(zim_ctx* ctx, const zim_diff_params* params, int cam,
                                    const int32_t* order, const float* residual, int rows,
                                    int cols, int32_t* rect_base, float* rect_res,
                                    int32_t* rect_order, void* stream);

/* One view: both cameras' decoded phase (rows*cols, device), the match columns
 * from zim_match (rect_h*rect_w, -1 = none) and a target plane: the loss of a
 * view is sum over its points of (n . P + d)^2, P in the rectified left frame.
 * A point enters when its four phase samples (left pixel, right columns
 * best-1..best+1) are valid, |disparity| >= 1e-5 and z_min < Z < z_max.
 * Optional device outputs: xyz (rect_h*rect_w*3, 0 where excluded) and mask
 * from the forward; grad_phase[c] (rows*cols) from the backward, ACCUMULATED
 * (+=) with FP32 atomics.  Optional input grad_xyz (rect_h*rect_w*3): an
 * upstream gradient of the points, added to loss_weight * dLoss/dP. */
typedef struct zim_diff_view {
    const int32_t* order[2];
    const float* residual[2];
    const int32_t* best_col;
    double plane[4];
    float* xyz;
    uint8_t* mask;
    const float* grad_xyz;
    float* grad_phase[2];
} zim_diff_view;

/* Sums over all views, reduced in FP64 in a fixed order (bit-reproducible):
 * loss, points used, the gradient of loss_weight * loss (+ the grad_xyz
 * terms) and J^T J of the point-to-plane distances (Gauss-Newton). */
typedef struct zim_diff_result {
    double loss;
    double n_points;
    double grad[ZIM_DIFF_NPARAMS];
    double jtj[ZIM_DIFF_NPARAMS * ZIM_DIFF_NPARAMS];
} zim_diff_result;

/* Forward over n_views views of one rig in one launch: loss and n_points (the
 * other result fields are zeroed), optional xyz/mask.  Synchronises `stream`. */
ZIM_API zim_status zim_diff_forward(zim_ctx* ctx, const zim_diff_params* params,
                                    const zim_diff_view* views, int n_views, int rows, int cols,
                                    double z_min, double z_max, zim_diff_result* out,
                                    void* stream);
/* Adjoint (recomputes the forward): every field of *out, and grad_phase if
 * requested.  Synchronises `stream`. */
ZIM_API zim_status zim_diff_backward(zim_ctx* ctx, const zim_diff_params* params,
                                     const zim_diff_view* views, int n_views, int rows, int cols,
                                     double z_min, double z_max, double loss_weight,
                                     zim_diff_result* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ZIM_H */
