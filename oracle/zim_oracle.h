/*
 * zim_oracle.h -- FP64 CPU restatement of the PhaseShiftGrayCode3D reconstruction
 * hot path.  TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA library
 * and the timed CPU baseline.  Nothing in the shipped path links or calls it.
 *
 * Parity status: pinned to the reference's own code where the reference has
 * the computation.  This restatement follows the reference source line by line
 * (citations on each function) and restates the OpenCV primitives it calls
 * from their documented behaviour (OpenCV is absent).  The reference's own
 * decoder, reconstructor and MLS sources, compiled against a minimal OpenCV
 * stand-in that calls these same primitives (oracle/ref_build.py,
 * oracle/_ref), must give the same results (tests/test_ref_pin.py).  The
 * primitives themselves and the computations the reference lacks (Gray code,
 * hierarchical unwrapping, SOR, metric Gaussian, adjoint) are checked against
 * analytic known answers (tests/test_oracle_kat.py) and independent
 * implementations.
 *
 * All arrays are row-major, tightly packed.  Decision-margin flag bits are
 * returned so tests can tell a genuine mismatch from an FP32-vs-FP64 decision
 * that sits within eps of its threshold.
 */
#ifndef ZIM_ORACLE_H
#define ZIM_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Encodings (same numbering as zim.h). */
#define ZO_ENC_HETERODYNE3 0
#define ZO_ENC_HIERARCHICAL 1
#define ZO_ENC_GRAYCODE 2
#define ZO_ENC_GRAYCODE_COMPLEMENTARY 3

/* Near-decision flag bits (decode). */
#define ZO_NEAR_WRAP 1u  /* a wrapped phase within eps of +-pi, or two compared phases within eps */
#define ZO_NEAR_ROUND 2u /* a round() argument within eps of a half integer */
#define ZO_NEAR_MOD 4u   /* normalised modulation within eps of the threshold */
#define ZO_NEAR_GRAY 8u  /* complementary-Gray branch phase within eps of +-pi/2 */

typedef struct {
    int encoding;
    int n_freq;            /* heterodyne: 3; hierarchical: 2..4; gray: 1 */
    double freq[4];        /* fringe counts; hierarchical ascending (1, 8, 64) */
    int shift_num[4];      /* phase steps per frequency */
    int gray_bits;         /* Gray-code bits (gray encodings) */
    double modulation_threshold;
    double preblur_sigma;  /* 3x3 Gaussian pre-blur sigma (<=0: OpenCV default) */
    int avg_three_phase;
    int post_smooth;
    int enable_hdr;        /* HDR least squares on raw samples (heterodyne / hierarchical) */
    double hdr_saturation_gray;
    double hdr_min_amplitude;
} zo_decode_cfg;

/* getGaussianKernel(3, sigma) (OpenCV imgproc, documented formula). */
void zo_gaussian_kernel3(double sigma, double k[3]);

/* GaussianBlur(3x3, k (x) k, BORDER_REPLICATE) on an f64 plane. */
void zo_blur3(const double* src, double* dst, int rows, int cols, const double k[3]);

/* Number of input frames the config consumes. */
int zo_frame_count(const zo_decode_cfg* cfg);

/* Decode one camera.  frames: F planes of rows*cols sample values.
 * phase = unsmoothed absolute phase (0 where invalid), order (-1 where invalid
 * with HDR, else 0), mod (frequency-0 normalised modulation), valid (1/0),
 * near (ZO_NEAR_* bits; may be NULL).  With enable_hdr the phase-shift frames
 * are not pre-blurred and each frequency is an HDR least-squares fit. */
int zo_decode(const zo_decode_cfg* cfg, const double* frames, int rows, int cols,
              double* phase, int32_t* order, double* mod, uint8_t* valid, uint8_t* near,
              double eps);

/* Post-decode smoothing: GaussianBlur(3x3, sigma 0) with BORDER_REPLICATE. */
void zo_post_smooth(const double* src, double* dst, int rows, int cols);
/* HDR post-smooth: the blur of the phase divided by the blur of the validity
 * (clamped at 1e-12), 0 where invalid (JSLAB_PhaseShiftDecoder_V2.cpp:280-291). */
void zo_post_smooth_hdr(const double* src, const uint8_t* valid, double* dst, int rows, int cols);

/* ---- calibration / rectification (FP64) ---- */
typedef struct {
    double K[2][9];  /* row-major 3x3 */
    double D[2][5];  /* k1 k2 p1 p2 k3 */
    double R[9];     /* left -> right rotation */
    double t[3];     /* left -> right translation */
    int width, height;
} zo_calib;

void zo_rodrigues_m2v(const double R[9], double r[3]);
void zo_rodrigues_v2m(const double r[3], double R[9]);
void zo_undistort_points(const double K[9], const double D[5], const double* R9,
                         const double* P, int p_cols, const float* src, float* dst, int n);
void zo_stereo_rectify(const zo_calib* c, double R1[9], double R2[9], double P1[12],
                       double P2[12], double Q[16]);
void zo_full_left(const zo_calib* c, const double R1[9], double P1[12], double P2[12],
                  double Q[16], int* rect_w, int* rect_h);
void zo_init_rectify_map(const double K[9], const double D[5], const double R[9],
                         const double P[12], int w, int h, float* mapx, float* mapy);

/* remap INTER_LINEAR (1/32 quantised, BORDER_CONSTANT 0) of an f64 plane. */
void zo_remap_linear(const double* src, int srows, int scols, const float* mapx,
                     const float* mapy, int drows, int dcols, double* dst);
/* remap INTER_LINEAR of an 8-bit image (OpenCV fixed point, BORDER_CONSTANT 0). */
void zo_remap_u8(const uint8_t* src, int srows, int scols, const float* mapx, const float* mapy, int drows,
                 int dcols, uint8_t* dst);
/* remap INTER_NEAREST (BORDER_CONSTANT 0) of an i32 plane. */
void zo_remap_nearest(const int32_t* src, int srows, int scols, const float* mapx,
                      const float* mapy, int drows, int dcols, int32_t* dst);

/* ---- reconstruction ---- */
/* stereoMatch: disp f64 (0 = no match), best right column (-1 = none),
 * near bit 1 = argmin tie within eps, bit 2 = min cost within eps of grad_threshold. */
void zo_stereo_match(const double* lph, const double* rph, const int32_t* lk,
                     const int32_t* rk, int rows, int cols, int pha_f, double grad_threshold,
                     double* disp, int32_t* best, uint8_t* near, double eps);

/* medianBlur(5) on f32, BORDER_REPLICATE. */
void zo_median5(const float* src, float* dst, int rows, int cols);

/* ROI matching (startCalculate_v2_roi): masked left window vs right column window. */
void zo_stereo_match_roi(const double* lph, const int32_t* lk, const uint8_t* lmask, int lcols, const double* rph,
                         const int32_t* rk, int rcols, int rows, int dx_off, int pha_f, double grad_threshold,
                         double* disp, int32_t* best, uint8_t* near, double eps);
/* Per-pixel polynomial reprojection (startCalculate_v2); maps rows*cols*4 floats. */
void zo_poly_reproject(const float* disp, int rows, int cols, const float* mx, const float* my, const float* mz,
                       const double R1[9], double min_depth, double max_depth, int use_rectified, float* xyz,
                       uint8_t* mask);
/* Q reprojection.  near: 1 = depth gate within eps. */
void zo_reproject(const float* disp, int rows, int cols, const double Q[16], const double R1[9],
                  double min_depth, double max_depth, int use_rectified, float* xyz,
                  uint8_t* mask, uint8_t* near, double eps);

/* 3x3 pixel Gaussian filter (sigma 0.7 px).  mask_out may be NULL (CPU keeps
 * the input mask); when given it is the updated mask (GPU semantics). */
void zo_px_gaussian(const float* xyz, const uint8_t* mask, int rows, int cols, float* out,
                    uint8_t* mask_out, uint8_t* near, double eps);

/* Radius outlier filter over a pixel window. */
void zo_ror(const float* xyz, const uint8_t* mask, int rows, int cols, float radius,
            int min_neighbors, int window_size, float* out, uint8_t* mask_out,
            uint8_t* near, double eps);

/* Organised-window MLS, iterations >= 1; out is FP64 (unrounded).  near: 1 = a neighbour within eps of the
 * cut-off.  jitter > 0 perturbs every neighbour offset by a relative factor in
 * [1 - jitter, 1 + jitter] (seeded) to estimate rounding sensitivity. */
void zo_mls(const float* xyz, const uint8_t* mask, int rows, int cols, int window,
            float sigma, int order, float max_radius, int iterations, double* out,
            uint8_t* near, double eps, double jitter, unsigned long long seed);

/* PCL StatisticalOutlierRemoval semantics over the valid points of an organised
 * cloud: mean distance to k nearest neighbours, threshold mean + std_mul*stddev.
 * meandist (may be NULL) receives each point's mean distance (0 for invalid). */
int zo_sor(const float* xyz, const uint8_t* mask, int n, int k, double std_mul,
           uint8_t* mask_out, double* meandist, double* threshold, uint8_t* near, double eps);

/* Metric Gaussian: radius 3 sigma, w = exp(-d^2 / 2 sigma^2), self included. */
void zo_metric_gaussian(const float* xyz, const uint8_t* mask, int n, double sigma,
                        float* out, uint8_t* near, double eps);

/* Differentiable matching + reprojection (zim_oracle_diff.c).  Fixed geometry:
 * nominal rectified-pixel -> ray matrices, p1 p2 k3 per camera, nominal Q and
 * baseline, sizes. */
typedef struct {
    double ir[2][9];
    double dist[2][3];
    double Q[16];
    double baseline0;
    int rect_w, rect_h, src_w, src_h;
} zo_diff_geom;

/* Loss sum (n . P + d)^2 over the points of one view, their count, and (each
 * optional, NULL to skip) the gradient of loss_weight * loss w.r.t. theta
 * (zim_diff_params order), J^T J of the distances, the points / mask and the
 * phase gradients (accumulated, +=).  cells (rect_w*rect_h*8 ints, may be
 * NULL): cells_mode 1 records each sample's bilinear cell, 2 reuses recorded
 * cells, so finite differences see one smooth patch per sample.  gabs (may be
 * NULL) receives, per parameter, the sum over points of |that point's term of
 * the gradient|: gabs[k] / |grad[k]| is the cancellation factor that scales
 * the rounding of the per-point terms into the error of component k. */
void zo_diff_eval(const zo_diff_geom* G, const double theta[16], const int32_t* order_l, const double* res_l,
                  const int32_t* order_r, const double* res_r, const int32_t* best, const double plane[4],
                  double zmin, double zmax, double loss_weight, double* loss, double* npts, double grad[16],
                  double jtj[256], double* xyz, uint8_t* mask, double* gphase_l, double* gphase_r, int32_t* cells,
                  int cells_mode, double gabs[16]);
/* on != 0: zo_diff_eval rounds each sample position (u, v) to FP32 before
 * the bilinear lookup (everything else FP64), to measure the floor FP32
 * positions put under the gradient; 0 restores exact positions. */
void zo_diff_round_positions(int on);

#ifdef __cplusplus
}
#endif
#endif
