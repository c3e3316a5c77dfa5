// ref_bridge.cpp -- a C interface over the reference's own classes, built
// from the unmodified reference sources into oracle/_ref/libzim_ref.so by
// oracle/ref_build.py.  TEST INFRASTRUCTURE ONLY: the tests call it to pin the
// oracle (and, through fixtures, the CUDA path) to the reference itself.
//
// What it drives, in the reference (src/ = PhaseShiftGrayCode3D/src/):
//   JSLAB_PhaseShiftDecoder::create(config, V2) (JSLAB_PhaseShiftDecoder.cpp:9-29),
//     setImages / startCalculate / getOrderMap / getModulationMap
//     (JSLAB_PhaseShiftDecoder_V2.cpp:6-310), and the decode body's unsmoothed
//     phase and validity (m_body, :184-199,297-300);
//   JSLAB_PhaseEpipolarReconstructor_V2 setCalibrationParams[V2] / setData /
//     startCalculate[_v2] / getDisparityMap (JSLAB_PhaseEpipolarReconstructor_V2.cpp:292-593,915-918),
//     its stereoMatch (:933-1006) and the point-cloud filters (:79-195);
//   applyMLSFilterToPointCloud_CPU (JSLAB_MLS_Filter.cpp:161-420).
// The build defines `private` as `public` so that the decode body, the
// rectified maps and stereoMatch are reachable from here.
#include <cstdio>
#include <cstring>
#include <exception>

#include "JSLAB_MLS_Filter.h"
#include "JSLAB_PhaseEpipolarReconstructor_V2.h"
#include "JSLAB_PhaseShiftDecoder_V2.h"

// Defined (without a header declaration) in JSLAB_PhaseEpipolarReconstructor_V2.cpp:79-195.
void applyGaussianFilterToPointCloudV2(const cv::Mat& src_xyz, const cv::Mat& P, cv::Mat& dst_xyz, const int win_size);
void applyRadiusOutlierFilterToPointCloud(const cv::Mat& src_xyz, const cv::Mat& P, cv::Mat& dst_xyz, cv::Mat& dst_P,
                                          const float search_radius, const int min_neighbors, const int window_size);

// The reference's dispatcher (JSLAB_MLS_Filter.cpp:423-441) names its CUDA MLS
// when CUDA is configured; the CPU build of the reference has no such code, so
// the bridge always selects the CPU filter and this symbol only satisfies the
// link.
void applyMLSFilterToPointCloud_GPU(const cv::Mat&, const cv::Mat&, cv::Mat&, int, float, int, float, int) {
    throw std::runtime_error("the reference's CUDA MLS is not part of the oracle/_ref CPU build");
}

extern "C" {

typedef struct {
    double freq[3];
    int shift_num[3];
    double modulation_threshold;
    double preblur_sigma;
    int avg_three_phase;
    int post_smooth;
    int enable_hdr;
    double hdr_saturation_gray;
    double hdr_min_amplitude;
} zr_decode_cfg;

typedef struct {
    double K[2][9];
    double D[2][5];
    double R[9];
    double t[3];
    int width, height;
} zr_calib;

typedef struct {
    double min_depth, max_depth, grad_threshold;
    int use_rectified_coords, use_disp_median_filter, use_full_left_rectification;
    float radius_search;
    int radius_min_neighbors, radius_window_size;
    int use_mls, mls_window_size;
    float mls_spatial_sigma;
    int mls_polynomial_order;
    float mls_max_radius;
    int mls_iterations;
} zr_recon_cfg;

static char g_err[512];
const char* zr_last_error(void) { return g_err; }

static int fail(const std::exception& e) {
    std::snprintf(g_err, sizeof g_err, "%s", e.what());
    return -2;
}

// Decodes one camera with the reference decoder V2.  frames: F planes of
// rows*cols samples, u8 (depth 0) or f64 (depth 6), in the reference's frame
// order.  phase = startCalculate's output (post-smoothed when configured),
// phase_raw = the decode body's phase before smoothing; both, order, mod and
// valid are rows*cols.  Returns 0, -1 when the factory rejects the config
// (nullptr), -2 on an exception (zr_last_error).
int zr_decode(const zr_decode_cfg* c, const void* frames, int depth, int rows, int cols, double* phase,
              double* phase_raw, int32_t* order, double* mod, uint8_t* valid) {
    try {
        JSLAB_PhaseShiftDecoder::Config cfg;
        for (int i = 0; i < 3; i++) {
            cfg.freq[i] = c->freq[i];
            cfg.shift_num[i] = c->shift_num[i];
        }
        cfg.modulation_threshold = c->modulation_threshold;
        cfg.preblur_sigma = c->preblur_sigma;
        cfg.avg_three_phase = c->avg_three_phase != 0;
        cfg.post_smooth = c->post_smooth != 0;
        cfg.enable_hdr = c->enable_hdr != 0;
        cfg.hdr_saturation_gray = c->hdr_saturation_gray;
        cfg.hdr_min_amplitude = c->hdr_min_amplitude;
        cv::Ptr<JSLAB_PhaseShiftDecoder> dec = JSLAB_PhaseShiftDecoder::create(cfg, JSLAB_PhaseShiftDecoder::Version::V2);
        if (!dec) return -1;
        const int F = c->shift_num[0] + c->shift_num[1] + c->shift_num[2];
        const int type = depth == CV_8U ? CV_8UC1 : CV_64FC1;
        const size_t plane = (size_t)rows * cols * (depth == CV_8U ? 1 : 8);
        std::vector<cv::Mat> images;
        for (int f = 0; f < F; f++)
            images.push_back(cv::Mat(rows, cols, type, (void*)((const uint8_t*)frames + plane * f)).clone());
        dec->setImages(images);
        cv::Mat ph, k, m, raw, v;
        dec->startCalculate(ph);
        dec->getOrderMap(k);
        dec->getModulationMap(m);
        auto* v2 = static_cast<JSLAB_PhaseShiftDecoderV2*>(dec.get());
        v2->m_body->getPhase(raw);
        v2->m_body->getValidMask(v);
        for (int r = 0; r < rows; r++) {
            std::memcpy(phase + (size_t)r * cols, ph.ptr<double>(r), sizeof(double) * cols);
            if (phase_raw) std::memcpy(phase_raw + (size_t)r * cols, raw.ptr<double>(r), sizeof(double) * cols);
            std::memcpy(order + (size_t)r * cols, k.ptr<int>(r), sizeof(int32_t) * cols);
            if (mod) std::memcpy(mod + (size_t)r * cols, m.ptr<double>(r), sizeof(double) * cols);
            if (valid)
                for (int x = 0; x < cols; x++) valid[(size_t)r * cols + x] = v.ptr<uchar>(r)[x] ? 1 : 0;
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

static JSLAB_PhaseEpipolarReconstructor_V2::Config recon_config(const zr_recon_cfg* c) {
    JSLAB_PhaseEpipolarReconstructor_V2::Config cfg;
    cfg.min_depth = c->min_depth;
    cfg.max_depth = c->max_depth;
    cfg.grad_threshold = c->grad_threshold;
    cfg.use_rectified_coords = c->use_rectified_coords != 0;
    cfg.use_disp_median_filter = c->use_disp_median_filter != 0;
    cfg.use_full_left_rectification = c->use_full_left_rectification != 0;
    cfg.radius_search = c->radius_search;
    cfg.radius_min_neighbors = c->radius_min_neighbors;
    cfg.radius_window_size = c->radius_window_size;
    cfg.use_mls = c->use_mls != 0;
    cfg.mls_window_size = c->mls_window_size;
    cfg.mls_spatial_sigma = c->mls_spatial_sigma;
    cfg.use_gpu_mls = false;  // the CPU MLS of JSLAB_MLS_Filter.cpp
    cfg.mls_polynomial_order = c->mls_polynomial_order;
    cfg.mls_max_radius = c->mls_max_radius;
    cfg.mls_iterations = c->mls_iterations;
    return cfg;
}

static cv::Mat f64(int rows, int cols, const double* v) {
    return cv::Mat(rows, cols, CV_64FC1, (void*)v).clone();
}

static JSLAB_StereoCalibParams_V1 calib_params(const zr_calib* c) {
    JSLAB_StereoCalibParams_V1 p;
    for (int cam = 0; cam < 2; cam++) {
        p.camera_matrix[cam] = f64(3, 3, c->K[cam]);
        p.dist_coeffs[cam] = f64(1, 5, c->D[cam]);
    }
    p.R = f64(3, 3, c->R);
    p.t = f64(3, 1, c->t);
    p.image_size = cv::Size(c->width, c->height);
    return p;
}

// A reconstructor with the calibration set (setCalibrationParams; with
// poly maps, setCalibrationParamsV2 whose xyz_calib_coeffs are the three
// CV_32FC4 maps of poly_rows x poly_cols).  *rect_w / *rect_h receive the
// rectified size.  NULL on failure (zr_last_error).
void* zr_recon_create(const zr_recon_cfg* c, const zr_calib* calib, const float* poly_x, const float* poly_y,
                      const float* poly_z, int poly_rows, int poly_cols, int* rect_w, int* rect_h) {
    try {
        auto* rec = new JSLAB_PhaseEpipolarReconstructor_V2(recon_config(c));
        if (poly_x && poly_y && poly_z) {
            JSLAB_StereoCalibParams_V1 v1 = calib_params(calib);
            JSLAB_StereoCalibParams_V2 v2;
            for (int cam = 0; cam < 2; cam++) {
                v2.camera_matrix[cam] = v1.camera_matrix[cam];
                v2.dist_coeffs[cam] = v1.dist_coeffs[cam];
            }
            v2.R = v1.R;
            v2.t = v1.t;
            v2.image_size = v1.image_size;
            const float* maps[3] = {poly_x, poly_y, poly_z};
            for (int k = 0; k < 3; k++)
                v2.xyz_calib_coeffs[k] = cv::Mat(poly_rows, poly_cols, CV_32FC4, (void*)maps[k]).clone();
            rec->setCalibrationParamsV2(v2);
        } else {
            rec->setCalibrationParams(calib_params(calib));
        }
        *rect_w = rec->m_left_remap[0].cols;
        *rect_h = rec->m_left_remap[0].rows;
        return rec;
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}

void zr_recon_destroy(void* rec) { delete static_cast<JSLAB_PhaseEpipolarReconstructor_V2*>(rec); }

// The rectification the reconstructor derived: R1 (9), Q (16) and the left and
// right maps (rect_h*rect_w floats each, NULL to skip).
int zr_recon_rectification(void* rp, double* R1, double* Q, float* lmx, float* lmy, float* rmx, float* rmy) {
    auto* rec = static_cast<JSLAB_PhaseEpipolarReconstructor_V2*>(rp);
    for (int i = 0; i < 9; i++) R1[i] = rec->m_R1.at<double>(i / 3, i % 3);
    for (int i = 0; i < 16; i++) Q[i] = rec->m_Q.at<double>(i / 4, i % 4);
    float* out[4] = {lmx, lmy, rmx, rmy};
    const cv::Mat* maps[4] = {&rec->m_left_remap[0], &rec->m_left_remap[1], &rec->m_right_remap[0],
                              &rec->m_right_remap[1]};
    for (int m = 0; m < 4; m++)
        if (out[m])
            for (int r = 0; r < maps[m]->rows; r++)
                std::memcpy(out[m] + (size_t)r * maps[m]->cols, maps[m]->ptr<float>(r), sizeof(float) * maps[m]->cols);
    return 0;
}

// setData then startCalculate (v2 = 0) or startCalculate_v2 (v2 = 1), on
// source-size (rows x cols) decoded maps.  Outputs are rectified-size:
// xyz (3 floats per pixel), P, the disparity map (getDisparityMap), the
// reprojected cloud before the filters (m_xyz, m_P) and, when non-NULL, the
// rectified phase / order maps setData produced.
int zr_recon_run(void* rp, const double* lph, const double* rph, const int32_t* lk, const int32_t* rk,
                 const double* lmod, int rows, int cols, int pha_f, int v2, float* xyz, uint8_t* P, double* disp,
                 float* raw_xyz, uint8_t* raw_P, double* rect_lph, double* rect_rph, int32_t* rect_lk,
                 int32_t* rect_rk) {
    try {
        auto* rec = static_cast<JSLAB_PhaseEpipolarReconstructor_V2*>(rp);
        cv::Mat L = f64(rows, cols, lph), R = f64(rows, cols, rph), M = f64(rows, cols, lmod);
        cv::Mat LK = cv::Mat(rows, cols, CV_32SC1, (void*)lk).clone(), RK = cv::Mat(rows, cols, CV_32SC1, (void*)rk).clone();
        rec->setData(L, R, LK, RK, M, pha_f);
        cv::Mat x, p, d;
        if (v2)
            rec->startCalculate_v2(x, p);
        else
            rec->startCalculate(x, p);
        rec->getDisparityMap(d);
        const int RH = x.rows, RW = x.cols;
        for (int r = 0; r < RH; r++) {
            std::memcpy(xyz + (size_t)r * RW * 3, x.ptr<float>(r), sizeof(float) * 3 * RW);
            std::memcpy(P + (size_t)r * RW, p.ptr<uchar>(r), RW);
            if (disp) std::memcpy(disp + (size_t)r * RW, d.ptr<double>(r), sizeof(double) * RW);
            if (raw_xyz) std::memcpy(raw_xyz + (size_t)r * RW * 3, rec->m_xyz.ptr<float>(r), sizeof(float) * 3 * RW);
            if (raw_P) std::memcpy(raw_P + (size_t)r * RW, rec->m_P.ptr<uchar>(r), RW);
            if (rect_lph) std::memcpy(rect_lph + (size_t)r * RW, rec->m_left.ptr<double>(r), sizeof(double) * RW);
            if (rect_rph) std::memcpy(rect_rph + (size_t)r * RW, rec->m_right.ptr<double>(r), sizeof(double) * RW);
            if (rect_lk) std::memcpy(rect_lk + (size_t)r * RW, rec->m_left_k.ptr<int>(r), sizeof(int32_t) * RW);
            if (rect_rk) std::memcpy(rect_rk + (size_t)r * RW, rec->m_right_k.ptr<int>(r), sizeof(int32_t) * RW);
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// stereoMatch alone on rectified maps (rows x cols); disp 0 = no match.
int zr_stereo_match(const double* lph, const double* rph, const int32_t* lk, const int32_t* rk, int rows, int cols,
                    int pha_f, double grad_threshold, double* disp) {
    try {
        JSLAB_PhaseEpipolarReconstructor_V2::Config cfg;
        cfg.grad_threshold = grad_threshold;
        JSLAB_PhaseEpipolarReconstructor_V2 rec(cfg);
        rec.m_pha_f = pha_f;  // stereoMatch reads the member, not its argument
        cv::Mat d;
        rec.stereoMatch(f64(rows, cols, lph), f64(rows, cols, rph), cv::Mat(rows, cols, CV_32SC1, (void*)lk).clone(),
                        cv::Mat(rows, cols, CV_32SC1, (void*)rk).clone(), pha_f, d);
        for (int r = 0; r < rows; r++) std::memcpy(disp + (size_t)r * cols, d.ptr<double>(r), sizeof(double) * cols);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

static void copy_cloud(const cv::Mat& x, float* out) {
    for (int r = 0; r < x.rows; r++) std::memcpy(out + (size_t)r * x.cols * 3, x.ptr<float>(r), sizeof(float) * 3 * x.cols);
}

// applyGaussianFilterToPointCloudV2(xyz, P, out, 3).
int zr_px_gaussian(const float* xyz, const uint8_t* P, int rows, int cols, float* out) {
    try {
        cv::Mat X = cv::Mat(rows, cols, CV_32FC3, (void*)xyz).clone(), M = cv::Mat(rows, cols, CV_8UC1, (void*)P).clone();
        cv::Mat o;
        applyGaussianFilterToPointCloudV2(X, M, o, 3);
        copy_cloud(o, out);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// applyRadiusOutlierFilterToPointCloud(xyz, P, out, out_P, radius, min_neighbors, window).
int zr_ror(const float* xyz, const uint8_t* P, int rows, int cols, float radius, int min_neighbors, int window,
           float* out, uint8_t* out_P) {
    try {
        cv::Mat X = cv::Mat(rows, cols, CV_32FC3, (void*)xyz).clone(), M = cv::Mat(rows, cols, CV_8UC1, (void*)P).clone();
        cv::Mat o, op;
        applyRadiusOutlierFilterToPointCloud(X, M, o, op, radius, min_neighbors, window);
        copy_cloud(o, out);
        for (int r = 0; r < rows; r++) std::memcpy(out_P + (size_t)r * cols, op.ptr<uchar>(r), cols);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// applyMLSFilterToPointCloud_CPU(xyz, P, out, window, sigma, order, max_radius, iterations).
int zr_mls(const float* xyz, const uint8_t* P, int rows, int cols, int window, float sigma, int order,
           float max_radius, int iterations, float* out) {
    try {
        cv::Mat X = cv::Mat(rows, cols, CV_32FC3, (void*)xyz).clone(), M = cv::Mat(rows, cols, CV_8UC1, (void*)P).clone();
        cv::Mat o;
        applyMLSFilterToPointCloud_CPU(X, M, o, window, sigma, order, max_radius, iterations);
        copy_cloud(o, out);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

}  // extern "C"
