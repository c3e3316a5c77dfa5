// zim_jslab.hpp -- header-only C++ adapter: the reference's decoder and
// reconstructor classes, same names and call sequence, over the C ABI of
// zim.h (GPU: sm_103a).  Link with libzim_gb300.so and libcudart.
//
// Reference classes mirrored (PhaseShiftGrayCode3D/src/):
//   JSLAB_PhaseShiftDecoder            JSLAB_PhaseShiftDecoder.h:10-92
//   JSLAB_StereoCalibParams_V1         JSLAB_StereoCalibParams_V1.h:9-20
//   JSLAB_StereoCalibParams_V2         JSLAB_StereoCalibParams_V2.h:8-30 (+ the .bin maps)
//   JSLAB_PhaseEpipolarReconstructor_V2 JSLAB_PhaseEpipolarReconstructor_V2.h:11-171
//
// Images are zim::Image<T> (rows x cols x channels, row-major, owning).  When
// OpenCV is available (ZIM_WITH_OPENCV, or <opencv2/core.hpp> found), cv::Mat
// overloads with the reference's exact signatures are added; when PCL is
// available (ZIM_WITH_PCL, or <pcl/point_cloud.h> found), startCalculate can
// fill a pcl::PointCloud<pcl::PointXYZ>.
// Errors: create() returns nullptr for an invalid config (like the
// reference's factory); every other failure throws zim::Error carrying the
// zim_status and zim_last_error() text (the reference throws cv::Exception).
#pragma once

#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "zim.h"

#if defined(ZIM_WITH_OPENCV) || (defined(__has_include) && __has_include(<opencv2/core.hpp>))
#include <opencv2/core.hpp>
#define ZIM_JSLAB_OPENCV 1
#endif
#if defined(ZIM_WITH_PCL) || (defined(__has_include) && __has_include(<pcl/point_cloud.h>))
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
#define ZIM_JSLAB_PCL 1
#endif

namespace zim {

struct Error : std::runtime_error {
    zim_status status;
    Error(zim_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(zim_status s, const zim_ctx* ctx, const char* what) {
    if (s != ZIM_OK) throw Error(s, std::string(what) + ": " + (ctx ? zim_last_error(ctx) : "status " + std::to_string(s)));
}

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(ZIM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct Image {
    int rows = 0, cols = 0, channels = 1;
    std::vector<T> data;
    Image() = default;
    Image(int r, int c, int ch = 1) : rows(r), cols(c), channels(ch), data((size_t)r * c * ch) {}
    T* ptr() { return data.data(); }
    const T* ptr() const { return data.data(); }
    size_t size() const { return data.size(); }
    bool empty() const { return data.empty(); }
};

// Owning device buffer.
template <typename T>
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t n) { resize(n); }
    ~DeviceBuffer() { cudaFree(p_); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    void resize(size_t n) {
        if (n == n_) return;
        cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
        if (n) cuda_check(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)), "cudaMalloc");
        n_ = n;
    }
    T* get() const { return p_; }
    size_t size() const { return n_; }
    void upload(const T* h, size_t n) {
        resize(n);
        cuda_check(cudaMemcpy(p_, h, n * sizeof(T), cudaMemcpyHostToDevice), "upload");
    }
    void download(T* h, size_t n) const { cuda_check(cudaMemcpy(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost), "download"); }

private:
    T* p_ = nullptr;
    size_t n_ = 0;
};

// One zim context, shared by the adapter objects of a thread.
class Context {
public:
    explicit Context(int device = 0) { check(zim_create(device, &ctx_), nullptr, "zim_create"); }
    ~Context() { zim_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    zim_ctx* get() const { return ctx_; }

private:
    zim_ctx* ctx_ = nullptr;
};

}  // namespace zim

// ------------------------------------------------------------ decoder ----

class JSLAB_PhaseShiftDecoder {
public:
    enum class Version { V1, V2 };

    // Fields of the reference Config (JSLAB_PhaseShiftDecoder.h:22-54), then this
    // library's encodings (default: the reference's three-frequency heterodyne).
    struct Config {
        double freq[3];
        int shift_num[3];
        double modulation_threshold = 1.0;
        double preblur_sigma = 3.0;
        bool avg_three_phase = true;
        bool post_smooth = true;
        bool enable_hdr = false;
        double hdr_saturation_gray = 255.0;
        double hdr_min_amplitude = 2.0;
        int encoding = ZIM_ENC_HETERODYNE3;
        int n_freq = 3;
        int gray_bits = 0;
        double freq4 = 0;  // fourth hierarchical frequency
        int shift_num4 = 0;
    };

    // nullptr on an invalid config (the reference factory's behaviour, JSLAB_PhaseShiftDecoder.cpp:9-29).
    // Version V1 selects the reference's V1 decoder, which this library does not provide: nullptr too.
    static std::unique_ptr<JSLAB_PhaseShiftDecoder> create(const Config& config, Version version = Version::V1,
                                                           std::shared_ptr<zim::Context> ctx = nullptr) {
        if (version != Version::V2) return nullptr;
        zim_decode_config c = to_c(config);
        if (zim_decode_validate(&c) != ZIM_OK) return nullptr;
        return std::unique_ptr<JSLAB_PhaseShiftDecoder>(
            new JSLAB_PhaseShiftDecoder(c, ctx ? ctx : std::make_shared<zim::Context>(0)));
    }

    // Frames in the reference order (frequency 0 steps, then 1, then 2; Gray
    // encodings: phase steps, Gray bits MSB first, complementary frame).
    void setImages(const std::vector<zim::Image<uint8_t>>& images) { set_images(images, ZIM_SAMPLE_U8); }
    void setImages(const std::vector<zim::Image<uint16_t>>& images) { set_images(images, ZIM_SAMPLE_U16); }

    // Absolute phase (post-smoothed when Config::post_smooth), CV_64F semantics.
    void startCalculate(zim::Image<double>& phase) {
        decode();
        phase = zim::Image<double>(rows_, cols_);
        zim::DeviceBuffer<double> d(size());
        const int mode = cfg_.enable_hdr ? (cfg_.post_smooth ? 2 : 3) : (cfg_.post_smooth ? 1 : 0);
        zim::check(zim_decode_phase_f64(ctx_->get(), order_.get(), res_.get(), rows_, cols_, mode, d.get(), nullptr),
                   ctx_->get(), "zim_decode_phase_f64");
        d.download(phase.ptr(), size());
    }
    void getOrderMap(zim::Image<int32_t>& k_map) const {
        k_map = zim::Image<int32_t>(rows_, cols_);
        if (decoded_) order_.download(k_map.ptr(), size());
    }
    void getModulationMap(zim::Image<double>& mod_map) const {
        mod_map = zim::Image<double>(rows_, cols_);
        if (!decoded_) return;
        std::vector<float> m(size());
        mod_.download(m.data(), size());
        for (size_t i = 0; i < size(); i++) mod_map.data[i] = m[i];
    }

    // Device-side results for the reconstructor (no host round trip).
    const int32_t* deviceOrder() const { return order_.get(); }
    const float* deviceResidual() const { return res_.get(); }
    int rows() const { return rows_; }
    int cols() const { return cols_; }
    int maxOrder() const { return zim_decode_max_order(&cfg_); }
    bool hdr() const { return cfg_.enable_hdr != 0; }
    std::shared_ptr<zim::Context> context() const { return ctx_; }

#ifdef ZIM_JSLAB_OPENCV
    void setImages(const std::vector<cv::Mat>& images) {
        if (images.empty()) throw zim::Error(ZIM_ERR_INVALID_ARG, "no images");
        const bool u16 = images[0].depth() == CV_16U;
        if (u16) {
            std::vector<zim::Image<uint16_t>> v;
            for (const cv::Mat& m : images) v.push_back(from_mat<uint16_t>(m));
            setImages(v);
        } else {
            std::vector<zim::Image<uint8_t>> v;
            for (const cv::Mat& m : images) v.push_back(from_mat<uint8_t>(m));
            setImages(v);
        }
    }
    void startCalculate(cv::Mat& phase) {
        zim::Image<double> p;
        startCalculate(p);
        cv::Mat(p.rows, p.cols, CV_64FC1, p.ptr()).copyTo(phase);
    }
    void getOrderMap(cv::Mat& k_map) {
        zim::Image<int32_t> k;
        getOrderMap(k);
        cv::Mat(k.rows, k.cols, CV_32SC1, k.ptr()).copyTo(k_map);
    }
    void getModulationMap(cv::Mat& mod_map) {
        zim::Image<double> m;
        getModulationMap(m);
        cv::Mat(m.rows, m.cols, CV_64FC1, m.ptr()).copyTo(mod_map);
    }
#endif

    static zim_decode_config to_c(const Config& c) {
        zim_decode_config d;
        zim_decode_config_default(&d);
        for (int i = 0; i < 3; i++) {
            d.freq[i] = c.freq[i];
            d.shift_num[i] = c.shift_num[i];
        }
        d.freq[3] = c.freq4;
        d.shift_num[3] = c.shift_num4;
        d.modulation_threshold = c.modulation_threshold;
        d.preblur_sigma = c.preblur_sigma;
        d.avg_three_phase = c.avg_three_phase;
        d.post_smooth = c.post_smooth;
        d.enable_hdr = c.enable_hdr;
        d.hdr_saturation_gray = c.hdr_saturation_gray;
        d.hdr_min_amplitude = c.hdr_min_amplitude;
        d.encoding = c.encoding;
        d.n_freq = c.n_freq;
        d.gray_bits = c.gray_bits;
        return d;
    }

private:
    JSLAB_PhaseShiftDecoder(const zim_decode_config& c, std::shared_ptr<zim::Context> ctx) : cfg_(c), ctx_(ctx) {}

    size_t size() const { return (size_t)rows_ * cols_; }

    template <typename T>
    void set_images(const std::vector<zim::Image<T>>& images, int sample_type) {
        const int F = zim_decode_frame_count(&cfg_);
        if ((int)images.size() != F)
            throw zim::Error(ZIM_ERR_INVALID_ARG, "expected " + std::to_string(F) + " images");
        rows_ = images[0].rows;
        cols_ = images[0].cols;
        std::vector<T> stack((size_t)F * size());
        for (int f = 0; f < F; f++) {
            if (images[f].rows != rows_ || images[f].cols != cols_ || images[f].channels != 1)
                throw zim::Error(ZIM_ERR_INVALID_ARG, "images differ in size or are not single-channel");
            std::memcpy(stack.data() + (size_t)f * size(), images[f].ptr(), size() * sizeof(T));
        }
        frames_.upload(reinterpret_cast<const uint8_t*>(stack.data()), stack.size() * sizeof(T));
        sample_type_ = sample_type;
        decoded_ = false;
    }

    void decode() {
        if (decoded_) return;
        if (!frames_.size()) throw zim::Error(ZIM_ERR_INVALID_ARG, "setImages first");
        order_.resize(size());
        res_.resize(size());
        mod_.resize(size());
        zim::check(zim_decode(ctx_->get(), &cfg_, frames_.get(), sample_type_, rows_, cols_, order_.get(), res_.get(),
                              mod_.get(), nullptr, nullptr),
                   ctx_->get(), "zim_decode");
        zim::cuda_check(cudaDeviceSynchronize(), "decode");
        decoded_ = true;
    }

#ifdef ZIM_JSLAB_OPENCV
    template <typename T>
    static zim::Image<T> from_mat(const cv::Mat& m) {
        zim::Image<T> im(m.rows, m.cols);
        for (int r = 0; r < m.rows; r++) std::memcpy(im.ptr() + (size_t)r * m.cols, m.ptr<T>(r), m.cols * sizeof(T));
        return im;
    }
#endif

    zim_decode_config cfg_;
    std::shared_ptr<zim::Context> ctx_;
    zim::DeviceBuffer<uint8_t> frames_;
    zim::DeviceBuffer<int32_t> order_;
    zim::DeviceBuffer<float> res_, mod_;
    int rows_ = 0, cols_ = 0, sample_type_ = ZIM_SAMPLE_U8;
    bool decoded_ = false;
};

// ------------------------------------------------------- calibration ----

struct JSLAB_StereoCalibParams_V1 {
    double camera_matrix[2][9];  // row-major K
    double dist_coeffs[2][5];    // k1 k2 p1 p2 k3
    double R[9];                 // left -> right
    double t[3];
    int image_width = 0, image_height = 0;

    zim_stereo_calib to_c() const {
        zim_stereo_calib c;
        std::memcpy(c.camera_matrix, camera_matrix, sizeof camera_matrix);
        std::memcpy(c.dist_coeffs, dist_coeffs, sizeof dist_coeffs);
        std::memcpy(c.R, R, sizeof R);
        std::memcpy(c.t, t, sizeof t);
        c.width = image_width;
        c.height = image_height;
        return c;
    }
};

// V2: per-pixel coefficient maps xyz_calib_coeffs[0..2] (X, Y, Z), each rows x
// cols x 4 floats (CV_32FC4), read from <base>_rx/_ry/_rz.bin.
struct JSLAB_StereoCalibParams_V2 : JSLAB_StereoCalibParams_V1 {
    zim::Image<float> xyz_calib_coeffs[3];

    // loadMatBinary (JSLAB_StereoCalibParams_V2.cpp:4-17): int type, rows, cols,
    // then the rows.  Float matrices only (CV_32FC1..4); false on a short file.
    static bool loadMatBinary(const std::string& filename, zim::Image<float>& mat) {
        std::ifstream fs(filename, std::ios::binary);
        if (!fs.is_open()) return false;
        int32_t head[3];
        if (!fs.read(reinterpret_cast<char*>(head), sizeof head)) return false;
        const int depth = head[0] & 7, cn = (head[0] >> 3) + 1;
        if (depth != 5 || head[1] < 0 || head[2] < 0) return false;  // CV_32F
        zim::Image<float> m(head[1], head[2], cn);
        if (!fs.read(reinterpret_cast<char*>(m.ptr()), (std::streamsize)(m.size() * sizeof(float)))) return false;
        mat = std::move(m);
        return true;
    }
    // saveMatBinary (JSLAB_StereoCalib_V2.cpp:22-30).
    static bool saveMatBinary(const std::string& filename, const zim::Image<float>& mat) {
        std::ofstream fs(filename, std::ios::binary);
        if (!fs.is_open()) return false;
        const int32_t head[3] = {5 + ((mat.channels - 1) << 3), mat.rows, mat.cols};
        fs.write(reinterpret_cast<const char*>(head), sizeof head);
        fs.write(reinterpret_cast<const char*>(mat.ptr()), (std::streamsize)(mat.size() * sizeof(float)));
        return (bool)fs;
    }
    // The maps of loadStereoCalibParams_V2 (JSLAB_StereoCalibParams_V2.cpp:34-43) for a
    // calibration file name (the part up to its last dot is the base).
    bool loadCoefficientMaps(const std::string& filename) {
        const std::string base = filename.substr(0, filename.find_last_of('.'));
        const char* sfx[3] = {"_rx.bin", "_ry.bin", "_rz.bin"};
        bool ok = true;
        for (int k = 0; k < 3; k++) ok = loadMatBinary(base + sfx[k], xyz_calib_coeffs[k]) && ok;
        return ok;
    }
};

// -------------------------------------------------------- reconstructor ----

class JSLAB_PhaseEpipolarReconstructor_V2 {
public:
    // Reference Config fields (JSLAB_PhaseEpipolarReconstructor_V2.h:18-55) plus
    // this library's filters; defaults as the reference.
    struct Config {
        zim_recon_config c;
        Config() { zim_recon_config_default(&c); }
    };

    explicit JSLAB_PhaseEpipolarReconstructor_V2(const Config& config, std::shared_ptr<zim::Context> ctx = nullptr)
        : cfg_(config.c), ctx_(ctx ? ctx : std::make_shared<zim::Context>(0)) {}

    void setCalibrationParams(const JSLAB_StereoCalibParams_V1& params) {
        const zim_stereo_calib c = params.to_c();
        zim::check(zim_set_calibration(ctx_->get(), &c, cfg_.use_full_left_rectification), ctx_->get(),
                   "zim_set_calibration");
        zim::check(zim_get_rectification(ctx_->get(), nullptr, nullptr, nullptr, nullptr, nullptr, &rw_, &rh_),
                   ctx_->get(), "zim_get_rectification");
        src_w_ = params.image_width;
        src_h_ = params.image_height;
    }

    // setCalibrationParamsV2 (V2.cpp:340-366): the V1 geometry, then the
    // coefficient maps when all three are present (4 channels each).
    void setCalibrationParamsV2(const JSLAB_StereoCalibParams_V2& params) {
        setCalibrationParams(params);
        const zim::Image<float>* m = params.xyz_calib_coeffs;
        use_v2_ = !m[0].empty() && !m[1].empty() && !m[2].empty();
        zim_ctx* c = ctx_->get();
        if (!use_v2_) {
            zim::check(zim_set_poly_calib(c, nullptr, nullptr, nullptr, 0, 0), c, "zim_set_poly_calib");
            return;
        }
        for (int k = 0; k < 3; k++)
            if (m[k].channels != 4 || m[k].rows != m[0].rows || m[k].cols != m[0].cols)
                throw zim::Error(ZIM_ERR_INVALID_ARG, "coefficient maps are rows x cols x 4");
        zim::check(zim_set_poly_calib(c, m[0].ptr(), m[1].ptr(), m[2].ptr(), m[0].rows, m[0].cols), c,
                   "zim_set_poly_calib");
    }

    // setData (JSLAB_PhaseEpipolarReconstructor_V2.h:67-69): absolute phase maps
    // (already post-smoothed by the decoder) and order maps.  The modulation
    // map is accepted for signature parity; the V2 path does not use it.
    void setData(const zim::Image<double>& left, const zim::Image<double>& right, const zim::Image<int32_t>& left_k,
                 const zim::Image<int32_t>& right_k, const zim::Image<double>& /*left_mod*/, int pha_f) {
        const zim::Image<double>* ph[2] = {&left, &right};
        const zim::Image<int32_t>* k[2] = {&left_k, &right_k};
        const size_t n = (size_t)src_w_ * src_h_;
        for (int c = 0; c < 2; c++) {
            if ((size_t)ph[c]->size() != n || k[c]->size() != n)
                throw zim::Error(ZIM_ERR_INVALID_ARG, "phase / order size differs from the calibration");
            std::vector<float> res(n);
            for (size_t i = 0; i < n; i++) res[i] = (float)(ph[c]->data[i] - 6.283185307179586 * k[c]->data[i]);
            order_[c].upload(k[c]->ptr(), n);
            res_[c].upload(res.data(), n);
        }
        smooth_mode_ = 0;  // the maps come smoothed (invalid pixels as phase 0, order -1 or 0)
        pha_f_ = pha_f;
    }

    // The same straight from two V2 decoders' device results (no host copies).
    void setData(const JSLAB_PhaseShiftDecoder& left, const JSLAB_PhaseShiftDecoder& right, int pha_f = 0,
                 bool post_smooth = true) {
        const size_t n = (size_t)src_w_ * src_h_;
        if ((size_t)left.rows() * left.cols() != n || (size_t)right.rows() * right.cols() != n)
            throw zim::Error(ZIM_ERR_INVALID_ARG, "decoder size differs from the calibration");
        const JSLAB_PhaseShiftDecoder* d[2] = {&left, &right};
        for (int c = 0; c < 2; c++) {
            order_[c].resize(n);
            res_[c].resize(n);
            zim::cuda_check(cudaMemcpy(order_[c].get(), d[c]->deviceOrder(), n * 4, cudaMemcpyDeviceToDevice), "copy");
            zim::cuda_check(cudaMemcpy(res_[c].get(), d[c]->deviceResidual(), n * 4, cudaMemcpyDeviceToDevice), "copy");
        }
        smooth_mode_ = left.hdr() ? (post_smooth ? 2 : 3) : (post_smooth ? 1 : 0);
        pha_f_ = pha_f > 0 ? pha_f : left.maxOrder();
    }

    // startCalculate (…V2.h:77): organised xyz (3 channels) and the valid mask P.
    void startCalculate(zim::Image<float>& xyz, zim::Image<uint8_t>& P) {
        run();
        xyz = zim::Image<float>(rh_, rw_, 3);
        P = zim::Image<uint8_t>(rh_, rw_);
        xyz_.download(xyz.ptr(), xyz.size());
        mask_.download(P.ptr(), P.size());
    }

    // startCalculate_v2 (…V2.h, V2.cpp:482-593): the same chain with the
    // per-pixel polynomial reprojection; no point without coefficient maps.
    void startCalculate_v2(zim::Image<float>& xyz, zim::Image<uint8_t>& P) {
        run(use_v2_ ? 1 : -1);
        xyz = zim::Image<float>(rh_, rw_, 3);
        P = zim::Image<uint8_t>(rh_, rw_);
        xyz_.download(xyz.ptr(), xyz.size());
        mask_.download(P.ptr(), P.size());
    }

    // The cloud as PCL PointXYZ records (x, y, z, pad), valid points in row order.
    void startCalculate(std::vector<zim_point_xyz>& cloud) {
        run();
        zim::DeviceBuffer<zim_point_xyz> pts((size_t)rw_ * rh_);
        zim::DeviceBuffer<uint64_t> cnt(1);
        zim::check(zim_compact_points(ctx_->get(), xyz_.get(), mask_.get(), rh_, rw_, pts.get(), cnt.get(), nullptr),
                   ctx_->get(), "zim_compact_points");
        uint64_t n = 0;
        cnt.download(&n, 1);
        cloud.resize(n);
        if (n) pts.download(cloud.data(), n);
    }

    void getDisparityMap(zim::Image<float>& disp) const {
        disp = zim::Image<float>(rh_, rw_);
        if (disp_.size()) disp_.download(disp.ptr(), disp.size());
    }

    // rectifyLeftImage (V2.cpp:920-924): 8-bit left image into the rectified frame.
    void rectifyLeftImage(const zim::Image<uint8_t>& image, zim::Image<uint8_t>& rectified) const {
        if (image.empty()) {
            rectified = zim::Image<uint8_t>();
            return;
        }
        zim::DeviceBuffer<uint8_t> src(image.size()), dst((size_t)rw_ * rh_);
        src.upload(image.ptr(), image.size());
        zim::check(zim_rectify_image(ctx_->get(), 0, src.get(), image.rows, image.cols, dst.get(), nullptr),
                   ctx_->get(), "zim_rectify_image");
        rectified = zim::Image<uint8_t>(rh_, rw_);
        dst.download(rectified.ptr(), rectified.size());
    }

    std::shared_ptr<zim::Context> context() const { return ctx_; }

#ifdef ZIM_JSLAB_PCL
    void startCalculate(pcl::PointCloud<pcl::PointXYZ>& cloud) {
        std::vector<zim_point_xyz> pts;
        startCalculate(pts);
        cloud.clear();
        cloud.reserve(pts.size());
        for (const zim_point_xyz& p : pts) cloud.push_back(pcl::PointXYZ(p.x, p.y, p.z));
    }
#endif
#ifdef ZIM_JSLAB_OPENCV
    void setData(const cv::Mat& left, const cv::Mat& right, const cv::Mat& left_k, const cv::Mat& right_k,
                 const cv::Mat& left_mod, int pha_f) {
        auto d = [](const cv::Mat& m) {
            zim::Image<double> im(m.rows, m.cols);
            for (int r = 0; r < m.rows; r++) std::memcpy(im.ptr() + (size_t)r * m.cols, m.ptr<double>(r), m.cols * 8);
            return im;
        };
        auto k = [](const cv::Mat& m) {
            zim::Image<int32_t> im(m.rows, m.cols);
            for (int r = 0; r < m.rows; r++) std::memcpy(im.ptr() + (size_t)r * m.cols, m.ptr<int32_t>(r), m.cols * 4);
            return im;
        };
        setData(d(left), d(right), k(left_k), k(right_k), left_mod.empty() ? zim::Image<double>() : d(left_mod), pha_f);
    }
    void startCalculate(cv::Mat& xyz, cv::Mat& P) {
        zim::Image<float> x;
        zim::Image<uint8_t> m;
        startCalculate(x, m);
        cv::Mat(x.rows, x.cols, CV_32FC3, x.ptr()).copyTo(xyz);
        cv::Mat(m.rows, m.cols, CV_8UC1, m.ptr()).copyTo(P);
    }
    void startCalculate_v2(cv::Mat& xyz, cv::Mat& P) {
        zim::Image<float> x;
        zim::Image<uint8_t> m;
        startCalculate_v2(x, m);
        cv::Mat(x.rows, x.cols, CV_32FC3, x.ptr()).copyTo(xyz);
        cv::Mat(m.rows, m.cols, CV_8UC1, m.ptr()).copyTo(P);
    }
    void getDisparityMap(cv::Mat& disp) const {
        zim::Image<float> d;
        getDisparityMap(d);
        cv::Mat(d.rows, d.cols, CV_32FC1, d.ptr()).copyTo(disp);
    }
#endif

private:
    // model: 0 Q matrix, 1 polynomial maps, -1 no point (startCalculate_v2 without maps)
    void run(int model = 0) {
        if (!order_[0].size()) throw zim::Error(ZIM_ERR_INVALID_ARG, "setData first");
        zim_ctx* c = ctx_->get();
        const size_t r = (size_t)rw_ * rh_;
        DevRect rect[2];
        for (int cam = 0; cam < 2; cam++) {
            rect[cam].base.resize(r);
            rect[cam].res.resize(r);
            rect[cam].order.resize(r);
            zim::check(zim_rectify(c, cam, order_[cam].get(), res_[cam].get(), src_h_, src_w_, smooth_mode_,
                                   rect[cam].base.get(), rect[cam].res.get(), rect[cam].order.get(), nullptr),
                       c, "zim_rectify");
        }
        zim::DeviceBuffer<float> raw(r);
        zim::check(zim_match(c, rect[0].base.get(), rect[0].res.get(), rect[0].order.get(), rect[1].base.get(),
                             rect[1].res.get(), rect[1].order.get(), rh_, rw_, pha_f_, cfg_.grad_threshold, raw.get(),
                             nullptr, nullptr),
                   c, "zim_match");
        disp_.resize(r);
        xyz_.resize(3 * r);
        mask_.resize(r);
        zim_recon_config rc = cfg_;
        rc.reproject_model = model > 0 ? model : 0;
        zim::check(zim_median_reproject(c, &rc, raw.get(), rh_, rw_, disp_.get(), xyz_.get(), mask_.get(), nullptr), c,
                   "zim_median_reproject");
        if (model < 0) {
            zim::cuda_check(cudaMemset(xyz_.get(), 0, 12 * r), "clear");
            zim::cuda_check(cudaMemset(mask_.get(), 0, r), "clear");
        } else {
            filters();
        }
        zim::cuda_check(cudaDeviceSynchronize(), "reconstruct");
    }

    // The filter chain of zim_reconstruct_pair, in place on xyz_ / mask_.
    void filters() {
        zim_ctx* c = ctx_->get();
        const size_t r = (size_t)rw_ * rh_;
        zim::DeviceBuffer<float> x2(3 * r);
        zim::DeviceBuffer<uint8_t> m2(r);
        auto swap_in = [&](bool mask_too) {
            zim::cuda_check(cudaMemcpy(xyz_.get(), x2.get(), 12 * r, cudaMemcpyDeviceToDevice), "copy");
            if (mask_too) zim::cuda_check(cudaMemcpy(mask_.get(), m2.get(), r, cudaMemcpyDeviceToDevice), "copy");
        };
        if (cfg_.use_px_gaussian) {
            zim::check(zim_filter_px_gaussian(c, xyz_.get(), mask_.get(), rh_, rw_, x2.get(),
                                              cfg_.px_gaussian_updates_mask ? m2.get() : nullptr, nullptr),
                       c, "zim_filter_px_gaussian");
            swap_in(cfg_.px_gaussian_updates_mask != 0);
        }
        if (cfg_.use_ror) {
            zim::check(zim_filter_ror(c, xyz_.get(), mask_.get(), rh_, rw_, cfg_.radius_search,
                                      cfg_.radius_min_neighbors, cfg_.radius_window_size, x2.get(), m2.get(), nullptr),
                       c, "zim_filter_ror");
            swap_in(true);
        }
        if (cfg_.use_sor) {
            zim::check(zim_filter_sor(c, xyz_.get(), mask_.get(), rh_, rw_, cfg_.sor_mean_k, cfg_.sor_std_mul,
                                      m2.get(), nullptr, nullptr),
                       c, "zim_filter_sor");
            zim::cuda_check(cudaMemcpy(mask_.get(), m2.get(), r, cudaMemcpyDeviceToDevice), "copy");
        }
        if (cfg_.use_mls) {
            zim::check(zim_filter_mls(c, xyz_.get(), mask_.get(), rh_, rw_, cfg_.mls_window_size,
                                      cfg_.mls_spatial_sigma, cfg_.mls_polynomial_order, cfg_.mls_max_radius,
                                      cfg_.mls_iterations, x2.get(), nullptr),
                       c, "zim_filter_mls");
            swap_in(false);
        }
        if (cfg_.use_metric_gaussian) {
            zim::check(zim_filter_metric_gaussian(c, xyz_.get(), mask_.get(), rh_, rw_, cfg_.metric_gaussian_sigma,
                                                  x2.get(), nullptr),
                       c, "zim_filter_metric_gaussian");
            swap_in(false);
        }
    }

    struct DevRect {
        zim::DeviceBuffer<int32_t> base, order;
        zim::DeviceBuffer<float> res;
    };

    zim_recon_config cfg_;
    std::shared_ptr<zim::Context> ctx_;
    int src_w_ = 0, src_h_ = 0, rw_ = 0, rh_ = 0, pha_f_ = 0;
    int smooth_mode_ = 0;  // zim_rectify post_smooth mode
    bool use_v2_ = false;  // coefficient maps set (m_use_v2_coeffs)
    zim::DeviceBuffer<int32_t> order_[2];
    zim::DeviceBuffer<float> res_[2];
    zim::DeviceBuffer<float> disp_, xyz_;
    zim::DeviceBuffer<uint8_t> mask_;
};

// ----------------------------------------------------------------- outputs ----
// The reference drivers' writers (main.cpp:85-184, JSLAB_PhaseDisparityExporter.cpp:115-141).
// The PLY vertex body is packed on the GPU (zim_pack_ply) and copied out once.

namespace zim {
inline bool write_ply(Context& ctx, const Image<float>& xyz, const Image<uint8_t>& P, const Image<uint8_t>* gray,
                      const std::string& file_name) {
    if (xyz.channels != 3 || xyz.rows != P.rows || xyz.cols != P.cols || P.channels != 1) return false;
    const bool with_gray = gray != nullptr;
    const size_t n = (size_t)P.rows * P.cols, rec = with_gray ? 15 : 12;
    DeviceBuffer<float> dx(xyz.size());
    DeviceBuffer<uint8_t> dm(n), dg(with_gray && !gray->empty() ? n : 0), body(n * rec);
    DeviceBuffer<uint64_t> cnt(1);
    dx.upload(xyz.ptr(), xyz.size());
    dm.upload(P.ptr(), n);
    if (dg.size()) dg.upload(gray->ptr(), n);
    check(zim_pack_ply(ctx.get(), dx.get(), dm.get(), dg.size() ? dg.get() : nullptr, with_gray ? 1 : 0, P.rows,
                       P.cols, body.get(), cnt.get(), nullptr),
          ctx.get(), "zim_pack_ply");
    uint64_t count = 0;
    cnt.download(&count, 1);
    std::vector<uint8_t> h(count * rec);
    if (count) body.download(h.data(), h.size());
    std::ofstream fs(file_name, std::ios::binary);
    if (!fs.is_open()) return false;
    fs << "ply\nformat binary_little_endian 1.0\nelement vertex " << count << "\n"
       << "property float x\nproperty float y\nproperty float z\n";
    if (with_gray) fs << "property uchar red\nproperty uchar green\nproperty uchar blue\n";
    fs << "end_header\n";
    fs.write(reinterpret_cast<const char*>(h.data()), (std::streamsize)h.size());
    return (bool)fs;
}
}  // namespace zim

inline bool savePointCloudToPlyBinary(zim::Context& ctx, const zim::Image<float>& xyz, const zim::Image<uint8_t>& P,
                                      const std::string& file_name) {
    return zim::write_ply(ctx, xyz, P, nullptr, file_name);
}

// gray_image: the rectified left image (same size), or empty for white points.
inline bool savePointCloudToPlyBinaryWithGray(zim::Context& ctx, const zim::Image<float>& xyz,
                                              const zim::Image<uint8_t>& P, const zim::Image<uint8_t>& gray_image,
                                              const std::string& file_name) {
    if (!gray_image.empty() && (gray_image.rows != P.rows || gray_image.cols != P.cols || gray_image.channels != 1))
        return false;
    return zim::write_ply(ctx, xyz, P, &gray_image, file_name);
}

// "x y z" lines of the points with -10000 < z < 10000 and |z| > 0.0001.
inline bool saveToTxt(const zim::Image<float>& xyz, const std::string& filename) {
    std::ofstream out(filename);
    if (!out.is_open()) return false;
    for (size_t i = 0; i + 2 < xyz.size(); i += 3) {
        const float x = xyz.data[i], y = xyz.data[i + 1], z = xyz.data[i + 2];
        if (z > -10000 && z < 10000 && std::fabs(z) > 0.0001f) out << x << " " << y << " " << z << "\n";
    }
    return true;
}

// Row-major doubles plus the info text of the reference's exporter.
inline bool saveRaw64F(const zim::Image<double>& data, const std::string& raw_path, const std::string& info_path) {
    if (data.empty() || data.channels != 1) return false;
    std::ofstream raw(raw_path, std::ios::binary);
    if (!raw.is_open()) return false;
    raw.write(reinterpret_cast<const char*>(data.ptr()), (std::streamsize)(data.size() * sizeof(double)));
    raw.close();
    std::ofstream info(info_path);
    if (info.is_open())
        info << "rows " << data.rows << "\n"
             << "cols " << data.cols << "\n"
             << "type CV_64FC1 (double)\n"
             << "layout row-major, one double per pixel\n"
             << "rows/cols written on the FIRST line as 'rows cols' for convenience\n";
    return true;
}
