// zim_cv.cpp -- bodies of the OpenCV stand-ins declared in
// opencv2/zim_cv.hpp.  TEST INFRASTRUCTURE ONLY (the oracle/_ref build).
//
// Mat bookkeeping is written here; every image-processing primitive forwards
// to the oracle's restatement of the documented OpenCV behaviour
// (oracle/zim_oracle.c), so the reference built on this shim and the oracle
// share those primitives bit for bit.
#include "opencv2/zim_cv.hpp"

#include <omp.h>

#include "../zim_oracle.h"

namespace cv {

namespace {

template <class T>
void fill_typed(Mat& m, const Scalar& v) {
    const int cn = m.channels();
    for (int r = 0; r < m.rows; r++) {
        T* p = m.ptr<T>(r);
        for (int c = 0; c < m.cols; c++)
            for (int k = 0; k < cn; k++) p[(size_t)c * cn + k] = static_cast<T>(v.val[k < 4 ? k : 3]);
    }
}

// OpenCV's saturate_cast: round to nearest (ties to even) and clamp for
// integer targets, a plain conversion for floating ones.
template <class T>
T sat(double v) {
    if (std::is_floating_point<T>::value) return static_cast<T>(v);
    double r = std::nearbyint(v);
    const double lo = (double)std::numeric_limits<T>::lowest(), hi = (double)std::numeric_limits<T>::max();
    return static_cast<T>(r < lo ? lo : (r > hi ? hi : r));
}

double get_as_double(const Mat& m, int r, int c, int k) {
    const int cn = m.channels();
    switch (m.depth()) {
    case CV_8U: return m.ptr<uint8_t>(r)[(size_t)c * cn + k];
    case CV_8S: return m.ptr<int8_t>(r)[(size_t)c * cn + k];
    case CV_16U: return m.ptr<uint16_t>(r)[(size_t)c * cn + k];
    case CV_16S: return m.ptr<int16_t>(r)[(size_t)c * cn + k];
    case CV_32S: return m.ptr<int32_t>(r)[(size_t)c * cn + k];
    case CV_32F: return m.ptr<float>(r)[(size_t)c * cn + k];
    case CV_64F: return m.ptr<double>(r)[(size_t)c * cn + k];
    }
    throw Exception("unsupported depth", __FILE__, __LINE__);
}

void set_from_double(Mat& m, int r, int c, int k, double v) {
    const int cn = m.channels();
    const size_t i = (size_t)c * cn + k;
    switch (m.depth()) {
    case CV_8U: m.ptr<uint8_t>(r)[i] = sat<uint8_t>(v); return;
    case CV_8S: m.ptr<int8_t>(r)[i] = sat<int8_t>(v); return;
    case CV_16U: m.ptr<uint16_t>(r)[i] = sat<uint16_t>(v); return;
    case CV_16S: m.ptr<int16_t>(r)[i] = sat<int16_t>(v); return;
    case CV_32S: m.ptr<int32_t>(r)[i] = sat<int32_t>(v); return;
    case CV_32F: m.ptr<float>(r)[i] = sat<float>(v); return;
    case CV_64F: m.ptr<double>(r)[i] = v; return;
    }
    throw Exception("unsupported depth", __FILE__, __LINE__);
}

// A continuous copy of a matrix's f64 entries (K, D, R, P arguments).
std::vector<double> as_f64(const Mat& m) {
    std::vector<double> v;
    if (m.empty()) return v;
    v.reserve(m.total() * m.channels());
    for (int r = 0; r < m.rows; r++)
        for (int c = 0; c < m.cols; c++)
            for (int k = 0; k < m.channels(); k++) v.push_back(get_as_double(m, r, c, k));
    return v;
}

Mat f64_mat(int rows, int cols, const double* v) {
    Mat m(rows, cols, CV_64FC1);
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) m.at<double>(r, c) = v[r * cols + c];
    return m;
}

Mat continuous(const Mat& m) { return m.isContinuous() ? m : m.clone(); }

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (the textbook
// method); used only for the small least-squares pseudo-inverses of the HDR
// fit.  Eigenvalues in ev, eigenvectors in the columns of V.
void jacobi3(const double A_in[3][3], double ev[3], double V[3][3]) {
    double A[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { A[i][j] = A_in[i][j]; V[i][j] = i == j ? 1.0 : 0.0; }
    for (int sweep = 0; sweep < 64; sweep++) {
        double off = std::fabs(A[0][1]) + std::fabs(A[0][2]) + std::fabs(A[1][2]);
        if (off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (A[p][q] == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; i++) ev[i] = A[i][i];
}

void gram3(const Mat& a, double G[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int r = 0; r < a.rows; r++) s += a.at<double>(r, i) * a.at<double>(r, j);
            G[i][j] = s;
        }
}

}  // namespace

Mat& Mat::operator=(const Scalar& v) {
    if (empty()) return *this;
    switch (depth()) {
    case CV_8U: fill_typed<uint8_t>(*this, v); break;
    case CV_8S: fill_typed<int8_t>(*this, v); break;
    case CV_16U: fill_typed<uint16_t>(*this, v); break;
    case CV_16S: fill_typed<int16_t>(*this, v); break;
    case CV_32S: fill_typed<int32_t>(*this, v); break;
    case CV_32F: fill_typed<float>(*this, v); break;
    case CV_64F: fill_typed<double>(*this, v); break;
    default: throw Exception("unsupported depth", __FILE__, __LINE__);
    }
    return *this;
}

Mat& Mat::setTo(const Scalar& v, const Mat& mask) {
    if (mask.empty()) return *this = v;
    CV_Assert(mask.rows == rows && mask.cols == cols && mask.depth() == CV_8U);
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++)
            if (mask.ptr<uint8_t>(r)[c])
                for (int k = 0; k < channels(); k++) set_from_double(*this, r, c, k, v.val[k < 4 ? k : 3]);
    return *this;
}

void Mat::convertTo(Mat& dst, int rtype, double alpha, double beta) const {
    if (empty()) { dst.release(); return; }
    const int dt = CV_MAKETYPE(CV_MAT_DEPTH(rtype), channels());
    Mat out(rows, cols, dt);
    const bool scale = !(alpha == 1.0 && beta == 0.0);
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++)
            for (int k = 0; k < channels(); k++) {
                double v = get_as_double(*this, r, c, k);
                if (scale) v = v * alpha + beta;
                set_from_double(out, r, c, k, v);
            }
    dst = out;
}

Mat Mat::t() const {
    Mat out(cols, rows, type());
    const size_t es = elemSize();
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) std::memcpy(out.ptr(c) + (size_t)r * es, ptr(r) + (size_t)c * es, es);
    return out;
}

Mat operator*(const Mat& a, const Mat& b) {
    CV_Assert(a.cols == b.rows && a.type() == b.type() && a.channels() == 1);
    CV_Assert(a.depth() == CV_32F || a.depth() == CV_64F);
    Mat out(a.rows, b.cols, a.type());
    for (int i = 0; i < a.rows; i++)
        for (int j = 0; j < b.cols; j++) {
            double s = 0;  // the product of two floats is exact in double
            for (int k = 0; k < a.cols; k++) s += get_as_double(a, i, k, 0) * get_as_double(b, k, j, 0);
            set_from_double(out, i, j, 0, s);
        }
    return out;
}

Mat operator==(const Mat& a, double v) {
    Mat out(a.rows, a.cols, CV_MAKETYPE(CV_8U, a.channels()));
    for (int r = 0; r < a.rows; r++)
        for (int c = 0; c < a.cols; c++)
            for (int k = 0; k < a.channels(); k++)
                out.ptr<uint8_t>(r)[(size_t)c * a.channels() + k] = get_as_double(a, r, c, k) == v ? 255 : 0;
    return out;
}

void parallel_for_(const Range& range, const ParallelLoopBody& body, double) {
    const int n = range.end - range.start;
    if (n <= 0) return;
    const int stripe = std::max(1, n / (8 * std::max(1, omp_get_max_threads())));
    const int nstripes = (n + stripe - 1) / stripe;
#pragma omp parallel for schedule(dynamic, 1)
    for (int s = 0; s < nstripes; s++) {
        const int a = range.start + s * stripe;
        body(Range(a, std::min(range.end, a + stripe)));
    }
}

Mat getGaussianKernel(int ksize, double sigma, int ktype) {
    CV_Assert(ksize == 3);
    CV_Assert(ktype == CV_32F || ktype == CV_64F);
    double k[3];
    zo_gaussian_kernel3(sigma, k);
    Mat m(3, 1, ktype);
    for (int i = 0; i < 3; i++) set_from_double(m, i, 0, 0, k[i]);
    return m;
}

void GaussianBlur(const Mat& src, Mat& dst, Size ksize, double sigmaX, double sigmaY, int borderType) {
    CV_Assert(ksize.width == 3 && ksize.height == 3 && borderType == BORDER_REPLICATE);
    CV_Assert(src.type() == CV_64FC1);
    CV_Assert(sigmaY == 0 || sigmaY == sigmaX);
    double k[3];
    zo_gaussian_kernel3(sigmaX, k);
    Mat s = continuous(src);
    Mat out(src.rows, src.cols, CV_64FC1);
    zo_blur3(s.ptr<double>(), out.ptr<double>(), src.rows, src.cols, k);
    dst = out;
}

void medianBlur(const Mat& src, Mat& dst, int ksize) {
    CV_Assert(ksize == 5 && src.type() == CV_32FC1);
    Mat s = continuous(src);
    Mat out(src.rows, src.cols, CV_32FC1);
    zo_median5(s.ptr<float>(), out.ptr<float>(), src.rows, src.cols);
    dst = out;
}

void remap(const Mat& src, Mat& dst, const Mat& map1, const Mat& map2, int interpolation, int borderMode,
           const Scalar& borderValue) {
    CV_Assert(borderMode == BORDER_CONSTANT && borderValue.val[0] == 0);
    CV_Assert(map1.type() == CV_32FC1 && map2.type() == CV_32FC1 && map1.size() == map2.size());
    Mat s = continuous(src), mx = continuous(map1), my = continuous(map2);
    Mat out(map1.rows, map1.cols, src.type());
    if (src.type() == CV_64FC1 && interpolation == INTER_LINEAR)
        zo_remap_linear(s.ptr<double>(), s.rows, s.cols, mx.ptr<float>(), my.ptr<float>(), out.rows, out.cols,
                        out.ptr<double>());
    else if (src.type() == CV_32SC1 && interpolation == INTER_NEAREST)
        zo_remap_nearest(s.ptr<int32_t>(), s.rows, s.cols, mx.ptr<float>(), my.ptr<float>(), out.rows, out.cols,
                         out.ptr<int32_t>());
    else if (src.type() == CV_8UC1 && interpolation == INTER_LINEAR)
        zo_remap_u8(s.ptr<uint8_t>(), s.rows, s.cols, mx.ptr<float>(), my.ptr<float>(), out.rows, out.cols,
                    out.ptr<uint8_t>());
    else
        throw Exception("remap: type / interpolation pair outside the shim", __FILE__, __LINE__);
    dst = out;
}

void max(const Mat& src, double v, Mat& dst) {
    CV_Assert(src.type() == CV_64FC1);
    Mat out(src.rows, src.cols, CV_64FC1);
    for (int r = 0; r < src.rows; r++)
        for (int c = 0; c < src.cols; c++) out.at<double>(r, c) = std::max(src.at<double>(r, c), v);
    dst = out;
}

void divide(const Mat& a, const Mat& b, Mat& dst, double scale) {
    CV_Assert(a.type() == CV_64FC1 && b.type() == CV_64FC1 && a.size() == b.size());
    Mat out(a.rows, a.cols, CV_64FC1);
    for (int r = 0; r < a.rows; r++)
        for (int c = 0; c < a.cols; c++) {
            const double d = b.at<double>(r, c);
            out.at<double>(r, c) = d != 0 ? a.at<double>(r, c) * scale / d : 0.0;
        }
    dst = out;
}

static zo_calib make_calib(const Mat& K1, const Mat& D1, const Mat& K2, const Mat& D2, Size size, const Mat& R,
                           const Mat& T) {
    zo_calib c{};
    const Mat* K[2] = {&K1, &K2};
    const Mat* D[2] = {&D1, &D2};
    for (int cam = 0; cam < 2; cam++) {
        std::vector<double> k = as_f64(*K[cam]), d = as_f64(*D[cam]);
        CV_Assert(k.size() == 9);
        for (int i = 0; i < 9; i++) c.K[cam][i] = k[i];
        for (int i = 0; i < 5; i++) c.D[cam][i] = i < (int)d.size() ? d[i] : 0.0;
    }
    std::vector<double> r = as_f64(R), t = as_f64(T);
    CV_Assert(r.size() == 9 && t.size() == 3);
    for (int i = 0; i < 9; i++) c.R[i] = r[i];
    for (int i = 0; i < 3; i++) c.t[i] = t[i];
    c.width = size.width;
    c.height = size.height;
    return c;
}

void stereoRectify(const Mat& K1, const Mat& D1, const Mat& K2, const Mat& D2, Size imageSize, const Mat& R,
                   const Mat& T, Mat& R1, Mat& R2, Mat& P1, Mat& P2, Mat& Q, int flags, double alpha,
                   Size newImageSize, Rect* roi1, Rect* roi2) {
    // the oracle restates flags = 0 (no CALIB_ZERO_DISPARITY), alpha = -1 and
    // an output size equal to the input size: the reference's only call
    CV_Assert(flags == 0 && alpha == -1.0 && newImageSize == imageSize);
    zo_calib c = make_calib(K1, D1, K2, D2, imageSize, R, T);
    double r1[9], r2[9], p1[12], p2[12], q[16];
    zo_stereo_rectify(&c, r1, r2, p1, p2, q);
    R1 = f64_mat(3, 3, r1);
    R2 = f64_mat(3, 3, r2);
    P1 = f64_mat(3, 4, p1);
    P2 = f64_mat(3, 4, p2);
    Q = f64_mat(4, 4, q);
    if (roi1) *roi1 = Rect();
    if (roi2) *roi2 = Rect();
}

void undistortPoints(const std::vector<Point2f>& src, std::vector<Point2f>& dst, const Mat& K, const Mat& D,
                     const Mat& R, const Mat& P) {
    std::vector<double> k = as_f64(K), d = as_f64(D), r = as_f64(R), p = as_f64(P);
    CV_Assert(k.size() == 9 && (r.empty() || r.size() == 9));
    double d5[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < d.size() && i < 5; i++) d5[i] = d[i];
    std::vector<float> in(2 * src.size()), out(2 * src.size());
    for (size_t i = 0; i < src.size(); i++) { in[2 * i] = src[i].x; in[2 * i + 1] = src[i].y; }
    zo_undistort_points(k.data(), d5, r.empty() ? nullptr : r.data(), p.empty() ? nullptr : p.data(),
                        P.empty() ? 3 : P.cols, in.data(), out.data(), (int)src.size());
    dst.resize(src.size());
    for (size_t i = 0; i < src.size(); i++) dst[i] = Point2f(out[2 * i], out[2 * i + 1]);
}

void initUndistortRectifyMap(const Mat& K, const Mat& D, const Mat& R, const Mat& P, Size size, int m1type,
                             Mat& map1, Mat& map2) {
    CV_Assert(m1type == CV_32FC1 && P.rows == 3 && P.cols == 4);
    std::vector<double> k = as_f64(K), d = as_f64(D), r = as_f64(R), p = as_f64(P);
    double d5[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < d.size() && i < 5; i++) d5[i] = d[i];
    Mat mx(size.height, size.width, CV_32FC1), my(size.height, size.width, CV_32FC1);
    zo_init_rectify_map(k.data(), d5, r.data(), p.data(), size.width, size.height, mx.ptr<float>(),
                        my.ptr<float>());
    map1 = mx;
    map2 = my;
}

SVD::SVD(const Mat& a, int) {
    CV_Assert(a.type() == CV_64FC1 && a.cols == 3 && a.rows >= 3);
    double G[3][3], ev[3], V[3][3];
    gram3(a, G);
    jacobi3(G, ev, V);
    std::sort(ev, ev + 3, [](double x, double y) { return x > y; });
    w = Mat(3, 1, CV_64FC1);
    for (int i = 0; i < 3; i++) w.at<double>(i, 0) = std::sqrt(std::max(ev[i], 0.0));
}

double invert(const Mat& src, Mat& dst, int flags) {
    CV_Assert(flags == DECOMP_SVD && src.type() == CV_64FC1 && src.cols == 3 && src.rows >= 3);
    // A+ = V diag(1 / lambda) V^T A^T for A^T A = V diag(lambda) V^T
    double G[3][3], ev[3], V[3][3];
    gram3(src, G);
    jacobi3(G, ev, V);
    double Gi[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += V[i][k] * V[j][k] / ev[k];
            Gi[i][j] = s;
        }
    Mat out(3, src.rows, CV_64FC1);
    for (int i = 0; i < 3; i++)
        for (int r = 0; r < src.rows; r++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += Gi[i][k] * src.at<double>(r, k);
            out.at<double>(i, r) = s;
        }
    dst = out;
    double mx = std::max(ev[0], std::max(ev[1], ev[2])), mn = std::min(ev[0], std::min(ev[1], ev[2]));
    return mx > 0 ? std::sqrt(std::max(mn, 0.0) / mx) : 0.0;
}

}  // namespace cv
