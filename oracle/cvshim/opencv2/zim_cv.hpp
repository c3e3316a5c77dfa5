// zim_cv.hpp -- the few OpenCV 4.7 types and functions that the reference's
// decoder, reconstructor and MLS sources use, so that those sources compile
// unmodified for the oracle/_ref build.  TEST INFRASTRUCTURE ONLY: it builds
// the reference as the checker of the oracle; nothing in the library uses it.
//
// Written from OpenCV's documented interface.  The image-processing
// primitives (getGaussianKernel, GaussianBlur, medianBlur, remap,
// stereoRectify, undistortPoints, initUndistortRectifyMap) are not
// reimplemented here: they call the oracle's own restatements
// (oracle/zim_oracle.c), so any difference between the reference built this
// way and the oracle lies in the reference's own code, not in a primitive.
// Those primitives stay "restated from documentation" (OpenCV is absent).
//
// Semantics kept from OpenCV because the reference's arithmetic depends on
// them: Mat assignment shares data (reference counted) and convertTo to a new
// type allocates a new buffer; Vec * scalar multiplies element-wise in the
// element type and Vec / scalar multiplies by the reciprocal (1.f / alpha for
// float); convertTo rounds to nearest for integer targets (saturating).
#pragma once

#include <math.h>    // the C++ <math.h> also puts the float overloads of abs
#include <stdlib.h>  // and friends in the global namespace, as MSVC does
#include <algorithm>
#include <cmath>
#include <limits>
#include <type_traits>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

typedef unsigned char uchar;
typedef unsigned short ushort;

#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_MAKETYPE(depth, cn) ((depth) + (((cn) - 1) << CV_CN_SHIFT))
#define CV_MAT_DEPTH(t) ((t) & 7)
#define CV_MAT_CN(t) ((((t) >> CV_CN_SHIFT) & 63) + 1)
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_16UC1 CV_MAKETYPE(CV_16U, 1)
#define CV_32SC1 CV_MAKETYPE(CV_32S, 1)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)
#define CV_32FC3 CV_MAKETYPE(CV_32F, 3)
#define CV_32FC4 CV_MAKETYPE(CV_32F, 4)
#define CV_64FC1 CV_MAKETYPE(CV_64F, 1)
#define CV_64FC3 CV_MAKETYPE(CV_64F, 3)
#define CV_PI 3.1415926535897932384626433832795

#define CV_Assert(expr)                                                           \
    do {                                                                          \
        if (!(expr)) throw cv::Exception(#expr, __FILE__, __LINE__);              \
    } while (0)

namespace cv {

struct Exception : std::runtime_error {
    Exception(const char* what, const char* file, int line)
        : std::runtime_error(std::string(file) + ":" + std::to_string(line) + ": " + what) {}
};

template <class T>
using Ptr = std::shared_ptr<T>;
template <class T, class... A>
Ptr<T> makePtr(A&&... a) {
    return std::make_shared<T>(std::forward<A>(a)...);
}

template <class T>
struct Point_ {
    T x = 0, y = 0;
    Point_() = default;
    Point_(T x_, T y_) : x(x_), y(y_) {}
};
typedef Point_<int> Point;
typedef Point_<float> Point2f;
typedef Point_<double> Point2d;

template <class T>
struct Size_ {
    T width = 0, height = 0;
    Size_() = default;
    Size_(T w, T h) : width(w), height(h) {}
    bool empty() const { return width <= 0 || height <= 0; }
    T area() const { return width * height; }
};
typedef Size_<int> Size;
typedef Size_<float> Size2f;
template <class T>
inline bool operator==(const Size_<T>& a, const Size_<T>& b) { return a.width == b.width && a.height == b.height; }
template <class T>
inline bool operator!=(const Size_<T>& a, const Size_<T>& b) { return !(a == b); }

struct Rect {
    int x = 0, y = 0, width = 0, height = 0;
    Rect() = default;
    Rect(int x_, int y_, int w, int h) : x(x_), y(y_), width(w), height(h) {}
    bool empty() const { return width <= 0 || height <= 0; }
    Size size() const { return Size(width, height); }
};

struct RotatedRect {
    Point2f center;
    Size2f size;
    float angle = 0;
};

struct Range {
    int start = 0, end = 0;
    Range() = default;
    Range(int s, int e) : start(s), end(e) {}
};

template <class T, int n>
struct Vec {
    T val[n];
    Vec() { for (int i = 0; i < n; i++) val[i] = T(0); }
    Vec(T a, T b) { static_assert(n == 2, ""); val[0] = a; val[1] = b; }
    Vec(T a, T b, T c) { static_assert(n == 3, ""); val[0] = a; val[1] = b; val[2] = c; }
    Vec(T a, T b, T c, T d) { static_assert(n == 4, ""); val[0] = a; val[1] = b; val[2] = c; val[3] = d; }
    T& operator[](int i) { return val[i]; }
    const T& operator[](int i) const { return val[i]; }
    Vec& operator+=(const Vec& o) { for (int i = 0; i < n; i++) val[i] = T(val[i] + o.val[i]); return *this; }
    Vec& operator-=(const Vec& o) { for (int i = 0; i < n; i++) val[i] = T(val[i] - o.val[i]); return *this; }
};
typedef Vec<float, 3> Vec3f;
typedef Vec<float, 4> Vec4f;
typedef Vec<double, 3> Vec3d;

// element-wise product in the element type (OpenCV's Matx scale operation)
template <class T, int n>
inline Vec<T, n> operator*(const Vec<T, n>& a, float alpha) {
    Vec<T, n> r;
    for (int i = 0; i < n; i++) r.val[i] = T(a.val[i] * alpha);
    return r;
}
template <class T, int n>
inline Vec<T, n> operator*(const Vec<T, n>& a, double alpha) {
    Vec<T, n> r;
    for (int i = 0; i < n; i++) r.val[i] = T(a.val[i] * alpha);
    return r;
}
template <class T, int n>
inline Vec<T, n> operator*(float alpha, const Vec<T, n>& a) { return a * alpha; }
template <class T, int n>
inline Vec<T, n> operator*(double alpha, const Vec<T, n>& a) { return a * alpha; }
// division multiplies by the reciprocal, as OpenCV's Vec operator/ does
template <class T, int n>
inline Vec<T, n> operator/(const Vec<T, n>& a, float alpha) { return a * (1.f / alpha); }
template <class T, int n>
inline Vec<T, n> operator/(const Vec<T, n>& a, double alpha) { return a * (1. / alpha); }
template <class T, int n>
inline Vec<T, n> operator+(const Vec<T, n>& a, const Vec<T, n>& b) { Vec<T, n> r = a; r += b; return r; }
template <class T, int n>
inline Vec<T, n> operator-(const Vec<T, n>& a, const Vec<T, n>& b) { Vec<T, n> r = a; r -= b; return r; }

struct Scalar {
    double val[4] = {0, 0, 0, 0};
    Scalar() = default;
    Scalar(double v0, double v1 = 0, double v2 = 0, double v3 = 0) { val[0] = v0; val[1] = v1; val[2] = v2; val[3] = v3; }
    template <class T, int n>
    Scalar(const Vec<T, n>& v) { for (int i = 0; i < n && i < 4; i++) val[i] = v.val[i]; }
    static Scalar all(double v) { return Scalar(v, v, v, v); }
};

class Mat {
public:
    int rows = 0, cols = 0;
    uchar* data = nullptr;
    size_t step = 0;  // bytes per row

    Mat() = default;
    Mat(int r, int c, int type) { create(r, c, type); }
    Mat(Size s, int type) { create(s.height, s.width, type); }
    Mat(int r, int c, int type, const Scalar& v) { create(r, c, type); *this = v; }
    Mat(Size s, int type, const Scalar& v) { create(s.height, s.width, type); *this = v; }
    // wraps caller memory (not owned)
    Mat(int r, int c, int type, void* ext, size_t step_ = 0)
        : rows(r), cols(c), data(static_cast<uchar*>(ext)), type_(type) {
        step = step_ ? step_ : (size_t)c * elemSize();
    }

    void create(int r, int c, int type) {
        if (data && owner_ && r == rows && c == cols && type == type_) return;
        rows = r; cols = c; type_ = type;
        step = (size_t)c * elemSize();
        owner_ = std::make_shared<std::vector<uchar>>((size_t)r * step + 16);
        data = owner_->data();
    }
    void create(Size s, int type) { create(s.height, s.width, type); }
    void release() { owner_.reset(); data = nullptr; rows = cols = 0; step = 0; }

    int type() const { return type_; }
    int depth() const { return CV_MAT_DEPTH(type_); }
    int channels() const { return CV_MAT_CN(type_); }
    size_t elemSize1() const {
        static const size_t s[8] = {1, 1, 2, 2, 4, 4, 8, 2};
        return s[depth()];
    }
    size_t elemSize() const { return elemSize1() * channels(); }
    Size size() const { return Size(cols, rows); }
    size_t total() const { return (size_t)rows * cols; }
    bool empty() const { return data == nullptr || rows <= 0 || cols <= 0; }
    bool isContinuous() const { return step == (size_t)cols * elemSize(); }

    template <class T = uchar>
    T* ptr(int r = 0) { return reinterpret_cast<T*>(data + step * (size_t)r); }
    template <class T = uchar>
    const T* ptr(int r = 0) const { return reinterpret_cast<const T*>(data + step * (size_t)r); }
    template <class T>
    T& at(int r, int c) { return ptr<T>(r)[c]; }
    template <class T>
    const T& at(int r, int c) const { return ptr<T>(r)[c]; }
    // single index: element i of a row or column vector
    template <class T>
    T& at(int i) { return cols == 1 ? ptr<T>(i)[0] : ptr<T>(0)[i]; }
    template <class T>
    const T& at(int i) const { return cols == 1 ? ptr<T>(i)[0] : ptr<T>(0)[i]; }

    Mat clone() const {
        Mat m;
        if (empty()) return m;
        m.create(rows, cols, type_);
        for (int r = 0; r < rows; r++) std::memcpy(m.ptr(r), ptr(r), (size_t)cols * elemSize());
        return m;
    }
    void copyTo(Mat& dst) const {
        if (empty()) { dst.release(); return; }
        if (&dst == this) return;
        Mat m = clone();
        dst = m;
    }
    static Mat zeros(int r, int c, int type) { return Mat(r, c, type, Scalar(0)); }
    static Mat zeros(Size s, int type) { return Mat(s, type, Scalar(0)); }

    Mat& operator=(const Scalar& v);
    Mat& setTo(const Scalar& v) { return *this = v; }
    Mat& setTo(const Scalar& v, const Mat& mask);
    void convertTo(Mat& dst, int rtype, double alpha = 1.0, double beta = 0.0) const;
    Mat t() const;

private:
    int type_ = 0;
    std::shared_ptr<std::vector<uchar>> owner_;
};

Mat operator*(const Mat& a, const Mat& b);  // matrix product (f32 / f64)
Mat operator==(const Mat& a, double v);     // 255 where equal, else 0 (CV_8U)

class ParallelLoopBody {
public:
    virtual ~ParallelLoopBody() {}
    virtual void operator()(const Range& range) const = 0;
};
void parallel_for_(const Range& range, const ParallelLoopBody& body, double nstripes = -1.);

enum { BORDER_CONSTANT = 0, BORDER_REPLICATE = 1 };
enum { INTER_NEAREST = 0, INTER_LINEAR = 1 };
enum { DECOMP_LU = 0, DECOMP_SVD = 1 };

Mat getGaussianKernel(int ksize, double sigma, int ktype = CV_64F);
void GaussianBlur(const Mat& src, Mat& dst, Size ksize, double sigmaX, double sigmaY = 0,
                  int borderType = BORDER_REPLICATE);
void medianBlur(const Mat& src, Mat& dst, int ksize);
void remap(const Mat& src, Mat& dst, const Mat& map1, const Mat& map2, int interpolation,
           int borderMode = BORDER_CONSTANT, const Scalar& borderValue = Scalar());
void max(const Mat& src, double v, Mat& dst);
void divide(const Mat& a, const Mat& b, Mat& dst, double scale = 1.0);
void stereoRectify(const Mat& K1, const Mat& D1, const Mat& K2, const Mat& D2, Size imageSize, const Mat& R,
                   const Mat& T, Mat& R1, Mat& R2, Mat& P1, Mat& P2, Mat& Q, int flags, double alpha,
                   Size newImageSize, Rect* roi1 = nullptr, Rect* roi2 = nullptr);
void undistortPoints(const std::vector<Point2f>& src, std::vector<Point2f>& dst, const Mat& K, const Mat& D,
                     const Mat& R, const Mat& P);
void initUndistortRectifyMap(const Mat& K, const Mat& D, const Mat& R, const Mat& P, Size size, int m1type,
                             Mat& map1, Mat& map2);

// Singular values (descending, a column of CV_64F) of a small matrix; only
// the NO_UV form the reference's HDR fit uses.
class SVD {
public:
    enum { NO_UV = 1 };
    SVD(const Mat& a, int flags = 0);
    Mat w;
};
// DECOMP_SVD: the Moore-Penrose pseudo-inverse of a full-column-rank matrix.
double invert(const Mat& src, Mat& dst, int flags = DECOMP_LU);

}  // namespace cv
