// ref_mls_f64.cpp -- the reference's CPU MLS (JSLAB_MLS_Filter.cpp) built a
// second time with its `float` arithmetic evaluated in double.  TEST
// INFRASTRUCTURE ONLY (oracle/_ref).
//
// The reference accumulates weighted centroids and covariances of points near
// 900 mm in float, so its FP32 output carries rounding of up to ~0.1 mm at
// some points; that says nothing about whether a restatement selects the same
// neighbours, weights, normal, polynomial order and projection.  Evaluating
// the same source with every `float` variable widened to double separates the
// two: the oracle's FP64 MLS must agree with this build to FP64 round-off,
// while the FP32 build bounds the reference's own rounding.
//
// Every header the reference file includes is included first, unchanged;
// only then is `float` redefined, so the macro reaches the reference file's
// own tokens and nothing else.  Points stay float (cv::Vec3f is defined by
// then), as do the input and output clouds; sums, weights, frames and
// solutions are double.  The entry points are renamed so that this build
// links beside the FP32 one.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "JSLAB_MLS_Filter.h"

// Widening leaves the reference's float literals as they are, so a call such
// as std::min(1.0f, r) with r now double needs these mixed overloads (same
// results as std::min / std::max on the common type).
namespace std {
inline double min(float a, double b) { return b < a ? b : (double)a; }
inline double min(double a, float b) { return b < a ? (double)b : a; }
inline double max(float a, double b) { return (double)a < b ? b : (double)a; }
inline double max(double a, float b) { return a < b ? (double)b : a; }
}  // namespace std

void applyMLSFilterToPointCloud_GPU_f64(const cv::Mat&, const cv::Mat&, cv::Mat&, int, double, int, double, int);

#define applyMLSFilterToPointCloud_CPU applyMLSFilterToPointCloud_CPU_f64
#define applyMLSFilterToPointCloud_GPU applyMLSFilterToPointCloud_GPU_f64
#define applyMLSFilterToPointCloud applyMLSFilterToPointCloud_f64
#define float double
#include "JSLAB_MLS_Filter.cpp"
#undef float

void applyMLSFilterToPointCloud_GPU_f64(const cv::Mat&, const cv::Mat&, cv::Mat&, int, double, int, double, int) {
    throw std::runtime_error("the reference's CUDA MLS is not part of the oracle/_ref CPU build");
}

extern "C" int zr_mls_f64(const float* xyz, const uint8_t* P, int rows, int cols, int window, double sigma,
                          int order, double max_radius, int iterations, float* out) {
    try {
        cv::Mat X = cv::Mat(rows, cols, CV_32FC3, (void*)xyz).clone(), M = cv::Mat(rows, cols, CV_8UC1, (void*)P).clone();
        cv::Mat o;
        applyMLSFilterToPointCloud_CPU_f64(X, M, o, window, sigma, order, max_radius, iterations);
        for (int r = 0; r < rows; r++)
            std::memcpy(out + (size_t)r * cols * 3, o.ptr<float>(r), sizeof(float) * 3 * cols);
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}
