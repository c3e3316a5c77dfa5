// C++ use of include/zim_jslab.hpp the way a reference caller uses the
// reference classes (decoder per camera, then the V2 reconstructor): a
// fronto-parallel plane seen by an ideal rig, hierarchical 1/8/64 x 4-step
// fringes rendered analytically.  Exit status 0 when the plane comes back at
// the expected depth.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "zim_jslab.hpp"

int main() {
    const int W = 640, H = 480;
    const double f = 600.0, B = 100.0, disparity = 80.0;  // Z = f B / d = 750 mm
    const double fr[3] = {1, 8, 64};
    // absolute phase at left pixel x (orders >= 3 everywhere)
    auto phase_left = [&](double x) { return 2.0 * M_PI * 64.0 * (x + 40.0) / (W + 80.0); };
    std::vector<zim::Image<uint8_t>> frames[2];
    for (int cam = 0; cam < 2; cam++)
        for (int fi = 0; fi < 3; fi++)
            for (int k = 0; k < 4; k++) {
                zim::Image<uint8_t> im(H, W);
                for (int y = 0; y < H; y++)
                    for (int x = 0; x < W; x++) {
                        // right pixel x sees the surface point of left pixel x + d
                        const double Phi = phase_left(cam == 0 ? x : x + disparity);
                        const double v = 128.0 + 100.0 * std::cos(Phi * fr[fi] / 64.0 + 2.0 * M_PI * k / 4.0);
                        im.data[(size_t)y * W + x] = (uint8_t)std::lround(v);
                    }
                frames[cam].push_back(im);
            }
    JSLAB_PhaseShiftDecoder::Config cfg;
    cfg.freq[0] = 1; cfg.freq[1] = 8; cfg.freq[2] = 64;
    cfg.shift_num[0] = cfg.shift_num[1] = cfg.shift_num[2] = 4;
    cfg.modulation_threshold = 0.3;
    cfg.encoding = ZIM_ENC_HIERARCHICAL;
    if (JSLAB_PhaseShiftDecoder::create(cfg, JSLAB_PhaseShiftDecoder::Version::V1)) {
        std::printf("V1 must not be provided\n");
        return 1;
    }
    JSLAB_PhaseShiftDecoder::Config bad = cfg;
    bad.freq[1] = 7;  // not an integer ratio
    if (JSLAB_PhaseShiftDecoder::create(bad, JSLAB_PhaseShiftDecoder::Version::V2)) {
        std::printf("invalid config must give nullptr\n");
        return 1;
    }
    auto ctx = std::make_shared<zim::Context>(0);
    auto left = JSLAB_PhaseShiftDecoder::create(cfg, JSLAB_PhaseShiftDecoder::Version::V2, ctx);
    auto right = JSLAB_PhaseShiftDecoder::create(cfg, JSLAB_PhaseShiftDecoder::Version::V2, ctx);
    left->setImages(frames[0]);
    right->setImages(frames[1]);
    zim::Image<double> phL, phR, modL;
    zim::Image<int32_t> kL, kR;
    left->startCalculate(phL);
    right->startCalculate(phR);
    left->getOrderMap(kL);
    right->getOrderMap(kR);
    left->getModulationMap(modL);

    JSLAB_StereoCalibParams_V1 calib{};
    for (int c = 0; c < 2; c++) {
        const double K[9] = {f, 0, (W - 1) / 2.0, 0, f, (H - 1) / 2.0, 0, 0, 1};
        std::copy(K, K + 9, calib.camera_matrix[c]);
    }
    const double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::copy(R, R + 9, calib.R);
    calib.t[0] = -B;
    calib.image_width = W;
    calib.image_height = H;

    JSLAB_PhaseEpipolarReconstructor_V2::Config rc;
    rc.c.use_ror = 0;
    JSLAB_PhaseEpipolarReconstructor_V2 rec(rc, ctx);
    rec.setCalibrationParams(calib);
    rec.setData(phL, phR, kL, kR, modL, left->maxOrder());  // the reference's host call sequence
    zim::Image<float> xyz;
    zim::Image<uint8_t> P;
    rec.startCalculate(xyz, P);
    std::vector<float> z;
    for (size_t i = 0; i < P.size(); i++)
        if (P.data[i]) z.push_back(xyz.data[3 * i + 2]);
    std::vector<zim_point_xyz> cloud;
    rec.setData(*left, *right);  // device-resident path from the decoders
    rec.startCalculate(cloud);
    if (z.empty()) {
        std::printf("no points\n");
        return 1;
    }
    std::nth_element(z.begin(), z.begin() + z.size() / 2, z.end());
    const double zmed = z[z.size() / 2];
    const double frac = (double)z.size() / P.size();
    std::printf("{\"points\": %zu, \"cloud\": %zu, \"valid_fraction\": %.3f, \"median_z\": %.3f}\n", z.size(),
                cloud.size(), frac, zmed);
    const bool ok = std::fabs(zmed - f * B / disparity) < 0.01 * f * B / disparity && frac > 0.5 &&
                    cloud.size() > z.size() / 2;
    return ok ? 0 : 2;
}
