// C++ use of include/zim_jslab.hpp the way a reference caller uses the
// reference classes (decoder per camera, then the V2 reconstructor): a
// fronto-parallel plane seen by an ideal rig, hierarchical 1/8/64 x 4-step
// fringes rendered analytically.  Exit status 0 when the plane comes back at
// the expected depth, and when the V2 path (coefficient maps equivalent to Q,
// written and read back as .bin files under argv[1]) reproduces it.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "zim_jslab.hpp"

// Inverse-depth maps (x-map tag -1) reproducing the Q reprojection.
static void q_maps(const double Q[16], int rows, int cols, JSLAB_StereoCalibParams_V2& p) {
    for (int k = 0; k < 3; k++) p.xyz_calib_coeffs[k] = zim::Image<float>(rows, cols, 4);
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            float* cx = p.xyz_calib_coeffs[0].ptr() + 4 * ((size_t)i * cols + j);
            float* cy = p.xyz_calib_coeffs[1].ptr() + 4 * ((size_t)i * cols + j);
            float* cz = p.xyz_calib_coeffs[2].ptr() + 4 * ((size_t)i * cols + j);
            cx[0] = (float)((j + Q[3]) / Q[11]); cx[3] = -1.0f;
            cy[0] = (float)((i + Q[7]) / Q[11]);
            cz[0] = (float)(Q[15] / Q[11]); cz[1] = (float)(Q[14] / Q[11]);
        }
}

int main(int argc, char** argv) {
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
    if (!ok) return 2;

    // V2: polynomial maps through the .bin format, then startCalculate_v2
    double Q[16];
    int rw = 0, rh = 0;
    zim::check(zim_get_rectification(ctx->get(), nullptr, nullptr, nullptr, nullptr, Q, &rw, &rh), ctx->get(), "rect");
    JSLAB_StereoCalibParams_V2 v2;
    static_cast<JSLAB_StereoCalibParams_V1&>(v2) = calib;
    q_maps(Q, rh, rw, v2);
    if (argc > 1) {
        const std::string fn = std::string(argv[1]) + "/stereo_v2.xml";
        const char* sfx[3] = {"_rx.bin", "_ry.bin", "_rz.bin"};
        for (int k = 0; k < 3; k++)
            if (!JSLAB_StereoCalibParams_V2::saveMatBinary(std::string(argv[1]) + "/stereo_v2" + sfx[k],
                                                           v2.xyz_calib_coeffs[k]))
                return 3;
        JSLAB_StereoCalibParams_V2 back;
        static_cast<JSLAB_StereoCalibParams_V1&>(back) = calib;
        if (!back.loadCoefficientMaps(fn)) return 4;
        for (int k = 0; k < 3; k++)
            if (back.xyz_calib_coeffs[k].data != v2.xyz_calib_coeffs[k].data) return 5;
        v2 = back;
    }
    rec.setCalibrationParamsV2(v2);
    rec.setData(*left, *right);
    zim::Image<float> xq, xp;
    zim::Image<uint8_t> pq, pp;
    rec.startCalculate(xq, pq);
    rec.startCalculate_v2(xp, pp);
    size_t n = 0, diff = 0;
    double worst = 0;
    for (size_t i = 0; i < pq.size(); i++) {
        diff += pq.data[i] != pp.data[i];
        if (pq.data[i] && pp.data[i]) {
            n++;
            for (int c = 0; c < 3; c++)
                worst = std::max(worst, (double)std::fabs(xq.data[3 * i + c] - xp.data[3 * i + c]) /
                                            (1.0 + std::fabs(xq.data[3 * i + c])));
        }
    }
    std::printf("{\"v2_points\": %zu, \"v2_mask_diff\": %zu, \"v2_max_rel\": %.3g}\n", n, diff, worst);
    if (!(n > z.size() / 2 && diff <= pq.size() / 10000 && worst < 1e-5)) return 6;

    // outputs: grey PLY from the rectified left image, .raw phase dump
    if (argc > 1) {
        zim::Image<uint8_t> gray;
        rec.rectifyLeftImage(frames[0][0], gray);
        if (gray.rows != rh || gray.cols != rw) return 7;
        const std::string dir = argv[1];
        size_t valid = 0;
        for (uint8_t m : pq.data) valid += m != 0;
        if (!savePointCloudToPlyBinaryWithGray(*ctx, xq, pq, gray, dir + "/cloud.ply")) return 8;
        std::ifstream ply(dir + "/cloud.ply", std::ios::binary | std::ios::ate);
        const std::string head = "ply\nformat binary_little_endian 1.0\nelement vertex " + std::to_string(valid) +
                                 "\nproperty float x\nproperty float y\nproperty float z\nproperty uchar red\n"
                                 "property uchar green\nproperty uchar blue\nend_header\n";
        if ((size_t)ply.tellg() != head.size() + 15 * valid) return 9;
        if (!saveRaw64F(phL, dir + "/phase_left_global.raw", dir + "/phase_left_global.info.txt")) return 10;
        std::printf("{\"ply_vertices\": %zu}\n", valid);
    }
    return 0;
}
