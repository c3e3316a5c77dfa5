// calib.cu -- setCalibrationParams (stereoRectify, full-left canvas, FP64
// rectification maps on the device) and setData's rectifying remap, fused with
// the decoder's 3x3 post-smooth.  Compiled with --fmad=false so the FP64 map
// arithmetic is plain IEEE multiply/add, identical to a CPU evaluation.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp
//   setCalibrationParams :292-339, computeFullLeftRectification :248-289,
//   setData :368-395 (remap INTER_LINEAR phase, INTER_NEAREST order).
#include <cfloat>
#include <cmath>
#include <cstring>

#include "zim_tiles.cuh"

namespace {

struct M3 {
    double a[9];
    double& operator()(int r, int c) { return a[r * 3 + c]; }
    double operator()(int r, int c) const { return a[r * 3 + c]; }
};

M3 mul(const M3& A, const M3& B) {
    M3 C;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += A(r, k) * B(k, c);
            C(r, c) = s;
        }
    return C;
}

M3 transpose(const M3& A) {
    M3 T;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) T(c, r) = A(r, c);
    return T;
}

M3 inverse(const M3& A) {  // adjugate / determinant
    M3 I;
    double c00 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
    double c01 = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
    double c02 = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
    double det = A(0, 0) * c00 + A(0, 1) * c01 + A(0, 2) * c02;
    double id = 1.0 / det;
    I(0, 0) = c00 * id;
    I(0, 1) = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) * id;
    I(0, 2) = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) * id;
    I(1, 0) = c01 * id;
    I(1, 1) = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) * id;
    I(1, 2) = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) * id;
    I(2, 0) = c02 * id;
    I(2, 1) = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) * id;
    I(2, 2) = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) * id;
    return I;
}

// Rotation vector -> matrix (Rodrigues).
M3 rot_from_vec(const double v[3]) {
    M3 R;
    double th = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (th < DBL_EPSILON) {
        for (int i = 0; i < 9; i++) R.a[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return R;
    }
    double c = std::cos(th), s = std::sin(th), c1 = 1.0 - c;
    double x = v[0] / th, y = v[1] / th, z = v[2] / th;
    double K[9] = {0, -z, y, z, 0, -x, -y, x, 0};
    double u[3] = {x, y, z};
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) R(r, q) = (r == q ? c : 0.0) + c1 * u[r] * u[q] + s * K[r * 3 + q];
    return R;
}

// Rotation matrix -> vector (Rodrigues), for an orthonormal input.
void vec_from_rot(const M3& R, double v[3]) {
    double px = R(2, 1) - R(1, 2), py = R(0, 2) - R(2, 0), pz = R(1, 0) - R(0, 1);
    double s = std::sqrt((px * px + py * py + pz * pz) * 0.25);
    double c = std::fmin(1.0, std::fmax(-1.0, (R(0, 0) + R(1, 1) + R(2, 2) - 1) * 0.5));
    double th = std::acos(c);
    if (s < 1e-5) {
        if (c > 0) { v[0] = v[1] = v[2] = 0; return; }
        px = std::sqrt(std::fmax((R(0, 0) + 1) * 0.5, 0.0));
        py = std::sqrt(std::fmax((R(1, 1) + 1) * 0.5, 0.0)) * (R(0, 1) < 0 ? -1.0 : 1.0);
        pz = std::sqrt(std::fmax((R(2, 2) + 1) * 0.5, 0.0)) * (R(0, 2) < 0 ? -1.0 : 1.0);
        if (std::fabs(px) < std::fabs(py) && std::fabs(px) < std::fabs(pz) && (R(1, 2) > 0) != (py * pz > 0)) pz = -pz;
        double sc = th / std::sqrt(px * px + py * py + pz * pz);
        v[0] = px * sc; v[1] = py * sc; v[2] = pz * sc;
        return;
    }
    double sc = th / (2 * s);
    v[0] = px * sc; v[1] = py * sc; v[2] = pz * sc;
}

// undistortPoints (5 fixed-point iterations), optional rectifying R and new
// projection P (3x3 part of a 3x4).  float in/out like the CV_32FC2 call sites.
void undistort(const double K[9], const double D[5], const M3* R, const double* P34, const float* in, float* out,
               int n) {
    M3 RR;
    for (int i = 0; i < 9; i++) RR.a[i] = (i % 4 == 0) ? 1.0 : 0.0;
    if (R) RR = *R;
    if (P34) {
        M3 P;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) P(r, c) = P34[r * 4 + c];
        RR = mul(P, RR);
    }
    const double fx = K[0], fy = K[4], cx = K[2], cy = K[5];
    const double ifx = 1. / fx, ify = 1. / fy;
    for (int i = 0; i < n; i++) {
        double u = in[2 * i], v = in[2 * i + 1];
        double x = (u - cx) * ifx, y = (v - cy) * ify;
        double x0 = x, y0 = y;
        for (int it = 0; it < 5; it++) {
            double r2 = x * x + y * y;
            double icd = 1.0 / (1 + ((D[4] * r2 + D[1]) * r2 + D[0]) * r2);
            if (icd < 0) {
                x = (u - cx) * ifx;
                y = (v - cy) * ify;
                break;
            }
            double dx = 2 * D[2] * x * y + D[3] * (r2 + 2 * x * x);
            double dy = D[2] * (r2 + 2 * y * y) + 2 * D[3] * x * y;
            x = (x0 - dx) * icd;
            y = (y0 - dy) * icd;
        }
        double xx = RR(0, 0) * x + RR(0, 1) * y + RR(0, 2);
        double yy = RR(1, 0) * x + RR(1, 1) * y + RR(1, 2);
        double ww = 1. / (RR(2, 0) * x + RR(2, 1) * y + RR(2, 2));
        out[2 * i] = (float)(xx * ww);
        out[2 * i + 1] = (float)(yy * ww);
    }
}

// cv::stereoRectify(flags = 0, alpha = -1, newImageSize = imageSize).
void stereo_rectify(const zim_stereo_calib& c, double R1[9], double R2[9], double P1[12], double P2[12],
                    double Q[16]) {
    M3 Rm;
    std::memcpy(Rm.a, c.R, sizeof Rm.a);
    double om[3];
    vec_from_rot(Rm, om);
    for (double& v : om) v *= -0.5;
    M3 r_r = rot_from_vec(om);
    double t[3];
    for (int i = 0; i < 3; i++) t[i] = r_r(i, 0) * c.t[0] + r_r(i, 1) * c.t[1] + r_r(i, 2) * c.t[2];
    const int idx = std::fabs(t[0]) > std::fabs(t[1]) ? 0 : 1;
    const double cc = t[idx], nt = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    double uu[3] = {0, 0, 0};
    uu[idx] = cc > 0 ? 1 : -1;
    double ww[3] = {t[1] * uu[2] - t[2] * uu[1], t[2] * uu[0] - t[0] * uu[2], t[0] * uu[1] - t[1] * uu[0]};
    double nw = std::sqrt(ww[0] * ww[0] + ww[1] * ww[1] + ww[2] * ww[2]);
    if (nw > 0.0) {
        double s = std::acos(std::fabs(cc) / nt) / nw;
        for (double& v : ww) v *= s;
    }
    M3 wR = rot_from_vec(ww);
    M3 Ri1 = mul(wR, transpose(r_r));
    M3 Ri2 = mul(wR, r_r);
    std::memcpy(R1, Ri1.a, sizeof Ri1.a);
    std::memcpy(R2, Ri2.a, sizeof Ri2.a);
    for (int i = 0; i < 3; i++) t[i] = Ri2(i, 0) * c.t[0] + Ri2(i, 1) * c.t[1] + Ri2(i, 2) * c.t[2];

    const double nx = c.width, ny = c.height;
    const double ratio = (idx == 1 ? nx / nx : ny / ny) / 2;
    const double fc = (c.camera_matrix[0][(idx ^ 1) * 4] + c.camera_matrix[1][(idx ^ 1) * 4]) * ratio;
    double ccx[2], ccy[2];
    for (int k = 0; k < 2; k++) {
        float pts[8], und[8];
        for (int i = 0; i < 4; i++) {
            pts[2 * i] = (float)((i % 2) * (nx - 1));
            pts[2 * i + 1] = (float)((i < 2 ? 0 : 1) * (ny - 1));
        }
        undistort(c.camera_matrix[k], c.dist_coeffs[k], nullptr, nullptr, pts, und, 4);
        const M3& Rk = k == 0 ? Ri1 : Ri2;
        double sx = 0, sy = 0;
        for (int i = 0; i < 4; i++) {
            double X = und[2 * i], Y = und[2 * i + 1];
            double xr = Rk(0, 0) * X + Rk(0, 1) * Y + Rk(0, 2);
            double yr = Rk(1, 0) * X + Rk(1, 1) * Y + Rk(1, 2);
            double zr = Rk(2, 0) * X + Rk(2, 1) * Y + Rk(2, 2);
            double iz = zr ? 1. / zr : 1;
            sx += (float)(fc * (xr * iz));
            sy += (float)(fc * (yr * iz));
        }
        ccx[k] = (nx - 1) / 2 - sx / 4;
        ccy[k] = (ny - 1) / 2 - sy / 4;
    }
    if (idx == 0) ccy[0] = ccy[1] = (ccy[0] + ccy[1]) * 0.5;
    else ccx[0] = ccx[1] = (ccx[0] + ccx[1]) * 0.5;
    const double cx1 = nx * ccx[0] / nx, cy1 = ny * ccy[0] / ny;
    const double cx2 = nx * ccx[1] / nx, cy2 = ny * ccy[1] / ny;
    std::memset(P1, 0, 12 * sizeof(double));
    std::memset(P2, 0, 12 * sizeof(double));
    P1[0] = P1[5] = fc; P1[2] = cx1; P1[6] = cy1; P1[10] = 1;
    P2[0] = P2[5] = fc; P2[2] = cx2; P2[6] = cy2; P2[10] = 1;
    P2[idx * 4 + 3] = t[idx] * fc;
    std::memset(Q, 0, 16 * sizeof(double));
    Q[0] = 1; Q[3] = -cx1;
    Q[5] = 1; Q[7] = -cy1;
    Q[11] = fc;
    Q[14] = -1. / t[idx];
    Q[15] = (idx == 0 ? cx1 - cx2 : cy1 - cy2) / t[idx];
}

// Full-left canvas (JSLAB_PhaseEpipolarReconstructor_V2.cpp:248-289).
void full_left(const zim_stereo_calib& c, const double R1[9], double P1[12], double P2[12], double Q[16], int* w,
               int* h) {
    float corners[8] = {0.0f, 0.0f, (float)c.width - 1.0f, 0.0f, (float)c.width - 1.0f, (float)c.height - 1.0f,
                        0.0f, (float)c.height - 1.0f};
    float rc[8];
    M3 R;
    std::memcpy(R.a, R1, sizeof R.a);
    undistort(c.camera_matrix[0], c.dist_coeffs[0], &R, P1, corners, rc, 4);
    float mnx = rc[0], mxx = rc[0], mny = rc[1], mxy = rc[1];
    for (int i = 0; i < 4; i++) {
        mnx = std::fmin(mnx, rc[2 * i]); mxx = std::fmax(mxx, rc[2 * i]);
        mny = std::fmin(mny, rc[2 * i + 1]); mxy = std::fmax(mxy, rc[2 * i + 1]);
    }
    double sx = -std::floor(mnx), sy = -std::floor(mny);
    *w = (int)std::ceil(mxx - mnx + 1.0f);
    *h = (int)std::ceil(mxy - mny + 1.0f);
    P1[2] += sx; P1[6] += sy;
    P2[2] += sx; P2[6] += sy;
    Q[3] -= sx; Q[7] -= sy;
}

struct MapParams {
    double ir[9];
    double fx, fy, u0, v0, k1, k2, p1, p2, k3;
};

// initUndistortRectifyMap(CV_32FC1), one thread per rectified pixel, FP64.
__global__ void map_kernel(MapParams p, int w, int h, float* __restrict__ mx, float* __restrict__ my) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    if (j >= w || i >= h) return;
    const double* ir = p.ir;
    double x_ = ir[0] * j + (ir[1] * i + ir[2]);
    double y_ = ir[3] * j + (ir[4] * i + ir[5]);
    double w_ = ir[6] * j + (ir[7] * i + ir[8]);
    double ww = 1. / w_, x = x_ * ww, y = y_ * ww;
    double x2 = x * x, y2 = y * y;
    double r2 = x2 + y2, _2xy = 2 * x * y;
    double kr = 1 + ((p.k3 * r2 + p.k2) * r2 + p.k1) * r2;
    double u = p.fx * (x * kr + p.p1 * _2xy + p.p2 * (r2 + 2 * x2)) + p.u0;
    double v = p.fy * (y * kr + p.p1 * (r2 + 2 * y2) + p.p2 * _2xy) + p.v0;
    mx[(size_t)i * w + j] = (float)u;
    my[(size_t)i * w + j] = (float)v;
}

// setData remap of one camera (zt::rectify_pixel per rectified pixel).
__global__ void rectify_kernel(const int32_t* __restrict__ order, const float* __restrict__ res, int srows,
                               int scols, const float* __restrict__ mapx, const float* __restrict__ mapy, int drows,
                               int dcols, int post_smooth, int32_t* __restrict__ rbase, float* __restrict__ rres,
                               int32_t* __restrict__ rorder) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= dcols || i >= drows) return;
    size_t o = (size_t)i * dcols + j;
    zt::rectify_pixel(order, res, srows, scols, mapx[o], mapy[o], post_smooth, rbase[o], rres[o], rorder[o]);
}

// Post-smooth once per source pixel (the reference smooths the decoded phase
// map before setData, JSLAB_PhaseShiftDecoder_V2.cpp:274-295) ...
__global__ void smooth_kernel(const int32_t* __restrict__ order, const float* __restrict__ res, int rows, int cols,
                              int hdr, int32_t* __restrict__ K16, float* __restrict__ R) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= cols || y >= rows) return;
    if (hdr) zt::smooth_pixel_hdr(order, res, rows, cols, x, y, K16, R);
    else zt::smooth_pixel(order, res, rows, cols, x, y, K16, R);
}

// ... then remap the smoothed taps.
__global__ void rectify_smoothed_kernel(const int32_t* __restrict__ K16, const float* __restrict__ R,
                                        const int32_t* __restrict__ order, int srows, int scols,
                                        const float* __restrict__ mapx, const float* __restrict__ mapy, int drows,
                                        int dcols, int32_t* __restrict__ rbase, float* __restrict__ rres,
                                        int32_t* __restrict__ rorder) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= dcols || i >= drows) return;
    size_t o = (size_t)i * dcols + j;
    zt::rectify_pixel_smoothed(K16, R, order, srows, scols, mapx[o], mapy[o], rbase[o], rres[o], rorder[o]);
}

// rectifyLeftImage: cv::remap INTER_LINEAR of an 8-bit image.  OpenCV rounds
// the map to 1/32 pixel and weights the four taps with (32 - fx or fx) x
// (32 - fy or fy) x 32, which sum to 32768 exactly; the result is
// (sum + 16384) >> 15, taps outside the image read 0 (BORDER_CONSTANT).
__global__ void rectify_image_kernel(const uint8_t* __restrict__ src, int srows, int scols,
                                     const float* __restrict__ mapx, const float* __restrict__ mapy, int drows,
                                     int dcols, uint8_t* __restrict__ dst) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= dcols || i >= drows) return;
    size_t o = (size_t)i * dcols + j;
    int sx = __float2int_rn(mapx[o] * 32.0f), sy = __float2int_rn(mapy[o] * 32.0f);
    int x0 = sx >> 5, y0 = sy >> 5, fx = sx & 31, fy = sy & 31;
    int acc = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        int xx = x0 + (t & 1), yy = y0 + (t >> 1);
        if (xx < 0 || yy < 0 || xx >= scols || yy >= srows) continue;
        int w = ((t >> 1) ? fy : 32 - fy) * ((t & 1) ? fx : 32 - fx) * 32;
        acc += w * (int)__ldg(src + (size_t)yy * scols + xx);
    }
    dst[o] = (uint8_t)min((acc + (1 << 14)) >> 15, 255);
}

}  // namespace

extern "C" ZIM_API zim_status zim_rectify_image(zim_ctx* ctx, int cam, const uint8_t* src, int rows, int cols,
                                                uint8_t* dst, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    if ((cam != 0 && cam != 1) || !src || !dst) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "image %dx%d differs from calibration %dx%d", cols, rows,
                        ctx->src_w, ctx->src_h);
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    dim3 blk(32, 8), grd((ctx->rect_w + 31) / 32, (ctx->rect_h + 7) / 8);
    rectify_image_kernel<<<grd, blk, 0, zim_stream(stream)>>>(src, rows, cols, ctx->d_map[cam][0], ctx->d_map[cam][1],
                                                               ctx->rect_h, ctx->rect_w, dst);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

void zim_rect_free(zim_rect_state& st) {
    for (int k = 0; k < 2; k++)
        for (int m = 0; m < 2; m++) {
            cudaFree(st.d_map[k][m]);
            st.d_map[k][m] = nullptr;
        }
}

// setCalibrationParams (JSLAB_PhaseEpipolarReconstructor_V2.cpp:292-339):
// stereoRectify, the optional full-left canvas and the two cameras' float
// rectification maps (FP64 on the device), into st (maps newly allocated).
zim_status zim_rect_build(zim_ctx* ctx, const zim_stereo_calib* c, int use_full_left, zim_rect_state& st) {
    if (!c || c->width <= 0 || c->height <= 0 || c->width > 65536 || c->height > 65536)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad calibration image size");
    for (int k = 0; k < 2; k++)
        if (!(c->camera_matrix[k][0] > 0) || !(c->camera_matrix[k][4] > 0))
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad camera matrix %d", k);
    if (c->t[0] == 0 && c->t[1] == 0 && c->t[2] == 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "zero baseline");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    st = zim_rect_state{};
    stereo_rectify(*c, st.R1, st.R2, st.P1, st.P2, st.Q);
    int rw = c->width, rh = c->height;
    if (use_full_left) full_left(*c, st.R1, st.P1, st.P2, st.Q, &rw, &rh);
    if (rw <= 0 || rh <= 0 || rw > 4 * c->width + 64 || rh > 4 * c->height + 64 || rw > 65536)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "degenerate rectification (%dx%d)", rw, rh);
    size_t n = (size_t)rw * rh;
    for (int k = 0; k < 2; k++)
        for (int m = 0; m < 2; m++)
            if (cudaMalloc(&st.d_map[k][m], n * sizeof(float)) != cudaSuccess) {
                cudaGetLastError();
                zim_rect_free(st);
                return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "map allocation failed");
            }
    for (int k = 0; k < 2; k++) {
        const double* Pk = k == 0 ? st.P1 : st.P2;
        M3 A, R;
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) A(r, q) = Pk[r * 4 + q];
        std::memcpy(R.a, k == 0 ? st.R1 : st.R2, sizeof R.a);
        M3 iR = inverse(mul(A, R));
        MapParams p;
        std::memcpy(p.ir, iR.a, sizeof p.ir);
        std::memcpy(st.ir[k], iR.a, sizeof st.ir[k]);
        const double* K = c->camera_matrix[k];
        const double* D = c->dist_coeffs[k];
        p.fx = K[0]; p.fy = K[4]; p.u0 = K[2]; p.v0 = K[5];
        p.k1 = D[0]; p.k2 = D[1]; p.p1 = D[2]; p.p2 = D[3]; p.k3 = D[4];
        dim3 blk(256), grd((rw + 255) / 256, rh);
        map_kernel<<<grd, blk>>>(p, rw, rh, st.d_map[k][0], st.d_map[k][1]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            zim_rect_free(st);
            return zim_fail(ctx, ZIM_ERR_CUDA, "map kernel launch failed: %s", cudaGetErrorString(e));
        }
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        zim_rect_free(st);
        return zim_fail(ctx, ZIM_ERR_CUDA, "map kernel failed: %s", cudaGetErrorString(e));
    }
    st.src_w = c->width;
    st.src_h = c->height;
    st.rect_w = rw;
    st.rect_h = rh;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_set_calibration(zim_ctx* ctx, const zim_stereo_calib* c, int use_full_left) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    zim_rect_state st;
    zim_status s = zim_rect_build(ctx, c, use_full_left, st);
    if (s) return s;
    for (int k = 0; k < 2; k++)
        for (int m = 0; m < 2; m++) {
            cudaFree(ctx->d_map[k][m]);
            ctx->d_map[k][m] = st.d_map[k][m];
        }
    ctx->calib = *c;
    std::memcpy(ctx->R1, st.R1, sizeof st.R1);
    std::memcpy(ctx->R2, st.R2, sizeof st.R2);
    std::memcpy(ctx->P1, st.P1, sizeof st.P1);
    std::memcpy(ctx->P2, st.P2, sizeof st.P2);
    std::memcpy(ctx->Q, st.Q, sizeof st.Q);
    std::memcpy(ctx->ir, st.ir, sizeof st.ir);
    ctx->src_w = st.src_w;
    ctx->src_h = st.src_h;
    ctx->rect_w = st.rect_w;
    ctx->rect_h = st.rect_h;
    ctx->calibrated = true;
    if (ctx->poly_w != ctx->rect_w || ctx->poly_h != ctx->rect_h) zim_set_poly_calib(ctx, nullptr, nullptr, nullptr, 0, 0);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_set_poly_calib(zim_ctx* ctx, const float* cx, const float* cy, const float* cz,
                                                 int rows, int cols) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const bool drop = !cx && !cy && !cz;
    if (!drop) {
        if (!cx || !cy || !cz) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "all three coefficient maps or none");
        if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "zim_set_calibration first");
        if (rows != ctx->rect_h || cols != ctx->rect_w)
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "coefficient maps %dx%d differ from the rectified size %dx%d",
                            cols, rows, ctx->rect_w, ctx->rect_h);
    }
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    const size_t n = drop ? 0 : (size_t)rows * cols;
    if (n != (size_t)ctx->poly_w * ctx->poly_h) {
        for (int k = 0; k < 3; k++) {
            cudaFree(ctx->d_poly[k]);
            ctx->d_poly[k] = nullptr;
        }
        ctx->poly_w = ctx->poly_h = 0;
        for (int k = 0; k < 3 && n; k++) ZIM_CUDA_TRY(ctx, cudaMalloc(&ctx->d_poly[k], n * sizeof(float4)));
    }
    if (drop) return ZIM_OK;
    const float* src[3] = {cx, cy, cz};
    for (int k = 0; k < 3; k++)
        ZIM_CUDA_TRY(ctx, cudaMemcpy(ctx->d_poly[k], src[k], n * sizeof(float4), cudaMemcpyHostToDevice));
    ctx->poly_w = cols;
    ctx->poly_h = rows;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_get_rectification(const zim_ctx* ctx, double R1[9], double R2[9], double P1[12],
                                                    double P2[12], double Q[16], int* rw, int* rh) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return ZIM_ERR_NOT_CALIBRATED;
    if (R1) std::memcpy(R1, ctx->R1, sizeof ctx->R1);
    if (R2) std::memcpy(R2, ctx->R2, sizeof ctx->R2);
    if (P1) std::memcpy(P1, ctx->P1, sizeof ctx->P1);
    if (P2) std::memcpy(P2, ctx->P2, sizeof ctx->P2);
    if (Q) std::memcpy(Q, ctx->Q, sizeof ctx->Q);
    if (rw) *rw = ctx->rect_w;
    if (rh) *rh = ctx->rect_h;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_get_rectify_maps(zim_ctx* ctx, int cam, float* mapx, float* mapy, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    if ((cam != 0 && cam != 1) || !mapx || !mapy) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    size_t n = (size_t)ctx->rect_w * ctx->rect_h * sizeof(float);
    cudaStream_t st = zim_stream(stream);
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(mapx, ctx->d_map[cam][0], n, cudaMemcpyDeviceToDevice, st));
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(mapy, ctx->d_map[cam][1], n, cudaMemcpyDeviceToDevice, st));
    return ZIM_OK;
}

zim_status zim_rectify_launch(zim_ctx* ctx, int cam, const int32_t* order, const float* residual, int rows, int cols,
                              int post_smooth, int32_t* smooth_k16, float* smooth_r, int32_t* rbase, float* rres,
                              int32_t* rorder, cudaStream_t st) {
    dim3 blk(32, 8), grd((ctx->rect_w + 31) / 32, (ctx->rect_h + 7) / 8);
    if (post_smooth == 1 || post_smooth == 2) {
        dim3 sgrd((cols + 31) / 32, (rows + 7) / 8);
        smooth_kernel<<<sgrd, blk, 0, st>>>(order, residual, rows, cols, post_smooth == 2 ? 1 : 0, smooth_k16,
                                            smooth_r);
        rectify_smoothed_kernel<<<grd, blk, 0, st>>>(smooth_k16, smooth_r, order, rows, cols, ctx->d_map[cam][0],
                                                     ctx->d_map[cam][1], ctx->rect_h, ctx->rect_w, rbase, rres,
                                                     rorder);
        ctx->launches += 2;
    } else {
        rectify_kernel<<<grd, blk, 0, st>>>(order, residual, rows, cols, ctx->d_map[cam][0], ctx->d_map[cam][1],
                                            ctx->rect_h, ctx->rect_w, post_smooth, rbase, rres, rorder);
        ctx->launches += 1;
    }
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

// The post-smooth alone (post_smooth 1 or 2; nothing to do otherwise), for
// the fused rectify + match of the whole-pair path.
zim_status zim_smooth_launch(zim_ctx* ctx, const int32_t* order, const float* residual, int rows, int cols,
                             int post_smooth, int32_t* smooth_k16, float* smooth_r, cudaStream_t st) {
    if (post_smooth != 1 && post_smooth != 2) return ZIM_OK;
    dim3 blk(32, 8), sgrd((cols + 31) / 32, (rows + 7) / 8);
    smooth_kernel<<<sgrd, blk, 0, st>>>(order, residual, rows, cols, post_smooth == 2 ? 1 : 0, smooth_k16, smooth_r);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_rectify(zim_ctx* ctx, int cam, const int32_t* order, const float* residual, int rows,
                                          int cols, int post_smooth, int32_t* rbase, float* rres, int32_t* rorder,
                                          void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!ctx->calibrated) return zim_fail(ctx, ZIM_ERR_NOT_CALIBRATED, "not calibrated");
    if ((cam != 0 && cam != 1) || !order || !residual || !rbase || !rres || !rorder)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows != ctx->src_h || cols != ctx->src_w)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "image size differs from calibration");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (post_smooth < 0 || post_smooth > 3) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "post_smooth must be 0..3");
    int32_t* sk = nullptr;
    float* sr = nullptr;
    if (post_smooth == 1 || post_smooth == 2) {
        const size_t src = (size_t)rows * cols;
        zim_status s = zim_scratch_reserve(ctx, 2 * zim_align256(src * 4) + 1024);
        if (s) return s;
        zim_scratch_reset(ctx);
        sk = (int32_t*)zim_scratch_take(ctx, src * 4);
        sr = (float*)zim_scratch_take(ctx, src * 4);
        if (!sk || !sr) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "rectify scratch");
    }
    return zim_rectify_launch(ctx, cam, order, residual, rows, cols, post_smooth, sk, sr, rbase, rres, rorder,
                              zim_stream(stream));
}
