/*
 * zim_oracle.c -- FP64 CPU restatement of the PhaseShiftGrayCode3D reconstruction
 * hot path (test infrastructure: the parity checker and the timed CPU baseline).
 *
 * Parity status: pinned to the reference's own code (compiled from its
 * sources as oracle/_ref; tests/test_ref_pin.py) for every computation the
 * reference has; the OpenCV primitives restated below and the computations
 * the reference lacks are checked against known answers instead (see
 * zim_oracle.h).  Every function cites the reference lines it restates.
 * "src/" below means PhaseShiftGrayCode3D/src/.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (no fast-math), so
 * results are IEEE-reproducible across x86-64 and aarch64.
 */
#include "zim_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ZO_PI 3.14159265358979323846

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ------------------------------------------------------------------------ */
/* OpenCV getGaussianKernel(3, sigma): fixed [1/4 1/2 1/4] for sigma <= 0,
 * else exp(-x^2 / (2 sigma^2)) normalised to unit sum (imgproc docs). */
void zo_gaussian_kernel3(double sigma, double k[3]) {
    if (sigma <= 0) {
        k[0] = 0.25; k[1] = 0.5; k[2] = 0.25;
        return;
    }
    double t = exp(-0.5 / (sigma * sigma));
    double sum = 2.0 * t + 1.0;
    double mul = 1.0 / sum;
    k[0] = t * mul; k[1] = mul; k[2] = t * mul;
}

/* GaussianBlur(3x3) with BORDER_REPLICATE on CV_64F: a row pass
 * (k0 s[x-1] + k1 s[x] + k2 s[x+1]) then a symmetric column pass
 * (k1 t[y] + k0 (t[y+1] + t[y-1])) -- OpenCV's separable filter order. */
void zo_blur3(const double* src, double* dst, int rows, int cols, const double k[3]) {
    double* tmp = (double*)malloc(sizeof(double) * (size_t)rows * cols);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < rows; y++) {
        const double* s = src + (size_t)y * cols;
        double* t = tmp + (size_t)y * cols;
        for (int x = 0; x < cols; x++) {
            double a = s[clampi(x - 1, 0, cols - 1)], b = s[x], c = s[clampi(x + 1, 0, cols - 1)];
            double v = k[0] * a;
            v += k[1] * b;
            v += k[2] * c;
            t[x] = v;
        }
    }
#pragma omp parallel for schedule(static)
    for (int y = 0; y < rows; y++) {
        const double* tu = tmp + (size_t)clampi(y - 1, 0, rows - 1) * cols;
        const double* tc = tmp + (size_t)y * cols;
        const double* td = tmp + (size_t)clampi(y + 1, 0, rows - 1) * cols;
        double* d = dst + (size_t)y * cols;
        for (int x = 0; x < cols; x++) d[x] = k[1] * tc[x] + k[2] * (td[x] + tu[x]);
    }
    free(tmp);
}

int zo_frame_count(const zo_decode_cfg* cfg) {
    int f = 0;
    if (cfg->encoding == ZO_ENC_HETERODYNE3) {
        for (int i = 0; i < 3; i++) f += cfg->shift_num[i];
    } else if (cfg->encoding == ZO_ENC_HIERARCHICAL) {
        for (int i = 0; i < cfg->n_freq; i++) f += cfg->shift_num[i];
    } else {
        f = cfg->shift_num[0] + cfg->gray_bits + (cfg->encoding == ZO_ENC_GRAYCODE_COMPLEMENTARY ? 1 : 0);
    }
    return f;
}

static inline double round_margin(double a) { /* distance of a to the nearest half integer */
    double f = a - floor(a);
    return fabs(f - 0.5);
}

/* Wrapped phase and modulation of one frequency (src/JSLAB_PhaseShiftDecoder_V2.cpp:67-118).
 * Returns the normalised modulation; writes wrap. */
static double wrapped_phase(const double* const* fr, size_t pix, int inum, double* wrap) {
    double sin_sum = 0, cos_sum = 0, sum_gray = 0;
    for (int k = 0; k < inum; k++) {
        const double st = sin(2.0 * ZO_PI * k / inum);
        const double ct = cos(2.0 * ZO_PI * k / inum);
        const double v = fr[k][pix];
        sin_sum -= st * v;
        cos_sum += ct * v;
        sum_gray += v;
    }
    *wrap = atan2(sin_sum, cos_sum);
    double b = sin_sum * sin_sum + cos_sum * cos_sum;
    double mean_val = sum_gray / inum;
    b = 2.0 * sqrt(b) / inum;
    double norm_mod = 0.0;
    if (mean_val > 1e-3) norm_mod = b / mean_val;
    return norm_mod;
}

/* HDR least squares of one frequency (JSLAB_HDRPhaseFit.h:10-61 applied as in
 * JSLAB_PhaseShiftDecoder_V2.cpp:73-90): samples with 0 <= I < saturation fit
 * I = A + C cos d - S sin d; the reference multiplies a cached pseudo-inverse
 * of the subset's design, restated here as the normal equations of the same
 * full-rank subset (the same least-squares solution).  Rejects fewer than 3
 * samples, hypot(C, S) <= min_amp or A <= 1e-3.  Returns the normalised
 * modulation (-1 if rejected); writes wrap. */
static double hdr_wrapped_phase(const double* const* fr, size_t pix, int inum, double sat, double min_amp,
                                double* wrap, uint8_t* nf, double eps) {
    double M[3][3] = {{0}}, r[3] = {0};
    int n = 0;
    for (int k = 0; k < inum; k++) {
        const double v = fr[k][pix];
        if (!(v >= 0.0 && v < sat)) continue;
        const double d = 2.0 * ZO_PI * k / inum;
        const double x[3] = {1.0, cos(d), -sin(d)};
        for (int a = 0; a < 3; a++) {
            r[a] += x[a] * v;
            for (int b = 0; b < 3; b++) M[a][b] += x[a] * x[b];
        }
        n++;
    }
    if (n < 3) return -1.0;
    const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1], c01 = M[0][2] * M[2][1] - M[0][1] * M[2][2],
                 c02 = M[0][1] * M[1][2] - M[0][2] * M[1][1];
    const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
    if (!(fabs(det) > 1e-10)) return -1.0;
    const double c11 = M[0][0] * M[2][2] - M[0][2] * M[2][0], c12 = M[0][2] * M[1][0] - M[0][0] * M[1][2],
                 c22 = M[0][0] * M[1][1] - M[0][1] * M[1][0];
    const double A = (c00 * r[0] + c01 * r[1] + c02 * r[2]) / det;
    const double C = (c01 * r[0] + c11 * r[1] + c12 * r[2]) / det;
    const double S = (c02 * r[0] + c12 * r[1] + c22 * r[2]) / det;
    if (fabs(hypot(C, S) - min_amp) < eps * (1.0 + min_amp)) *nf |= ZO_NEAR_MOD;
    if (!(hypot(C, S) > min_amp) || !(A > 1e-3)) return -1.0;
    const double cos_sum = C * inum / 2.0, sin_sum = S * inum / 2.0, sum_gray = A * inum;
    *wrap = atan2(sin_sum, cos_sum);
    const double b = 2.0 * sqrt(sin_sum * sin_sum + cos_sum * cos_sum) / inum;
    const double mean_val = sum_gray / inum;
    return mean_val > 1e-3 ? b / mean_val : 0.0;
}

static inline uint8_t wrap_flag(double w, double eps) { return (ZO_PI - fabs(w) < eps) ? ZO_NEAR_WRAP : 0; }

int zo_decode(const zo_decode_cfg* cfg, const double* frames, int rows, int cols, double* phase,
              int32_t* order, double* mod, uint8_t* valid, uint8_t* near, double eps) {
    const size_t npx = (size_t)rows * cols;
    const int F = zo_frame_count(cfg);
    const int n_ps = (cfg->encoding == ZO_ENC_HETERODYNE3) ? 3
                     : (cfg->encoding == ZO_ENC_HIERARCHICAL ? cfg->n_freq : 1);
    int n_blur = 0;
    for (int i = 0; i < n_ps; i++) n_blur += cfg->shift_num[i];
    if (n_blur <= 0 || F <= 0) return -1;
    if (cfg->encoding == ZO_ENC_HIERARCHICAL) {
        if (cfg->n_freq < 2 || cfg->n_freq > 4 || cfg->freq[0] != 1.0) return -1;
    }

    /* Pre-blur every phase-shift frame (src/JSLAB_PhaseShiftDecoder_V2.cpp:18-28).
     * Gray-code frames are thresholded raw (no blur). */
    double kb[3];
    zo_gaussian_kernel3(cfg->preblur_sigma, kb);
    double* blurred = (double*)malloc(sizeof(double) * npx * n_blur);
    const int hdr = cfg->enable_hdr && (cfg->encoding == ZO_ENC_HETERODYNE3 || cfg->encoding == ZO_ENC_HIERARCHICAL);
    for (int f = 0; f < n_blur; f++) {
        /* HDR classifies saturation on the raw samples: no pre-blur */
        if (hdr) memcpy(blurred + npx * f, frames + npx * f, sizeof(double) * npx);
        else zo_blur3(frames + npx * f, blurred + npx * f, rows, cols, kb);
    }

    const double TWO_PI = 2 * ZO_PI;
#pragma omp parallel for schedule(dynamic, 4)
    for (int r = 0; r < rows; r++) {
        const double* fr[64];
        for (int jcol = 0; jcol < cols; jcol++) {
            const size_t pix = (size_t)r * cols + jcol;
            uint8_t nf = 0;
            double wrap[4] = {0, 0, 0, 0};
            double m0 = 0;
            int ok = 1, base = 0;
            for (int i = 0; i < n_ps; i++) {
                const int inum = cfg->shift_num[i];
                for (int k = 0; k < inum; k++) fr[k] = blurred + npx * (base + k);
                base += inum;
                double nm;
                if (hdr) {
                    nm = hdr_wrapped_phase(fr, pix, inum, cfg->hdr_saturation_gray, cfg->hdr_min_amplitude, &wrap[i],
                                           &nf, eps);
                    if (nm < 0) { ok = 0; break; }
                } else {
                    nm = wrapped_phase(fr, pix, inum, &wrap[i]);
                }
                nf |= wrap_flag(wrap[i], eps);
                if (fabs(nm - cfg->modulation_threshold) < eps) nf |= ZO_NEAR_MOD;
                if (i == 0) m0 = nm;
                if (nm < cfg->modulation_threshold) { ok = 0; break; }
            }
            mod[pix] = m0;
            phase[pix] = 0.0;
            order[pix] = hdr ? -1 : 0;
            valid[pix] = 0;
            if (!ok) { if (near) near[pix] = nf; continue; }

            if (cfg->encoding == ZO_ENC_HETERODYNE3) {
                /* Heterodyne unwrap, src/JSLAB_PhaseShiftDecoder_V2.cpp:124-179. */
                const double* fq = cfg->freq;
                double phase12, phase23, phase123;
                if (fabs(wrap[0] - wrap[1]) < eps) nf |= ZO_NEAR_WRAP;
                if (fabs(wrap[1] - wrap[2]) < eps) nf |= ZO_NEAR_WRAP;
                if (wrap[0] > wrap[1]) phase12 = wrap[0] - wrap[1];
                else phase12 = wrap[0] - wrap[1] + 2 * ZO_PI;
                if (fq[1] > fq[2]) {
                    if (wrap[1] > wrap[2]) phase23 = wrap[1] - wrap[2];
                    else phase23 = wrap[1] - wrap[2] + 2 * ZO_PI;
                } else {
                    if (wrap[2] > wrap[1]) phase23 = wrap[2] - wrap[1];
                    else phase23 = wrap[2] - wrap[1] + 2 * ZO_PI;
                }
                if (fabs(phase12 - phase23) < eps) nf |= ZO_NEAR_WRAP;
                if (phase12 > phase23) phase123 = phase12 - phase23;
                else phase123 = phase12 - phase23 + 2 * ZO_PI;
                int f12 = abs((int)(fq[0] - fq[1]));
                int f23 = abs((int)(fq[1] - fq[2]));
                double a12 = (phase123 * f12 - phase12) / (2 * ZO_PI);
                double uphase12 = phase12 + round(a12) * 2 * ZO_PI;
                double ak = (uphase12 * fq[0] / f12 - wrap[0]) / (2 * ZO_PI);
                double uphase1 = wrap[0] + round(ak) * 2 * ZO_PI;
                double k_val = round((uphase12 * (double)fq[0] / f12 - wrap[0]) / (2 * ZO_PI));
                double a23 = (phase123 * f23 - phase23) / (2 * ZO_PI);
                double uphase23 = phase23 + round(a23) * 2 * ZO_PI;
                double a2 = (uphase23 * fq[1] / f23 - wrap[1]) / (2 * ZO_PI);
                double uphase2 = wrap[1] + round(a2) * 2 * ZO_PI;
                uphase2 = (uphase2 * fq[0]) / fq[1];
                double a3 = (uphase23 * fq[2] / f23 - wrap[2]) / (2 * ZO_PI);
                double uphase3 = wrap[2] + round(a3) * 2 * ZO_PI;
                uphase3 = (uphase3 * fq[0]) / fq[2];
                if (round_margin(a12) < eps || round_margin(ak) < eps) nf |= ZO_NEAR_ROUND;
                if (cfg->avg_three_phase && (round_margin(a23) < eps || round_margin(a2) < eps ||
                                             round_margin(a3) < eps))
                    nf |= ZO_NEAR_ROUND;
                phase[pix] = cfg->avg_three_phase ? (uphase1 + uphase2 + uphase3) / 3.0 : uphase1;
                order[pix] = (int)k_val;
            } else if (cfg->encoding == ZO_ENC_HIERARCHICAL) {
                /* Hierarchical temporal unwrapping (no reference counterpart):
                 * pattern phase theta_f = 2 pi f x - pi, Psi_f = phi_f + pi + 2 pi k_f,
                 * k_i = round((r Psi_{i-1} - (phi_i + pi)) / 2 pi), r = f_i / f_{i-1}. */
                double psi = wrap[0] + ZO_PI;
                int k = 0;
                for (int i = 1; i < cfg->n_freq; i++) {
                    double ratio = cfg->freq[i] / cfg->freq[i - 1];
                    double a = (ratio * psi - (wrap[i] + ZO_PI)) / TWO_PI;
                    if (round_margin(a) < eps) nf |= ZO_NEAR_ROUND;
                    k = (int)round(a);
                    psi = wrap[i] + ZO_PI + TWO_PI * k;
                }
                const int last = cfg->n_freq - 1;
                phase[pix] = wrap[last] + TWO_PI * k;
                order[pix] = k;
            } else {
                /* Gray code (+ complementary bit).  Bits are raw frames compared with
                 * the raw phase-shift mean: N * I_gc > sum(I_n) (exact in integers). */
                const int N = cfg->shift_num[0];
                const int nb = cfg->gray_bits;
                double sum_raw = 0;
                for (int k = 0; k < N; k++) sum_raw += frames[npx * k + pix];
                int bin = 0, v1 = 0;
                for (int b = 0; b < nb; b++) {
                    int g = (N * frames[npx * (N + b) + pix] > sum_raw) ? 1 : 0;
                    bin ^= g;
                    v1 = (v1 << 1) | bin;
                }
                int K = v1;
                if (cfg->encoding == ZO_ENC_GRAYCODE_COMPLEMENTARY) {
                    int g = (N * frames[npx * (N + nb) + pix] > sum_raw) ? 1 : 0;
                    int v2 = (v1 << 1) | (bin ^ g);
                    int k2 = (v2 + 1) >> 1;
                    double w = wrap[0];
                    if (fabs(w + ZO_PI / 2) < eps || fabs(w - ZO_PI / 2) < eps) nf |= ZO_NEAR_GRAY;
                    if (w <= -ZO_PI / 2) K = k2;
                    else if (w >= ZO_PI / 2) K = k2 - 1;
                    else K = v1;
                }
                phase[pix] = wrap[0] + TWO_PI * K;
                order[pix] = K;
            }
            valid[pix] = 1;
            if (near) near[pix] = nf;
        }
    }
    free(blurred);
    return 0;
}

void zo_post_smooth_hdr(const double* src, const uint8_t* valid, double* dst, int rows, int cols) {
    double k[3];
    zo_gaussian_kernel3(0.0, k);
    const size_t n = (size_t)rows * cols;
    double* w = (double*)malloc(sizeof(double) * n);
    double* bw = (double*)malloc(sizeof(double) * n);
    for (size_t i = 0; i < n; i++) w[i] = valid[i] ? 1.0 : 0.0;
    zo_blur3(src, dst, rows, cols, k);
    zo_blur3(w, bw, rows, cols, k);
    for (size_t i = 0; i < n; i++) dst[i] = valid[i] ? dst[i] / (bw[i] > 1e-12 ? bw[i] : 1e-12) : 0.0;
    free(w);
    free(bw);
}

void zo_post_smooth(const double* src, double* dst, int rows, int cols) {
    /* src/JSLAB_PhaseShiftDecoder_V2.cpp:292: GaussianBlur(3x3, sigma 0, REPLICATE). */
    double k[3];
    zo_gaussian_kernel3(0.0, k);
    zo_blur3(src, dst, rows, cols, k);
}

/* ------------------------------------------------------------------------ */
/* Rodrigues conversions (calib3d documented formulas). */
void zo_rodrigues_v2m(const double r[3], double R[9]) {
    double theta = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (theta < DBL_EPSILON) {
        for (int i = 0; i < 9; i++) R[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    double c = cos(theta), s = sin(theta), c1 = 1.0 - c;
    double it = 1.0 / theta;
    double x = r[0] * it, y = r[1] * it, z = r[2] * it;
    double rrt[9] = {x * x, x * y, x * z, x * y, y * y, y * z, x * z, y * z, z * z};
    double rx[9] = {0, -z, y, z, 0, -x, -y, x, 0};
    for (int i = 0; i < 9; i++) R[i] = ((i % 4 == 0) ? c : 0.0) + c1 * rrt[i] + s * rx[i];
}

void zo_rodrigues_m2v(const double R[9], double r[3]) {
    double rx = R[7] - R[5], ry = R[2] - R[6], rz = R[3] - R[1];
    double s = sqrt((rx * rx + ry * ry + rz * rz) * 0.25);
    double c = (R[0] + R[4] + R[8] - 1) * 0.5;
    c = c > 1. ? 1. : (c < -1. ? -1. : c);
    double theta = acos(c);
    if (s < 1e-5) {
        if (c > 0) { r[0] = r[1] = r[2] = 0; return; }
        double t = (R[0] + 1) * 0.5;
        rx = sqrt(t > 0 ? t : 0.);
        t = (R[4] + 1) * 0.5;
        ry = sqrt(t > 0 ? t : 0.) * (R[1] < 0 ? -1. : 1.);
        t = (R[8] + 1) * 0.5;
        rz = sqrt(t > 0 ? t : 0.) * (R[2] < 0 ? -1. : 1.);
        if (fabs(rx) < fabs(ry) && fabs(rx) < fabs(rz) && (R[5] > 0) != (ry * rz > 0)) rz = -rz;
        double n = sqrt(rx * rx + ry * ry + rz * rz);
        theta /= n;
        r[0] = rx * theta; r[1] = ry * theta; r[2] = rz * theta;
        return;
    }
    double vth = 1 / (2 * s);
    vth *= theta;
    r[0] = rx * vth; r[1] = ry * vth; r[2] = rz * vth;
}

static void mat3_mul(const double* A, const double* B, double* C) {
    double t[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += A[i * 3 + k] * B[k * 3 + j];
            t[i * 3 + j] = s;
        }
    memcpy(C, t, sizeof t);
}

/* 3x3 inverse by Gaussian elimination with partial pivoting (DECOMP_LU). */
static void mat3_inv(const double* A, double* Ai) {
    double a[3][6];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 6; j++) a[i][j] = j < 3 ? A[i * 3 + j] : (j - 3 == i ? 1.0 : 0.0);
    for (int c = 0; c < 3; c++) {
        int p = c;
        for (int i = c + 1; i < 3; i++)
            if (fabs(a[i][c]) > fabs(a[p][c])) p = i;
        if (p != c)
            for (int j = 0; j < 6; j++) { double t = a[c][j]; a[c][j] = a[p][j]; a[p][j] = t; }
        double d = 1.0 / a[c][c];
        for (int j = 0; j < 6; j++) a[c][j] *= d;
        for (int i = 0; i < 3; i++)
            if (i != c) {
                double f = a[i][c];
                for (int j = 0; j < 6; j++) a[i][j] -= f * a[c][j];
            }
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Ai[i * 3 + j] = a[i][j + 3];
}

/* undistortPoints with the default 5 fixed-point iterations (calib3d,
 * cvUndistortPointsInternal); R9 and P (p_cols 3 or 4) optional.  float in/out. */
void zo_undistort_points(const double K[9], const double D[5], const double* R9, const double* P,
                         int p_cols, const float* src, float* dst, int n) {
    double RR[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (R9) memcpy(RR, R9, sizeof RR);
    if (P) {
        double PP[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) PP[i * 3 + j] = P[i * p_cols + j];
        mat3_mul(PP, RR, RR);
    }
    const double fx = K[0], fy = K[4], cx = K[2], cy = K[5];
    const double ifx = 1. / fx, ify = 1. / fy;
    const double k0 = D ? D[0] : 0, k1 = D ? D[1] : 0, k2 = D ? D[2] : 0, k3 = D ? D[3] : 0,
                 k4 = D ? D[4] : 0;
    for (int i = 0; i < n; i++) {
        double x = src[2 * i], y = src[2 * i + 1];
        double u = x, v = y;
        x = (x - cx) * ifx;
        y = (y - cy) * ify;
        if (D) {
            double x0 = x, y0 = y;
            for (int j = 0; j < 5; j++) {
                double r2 = x * x + y * y;
                double icdist = 1.0 / (1 + ((k4 * r2 + k1) * r2 + k0) * r2);
                if (icdist < 0) {
                    x = (u - cx) * ifx;
                    y = (v - cy) * ify;
                    break;
                }
                double deltaX = 2 * k2 * x * y + k3 * (r2 + 2 * x * x);
                double deltaY = k2 * (r2 + 2 * y * y) + 2 * k3 * x * y;
                x = (x0 - deltaX) * icdist;
                y = (y0 - deltaY) * icdist;
            }
        }
        double xx = RR[0] * x + RR[1] * y + RR[2];
        double yy = RR[3] * x + RR[4] * y + RR[5];
        double ww = 1. / (RR[6] * x + RR[7] * y + RR[8]);
        dst[2 * i] = (float)(xx * ww);
        dst[2 * i + 1] = (float)(yy * ww);
    }
}

/* cv::stereoRectify(flags=0, alpha=-1, newImageSize=imageSize), the call at
 * src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:304-307. */
void zo_stereo_rectify(const zo_calib* c, double R1[9], double R2[9], double P1[12], double P2[12],
                       double Q[16]) {
    double om[3], r_r[9], t[3], uu[3] = {0, 0, 0}, ww[3], wR[9], Ri[9];
    const double nx = c->width, ny = c->height;
    zo_rodrigues_m2v(c->R, om);
    for (int i = 0; i < 3; i++) om[i] *= -0.5;
    zo_rodrigues_v2m(om, r_r);
    for (int i = 0; i < 3; i++) t[i] = r_r[i * 3] * c->t[0] + r_r[i * 3 + 1] * c->t[1] + r_r[i * 3 + 2] * c->t[2];
    int idx = fabs(t[0]) > fabs(t[1]) ? 0 : 1;
    double cc = t[idx], nt = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    uu[idx] = cc > 0 ? 1 : -1;
    ww[0] = t[1] * uu[2] - t[2] * uu[1];
    ww[1] = t[2] * uu[0] - t[0] * uu[2];
    ww[2] = t[0] * uu[1] - t[1] * uu[0];
    double nw = sqrt(ww[0] * ww[0] + ww[1] * ww[1] + ww[2] * ww[2]);
    if (nw > 0.0) {
        double s = acos(fabs(cc) / nt) / nw;
        for (int i = 0; i < 3; i++) ww[i] *= s;
    }
    zo_rodrigues_v2m(ww, wR);
    /* R1 = wR * r_r^T ; R2 = wR * r_r */
    double rrT[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) rrT[i * 3 + j] = r_r[j * 3 + i];
    mat3_mul(wR, rrT, Ri);
    memcpy(R1, Ri, sizeof Ri);
    mat3_mul(wR, r_r, Ri);
    memcpy(R2, Ri, sizeof Ri);
    for (int i = 0; i < 3; i++) t[i] = Ri[i * 3] * c->t[0] + Ri[i * 3 + 1] * c->t[1] + Ri[i * 3 + 2] * c->t[2];

    const double ratio = (idx == 1 ? nx / nx : ny / ny) / 2; /* newImageSize == imageSize */
    double fc_new = (c->K[0][(idx ^ 1) * 4] + c->K[1][(idx ^ 1) * 4]) * ratio;
    double ccx[2], ccy[2];
    for (int k = 0; k < 2; k++) {
        float pts[8], und[8];
        for (int i = 0; i < 4; i++) {
            int j = (i < 2) ? 0 : 1;
            pts[2 * i] = (float)((i % 2) * (nx - 1));
            pts[2 * i + 1] = (float)(j * (ny - 1));
        }
        zo_undistort_points(c->K[k], c->D[k], NULL, NULL, 3, pts, und, 4);
        const double* Rk = k == 0 ? R1 : R2;
        double sx = 0, sy = 0;
        for (int i = 0; i < 4; i++) {
            double X = und[2 * i], Y = und[2 * i + 1], Z = 1.0;
            double xr = Rk[0] * X + Rk[1] * Y + Rk[2] * Z;
            double yr = Rk[3] * X + Rk[4] * Y + Rk[5] * Z;
            double zr = Rk[6] * X + Rk[7] * Y + Rk[8] * Z;
            double iz = zr ? 1. / zr : 1;
            float px = (float)(fc_new * (xr * iz)), py = (float)(fc_new * (yr * iz));
            sx += px;
            sy += py;
        }
        ccx[k] = (nx - 1) / 2 - sx / 4;
        ccy[k] = (ny - 1) / 2 - sy / 4;
    }
    if (idx == 0) ccy[0] = ccy[1] = (ccy[0] + ccy[1]) * 0.5;
    else ccx[0] = ccx[1] = (ccx[0] + ccx[1]) * 0.5;
    /* alpha < 0: no scaling; newImageSize == imageSize */
    double cx1 = nx * ccx[0] / nx, cy1 = ny * ccy[0] / ny;
    double cx2 = nx * ccx[1] / nx, cy2 = ny * ccy[1] / ny;
    memset(P1, 0, 12 * sizeof(double));
    memset(P2, 0, 12 * sizeof(double));
    P1[0] = P1[5] = fc_new; P1[2] = cx1; P1[6] = cy1; P1[10] = 1;
    P2[0] = P2[5] = fc_new; P2[2] = cx2; P2[6] = cy2; P2[10] = 1;
    P2[idx * 4 + 3] = t[idx] * fc_new;
    memset(Q, 0, 16 * sizeof(double));
    Q[0] = 1; Q[3] = -cx1;
    Q[5] = 1; Q[7] = -cy1;
    Q[11] = fc_new;
    Q[14] = -1. / t[idx];
    Q[15] = (idx == 0 ? cx1 - cx2 : cy1 - cy2) / t[idx];
}

/* computeFullLeftRectification, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:248-289. */
void zo_full_left(const zo_calib* c, const double R1[9], double P1[12], double P2[12], double Q[16],
                  int* rect_w, int* rect_h) {
    float corners[8] = {0.0f, 0.0f, (float)c->width - 1.0f, 0.0f, (float)c->width - 1.0f,
                        (float)c->height - 1.0f, 0.0f, (float)c->height - 1.0f};
    float rc[8];
    zo_undistort_points(c->K[0], c->D[0], R1, P1, 4, corners, rc, 4);
    float min_x = rc[0], max_x = rc[0], min_y = rc[1], max_y = rc[1];
    for (int i = 0; i < 4; i++) {
        min_x = fminf(min_x, rc[2 * i]); max_x = fmaxf(max_x, rc[2 * i]);
        min_y = fminf(min_y, rc[2 * i + 1]); max_y = fmaxf(max_y, rc[2 * i + 1]);
    }
    double shift_x = -floor(min_x), shift_y = -floor(min_y);
    *rect_w = (int)ceil(max_x - min_x + 1.0f);
    *rect_h = (int)ceil(max_y - min_y + 1.0f);
    P1[2] += shift_x; P1[6] += shift_y;
    P2[2] += shift_x; P2[6] += shift_y;
    Q[3] -= shift_x; Q[7] -= shift_y;
}

/* initUndistortRectifyMap(..., CV_32FC1).  The homogeneous ray of pixel (j, i)
 * is evaluated directly as ir*(j, i, 1) instead of OpenCV's running sum. */
void zo_init_rectify_map(const double K[9], const double D[5], const double R[9], const double P[12],
                         int w, int h, float* mapx, float* mapy) {
    double A[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]}, AR[9], ir[9];
    mat3_mul(A, R, AR);
    mat3_inv(AR, ir);
    const double u0 = K[2], v0 = K[5], fx = K[0], fy = K[4];
    const double k1 = D[0], k2 = D[1], p1 = D[2], p2 = D[3], k3 = D[4];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < h; i++) {
        for (int j = 0; j < w; j++) {
            double _x = ir[0] * j + (ir[1] * i + ir[2]);
            double _y = ir[3] * j + (ir[4] * i + ir[5]);
            double _w = ir[6] * j + (ir[7] * i + ir[8]);
            double ww = 1. / _w, x = _x * ww, y = _y * ww;
            double x2 = x * x, y2 = y * y;
            double r2 = x2 + y2, _2xy = 2 * x * y;
            double kr = 1 + ((k3 * r2 + k2) * r2 + k1) * r2;
            double u = fx * (x * kr + p1 * _2xy + p2 * (r2 + 2 * x2)) + u0;
            double v = fy * (y * kr + p1 * (r2 + 2 * y2) + p2 * _2xy) + v0;
            mapx[(size_t)i * w + j] = (float)u;
            mapy[(size_t)i * w + j] = (float)v;
        }
    }
}

/* remap INTER_LINEAR: position rounded to 1/32 px (INTER_BITS = 5), weights
 * (1-fx, fx) x (1-fy, fy), taps outside the source read 0 (BORDER_CONSTANT). */
void zo_remap_linear(const double* src, int srows, int scols, const float* mapx, const float* mapy,
                     int drows, int dcols, double* dst) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < drows; i++) {
        for (int j = 0; j < dcols; j++) {
            size_t o = (size_t)i * dcols + j;
            int sx = (int)lrintf(mapx[o] * 32.0f), sy = (int)lrintf(mapy[o] * 32.0f);
            int x0 = sx >> 5, y0 = sy >> 5;
            double fx = (sx & 31) / 32.0, fy = (sy & 31) / 32.0;
            float wx[2] = {(float)(1.0 - fx), (float)fx}, wy[2] = {(float)(1.0 - fy), (float)fy};
            double v[4];
            for (int t = 0; t < 4; t++) {
                int xx = x0 + (t & 1), yy = y0 + (t >> 1);
                v[t] = (xx >= 0 && yy >= 0 && xx < scols && yy < srows) ? src[(size_t)yy * scols + xx] : 0.0;
            }
            double r = v[0] * (double)(wy[0] * wx[0]);
            r += v[1] * (double)(wy[0] * wx[1]);
            r += v[2] * (double)(wy[1] * wx[0]);
            r += v[3] * (double)(wy[1] * wx[1]);
            dst[o] = r;
        }
    }
}

/* remap INTER_LINEAR of an 8-bit image (rectifyLeftImage, V2.cpp:920-924):
 * OpenCV's fixed-point path -- 1/32-pixel positions, integer weights
 * (32 - f or f) x (32 - g or g) x 32 summing to 32768, (sum + 2^14) >> 15,
 * BORDER_CONSTANT 0. */
void zo_remap_u8(const uint8_t* src, int srows, int scols, const float* mapx, const float* mapy, int drows,
                 int dcols, uint8_t* dst) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < drows; i++) {
        for (int j = 0; j < dcols; j++) {
            size_t o = (size_t)i * dcols + j;
            int sx = (int)lrintf(mapx[o] * 32.0f), sy = (int)lrintf(mapy[o] * 32.0f);
            int x0 = sx >> 5, y0 = sy >> 5, fx = sx & 31, fy = sy & 31;
            int wx[2] = {32 - fx, fx}, wy[2] = {32 - fy, fy};
            int acc = 0;
            for (int t = 0; t < 4; t++) {
                int xx = x0 + (t & 1), yy = y0 + (t >> 1);
                int v = (xx >= 0 && yy >= 0 && xx < scols && yy < srows) ? src[(size_t)yy * scols + xx] : 0;
                acc += v * wy[t >> 1] * wx[t & 1] * 32;
            }
            acc = (acc + (1 << 14)) >> 15;
            dst[o] = (uint8_t)(acc > 255 ? 255 : acc);
        }
    }
}

/* remap INTER_NEAREST: position rounded to nearest (ties to even), BORDER_CONSTANT 0. */
void zo_remap_nearest(const int32_t* src, int srows, int scols, const float* mapx, const float* mapy,
                      int drows, int dcols, int32_t* dst) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < drows; i++) {
        for (int j = 0; j < dcols; j++) {
            size_t o = (size_t)i * dcols + j;
            int xx = (int)lrintf(mapx[o]), yy = (int)lrintf(mapy[o]);
            dst[o] = (xx >= 0 && yy >= 0 && xx < scols && yy < srows) ? src[(size_t)yy * scols + xx] : 0;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* stereoMatch, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:933-1006. */
/* ROI matching, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:719-778: left window
 * (lcols wide, masked) against a right column window (rcols wide) of the same
 * rows; edge rejection relative to the right window; disparity = global left
 * x - global right x - delta with dx_off = left x - right x. */
void zo_stereo_match_roi(const double* lph, const int32_t* lk, const uint8_t* lmask, int lcols, const double* rph,
                         const int32_t* rk, int rcols, int rows, int dx_off, int pha_f, double grad_threshold,
                         double* disp, int32_t* best, uint8_t* near, double eps) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < rows; i++) {
        const double* rp = rph + (size_t)i * rcols;
        const int32_t* rkr = rk + (size_t)i * rcols;
        for (int j = 0; j < lcols; j++) {
            size_t o = (size_t)i * lcols + j;
            disp[o] = 0.0;
            if (best) best[o] = -1;
            if (near) near[o] = 0;
            if (!lmask[o]) continue;
            int k = lk[o];
            if (k > pha_f || k <= 0) continue;
            double min_cost = 1e9, second = 1e9;
            int best_jR = -1;
            double l_val = lph[o];
            for (int c = 0; c < rcols; c++) {
                if (rkr[c] != k) continue;
                double diff = fabs(rp[c] - l_val);
                if (diff < min_cost) {
                    second = min_cost;
                    min_cost = diff;
                    best_jR = c;
                } else if (diff < second) {
                    second = diff;
                }
            }
            if (best_jR < 0) continue;
            if (near) {
                uint8_t f = 0;
                if (second - min_cost < eps) f |= 1;
                if (fabs(min_cost - grad_threshold) < eps) f |= 2;
                near[o] = f;
            }
            if (min_cost >= grad_threshold) continue;
            if (best_jR < 2 || best_jR >= rcols - 1) continue;
            double cost0 = rp[best_jR - 1] - l_val;
            double cost1 = rp[best_jR] - l_val;
            double cost2 = rp[best_jR + 1] - l_val;
            double num = cost1 * (cost0 - cost2);
            double den = 2.0 * (cost0 - cost1) * (cost1 - cost2);
            double delta = 0.0;
            if (fabs(den) > 1e-9) delta = num / den;
            disp[o] = (double)(j + dx_off) - (double)best_jR - delta;
            if (best) best[o] = best_jR;
        }
    }
}

void zo_stereo_match(const double* lph, const double* rph, const int32_t* lk, const int32_t* rk,
                     int rows, int cols, int pha_f, double grad_threshold, double* disp,
                     int32_t* best, uint8_t* near, double eps) {
    const int knum = pha_f;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < rows; i++) {
        const double* lp = lph + (size_t)i * cols;
        const double* rp = rph + (size_t)i * cols;
        const int32_t* lkr = lk + (size_t)i * cols;
        const int32_t* rkr = rk + (size_t)i * cols;
        for (int j = 0; j < cols; j++) {
            size_t o = (size_t)i * cols + j;
            disp[o] = 0.0;
            if (best) best[o] = -1;
            if (near) near[o] = 0;
            int k = lkr[j];
            if (k > pha_f || k <= 0) continue;
            if (k > knum) continue;
            double min_cost = 1e9, second = 1e9;
            int best_jR = -1;
            double l_val = lp[j];
            for (int c = 0; c < cols; c++) {
                if (rkr[c] != k) continue;
                double diff = fabs(rp[c] - l_val);
                if (diff < min_cost) {
                    second = min_cost;
                    min_cost = diff;
                    best_jR = c;
                } else if (diff < second) {
                    second = diff;
                }
            }
            if (best_jR < 0) continue;
            if (near) {
                uint8_t f = 0;
                if (second - min_cost < eps) f |= 1;
                if (fabs(min_cost - grad_threshold) < eps) f |= 2;
                near[o] = f;
            }
            if (min_cost >= grad_threshold) continue;
            if (best_jR < 2 || best_jR >= cols - 1) continue;
            double cost0 = rp[best_jR - 1] - l_val;
            double cost1 = rp[best_jR] - l_val;
            double cost2 = rp[best_jR + 1] - l_val;
            double num = cost1 * (cost0 - cost2);
            double den = 2.0 * (cost0 - cost1) * (cost1 - cost2);
            double delta = 0.0;
            if (fabs(den) > 1e-9) delta = num / den;
            disp[o] = (double)j - (double)best_jR - delta;
            if (best) best[o] = best_jR;
        }
    }
}

static int cmp_float(const void* a, const void* b) {
    float x = *(const float*)a, y = *(const float*)b;
    return (x > y) - (x < y);
}

/* medianBlur(ksize 5) on CV_32F: order statistic 13 of 25, BORDER_REPLICATE. */
void zo_median5(const float* src, float* dst, int rows, int cols) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++) {
        float v[25];
        for (int j = 0; j < cols; j++) {
            int n = 0;
            for (int dy = -2; dy <= 2; dy++)
                for (int dx = -2; dx <= 2; dx++)
                    v[n++] = src[(size_t)clampi(i + dy, 0, rows - 1) * cols + clampi(j + dx, 0, cols - 1)];
            qsort(v, 25, sizeof(float), cmp_float);
            dst[(size_t)i * cols + j] = v[12];
        }
    }
}

/* Reprojection, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:414-461. */
void zo_reproject(const float* disp, int rows, int cols, const double Q[16], const double R1[9],
                  double min_depth, double max_depth, int use_rectified, float* xyz, uint8_t* mask,
                  uint8_t* near, double eps) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            size_t o = (size_t)i * cols + j;
            xyz[3 * o] = xyz[3 * o + 1] = xyz[3 * o + 2] = 0.0f;
            mask[o] = 0;
            if (near) near[o] = 0;
            double d = disp[o];
            if (fabs(d) < 1e-5) continue;
            double w = Q[14] * d + Q[15];
            double x = j + Q[3];
            double y = i + Q[7];
            double z = Q[11];
            double inv_w = 1.0 / w;
            x *= inv_w; y *= inv_w; z *= inv_w;
            double rx = R1[0] * x + R1[3] * y + R1[6] * z;
            double ry = R1[1] * x + R1[4] * y + R1[7] * z;
            double rz = R1[2] * x + R1[5] * y + R1[8] * z;
            double gz = use_rectified ? z : rz;
            if (near && (fabs(gz - min_depth) < eps * (1 + fabs(gz)) ||
                         fabs(gz - max_depth) < eps * (1 + fabs(gz))))
                near[o] = 1;
            if (gz > min_depth && gz < max_depth) {
                if (use_rectified) {
                    xyz[3 * o] = (float)x; xyz[3 * o + 1] = (float)y; xyz[3 * o + 2] = (float)z;
                } else {
                    xyz[3 * o] = (float)rx; xyz[3 * o + 1] = (float)ry; xyz[3 * o + 2] = (float)rz;
                }
                mask[o] = 1;
            }
        }
    }
}

/* evaluateV2CalibPoint, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76: model
 * tags in c3 of the x map (-1 inverse depth, -2 fitted ray, -3 z-linear x/y) and
 * of the z map (-1 inverse depth, -4 rational); otherwise cubics in d.  Tag tests
 * are float arithmetic, the evaluation double (built without contraction). */
static int zo_poly_point(const float* cx, const float* cy, const float* cz, double d, double* xr, double* yr,
                         double* zr) {
    const float inv_tag = -1.0f, ray_tag = -2.0f, lin_tag = -3.0f, rat_tag = -4.0f;
    if (fabsf(cz[0]) <= 1e-9 && fabsf(cz[1]) <= 1e-9 && fabsf(cz[2]) <= 1e-9 && fabsf(cz[3]) <= 1e-9) return 0;
    if (fabsf(cx[3] - inv_tag) < 1e-6f) {
        double d2 = d * d;
        double inv_z = cz[0] + cz[1] * d + cz[2] * d2 + cz[3] * d2 * d;
        if (!isfinite(inv_z) || fabs(inv_z) < 1e-12) return 0;
        *zr = 1.0 / inv_z;
        *xr = cx[0] * *zr;
        *yr = cy[0] * *zr;
    } else if (fabsf(cx[3] - ray_tag) < 1e-6f) {
        double d2 = d * d;
        if (fabsf(cz[3] - inv_tag) < 1e-6f) {
            double inv_z = cz[0] + cz[1] * d + cz[2] * d2;
            if (!isfinite(inv_z) || fabs(inv_z) < 1e-12) return 0;
            *zr = 1.0 / inv_z;
        } else {
            *zr = cz[0] + cz[1] * d + cz[2] * d2 + cz[3] * d2 * d;
        }
        *xr = cx[0] * *zr;
        *yr = cy[0] * *zr;
    } else if (fabsf(cx[3] - lin_tag) < 1e-6f) {
        if (fabsf(cz[3] - rat_tag) < 1e-6f) {
            double denom = cz[1] * d + 1.0;
            if (!isfinite(denom) || fabs(denom) < 1e-12) return 0;
            *zr = cz[0] / denom;
        } else {
            double d2 = d * d, d3 = d2 * d;
            *zr = cz[0] + cz[1] * d + cz[2] * d2 + cz[3] * d3;
        }
        *xr = cx[0] * *zr + cx[1];
        *yr = cy[0] * *zr + cy[1];
    } else if (fabsf(cz[3] - inv_tag) < 1e-6f) {
        double inv_z = cz[0] + cz[1] * d + cz[2] * d * d;
        if (!isfinite(inv_z) || fabs(inv_z) < 1e-12) return 0;
        *zr = 1.0 / inv_z;
        *xr = cx[0] * *zr;
        *yr = cy[0] * *zr;
    } else {
        double d2 = d * d, d3 = d2 * d;
        *xr = cx[0] + cx[1] * d + cx[2] * d2 + cx[3] * d3;
        *yr = cy[0] + cy[1] * d + cy[2] * d2 + cy[3] * d3;
        *zr = cz[0] + cz[1] * d + cz[2] * d2 + cz[3] * d3;
    }
    return isfinite(*xr) && isfinite(*yr) && isfinite(*zr);
}

/* startCalculate_v2's reprojection loop, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:500-566
 * (maps: rows*cols*4 floats each). */
void zo_poly_reproject(const float* disp, int rows, int cols, const float* mx, const float* my, const float* mz,
                       const double R1[9], double min_depth, double max_depth, int use_rectified, float* xyz,
                       uint8_t* mask) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            size_t o = (size_t)i * cols + j;
            xyz[3 * o] = xyz[3 * o + 1] = xyz[3 * o + 2] = 0.0f;
            mask[o] = 0;
            double d = disp[o];
            if (fabs(d) < 1e-5) continue;
            double x, y, z;
            if (!zo_poly_point(mx + 4 * o, my + 4 * o, mz + 4 * o, d, &x, &y, &z)) continue;
            double rx = R1[0] * x + R1[3] * y + R1[6] * z;
            double ry = R1[1] * x + R1[4] * y + R1[7] * z;
            double rz = R1[2] * x + R1[5] * y + R1[8] * z;
            if (use_rectified) {
                if (z > min_depth && z < max_depth) {
                    xyz[3 * o] = (float)x; xyz[3 * o + 1] = (float)y; xyz[3 * o + 2] = (float)z;
                    mask[o] = 1;
                }
            } else if (rz > min_depth && rz < max_depth) {
                xyz[3 * o] = (float)rx; xyz[3 * o + 1] = (float)ry; xyz[3 * o + 2] = (float)rz;
                mask[o] = 1;
            }
        }
    }
}

/* applyGaussianFilterToPointCloudV2, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:79-124
 * (win 3, sigma 0.7 px, float kernel), GPU mask update from
 * src/JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:220-274. */
void zo_px_gaussian(const float* xyz, const uint8_t* mask, int rows, int cols, float* out,
                    uint8_t* mask_out, uint8_t* near, double eps) {
    double k[3];
    zo_gaussian_kernel3(0.7, k);
    float kf[3] = {(float)k[0], (float)k[1], (float)k[2]};
    float w[9];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) w[a * 3 + b] = kf[a] * kf[b];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            size_t o = (size_t)i * cols + j;
            out[3 * o] = out[3 * o + 1] = out[3 * o + 2] = 0.0f;
            if (mask_out) mask_out[o] = 0;
            if (near) near[o] = 0;
            if (i < 1 || i >= rows - 1 || j < 1 || j >= cols - 1) continue;
            if (!mask[o]) continue;
            double sx = 0, sy = 0, sz = 0, cnt = 0;
            uint8_t nf = 0;
            const double cx = xyz[3 * o];
            for (int ik = -1; ik <= 1; ik++)
                for (int jk = -1; jk <= 1; jk++) {
                    size_t q = (size_t)(i + ik) * cols + (j + jk);
                    if (!mask[q]) continue;
                    double dx = fabs((double)xyz[3 * q] - cx);
                    if (fabs(dx - 3.0) < eps) nf = 1;
                    if (dx < 3.0) {
                        double ww = w[(ik + 1) * 3 + (jk + 1)];
                        sx += xyz[3 * q] * ww; sy += xyz[3 * q + 1] * ww; sz += xyz[3 * q + 2] * ww;
                        cnt += ww;
                    }
                }
            if (fabs(cnt - 0.8) < eps) nf = 1;
            if (near) near[o] = nf;
            if (cnt > 0.8) {
                out[3 * o] = (float)(sx / cnt); out[3 * o + 1] = (float)(sy / cnt); out[3 * o + 2] = (float)(sz / cnt);
                if (mask_out) mask_out[o] = 1;
            }
        }
    }
}

/* applyRadiusOutlierFilterToPointCloud, src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:126-195. */
void zo_ror(const float* xyz, const uint8_t* mask, int rows, int cols, float radius, int min_neighbors,
            int window_size, float* out, uint8_t* mask_out, uint8_t* near, double eps) {
    const double r2 = (double)radius * (double)radius;
    const int hw = window_size / 2;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            size_t o = (size_t)i * cols + j;
            out[3 * o] = out[3 * o + 1] = out[3 * o + 2] = 0.0f;
            mask_out[o] = 0;
            if (near) near[o] = 0;
            if (!mask[o]) continue;
            int sure = 0, maybe = 0;
            for (int ii = (i - hw < 0 ? 0 : i - hw); ii < (i + hw + 1 > rows ? rows : i + hw + 1); ii++)
                for (int jj = (j - hw < 0 ? 0 : j - hw); jj < (j + hw + 1 > cols ? cols : j + hw + 1); jj++) {
                    size_t q = (size_t)ii * cols + jj;
                    if (!mask[q] || q == o) continue;
                    double dx = (double)xyz[3 * o] - xyz[3 * q], dy = (double)xyz[3 * o + 1] - xyz[3 * q + 1],
                           dz = (double)xyz[3 * o + 2] - xyz[3 * q + 2];
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (fabs(d2 - r2) < 0.1 * eps * r2) maybe++; /* FP32 |d|^2 is good to ~3e-7 relative */
                    else if (d2 <= r2) sure++;
                }
            if (near && sure < min_neighbors && sure + maybe >= min_neighbors) near[o] = 1;
            /* the decision proper, counting the ambiguous ones by their exact value */
            int cnt = 0;
            for (int ii = (i - hw < 0 ? 0 : i - hw); ii < (i + hw + 1 > rows ? rows : i + hw + 1) && cnt < min_neighbors; ii++)
                for (int jj = (j - hw < 0 ? 0 : j - hw); jj < (j + hw + 1 > cols ? cols : j + hw + 1); jj++) {
                    size_t q = (size_t)ii * cols + jj;
                    if (!mask[q] || q == o) continue;
                    double dx = (double)xyz[3 * o] - xyz[3 * q], dy = (double)xyz[3 * o + 1] - xyz[3 * q + 1],
                           dz = (double)xyz[3 * o + 2] - xyz[3 * q + 2];
                    if (dx * dx + dy * dy + dz * dz <= r2) {
                        if (++cnt >= min_neighbors) break;
                    }
                }
            if (cnt >= min_neighbors) {
                out[3 * o] = xyz[3 * o]; out[3 * o + 1] = xyz[3 * o + 1]; out[3 * o + 2] = xyz[3 * o + 2];
                mask_out[o] = 1;
            }
        }
    }
}

/* ---- MLS (src/JSLAB_MLS_Filter.cpp:11-441), in FP64 ---- */
static void sym_eigen3(const double C[3][3], double ev[3], double evec[3][3]) {
    /* src/JSLAB_MLS_Filter.cpp:11-106 */
    const double p1 = C[0][1] * C[0][1] + C[0][2] * C[0][2] + C[1][2] * C[1][2];
    if (p1 < 1e-20) {
        ev[0] = C[0][0]; ev[1] = C[1][1]; ev[2] = C[2][2];
        double E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int i = 0; i < 2; i++)
            for (int j = i + 1; j < 3; j++)
                if (ev[i] > ev[j]) {
                    double t = ev[i]; ev[i] = ev[j]; ev[j] = t;
                    for (int c = 0; c < 3; c++) { t = E[i][c]; E[i][c] = E[j][c]; E[j][c] = t; }
                }
        memcpy(evec, E, sizeof E);
        return;
    }
    const double trace = C[0][0] + C[1][1] + C[2][2];
    const double q = trace / 3.0;
    double B[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] = C[i][j];
    B[0][0] -= q; B[1][1] -= q; B[2][2] -= q;
    double p2 = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2] + 2.0 * p1;
    double p = sqrt(p2 / 6.0);
    double inv_p = (p > 1e-15) ? (1.0 / p) : 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] *= inv_p;
    double detB = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) -
                  B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                  B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
    double r = detB * 0.5;
    r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
    double phi = acos(r) / 3.0;
    ev[0] = q + 2.0 * p * cos(phi + 2.0 * ZO_PI / 3.0);
    ev[2] = q + 2.0 * p * cos(phi);
    ev[1] = trace - ev[0] - ev[2];
    for (int idx = 0; idx < 3; idx++) {
        double A[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) A[i][j] = C[i][j];
        A[0][0] -= ev[idx]; A[1][1] -= ev[idx]; A[2][2] -= ev[idx];
        double c01[3] = {A[0][1] * A[1][2] - A[0][2] * A[1][1], A[0][2] * A[1][0] - A[0][0] * A[1][2],
                         A[0][0] * A[1][1] - A[0][1] * A[1][0]};
        double c02[3] = {A[0][1] * A[2][2] - A[0][2] * A[2][1], A[0][2] * A[2][0] - A[0][0] * A[2][2],
                         A[0][0] * A[2][1] - A[0][1] * A[2][0]};
        double c12[3] = {A[1][1] * A[2][2] - A[1][2] * A[2][1], A[1][2] * A[2][0] - A[1][0] * A[2][2],
                         A[1][0] * A[2][1] - A[1][1] * A[2][0]};
        double l01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
        double l02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
        double l12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
        double* bst = c12;
        double bl = l12;
        if (l01 > bl) { bst = c01; bl = l01; }
        if (l02 > bl) { bst = c02; bl = l02; }
        double il = (bl > 1e-20) ? (1.0 / sqrt(bl)) : 0.0;
        for (int c = 0; c < 3; c++) evec[idx][c] = bst[c] * il;
    }
}

static int cholesky_solve(double A[6][6], const double b[6], double x[6], int nc) {
    /* src/JSLAB_MLS_Filter.cpp:113-156 */
    double L[6][6] = {{0}};
    for (int i = 0; i < nc; i++)
        for (int j = 0; j <= i; j++) {
            double s = A[i][j];
            for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (s <= 1e-12) return 0;
                L[i][j] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    double y[6] = {0};
    for (int i = 0; i < nc; i++) {
        double s = b[i];
        for (int k = 0; k < i; k++) s -= L[i][k] * y[k];
        y[i] = s / L[i][i];
    }
    for (int i = nc - 1; i >= 0; i--) {
        double s = y[i];
        for (int k = i + 1; k < nc; k++) s -= L[k][i] * x[k];
        x[i] = s / L[i][i];
    }
    return 1;
}

/* Deterministic factor in [1 - j, 1 + j] for neighbour q of point o (jitter
 * used to estimate a point's sensitivity to rounding; 1 when j == 0). */
static inline double jit(double j, uint64_t seed, size_t o, size_t q) {
    if (j == 0) return 1.0;
    uint64_t h = seed * 0x9E3779B97F4A7C15ull ^ (o * 0xBF58476D1CE4E5B9ull) ^ (q * 0x94D049BB133111EBull);
    h ^= h >> 31; h *= 0xD6E8FEB86659FD93ull; h ^= h >> 32;
    return 1.0 + j * (((double)(h >> 11) / 9007199254740992.0) * 2.0 - 1.0);
}

/* One MLS pass, src/JSLAB_MLS_Filter.cpp:161-391 (CPU order fallback: order
 * drops to 0 when fewer than min_neighbors[order] neighbours, :277-280).
 * jitter > 0 scales every neighbour offset q - p by a pseudo-random factor in
 * [1 - jitter, 1 + jitter] (sensitivity estimate only). */
static void mls_pass(const float* src, const uint8_t* mask, int rows, int cols, int hw, double sigma,
                     int order_in, double r2c, double* dst, uint8_t* near, double eps, double jitter,
                     uint64_t seed) {
    const double inv_2s2 = 1.0 / (2.0 * sigma * sigma);
    const int min_nb[3] = {3, 5, 8};
    const int order = order_in < 0 ? 0 : (order_in > 2 ? 2 : order_in);
    for (size_t i = 0; i < 3 * (size_t)rows * cols; i++) dst[i] = src[i];
#pragma omp parallel for schedule(dynamic, 2)
    for (int irow = 0; irow < rows; irow++) {
        for (int jcol = 0; jcol < cols; jcol++) {
            size_t o = (size_t)irow * cols + jcol;
            if (!mask[o]) continue;
            const double px = src[3 * o], py = src[3 * o + 1], pz = src[3 * o + 2];
            int r0 = irow - hw < 0 ? 0 : irow - hw, r1 = irow + hw + 1 > rows ? rows : irow + hw + 1;
            int c0 = jcol - hw < 0 ? 0 : jcol - hw, c1 = jcol + hw + 1 > cols ? cols : jcol + hw + 1;
            double cx = 0, cy = 0, cz = 0, wsum = 0;
            int nv = 0;
            uint8_t nf = 0;
            for (int ir = r0; ir < r1; ir++)
                for (int jc = c0; jc < c1; jc++) {
                    size_t q = (size_t)ir * cols + jc;
                    if (!mask[q]) continue;
                    const double jf = jit(jitter, seed, o, q);
                    const double qx = px + (src[3 * q] - px) * jf, qy = py + (src[3 * q + 1] - py) * jf,
                                 qz = pz + (src[3 * q + 2] - pz) * jf;
                    double dx = qx - px, dy = qy - py, dz = qz - pz;
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (fabs(d2 - r2c) < 0.1 * eps * r2c) nf = 1;
                    if (d2 > r2c) continue;
                    double w = exp(-d2 * inv_2s2);
                    cx += w * qx; cy += w * qy; cz += w * qz;
                    wsum += w;
                    nv++;
                }
            if (near) near[o] = nf;
            if (nv < min_nb[0] || wsum < 1e-12) continue;
            double iw = 1.0 / wsum;
            cx *= iw; cy *= iw; cz *= iw;
            double cov[3][3] = {{0}};
            for (int ir = r0; ir < r1; ir++)
                for (int jc = c0; jc < c1; jc++) {
                    size_t q = (size_t)ir * cols + jc;
                    if (!mask[q]) continue;
                    const double jf = jit(jitter, seed, o, q);
                    const double qx = px + (src[3 * q] - px) * jf, qy = py + (src[3 * q + 1] - py) * jf,
                                 qz = pz + (src[3 * q + 2] - pz) * jf;
                    double dx = qx - px, dy = qy - py, dz = qz - pz;
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > r2c) continue;
                    double w = exp(-d2 * inv_2s2);
                    double ex = qx - cx, ey = qy - cy, ez = qz - cz;
                    cov[0][0] += w * ex * ex; cov[0][1] += w * ex * ey; cov[0][2] += w * ex * ez;
                    cov[1][1] += w * ey * ey; cov[1][2] += w * ey * ez; cov[2][2] += w * ez * ez;
                }
            cov[1][0] = cov[0][1]; cov[2][0] = cov[0][2]; cov[2][1] = cov[1][2];
            double ev[3], E[3][3];
            sym_eigen3(cov, ev, E);
            double nx = E[0][0], ny = E[0][1], nz = E[0][2];
            double t1x = E[1][0], t1y = E[1][1], t1z = E[1][2];
            double t2x = E[2][0], t2y = E[2][1], t2z = E[2][2];
            int cur = (nv >= min_nb[order]) ? order : 0;
            /* FP32 conditioning of the frame: a covariance known to a relative 2^-23
             * turns the normal by about 2^-23 * l2 / (l1 - l0); flag the point when
             * that moves the projection by more than eps (mm). */
            const double lever = sqrt((px - cx) * (px - cx) + (py - cy) * (py - cy) + (pz - cz) * (pz - cz)) +
                                 sqrt(fmax(ev[2], 0.0) / wsum);
            const double kappa = fabs(ev[2]) / fmax(ev[1] - ev[0], 1e-300);
            if (near && 4.0 * 1.2e-7 * kappa * lever > eps) near[o] = 1;
            double* out = dst + 3 * o;
            if (cur == 0) {
                double dot = (px - cx) * nx + (py - cy) * ny + (pz - cz) * nz;
                out[0] = px - dot * nx; out[1] = py - dot * ny; out[2] = pz - dot * nz;
                continue;
            }
            const int nc = (cur == 1) ? 3 : 6;
            double AtWA[6][6] = {{0}}, AtWf[6] = {0};
            for (int ir = r0; ir < r1; ir++)
                for (int jc = c0; jc < c1; jc++) {
                    size_t q = (size_t)ir * cols + jc;
                    if (!mask[q]) continue;
                    const double jf = jit(jitter, seed, o, q);
                    const double qx = px + (src[3 * q] - px) * jf, qy = py + (src[3 * q + 1] - py) * jf,
                                 qz = pz + (src[3 * q + 2] - pz) * jf;
                    double dx = qx - px, dy = qy - py, dz = qz - pz;
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > r2c) continue;
                    double w = exp(-d2 * inv_2s2);
                    double ex = qx - cx, ey = qy - cy, ez = qz - cz;
                    double u = ex * t1x + ey * t1y + ez * t1z;
                    double v = ex * t2x + ey * t2y + ez * t2z;
                    double f = ex * nx + ey * ny + ez * nz;
                    double bs[6] = {1.0, u, v, u * u, u * v, v * v};
                    for (int a = 0; a < nc; a++) {
                        AtWf[a] += w * bs[a] * f;
                        for (int b = a; b < nc; b++) AtWA[a][b] += w * bs[a] * bs[b];
                    }
                }
            for (int a = 0; a < nc; a++)
                for (int b = 0; b < a; b++) AtWA[a][b] = AtWA[b][a];
            if (near) {
                /* FP32 conditioning of the normal equations in a basis scaled by the
                 * cut-off radius: pivot ratio of the scaled Cholesky factor. */
                static const int deg[6] = {0, 1, 1, 2, 2, 2};
                double h = sqrt(r2c), S[6][6], L[6][6] = {{0}}, lmin = DBL_MAX, lmax = 0;
                int ok = 1;
                for (int a = 0; a < nc; a++)
                    for (int b = 0; b < nc; b++) S[a][b] = AtWA[a][b] / pow(h, deg[a] + deg[b]);
                for (int i = 0; i < nc && ok; i++)
                    for (int j = 0; j <= i; j++) {
                        double s = S[i][j];
                        for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
                        if (i == j) {
                            if (s <= 0) { ok = 0; break; }
                            L[i][i] = sqrt(s);
                            lmin = fmin(lmin, L[i][i]);
                            lmax = fmax(lmax, L[i][i]);
                        } else {
                            L[i][j] = s / L[j][j];
                        }
                    }
                double condA = ok ? (lmax / lmin) * (lmax / lmin) : 1e300;
                double fscale = sqrt(fmax(ev[0], 0.0) / wsum);
                if (4.0 * 1.2e-7 * condA * fscale > eps) near[o] = 1;
            }
            double co[6] = {0};
            int solved = cholesky_solve(AtWA, AtWf, co, nc);
            if (!solved && cur == 2) {
                double A1[6][6] = {{0}}, b1[6] = {0};
                for (int a = 0; a < 3; a++) {
                    b1[a] = AtWf[a];
                    for (int b = 0; b < 3; b++) A1[a][b] = AtWA[a][b];
                }
                solved = cholesky_solve(A1, b1, co, 3);
                if (solved) cur = 1;
            }
            if (!solved) {
                double dot = (px - cx) * nx + (py - cy) * ny + (pz - cz) * nz;
                out[0] = px - dot * nx; out[1] = py - dot * ny; out[2] = pz - dot * nz;
                continue;
            }
            double ex0 = px - cx, ey0 = py - cy, ez0 = pz - cz;
            double u0 = ex0 * t1x + ey0 * t1y + ez0 * t1z;
            double v0 = ex0 * t2x + ey0 * t2y + ez0 * t2z;
            double ff = co[0] + co[1] * u0 + co[2] * v0;
            if (cur == 2) ff += co[3] * u0 * u0 + co[4] * u0 * v0 + co[5] * v0 * v0;
            out[0] = cx + u0 * t1x + v0 * t2x + ff * nx;
            out[1] = cy + u0 * t1y + v0 * t2y + ff * ny;
            out[2] = cz + u0 * t1z + v0 * t2z + ff * nz;
        }
    }
}

void zo_mls(const float* xyz, const uint8_t* mask, int rows, int cols, int window, float sigma, int order,
            float max_radius, int iterations, double* out, uint8_t* near, double eps, double jitter,
            unsigned long long seed) {
    /* src/JSLAB_MLS_Filter.cpp:397-415: cut-off max_radius^2, or 9 sigma^2 when 0. */
    const double r2c = (max_radius > 0.0f) ? (double)max_radius * max_radius : 9.0 * (double)sigma * sigma;
    const int n_iter = iterations < 1 ? 1 : iterations;
    size_t n = (size_t)rows * cols * 3;
    float* cur = (float*)malloc(sizeof(float) * n);
    memcpy(cur, xyz, sizeof(float) * n);
    uint8_t* nf = near ? (uint8_t*)calloc((size_t)rows * cols, 1) : NULL;
    for (int it = 0; it < n_iter; it++) {
        mls_pass(cur, mask, rows, cols, window, sigma, order, r2c, out, nf, eps, jitter, seed + it);
        if (near)
            for (size_t i = 0; i < (size_t)rows * cols; i++) near[i] |= nf[i];
        if (it + 1 < n_iter)
            for (size_t i = 0; i < n; i++) cur[i] = (float)out[i]; /* the reference iterates on CV_32F */
    }
    free(cur);
    free(nf);
}

/* ---- uniform grid for exact kNN / radius queries (oracle side) ---- */
typedef struct {
    int n;
    const float* p;       /* 3 floats per point */
    int* idx;             /* point ids sorted by cell */
    long long* key;       /* cell keys, sorted, parallel to idx */
    double cell, ox, oy, oz;
    int nx, ny, nz;
} zo_grid;

static long long cell_key(const zo_grid* g, int ix, int iy, int iz) {
    return ((long long)iz * g->ny + iy) * g->nx + ix;
}

static int cmp_pair(const void* a, const void* b) {
    const long long* x = (const long long*)a;
    const long long* y = (const long long*)b;
    if (x[0] != y[0]) return (x[0] > y[0]) - (x[0] < y[0]);
    return (x[1] > y[1]) - (x[1] < y[1]);
}

static void grid_build(zo_grid* g, const float* p, const int* ids, int n, double cell) {
    g->n = n; g->p = p; g->cell = cell;
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            double v = p[3 * ids[i] + c];
            if (v < mn[c]) mn[c] = v;
            if (v > mx[c]) mx[c] = v;
        }
    g->ox = mn[0]; g->oy = mn[1]; g->oz = mn[2];
    g->nx = (int)((mx[0] - mn[0]) / cell) + 1;
    g->ny = (int)((mx[1] - mn[1]) / cell) + 1;
    g->nz = (int)((mx[2] - mn[2]) / cell) + 1;
    long long* pairs = (long long*)malloc(sizeof(long long) * 2 * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        const float* q = p + 3 * ids[i];
        int ix = (int)((q[0] - g->ox) / cell), iy = (int)((q[1] - g->oy) / cell), iz = (int)((q[2] - g->oz) / cell);
        pairs[2 * i] = cell_key(g, ix, iy, iz);
        pairs[2 * i + 1] = ids[i];
    }
    qsort(pairs, n, 2 * sizeof(long long), cmp_pair);
    g->idx = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    g->key = (long long*)malloc(sizeof(long long) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) { g->key[i] = pairs[2 * i]; g->idx[i] = (int)pairs[2 * i + 1]; }
    free(pairs);
}

static void grid_free(zo_grid* g) { free(g->idx); free(g->key); }

static int lower_bound_ll(const long long* a, int n, long long v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (a[m] < v) lo = m + 1; else hi = m;
    }
    return lo;
}

/* Visit every point in cells with Chebyshev ring distance exactly r from (cx,cy,cz). */
typedef void (*visit_fn)(void* st, int id);
static void grid_ring(const zo_grid* g, int cx, int cy, int cz, int r, visit_fn fn, void* st) {
    for (int iz = cz - r; iz <= cz + r; iz++) {
        if (iz < 0 || iz >= g->nz) continue;
        for (int iy = cy - r; iy <= cy + r; iy++) {
            if (iy < 0 || iy >= g->ny) continue;
            for (int ix = cx - r; ix <= cx + r; ix++) {
                if (ix < 0 || ix >= g->nx) continue;
                int ring = abs(ix - cx);
                if (abs(iy - cy) > ring) ring = abs(iy - cy);
                if (abs(iz - cz) > ring) ring = abs(iz - cz);
                if (ring != r) continue;
                long long key = cell_key(g, ix, iy, iz);
                int s = lower_bound_ll(g->key, g->n, key);
                for (int t = s; t < g->n && g->key[t] == key; t++) fn(st, g->idx[t]);
            }
        }
    }
}

typedef struct {
    const float* p;
    double qx, qy, qz;
    int self, k;
    double* d2; /* k+1 best squared distances, ascending (self included) */
    int cnt;
} knn_state;

static void knn_visit(void* vs, int id) {
    knn_state* s = (knn_state*)vs;
    double dx = s->p[3 * id] - s->qx, dy = s->p[3 * id + 1] - s->qy, dz = s->p[3 * id + 2] - s->qz;
    double d2 = dx * dx + dy * dy + dz * dz;
    int cap = s->k + 1;
    if (s->cnt < cap) {
        int i = s->cnt++;
        while (i > 0 && s->d2[i - 1] > d2) { s->d2[i] = s->d2[i - 1]; i--; }
        s->d2[i] = d2;
    } else if (d2 < s->d2[cap - 1]) {
        int i = cap - 1;
        while (i > 0 && s->d2[i - 1] > d2) { s->d2[i] = s->d2[i - 1]; i--; }
        s->d2[i] = d2;
    }
}

/* PCL StatisticalOutlierRemoval::applyFilterIndices semantics (documented
 * algorithm; PCL is not part of the reference tree): nearestKSearch(k + 1)
 * including the query, mean of sqrt(d^2) over the k others, threshold
 * mean + std_mul * stddev over all valid points, keep d <= threshold. */
int zo_sor(const float* xyz, const uint8_t* mask, int n, int k, double std_mul, uint8_t* mask_out,
           double* meandist, double* threshold, uint8_t* near, double eps) {
    int* ids = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int m = 0;
    for (int i = 0; i < n; i++) if (mask[i]) ids[m++] = i;
    for (int i = 0; i < n; i++) { mask_out[i] = 0; if (meandist) meandist[i] = 0; if (near) near[i] = 0; }
    if (m <= k) { free(ids); if (threshold) *threshold = 0; return -1; }
    /* cell ~ spacing that holds ~k/8 points per cell for a 2-D surface */
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = 0; i < m; i++)
        for (int c = 0; c < 3; c++) {
            double v = xyz[3 * ids[i] + c];
            if (v < mn[c]) mn[c] = v;
            if (v > mx[c]) mx[c] = v;
        }
    double ext = fmax(mx[0] - mn[0], mx[1] - mn[1]);
    double cell = ext * sqrt((double)k / m) * 0.5;
    if (!(cell > 1e-6)) cell = 1e-6;
    zo_grid g;
    grid_build(&g, xyz, ids, m, cell);
    float* md = (float*)malloc(sizeof(float) * (size_t)m);
#pragma omp parallel
    {
        double* buf = (double*)malloc(sizeof(double) * (k + 1));
#pragma omp for schedule(dynamic, 64)
        for (int t = 0; t < m; t++) {
            int id = ids[t];
            knn_state s = {xyz, xyz[3 * id], xyz[3 * id + 1], xyz[3 * id + 2], id, k, buf, 0};
            int cx = (int)((s.qx - g.ox) / cell), cy = (int)((s.qy - g.oy) / cell), cz = (int)((s.qz - g.oz) / cell);
            for (int r = 0;; r++) {
                grid_ring(&g, cx, cy, cz, r, knn_visit, &s);
                if (s.cnt >= k + 1 && sqrt(s.d2[k]) <= r * cell) break;
                if (r > g.nx + g.ny + g.nz) break;
            }
            double sum = 0;
            for (int i = 1; i < k + 1; i++) sum += sqrt(s.d2[i]);
            md[t] = (float)(sum / k);
        }
        free(buf);
    }
    double sum = 0, sq = 0;
    for (int t = 0; t < m; t++) { sum += md[t]; sq += (double)(md[t] * md[t]); }
    double mean = sum / m;
    double var = (sq - sum * sum / m) / (m - 1);
    double thr = mean + std_mul * sqrt(var);
    for (int t = 0; t < m; t++) {
        int id = ids[t];
        if (meandist) meandist[id] = md[t];
        if (near && fabs(md[t] - thr) < eps * thr) near[id] = 1;
        mask_out[id] = (md[t] > thr) ? 0 : 1;
    }
    if (threshold) *threshold = thr;
    grid_free(&g);
    free(md);
    free(ids);
    return 0;
}

typedef struct {
    const float* p;
    double qx, qy, qz, r2, inv2s2, eps;
    double sx, sy, sz, sw;
    int near;
} rad_state;

static void rad_visit(void* vs, int id) {
    rad_state* s = (rad_state*)vs;
    double dx = s->p[3 * id] - s->qx, dy = s->p[3 * id + 1] - s->qy, dz = s->p[3 * id + 2] - s->qz;
    double d2 = dx * dx + dy * dy + dz * dz;
    if (fabs(d2 - s->r2) < 0.1 * s->eps * s->r2) s->near = 1;
    if (d2 > s->r2) return;
    double w = exp(-d2 * s->inv2s2);
    s->sx += w * dx; s->sy += w * dy; s->sz += w * dz; s->sw += w;
}

/* Metric Gaussian point filter (new; no reference counterpart): for each valid
 * point p, out = p + sum_q w (q - p) / sum_q w over valid q with |q - p| <= 3 sigma,
 * w = exp(-|q - p|^2 / 2 sigma^2) (p itself has w = 1). */
void zo_metric_gaussian(const float* xyz, const uint8_t* mask, int n, double sigma, float* out,
                        uint8_t* near, double eps) {
    int* ids = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int m = 0;
    for (int i = 0; i < n; i++) {
        out[3 * i] = xyz[3 * i]; out[3 * i + 1] = xyz[3 * i + 1]; out[3 * i + 2] = xyz[3 * i + 2];
        if (near) near[i] = 0;
        if (mask[i]) ids[m++] = i;
    }
    if (m == 0) { free(ids); return; }
    const double rad = 3.0 * sigma;
    zo_grid g;
    grid_build(&g, xyz, ids, m, rad);
#pragma omp parallel for schedule(dynamic, 64)
    for (int t = 0; t < m; t++) {
        int id = ids[t];
        rad_state s = {xyz, xyz[3 * id], xyz[3 * id + 1], xyz[3 * id + 2], rad * rad, 1.0 / (2 * sigma * sigma), eps,
                       0, 0, 0, 0, 0};
        int cx = (int)((s.qx - g.ox) / rad), cy = (int)((s.qy - g.oy) / rad), cz = (int)((s.qz - g.oz) / rad);
        grid_ring(&g, cx, cy, cz, 0, rad_visit, &s);
        grid_ring(&g, cx, cy, cz, 1, rad_visit, &s);
        out[3 * id] = (float)(s.qx + s.sx / s.sw);
        out[3 * id + 1] = (float)(s.qy + s.sy / s.sw);
        out[3 * id + 2] = (float)(s.qz + s.sz / s.sw);
        if (near) near[id] = (uint8_t)s.near;
    }
    grid_free(&g);
    free(ids);
}
