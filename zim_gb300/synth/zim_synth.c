/*
 * zim_synth.c -- seeded synthetic structured-light scenes for the benchmark and
 * the tests: ray-casts a pinhole stereo rig (Brown-Conrady k1 k2 p1 p2 k3
 * distortion) against a plane + sphere, a height field of Gaussian bumps with
 * box occluders, or a posed plane; shades each camera pixel with the projector's
 * fringe / Gray-code patterns (projector shadows give zero fringe contrast) and
 * writes u8 or u16 frames in the decoder's frame order.
 *
 * Pattern conventions (x = projector column / projector width):
 *   heterodyne3:   I_n = A + B cos(2 pi f x + 2 pi n / N)
 *   hierarchical and Gray:   I_n = A + B cos(2 pi f x - pi + 2 pi n / N)
 *   Gray frames:   I = A + B (2 s - 1), s the Gray-code bit of floor(f x)
 *   complementary Gray frame: the next, half-period Gray bit.
 * Noise is N(0, sigma^2) per sample; A, B are uniform per pixel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "zim_synth.h"

#define ZS_PI 3.14159265358979323846

static inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline double u01(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
    uint64_t h = splitmix64(seed ^ splitmix64(a * 0x100000001B3ull ^ splitmix64(b * 0xC2B2AE3D27D4EB4Full ^ c)));
    return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static inline double gauss01(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
    double u1 = u01(seed, a, b, 2 * c), u2 = u01(seed, a, b, 2 * c + 1);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * ZS_PI * u2);
}

/* Height of the bump field at (x, y) and its gradient. */
static double hf_eval(const zs_scene* s, double x, double y, double* gx, double* gy) {
    double h = s->plane_z, dx = 0, dy = 0;
    for (int i = 0; i < s->n_bumps; i++) {
        const double* b = s->bumps[i];
        double ex = x - b[0], ey = y - b[1];
        double is2 = 1.0 / (2.0 * b[3] * b[3]);
        double e = b[2] * exp(-(ex * ex + ey * ey) * is2);
        h -= e;
        dx += 2.0 * ex * is2 * e;
        dy += 2.0 * ey * is2 * e;
    }
    if (gx) *gx = dx;
    if (gy) *gy = dy;
    return h;
}

/* First hit of the ray o + t d (t > tmin) with the scene; returns t or -1. */
static double intersect(const zs_scene* s, const double o[3], const double d[3], double tmin) {
    double best = -1;
    if (s->scene_kind == 0 || s->scene_kind == 2) {
        const double* n = s->plane_n;
        double den = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
        if (fabs(den) > 1e-12) {
            double t = (s->plane_d - (n[0] * o[0] + n[1] * o[1] + n[2] * o[2])) / den;
            if (t > tmin) best = t;
        }
    }
    if (s->scene_kind == 0 && s->sphere[3] > 0) {
        double oc[3] = {o[0] - s->sphere[0], o[1] - s->sphere[1], o[2] - s->sphere[2]};
        double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double b = 2 * (oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2]);
        double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - s->sphere[3] * s->sphere[3];
        double disc = b * b - 4 * a * c;
        if (disc >= 0) {
            double sq = sqrt(disc);
            double t0 = (-b - sq) / (2 * a), t1 = (-b + sq) / (2 * a);
            double t = t0 > tmin ? t0 : (t1 > tmin ? t1 : -1);
            if (t > 0 && (best < 0 || t < best)) best = t;
        }
    }
    if (s->scene_kind == 1) {
        /* height field: g(t) = z(t) - h(x(t), y(t)) is monotone for the slopes used */
        double zlo = s->plane_z - s->max_relief - 1.0, zhi = s->plane_z + 1.0;
        if (fabs(d[2]) > 1e-12) {
            double ta = (zlo - o[2]) / d[2], tb = (zhi - o[2]) / d[2];
            if (ta > tb) { double tt = ta; ta = tb; tb = tt; }
            if (ta < tmin) ta = tmin;
            double ga = o[2] + ta * d[2] - hf_eval(s, o[0] + ta * d[0], o[1] + ta * d[1], 0, 0);
            double gb = o[2] + tb * d[2] - hf_eval(s, o[0] + tb * d[0], o[1] + tb * d[1], 0, 0);
            if ((ga <= 0 && gb >= 0) || (ga >= 0 && gb <= 0)) {
                double t = ta - ga * (tb - ta) / (gb - ga);
                for (int it = 0; it < 60; it++) {
                    double gx, gy;
                    double x = o[0] + t * d[0], y = o[1] + t * d[1];
                    double g = o[2] + t * d[2] - hf_eval(s, x, y, &gx, &gy);
                    if ((g <= 0) == (ga <= 0)) { ta = t; ga = g; } else { tb = t; gb = g; }
                    double dg = d[2] - gx * d[0] - gy * d[1];
                    double tn = t - g / dg;
                    if (!(tn > ta && tn < tb)) tn = 0.5 * (ta + tb);
                    if (fabs(tn - t) < 1e-10 * (1 + fabs(t))) { t = tn; break; }
                    t = tn;
                }
                best = t;
            }
        }
        for (int i = 0; i < s->n_boxes; i++) {
            const double* bx = s->boxes[i];
            double lo[3] = {bx[0], bx[2], bx[4]}, hi[3] = {bx[1], bx[3], s->plane_z + 1.0};
            double t0 = -1e300, t1 = 1e300;
            int ok = 1;
            for (int a = 0; a < 3 && ok; a++) {
                if (fabs(d[a]) < 1e-15) {
                    if (o[a] < lo[a] || o[a] > hi[a]) ok = 0;
                } else {
                    double ta = (lo[a] - o[a]) / d[a], tb = (hi[a] - o[a]) / d[a];
                    if (ta > tb) { double tt = ta; ta = tb; tb = tt; }
                    if (ta > t0) t0 = ta;
                    if (tb < t1) t1 = tb;
                }
            }
            if (ok && t0 <= t1 && t0 > tmin && (best < 0 || t0 < best)) best = t0;
        }
    }
    return best;
}

/* Undistort a pixel into a normalised ray (x, y, 1) by fixed-point iteration. */
static void pixel_ray(const double K[9], const double D[5], double u, double v, double* x, double* y) {
    double xd = (u - K[2]) / K[0], yd = (v - K[5]) / K[4];
    double xx = xd, yy = yd;
    for (int it = 0; it < 40; it++) {
        double r2 = xx * xx + yy * yy;
        double kr = 1 + ((D[4] * r2 + D[1]) * r2 + D[0]) * r2;
        double dx = 2 * D[2] * xx * yy + D[3] * (r2 + 2 * xx * xx);
        double dy = D[2] * (r2 + 2 * yy * yy) + 2 * D[3] * xx * yy;
        double nx = (xd - dx) / kr, ny = (yd - dy) / kr;
        if (fabs(nx - xx) < 1e-15 && fabs(ny - yy) < 1e-15) { xx = nx; yy = ny; break; }
        xx = nx; yy = ny;
    }
    *x = xx;
    *y = yy;
}

int zs_frame_count(const zs_scene* s) {
    int f = 0;
    if (s->encoding == 0) { for (int i = 0; i < 3; i++) f += s->shift_num[i]; }
    else if (s->encoding == 1) { for (int i = 0; i < s->n_freq; i++) f += s->shift_num[i]; }
    else f = s->shift_num[0] + s->gray_bits + (s->encoding == 3 ? 1 : 0);
    return f;
}

int zs_render(const zs_scene* s, int cam, void* frames, float* xyz) {
    const int W = s->width, H = s->height;
    const size_t npx = (size_t)W * H;
    const int F = zs_frame_count(s);
    const double maxv = s->bit_depth == 8 ? 255.0 : (double)((1 << s->bit_depth) - 1);
    /* camera centre and rotation in left-camera coordinates: X_r = R X_l + t */
    double C[3] = {0, 0, 0}, Rt[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (cam == 1) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Rt[i * 3 + j] = s->R[j * 3 + i];
        for (int i = 0; i < 3; i++) C[i] = -(Rt[i * 3] * s->t[0] + Rt[i * 3 + 1] * s->t[1] + Rt[i * 3 + 2] * s->t[2]);
    }
    double PC[3];
    for (int i = 0; i < 3; i++)
        PC[i] = -(s->proj_R[i] * s->proj_t[0] + s->proj_R[3 + i] * s->proj_t[1] + s->proj_R[6 + i] * s->proj_t[2]);
#pragma omp parallel for schedule(dynamic, 4)
    for (int v = 0; v < H; v++) {
        for (int u = 0; u < W; u++) {
            size_t pix = (size_t)v * W + u;
            double x, y;
            pixel_ray(s->K[cam], s->D[cam], u, v, &x, &y);
            double dc[3] = {x, y, 1.0}, d[3];
            for (int i = 0; i < 3; i++) d[i] = Rt[i * 3] * dc[0] + Rt[i * 3 + 1] * dc[1] + Rt[i * 3 + 2] * dc[2];
            double t = intersect(s, C, d, 1e-6);
            double X[3] = {C[0] + t * d[0], C[1] + t * d[1], C[2] + t * d[2]};
            int lit = t > 0;
            double xp = 0;
            if (lit) {
                double Xp[3];
                for (int i = 0; i < 3; i++)
                    Xp[i] = s->proj_R[i * 3] * X[0] + s->proj_R[i * 3 + 1] * X[1] + s->proj_R[i * 3 + 2] * X[2] + s->proj_t[i];
                if (Xp[2] <= 0) lit = 0;
                else {
                    xp = s->proj_K[0] * Xp[0] / Xp[2] + s->proj_K[2];
                    double yp = s->proj_K[4] * Xp[1] / Xp[2] + s->proj_K[5];
                    if (xp < 0 || xp >= s->proj_width || yp < 0 || yp >= s->proj_height) lit = 0;
                }
                if (lit) { /* shadow ray from the projector */
                    double e[3] = {X[0] - PC[0], X[1] - PC[1], X[2] - PC[2]};
                    double th = intersect(s, PC, e, 1e-9);
                    if (th > 0 && th < 1.0 - 1e-7) lit = 0;
                }
            }
            if (xyz) {
                if (t > 0) { xyz[3 * pix] = (float)X[0]; xyz[3 * pix + 1] = (float)X[1]; xyz[3 * pix + 2] = (float)X[2]; }
                else { xyz[3 * pix] = xyz[3 * pix + 1] = xyz[3 * pix + 2] = NAN; }
            }
            double A = s->A_lo + (s->A_hi - s->A_lo) * u01(s->seed, 1 + cam, pix, 0);
            double B = lit ? s->B_lo + (s->B_hi - s->B_lo) * u01(s->seed, 1 + cam, pix, 1) : 0.0;
            double xn = xp / s->proj_width;
            int f = 0;
            int nps = s->encoding == 0 ? 3 : (s->encoding == 1 ? s->n_freq : 1);
            for (int i = 0; i < nps; i++) {
                double th0 = 2 * ZS_PI * s->freq[i] * xn - (s->encoding == 0 ? 0.0 : ZS_PI);
                for (int n = 0; n < s->shift_num[i]; n++, f++) {
                    double I = A + B * cos(th0 + 2 * ZS_PI * n / s->shift_num[i]) +
                               s->noise_sigma * gauss01(s->seed, 16 + cam, f, pix);
                    I = floor(I + 0.5);
                    I = I < 0 ? 0 : (I > maxv ? maxv : I);
                    if (s->bit_depth == 8) ((uint8_t*)frames)[npx * f + pix] = (uint8_t)I;
                    else ((uint16_t*)frames)[npx * f + pix] = (uint16_t)I;
                }
            }
            if (s->encoding >= 2) {
                int nb = s->gray_bits;
                int period = (int)floor(s->freq[0] * xn);
                int half = (int)floor(2.0 * s->freq[0] * xn);
                int g1 = period ^ (period >> 1), g2 = half ^ (half >> 1);
                int nbits = nb + (s->encoding == 3 ? 1 : 0);
                for (int b = 0; b < nbits; b++, f++) {
                    int bit = b < nb ? (g1 >> (nb - 1 - b)) & 1 : g2 & 1;
                    double I = A + B * (2.0 * bit - 1.0) + s->noise_sigma * gauss01(s->seed, 16 + cam, f, pix);
                    I = floor(I + 0.5);
                    I = I < 0 ? 0 : (I > maxv ? maxv : I);
                    if (s->bit_depth == 8) ((uint8_t*)frames)[npx * f + pix] = (uint8_t)I;
                    else ((uint16_t*)frames)[npx * f + pix] = (uint16_t)I;
                }
            }
            (void)F;
        }
    }
    return 0;
}
