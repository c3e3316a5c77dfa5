/* zim_oracle_diff.c -- FP64 restatement of the differentiable sub-pixel
 * matching + reprojection and its analytic gradient.  TEST INFRASTRUCTURE:
 * only tests/, the smoke check and the bench's CPU baseline use it.
 *
 * The forward restates the reference's sub-pixel refinement and rectified
 * reprojection (PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp
 * :985-1000 and :414-461) on rectified phase that is sampled, with exact
 * bilinear weights, from the source phase through initUndistortRectifyMap's
 * ray model (:329-337, distortion k1 k2 p1 p2 k3).  Parameter layout and
 * sample rules are those of include/zim.h (zim_diff_params, zim_diff_view).
 * Parity is unpinned: the reference has no gradients; the tests pin this
 * restatement against central finite differences of its own FP64 loss. */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "zim_oracle.h"

#define TWO_PI 6.283185307179586476925286766559

static void rodrigues(const double v[3], double R[9]) {
    double th = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double k[3] = {0, 0, 0}, c = 1.0, s = 0.0, cc = 0.0;
    if (th > 0) {
        for (int a = 0; a < 3; a++) k[a] = v[a] / th;
        c = cos(th);
        s = sin(th);
        cc = 1.0 - c;
    }
    R[0] = c + cc * k[0] * k[0];        R[1] = cc * k[0] * k[1] - s * k[2]; R[2] = cc * k[0] * k[2] + s * k[1];
    R[3] = cc * k[1] * k[0] + s * k[2]; R[4] = c + cc * k[1] * k[1];        R[5] = cc * k[1] * k[2] - s * k[0];
    R[6] = cc * k[2] * k[0] - s * k[1]; R[7] = cc * k[2] * k[1] + s * k[0]; R[8] = c + cc * k[2] * k[2];
}

typedef struct {
    double ir[9];
    double fx, fy, cx, cy, k1, k2, p1, p2, k3;
} cam_t;

typedef struct {
    int ok, x0, y0;
    double phase, a, b, gu, gv;
    double ju[9], jv[9];
} samp_t;

/* When set, each sample position (u, v) is rounded to FP32 before the
 * bilinear lookup, everything else staying FP64: the gradient's change under
 * this one rounding is the floor that FP32 sample positions put under an FP32
 * implementation (zo_diff_round_positions). */
static int g_round_positions = 0;
void zo_diff_round_positions(int on) { g_round_positions = on; }

static int sample(const cam_t* c, double col, double row, const int32_t* ord, const double* res, int sw, int sh,
                  samp_t* s, int32_t* cell, int cells_mode) {
    double X0 = c->ir[0] * col + c->ir[1] * row + c->ir[2];
    double X1 = c->ir[3] * col + c->ir[4] * row + c->ir[5];
    double X2 = c->ir[6] * col + c->ir[7] * row + c->ir[8];
    double x = X0 / X2, y = X1 / X2;
    double r2 = x * x + y * y;
    double sd = 1.0 + r2 * (c->k1 + r2 * (c->k2 + r2 * c->k3));
    double xd = x * sd + 2.0 * c->p1 * x * y + c->p2 * (r2 + 2.0 * x * x);
    double yd = y * sd + c->p1 * (r2 + 2.0 * y * y) + 2.0 * c->p2 * x * y;
    double u = c->fx * xd + c->cx, v = c->fy * yd + c->cy;
    if (g_round_positions) {
        u = (double)(float)u;
        v = (double)(float)v;
    }
    s->ok = 0;
    int x0, y0;
    if (cells_mode == 2) {
        /* the bilinear cell is a frozen decision: the patch extends past [0, 1) */
        x0 = cell[0];
        y0 = cell[1];
        if (x0 < 0) return 0;
    } else {
        if (!(u >= 0.0 && v >= 0.0 && u < sw - 1 && v < sh - 1)) return 0;
        x0 = (int)u;
        y0 = (int)v;
        if (cells_mode == 1) { cell[0] = x0; cell[1] = y0; }
    }
    size_t o = (size_t)y0 * sw + x0;
    int32_t k00 = ord[o], k10 = ord[o + 1], k01 = ord[o + sw], k11 = ord[o + sw + 1];
    if (k00 < 1 || k10 < 1 || k01 < 1 || k11 < 1) return 0;
    double f00 = TWO_PI * k00 + res[o], f10 = TWO_PI * k10 + res[o + 1];
    double f01 = TWO_PI * k01 + res[o + sw], f11 = TWO_PI * k11 + res[o + sw + 1];
    double a = u - x0, b = v - y0;
    s->phase = (1 - a) * (1 - b) * f00 + a * (1 - b) * f10 + (1 - a) * b * f01 + a * b * f11;
    s->gu = (1 - b) * (f10 - f00) + b * (f11 - f01);
    s->gv = (1 - a) * (f01 - f00) + a * (f11 - f10);
    s->x0 = x0;
    s->y0 = y0;
    s->a = a;
    s->b = b;
    double r4 = r2 * r2;
    double ju[9] = {xd, 0, 1, 0, c->fx * x * r2, c->fx * x * r4, 0, 0, 0};
    double jv[9] = {0, yd, 0, 1, c->fy * y * r2, c->fy * y * r4, 0, 0, 0};
    /* right-multiplied rotation update: ray X -> X + X x eps */
    double dx[3] = {x * y, -1.0 - x * x, y}, dy[3] = {1.0 + y * y, -x * y, -x};
    double s1 = c->k1 + r2 * (2.0 * c->k2 + 3.0 * c->k3 * r2);
    double dxd_dx = sd + 2.0 * x * x * s1 + 2.0 * c->p1 * y + 6.0 * c->p2 * x;
    double dxd_dy = 2.0 * x * y * s1 + 2.0 * c->p1 * x + 2.0 * c->p2 * y;
    double dyd_dx = dxd_dy;
    double dyd_dy = sd + 2.0 * y * y * s1 + 6.0 * c->p1 * y + 2.0 * c->p2 * x;
    for (int k = 0; k < 3; k++) {
        ju[6 + k] = c->fx * (dxd_dx * dx[k] + dxd_dy * dy[k]);
        jv[6 + k] = c->fy * (dyd_dx * dx[k] + dyd_dy * dy[k]);
    }
    memcpy(s->ju, ju, sizeof ju);
    memcpy(s->jv, jv, sizeof jv);
    s->ok = 1;
    return 1;
}

static void scatter(double* g, int sw, const samp_t* s, double v) {
    if (!g) return;
    size_t o = (size_t)s->y0 * sw + s->x0;
    g[o] += v * (1 - s->a) * (1 - s->b);
    g[o + 1] += v * s->a * (1 - s->b);
    g[o + sw] += v * (1 - s->a) * s->b;
    g[o + sw + 1] += v * s->a * s->b;
}

void zo_diff_eval(const zo_diff_geom* G, const double theta[16], const int32_t* order_l, const double* res_l,
                  const int32_t* order_r, const double* res_r, const int32_t* best, const double plane[4],
                  double zmin, double zmax, double loss_weight, double* loss, double* npts, double grad[16],
                  double jtj[256], double* xyz, uint8_t* mask, double* gphase_l, double* gphase_r, int32_t* cells,
                  int cells_mode, double gabs[16]) {
    cam_t cam[2];
    for (int c = 0; c < 2; c++) {
        if (c == 0) {
            memcpy(cam[0].ir, G->ir[0], sizeof cam[0].ir);
        } else {
            double E[9];
            rodrigues(theta + 13, E);
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++) {
                    double s = 0;
                    for (int m = 0; m < 3; m++) s += E[m * 3 + r] * G->ir[1][m * 3 + q];
                    cam[1].ir[r * 3 + q] = s;
                }
        }
        cam[c].fx = theta[6 * c + 0];
        cam[c].fy = theta[6 * c + 1];
        cam[c].cx = theta[6 * c + 2];
        cam[c].cy = theta[6 * c + 3];
        cam[c].k1 = theta[6 * c + 4];
        cam[c].k2 = theta[6 * c + 5];
        cam[c].p1 = G->dist[c][0];
        cam[c].p2 = G->dist[c][1];
        cam[c].k3 = G->dist[c][2];
    }
    const double* Q = G->Q;
    double Tx0 = -1.0 / Q[14], dcx = Q[15] * Tx0;
    double Tx = Tx0 * theta[12] / G->baseline0, dTx = Tx0 / G->baseline0;
    double q32 = -1.0 / Tx, q33 = dcx / Tx, dq32 = dTx / (Tx * Tx), dq33 = -dcx * dTx / (Tx * Tx);
    double L = 0, cnt = 0, g[16] = {0}, H[256] = {0}, ga[16] = {0};
    const int rw = G->rect_w, rh = G->rect_h, sw = G->src_w, sh = G->src_h;
    for (int i = 0; i < rh; i++)
        for (int j = 0; j < rw; j++) {
            size_t pix = (size_t)i * rw + j;
            if (xyz) xyz[3 * pix] = xyz[3 * pix + 1] = xyz[3 * pix + 2] = 0;
            if (mask) mask[pix] = 0;
            int32_t* pc = cells ? cells + pix * 8 : NULL;
            int cm = cells ? cells_mode : 0;
            if (cm == 1)
                for (int a = 0; a < 8; a++) pc[a] = -1;
            int b = best[pix];
            if (b < 1 || b + 1 >= rw) continue;
            samp_t sL, sR[3];
            if (!sample(&cam[0], j, i, order_l, res_l, sw, sh, &sL, pc, cm)) continue;
            int ok = 1;
            for (int m = 0; m < 3 && ok; m++)
                ok = sample(&cam[1], b - 1 + m, i, order_r, res_r, sw, sh, &sR[m], pc ? pc + 2 * (m + 1) : NULL, cm);
            if (!ok) continue;
            double c[3], dd[3] = {0, 0, 0}, delta = 0;
            for (int m = 0; m < 3; m++) c[m] = sR[m].phase - sL.phase;
            double num = c[1] * (c[0] - c[2]), den = 2.0 * (c[0] - c[1]) * (c[1] - c[2]);
            if (fabs(den) > 1e-9) {
                delta = num / den;
                dd[0] = (c[1] - delta * 2.0 * (c[1] - c[2])) / den;
                dd[1] = ((c[0] - c[2]) - delta * 2.0 * (c[0] - 2.0 * c[1] + c[2])) / den;
                dd[2] = (-c[1] + delta * 2.0 * (c[0] - c[1])) / den;
            }
            double d = (j - b) - delta;
            if (fabs(d) < 1e-5) continue;
            double w = q32 * d + q33;
            double X = (j + Q[3]) / w, Y = (i + Q[7]) / w, Z = Q[11] / w;
            if (!(Z > zmin && Z < zmax)) continue;
            if (xyz) { xyz[3 * pix] = X; xyz[3 * pix + 1] = Y; xyz[3 * pix + 2] = Z; }
            if (mask) mask[pix] = 1;
            double r = plane[0] * X + plane[1] * Y + plane[2] * Z + plane[3];
            L += r * r;
            cnt += 1;
            if (!grad && !jtj && !gphase_l && !gphase_r) continue;
            /* P depends on the parameters through w only: dP/dw = -P/w.  With the
             * upstream g = lw 2 r n: dLoss/dw = -lw 2 r (n . P)/w; dr/dw = -(n . P)/w */
            double nP = plane[0] * X + plane[1] * Y + plane[2] * Z;
            double s_up = -loss_weight * 2.0 * r * nP / w;
            double s_r = -nP / w;
            double wR[3] = {-q32 * dd[0], -q32 * dd[1], -q32 * dd[2]};
            double wL = -(wR[0] + wR[1] + wR[2]);
            double Jw[16] = {0};
            Jw[12] = d * dq32 + dq33;
            for (int k = 0; k < 6; k++) Jw[k] = wL * (sL.gu * sL.ju[k] + sL.gv * sL.jv[k]);
            for (int m = 0; m < 3; m++) {
                for (int k = 0; k < 6; k++) Jw[6 + k] += wR[m] * (sR[m].gu * sR[m].ju[k] + sR[m].gv * sR[m].jv[k]);
                for (int k = 0; k < 3; k++)
                    Jw[13 + k] += wR[m] * (sR[m].gu * sR[m].ju[6 + k] + sR[m].gv * sR[m].jv[6 + k]);
            }
            for (int k = 0; k < 16; k++) {
                g[k] += s_up * Jw[k];
                ga[k] += fabs(s_up * Jw[k]);
            }
            for (int a = 0; a < 16; a++)
                for (int q = 0; q < 16; q++) H[a * 16 + q] += (s_r * Jw[a]) * (s_r * Jw[q]);
            scatter(gphase_l, sw, &sL, s_up * wL);
            for (int m = 0; m < 3; m++) scatter(gphase_r, sw, &sR[m], s_up * wR[m]);
        }
    *loss = L;
    *npts = cnt;
    if (grad) memcpy(grad, g, sizeof g);
    if (jtj) memcpy(jtj, H, sizeof H);
    if (gabs) memcpy(gabs, ga, sizeof ga);
}
