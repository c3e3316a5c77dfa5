/* zim_synth.h -- seeded synthetic structured-light scene renderer (see zim_synth.c). */
#ifndef ZIM_SYNTH_H
#define ZIM_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int width, height;
    double K[2][9], D[2][5], R[9], t[3]; /* stereo rig, X_r = R X_l + t */
    double proj_K[9];
    int proj_width, proj_height;
    double proj_R[9], proj_t[3];         /* X_p = proj_R X_l + proj_t */
    int scene_kind;                      /* 0 plane+sphere, 1 bumps+boxes, 2 plane */
    double plane_z, max_relief;
    double plane_n[3], plane_d;          /* kinds 0 and 2: n . X = d */
    double sphere[4];                    /* centre, radius (kind 0) */
    int n_bumps;
    double bumps[32][4];                 /* x, y, amplitude, sigma */
    int n_boxes;
    double boxes[4][5];                  /* x0 x1 y0 y1 ztop */
    int encoding, n_freq, gray_bits;
    double freq[4];
    int shift_num[4];
    int bit_depth;
    double A_lo, A_hi, B_lo, B_hi, noise_sigma;
    uint64_t seed;
} zs_scene;

int zs_frame_count(const zs_scene* s);
/* frames: F planes of width*height (u8 if bit_depth == 8 else u16);
 * xyz (optional): ground-truth hit point per pixel in left-camera coordinates. */
int zs_render(const zs_scene* s, int cam, void* frames, float* xyz);

#ifdef __cplusplus
}
#endif
#endif
