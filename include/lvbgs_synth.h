/* lvbgs_synth.h -- seeded synthetic video streams for tests and benchmarks.
 *
 * No counterpart in the reference, which evaluates on CDnet (apps/changedet/src/main.cpp:42);
 * CDnet is not available here, so seeded synthetic scenes with the benchmark's shapes, sizes and
 * value distributions stand in for it. Generation is integer-only, so the host renderer (used to
 * feed the CPU oracle) and the device renderer (used to keep benchmark inputs resident in HBM)
 * produce byte-identical frames.
 *
 * Scene: a uniform-random texture smoothed by a Gaussian of sigma 4 (integer separable kernel,
 * replicate border) and contrast-stretched x6 around 128; optional ripple region
 * 20*sin(2*pi*(x/37 + t/11)) and global illumination drift 15*sin(2*pi*t/250); solid rectangles /
 * ellipses of uniform-random colour moving linearly (reflecting at the borders), some of which
 * stop for 100 frames; i.i.d. zero-mean noise per channel (Irwin-Hall sum of 4 uniform bytes,
 * scaled to the requested sigma), clipped to [0,255]. Ground truth is the union of the shapes.
 */
#ifndef LVBGS_SYNTH_H
#define LVBGS_SYNTH_H
#include <stddef.h>
#include <stdint.h>

#include "lvbgs.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LVSYNTH_MAX_SHAPES 16

typedef struct {
    int width, height, channels;
    uint64_t seed;
    int noise_sigma_milli;       /* noise standard deviation x 1000 */
    int n_shapes;                /* <= LVSYNTH_MAX_SHAPES */
    int shape_min, shape_max;    /* shape size range in pixels */
    int speed_min_q8, speed_max_q8; /* per-axis speed range, 1/256 pixel per frame */
    int ellipses_only;           /* 1: all shapes are ellipses */
    int ripple;                  /* 1: a 400x300 ripple region */
    int drift;                   /* 1: +-15 global illumination drift over 250 frames */
    int n_stopping;              /* the first n shapes stop for 100 frames */
    int n_frames;                /* nominal sequence length */
    int thermal;                 /* 1: thermal-like scene (see below); shape sizes are blob radii and speeds
                                    are the random-walk step range in whole pixels */
} lvsynth_config;

/* Thermal-like scene (config 2): a smooth diagonal gradient 80..140 plus low-frequency value noise
 * of amplitude 10 (random values on a 64-pixel grid, bilinear), warm blobs of intensity 180..240
 * with a Gaussian falloff (sigma = radius/2, cut at two radii), each on a random walk of 1..5 pixels
 * per frame in one of eight directions (reflected at the borders); ground truth = within one radius. */

typedef struct lvsynth_scene* lvsynth_handle;

/* Benchmark presets: config 0 (320x240 BGR, 200 frames), 1 (1920x1080 BGR, 500 frames, ripple,
 * drift, 8 ellipses, two stopping), 3 (stream `index` of the 64-stream mix: 16x320x240,
 * 24x640x480, 16x1280x720, 8x1920x1080; every fourth stream single-channel; noise sigma U[2,6];
 * 2-10 shapes; 300 frames), 2 (640x480 single-channel thermal-like scene, six blobs of radius 10-40,
 * noise sigma 2, 300 frames), 4 (a serving stream: index = 2 * resolution class {320x240, 640x480,
 * 1280x720, 1920x1080} + 1 for single-channel, content as in the 64-stream mix). base_seed
 * selects the sequence. */
lvbgs_status lvsynth_preset(int config, int index, uint64_t base_seed, lvsynth_config* out);
lvbgs_status lvsynth_create(const lvsynth_config* cfg, lvsynth_handle* out);
void lvsynth_destroy(lvsynth_handle h);
/* renders frame t into host buffers (frame: w*h*c bytes, gt: w*h bytes, either may be NULL) */
lvbgs_status lvsynth_render(lvsynth_handle h, int t, uint8_t* frame, uint8_t* gt);
/* renders frame t into device buffers on cuda_stream (device copy of the texture made on first use) */
lvbgs_status lvsynth_render_device(lvsynth_handle h, int t, uint8_t* frame, uint8_t* gt, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
