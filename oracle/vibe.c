/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's ViBe (modules/video/src/BackgroundSubtractorViBe.cpp:22-191,
 * BackgroundSubtractorViBe.hpp:39-52 for the defaults and switches): BackgroundSubtractorViBe_1ch for
 * single-channel frames and BackgroundSubtractorViBe_3ch for three-channel frames, with the header's
 * configuration (no single-channel threshold validation, the L2 distance).
 *
 * The three-channel distance is lv::L2dist<3>(const uchar*, const uchar*) (utils/math.hpp:391-396):
 * the squared channel differences are accumulated in decltype(L2sqrdist(uchar, uchar)), uint16_t, so
 * the sum wraps modulo 65536 before the square root; the result goes through float and is compared
 * with the size_t threshold 3R converted to float.
 *
 * rand() is draw k of pixel p in frame t of the counter-based generator (philox.h). ViBe keeps no
 * frame counter, so t counts apply() calls (initialize() is frame 0); the k-th draw a pixel's loop
 * iteration makes in a frame is its draw k (initialize(): the draw of sample s is k = s).
 * Pinned to the reference by tests/test_oracle_reference.py (oracle/_ref, rvibe_*).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"
#include "philox.h"

struct ovibe {
    ovibe_params p;
    int initialized;
    int W, H, C;
    size_t npx;
    uint8_t* samples; /* [N][npx*C] */
    uint32_t* kctr;
    uint64_t frames;
    uint64_t st_samples, st_writes;
};

static int vdraw(ovibe_t* o, size_t px) {
    const uint32_t k = o->kctr[px]++;
    const uint32_t ctr[4] = {k >> 2, (uint32_t)px, (uint32_t)o->frames, 0u};
    const uint32_t key[2] = {(uint32_t)o->p.seed, (uint32_t)(o->p.seed >> 32)};
    uint32_t out[4];
    ophilox4x32_10(ctr, key, out);
    return (int)(out[k & 3u] & 0x7fffffffu);
}

void ovibe_default_params(ovibe_params* p) {
    /* BackgroundSubtractorViBe.hpp:39-46 */
    p->color_dist_threshold = 20;
    p->bg_samples = 20;
    p->required_bg_samples = 2;
    p->seed = 0;
}

ovibe_t* ovibe_create(const ovibe_params* p) {
    /* BackgroundSubtractorViBe.cpp:22-29 */
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return NULL;
    ovibe_t* o = (ovibe_t*)calloc(1, sizeof(ovibe_t));
    o->p = *p;
    return o;
}

static void vibe_free(ovibe_t* o) {
    free(o->samples);
    free(o->kctr);
    ovibe_params p = o->p;
    memset(o, 0, sizeof(*o));
    o->p = p;
}

void ovibe_destroy(ovibe_t* o) {
    if (!o) return;
    vibe_free(o);
    free(o);
}

/* BackgroundSubtractorViBe_1ch::initialize (:57-75) and _3ch::initialize (:112-134): every sample of
 * every pixel from a 7x7 Gaussian position of the frame (no border) */
int ovibe_initialize(ovibe_t* o, const uint8_t* img, int W, int H, int C) {
    if (!img || W <= 0 || H <= 0) return OSUB_EBADARG;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED;
    vibe_free(o);
    o->W = W;
    o->H = H;
    o->C = C;
    o->npx = (size_t)W * H;
    const size_t N = o->p.bg_samples, npx = o->npx;
    o->samples = (uint8_t*)calloc(N * npx * C, 1);
    o->kctr = (uint32_t*)calloc(npx, sizeof(uint32_t));
    o->frames = 0;
    for (size_t s = 0; s < N; ++s)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t px = (size_t)y * W + x;
                int sx, sy;
                sample_pos_7x7(vdraw(o, px), &sx, &sy, x, y, 0, W, H);
                for (int c = 0; c < C; ++c)
                    o->samples[s * npx * C + px * C + c] = img[((size_t)sy * W + sx) * C + c];
            }
    o->initialized = 1;
    return OSUB_OK;
}

/* (float) lv::L2dist<3>(uchar*, uchar*) < (float)(3R), with the uint16_t accumulator */
static int vibe_l2_match(const uint8_t* a, const uint8_t* b, size_t R) {
    uint16_t acc = 0;
    for (int c = 0; c < 3; ++c) {
        const int16_t d = (int16_t)((int)a[c] - (int)b[c]);
        acc = (uint16_t)(acc + (uint16_t)((int)d * (int)d));
    }
    return (float)sqrt((double)acc) < (float)(R * 3);
}

/* BackgroundSubtractorViBe_1ch::apply (:77-103) and _3ch::apply (:136-191) */
int ovibe_apply(ovibe_t* o, const uint8_t* img, uint8_t* mask, double lr) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!img || !mask || !(lr > 0)) return OSUB_EBADARG;
    const int W = o->W, H = o->H, C = o->C;
    const size_t N = o->p.bg_samples, npx = o->npx, nreq = o->p.required_bg_samples, R = o->p.color_dist_threshold;
    /* (size_t)ceil(lr); +inf (undefined behaviour in the conversion) is taken as SIZE_MAX, as LOBSTER does */
    const size_t nLR = isinf(lr) ? (size_t)-1 : (size_t)ceil(lr);
    ++o->frames;
    memset(o->kctr, 0, npx * sizeof(uint32_t));
    memset(mask, 0, npx);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t px = (size_t)y * W + x;
            const uint8_t* in = img + px * C;
            size_t nGood = 0, s = 0;
            while (nGood < nreq && s < N) {
                const uint8_t* bg = o->samples + s * npx * C + px * C;
                ++o->st_samples;
                if (C == 1 ? absdiff(in[0], bg[0]) < R : vibe_l2_match(in, bg, R)) ++nGood;
                ++s;
            }
            if (nGood < nreq) {
                mask[px] = 255;
                continue;
            }
            if (((size_t)vdraw(o, px) % nLR) == 0) {
                const size_t rs = (size_t)vdraw(o, px) % N;
                memcpy(o->samples + rs * npx * C + px * C, in, (size_t)C);
                ++o->st_writes;
            }
            if (((size_t)vdraw(o, px) % nLR) == 0) {
                int nx, ny;
                neighbor_pos(vdraw(o, px), 1, &nx, &ny, x, y, 0, W, H);
                const size_t rs = (size_t)vdraw(o, px) % N;
                memcpy(o->samples + rs * npx * C + ((size_t)ny * W + nx) * C, in, (size_t)C);
                ++o->st_writes;
            }
        }
    return OSUB_OK;
}

/* BackgroundSubtractorViBe::getBackgroundImage (:33-48) */
int ovibe_get_background(const ovibe_t* o, uint8_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t N = o->p.bg_samples, n = o->npx * (size_t)o->C;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->samples[s * n + i]) / (float)N;
        out[i] = sat_u8f(acc);
    }
    return OSUB_OK;
}

const void* ovibe_samples(const ovibe_t* o, size_t* nbytes) {
    if (nbytes) *nbytes = o->initialized ? o->p.bg_samples * o->npx * (size_t)o->C : 0;
    return o->initialized ? o->samples : NULL;
}

void ovibe_get_stats(const ovibe_t* o, uint64_t out[3]) {
    out[0] = o->frames;
    out[1] = o->st_samples;
    out[2] = o->st_writes;
}
