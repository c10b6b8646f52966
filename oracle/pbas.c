/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's PBAS (modules/video/src/BackgroundSubtractorPBAS.cpp:22-496,
 * BackgroundSubtractorPBAS.hpp:41-93 for the defaults and switches): BackgroundSubtractorPBAS_1ch for
 * single-channel frames and BackgroundSubtractorPBAS_3ch for three-channel frames, with the header's
 * configuration (self diffusion on, no R2 acceleration, no advanced morphology).
 *
 * The gradient image of a frame (:127-135 / :338-346) is GaussianBlur 3x3 (sigma 0), the two Scharr
 * derivatives in int16, convertScaleAbs and addWeighted(0.5, 0.5), all with BORDER_REFLECT_101; the
 * definitions used here (and by the GPU and the OpenCV stand-in of oracle/refshim) are: blur = (sum of
 * [1 2 1; 2 4 2; 1 2 1] * p + 8) >> 4; Scharr x = [-3 0 3; -10 0 10; -3 0 3] (y: its transpose);
 * |v| saturated to 255; (a + b) * 0.5 rounded half to even. Their parity with a real OpenCV build is
 * unpinned (OpenCV is not installed).
 *
 * The three-channel colour and gradient distances are lv::L2dist of two Vec3b (utils/math.hpp:391-396,
 * 458-466): the squared differences add up in uint16_t (wrapping modulo 65536), then the square root in
 * double, converted to float. The frame-level mean gradient distance of the three-channel path is a float
 * sum in raster order (:366-394), which is kept: the next frame's distances depend on it.
 *
 * rand() is draw k of pixel p in frame t; PBAS keeps no frame counter, so t counts apply() calls
 * (initialize() is frame 0, where sample s of pixel p is its draw s). Pinned to the reference by
 * tests/test_oracle_reference.py (oracle/_ref, rpbas_*).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"
#include "philox.h"

#define PBAS_R_SCALE 5.0000f
#define PBAS_R_INCR 1.0500f
#define PBAS_R_DECR 0.9500f
#define PBAS_R_LOWER 0.6000f
#define PBAS_R_UPPER 99.0000f
#define PBAS_R_OFFST 0.0000f
#define PBAS_T_OFFST 1.0000f
#define PBAS_T_SCALE 255.00f
#define PBAS_T_DECR 0.0500f
#define PBAS_T_INCR 1.0000f
#define PBAS_T_LOWER 2.0000f
#define PBAS_T_UPPER 200.00f
#define PBAS_GRAD_WEIGHT_ALPHA 10.0f

struct opbas {
    opbas_params p;
    int initialized;
    int W, H, C;
    size_t npx;
    uint8_t *scol, *sgrad; /* [N][npx*C] */
    float *R, *T, *D;      /* distance threshold factor, update rate, mean minimal distance */
    uint8_t *grad, *rawFG;
    uint16_t* colcnt;
    float meanGrad; /* m_fFormerMeanGradDist */
    uint32_t* kctr;
    uint64_t frames;
};

static int pdraw(opbas_t* o, size_t px) {
    const uint32_t k = o->kctr[px]++;
    const uint32_t ctr[4] = {k >> 2, (uint32_t)px, (uint32_t)o->frames, 0u};
    const uint32_t key[2] = {(uint32_t)o->p.seed, (uint32_t)(o->p.seed >> 32)};
    uint32_t out[4];
    ophilox4x32_10(ctr, key, out);
    return (int)(out[k & 3u] & 0x7fffffffu);
}

void opbas_default_params(opbas_params* p) {
    /* BackgroundSubtractorPBAS.hpp:48-55 */
    p->color_dist_threshold = 30;
    p->update_rate = 16.0f;
    p->bg_samples = 35;
    p->required_bg_samples = 2;
    p->seed = 0;
}

opbas_t* opbas_create(const opbas_params* p) {
    /* BackgroundSubtractorPBAS.cpp:21-32 */
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return NULL;
    if (!(p->update_rate > 0 && p->update_rate <= 255)) return NULL;
    opbas_t* o = (opbas_t*)calloc(1, sizeof(opbas_t));
    o->p = *p;
    o->meanGrad = 20.0f; /* m_fFormerMeanGradDist(20) (:29); initialize() keeps it */
    return o;
}

static void pbas_free(opbas_t* o) {
    void* ptrs[] = {o->scol, o->sgrad, o->R, o->T, o->D, o->grad, o->rawFG, o->colcnt, o->kctr};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    opbas_params p = o->p;
    const float mean = o->meanGrad;
    memset(o, 0, sizeof(*o));
    o->p = p;
    o->meanGrad = mean;
}

void opbas_destroy(opbas_t* o) {
    if (!o) return;
    pbas_free(o);
    free(o);
}

static int reflect101(int i, int n) {
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
    return i;
}

/* the gradient image of a frame (:127-135 / :338-346), per channel */
void opbas_gradient(const uint8_t* img, int W, int H, int C, uint8_t* out) {
    uint8_t* blur = (uint8_t*)malloc((size_t)W * H * C);
    static const int wb[3] = {1, 2, 1};
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                int acc = 0;
                for (int j = -1; j <= 1; ++j)
                    for (int i = -1; i <= 1; ++i)
                        acc += wb[j + 1] * wb[i + 1] *
                               img[((size_t)reflect101(y + j, H) * W + reflect101(x + i, W)) * C + c];
                blur[((size_t)y * W + x) * C + c] = (uint8_t)((acc + 8) >> 4);
            }
    static const int ws[3] = {3, 10, 3};
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                int gx = 0, gy = 0;
                for (int k = -1; k <= 1; ++k) {
                    const int yy = reflect101(y + k, H), xx = reflect101(x + k, W);
                    gx += ws[k + 1] * ((int)blur[((size_t)yy * W + reflect101(x + 1, W)) * C + c] -
                                       (int)blur[((size_t)yy * W + reflect101(x - 1, W)) * C + c]);
                    gy += ws[k + 1] * ((int)blur[((size_t)reflect101(y + 1, H) * W + xx) * C + c] -
                                       (int)blur[((size_t)reflect101(y - 1, H) * W + xx) * C + c]);
                }
                const int ax = gx < 0 ? (-gx > 255 ? 255 : -gx) : (gx > 255 ? 255 : gx);
                const int ay = gy < 0 ? (-gy > 255 ? 255 : -gy) : (gy > 255 ? 255 : gy);
                /* (ax + ay) * 0.5 rounded half to even */
                const int sum = ax + ay;
                out[((size_t)y * W + x) * C + c] = (uint8_t)((sum >> 1) + ((sum & 1) & ((sum >> 1) & 1)));
            }
    free(blur);
}

/* (float) lv::L2dist of two Vec3b: uint16_t accumulation, double square root */
static float pbas_l2(const uint8_t* a, const uint8_t* b) {
    uint16_t acc = 0;
    for (int c = 0; c < 3; ++c) {
        const int16_t d = (int16_t)((int)a[c] - (int)b[c]);
        acc = (uint16_t)(acc + (uint16_t)((int)d * (int)d));
    }
    return (float)sqrt((double)acc);
}

/* initialize (:61-109 / :287-324): maps at their starting values, every sample of every pixel (colour
 * and gradient) from a 7x7 Gaussian position of the frame; the frame-level mean gradient distance is
 * the constructor's (20) or the last frame's */
int opbas_initialize(opbas_t* o, const uint8_t* img, int W, int H, int C) {
    if (!img || W <= 0 || H <= 0) return OSUB_EBADARG;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED;
    pbas_free(o);
    o->W = W;
    o->H = H;
    o->C = C;
    o->npx = (size_t)W * H;
    const size_t N = o->p.bg_samples, npx = o->npx;
    o->scol = (uint8_t*)calloc(N * npx * C, 1);
    o->sgrad = (uint8_t*)calloc(N * npx * C, 1);
    o->R = (float*)malloc(npx * sizeof(float));
    o->T = (float*)malloc(npx * sizeof(float));
    o->D = (float*)calloc(npx, sizeof(float));
    o->grad = (uint8_t*)malloc(npx * C);
    o->rawFG = (uint8_t*)calloc(npx, 1);
    o->colcnt = (uint16_t*)calloc(npx, sizeof(uint16_t));
    o->kctr = (uint32_t*)calloc(npx, sizeof(uint32_t));
    for (size_t i = 0; i < npx; ++i) {
        o->R[i] = 1.0f;
        o->T[i] = o->p.update_rate;
    }
    o->frames = 0;
    opbas_gradient(img, W, H, C, o->grad);
    for (size_t s = 0; s < N; ++s)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t px = (size_t)y * W + x;
                int sx, sy;
                sample_pos_7x7(pdraw(o, px), &sx, &sy, x, y, 0, W, H);
                const size_t sp = (size_t)sy * W + sx;
                for (int c = 0; c < C; ++c) {
                    o->scol[s * npx * C + px * C + c] = img[sp * C + c];
                    o->sgrad[s * npx * C + px * C + c] = o->grad[sp * C + c];
                }
            }
    o->initialized = 1;
    return OSUB_OK;
}

/* apply (:111-281 / :326-496) */
int opbas_apply(opbas_t* o, const uint8_t* img, uint8_t* mask, double lr_override) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!img || !mask) return OSUB_EBADARG;
    const int W = o->W, H = o->H, C = o->C;
    const size_t N = o->p.bg_samples, npx = o->npx, nreq = o->p.required_bg_samples;
    const float R0 = (float)o->p.color_dist_threshold;
    const float nsm = (float)N; /* BGSPBAS_N_SAMPLES_FOR_MEAN */
    ++o->frames;
    memset(o->kctr, 0, npx * sizeof(uint32_t));
    memset(o->rawFG, 0, npx);
    opbas_gradient(img, W, H, C, o->grad);
    size_t totGrad = 0;    /* single channel: size_t sum of the bad samples' gradient distances */
    float totGradF = 0.0f; /* three channels: float sum, in raster order */
    size_t nBad = 1;
    const float gw = PBAS_GRAD_WEIGHT_ALPHA / o->meanGrad;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t px = (size_t)y * W + x;
            const uint8_t* in = img + px * C;
            const uint8_t* ig = o->grad + px * C;
            float fMinDist = 255.0f;
            const float thr = o->R[px] * R0;
            size_t nGood = 0, s = 0;
            while (nGood < nreq && s < N) {
                const uint8_t* bc = o->scol + s * npx * C + px * C;
                const uint8_t* bg = o->sgrad + s * npx * C + px * C;
                float fSum, fGrad = 0.0f;
                size_t nGrad = 0;
                if (C == 1) {
                    const size_t nCol = absdiff(in[0], bc[0]);
                    nGrad = absdiff(ig[0], bg[0]);
                    fSum = gw * (float)nGrad + (float)nCol;
                } else {
                    const float fCol = pbas_l2(in, bc);
                    fGrad = pbas_l2(ig, bg);
                    fSum = gw * fGrad + fCol;
                }
                if (fSum > 255.0f) fSum = 255.0f; /* std::min(.., (float)nChannelSize) */
                if (fSum <= thr) {
                    if (fMinDist > fSum) fMinDist = fSum;
                    ++nGood;
                } else {
                    if (C == 1) totGrad += nGrad;
                    else totGradF += fGrad;
                    ++nBad;
                }
                ++s;
            }
            float* Dp = &o->D[px];
            *Dp = ((*Dp) * (nsm - 1) + (fMinDist / 255.0f)) / nsm;
            float* Tp = &o->T[px];
            if (nGood < nreq) {
                o->rawFG[px] = 255;
                *Tp += PBAS_T_INCR / ((*Dp) * PBAS_T_SCALE + PBAS_T_OFFST);
                if (*Tp > PBAS_T_UPPER) *Tp = PBAS_T_UPPER;
            } else {
                /* +inf (undefined behaviour in the conversion) is taken as SIZE_MAX, as LOBSTER does */
                const size_t nLR = lr_override > 0 ? (isinf(lr_override) ? (size_t)-1 : (size_t)ceil(lr_override))
                                                   : (size_t)ceil((double)*Tp);
                if (((size_t)pdraw(o, px) % nLR) == 0) {
                    const size_t rs = (size_t)pdraw(o, px) % N;
                    memcpy(o->scol + rs * npx * C + px * C, in, (size_t)C);
                    memcpy(o->sgrad + rs * npx * C + px * C, ig, (size_t)C);
                }
                if (((size_t)pdraw(o, px) % nLR) == 0) {
                    int nx, ny;
                    neighbor_pos(pdraw(o, px), 1, &nx, &ny, x, y, 0, W, H);
                    const size_t rs = (size_t)pdraw(o, px) % N;
                    const size_t np = (size_t)ny * W + nx;
                    /* self diffusion: the neighbour's sample takes the neighbour's own values (:192-194) */
                    memcpy(o->scol + rs * npx * C + np * C, img + np * C, (size_t)C);
                    memcpy(o->sgrad + rs * npx * C + np * C, o->grad + np * C, (size_t)C);
                }
                *Tp -= PBAS_T_DECR / ((*Dp) * PBAS_T_SCALE + PBAS_T_OFFST);
                if (*Tp < PBAS_T_LOWER) *Tp = PBAS_T_LOWER;
            }
            float* Rp = &o->R[px];
            if (*Rp < PBAS_R_LOWER + (*Dp) * PBAS_R_SCALE + PBAS_R_OFFST) {
                if (*Rp < PBAS_R_UPPER) *Rp *= PBAS_R_INCR;
            } else if (*Rp > PBAS_R_LOWER) {
                *Rp *= PBAS_R_DECR;
            }
        }
    /* :232 / :460 */
    const float mean = C == 1 ? ((float)totGrad) / (float)nBad : totGradF / (float)nBad;
    o->meanGrad = mean > 20.0f ? mean : 20.0f;
    /* cv::medianBlur(oFGMask, oFGMask, 9) (:278 / :493) */
    median_binary(o->rawFG, mask, o->colcnt, W, H, 9);
    return OSUB_OK;
}

/* BackgroundSubtractorPBAS::getBackgroundImage (:36-51) */
int opbas_get_background(const opbas_t* o, uint8_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t N = o->p.bg_samples, n = o->npx * (size_t)o->C;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->scol[s * n + i]) / (float)N;
        out[i] = sat_u8f(acc);
    }
    return OSUB_OK;
}

const void* opbas_map(const opbas_t* o, int which, size_t* nbytes) {
    const size_t npx = o->npx, C = (size_t)o->C, N = o->p.bg_samples;
    size_t n = 0;
    const void* p = NULL;
    switch (which) {
        case OPBAS_MAP_SAMPLE_COLOR: p = o->scol; n = N * npx * C; break;
        case OPBAS_MAP_SAMPLE_GRAD: p = o->sgrad; n = N * npx * C; break;
        case OPBAS_MAP_R: p = o->R; n = npx * 4; break;
        case OPBAS_MAP_T: p = o->T; n = npx * 4; break;
        case OPBAS_MAP_D: p = o->D; n = npx * 4; break;
        case OPBAS_MAP_GRAD: p = o->grad; n = npx * C; break;
        default: break;
    }
    if (nbytes) *nbytes = o->initialized ? n : 0;
    return o->initialized ? p : NULL;
}

float opbas_mean_grad(const opbas_t* o) { return o->meanGrad; }
