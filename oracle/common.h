/* ORACLE (test infrastructure only): helpers shared by the SuBSENSE and PAWCS restatements --
 * the LBSP pattern and sampling tables of the reference, its small arithmetic helpers, and the
 * OpenCV image operations both paths call (definitions stated beside each; parity with the real
 * OpenCV is unpinned). */
#ifndef LV_ORACLE_COMMON_H
#define LV_ORACLE_COMMON_H
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#if defined(__GNUC__)
#define OC_UNUSED __attribute__((unused))
#else
#define OC_UNUSED
#endif

#define LBSP_BORDER 2

/* LBSP 16-bit double-cross pattern, LBSP.hpp:297-298 (x, y offsets per bit) */
static const int k_lbsp_dx[16] = {-2, 2, 0, 0, -2, 2, 2, -2, 0, -1, 0, 1, -1, 1, 1, -1};

static const int k_lbsp_dy[16] = {0, 0, -2, 2, 2, -2, 2, -2, 1, 0, -1, 0, -1, 1, -1, 1};

/* sampling kernels, opencv.hpp:915-923 (7x7 Gaussian weights, sum 512),
 * :945-949 (3x3 neighbours) and :958-964 (5x5 neighbours); pairs are (dx, dy) */
static const int k_pat7[7][7] = {
    {2, 4, 6, 7, 6, 4, 2},     {4, 8, 12, 14, 12, 8, 4}, {6, 12, 21, 25, 21, 12, 6}, {7, 14, 25, 28, 25, 14, 7},
    {6, 12, 21, 25, 21, 12, 6}, {4, 8, 12, 14, 12, 8, 4}, {2, 4, 6, 7, 6, 4, 2}};

static const int k_nb3[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};

static const int k_nb5[24][2] = {{-2, 2}, {-1, 2}, {0, 2},   {1, 2},   {2, 2},  {-2, 1},  {-1, 1},  {0, 1},
                                 {1, 1},  {2, 1},  {-2, 0},  {-1, 0},  {1, 0},  {2, 0},   {-2, -1}, {-1, -1},
                                 {0, -1}, {1, -1}, {2, -1},  {-2, -2}, {-1, -2}, {0, -2}, {1, -2},  {2, -2}};

/* saturate_cast<uchar>(float): cvRound (round half to even) then clamp */
OC_UNUSED static uint8_t sat_u8f(float v) {
    long r = lrintf(v);
    return (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
}

OC_UNUSED static uint8_t sat_u8d(double v) {
    long r = lrint(v);
    return (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
}

OC_UNUSED static uint16_t sat_u16f(float v) {
    long r = lrintf(v);
    return (uint16_t)(r < 0 ? 0 : r > 65535 ? 65535 : r);
}

/* population count of the low 16 bits (bit-parallel sums: no -march flags here, so the builtin would
 * be a library call) */
OC_UNUSED static unsigned popc16(unsigned v) {
    v &= 0xffffu;
    v = v - ((v >> 1) & 0x5555u);
    v = (v & 0x3333u) + ((v >> 2) & 0x3333u);
    v = (v + (v >> 4)) & 0x0f0fu;
    return (v + (v >> 8)) & 0x1fu;
}

OC_UNUSED static size_t absdiff(int a, int b) { return (size_t)(a > b ? a - b : b - a); }

OC_UNUSED static float minf_std(float a, float b) { return (b < a) ? b : a; } /* std::min */
OC_UNUSED static float maxf_std(float a, float b) { return (a < b) ? b : a; } /* std::max */

/* clampImageCoords, opencv.hpp:859-870 */
OC_UNUSED static void clamp_coords(int* x, int* y, int border, int W, int H) {
    if (*x < border) *x = border;
    else if (*x >= W - border) *x = W - border - 1;
    if (*y < border) *y = border;
    else if (*y >= H - border) *y = H - border - 1;
}

/* getSamplePosition_7x7_std2 via getSamplePosition<7,7>, opencv.hpp:873-891,909-925 */
OC_UNUSED static void sample_pos_7x7(int rnd, int* sx, int* sy, int x0, int y0, int border, int W, int H) {
    int r = 1 + (rnd % 512), x = 0, y = 0;
    for (y = 0; y < 7; ++y) {
        for (x = 0; x < 7; ++x) {
            r -= k_pat7[y][x];
            if (r <= 0) goto stop;
        }
    }
stop:
    x += x0 - 3;
    y += y0 - 3;
    clamp_coords(&x, &y, border, W, H);
    *sx = x;
    *sy = y;
}

/* getNeighborPosition_3x3 / _5x5 via getNeighborPosition<N>, opencv.hpp:928-966 */
OC_UNUSED static void neighbor_pos(int rnd, int use3x3, int* nx, int* ny, int x0, int y0, int border, int W, int H) {
    const int r = use3x3 ? rnd % 8 : rnd % 24;
    int x = x0 + (use3x3 ? k_nb3[r][0] : k_nb5[r][0]);
    int y = y0 + (use3x3 ? k_nb3[r][1] : k_nb5[r][1]);
    clamp_coords(&x, &y, border, W, H);
    *nx = x;
    *ny = y;
}

/* LBSP::lookup_16bits_dbcross (LBSP.hpp:300-319) for channel c of an interleaved image */
OC_UNUSED static void lbsp_lookup(const uint8_t* img, int W, int C, int x, int y, int c, uint8_t vals[16]) {
    const size_t row = (size_t)W * C;
    const uint8_t* base = img + (size_t)y * row + (size_t)x * C + c;
    for (int n = 0; n < 16; ++n) vals[n] = base[(long)row * k_lbsp_dy[n] + (long)C * k_lbsp_dx[n]];
}

/* LBSP::computeDescriptor_threshold (LBSP.hpp:193-202): bit n = |val_n - ref| > thr, written as
 * the equivalent range test val_n < lo || val_n > hi with lo = max(ref - thr, 0) and
 * hi = min(ref + thr, 255), on eight taps at a time in 16-bit lanes of a 64-bit word: with a tap in
 * bits 0-7 of a lane, bit 8 of tap + (256 - lo) is tap >= lo and bit 8 of tap + (255 - hi) is
 * tap > hi (no carry leaves a lane) */
OC_UNUSED static uint16_t lbsp_threshold(const uint8_t vals[16], uint8_t ref, uint8_t thr) {
    const uint64_t lo = ref > thr ? (uint64_t)(ref - thr) : 0u;
    const uint64_t hi = (unsigned)ref + thr < 255u ? (uint64_t)ref + thr : 255u;
    const uint64_t lanes = 0x0001000100010001ull, k1 = (256u - lo) * lanes, k2 = (255u - hi) * lanes;
    unsigned d = 0;
    for (int h = 0; h < 2; ++h) {
        const uint8_t* v = vals + 8 * h;
        /* taps 0, 2, 4, 6 of this half in the lanes of e; taps 1, 3, 5, 7 in those of o */
        const uint64_t e = (uint64_t)v[0] | ((uint64_t)v[2] << 16) | ((uint64_t)v[4] << 32) | ((uint64_t)v[6] << 48);
        const uint64_t o = (uint64_t)v[1] | ((uint64_t)v[3] << 16) | ((uint64_t)v[5] << 32) | ((uint64_t)v[7] << 48);
        const uint64_t fe = (~(e + k1) | (e + k2)) & 0x0100010001000100ull;
        const uint64_t fo = (~(o + k1) | (o + k2)) & 0x0100010001000100ull;
        uint64_t m = (fe | (fo << 1)) >> 8; /* taps 2i, 2i+1 at bits 16i, 16i+1 */
        m |= m >> 14;                       /* taps 0-3 at bits 0-3, taps 4-7 at bits 32-35 */
        m |= m >> 28;                       /* taps 4-7 at bits 4-7 */
        d |= (unsigned)(m & 0xffu) << (8 * h);
    }
    return (uint16_t)d;
}

/* cv::dilate / cv::erode with a (2r+1)x(2r+1) rectangle and the default border value
 * (morphologyDefaultBorderValue: out-of-image pixels never win), i.e. max/min over the
 * window clipped to the image. A 3x3 rectangle applied n times equals one (2n+1)^2
 * rectangle for this border rule. Computed separably (rows, then columns). */
OC_UNUSED static void box_minmax(const uint8_t* src, uint8_t* dst, uint8_t* tmp, int W, int H, int r, int is_max) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int v = is_max ? 0 : 255;
            for (int d = -r; d <= r; ++d) {
                const int xx = x + d;
                if (xx < 0 || xx >= W) continue;
                const int s = src[(size_t)y * W + xx];
                v = is_max ? (s > v ? s : v) : (s < v ? s : v);
            }
            tmp[(size_t)y * W + x] = (uint8_t)v;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int v = is_max ? 0 : 255;
            for (int d = -r; d <= r; ++d) {
                const int yy = y + d;
                if (yy < 0 || yy >= H) continue;
                const int s = tmp[(size_t)yy * W + x];
                v = is_max ? (s > v ? s : v) : (s < v ? s : v);
            }
            dst[(size_t)y * W + x] = (uint8_t)v;
        }
}

/* cv::medianBlur(k) of a 0/255 mask with BORDER_REPLICATE: the median of k*k binary
 * values is 255 iff more than half of them are 255 (k is odd). */
OC_UNUSED static void median_binary(const uint8_t* src, uint8_t* dst, uint16_t* colcnt, int W, int H, int k) {
    const int r = k / 2;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int cnt = 0;
            for (int d = -r; d <= r; ++d) {
                int yy = y + d;
                yy = yy < 0 ? 0 : yy >= H ? H - 1 : yy;
                cnt += src[(size_t)yy * W + x] != 0;
            }
            colcnt[(size_t)y * W + x] = (uint16_t)cnt;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int cnt = 0;
            for (int d = -r; d <= r; ++d) {
                int xx = x + d;
                xx = xx < 0 ? 0 : xx >= W ? W - 1 : xx;
                cnt += colcnt[(size_t)y * W + xx];
            }
            dst[(size_t)y * W + x] = (2 * cnt > k * k) ? 255 : 0;
        }
}

/* cv::addWeighted(A (CV_32F), alpha, M (CV_8U), beta, 0, A, CV_32F): M is converted to
 * float and A = A*(float)alpha + M*(float)beta + 0 in float, no fused multiply-add. */
OC_UNUSED static void add_weighted_mask(float* a, const uint8_t* m, size_t n, double alpha, double beta) {
    const float fa = (float)alpha, fb = (float)beta;
    for (size_t i = 0; i < n; ++i) {
        const float t1 = a[i] * fa;
        const float t2 = (float)m[i] * fb;
        a[i] = (t1 + t2) + 0.0f;
    }
}

/* cv::resize(src, dst, (dw, dh), INTER_AREA) of an 8-bit image with C interleaved channels.
 * When the source size is an integral multiple of the output (OpenCV's "area fast" case) each output
 * is the block mean computed as cvRound(sum * (1.f/area)) (round half to even). Otherwise it is the
 * exact area-weighted mean of the source pixels under the output pixel's footprint: in units of 1/dw
 * (1/dh) source pixel i spans [i*dw, (i+1)*dw) and output x spans [x*W, (x+1)*W), every overlap is an
 * integer, and the output is round(sum(ox * oy * src) / (W * H)) with ties to even, in integers. The
 * definition follows the mathematics of the area relation (OpenCV documents INTER_AREA as
 * "resampling using pixel area relation"; its own arithmetic for this case is unpinned here).
 * Returns 0 when the output is empty. */
OC_UNUSED static int resize_area_u8(const uint8_t* src, int W, int H, int C, uint8_t* dst, int dw, int dh) {
    if (dw <= 0 || dh <= 0) return 0;
    if (W % dw == 0 && H % dh == 0) {
        const int sx = W / dw, sy = H / dh;
        const float scale = 1.f / (float)(sx * sy);
        for (int y = 0; y < dh; ++y)
            for (int x = 0; x < dw; ++x)
                for (int c = 0; c < C; ++c) {
                    int sum = 0;
                    for (int yy = 0; yy < sy; ++yy)
                        for (int xx = 0; xx < sx; ++xx) sum += src[((size_t)(y * sy + yy) * W + (x * sx + xx)) * C + c];
                    dst[((size_t)y * dw + x) * C + c] = sat_u8f((float)sum * scale);
                }
        return 1;
    }
    const unsigned long long den = (unsigned long long)W * (unsigned long long)H;
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            const long long x0 = (long long)x * W, x1 = x0 + W, y0 = (long long)y * H, y1 = y0 + H;
            const int i0 = (int)(x0 / dw), i1 = (int)((x1 + dw - 1) / dw);
            const int j0 = (int)(y0 / dh), j1 = (int)((y1 + dh - 1) / dh);
            for (int c = 0; c < C; ++c) {
                unsigned long long num = 0;
                for (int j = j0; j < j1; ++j) {
                    const long long a = (long long)j * dh, b = a + dh;
                    const long long oy = (b < y1 ? b : y1) - (a > y0 ? a : y0);
                    unsigned long long row = 0;
                    for (int i = i0; i < i1; ++i) {
                        const long long cc = (long long)i * dw, d = cc + dw;
                        const long long ox = (d < x1 ? d : x1) - (cc > x0 ? cc : x0);
                        row += (unsigned long long)ox * src[((size_t)j * W + i) * C + c];
                    }
                    num += row * (unsigned long long)oy;
                }
                unsigned long long q = num / den;
                const unsigned long long r2 = (num % den) * 2ull;
                if (r2 > den || (r2 == den && (q & 1ull))) ++q;
                dst[((size_t)y * dw + x) * C + c] = (uint8_t)(q > 255ull ? 255ull : q);
            }
        }
    return 1;
}
/* the frame-level down-sampling of SuBSENSE (BackgroundSubtractorSuBSENSE.cpp:568) */
OC_UNUSED static int resize_area_div8(const uint8_t* src, int W, int H, int C, uint8_t* dst, int dw, int dh) {
    return resize_area_u8(src, W, H, C, dst, dw, dh);
}

/* cv::accumulateWeighted(src, dst, alpha): dst = src*a + dst*(1-a) with a = (float)alpha,
 * in float, no fused multiply-add. */
OC_UNUSED static void accumulate_weighted(const uint8_t* src, float* dst, size_t n, double alpha) {
    const float a = (float)alpha, b = 1.0f - a;
    for (size_t i = 0; i < n; ++i) {
        const float t1 = (float)src[i] * a;
        const float t2 = dst[i] * b;
        dst[i] = t1 + t2;
    }
}

#endif
