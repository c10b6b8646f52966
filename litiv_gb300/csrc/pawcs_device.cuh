// Device helpers shared by the one- and three-channel PAWCS kernels (pawcs_kernels.cu,
// pawcs3_kernels.cu): the reference's tables, draws, word weights, thresholds and LBSP.
#pragma once
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "pawcs_internal.h"

namespace lvbgs {

// LBSP double-cross taps (LBSP.hpp:297-298), sampling tables (opencv.hpp:915-964)
static __constant__ int pw_dx[16] = {-2, 2, 0, 0, -2, 2, 2, -2, 0, -1, 0, 1, -1, 1, 1, -1};
static __constant__ int pw_dy[16] = {0, 0, -2, 2, 2, -2, 2, -2, 1, 0, -1, 0, -1, 1, -1, 1};
static __constant__ int pw_pat7[49] = {2, 4, 6, 7, 6, 4, 2, 4, 8, 12, 14, 12, 8, 4, 6, 12, 21, 25, 21, 12, 6, 7, 14, 25, 28,
                                25, 14, 7, 6, 12, 21, 25, 21, 12, 6, 4, 8, 12, 14, 12, 8, 4, 2, 4, 6, 7, 6, 4, 2};
static __constant__ int pw_nb3[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};
static __constant__ int pw_nb5[24][2] = {{-2, 2}, {-1, 2}, {0, 2},   {1, 2},   {2, 2},   {-2, 1},  {-1, 1}, {0, 1},
                                  {1, 1},  {2, 1},  {-2, 0},  {-1, 0},  {1, 0},   {2, 0},   {-2, -1}, {-1, -1},
                                  {0, -1}, {1, -1}, {2, -1},  {-2, -2}, {-1, -2}, {0, -2},  {1, -2},  {2, -2}};

constexpr float kTLower = 1.0f, kTUpper = 256.0f, kTIncr = 0.5f, kTDecr = 0.25f;
constexpr float kVIncr = 1.0f, kVDecr = 0.1f, kRVar = 0.01f, kUnstRatio = 0.1f, kUnstR = 3.0f;
constexpr int kBootWin = kPwBootWin;

__device__ __forceinline__ int pw_stream_by_tile(const PwParams& P, int t) {
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.streams[mid].sd.tileBase <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int pw_stream_by_row(const PwParams& P, int r) {
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.streams[mid].sd.rowBase <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// one rand() of the reference: draw k of pixel px in frame f
__device__ __forceinline__ uint32_t pw_draw(unsigned long long seed, uint32_t f, uint32_t px, uint32_t k) {
    uint32_t c[4] = {k >> 2, px, f, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return c[k & 3u] & 0x7fffffffu;
}
// draw % m for the reference's size_t moduli (rand() < 2^31, so a modulus above 2^32 leaves it as is)
__device__ __forceinline__ uint32_t pw_mod(uint32_t r, unsigned long long m) {
    return m > 0xffffffffull ? r : r % (uint32_t)m;
}

// GetLocalWordWeight (:1596-1598): (float)occ / (float)((last-first) + (t-last)*2 + offset)
__device__ __forceinline__ float pw_weight(uint32_t occ, uint32_t first, uint32_t last, uint32_t t,
                                           unsigned long long off) {
    const unsigned long long den = (unsigned long long)(last - first) + (unsigned long long)(t - last) * 2ull + off;
    return (float)occ / (float)den;
}

struct PwThr {
    uint32_t color, desc;
};

// (size_t)(sqrt(R) * m) as the reference evaluates it: an unqualified sqrt of a float there is the
// C library's double sqrt, and the product is taken in double (:119, :267, :663, :993). For a float R
// and a small integer m that truncation equals the exact floor(m * sqrt(R)), the largest k with
// k^2 <= m^2 R (a float R lies at least 2^-24/m^2 in relative terms from any such boundary, far more
// than the two double roundings move the product). A float candidate is corrected by one with an
// exact comparison: hi + lo = m^2 R exactly (two-product), k^2 exact in float below 2^24.
__device__ __forceinline__ uint32_t pw_sqrt_floor(float R, uint32_t m) {
    uint32_t k = (uint32_t)(__fsqrt_rn(R) * (float)m);
    const float mm = (float)(m * m);
    if (m * m >= (1u << 24) || k >= 4095u) return (uint32_t)(__dsqrt_rn((double)R) * (double)m);
    const float hi = mm * R, lo = __fmaf_rn(mm, R, -hi);
    const auto le = [&](uint32_t kk) {  // kk^2 <= m^2 R
        const float k2 = (float)(kk * kk);
        return k2 < hi || (k2 == hi && lo >= 0.0f);
    };
    if (!le(k)) --k;
    else if (le(k + 1)) ++k;
    return k;
}
// nCurrColorDistThreshold / nCurrDescDistThreshold of one channel (:633-634)
__device__ __forceinline__ PwThr pw_thresholds(float R, uint32_t unstable, uint32_t minColor, uint32_t descOff) {
    PwThr t;
    t.color = pw_sqrt_floor(R, minColor) / 2u;
    const unsigned long long sh = (unsigned long long)floorf(R + 0.5f);
    const unsigned long long d = (sh < 64 ? (1ull << sh) : 0ull) + descOff + (unsigned long long)unstable * descOff;
    t.desc = d > 0xffffffffull ? 0xffffffffu : (uint32_t)d;
    return t;
}

__device__ __forceinline__ uint32_t pw_absdiff(uint32_t a, uint32_t b) { return a > b ? a - b : b - a; }

// current frame: LBSP lookups of pixel (x, y) and its descriptor
__device__ __forceinline__ void pw_taps(const uint8_t* img, int W, int x, int y, uint8_t taps[16]) {
#pragma unroll
    for (int n = 0; n < 16; ++n) taps[n] = __ldg(img + (size_t)(y + pw_dy[n]) * W + (x + pw_dx[n]));
}
__device__ __forceinline__ uint32_t pw_lbsp(const uint8_t taps[16], uint32_t ref, uint32_t thr) {
    uint32_t d = 0;
#pragma unroll
    for (int n = 0; n < 16; ++n) d |= (uint32_t)(pw_absdiff(taps[n], ref) > thr) << n;
    return d;
}

// rolling-average factors of frame f (:570-573)
__device__ __forceinline__ void pw_factors(unsigned long long f, int nmv, float* fLT, float* fST) {
    const int boot = f <= (unsigned long long)kBootWin;
    const unsigned long long nlt = boot ? (unsigned long long)(nmv / 2) : (unsigned long long)nmv, nst = nlt / 4;
    *fLT = 1.0f / (float)(f < nlt ? f : nlt);
    *fST = 1.0f / (float)(f < nst ? f : nst);
}

__device__ __forceinline__ size_t pw_slot(const PawcsDev& S, int buf, int j, int p) {
    return ((size_t)buf * S.L + j) * S.sd.npx + p;
}

}  // namespace lvbgs

namespace lvbgs {

// ---- three channels: packed colours (c0 | c1 << 8 | c2 << 16), descriptors (d0 | d1 << 16, d2) ----

// nCurrColorDistThreshold / nCurrDescDistThreshold of three channels (:1011-1012)
__device__ __forceinline__ PwThr pw3_thresholds(float R, uint32_t unstable, uint32_t minColor, uint32_t descOff) {
    PwThr t;
    t.color = pw_sqrt_floor(R, minColor) * 3u;
    const unsigned long long sh = (unsigned long long)floorf(R + 0.5f);
    const unsigned long long d = ((sh < 64 ? (1ull << sh) : 0ull) + descOff + (unsigned long long)unstable * descOff) * 3ull;
    t.desc = d > 0xffffffffull ? 0xffffffffu : (uint32_t)d;
    return t;
}
__device__ __forceinline__ uint32_t pw3_ch(uint32_t c, int k) { return (c >> (8 * k)) & 255u; }
// lv::L1dist of two three-byte colours (math.hpp:226-250): the reference accumulates the sum in
// the type of L1dist(uchar, uchar), unsigned char, so it wraps modulo 256 (every three-channel colour
// L1 of PAWCS goes through it, directly or through cmixdist)
__device__ __forceinline__ uint32_t pw3_l1(uint32_t a, uint32_t b) {
    return (pw_absdiff(pw3_ch(a, 0), pw3_ch(b, 0)) + pw_absdiff(pw3_ch(a, 1), pw3_ch(b, 1)) +
            pw_absdiff(pw3_ch(a, 2), pw3_ch(b, 2))) & 0xffu;
}
// lv::cdist<3> of two byte colours (math.hpp:474-496): sqrt of the colour distortion, 0 for a grey
// pair or identical colours
__device__ __forceinline__ uint32_t pw3_cdist(uint32_t a, uint32_t b) {
    const uint32_t a0 = pw3_ch(a, 0), a1 = pw3_ch(a, 1), a2 = pw3_ch(a, 2);
    const uint32_t b0 = pw3_ch(b, 0), b1 = pw3_ch(b, 1), b2 = pw3_ch(b, 2);
    const bool nonconst = a1 != a0 || b1 != b0 || a2 != a1 || b2 != b1;
    const bool nonnull = a0 != b0 || a1 != b1 || a2 != b2;
    if (!nonconst || !nonnull) return 0u;
    const unsigned long long cs = a0 * a0 + a1 * a1 + a2 * a2, bs = b0 * b0 + b1 * b1 + b2 * b2;
    const unsigned long long mix = a0 * b0 + a1 * b1 + a2 * b2;
    const float sq = (float)(cs - (mix * mix) / (bs > 1ull ? bs : 1ull));
    return (uint32_t)__fsqrt_rn(sq);
}
// lv::cmixdist (math.hpp:596-605)
__device__ __forceinline__ uint32_t pw3_cmix(uint32_t a, uint32_t b) { return pw3_l1(a, b) / 2u + pw3_cdist(a, b) * 4u; }
__device__ __forceinline__ uint32_t pw3_hd(uint32_t a01, uint32_t a2, uint32_t b01, uint32_t b2) {
    return (uint32_t)__popc(a01 ^ b01) + (uint32_t)__popc((a2 ^ b2) & 0xffffu);
}
// the 16 taps of each channel of pixel (x, y) of an interleaved BGR frame
__device__ __forceinline__ void pw3_taps(const uint8_t* img, int W, int x, int y, uint8_t taps[3][16]) {
#pragma unroll
    for (int n = 0; n < 16; ++n) {
        const uint8_t* q = img + ((size_t)(y + pw_dy[n]) * W + (x + pw_dx[n])) * 3;
        taps[0][n] = q[0];
        taps[1][n] = q[1];
        taps[2][n] = q[2];
    }
}
__device__ __forceinline__ uint32_t pw3_color(const uint8_t* img, int p) {
    const uint8_t* q = img + (size_t)p * 3;
    return (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16);
}

}  // namespace lvbgs
