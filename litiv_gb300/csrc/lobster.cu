// LOBSTER, ViBe and PBAS frame steps for sm_103a (BackgroundSubtractorLOBSTER.cpp:459-581, the
// non-parallel path; BackgroundSubtractorViBe.cpp:77-191; BackgroundSubtractorPBAS.cpp:111-496). The
// kernels are written for LOBSTER and take the algorithm as a template parameter: ViBe evaluates every
// pixel (no ROI), matches colours only, keeps plain colour samples and outputs its raw mask, and its
// neighbour positions are clamped to the frame instead of the LBSP border; PBAS adds a gradient image,
// gradient samples, per-pixel R/T/D maps and a frame-level mean gradient distance, and its neighbour
// update writes the target's own values (self diffusion). The scheme below is the same for all three.
//
// The reference scans the ROI pixels in raster order. A pixel reads its own samples, which an earlier
// pixel's neighbour update may have overwritten in the same frame (:510-512 / :569-574); nothing else
// it reads changes during the frame. Random draws are keyed by (seed, frame, pixel, draw index), so
// they do not depend on the scan order. A frame step therefore
//   1. evaluates every pixel against the frame-start samples (lob_k_eval): decision, samples scanned
//      e, and the model writes it makes (own sample, neighbour target and sample), in an intent word;
//   2. marks the pixels whose scan read a sample that an earlier neighbour writes (lob_k_mark);
//   3. re-evaluates the marked pixels with the samples the raster scan would see (the latest earlier
//      writer of each sample), and marks the later pixels whose incoming writes changed, round after
//      round until nothing changes (lob_k_round; the dependencies follow raster order, so this is the
//      raster-order fixed point). Rounds are enqueued ahead; a converged flag makes the rest return;
//   4. commits every sample write in raster order, each pixel gathering the writes aimed at it from
//      its 3x3 neighbourhood (lob_k_commit), then the median blur of the mask (:577-579).
// The writers of a pixel are within one pixel of it: getNeighborPosition_3x3 moves one step and
// clamps into the LBSP border, and ROI pixels lie inside that border.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "lbsp_device.cuh"
#include "lobster_internal.h"

namespace lvbgs {

namespace {

// LBSP 16-bit double-cross pattern (LBSP.hpp:297-298) as compile-time offsets: (offset + 2) in three
// bits per tap, so that unrolled tap loops fold the offsets into immediates
constexpr unsigned long long pack3(const int (&a)[16]) {
    unsigned long long v = 0;
    for (int i = 0; i < 16; ++i) v |= (unsigned long long)(a[i] + 2) << (3 * i);
    return v;
}
constexpr int kDx[16] = {-2, 2, 0, 0, -2, 2, 2, -2, 0, -1, 0, 1, -1, 1, 1, -1};
constexpr int kDy[16] = {0, 0, -2, 2, 2, -2, 2, -2, 1, 0, -1, 0, -1, 1, -1, 1};
constexpr unsigned long long kDx3 = pack3(kDx), kDy3 = pack3(kDy);
__device__ __forceinline__ constexpr int tap_dx(int n) { return (int)((kDx3 >> (3 * n)) & 7ull) - 2; }
__device__ __forceinline__ constexpr int tap_dy(int n) { return (int)((kDy3 >> (3 * n)) & 7ull) - 2; }

// 7x7 Gaussian sampling weights (opencv.hpp:915-923) and the 3x3 neighbour table (opencv.hpp:945-953)
__constant__ int c_lob_pat7[49] = {2,  4,  6,  7,  6,  4,  2,  4,  8,  12, 14, 12, 8,  4,  6, 12, 21,
                                   25, 21, 12, 6,  7,  14, 25, 28, 25, 14, 7,  6,  12, 21, 25, 21, 12,
                                   6,  4,  8,  12, 14, 12, 8,  4,  2,  4,  6,  7,  6,  4,  2};
__constant__ int c_lob_nb3[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};

constexpr int kThreadsL = 256;
constexpr int kMaxRoundsL = 4096;  // repair rounds of one frame step before LVBGS_DEVICE_ERROR

// ---- intent word ----
// bit 0 valid (ROI pixel evaluated), bit 1 foreground, bits 2-8 samples scanned, bit 9 own-sample write,
// bits 10-15 its sample, bit 16 neighbour write, bits 17-20 neighbour code (dy+1)*3+(dx+1), bits 21-26
// its sample, bits 27-29 draws consumed
constexpr uint32_t kIValid = 1u, kIFG = 2u, kIOwn = 1u << 9, kINb = 1u << 16;
__device__ __forceinline__ int i_e(uint32_t w) { return (int)((w >> 2) & 127u); }
__device__ __forceinline__ int i_sown(uint32_t w) { return (int)((w >> 10) & 63u); }
__device__ __forceinline__ int i_code(uint32_t w) { return (int)((w >> 17) & 15u); }
__device__ __forceinline__ int i_snb(uint32_t w) { return (int)((w >> 21) & 63u); }
__device__ __forceinline__ int i_draws(uint32_t w) { return (int)((w >> 27) & 7u); }
// the neighbour-write part of an intent (target and sample)
__device__ __forceinline__ uint32_t i_nbpart(uint32_t w) { return (w & kIValid) ? (w & (kINb | (1023u << 17))) : 0u; }
__device__ __forceinline__ int nb_target(uint32_t w, int q, int W) {
    const int c = i_code(w);
    return q + (c / 3 - 1) * W + (c % 3 - 1);
}

__device__ __forceinline__ unsigned int ld_vol(const unsigned int* p) { return *(const volatile unsigned int*)p; }

// draw k of pixel p in frame t (the counter-based generator that replaces rand())
struct Draws {
    uint32_t blk, v[4];
};
__device__ __forceinline__ uint32_t draw(const LobDev& D, uint32_t p, uint32_t k, Draws& ds) {
    const uint32_t blk = k >> 2;
    if (blk != ds.blk) {
        uint32_t c[4] = {blk, p, D.frameKey, 0u};
        philox4x32_10(c, (uint32_t)D.seed, (uint32_t)(D.seed >> 32));
        ds.v[0] = c[0];
        ds.v[1] = c[1];
        ds.v[2] = c[2];
        ds.v[3] = c[3];
        ds.blk = blk;
    }
    return ds.v[k & 3u] & 0x7fffffffu;
}
// rand() % m for a 31-bit draw and a size_t modulus
__device__ __forceinline__ unsigned long long mod64(uint32_t a, unsigned long long m) {
    if (m > 0xffffffffull) return a;
    const uint32_t m32 = (uint32_t)m;
    if ((m32 & (m32 - 1u)) == 0u) return a & (m32 - 1u);
    return a % m32;
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

// the 16 LBSP taps of channel c at pixel index p of a dense image, packed four to a word
template <int C>
__device__ __forceinline__ void taps(const uint8_t* img, int W, int p, int c, uint32_t (&v)[4]) {
    const uint8_t* base = img + (size_t)p * C + c;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint32_t w = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int n = 4 * j + i;
            w |= (uint32_t)__ldg(base + (tap_dy(n) * W + tap_dx(n)) * C) << (8 * i);
        }
        v[j] = w;
    }
}

// sample s of pixel p: LOBSTER, the packed word and the colour byte; ViBe, the colour bytes packed into d
template <int C, int ALG>
__device__ __forceinline__ void load_sample(const LobDev& D, int s, int p, unsigned long long& d, uint32_t& c2) {
    if (ALG == ALG_VIBE || ALG == ALG_PBAS) {
        // colour c at bits 8c; PBAS: gradient c at bits 24 + 8c
        const size_t o = ((size_t)s * D.npx + p) * C;
        d = 0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            d |= (unsigned long long)__ldg(D.sC + o + c) << (8 * c);
            if (ALG == ALG_PBAS) d |= (unsigned long long)__ldg(D.sG + o + c) << (24 + 8 * c);
        }
        c2 = 0;
        return;
    }
    if (C == 3) d = __ldg((const unsigned long long*)D.sD + (size_t)s * D.npx + p);
    else d = __ldg((const uint16_t*)D.sD + (size_t)s * D.npx + p);
    c2 = __ldg(D.sC + (size_t)s * D.npx + p);
}

// one sample against the pixel: LOBSTER (:479-494 / :522-541); ViBe (BackgroundSubtractorViBe.cpp:87 /
// :165-170): |in - bg| < R on one channel; on three, lv::L2dist<3>(uchar*, uchar*) < 3R, whose squared
// differences add up in uint16_t (utils/math.hpp:391-396), so the sum s wraps modulo 65536 before the
// square root. For integers s < 65536 and T = 3R, (float)sqrt(s) < (float)T is exactly s < T*T when
// T < 256 (sqrt(T*T - 1) < T - 1/(2T), and 1/(2T) is far above the float spacing near T), and always true
// when T >= 256
template <int C, int ALG>
__device__ __forceinline__ bool match(const LobDev& D, const uint32_t (&vals)[C][4], const uint32_t (&curr)[C],
                                      unsigned long long d, uint32_t c2) {
    if (ALG == ALG_VIBE) {
        if (C == 1) return (uint32_t)abs((int)curr[0] - (int)(d & 0xffu)) < D.colThr;
        uint32_t acc = 0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int dv = (int)curr[c] - (int)((d >> (8 * c)) & 0xffu);
            acc += (uint32_t)(dv * dv);
        }
        const unsigned long long T = 3ull * D.colThr;
        return T >= 256ull || (unsigned long long)(acc & 0xffffu) < T * T;
    }
    if (C == 1) {
        const uint32_t bgc = c2, bgd = (uint32_t)d & 0xffffu;
        if ((uint32_t)abs((int)curr[0] - (int)bgc) > D.colThr / 2u) return false;
        return (uint32_t)__popc(lbsp_thr(vals[0], bgc, __ldg(D.lut + bgc)) ^ bgd) <= D.descThr;
    } else {
        const uint32_t descThr = D.descThr * 3u, colThr = D.colThr * 3u;
        const uint32_t scDesc = descThr / 2u, scCol = colThr / 2u;
        uint32_t totCol = 0, totDesc = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint32_t bgc = c == 0 ? (uint32_t)(d >> 48) & 0xffu : c == 1 ? (uint32_t)(d >> 56) & 0xffu : c2;
            const uint32_t bgd = (uint32_t)(d >> (16 * c)) & 0xffffu;
            const uint32_t colDist = (uint32_t)abs((int)curr[c] - (int)bgc);
            if (colDist > scCol) return false;
            const uint32_t descDist = (uint32_t)__popc(lbsp_thr(vals[c], bgc, __ldg(D.lut + bgc)) ^ bgd);
            if (descDist > scDesc) return false;
            totCol += colDist;
            totDesc += descDist;
        }
        return totDesc <= descThr && totCol <= colThr;
    }
}

// overrides of a re-evaluation: the samples that earlier neighbours write (latest writer last)
struct LobOvr {
    int n;
    int s[4];
    unsigned long long d[4];
    uint32_t c[4];
    unsigned long long mask;
};

// the evaluation of pixel p (x, y): ordered scan (with overrides), then the decision and the model
// writes with their draws (:497-513 / :545-575); returns the intent word
template <int C, int ALG, bool OVR>
__device__ uint32_t eval_px(const LobDev& D, int p, int x, int y, const uint32_t (&vals)[C][4],
                            const uint32_t (&curr)[C], const LobOvr& ov, unsigned long long* scanned) {
    int nGood = 0, s = 0;
    unsigned long long dB = 0;
    uint32_t cB = 0;
    if (D.N > 0) load_sample<C, ALG>(D, 0, p, dB, cB);
    while (nGood < D.nreq && s < D.N) {
        unsigned long long d = dB;
        uint32_t c2 = cB;
        if (s + 1 < D.N) load_sample<C, ALG>(D, s + 1, p, dB, cB);
        if (OVR && ((ov.mask >> s) & 1ull)) {
            for (int k = 0; k < ov.n; ++k)
                if (ov.s[k] == s) {
                    d = ov.d[k];
                    c2 = ov.c[k];
                }
        }
        if (match<C, ALG>(D, vals, curr, d, c2)) ++nGood;
        ++s;
    }
    *scanned += (unsigned long long)s;
    uint32_t w = kIValid | ((uint32_t)s << 2);
    if (nGood < D.nreq) return w | kIFG;
    Draws ds;
    ds.blk = 0xffffffffu;
    uint32_t k = 0;
    if (mod64(draw(D, (uint32_t)p, k++, ds), D.nLR) == 0ull) {
        const uint32_t so = draw(D, (uint32_t)p, k++, ds) % (uint32_t)D.N;
        w |= kIOwn | (so << 10);
    }
    if (mod64(draw(D, (uint32_t)p, k++, ds), D.nLR) == 0ull) {
        // getNeighborPosition_3x3 (opencv.hpp:945-953), clamped into the LBSP border (LOBSTER) or the frame (ViBe)
        constexpr int bord = ALG == ALG_VIBE ? 0 : kBorder;
        const int r = (int)(draw(D, (uint32_t)p, k++, ds) % 8u);
        const int nx = clampi(x + c_lob_nb3[r][0], bord, D.W - bord - 1);
        const int ny = clampi(y + c_lob_nb3[r][1], bord, D.H - bord - 1);
        const uint32_t sn = draw(D, (uint32_t)p, k++, ds) % (uint32_t)D.N;
        const uint32_t code = (uint32_t)((ny - y + 1) * 3 + (nx - x + 1));
        w |= kINb | (code << 17) | (sn << 21);
    }
    return w | (k << 27);
}

// PBAS's evaluation of pixel p (:146-231 / :365-458): the ordered scan with the colour + weighted
// gradient distance against the threshold R(x) * R0, the bad samples' gradient distances for the frame
// level, then the D(x), T(x) and R(x) updates (written to the maps of the next parity) and the model
// updates with their draws. g holds the pixel's gradient. Three-channel distances: (float)sqrt((double)s)
// of the uint16 sum s equals sqrtf((float)s), since double rounding through double is innocuous for the
// square root (53 >= 2 * 24 + 2 bits).
template <int C, bool OVR>
__device__ uint32_t pbas_eval_px(const LobDev& D, int p, int x, int y, const uint32_t (&curr)[C], const uint32_t (&g)[C],
                                 const LobOvr& ov, unsigned long long* scanned) {
    const size_t npx = (size_t)D.npx;
    const float* fc = D.fm + (size_t)D.cur * 3 * npx;
    float* fn = D.fm + (size_t)(D.cur ^ 1) * 3 * npx;
    const float R = fc[p], T = fc[npx + p], Dm = fc[2 * npx + p];
    const float thr = R * D.R0;
    const float gw = 10.0f / *D.meanGrad;  // BGSPBAS_GRAD_WEIGHT_ALPHA / m_fFormerMeanGradDist
    float fMin = 255.0f;
    int nGood = 0, s = 0, nb = 0;
    uint32_t badSum = 0;
    unsigned long long dB = 0;
    uint32_t cB = 0;
    if (D.N > 0) load_sample<C, ALG_PBAS>(D, 0, p, dB, cB);
    while (nGood < D.nreq && s < D.N) {
        unsigned long long d = dB;
        if (s + 1 < D.N) load_sample<C, ALG_PBAS>(D, s + 1, p, dB, cB);
        if (OVR && ((ov.mask >> s) & 1ull)) d = ov.d[0];  // self diffusion: the pixel's own values
        float fSum, fGrad = 0.0f;
        uint32_t nGrad = 0;
        if (C == 1) {
            const uint32_t nCol = (uint32_t)abs((int)curr[0] - (int)(d & 0xffu));
            nGrad = (uint32_t)abs((int)g[0] - (int)((d >> 24) & 0xffu));
            fSum = gw * (float)nGrad + (float)nCol;
        } else {
            uint32_t aC = 0, aG = 0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int dc = (int)curr[c] - (int)((d >> (8 * c)) & 0xffu);
                const int dg = (int)g[c] - (int)((d >> (24 + 8 * c)) & 0xffu);
                aC += (uint32_t)(dc * dc);
                aG += (uint32_t)(dg * dg);
            }
            fGrad = __fsqrt_rn((float)(aG & 0xffffu));
            fSum = gw * fGrad + __fsqrt_rn((float)(aC & 0xffffu));
        }
        if (fSum > 255.0f) fSum = 255.0f;
        if (fSum <= thr) {
            if (fMin > fSum) fMin = fSum;
            ++nGood;
        } else {
            if (C == 1) badSum += nGrad;
            else D.badVals[(size_t)p * D.N + nb] = fGrad;
            ++nb;
        }
        ++s;
    }
    *scanned += (unsigned long long)s;
    const float Nf = (float)D.N;
    const float Dn = (Dm * (Nf - 1.0f) + fMin / 255.0f) / Nf;
    uint32_t w = kIValid | ((uint32_t)s << 2);
    float Tn;
    uint32_t k = 0;
    if (nGood < D.nreq) {
        w |= kIFG;
        Tn = T + 1.0000f / (Dn * 255.00f + 1.0000f);
        if (Tn > 200.00f) Tn = 200.00f;
    } else {
        const unsigned long long nLR = D.lrOverride ? D.nLR : (unsigned long long)__float2uint_rz(ceilf(T));
        Draws ds;
        ds.blk = 0xffffffffu;
        if (mod64(draw(D, (uint32_t)p, k++, ds), nLR) == 0ull) {
            const uint32_t so = draw(D, (uint32_t)p, k++, ds) % (uint32_t)D.N;
            w |= kIOwn | (so << 10);
        }
        if (mod64(draw(D, (uint32_t)p, k++, ds), nLR) == 0ull) {
            const int r = (int)(draw(D, (uint32_t)p, k++, ds) % 8u);
            const int nx = clampi(x + c_lob_nb3[r][0], 0, D.W - 1);
            const int ny = clampi(y + c_lob_nb3[r][1], 0, D.H - 1);
            const uint32_t sn = draw(D, (uint32_t)p, k++, ds) % (uint32_t)D.N;
            w |= kINb | ((uint32_t)((ny - y + 1) * 3 + (nx - x + 1)) << 17) | (sn << 21);
        }
        Tn = T - 0.0500f / (Dn * 255.00f + 1.0000f);
        if (Tn < 2.0000f) Tn = 2.0000f;
    }
    float Rn = R;
    if (R < 0.6000f + Dn * 5.0000f + 0.0000f) {
        if (R < 99.0000f) Rn = R * 1.0500f;
    } else if (R > 0.6000f) {
        Rn = R * 0.9500f;
    }
    fn[p] = Rn;
    fn[npx + p] = Tn;
    fn[2 * npx + p] = Dn;
    if (C == 1) D.badSum[p] = badSum;  // three channels keep the values themselves (badVals)
    D.badCnt[p] = (uint8_t)nb;
    return w | (k << 27);
}

// the pixel's colour and (LOBSTER) its LBSP taps
template <int C, int ALG>
__device__ __forceinline__ void pixel_inputs(const LobDev& D, int p, uint32_t (&vals)[C][4], uint32_t (&curr)[C]) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
        if (ALG == ALG_LOBSTER) taps<C>(D.frame, D.W, p, c, vals[c]);
        curr[c] = __ldg(D.frame + (size_t)p * C + c);
    }
}

// warp-aggregated count of a per-thread value into a 64-bit counter
__device__ __forceinline__ void warp_add(unsigned long long* ctr, unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(ctr, v);
}

// list push with per-round dedupe; the lanes that push together share one counter atomic
__device__ __forceinline__ void push(const LobDev& D, uint32_t* list, unsigned int* count, uint32_t stamp, int t) {
    if (atomicExch(&D.stamp[t], stamp) == stamp) return;
    const unsigned am = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(am) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(am));
    base = __shfl_sync(am, base, leader);
    const unsigned int i = base + (unsigned int)__popc(am & ((1u << lane) - 1u));
    if (i < D.listCap) list[i] = (uint32_t)t;
    else atomicOr(&D.flags[LOB_F_ERR], 1u);
}

}  // namespace

// 1. every ROI pixel (ViBe: every pixel) against the frame-start samples
template <int C, int ALG>
__global__ void __launch_bounds__(kThreadsL) lob_k_eval(LobDev D) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long scanned = 0;
    if (p < D.npx) {
        if (ALG == ALG_LOBSTER && !D.roi[p]) {
            D.intent[p] = 0u;
        } else {
            const int x = p % D.W, y = p / D.W;
            uint32_t vals[C][4], curr[C];
            pixel_inputs<C, ALG>(D, p, vals, curr);
            // the sample word this pixel writes: LOBSTER, its descriptors (:499-500 / :548-550) and colour;
            // ViBe, its colour; PBAS, its colour and gradient (also what a neighbour update writes into it)
            unsigned long long wd = 0;
            LobOvr none;
            none.n = 0;
            none.mask = 0;
            if (ALG == ALG_PBAS) {
                uint32_t g[C];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    g[c] = __ldg(D.grad + (size_t)p * C + c);
                    wd |= ((unsigned long long)curr[c] << (8 * c)) | ((unsigned long long)g[c] << (24 + 8 * c));
                }
                D.wD[p] = wd;
                D.intent[p] = pbas_eval_px<C, false>(D, p, x, y, curr, g, none, &scanned);
            } else {
                if (ALG == ALG_VIBE) {
#pragma unroll
                    for (int c = 0; c < C; ++c) wd |= (unsigned long long)curr[c] << (8 * c);
                } else {
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        wd |= (unsigned long long)lbsp_thr(vals[c], curr[c], __ldg(D.lut + curr[c])) << (16 * c);
                    if (C == 3) wd |= ((unsigned long long)curr[0] << 48) | ((unsigned long long)curr[1] << 56);
                }
                D.wD[p] = wd;
                D.intent[p] = eval_px<C, ALG, false>(D, p, x, y, vals, curr, none, &scanned);
            }
        }
    }
    warp_add(&D.stats[0], scanned);
}

// 2. the pixels whose scan read a sample that an earlier neighbour writes
__global__ void __launch_bounds__(kThreadsL) lob_k_mark(LobDev D) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.npx) return;
    const uint32_t w = D.intent[p];
    if (!(w & kIValid)) return;
    const int x = p % D.W, y = p / D.W, e = i_e(w);
    bool dirty = false;
    // earlier pixels within one step: the row above, then the left neighbour
    const int q4[4] = {p - D.W - 1, p - D.W, p - D.W + 1, p - 1};
    const bool ok4[4] = {y > 0 && x > 0, y > 0, y > 0 && x + 1 < D.W, x > 0};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!ok4[i]) continue;
        const uint32_t wq = D.intent[q4[i]];
        if ((wq & kIValid) && (wq & kINb) && nb_target(wq, q4[i], D.W) == p && i_snb(wq) < e) dirty = true;
    }
    if (dirty) push(D, D.list0, &D.flags[LOB_F_COUNT0], D.stampBase, p);
}

// 3. one repair round: re-evaluates the pixels of list (round & 1) with the samples their earlier
// neighbours write now, and lists the later pixels whose incoming writes changed
template <int C, int ALG>
__global__ void __launch_bounds__(kThreadsL) lob_k_round(LobDev D, int round) {
    if (ld_vol(&D.flags[LOB_F_CONV])) return;
    const int cur = round & 1;
    const unsigned int n0 = ld_vol(&D.flags[cur]);
    const unsigned int n = n0 < D.listCap ? n0 : D.listCap;
    const uint32_t* in = cur ? D.list1 : D.list0;
    uint32_t* out = cur ? D.list0 : D.list1;
    unsigned int* outCount = &D.flags[cur ^ 1];
    const uint32_t stamp = D.stampBase + (uint32_t)round + 1u;
    unsigned long long scanned = 0;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = (int)__ldcg(in + i);
        const int x = p % D.W, y = p / D.W;
        LobOvr ov;
        ov.n = 0;
        ov.mask = 0;
        const int q4[4] = {p - D.W - 1, p - D.W, p - D.W + 1, p - 1};
        const bool ok4[4] = {y > 0 && x > 0, y > 0, y > 0 && x + 1 < D.W, x > 0};
        for (int j = 0; j < 4; ++j) {
            if (!ok4[j]) continue;
            const uint32_t wq = ld_vol(&D.intent[q4[j]]);
            if ((wq & kIValid) && (wq & kINb) && nb_target(wq, q4[j], D.W) == p) {
                const int s = i_snb(wq);
                ov.s[ov.n] = s;
                ov.d[ov.n] = __ldcg(D.wD + q4[j]);
                ov.c[ov.n] = ALG != ALG_LOBSTER ? 0u : __ldg(D.frame + (size_t)q4[j] * C + (C == 3 ? 2 : 0));
                ++ov.n;
                ov.mask |= 1ull << s;
            }
        }
        uint32_t vals[C][4], curr[C];
        pixel_inputs<C, ALG>(D, p, vals, curr);
        uint32_t wNew;
        if (ALG == ALG_PBAS) {
            // self diffusion: a sample that an earlier neighbour writes holds the pixel's own values
            uint32_t g[C];
#pragma unroll
            for (int c = 0; c < C; ++c) g[c] = __ldg(D.grad + (size_t)p * C + c);
            ov.d[0] = __ldcg(D.wD + p);
            wNew = pbas_eval_px<C, true>(D, p, x, y, curr, g, ov, &scanned);
        } else {
            wNew = eval_px<C, ALG, true>(D, p, x, y, vals, curr, ov, &scanned);
        }
        const uint32_t wOld = ld_vol(&D.intent[p]);
        if (wNew == wOld) continue;
        *(volatile uint32_t*)&D.intent[p] = wNew;
        if (i_nbpart(wNew) == i_nbpart(wOld)) continue;
        // the targets of the old and the new neighbour write that come later in raster order
        if (wOld & kINb) {
            const int t = nb_target(wOld, p, D.W);
            if (t > p) push(D, out, outCount, stamp, t);
        }
        if (wNew & kINb) {
            const int t = nb_target(wNew, p, D.W);
            if (t > p) push(D, out, outCount, stamp, t);
        }
    }
    warp_add(&D.stats[0], scanned);
}

// end of repair round `round`: converged when the round listed nothing; otherwise its input list
// becomes the next round's output
__global__ void lob_k_round_end(LobDev D, int round) {
    if (D.flags[LOB_F_CONV]) return;
    const int cur = round & 1;
    const unsigned int next = D.flags[cur ^ 1];
    D.flags[LOB_F_ROUNDS] = (unsigned int)round + 1u;
    if (next > D.listCap) {
        D.flags[LOB_F_ERR] |= 1u;
        D.flags[LOB_F_CONV] = 1u;
    } else if (next == 0u) {
        D.flags[LOB_F_CONV] = 1u;
    } else {
        D.flags[cur] = 0u;
    }
}

// 4. every pixel gathers the sample writes aimed at it, in raster order of the writers (own update
// before neighbour update within a writer); the raw mask (ViBe: the output, :84 / :176) and the draw
// counters of the frame
template <int C, int ALG>
__global__ void __launch_bounds__(kThreadsL) lob_k_commit(LobDev D) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long writes = 0;
    if (p < D.npx) {
        const uint32_t wp = D.intent[p];
        const bool valid = (wp & kIValid) != 0;
        const uint8_t raw = (valid && (wp & kIFG)) ? 255 : 0;
        if (ALG == ALG_VIBE) D.maskOut[p] = raw;
        else D.rawFG[p] = raw;
        // PBAS: every write into pixel p holds p's own colour and gradient
        const unsigned long long wOwn = ALG == ALG_PBAS ? D.wD[p] : 0ull;
        D.kctr[p] = (uint16_t)(valid ? i_draws(wp) : 0);
        if (valid) writes = ((wp & kIOwn) ? 1ull : 0ull) + ((wp & kINb) ? 1ull : 0ull);
        const int x = p % D.W, y = p / D.W;
        // the pixels a write can reach: inside the LBSP border (LOBSTER), the whole frame (ViBe, PBAS)
        constexpr int bord = ALG == ALG_LOBSTER ? kBorder : 0;
        if (x >= bord && y >= bord && x < D.W - bord && y < D.H - bord) {
            int ns = 0;
            int ss[10], sq[10];
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    if (y + dy < 0 || y + dy >= D.H || x + dx < 0 || x + dx >= D.W) continue;
                    const int q = p + dy * D.W + dx;
                    const uint32_t wq = D.intent[q];
                    if (!(wq & kIValid)) continue;
                    int sv[2], nv = 0;
                    if (q == p && (wq & kIOwn)) sv[nv++] = i_sown(wq);
                    if ((wq & kINb) && nb_target(wq, q, D.W) == p) sv[nv++] = i_snb(wq);
                    for (int v = 0; v < nv; ++v) {
                        int k = 0;
                        while (k < ns && ss[k] != sv[v]) ++k;
                        ss[k] = sv[v];
                        sq[k] = q;
                        if (k == ns) ++ns;
                    }
                }
            for (int k = 0; k < ns; ++k) {
                const size_t o = (size_t)ss[k] * D.npx + p;
                const int q = sq[k];
                if (ALG == ALG_PBAS) {
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        D.sC[o * C + c] = (uint8_t)(wOwn >> (8 * c));
                        D.sG[o * C + c] = (uint8_t)(wOwn >> (24 + 8 * c));
                    }
                } else if (ALG == ALG_VIBE) {
                    const unsigned long long wq = D.wD[q];
#pragma unroll
                    for (int c = 0; c < C; ++c) D.sC[o * C + c] = (uint8_t)(wq >> (8 * c));
                } else {
                    if (C == 3) ((unsigned long long*)D.sD)[o] = D.wD[q];
                    else ((uint16_t*)D.sD)[o] = (uint16_t)D.wD[q];
                    D.sC[o] = __ldg(D.frame + (size_t)q * C + (C == 3 ? 2 : 0));
                }
            }
        }
    }
    warp_add(&D.stats[1], writes);
}

// cv::medianBlur(raw mask, k) with replicated borders: 255 where more than half of the k*k window is
// set (:577), which becomes the last mask and the output (:578); the frame becomes the last colour
// frame (:580). One block per kMedTile x kMedTile tile: the raw mask with its clamped halo in shared
// memory, the row-window counts, then the column sums of those.
constexpr int kMedTile = 32, kMedMaxR = 15, kMedS = kMedTile + 2 * kMedMaxR;
template <int C, bool KEEP>
__global__ void __launch_bounds__(kThreadsL) lob_k_median(LobDev D) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    __shared__ uint8_t raw[kMedS][kMedS];
    __shared__ uint8_t rows[kMedS][kMedTile];
    const int r = D.medianK / 2, span = kMedTile + 2 * r;
    const int x0 = blockIdx.x * kMedTile, y0 = blockIdx.y * kMedTile, t = threadIdx.x;
    for (int i = t; i < span * span; i += blockDim.x) {
        const int ty = i / span, tx = i % span;
        const int gy = clampi(y0 - r + ty, 0, D.H - 1), gx = clampi(x0 - r + tx, 0, D.W - 1);
        raw[ty][tx] = D.rawFG[(size_t)gy * D.W + gx] != 0;
    }
    __syncthreads();
    for (int i = t; i < span * kMedTile; i += blockDim.x) {
        const int ty = i / kMedTile, tx = i % kMedTile;
        int c = 0;
        for (int d = 0; d <= 2 * r; ++d) c += raw[ty][tx + d];
        rows[ty][tx] = (uint8_t)c;
    }
    __syncthreads();
    for (int i = t; i < kMedTile * kMedTile; i += blockDim.x) {
        const int ty = i / kMedTile, tx = i % kMedTile;
        const int x = x0 + tx, y = y0 + ty;
        if (x >= D.W || y >= D.H) continue;
        int cnt = 0;
        for (int d = 0; d <= 2 * r; ++d) cnt += rows[ty + d][tx];
        const size_t p = (size_t)y * D.W + x;
        const uint8_t m = (2 * cnt > D.medianK * D.medianK) ? 255 : 0;
        D.maskOut[p] = m;
        if (!KEEP) continue;  // PBAS keeps neither
        D.lastFG[p] = m;
#pragma unroll
        for (int c = 0; c < C; ++c) D.lastColor[p * C + c] = __ldg(D.frame + p * C + c);
    }
}

// initialize() (:442-457 with BackgroundSubtractionUtils.cpp:70-155, BackgroundSubtractorLBSP.cpp:21-65):
// last colour frame = the ROI part of the frame, last descriptors of the strict interior ROI pixels
template <int C>
__global__ void __launch_bounds__(kThreadsL) lob_k_init(LobDev D, const uint8_t* img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.npx) return;
    const int x = p % D.W, y = p / D.W;
    const bool in = D.roi[p] != 0;
    const bool desc = in && x > kBorder && y > kBorder && x < D.W - kBorder && y < D.H - kBorder;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const uint32_t v = __ldg(img + (size_t)p * C + c);
        D.lastColor[(size_t)p * C + c] = in ? (uint8_t)v : 0;
        uint16_t d = 0;
        if (desc) {
            uint32_t t[4];
            taps<C>(img, D.W, p, c, t);
            d = (uint16_t)lbsp_thr(t, v, __ldg(D.lut + v));
        }
        D.lastDesc[(size_t)p * C + c] = d;
    }
    D.lastFG[p] = 0;
    D.kctr[p] = 0;
}

// ViBe's initialize() (BackgroundSubtractorViBe.cpp:57-75 / :112-134): sample s of every pixel from a
// 7x7 Gaussian position of the frame clamped to the frame (draw s of the pixel in frame 0)
template <int C>
__global__ void __launch_bounds__(kThreadsL) lob_k_vibe_init(LobDev D, const uint8_t* img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.npx) return;
    const int x0 = p % D.W, y0 = p / D.W;
    Draws ds;
    ds.blk = 0xffffffffu;
    for (int s = 0; s < D.N; ++s) {
        int r = 1 + (int)(draw(D, (uint32_t)p, (uint32_t)s, ds) % 512u);
        int sx = 0, sy = 0;
        for (int i = 0; i < 49; ++i) {
            r -= c_lob_pat7[i];
            if (r <= 0) {
                sy = i / 7;
                sx = i % 7;
                break;
            }
        }
        sx = clampi(sx + x0 - 3, 0, D.W - 1);
        sy = clampi(sy + y0 - 3, 0, D.H - 1);
        const uint8_t* src = img + ((size_t)sy * D.W + sx) * C;
        uint8_t* dst = D.sC + ((size_t)s * D.npx + p) * C;
#pragma unroll
        for (int c = 0; c < C; ++c) dst[c] = __ldg(src + c);
    }
}

// ---- PBAS (BackgroundSubtractorPBAS.cpp) ----

__device__ __forceinline__ int reflect101(int i, int n) {
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
    return i;
}

// the gradient image of a frame (:127-135 / :338-346), first pass: GaussianBlur 3x3 (sigma 0), the
// separable [1 2 1] / 4 kernel in 8-bit fixed point, (sum + 8) >> 4, with BORDER_REFLECT_101
template <int C>
__global__ void __launch_bounds__(kThreadsL) pbas_k_blur(LobDev D, const uint8_t* img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.npx * C) return;
    const int p = i / C, c = i % C, x = p % D.W, y = p / D.W;
    const int xs[3] = {reflect101(x - 1, D.W), x, reflect101(x + 1, D.W)};
    const int ys[3] = {reflect101(y - 1, D.H), y, reflect101(y + 1, D.H)};
    int acc = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const uint8_t* row = img + (size_t)ys[j] * D.W * C + c;
        const int r = __ldg(row + xs[0] * C) + 2 * __ldg(row + xs[1] * C) + __ldg(row + xs[2] * C);
        acc += (j == 1 ? 2 : 1) * r;
    }
    D.blur[i] = (uint8_t)((acc + 8) >> 4);
}

// second pass: the Scharr derivatives ([-3 0 3; -10 0 10; -3 0 3] and its transpose, int16, no
// overflow at these magnitudes), convertScaleAbs (|v| saturated to 255) and addWeighted(0.5, 0.5)
// ((a + b) * 0.5 rounded half to even), BORDER_REFLECT_101
template <int C>
__global__ void __launch_bounds__(kThreadsL) pbas_k_grad(LobDev D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.npx * C) return;
    const int p = i / C, c = i % C, x = p % D.W, y = p / D.W;
    const int xs[3] = {reflect101(x - 1, D.W), x, reflect101(x + 1, D.W)};
    const int ys[3] = {reflect101(y - 1, D.H), y, reflect101(y + 1, D.H)};
    int v[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) v[j][k] = __ldg(D.blur + ((size_t)ys[j] * D.W + xs[k]) * C + c);
    const int gx = 3 * (v[0][2] - v[0][0]) + 10 * (v[1][2] - v[1][0]) + 3 * (v[2][2] - v[2][0]);
    const int gy = 3 * (v[2][0] - v[0][0]) + 10 * (v[2][1] - v[0][1]) + 3 * (v[2][2] - v[0][2]);
    const int ax = min(abs(gx), 255), ay = min(abs(gy), 255);
    const int sum = ax + ay;
    D.grad[i] = (uint8_t)((sum >> 1) + ((sum & 1) & ((sum >> 1) & 1)));
}

// PBAS's initialize() (:61-109 / :287-324): R = 1, T = the default update rate, D = 0 in the maps of
// parity 0, the mean gradient distance mean0 (20, or the last one), and sample s of every pixel (colour and gradient) from a 7x7
// Gaussian position of the frame clamped to the frame (draw s of the pixel in frame 0)
template <int C>
__global__ void __launch_bounds__(kThreadsL) pbas_k_init(LobDev D, const uint8_t* img, float mean0) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.npx) return;
    const size_t npx = (size_t)D.npx;
    D.fm[p] = 1.0f;
    D.fm[npx + p] = D.updateRate;
    D.fm[2 * npx + p] = 0.0f;
    if (p == 0) *D.meanGrad = mean0;
    const int x0 = p % D.W, y0 = p / D.W;
    Draws ds;
    ds.blk = 0xffffffffu;
    for (int s = 0; s < D.N; ++s) {
        int r = 1 + (int)(draw(D, (uint32_t)p, (uint32_t)s, ds) % 512u);
        int sx = 0, sy = 0;
        for (int i = 0; i < 49; ++i) {
            r -= c_lob_pat7[i];
            if (r <= 0) {
                sy = i / 7;
                sx = i % 7;
                break;
            }
        }
        sx = clampi(sx + x0 - 3, 0, D.W - 1);
        sy = clampi(sy + y0 - 3, 0, D.H - 1);
        const size_t src = ((size_t)sy * D.W + sx) * C, dst = ((size_t)s * npx + p) * C;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            D.sC[dst + c] = __ldg(img + src + c);
            D.sG[dst + c] = D.grad[src + c];
        }
    }
}

// the frame-level mean gradient distance of the bad samples, single channel (:232): the size_t sum
// of their gradient distances and their count (which starts at 1), per block into two counters
__global__ void __launch_bounds__(kThreadsL) pbas_k_mean1(LobDev D) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    unsigned long long sum = 0, cnt = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        sum += D.badSum[p];
        cnt += D.badCnt[p];
    }
    warp_add(&D.stats[2], sum);
    warp_add(&D.stats[3], cnt);
}
__global__ void pbas_k_mean1_end(LobDev D) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    const float mean = (float)D.stats[2] / (float)(D.stats[3] + 1ull);
    *D.meanGrad = mean > 20.0f ? mean : 20.0f;
}

// three channels (:460): the float sum of the bad samples' gradient distances in raster order (pixel,
// then scan order), s <- RN(s + v) value after value. The values are non-negative, so s only grows, and
// while s stays in one binade [2^e, 2^(e+1)) with ulp u = 2^(e-23), RN(s + v) = s + u * q where q is
// v / u rounded to an integer: up when the fraction is above 1/2, down when below, and on an exact 1/2
// to the even quotient, which depends on the parity of s / u. The sum over a chunk of values is
// therefore a function of that parity only: a transfer (d0, d1), the increment in ulps for an even or
// odd start, composed value by value (d'_p = d_p + d2_{(p + d_p) & 1}).
//   pbas_k_sum_chunks: the count of bad samples, and each chunk's total in double precision;
//   pbas_k_sum_scan: their exclusive prefix, which predicts the binade of s at each chunk's start;
//   pbas_k_sum_tr: each chunk's transfers for the predicted binade and the two beside it;
//   pbas_k_sum_walk: from s = 0, chunk after chunk, applies the chunk's transfer when s is at least 1024,
//     its binade is one of the chunk's three and the chunk cannot leave it (s / u + increment + 1 < 2^24:
//     no value of the chunk reaches the next binade), and otherwise adds the chunk's values one by one.
// The result is the sequential sum bit for bit; only the first chunks, those where s crosses a power of
// two and those whose binade was mispredicted are summed value by value.
constexpr int kSumChunk = 256, kSumNB = 3, kSumEMin = 10, kSumScan = 1024;
struct Tr {
    unsigned long long d0, d1;
};
__device__ __forceinline__ Tr tr_then(Tr a, Tr b) {
    Tr r;
    r.d0 = a.d0 + ((a.d0 & 1ull) ? b.d1 : b.d0);
    r.d1 = a.d1 + ((a.d1 & 1ull) ? b.d0 : b.d1);
    return r;
}
// one value v >= 0 in binade e: its increment in ulps for an even / odd s / u
__device__ __forceinline__ Tr tr_value(float v, int e) {
    const float x = v * __int_as_float((127 + 23 - e) << 23);  // v / u, exact (a power of two)
    const float a = floorf(x), r = x - a;
    const unsigned long long ai = (unsigned long long)a;
    Tr t;
    if (r > 0.5f) t.d0 = t.d1 = ai + 1ull;
    else if (r < 0.5f) t.d0 = t.d1 = ai;
    else {
        t.d0 = ai + (ai & 1ull);  // even s/u: s/u + a is even when a is
        t.d1 = ai + ((ai + 1ull) & 1ull);
    }
    return t;
}
__device__ __forceinline__ Tr tr_shfl_down(Tr t, int o) {
    Tr r;
    r.d0 = __shfl_down_sync(0xffffffffu, t.d0, o);
    r.d1 = __shfl_down_sync(0xffffffffu, t.d1, o);
    return r;
}
// binade of a positive float
__device__ __forceinline__ int binade(float s) { return (int)((__float_as_uint(s) >> 23) & 0xffu) - 127; }

struct SumWork {
    double* chunkSum;  // [nChunks], then their exclusive prefix
    Tr* tr;            // [nChunks][kSumNB]
    Tr* trw;           // [nChunks][kSumChunk / 32][kSumNB]: the transfers of each chunk's 32-pixel granules
    int* eb;           // [nChunks]: the first of the chunk's binades
};
constexpr int kSumGran = kSumChunk / 32;

__global__ void __launch_bounds__(kSumChunk) pbas_k_sum_chunks(LobDev D, SumWork W) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    __shared__ double sm[kSumChunk / 32];
    const int t = threadIdx.x, p = blockIdx.x * kSumChunk + t;
    const int n = p < D.npx ? (int)D.badCnt[p] : 0;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) acc += (double)__ldg(D.badVals + (size_t)p * D.N + k);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((t & 31) == 0) sm[t >> 5] = acc;
    __syncthreads();
    if (t == 0) {
        double c = 0.0;
        for (int w = 0; w < kSumChunk / 32; ++w) c += sm[w];
        W.chunkSum[blockIdx.x] = c;
    }
    warp_add(&D.stats[3], (unsigned long long)n);
}

__global__ void __launch_bounds__(kSumScan) pbas_k_sum_scan(LobDev D, SumWork W, int nChunks) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    __shared__ double sm[kSumScan];
    const int t = threadIdx.x, per = (nChunks + kSumScan - 1) / kSumScan;
    const int c0 = min(t * per, nChunks), c1 = min(c0 + per, nChunks);
    double own = 0.0;
    for (int c = c0; c < c1; ++c) own += W.chunkSum[c];
    sm[t] = own;
    __syncthreads();
    for (int o = 1; o < kSumScan; o <<= 1) {
        const double v = t >= o ? sm[t - o] : 0.0;
        __syncthreads();
        sm[t] += v;
        __syncthreads();
    }
    double run = sm[t] - own;
    for (int c = c0; c < c1; ++c) {
        const double v = W.chunkSum[c];
        W.chunkSum[c] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kSumChunk) pbas_k_sum_tr(LobDev D, SumWork W) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    __shared__ Tr sm[kSumChunk / 32][kSumNB];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int p = blockIdx.x * kSumChunk + t;
    const int n = p < D.npx ? (int)D.badCnt[p] : 0;
    const float* v = D.badVals + (size_t)(p < D.npx ? p : 0) * D.N;
    const float pre = (float)W.chunkSum[blockIdx.x];
    const int e0 = max(pre >= 1.0f ? binade(pre) - 1 : kSumEMin, kSumEMin);
    Tr acc[kSumNB];
#pragma unroll
    for (int j = 0; j < kSumNB; ++j) acc[j].d0 = acc[j].d1 = 0ull;
    for (int k = 0; k < n; ++k) {
        const float x = __ldg(v + k);
#pragma unroll
        for (int j = 0; j < kSumNB; ++j) acc[j] = tr_then(acc[j], tr_value(x, e0 + j));
    }
    // ordered reduction: lane 0 of each warp, then the warps in order
#pragma unroll
    for (int j = 0; j < kSumNB; ++j) {
        for (int o = 1; o < 32; o <<= 1) {
            const Tr y = tr_shfl_down(acc[j], o);
            if ((lane & (2 * o - 1)) == 0) acc[j] = tr_then(acc[j], y);
        }
        if (lane == 0) {
            sm[wid][j] = acc[j];
            W.trw[((size_t)blockIdx.x * kSumGran + wid) * kSumNB + j] = acc[j];
        }
    }
    __syncthreads();
    if (t < kSumNB) {
        Tr r = sm[0][t];
        for (int w = 1; w < kSumChunk / 32; ++w) r = tr_then(r, sm[w][t]);
        W.tr[(size_t)blockIdx.x * kSumNB + t] = r;
        if (t == 0) W.eb[blockIdx.x] = e0;
    }
}

// s advanced by a transfer when s >= 1024 and the transfer keeps s in its binade; false otherwise
__device__ __forceinline__ bool tr_apply(float& s, Tr t) {
    if (s < 1024.0f) return false;
    const unsigned int bits = __float_as_uint(s);
    const unsigned long long m = (unsigned long long)((bits & 0x7fffffu) | 0x800000u);
    const unsigned long long m2 = m + ((m & 1ull) ? t.d1 : t.d0);
    if (m2 + 1ull >= (1ull << 24)) return false;
    s = __uint_as_float((bits & 0xff800000u) | ((unsigned int)m2 & 0x7fffffu));
    return true;
}

// the walk over the chunks (one warp; every lane holds the same sum), then the mean and its floor of 20:
// 32 chunks at once when all of them have transfers for the binade of s (their ordered composition),
// else chunk by chunk, else 32-pixel granule by granule, else value by value
__global__ void __launch_bounds__(32) pbas_k_sum_walk(LobDev D, SumWork W, int nChunks) {
    if (!ld_vol(&D.flags[LOB_F_CONV])) return;
    __shared__ float vals[32 * 64];
    const int lane = threadIdx.x;
    float s = 0.0f;
    for (int c0 = 0; c0 < nChunks; c0 += 32) {
        // the window's transfers, one chunk per lane
        Tr tw[kSumNB];
        int ew = 0;
        const bool in = c0 + lane < nChunks;
#pragma unroll
        for (int i = 0; i < kSumNB; ++i) tw[i].d0 = tw[i].d1 = 0ull;
        if (in) {
#pragma unroll
            for (int i = 0; i < kSumNB; ++i) tw[i] = W.tr[(size_t)(c0 + lane) * kSumNB + i];
            ew = W.eb[c0 + lane];
        }
        {
            const int k = binade(s) - ew;
            Tr t;
            t.d0 = t.d1 = 0ull;
#pragma unroll
            for (int i = 0; i < kSumNB; ++i)
                if (k == i) t = tw[i];
            if (__all_sync(0xffffffffu, !in || (k >= 0 && k < kSumNB))) {
                for (int o = 1; o < 32; o <<= 1) {
                    const Tr y = tr_shfl_down(t, o);
                    if ((lane & (2 * o - 1)) == 0) t = tr_then(t, y);
                }
                Tr tot;
                tot.d0 = __shfl_sync(0xffffffffu, t.d0, 0);
                tot.d1 = __shfl_sync(0xffffffffu, t.d1, 0);
                if (tr_apply(s, tot)) continue;
            }
        }
        for (int j = 0; j < 32 && c0 + j < nChunks; ++j) {
            const int c = c0 + j;
            const int eb = __shfl_sync(0xffffffffu, ew, j);
            int k = binade(s) - eb;
            Tr tc;
            tc.d0 = tc.d1 = 0ull;
#pragma unroll
            for (int i = 0; i < kSumNB; ++i) {
                const unsigned long long a = __shfl_sync(0xffffffffu, tw[i].d0, j);
                const unsigned long long b = __shfl_sync(0xffffffffu, tw[i].d1, j);
                if (k == i) {
                    tc.d0 = a;
                    tc.d1 = b;
                }
            }
            if (k >= 0 && k < kSumNB && tr_apply(s, tc)) continue;
            const int pEnd = min((c + 1) * kSumChunk, D.npx);
            for (int g = 0; g < kSumGran; ++g) {
                const int pg = c * kSumChunk + g * 32;
                if (pg >= pEnd) break;
                k = binade(s) - eb;
                if (k >= 0 && k < kSumNB && tr_apply(s, W.trw[((size_t)c * kSumGran + g) * kSumNB + k])) continue;
                // value by value, the granule's values staged in shared memory, every lane adding them in order
                const int p = pg + lane;
                const int n = p < pEnd ? (int)D.badCnt[p] : 0;
                int off = n;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, off, o);
                    if (lane >= o) off += y;
                }
                const int total = __shfl_sync(0xffffffffu, off, 31);
                off -= n;
                for (int q = 0; q < n; ++q) vals[off + q] = D.badVals[(size_t)p * D.N + q];
                __syncwarp();
                for (int q = 0; q < total; ++q) s += vals[q];
                __syncwarp();
            }
        }
    }
    if (lane == 0) {
        const float mean = s / (float)(D.stats[3] + 1ull);
        *D.meanGrad = mean > 20.0f ? mean : 20.0f;
    }
}

// refreshModel(frac, force) (:410-440): samples [start, start+nref) of every ROI pixel (not in the last
// foreground unless forced) from a 7x7 Gaussian position of the last colour frame, with its descriptor,
// which also goes to the last descriptor frame (:427-433); the draws continue the frame's counters
template <int C>
__global__ void __launch_bounds__(kThreadsL) lob_k_refresh(LobDev D, int start, int nref, int force) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= D.npx || !D.roi[p]) return;
    if (!force && D.lastFG[p]) return;
    const int x0 = p % D.W, y0 = p / D.W;
    uint32_t k = D.kctr[p];
    Draws ds;
    ds.blk = 0xffffffffu;
    for (int s = start; s < start + nref; ++s) {
        int r = 1 + (int)(draw(D, (uint32_t)p, k++, ds) % 512u);
        int sx = 0, sy = 0;
        for (int i = 0; i < 49; ++i) {
            r -= c_lob_pat7[i];
            if (r <= 0) {
                sy = i / 7;
                sx = i % 7;
                break;
            }
        }
        sx = clampi(sx + x0 - 3, kBorder, D.W - kBorder - 1);
        sy = clampi(sy + y0 - 3, kBorder, D.H - kBorder - 1);
        const int sp = sy * D.W + sx;
        if (!force && D.lastFG[sp]) continue;
        const int rs = s % D.N;
        unsigned long long wd = 0;
        uint32_t col[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            col[c] = D.lastColor[(size_t)sp * C + c];
            uint32_t t[4];
            taps<C>(D.lastColor, D.W, sp, c, t);
            const uint16_t d = (uint16_t)lbsp_thr(t, col[c], __ldg(D.lut + col[c]));
            D.lastDesc[(size_t)sp * C + c] = d;
            wd |= (unsigned long long)d << (16 * c);
        }
        const size_t o = (size_t)rs * D.npx + p;
        if (C == 3) {
            ((unsigned long long*)D.sD)[o] = wd | ((unsigned long long)col[0] << 48) | ((unsigned long long)col[1] << 56);
            D.sC[o] = (uint8_t)col[2];
        } else {
            ((uint16_t*)D.sD)[o] = (uint16_t)wd;
            D.sC[o] = (uint8_t)col[0];
        }
    }
    D.kctr[p] = (uint16_t)k;
}

// getBackgroundImage / getBackgroundDescriptorsImage (:583-620): per channel the float sum of
// sample / N in sample order, converted with rounding and saturation
template <int C>
__global__ void lob_k_background(LobDev D, void* out, int descriptors) {
    const size_t n = (size_t)D.npx * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / C), c = (int)(i % C);
        float acc = 0.0f;
        for (int s = 0; s < D.N; ++s) {
            const size_t o = (size_t)s * D.npx + p;
            uint32_t v;
            if (D.alg != ALG_LOBSTER) {
                v = D.sC[o * C + c];
            } else if (descriptors) {
                v = C == 3 ? (uint32_t)(((const unsigned long long*)D.sD)[o] >> (16 * c)) & 0xffffu
                           : ((const uint16_t*)D.sD)[o];
            } else if (C == 3 && c < 2) {
                v = (uint32_t)(((const unsigned long long*)D.sD)[o] >> (48 + 8 * c)) & 0xffu;
            } else {
                v = D.sC[o];
            }
            acc += (float)v / (float)D.N;
        }
        const int r = __float2int_rn(acc);
        if (descriptors) ((uint16_t*)out)[i] = (uint16_t)clampi(r, 0, 65535);
        else ((uint8_t*)out)[i] = (uint8_t)clampi(r, 0, 255);
    }
}

// the sample planes in the reference's layout ([N][H*W*C] colours or descriptors)
template <int C>
__global__ void lob_k_export_samples(LobDev D, void* out, int descriptors) {
    const size_t n = (size_t)D.N * D.npx * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t sp = i / C;
        const int c = (int)(i % C);
        if (descriptors) {
            ((uint16_t*)out)[i] = C == 3 ? (uint16_t)(((const unsigned long long*)D.sD)[sp] >> (16 * c))
                                         : ((const uint16_t*)D.sD)[sp];
        } else {
            ((uint8_t*)out)[i] = (C == 3 && c < 2) ? (uint8_t)(((const unsigned long long*)D.sD)[sp] >> (48 + 8 * c))
                                                   : D.sC[sp];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------------
namespace {

inline size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

inline uint8_t sat_round_u8f(float v) {
    const float r = std::nearbyint(v);
    return (uint8_t)(r < 0.f ? 0.f : r > 255.f ? 255.f : r);
}

#define LOB_CUDA(call, what)                                                      \
    do {                                                                          \
        const cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string(what) + ": " + cudaGetErrorString(e_);              \
            return e_ == cudaErrorMemoryAllocation ? LVBGS_OOM : LVBGS_DEVICE_ERROR; \
        }                                                                         \
    } while (0)

inline int blocks_for(size_t n) { return (int)((n + kThreadsL - 1) / kThreadsL); }

}  // namespace

void lob_release(LobState& L) {
    if (L.meanDone) cudaEventSynchronize(L.meanDone);
    if (L.done) cudaEventDestroy(L.done);
    if (L.meanDone) cudaEventDestroy(L.meanDone);
    L.done = L.meanDone = nullptr;
    cudaFree(L.mem);
    L.mem = nullptr;
    L.bytes = 0;
    if (L.h_flags) cudaFreeHost(L.h_flags);
    L.h_flags = nullptr;
}

lvbgs_status lob_setup(LobState& L, int alg, const lvbgs_params& prm, int W, int H, int C,
                       const std::vector<uint8_t>& roi, size_t orig, size_t fin, cudaStream_t st, std::string& err) {
    // PBAS keeps its former mean gradient distance when initialized again (it is set by the
    // constructor only, BackgroundSubtractorPBAS.cpp:29)
    if (L.mem && L.d.alg == ALG_PBAS && L.d.meanGrad) {
        LOB_CUDA(cudaEventSynchronize(L.meanDone), "frame step");
        LOB_CUDA(cudaMemcpy(&L.pbasMean, L.d.meanGrad, sizeof(float), cudaMemcpyDeviceToHost), "state read-back");
    }
    cudaFree(L.mem);
    L.mem = nullptr;
    const size_t npx = (size_t)W * H, N = prm.bg_samples;
    // ViBe keeps only colour samples ([N][npx*C] bytes); PBAS colour and gradient samples and its maps;
    // LOBSTER the packed descriptor plane and a colour byte
    const bool vibe = alg != ALG_LOBSTER, pbas = alg == ALG_PBAS;
    const size_t lob = vibe ? 0 : 1, pb = pbas ? 1 : 0;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += al(bytes);
        return o;
    };
    const size_t oRoi = take(npx), oLastColor = take(lob * npx * C), oLastFG = take(lob * npx),
                 oRawFG = take(lob * npx), oLut = take(256), oLastDesc = take(lob * npx * C * 2), oKctr = take(npx * 2),
                 oSD = take(lob * N * npx * (C == 3 ? 8 : 2)), oSC = take(vibe ? N * npx * C : N * npx),
                 oIntent = take(npx * 4),
                 oWD = take(npx * 8), oList0 = take(npx * 4), oList1 = take(npx * 4), oStamp = take(npx * 4),
                 oFlags = take(LOB_F_WORDS * 4), oStats = take(32), oFrame = take(npx * C), oMask = take(npx),
                 oSG = take(pb * N * npx * C), oGrad = take(pb * npx * C), oBlur = take(pb * npx * C),
                 oFm = take(pb * 6 * npx * 4), oMean = take(pb * 4), oBadSum = take(pb * (C == 1 ? npx * 4 : 0)),
                 oBadCnt = take(pb * npx), oBadVals = take(pb * (C == 3 ? npx * N * 4 : 0)),
                 oSumTr = take(pb * (C == 3 ? (npx + kSumChunk - 1) / kSumChunk *
                                                  (sizeof(double) + (1 + kSumGran) * kSumNB * sizeof(Tr) + sizeof(int))
                                            : 0)),
                 oRawPb = take(pb * npx);
    LOB_CUDA(cudaMalloc(&L.mem, off), "model allocation");
    if (!L.h_flags) LOB_CUDA(cudaHostAlloc((void**)&L.h_flags, LOB_F_WORDS * 4, cudaHostAllocDefault), "pinned allocation");
    if (!L.done) LOB_CUDA(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming), "event creation");
    if (!L.meanDone) LOB_CUDA(cudaEventCreateWithFlags(&L.meanDone, cudaEventDisableTiming), "event creation");
    L.bytes = off;
    LobDev& D = L.d;
    D = LobDev{};
    D.alg = alg;
    D.W = W;
    D.H = H;
    D.C = C;
    D.N = (int)N;
    D.nreq = (int)prm.required_bg_samples;
    D.npx = (int)npx;
    D.descThr = (unsigned int)prm.desc_dist_threshold_offset;
    D.colThr = (unsigned int)prm.min_color_dist_threshold;
    D.seed = prm.seed;
    D.medianK = prm.default_median_blur_kernel_size;
    D.listCap = (unsigned int)npx;
    D.stampBase = 1;  // nonzero: the stamps start at 0
    uint8_t* b = L.mem;
    D.roi = b + oRoi;
    D.lastColor = b + oLastColor;
    D.lastFG = b + oLastFG;
    D.rawFG = b + oRawFG;
    D.lut = b + oLut;
    D.lastDesc = (uint16_t*)(b + oLastDesc);
    D.kctr = (uint16_t*)(b + oKctr);
    D.sD = b + oSD;
    D.sC = b + oSC;
    D.intent = (uint32_t*)(b + oIntent);
    D.wD = (unsigned long long*)(b + oWD);
    D.list0 = (uint32_t*)(b + oList0);
    D.list1 = (uint32_t*)(b + oList1);
    D.stamp = (uint32_t*)(b + oStamp);
    D.flags = (unsigned int*)(b + oFlags);
    D.stats = (unsigned long long*)(b + oStats);
    L.d_frame = b + oFrame;
    L.d_mask = b + oMask;
    if (pbas) {
        D.sG = b + oSG;
        D.grad = b + oGrad;
        D.blur = b + oBlur;
        D.fm = (float*)(b + oFm);
        D.meanGrad = (float*)(b + oMean);
        D.badSum = (uint32_t*)(b + oBadSum);
        D.badCnt = b + oBadCnt;
        D.badVals = (float*)(b + oBadVals);
        D.sumTr = b + oSumTr;
        D.rawFG = b + oRawPb;
        // the constructor's arguments (BackgroundSubtractorPBAS.cpp:21-32) and medianBlur(.., 9) (:266 / :494)
        D.R0 = (float)prm.min_color_dist_threshold;
        D.updateRate = prm.update_rate;
        D.medianK = 9;
        D.cur = 0;
    }
    L.ksent = 0;
    L.lastRounds = 1;
    L.frames = 0;
    L.n_rel = fin;
    L.orig_roi = orig;
    // BackgroundSubtractorLBSP.cpp:30-34 / :47-48: the LBSP threshold LUT (one channel divides by 3)
    uint8_t lut[256];
    const float rel = prm.rel_lbsp_threshold;
    for (int t = 0; t <= 255; ++t)
        lut[t] = C == 1 ? sat_round_u8f(((float)t * rel + (float)prm.lbsp_threshold_offset) / 3)
                        : sat_round_u8f((float)t * rel + (float)prm.lbsp_threshold_offset);
    LOB_CUDA(cudaMemsetAsync(L.mem, 0, off, st), "model reset");
    LOB_CUDA(cudaMemcpyAsync(D.roi, roi.data(), npx, cudaMemcpyHostToDevice, st), "roi upload");
    LOB_CUDA(cudaMemcpyAsync(D.lut, lut, 256, cudaMemcpyHostToDevice, st), "lut upload");
    return LVBGS_OK;
}

namespace {
// one kernel of the frame step for the stream's (channels, algorithm)
template <template <int, int> class K, typename... A>
void launch(const LobDev& D, int blocks, cudaStream_t st, A... args) {
    if (D.alg == ALG_VIBE) {
        if (D.C == 3) K<3, ALG_VIBE>::run(blocks, st, D, args...);
        else K<1, ALG_VIBE>::run(blocks, st, D, args...);
    } else if (D.alg == ALG_PBAS) {
        if (D.C == 3) K<3, ALG_PBAS>::run(blocks, st, D, args...);
        else K<1, ALG_PBAS>::run(blocks, st, D, args...);
    } else {
        if (D.C == 3) K<3, ALG_LOBSTER>::run(blocks, st, D, args...);
        else K<1, ALG_LOBSTER>::run(blocks, st, D, args...);
    }
}
template <int C, int ALG>
struct Eval {
    static void run(int b, cudaStream_t st, const LobDev& D) { lob_k_eval<C, ALG><<<b, kThreadsL, 0, st>>>(D); }
};
template <int C, int ALG>
struct Round {
    static void run(int b, cudaStream_t st, const LobDev& D, int r) { lob_k_round<C, ALG><<<b, kThreadsL, 0, st>>>(D, r); }
};
template <int C, int ALG>
struct Commit {
    static void run(int b, cudaStream_t st, const LobDev& D) { lob_k_commit<C, ALG><<<b, kThreadsL, 0, st>>>(D); }
};

// PBAS's gradient image of a device frame into D.grad
void pbas_gradient(const LobDev& D, const uint8_t* img, cudaStream_t st) {
    const int nb = blocks_for((size_t)D.npx * D.C);
    if (D.C == 3) {
        pbas_k_blur<3><<<nb, kThreadsL, 0, st>>>(D, img);
        pbas_k_grad<3><<<nb, kThreadsL, 0, st>>>(D);
    } else {
        pbas_k_blur<1><<<nb, kThreadsL, 0, st>>>(D, img);
        pbas_k_grad<1><<<nb, kThreadsL, 0, st>>>(D);
    }
}

// PBAS's frame-level mean gradient distance, after the commit
lvbgs_status pbas_mean_launch(const LobDev& D, int sms, cudaStream_t st, std::string& err) {
    if (D.C == 1) {
        pbas_k_mean1<<<2 * sms, kThreadsL, 0, st>>>(D);
        pbas_k_mean1_end<<<1, 1, 0, st>>>(D);
    } else {
        const int nChunks = (D.npx + kSumChunk - 1) / kSumChunk;
        SumWork W;
        W.chunkSum = (double*)D.sumTr;
        W.tr = (Tr*)(W.chunkSum + nChunks);
        W.trw = W.tr + (size_t)nChunks * kSumNB;
        W.eb = (int*)(W.trw + (size_t)nChunks * kSumGran * kSumNB);
        pbas_k_sum_chunks<<<nChunks, kSumChunk, 0, st>>>(D, W);
        pbas_k_sum_scan<<<1, kSumScan, 0, st>>>(D, W, nChunks);
        pbas_k_sum_tr<<<nChunks, kSumChunk, 0, st>>>(D, W);
        pbas_k_sum_walk<<<1, 32, 0, st>>>(D, W, nChunks);
    }
    return LVBGS_OK;
}

lvbgs_status lob_refresh_launch(LobState& L, float frac, int force, cudaStream_t st, std::string& err) {
    LobDev& D = L.d;
    const int N = D.N;
    const int nref = frac < 1.0f ? (int)(frac * (float)N) : N;
    int start = 0;
    if (frac < 1.0f) {
        // the frame-level draw of the start position (:416)
        uint32_t c[4] = {L.ksent >> 2, kSentinelPx, D.frameKey, 0u};
        philox4x32_10(c, (uint32_t)D.seed, (uint32_t)(D.seed >> 32));
        start = (int)((c[L.ksent & 3u] & 0x7fffffffu) % (uint32_t)N);
        ++L.ksent;
    }
    if (nref > 0) {
        if (D.C == 3) lob_k_refresh<3><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, start, nref, force);
        else lob_k_refresh<1><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, start, nref, force);
        LOB_CUDA(cudaGetLastError(), "refresh launch");
    }
    return LVBGS_OK;
}
}  // namespace

lvbgs_status lob_init_model(LobState& L, const uint8_t* dimg, cudaStream_t st, std::string& err) {
    LobDev& D = L.d;
    D.frameKey = 0;
    L.ksent = 0;
    if (D.alg == ALG_PBAS) {
        D.cur = 0;
        pbas_gradient(D, dimg, st);
        if (D.C == 3) pbas_k_init<3><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg, L.pbasMean);
        else pbas_k_init<1><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg, L.pbasMean);
        LOB_CUDA(cudaGetLastError(), "init launch");
        LOB_CUDA(cudaStreamSynchronize(st), "initialization");
        return LVBGS_OK;
    }
    if (D.alg == ALG_VIBE) {
        if (D.C == 3) lob_k_vibe_init<3><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg);
        else lob_k_vibe_init<1><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg);
        LOB_CUDA(cudaGetLastError(), "init launch");
        LOB_CUDA(cudaStreamSynchronize(st), "initialization");
        return LVBGS_OK;
    }
    if (D.C == 3) lob_k_init<3><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg);
    else lob_k_init<1><<<blocks_for(D.npx), kThreadsL, 0, st>>>(D, dimg);
    LOB_CUDA(cudaGetLastError(), "init launch");
    // refreshModel(1.0f, true) (:455)
    lvbgs_status s = lob_refresh_launch(L, 1.0f, 1, st, err);
    if (s != LVBGS_OK) return s;
    LOB_CUDA(cudaStreamSynchronize(st), "initialization");
    return LVBGS_OK;
}

lvbgs_status lob_refresh(LobState& L, float frac, int force, cudaStream_t st, std::string& err) {
    lvbgs_status s = lob_refresh_launch(L, frac, force, st, err);
    if (s != LVBGS_OK) return s;
    LOB_CUDA(cudaStreamSynchronize(st), "refresh");
    return LVBGS_OK;
}

lvbgs_status lob_apply(LobState& L, const uint8_t* dimg, uint8_t* dmask, uint8_t* hostMask, double lr,
                       cudaStream_t st, std::string& err) {
    LobDev& D = L.d;
    D.frame = dimg;
    D.maskOut = dmask;
    D.nLR = std::isinf(lr) ? ~0ull : (unsigned long long)std::ceil(lr);  // :470
    if (D.alg == ALG_PBAS) {
        // learningRateOverride > 0 replaces ceil(T(x)) (:174 / :402)
        D.lrOverride = lr > 0 ? 1 : 0;
        if (!(lr > 0)) D.nLR = 0;
    }
    ++L.frames;
    D.frameKey = (uint32_t)L.frames;
    L.ksent = 0;
    const int C = D.C, nb = blocks_for(D.npx);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int roundBlocks = 2 * (sms > 0 ? sms : 1);
    LOB_CUDA(cudaMemsetAsync(D.flags, 0, LOB_F_WORDS * 4, st), "flag reset");
    if (D.alg == ALG_PBAS) {
        LOB_CUDA(cudaMemsetAsync(D.stats + 2, 0, 16, st), "counter reset");
        pbas_gradient(D, dimg, st);
    }
    launch<Eval>(D, nb, st);
    lob_k_mark<<<nb, kThreadsL, 0, st>>>(D);
    LOB_CUDA(cudaGetLastError(), "evaluation launch");
    int round = 0, chunk = L.lastRounds + 1;
    for (;;) {
        for (int i = 0; i < chunk; ++i, ++round) {
            launch<Round>(D, roundBlocks, st, round);
            lob_k_round_end<<<1, 1, 0, st>>>(D, round);
        }
        launch<Commit>(D, nb, st);
        // LOBSTER's median blur, last mask and last colour frame; PBAS's median blur (ViBe outputs its
        // raw mask)
        const dim3 mg((D.W + kMedTile - 1) / kMedTile, (D.H + kMedTile - 1) / kMedTile);
        if (D.alg == ALG_LOBSTER) {
            if (C == 3) lob_k_median<3, true><<<mg, kThreadsL, 0, st>>>(D);
            else lob_k_median<1, true><<<mg, kThreadsL, 0, st>>>(D);
        } else if (D.alg == ALG_PBAS) {
            lob_k_median<1, false><<<mg, kThreadsL, 0, st>>>(D);
        }
        LOB_CUDA(cudaGetLastError(), "repair launch");
        if (hostMask) LOB_CUDA(cudaMemcpyAsync(hostMask, dmask, (size_t)D.npx, cudaMemcpyDeviceToHost, st), "mask download");
        LOB_CUDA(cudaMemcpyAsync(L.h_flags, D.flags, LOB_F_WORDS * 4, cudaMemcpyDeviceToHost, st), "flag read-back");
        // PBAS's frame-level mean gradient distance is only needed by the next frame step: the host does
        // not wait for it
        if (D.alg == ALG_PBAS) {
            LOB_CUDA(cudaEventRecord(L.done, st), "event record");
            lvbgs_status ms = pbas_mean_launch(D, sms, st, err);
            if (ms != LVBGS_OK) return ms;
            LOB_CUDA(cudaGetLastError(), "mean launch");
            LOB_CUDA(cudaEventRecord(L.meanDone, st), "event record");
            LOB_CUDA(cudaEventSynchronize(L.done), "frame step");
        } else {
            LOB_CUDA(cudaStreamSynchronize(st), "frame step");
        }
        if (L.h_flags[LOB_F_ERR]) {
            err = "LOBSTER repair list overflow";
            return LVBGS_DEVICE_ERROR;
        }
        if (L.h_flags[LOB_F_CONV]) break;
        if (round >= kMaxRoundsL) {
            err = "LOBSTER raster-order repair did not converge";
            return LVBGS_DEVICE_ERROR;
        }
        chunk *= 2;
    }
    L.lastRounds = (int)L.h_flags[LOB_F_ROUNDS];
    D.stampBase += (uint32_t)round + 2u;
    if (D.alg == ALG_PBAS) D.cur ^= 1;  // the maps this frame step wrote are the next one's start
    return LVBGS_OK;
}

lvbgs_status lob_background(LobState& L, void* hostOut, bool descriptors, cudaStream_t st, std::string& err) {
    LobDev& D = L.d;
    LOB_CUDA(cudaEventSynchronize(L.meanDone), "frame step");  // the last frame step may run on another stream
    const size_t n = (size_t)D.npx * D.C * (descriptors ? 2 : 1);
    void* tmp = nullptr;
    LOB_CUDA(cudaMallocAsync(&tmp, n, st), "staging allocation");
    if (D.C == 3) lob_k_background<3><<<1024, 256, 0, st>>>(D, tmp, descriptors ? 1 : 0);
    else lob_k_background<1><<<1024, 256, 0, st>>>(D, tmp, descriptors ? 1 : 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hostOut, tmp, n, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    LOB_CUDA(e, "background image");
    return LVBGS_OK;
}

size_t lob_map_bytes(const LobState& L, int which) {
    const size_t npx = (size_t)L.d.npx, C = (size_t)L.d.C, N = (size_t)L.d.N;
    if (L.d.alg == ALG_VIBE) return which == LVBGS_MAP_SAMPLE_COLOR ? N * npx * C : which == LVBGS_MAP_ROI ? npx : 0;
    if (L.d.alg == ALG_PBAS) switch (which) {
            case LVBGS_MAP_SAMPLE_COLOR:
            case LVBGS_MAP_SAMPLE_GRAD: return N * npx * C;
            case LVBGS_MAP_R:
            case LVBGS_MAP_T:
            case LVBGS_MAP_DMIN_LT: return npx * 4;
            case LVBGS_MAP_GRAD: return npx * C;
            case LVBGS_MAP_MEAN_GRAD: return 4;
            case LVBGS_MAP_ROI: return npx;
            default: return 0;
        }
    switch (which) {
        case LVBGS_MAP_LAST_FG:
        case LVBGS_MAP_ROI: return npx;
        case LVBGS_MAP_LAST_COLOR: return npx * C;
        case LVBGS_MAP_LAST_DESC: return npx * C * 2;
        case LVBGS_MAP_SAMPLE_COLOR: return N * npx * C;
        case LVBGS_MAP_SAMPLE_DESC: return N * npx * C * 2;
        case LVBGS_MAP_LUT: return 256;
        default: return 0;
    }
}

lvbgs_status lob_get_map(LobState& L, int which, void* hostOut, size_t bytes, cudaStream_t st, std::string& err) {
    LobDev& D = L.d;
    LOB_CUDA(cudaEventSynchronize(L.meanDone), "frame step");
    const size_t need = lob_map_bytes(L, which);
    if (need == 0) {
        err = "map not kept by LOBSTER";
        return LVBGS_BAD_ARG;
    }
    if (bytes < need) {
        err = "output buffer too small";
        return LVBGS_BAD_ARG;
    }
    const void* src = nullptr;
    const float* fm = D.fm ? D.fm + (size_t)D.cur * 3 * D.npx : nullptr;
    if (D.alg == ALG_VIBE) src = which == LVBGS_MAP_ROI ? (const void*)D.roi : (const void*)D.sC;
    else if (D.alg == ALG_PBAS) switch (which) {
            case LVBGS_MAP_SAMPLE_COLOR: src = D.sC; break;
            case LVBGS_MAP_SAMPLE_GRAD: src = D.sG; break;
            case LVBGS_MAP_R: src = fm; break;
            case LVBGS_MAP_T: src = fm + D.npx; break;
            case LVBGS_MAP_DMIN_LT: src = fm + 2 * (size_t)D.npx; break;
            case LVBGS_MAP_GRAD: src = D.grad; break;
            case LVBGS_MAP_MEAN_GRAD: src = D.meanGrad; break;
            default: src = D.roi; break;
        }
    else switch (which) {
        case LVBGS_MAP_LAST_FG: src = D.lastFG; break;
        case LVBGS_MAP_ROI: src = D.roi; break;
        case LVBGS_MAP_LAST_COLOR: src = D.lastColor; break;
        case LVBGS_MAP_LAST_DESC: src = D.lastDesc; break;
        case LVBGS_MAP_LUT: src = D.lut; break;
        default: break;
    }
    if (src) {
        LOB_CUDA(cudaMemcpyAsync(hostOut, src, need, cudaMemcpyDeviceToHost, st), "map download");
        LOB_CUDA(cudaStreamSynchronize(st), "map download");
        return LVBGS_OK;
    }
    void* tmp = nullptr;
    LOB_CUDA(cudaMallocAsync(&tmp, need, st), "staging allocation");
    const int desc = which == LVBGS_MAP_SAMPLE_DESC ? 1 : 0;
    if (D.C == 3) lob_k_export_samples<3><<<1024, 256, 0, st>>>(D, tmp, desc);
    else lob_k_export_samples<1><<<1024, 256, 0, st>>>(D, tmp, desc);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hostOut, tmp, need, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    LOB_CUDA(e, "sample export");
    return LVBGS_OK;
}

lvbgs_status lob_stats(LobState& L, unsigned long long out[2], cudaStream_t st, std::string& err) {
    LOB_CUDA(cudaEventSynchronize(L.meanDone), "frame step");
    LOB_CUDA(cudaMemcpyAsync(out, L.d.stats, 16, cudaMemcpyDeviceToHost, st), "statistics download");
    LOB_CUDA(cudaStreamSynchronize(st), "statistics download");
    return LVBGS_OK;
}

}  // namespace lvbgs
