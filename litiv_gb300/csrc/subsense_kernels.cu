// SuBSENSE frame step for sm_103a: one tick processes one frame of every stream in the batch as a
// sequence of ordinary launches over a per-stream descriptor table (a tile, row or segment index is
// mapped to its stream by binary search); only the repair rounds run as one cooperative kernel whose
// rounds are separated by a bounded grid barrier.
//
// Exactness of the reference's sequential raster scan (BackgroundSubtractorSuBSENSE.cpp:201-481):
// a pixel p reads two things another pixel writes during the same frame -- its own samples, which
// an earlier pixel's neighbour update may have overwritten (:296-299/:442-448), and the D_last /
// raw-segmentation-ST values of its randomly chosen neighbour q, which are this frame's values when
// q precedes p (:292-293/:438-439). Random draws are keyed by (stream, frame, pixel, draw index),
// so they do not depend on the scan order. The tick therefore
//   A  evaluates every pixel against the frame-start model and records an "intent" (decision,
//      samples evaluated, own/neighbour sample writes, neighbour-update state),
//   B  resolves the ghost test of each neighbour update against the values the scan would see,
//      and marks every pixel whose evaluated samples were overwritten by an earlier pixel,
//   M/R repairs: re-evaluates marked pixels with the overwritten samples (M) and re-resolves the
//      ghost tests that read a pixel whose decision changed (R), marking the pixels whose incoming
//      writes changed, until nothing changes (the dependencies follow raster order, so this is a
//      fixed point reached in at most the length of the longest dependency chain),
//   F  commits every sample write in raster order (last writer wins) and starts post-processing.
// Post-processing, frame-level statistics and the automatic model reset follow in later launches of
// the same tick.
#include <cuda_runtime.h>

#include "lbsp_device.cuh"
#include "lvbgs_internal.h"

namespace lvbgs {

// LBSP 16-bit double-cross pattern (LBSP.hpp:297-298)
__constant__ int c_lbsp_dx[16] = {-2, 2, 0, 0, -2, 2, 2, -2, 0, -1, 0, 1, -1, 1, 1, -1};
__constant__ int c_lbsp_dy[16] = {0, 0, -2, 2, 2, -2, 2, -2, 1, 0, -1, 0, -1, 1, -1, 1};
// 7x7 Gaussian sampling weights (opencv.hpp:915-923) and 3x3 / 5x5 neighbour tables (opencv.hpp:945-964)
__constant__ int c_pat7[49] = {2, 4, 6, 7, 6, 4, 2,     4, 8, 12, 14, 12, 8, 4, 6, 12, 21, 25, 21, 12, 6, 7, 14, 25, 28,
                               25, 14, 7, 6, 12, 21, 25, 21, 12, 6, 4, 8, 12, 14, 12, 8, 4, 2, 4, 6, 7, 6, 4, 2};
__constant__ int c_nb3[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};
__constant__ int c_nb5[24][2] = {{-2, 2}, {-1, 2}, {0, 2},   {1, 2},   {2, 2},   {-2, 1},  {-1, 1}, {0, 1},
                                 {1, 1},  {2, 1},  {-2, 0},  {-1, 0},  {1, 0},   {2, 0},   {-2, -1}, {-1, -1},
                                 {0, -1}, {1, -1}, {2, -1},  {-2, -2}, {-1, -2}, {0, -2},  {1, -2}, {2, -2}};

constexpr int kUFLimit = 1 << 22;

// ------------------------------------------------------------------------------------------
// small helpers
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned int ld_volatile(const unsigned int* p) { return *(const volatile unsigned int*)p; }

// Grid-wide barrier for a cooperative launch (all CTAs co-resident). The wait is bounded: after
// timeoutNs the CTA records ERR_BARRIER_TIMEOUT and every CTA leaves at its next check.
__device__ bool grid_sync(TickWork* w, unsigned long long timeoutNs) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int gen = ld_volatile(&w->bar_gen);
        __threadfence();
        const unsigned int arrived = atomicAdd(&w->bar_count, 1u) + 1u;
        int ok = 1;
        if (arrived == gridDim.x) {
            atomicExch(&w->bar_count, 0u);
            __threadfence();
            atomicAdd(&w->bar_gen, 1u);
        } else {
            const unsigned long long t0 = gtimer();
            while (ld_volatile(&w->bar_gen) == gen) {
                if (ld_volatile(&w->err) != 0u) {
                    ok = 0;
                    break;
                }
                __nanosleep(40);
                if (gtimer() - t0 > timeoutNs) {
                    atomicOr(&w->err, ERR_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok && (ld_volatile(&w->err) == 0u);
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0 && w->nts < 40u) w->ts[w->nts++] = gtimer();
    return s_ok != 0;
}

__device__ __forceinline__ int find_stream_by_tile(const TickParams& P, int t) {
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.streams[mid].tileBase <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct DrawState {
    uint32_t blk;
    uint32_t v[4];
};
__device__ __forceinline__ uint32_t draw_k(unsigned long long seed, uint32_t frame, uint32_t px, uint32_t k,
                                           DrawState& ds) {
    const uint32_t blk = k >> 2;
    if (blk != ds.blk) {
        uint32_t c[4] = {blk, px, frame, 0u};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        ds.v[0] = c[0];
        ds.v[1] = c[1];
        ds.v[2] = c[2];
        ds.v[3] = c[3];
        ds.blk = blk;
    }
    return ds.v[k & 3u] & 0x7fffffffu;
}
// a % m for a 31-bit draw and a size_t modulus (m >= 2^32 leaves a unchanged)
__device__ __forceinline__ unsigned long long mod_draw(uint32_t a, unsigned long long m) {
    if (m > 0xffffffffull) return (unsigned long long)a;
    const uint32_t m32 = (uint32_t)m;
    if ((m32 & (m32 - 1u)) == 0u) return (unsigned long long)(a & (m32 - 1u));  // powers of two (T = 2, 4, ...)
    return (unsigned long long)(a % m32);
}
// a % N for a 31-bit draw with the stream's multiplier M = ceil(2^40 / N): for N <= 64 the
// quotient error a*(M - 2^40/N)/2^40 < 2^-9 < 1/N, so floor(a*M / 2^40) is the exact quotient
__device__ __forceinline__ uint32_t mod_n(uint32_t a, const StreamDev& S) {
    const uint32_t q = (uint32_t)(((unsigned long long)a * S.nMagic) >> 40);
    return a - q * (uint32_t)S.N;
}

__device__ __forceinline__ void clamp_xy(int& x, int& y, int W, int H) {
    if (x < kBorder) x = kBorder;
    else if (x >= W - kBorder) x = W - kBorder - 1;
    if (y < kBorder) y = kBorder;
    else if (y >= H - kBorder) y = H - kBorder - 1;
}

__device__ __forceinline__ float fmin_std(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float fmax_std(float a, float b) { return (a < b) ? b : a; }

struct FrameK {
    float fLT, fST, t_lo, t_hi;
    uint32_t frame;  // frame index of this tick (m_nFrameIdx after ++)
    int cur, nxt;
    int cooldown;  // m_nModelResetCooldown != 0
    int use3x3;
};
// exact quotients i/765, i/255, i/48 and i/16 (IEEE division on the device, done once): the
// normalized distances of :254/:258/:272 and :396/:400/:416 divide small integers by constants
__device__ float g_div_col3[766], g_div_col1[256], g_div_desc3[49], g_div_desc1[17];
extern "C" __global__ void lvbgs_init_tables() {
    for (int i = threadIdx.x; i < 766; i += blockDim.x) g_div_col3[i] = (float)i / 765.0f;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) g_div_col1[i] = (float)i / 255.0f;
    for (int i = threadIdx.x; i < 49; i += blockDim.x) g_div_desc3[i] = (float)i / 48.0f;
    for (int i = threadIdx.x; i < 17; i += blockDim.x) g_div_desc1[i] = (float)i / 16.0f;
}

__device__ __forceinline__ FrameK frame_consts(const StreamDev& S) {
    const StreamCtl* ctl = S.ctl;
    FrameK F;
    const unsigned long long f = ctl->frame_idx + 1ull;
    F.fLT = ctl->fLT;
    F.fST = ctl->fST;
    F.frame = (uint32_t)f;
    F.cur = (int)(ctl->frame_idx & 1ull);
    F.nxt = F.cur ^ 1;
    F.cooldown = ctl->cooldown != 0ull;
    F.t_lo = ctl->t_lo;
    F.t_hi = ctl->t_hi;
    F.use3x3 = ctl->use3x3;
    return F;
}

// one override of a sample read: an earlier pixel's neighbour update of this pixel
struct Ovr {
    int s;
    uint32_t col;      // packed colour bytes
    uint64_t desc;     // packed descriptors
};

// ------------------------------------------------------------------------------------------
// per-pixel evaluation: one iteration of the reference's raster loop for pixel p, against the
// frame-start samples (optionally overridden). Writes the pixel's next-frame maps and returns
// its intent word. (1ch: BackgroundSubtractorSuBSENSE.cpp:201-330, 3ch: :333-481)
// ------------------------------------------------------------------------------------------
// per-pixel inputs of one evaluation, loaded up front so that all of them are in flight together
template <int C>
struct PixIn {
    float R, V, T, DL, DmLT, DmST, RwLT, RwST, FnLT, FnST;
    uint32_t uOld, lastFG, blink;
    uint32_t lc[C], ld[C];
    uint64_t d0, d1;  // samples 0 and 1 (descriptor plane word)
    uint32_t c0, c1;  // samples 0 and 1 (colour byte plane)
};
template <int C>
__device__ __forceinline__ void load_pix(const StreamDev& S, const FrameK& F, int p, PixIn<C>& in) {
    const int npx = S.npx;
    const float* fc = S.fm + (size_t)F.cur * kNumFloatMaps * npx;
    in.R = fc[FM_R * npx + p];
    in.V = fc[FM_V * npx + p];
    in.T = fc[FM_T * npx + p];
    in.DL = fc[FM_DLAST * npx + p];
    in.DmLT = fc[FM_DMIN_LT * npx + p];
    in.DmST = fc[FM_DMIN_ST * npx + p];
    in.RwLT = fc[FM_RAW_LT * npx + p];
    in.RwST = fc[FM_RAW_ST * npx + p];
    in.FnLT = fc[FM_FIN_LT * npx + p];
    in.FnST = fc[FM_FIN_ST * npx + p];
    in.uOld = S.unst[(size_t)F.cur * npx + p];
    in.lastFG = S.lastFG[p];
    in.blink = S.blinks[p];
    const uint8_t* lc = S.lastCol + (size_t)F.cur * npx * C + (size_t)p * C;
    const uint16_t* ld = S.lastDesc + (size_t)F.cur * npx * C + (size_t)p * C;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        in.lc[c] = lc[c];
        in.ld[c] = ld[c];
    }
    in.d0 = in.d1 = 0;
    in.c0 = in.c1 = 0;
    if (S.N > 0) {
        in.d0 = C == 3 ? ((const uint64_t*)S.sD)[p] : (uint64_t)((const uint16_t*)S.sD)[p];
        in.c0 = S.sC[p];
    }
    if (S.N > 1) {
        in.d1 = C == 3 ? ((const uint64_t*)S.sD)[(size_t)npx + p] : (uint64_t)((const uint16_t*)S.sD)[(size_t)npx + p];
        in.c1 = S.sC[(size_t)npx + p];
    }
}

// thresholds of one evaluation from R(x) and the previous unstable flag, and the new unstable flag
// descThr is clamped to 255: a descriptor distance is at most 16 per channel (48 summed), so every
// comparison against the clamped value (or three times it) has the result of the unclamped one
struct EvalThr {
    uint32_t colThr;
    uint32_t descThr;
    uint32_t uNew;
};
__device__ __forceinline__ EvalThr eval_thresholds(const StreamDev& S, float R, float RwLT, float RwST, float FnLT,
                                                   float FnST, uint32_t uOld) {
    EvalThr t;
    t.colThr =
        (uint32_t)__float2ull_rz(R * (float)S.minColor - (float)((uint32_t)(uOld == 0u) * (uint32_t)S.stabColorOff));
    const unsigned long long descThr = (1ull << (unsigned)__float2ull_rz(floorf(R + 0.5f))) +
                                       (unsigned long long)S.descOff + (unsigned long long)uOld * S.descOff;
    t.descThr = descThr < 255ull ? (uint32_t)descThr : 255u;
    t.uNew = (R > 3.000f || (RwLT - FnLT) > 0.100f || (RwST - FnST) > 0.100f) ? 1u : 0u;
    return t;
}

// state of the ordered sample scan: next sample, good samples so far, minima over the good ones
struct ScanSt {
    int s, nGood;
    uint32_t minDesc, minSum;
    int g0, g1;                   // indices of the first two good samples (-1: none)
    uint32_t g0d, g0s, g1d, g1s;  // their descriptor and summed distances
};

// one sample against the pixel (the body of the sample loops, :226-250 / :357-393): whether it is a
// good match, and its descriptor and summed distances. The reference rejects a sample at the first
// failed check; the verdict is the conjunction of all checks, so the three-channel form tests the
// three colour distances first (one branch), then evaluates the three channels without branches.
template <int C>
__device__ __forceinline__ bool sample_match(const uint8_t* __restrict__ lut, const uint32_t (&vals)[C][4],
                                             const uint32_t (&curr)[C], const uint32_t (&intra)[C],
                                             const EvalThr& th, uint64_t d, uint32_t c2, uint32_t& dd,
                                             uint32_t& sd) {
    if (C == 1) {
        const uint32_t cthr = th.colThr / 2u;
        const uint32_t bgc = c2, bgd = (uint32_t)d & 0xffffu;
        const uint32_t colDist = (uint32_t)abs((int)curr[0] - (int)bgc);
        if (colDist > cthr) return false;
        const uint32_t intraD = __popc(intra[0] ^ bgd);
        const uint32_t interD = __popc((lbsp_thr_raw(vals[0], bgc, lut[bgc]) ^ bgd) & 0xffffu);
        const uint32_t descDist = (intraD + interD) / 2u;
        if (descDist > th.descThr) return false;
        uint32_t sumDist = (descDist / 4u) * 15u + colDist;
        if (sumDist > 255u) sumDist = 255u;
        if (sumDist > cthr) return false;
        dd = descDist;
        sd = sumDist;
        return true;
    } else {
        const uint32_t totColThr = th.colThr * 3u, scThr = totColThr / 2u;
        const uint32_t hiw = (uint32_t)(d >> 32), low = (uint32_t)d;
        // bytes 0-2: the sample's colours (d bits 48-55, 56-63, c2); byte 3 repeats byte 2
        const uint32_t bgW = __byte_perm(hiw, c2, 0x4432);
        const uint32_t currW = curr[0] | (curr[1] << 8) | (curr[2] * 0x01010000u);
        const uint32_t cd = __vabsdiffu4(currW, bgW);
        const uint32_t col0 = cd & 0xffu, col1 = (cd >> 8) & 0xffu, col2 = (cd >> 16) & 0xffu;
        if (max(max(col0, col1), col2) > scThr) return false;
        const uint32_t col[3] = {col0, col1, col2};
        const uint32_t bgc[3] = {bgW & 0xffu, (bgW >> 8) & 0xffu, (bgW >> 16) & 0xffu};
        const uint32_t bgd[3] = {low & 0xffffu, low >> 16, hiw & 0xffffu};
        uint32_t totDesc = 0, totSum = 0;
        bool bad = false;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint32_t intraD = __popc(intra[c] ^ bgd[c]);
            const uint32_t interD = __popc((lbsp_thr_raw(vals[c], bgc[c], lut[bgc[c]]) ^ bgd[c]) & 0xffffu);
            const uint32_t descDist = (intraD + interD) / 2u;
            const uint32_t sumDist = min((descDist / 2u) * 15u + col[c], 255u);
            bad |= sumDist > scThr;
            totDesc += descDist;
            totSum += sumDist;
        }
        if (bad || totDesc > th.descThr * 3u || totSum > totColThr) return false;
        dd = totDesc;
        sd = totSum;
        return true;
    }
}

// the ordered sample scan, continued from state st until nreq good samples or sample sEnd; dA/cA and
// dB/cB hold samples st.s and st.s+1 (they arrive with the feedback maps), and the loop requests
// sample s+2 while it evaluates sample s. OVR: the samples that earlier pixels overwrite this frame
// (repair)
// L2 prefetch of sample k of pixel p (both planes): a hint without registers, so that a long scan keeps
// several samples in flight
template <int C>
__device__ __forceinline__ void prefetch_sample(const StreamDev& S, int k, int p) {
    const void* a = C == 3 ? (const void*)((const uint64_t*)S.sD + (size_t)k * S.npx + p)
                           : (const void*)((const uint16_t*)S.sD + (size_t)k * S.npx + p);
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(S.sC + (size_t)k * S.npx + p));
}
constexpr int kScanPrefetch = 8;  // samples prefetched ahead of the loads of a long scan

template <int C>
__device__ __forceinline__ void scan_init(ScanSt& st) {
    st.s = 0;
    st.nGood = 0;
    st.g0 = st.g1 = -1;
    st.g0d = st.g0s = st.g1d = st.g1s = 0;
    st.minDesc = C == 1 ? 16u : 48u;
    st.minSum = C == 1 ? 255u : 765u;
}
template <int C, bool OVR, bool REC = true>
__device__ __forceinline__ void scan_samples(const StreamDev& S, const uint8_t* __restrict__ lut, int p,
                                             const uint32_t (&vals)[C][4], const uint32_t (&curr)[C],
                                             const uint32_t (&intra)[C], const EvalThr& th, const Ovr* ov, int nov,
                                             uint64_t ovmask, int sEnd, uint64_t dA, uint32_t cA, uint64_t dB,
                                             uint32_t cB, ScanSt& st) {
    const int npx = S.npx, N = S.N, nreq = S.nreq;
    const int sMax = sEnd < N ? sEnd : N;
    int nGood = st.nGood, s = st.s;
    uint32_t minDesc = st.minDesc, minSum = st.minSum;
    int g0 = st.g0, g1 = st.g1;
    uint32_t g0d = st.g0d, g0s = st.g0s, g1d = st.g1d, g1s = st.g1s;
    // scans that may run past the evaluation's cap (long scans, repair) prefetch ahead into L2
    const bool deep = sMax > kScanCap;
    if (deep && nGood < nreq)
        for (int k = s + 2; k < min(N, s + 2 + kScanPrefetch); ++k) prefetch_sample<C>(S, k, p);
    while (nGood < nreq && s < sMax) {
        uint64_t d = dA;
        uint32_t c2 = cA;
        dA = dB;
        cA = cB;
        if (s + 2 < sMax) {
            dB = C == 3 ? ((const uint64_t*)S.sD)[(size_t)(s + 2) * npx + p]
                        : (uint64_t)((const uint16_t*)S.sD)[(size_t)(s + 2) * npx + p];
            cB = S.sC[(size_t)(s + 2) * npx + p];
            if (deep && s + 2 + kScanPrefetch < N) prefetch_sample<C>(S, s + 2 + kScanPrefetch, p);
        }
        if (OVR && ((ovmask >> s) & 1ull)) {
            int k = nov - 1;
            while (ov[k].s != s) --k;
            if (C == 3) {
                d = ov[k].desc | ((uint64_t)(ov[k].col & 0xffffu) << 48);
                c2 = (ov[k].col >> 16) & 0xffu;
            } else {
                d = ov[k].desc & 0xffffu;
                c2 = ov[k].col & 0xffu;
            }
        }
        uint32_t dd, sd;
        if (sample_match<C>(lut, vals, curr, intra, th, d, c2, dd, sd)) {
            if (minDesc > dd) minDesc = dd;
            if (minSum > sd) minSum = sd;
            if (g0 < 0) {
                g0 = s;
                if (REC) {
                    g0d = dd;
                    g0s = sd;
                }
            } else if (REC && g1 < 0) {
                g1 = s;
                g1d = dd;
                g1s = sd;
            }
            ++nGood;
        }
        ++s;
    }
    st.s = s;
    st.nGood = nGood;
    st.minDesc = minDesc;
    st.minSum = minSum;
    st.g0 = g0;
    st.g0d = g0d;
    st.g0s = g0s;
    st.g1 = g1;
    st.g1d = g1d;
    st.g1s = g1s;
}

// With nreq <= 2 a scan's outcome is fixed by its stop position and its (at most two) good samples:
// every other sample it evaluated is bad. Recording them for the long scans lets the repair re-match
// such a pixel from the samples that earlier pixels overwrite (the others keep their frame-start
// values, so their verdicts), scanning on only when an overwrite removed a good sample.
// Record: frame tag | stop | count | indices | descriptor distances | summed distances.
__device__ __forceinline__ void record_scan(const StreamDev& S, const FrameK& F, int p, const ScanSt& st) {
    if (S.nreq > 2) return;
    const int n = st.nGood < 2 ? st.nGood : 2;
    uint4 r;
    r.x = F.frame;
    r.y = (uint32_t)st.s | ((uint32_t)n << 8) | ((uint32_t)(st.g0 < 0 ? 255 : st.g0) << 16) |
          ((uint32_t)(st.g1 < 0 ? 255 : st.g1) << 24);
    r.z = (st.g0d & 0xffffu) | (st.g1d << 16);
    r.w = (st.g0s & 0xffffu) | (st.g1s << 16);
    S.goodRec[p] = r;
}

// the rest of one evaluation after the sample scan (:254-330 / :396-481): D_last, D_min, the raw
// segmentation averages, the model/neighbour update decisions and draws, T, v and R; writes the
// next-frame maps and returns the intent word
template <int C>
__device__ uint32_t eval_tail(const StreamDev& S, const FrameK& F, int x, int y, int p, const PixIn<C>& in,
                              const uint32_t (&curr)[C], const uint32_t (&intra)[C], uint32_t uNew,
                              const ScanSt& st) {
    const int npx = S.npx;
    float* fn = S.fm + (size_t)F.nxt * kNumFloatMaps * npx;
    float R = in.R, V = in.V, T = in.T;
    const float DL = in.DL;
    float DmLT = in.DmLT, DmST = in.DmST, RwLT = in.RwLT, RwST = in.RwST;
    const uint32_t lastFG = in.lastFG, blink = in.blink;
    const int nreq = S.nreq, nGood = st.nGood, s = st.s;
    const uint32_t minDesc = st.minDesc, minSum = st.minSum;

    // D_last (:254-255 / :396-397): depends on the pixel alone. With three channels the reference
    // takes the colour term from lv::L1dist<3>(const uchar*, const uchar*) (math.hpp:226-232), whose
    // accumulator type is that of L1dist(uchar, uchar), unsigned char: the sum wraps modulo 256.
    uint32_t l1 = 0, hd = 0;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        l1 += (uint32_t)abs((int)in.lc[c] - (int)curr[c]);
        hd += __popc(in.ld[c] ^ intra[c]);
    }
    if (C == 3) l1 &= 0xffu;
    const float* divCol = C == 1 ? g_div_col1 : g_div_col3;    // i / 255 or i / 765
    const float* divDesc = C == 1 ? g_div_desc1 : g_div_desc3;  // i / 16 or i / 48
    const float normLast = (__ldg(&divCol[l1]) + __ldg(&divDesc[hd])) / 2;
    const float DLn = DL * (1.0f - F.fST) + normLast * F.fST;

    uint32_t intent = kInValid | ((uint32_t)s << kInEShift);
    DrawState ds;
    ds.blk = 0xffffffffu;
    const uint32_t seedFrame = F.frame;
    const bool fg = nGood < nreq;
    if (fg) {
        const float md = (__ldg(&divCol[minSum]) + __ldg(&divDesc[minDesc])) / 2 + (float)(nreq - nGood) / (float)nreq;
        const float nmd = fmin_std(1.0f, md);
        DmLT = DmLT * (1.0f - F.fLT) + nmd * F.fLT;
        DmST = DmST * (1.0f - F.fST) + nmd * F.fST;
        RwLT = RwLT * (1.0f - F.fLT) + F.fLT;
        RwST = RwST * (1.0f - F.fST) + F.fST;
        intent |= kInFG;
        if (F.cooldown && (draw_k(S.seed, seedFrame, (uint32_t)p, 0u, ds) % 2u) == 0u) {
            const uint32_t so = mod_n(draw_k(S.seed, seedFrame, (uint32_t)p, 1u, ds), S);
            intent |= kInOwn | (so << kInSOwnShift);
        }
    } else {
        const float nmd = (__ldg(&divCol[minSum]) + __ldg(&divDesc[minDesc])) / 2;
        DmLT = DmLT * (1.0f - F.fLT) + nmd * F.fLT;
        DmST = DmST * (1.0f - F.fST) + nmd * F.fST;
        RwLT = RwLT * (1.0f - F.fLT);
        RwST = RwST * (1.0f - F.fST);
        const unsigned long long nLR = S.lrMode ? S.lrFixed : (unsigned long long)__float2ull_rz(ceilf(T));
        uint32_t k = 0;
        if (mod_draw(draw_k(S.seed, seedFrame, (uint32_t)p, k++, ds), nLR) == 0ull) {
            const uint32_t so = mod_n(draw_k(S.seed, seedFrame, (uint32_t)p, k++, ds), S);
            intent |= kInOwn | (so << kInSOwnShift);
        }
        const bool use3 = F.use3x3 && !uNew;
        const uint32_t rn = draw_k(S.seed, seedFrame, (uint32_t)p, k++, ds);
        int nx, ny;
        if (use3) {
            const int r = (int)(rn % 8u);
            nx = x + c_nb3[r][0];
            ny = y + c_nb3[r][1];
        } else {
            const int r = (int)(rn % 24u);
            nx = x + c_nb5[r][0];
            ny = y + c_nb5[r][1];
        }
        clamp_xy(nx, ny, S.W, S.H);
        const uint32_t code = (uint32_t)((ny - y + 2) * 5 + (nx - x + 2));
        const uint32_t nrand = draw_k(S.seed, seedFrame, (uint32_t)p, k++, ds);
        const unsigned long long X = use3 ? nLR : (nLR / 2ull + 1ull);
        uint32_t st;
        if (mod_draw(nrand, X) == 0ull) st = NB_WRITE;
        else if (mod_draw(nrand, (unsigned long long)__float2ull_rz(F.t_lo)) == 0ull) st = NB_PENDING;
        else st = NB_NO;
        const uint32_t snb = mod_n(draw_k(S.seed, seedFrame, (uint32_t)p, k, ds), S);
        intent |= (code << kInCodeShift) | (st << kInNStShift) | (snb << kInSNbShift);
    }

    // feedback: T (:302-311), v (:312-318), R (:319-325)
    const float mn = fmin_std(DmLT, DmST), mx = fmax_std(DmLT, DmST);
    if (lastFG || (mn < 0.100f && fg)) {
        if (T < F.t_hi) T += 0.5000f / (mx * V);
    } else if (T > F.t_lo) {
        T -= 0.2500f * V / mx;
    }
    if (T < F.t_lo) T = F.t_lo;
    else if (T > F.t_hi) T = F.t_hi;
    if (mx > 0.100f && blink) {
        V += 1.000f;
    } else if (V > 0.100f) {
        V -= lastFG ? 0.100f / 4 : uNew ? 0.100f / 2 : 0.100f;
        if (V < 0.100f) V = 0.100f;
    }
    // R < pow(1+2*min, 2) is evaluated in double by the reference; x*x of a float is exact in
    // double, so compare exactly with the two-product split hi + lo of x*x
    const float rx = 1.0f + mn * 2;
    const float hi = rx * rx;
    const float lo = fmaf(rx, rx, -hi);
    if (R < hi || (R == hi && lo > 0.0f)) {
        R += 0.01f * (V - 0.100f);
    } else {
        R -= 0.01f / V;
        if (R < 1.0f) R = 1.0f;
    }
    fn[FM_R * npx + p] = R;
    fn[FM_V * npx + p] = V;
    fn[FM_T * npx + p] = T;
    __stcg(&fn[FM_DLAST * npx + p], DLn);
    fn[FM_DMIN_LT * npx + p] = DmLT;
    fn[FM_DMIN_ST * npx + p] = DmST;
    fn[FM_RAW_LT * npx + p] = RwLT;
    __stcg(&fn[FM_RAW_ST * npx + p], RwST);
    S.unst[(size_t)F.nxt * npx + p] = (uint8_t)uNew;
    uint8_t* lcn = S.lastCol + (size_t)F.nxt * npx * C + (size_t)p * C;
    uint16_t* ldn = S.lastDesc + (size_t)F.nxt * npx * C + (size_t)p * C;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        lcn[c] = (uint8_t)curr[c];
        __stcg(&ldn[c], (uint16_t)intra[c]);
    }
    return intent;
}

// a full evaluation: thresholds, the whole ordered scan, the tail (the repair's re-match)
template <int C, bool OVR>
__device__ uint32_t eval_pixel(const StreamDev& S, const FrameK& F, const uint8_t* __restrict__ lut, int x, int y,
                               int p, const PixIn<C>& in, const uint32_t (&vals)[C][4], const uint32_t (&curr)[C],
                               const uint32_t (&intra)[C], const Ovr* ov, int nov, uint64_t ovmask, int& e_out) {
    const EvalThr th = eval_thresholds(S, in.R, in.RwLT, in.RwST, in.FnLT, in.FnST, in.uOld);
    ScanSt st;
    scan_init<C>(st);
    scan_samples<C, OVR>(S, lut, p, vals, curr, intra, th, ov, nov, ovmask, S.N, in.d0, in.c0, in.d1, in.c1, st);
    e_out = st.s;
    return eval_tail<C>(S, F, x, y, p, in, curr, intra, th.uNew, st);
}

// non-zero LBSP descriptor test of the frame-level statistics (:264-265 / :405-407)
template <int C>
__device__ __forceinline__ int desc_nonzero(const uint32_t (&intra)[C]) {
    uint32_t pc = 0;
#pragma unroll
    for (int c = 0; c < C; ++c) pc += __popc(intra[c]);
    return pc >= (C == 1 ? 2u : 4u) ? 1 : 0;
}

// adds two per-thread counts of a tile block to per-stream counters with one atomic each per block
// (every thread of the block calls it; b may be null)
__device__ __forceinline__ void block_add_stats(unsigned long long* a, unsigned long long va, unsigned long long* b,
                                                unsigned long long vb) {
    __shared__ unsigned long long red[2][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        va += __shfl_xor_sync(0xffffffffu, va, o);
        vb += __shfl_xor_sync(0xffffffffu, vb, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = va;
        red[1][threadIdx.x >> 5] = vb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long sa = 0, sb = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            sa += red[0][i];
            sb += red[1][i];
        }
        if (sa) atomicAdd(a, sa);
        if (b && sb) atomicAdd(b, sb);
    }
}

// block-aggregated list reservation: every thread of the block calls it; returns this thread's slot
// (or ~0u when it does not want one). One counter atomic per block: the lists' counters are shared by
// all streams of the batch, and same-address atomics serialize.
__device__ __forceinline__ unsigned int block_reserve(bool want, unsigned int* count) {
    __shared__ unsigned int sWarp[32];
    __shared__ unsigned int sBase;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (lane == 0) sWarp[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int run = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            const unsigned int v = sWarp[i];
            sWarp[i] = run;
            run += v;
        }
        sBase = run ? atomicAdd(count, run) : 0u;
    }
    __syncthreads();
    const unsigned int r = want ? sBase + sWarp[warp] + (unsigned int)__popc(m & ((1u << lane) - 1u)) : ~0u;
    __syncthreads();  // the shared slots are reused by the next call
    return r;
}

// gathers the 16 LBSP taps of channel c at (x, y) from a byte image (tile or frame)
template <int C>
__device__ __forceinline__ void gather_taps(const uint8_t* base, int rowStride, int c, uint32_t (&v)[4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint32_t w = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int n = j * 4 + i;
            w |= (uint32_t)base[c_lbsp_dy[n] * rowStride + c_lbsp_dx[n] * C + c] << (8 * i);
        }
        v[j] = w;
    }
}

// the evaluation's shared-memory frame tile: byte 0 of a tile row buffer is kTileDelta<C> bytes before
// the frame byte (x0-2)*C - 2 of the tile's leftmost tap, which puts it on a 16-byte boundary of the
// frame row (x0 = 32 * tile column: (96k - 8) - 8 for C = 3, (32k - 4) - 12 for C = 1); kTileRW<C> is
// the row stride, a multiple of 16 that covers the (kTileW + 4) * C + 2 bytes of taps after the delta
template <int C>
constexpr int kTileDelta = C == 3 ? 8 : 12;
template <int C>
constexpr int kTileRW = (kTileDelta<C> + (kTileW + 2 * kBorder) * C + 2 + 15) / 16 * 16;
static_assert(kTileW == 32 && kBorder == 2, "the tile deltas assume 32-pixel tile columns and a 2-pixel border");

// ------------------------------------------------------------------------------------------
// phase A: evaluate every pixel of a tile against the frame-start model
// ------------------------------------------------------------------------------------------
template <int C>
__device__ void phaseA_tile(const TickParams& P, int si, const StreamDev& S, int lt, uint8_t* smem) {
    const int tx = lt % S.tilesX, ty = lt / S.tilesX;
    const int x0 = tx * kTileW, y0 = ty * kTileH;
    // The tile holds rows y0-2 .. y0+9 of the frame. The taps of the tile's pixels span frame bytes
    // b0 = (x0-2)*C - 2 .. b0 + (kTileW+4)*C + 1 of a row; a tile row buffer starts kTileDelta<C> bytes
    // before b0, at a 16-byte boundary of the row (x0 is a multiple of 32), so it is filled with
    // aligned 128-bit loads when the frame rows are 16-byte aligned (else 32-bit words, or bytes).
    constexpr int RW = kTileRW<C>;  // tile row stride (bytes)
    constexpr int NCH = RW / 16;    // 16-byte chunks per tile row
    constexpr int RH = kTileH + 2 * kBorder;
    const FrameK F = frame_consts(S);
    const int lx = threadIdx.x % kTileW, ly = threadIdx.x / kTileW;
    const int x = x0 + lx, y = y0 + ly;
    const bool inFrame = x < S.W && y < S.H;
    const int p = y * S.W + x;
    const bool active = inFrame && S.roi[p] != 0;
    // the scan's inputs first (they overlap the tile load below); the other maps after the scan
    float tR = 0, tRwLT = 0, tRwST = 0, tFnLT = 0, tFnST = 0;
    uint32_t tU = 0, c0 = 0, c1 = 0;
    uint64_t d0 = 0, d1 = 0;
    if (active) {
        const int npx = S.npx;
        const float* fc = S.fm + (size_t)F.cur * kNumFloatMaps * npx;
        tR = fc[FM_R * npx + p];
        tRwLT = fc[FM_RAW_LT * npx + p];
        tRwST = fc[FM_RAW_ST * npx + p];
        tFnLT = fc[FM_FIN_LT * npx + p];
        tFnST = fc[FM_FIN_ST * npx + p];
        tU = S.unst[(size_t)F.cur * npx + p];
        if (S.N > 0) {
            d0 = C == 3 ? ((const uint64_t*)S.sD)[p] : (uint64_t)((const uint16_t*)S.sD)[p];
            c0 = S.sC[p];
        }
        if (S.N > 1) {
            d1 = C == 3 ? ((const uint64_t*)S.sD)[(size_t)npx + p] : (uint64_t)((const uint16_t*)S.sD)[(size_t)npx + p];
            c1 = S.sC[(size_t)npx + p];
        }
    }
    uint8_t* tile = smem;
    uint8_t* lut = smem + RW * RH;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = S.ctl->lut[i];
    const long rowBytes = (long)S.W * C;
    const long ws = (long)(x0 - kBorder) * C - 2 - kTileDelta<C>;  // frame byte of a tile row buffer's byte 0
    const bool vecPath = (rowBytes & 15) == 0 && (((uintptr_t)S.frame) & 15) == 0;
    const bool wordPath = (rowBytes & 3) == 0 && (((uintptr_t)S.frame) & 3) == 0;
    for (int i = threadIdx.x; i < NCH * RH; i += blockDim.x) {
        const int r = i / NCH, ci = i % NCH;
        const int gy = y0 - kBorder + r;
        const long b = ws + 16 * ci;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (gy >= 0 && gy < S.H) {
            const uint8_t* row = S.frame + (size_t)gy * rowBytes;
            if (vecPath && b >= 0 && b + 16 <= rowBytes) {
                v = __ldg((const uint4*)(row + b));
            } else {
                uint32_t w[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const long bw = b + 4 * j;
                    w[j] = 0;
                    if (wordPath && bw >= 0 && bw + 4 <= rowBytes) {
                        w[j] = __ldg((const uint32_t*)(row + bw));
                    } else {
                        for (int k = 0; k < 4; ++k)
                            if (bw + k >= 0 && bw + k < rowBytes) w[j] |= (uint32_t)__ldg(row + bw + k) << (8 * k);
                    }
                }
                v = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        *(uint4*)(tile + r * RW + 16 * ci) = v;
    }
    __syncthreads();
    int nz = 0;
    bool defer = false;
    unsigned long long scanWord = 0;
    if (inFrame) {
        uint32_t intent = 0;
        if (active) {
            const uint8_t* base = tile + (ly + kBorder) * RW + kTileDelta<C> + (lx + kBorder) * C + 2;
            uint32_t vals[C][4], curr[C], intra[C];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                gather_taps<C>(base, RW, c, vals[c]);
                curr[c] = base[c];
                intra[c] = lbsp_thr(vals[c], curr[c], lut[curr[c]]);
            }
            nz = desc_nonzero<C>(intra);
            const EvalThr th = eval_thresholds(S, tR, tRwLT, tRwST, tFnLT, tFnST, tU);
            ScanSt st;
            scan_init<C>(st);
            // the first good sample's index is tracked (the long-scan record keeps it), not the distances
            // of the first two good samples (only a scan that ends unsettled records them)
            scan_samples<C, false, false>(S, lut, p, vals, curr, intra, th, nullptr, 0, 0ull, kScanCap, d0, c0, d1,
                                          c1, st);
            if (st.nGood < S.nreq) {
                // a long scan, or a scan that ended unsettled within the cap (N <= kScanCap): continued,
                // recorded and finished by lvbgs_k_longscan over the compacted list, so that its warps
                // hold only long scans
                defer = true;
                // s | nGood | first good index (255: none) | minDesc | minSum
                scanWord = (unsigned long long)st.s | ((unsigned long long)st.nGood << 8) |
                           ((unsigned long long)(st.g0 < 0 ? 255 : st.g0) << 16) |
                           ((unsigned long long)st.minDesc << 32) | ((unsigned long long)st.minSum << 48);
            } else {
                PixIn<C> in;
                load_pix<C>(S, F, p, in);
                intent = eval_tail<C>(S, F, x, y, p, in, curr, intra, th.uNew, st);
            }
        }
        __stcg(&S.intent[p], intent);
    }
    {
        // warp-aggregated append to the long-scan list (pixel key, scan state)
        const unsigned m = __ballot_sync(0xffffffffu, defer);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            unsigned int base = 0;
            if (lane == leader) base = atomicAdd(&P.work->lcount, (unsigned int)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (defer) {
                const unsigned int i = base + (unsigned int)__popc(m & ((1u << lane) - 1u));
                if (i < P.listCap) {
                    P.rlist[0][i] = ((unsigned long long)si << 40) | (unsigned long long)(unsigned)p;
                    P.rlist[1][i] = scanWord;
                } else {
                    atomicOr(&P.work->err, ERR_REPAIR_LIMIT);
                }
            }
        }
    }
    // per-warp reduction of the non-zero descriptor count (final: the descriptor does not depend
    // on the repair)
    for (int o = 16; o > 0; o >>= 1) nz += __shfl_xor_sync(0xffffffffu, nz, o);
    if ((threadIdx.x & 31) == 0 && nz) atomicAdd(&S.ctl->nz_acc, (unsigned long long)nz);
}

// ------------------------------------------------------------------------------------------
// list helpers for the repair loop
// ------------------------------------------------------------------------------------------
// push of one item from divergent code: the lanes that arrive together share one counter atomic
// (the counters are shared by all streams, and same-address atomics serialize)
__device__ __forceinline__ void push_item(unsigned long long* list, unsigned int* count, unsigned int cap,
                                          uint32_t* stamps, uint32_t stamp, int si, int p, TickWork* w) {
    if (atomicExch(&stamps[p], stamp) == stamp) return;
    const unsigned am = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(am) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(am));
    base = __shfl_sync(am, base, leader);
    const unsigned int i = base + (unsigned int)__popc(am & ((1u << lane) - 1u));
    if (i < cap) list[i] = ((unsigned long long)si << 40) | (unsigned long long)(unsigned)p;
    else atomicOr(&w->err, ERR_REPAIR_LIMIT);
}

// target pixel of a neighbour code relative to (x, y)
__device__ __forceinline__ int code_target(int code, int x, int y, int W) {
    const int dy = code / 5 - 2, dx = code % 5 - 2;
    return (y + dy) * W + (x + dx);
}

// ghost test of pixel p's neighbour update (:292-295 / :438-441), reading the target's values as
// the raster scan would: this frame's value when the target precedes (or is) p, else the previous
// frame's
__device__ __forceinline__ uint32_t resolve_ghost(const StreamDev& S, const FrameK& F, int p, int q) {
    const int npx = S.npx;
    const int buf = (q <= p) ? F.nxt : F.cur;
    const float* fb = S.fm + (size_t)buf * kNumFloatMaps * npx;
    const float qD = __ldcg(&fb[FM_DLAST * npx + q]);
    const float qR = __ldcg(&fb[FM_RAW_ST * npx + q]);
    return (qR > 0.995f && qD < 0.010f) ? NB_GHOST_WRITE : NB_GHOST_NO;
}

__device__ __forceinline__ uint32_t set_nst(uint32_t w, uint32_t st) {
    return (w & ~(7u << kInNStShift)) | (st << kInNStShift);
}

// phase B: resolve pending ghost tests with the phase-A values; mark the pixels whose evaluated
// samples an earlier pixel overwrites (initial repair frontier). A block takes kResolveTiles tiles,
// one pixel of each per thread, with the loads of all of them issued before any is used: the work
// is a short chain of dependent loads per pixel, so more pixels in flight per thread hide it.
__device__ void phaseB_tiles(const TickParams& P, int t0) {
    // the stream of each tile and its stamp, found once per block
    __shared__ int sSi[kResolveTiles];
    __shared__ uint32_t sStamp[kResolveTiles];
    if (threadIdx.x < kResolveTiles) {
        const int t = t0 + (int)threadIdx.x;
        int si = 0;
        uint32_t stamp = 0;
        if (t < P.totalTiles) {
            si = find_stream_by_tile(P, t);
            stamp = P.streams[si].ctl->stamp_base + 1u;
        }
        sSi[threadIdx.x] = si;
        sStamp[threadIdx.x] = stamp;
    }
    __syncthreads();
    uint32_t w[kResolveTiles];
    int ps[kResolveTiles], xs[kResolveTiles], ys[kResolveTiles];
#pragma unroll
    for (int j = 0; j < kResolveTiles; ++j) {
        const int t = t0 + j;
        w[j] = 0u;
        ps[j] = xs[j] = ys[j] = 0;
        if (t < P.totalTiles) {
            const StreamDev& S = P.streams[sSi[j]];
            const int lt = t - S.tileBase;
            const int x = (lt % S.tilesX) * kTileW + threadIdx.x % kTileW;
            const int y = (lt / S.tilesX) * kTileH + threadIdx.x / kTileW;
            xs[j] = x;
            ys[j] = y;
            if (x < S.W && y < S.H) {
                ps[j] = y * S.W + x;
                w[j] = __ldcg(&S.intent[ps[j]]);
            }
        }
    }
    int qs[kResolveTiles];
    uint32_t wq[kResolveTiles];
#pragma unroll
    for (int j = 0; j < kResolveTiles; ++j) {
        qs[j] = 0;
        wq[j] = 0u;
        if (!(w[j] & kInValid)) continue;
        const StreamDev& S = P.streams[sSi[j]];
        if (in_nst(w[j]) == NB_PENDING) {
            const FrameK F = frame_consts(S);
            w[j] = set_nst(w[j], resolve_ghost(S, F, ps[j], code_target((int)in_code(w[j]), xs[j], ys[j], S.W)));
            __stcg(&S.intent[ps[j]], w[j]);
        }
        if (in_nb_writes(w[j])) {
            qs[j] = code_target((int)in_code(w[j]), xs[j], ys[j], S.W);
            if (qs[j] > ps[j]) wq[j] = __ldcg(&S.intent[qs[j]]);
        }
    }
#pragma unroll
    for (int j = 0; j < kResolveTiles; ++j) {
        if (t0 + j >= P.totalTiles) break;  // uniform over the block
        const bool want = (w[j] & kInValid) && in_nb_writes(w[j]) && qs[j] > ps[j] && (wq[j] & kInValid) &&
                          in_snb(w[j]) < in_e(wq[j]);
        // one list item per target and stamp generation; slots reserved once per block
        const bool ok = want && atomicExch(&P.streams[sSi[j]].stampD[qs[j]], sStamp[j]) != sStamp[j];
        const unsigned int i = block_reserve(ok, &P.work->dcount[0]);
        if (ok) {
            if (i < P.listCap) P.dlist[0][i] = ((unsigned long long)sSi[j] << 40) | (unsigned long long)(unsigned)qs[j];
            else atomicOr(&P.work->err, ERR_REPAIR_LIMIT);
        }
    }
}

// frame down-sampling for the frame-level analysis (:568-584): one output pixel per thread
__device__ void ds_item(const StreamDev& S, int i) {
    const int C = S.C;
    const int dx = i % S.dsW, dy = i / S.dsW;
    const FrameK F = frame_consts(S);
    uint32_t dmax = 0;
    for (int c = 0; c < C; ++c) {
        const uint8_t* fr = S.frame;
        const int W = S.W;
        const int v = area_resample(S.W, S.H, S.dsW, S.dsH, dx, dy,
                                    [&](int sx, int sy) { return (int)__ldg(fr + ((size_t)sy * W + sx) * C + c); });
        const size_t k = (size_t)i * C + c;
        // accumulateWeighted: dst = src*a + dst*(1-a)
        const float aL = F.fLT, bL = 1.0f - aL, aS = F.fST, bS = 1.0f - aS;
        const float lt = (float)v * aL + S.dsLT[k] * bL;
        const float st = (float)v * aS + S.dsST[k] * bS;
        S.dsLT[k] = lt;
        S.dsST[k] = st;
        const uint32_t d = (uint32_t)__float2ull_rz(fabsf(st - lt));
        if (C == 1) dmax = d / 2u;
        else dmax = c == 0 ? d : (d > dmax ? d : dmax);
    }
    // reference order: max(d0, max(d1, d2)) -- identical to the running max for integers
    if (dmax) atomicAdd(&S.ctl->colordiff_acc, (unsigned long long)dmax);
}

// ------------------------------------------------------------------------------------------
// repair loop bodies
// ------------------------------------------------------------------------------------------
template <int C>
__device__ bool rematch_item(const TickParams& P, int si, const StreamDev& S, int q, uint32_t stampNext,
                             int iterParity) {
    const int W = S.W, x = q % W, y = q / W;
    const FrameK F = frame_consts(S);
    const uint32_t wOld = __ldcg(&S.intent[q]);
    if (!(wOld & kInValid)) return false;
    // overrides: earlier pixels of the 5x5 window whose neighbour update targets q, raster order
    Ovr ov[12];
    int nov = 0;
    uint64_t mask = 0;
    for (int dy = -2; dy <= 0; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
            if (dy == 0 && dx >= 0) break;
            const int px = x + dx, py = y + dy;
            if (px < 0 || px >= W || py < 0) continue;
            const int p = py * W + px;
            const uint32_t w = __ldcg(&S.intent[p]);
            if (!in_nb_writes(w) || (int)in_code(w) != (-dy + 2) * 5 + (-dx + 2)) continue;
            const int sn = (int)in_snb(w);
            uint32_t col = 0;
            uint64_t desc = 0;
            const uint16_t* ldn = S.lastDesc + (size_t)F.nxt * S.npx * C + (size_t)p * C;
            for (int c = 0; c < C; ++c) {
                col |= (uint32_t)__ldg(S.frame + (size_t)p * C + c) << (8 * c);
                desc |= (uint64_t)__ldcg(&ldn[c]) << (16 * c);
            }
            int k = 0;
            while (k < nov && ov[k].s != sn) ++k;
            if (k == nov) ++nov;
            ov[k].s = sn;
            ov[k].col = col;
            ov[k].desc = desc;
            mask |= 1ull << sn;
        }
    // order matters only within one sample index (last writer wins); entries with distinct s are
    // independent, and an overwritten entry keeps its slot but takes the latest writer's values
    uint32_t vals[C][4], curr[C], intra[C];
    const uint8_t* base = S.frame + (size_t)q * C;
    for (int c = 0; c < C; ++c) {
        for (int j = 0; j < 4; ++j) {
            uint32_t wv = 0;
            for (int i = 0; i < 4; ++i) {
                const int n = j * 4 + i;
                wv |= (uint32_t)__ldg(base + (c_lbsp_dy[n] * W + c_lbsp_dx[n]) * C + c) << (8 * i);
            }
            vals[c][j] = wv;
        }
        curr[c] = __ldg(base + c);
        intra[c] = lbsp_thr(vals[c], curr[c], S.ctl->lut[curr[c]]);
    }
    int e = 0;
    PixIn<C> in;
    load_pix<C>(S, F, q, in);
    uint32_t wNew;
    const uint4 gr = S.nreq <= 2 ? __ldcg(&S.goodRec[q]) : make_uint4(0u, 0u, 0u, 0u);
    if (S.nreq <= 2 && gr.x == F.frame) {
        // q's frame-start scan is recorded: up to its stop eA, its good samples are the recorded ones
        // not overwritten and the overwritten ones that match now. The ordered scan over them stops
        // at the nreq-th good index, with minima over the good samples up to there; with fewer, it
        // goes on from eA (with the overwrites) as a scan from the start would.
        const EvalThr th = eval_thresholds(S, in.R, in.RwLT, in.RwST, in.FnLT, in.FnST, in.uOld);
        const int eA = (int)(gr.y & 255u), nA = (int)((gr.y >> 8) & 255u);
        int gi[2] = {S.N, S.N};  // the two smallest good indices
        uint32_t gd[2] = {0u, 0u}, gs[2] = {0u, 0u};
        int cnt = 0;
        auto add = [&](int idx, uint32_t dd, uint32_t sd) {
            ++cnt;
            if (idx < gi[0]) {
                gi[1] = gi[0];
                gd[1] = gd[0];
                gs[1] = gs[0];
                gi[0] = idx;
                gd[0] = dd;
                gs[0] = sd;
            } else if (idx < gi[1]) {
                gi[1] = idx;
                gd[1] = dd;
                gs[1] = sd;
            }
        };
        for (int j = 0; j < nA; ++j) {
            const int g = (int)((gr.y >> (16 + 8 * j)) & 255u);
            if (!((mask >> g) & 1ull)) add(g, (j ? gr.z >> 16 : gr.z) & 0xffffu, (j ? gr.w >> 16 : gr.w) & 0xffffu);
        }
        for (int k = 0; k < nov; ++k) {
            if (ov[k].s >= eA) continue;
            uint64_t d;
            uint32_t c2;
            if (C == 3) {
                d = ov[k].desc | ((uint64_t)(ov[k].col & 0xffffu) << 48);
                c2 = (ov[k].col >> 16) & 0xffu;
            } else {
                d = ov[k].desc & 0xffffu;
                c2 = ov[k].col & 0xffu;
            }
            uint32_t dd, sd;
            if (sample_match<C>(S.ctl->lut, vals, curr, intra, th, d, c2, dd, sd)) add(ov[k].s, dd, sd);
        }
        ScanSt st;
        scan_init<C>(st);
        const int take = cnt < S.nreq ? cnt : S.nreq;
        for (int j = 0; j < take; ++j) {
            if (st.minDesc > gd[j]) st.minDesc = gd[j];
            if (st.minSum > gs[j]) st.minSum = gs[j];
        }
        st.nGood = take;
        if (cnt >= S.nreq) {
            st.s = gi[S.nreq - 1] + 1;
        } else {
            st.s = eA;
            if (eA < S.N) {
                const int npx = S.npx;
                uint64_t dA = 0, dB = 0;
                uint32_t cA = 0, cB = 0;
                dA = C == 3 ? ((const uint64_t*)S.sD)[(size_t)eA * npx + q] : (uint64_t)((const uint16_t*)S.sD)[(size_t)eA * npx + q];
                cA = S.sC[(size_t)eA * npx + q];
                if (eA + 1 < S.N) {
                    dB = C == 3 ? ((const uint64_t*)S.sD)[(size_t)(eA + 1) * npx + q]
                                : (uint64_t)((const uint16_t*)S.sD)[(size_t)(eA + 1) * npx + q];
                    cB = S.sC[(size_t)(eA + 1) * npx + q];
                }
                scan_samples<C, true>(S, S.ctl->lut, q, vals, curr, intra, th, ov, nov, mask, S.N, dA, cA, dB, cB, st);
            }
        }
        e = st.s;
        wNew = eval_tail<C>(S, F, x, y, q, in, curr, intra, th.uNew, st);
    } else {
        wNew = eval_pixel<C, true>(S, F, S.ctl->lut, x, y, q, in, vals, curr, intra, ov, nov, mask, e);
    }
    const bool decChanged = ((wNew ^ wOld) & kInFG) != 0u;
    if (!decChanged) {
        // same decision: same draws, same updates; keep the resolved neighbour state
        wNew = (wOld & ~(127u << kInEShift)) | ((uint32_t)e << kInEShift);
        __stcg(&S.intent[q], wNew);
        return true;
    }
    __stcg(&S.intent[q], wNew);
    unsigned int* dcnt = &P.work->dcount[iterParity ^ 1];
    unsigned long long* dl = P.dlist[iterParity ^ 1];
    // the write that disappeared or appeared changes what its (later) target reads
    if (in_nb_writes(wOld)) {
        const int t = code_target((int)in_code(wOld), x, y, W);
        if (t > q) push_item(dl, dcnt, P.listCap, S.stampD, stampNext, si, t, P.work);
    }
    if (in_nb_writes(wNew)) {
        const int t = code_target((int)in_code(wNew), x, y, W);
        if (t > q) push_item(dl, dcnt, P.listCap, S.stampD, stampNext, si, t, P.work);
    }
    // the raw-segmentation value of q changed: re-resolve ghost tests that read it (q itself and
    // later pixels of its 5x5 window), and q's own new pending test
    unsigned long long* rl = P.rlist[iterParity];
    unsigned int* rcnt = &P.work->rcount[iterParity];
    const uint32_t rstamp = stampNext;  // separate stamp array: one generation per iteration
    for (int dy = 0; dy <= 2; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
            if (dy == 0 && dx < 0) continue;
            const int px = x + dx, py = y + dy;
            if (px < 0 || px >= W || py >= S.H) continue;
            const int p = py * W + px;
            const uint32_t w = (p == q) ? wNew : __ldcg(&S.intent[p]);
            if (in_ghost(w) && code_target((int)in_code(w), px, py, W) == q)
                push_item(rl, rcnt, P.listCap, S.stampR, rstamp, si, p, P.work);
        }
    if (in_nst(wNew) == NB_PENDING) push_item(rl, rcnt, P.listCap, S.stampR, rstamp, si, q, P.work);
    return true;
}

__device__ void reresolve_item(const TickParams& P, int si, const StreamDev& S, int p, uint32_t stampNext,
                               int iterParity) {
    const int W = S.W, x = p % W, y = p / W;
    const uint32_t w = __ldcg(&S.intent[p]);
    if (!in_ghost(w)) return;
    const FrameK F = frame_consts(S);
    const int q = code_target((int)in_code(w), x, y, W);
    const uint32_t st = resolve_ghost(S, F, p, q);
    const uint32_t old = in_nst(w);
    if (st == old) return;
    __stcg(&S.intent[p], set_nst(w, st));
    // readers during the last re-match pass saw PENDING as "no write"
    const bool wroteBefore = old == NB_GHOST_WRITE, writesNow = st == NB_GHOST_WRITE;
    if (wroteBefore != writesNow && q > p)
        push_item(P.dlist[iterParity ^ 1], &P.work->dcount[iterParity ^ 1], P.listCap, S.stampD, stampNext, si, q,
                  P.work);
}

// ------------------------------------------------------------------------------------------
// phase F: commit the sample writes of the frame in raster order, the draw counters, the blink
// maps and the 3x3 closing (:536-540); initializes the union-find labels of the hole filling
// ------------------------------------------------------------------------------------------
template <int C>
__device__ void phaseF_tile(const TickParams& P, const StreamDev& S, int lt, uint8_t* smem) {
    const int tx = lt % S.tilesX, ty = lt / S.tilesX;
    const int x0 = tx * kTileW, y0 = ty * kTileH;
    constexpr int IW = kTileW + 4, IH = kTileH + 4;  // intents with a 2-pixel halo
    uint32_t* it = (uint32_t*)smem;
    uint8_t* dil = smem + IW * IH * 4;  // (kTileW+2) x (kTileH+2) dilated raw mask
    const int W = S.W, H = S.H, npx = S.npx;
    const int lx0 = threadIdx.x % kTileW, ly0 = threadIdx.x / kTileW;
    const bool inF = x0 + lx0 < W && y0 + ly0 < H;
    const int q0 = (y0 + ly0) * W + x0 + lx0;
    const uint8_t lastRaw = inF ? S.lastRawFG[q0] : 0, lastRawBlink = inF ? S.lastRawBlink[q0] : 0;
    for (int i = threadIdx.x; i < IW * IH; i += blockDim.x) {
        const int gy = y0 - 2 + i / IW, gx = x0 - 2 + i % IW;
        it[i] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? __ldcg(&S.intent[gy * W + gx]) : 0u;
    }
    __syncthreads();
    // 3x3 dilation of the raw mask (out-of-frame pixels never win)
    for (int i = threadIdx.x; i < (kTileW + 2) * (kTileH + 2); i += blockDim.x) {
        const int ry = i / (kTileW + 2), rx = i % (kTileW + 2);
        uint32_t v = 0;
        for (int dy = 0; dy < 3; ++dy)
            for (int dx = 0; dx < 3; ++dx) v |= it[(ry + dy) * IW + rx + dx] & kInFG;
        dil[i] = v ? 255 : 0;
    }
    __syncthreads();
    const FrameK F = frame_consts(S);
    const int lx = threadIdx.x % kTileW, ly = threadIdx.x / kTileW;
    const int x = x0 + lx, y = y0 + ly;
    int nw = 0, ne = 0;
    bool rawBit = false, closedBit = false;
    if (x < W && y < H) {
        const int q = y * W + x;
        // raster-ordered commit of every write targeting q (own write before own neighbour write).
        // A writer at window slot k = (dy+2)*5 + (dx+2) targets q iff it is valid, its neighbour
        // state is WRITE or GHOST_WRITE (state & 5 == 1) and its code is 24 - k.
        constexpr uint32_t kNbMask = kInValid | (31u << kInCodeShift) | (5u << kInNStShift);
        auto commit_write = [&](int p, int s) {
            const uint16_t* ldn = S.lastDesc + (size_t)F.nxt * npx * C + (size_t)p * C;
            if (C == 3) {
                // the writers' descriptors were written by earlier kernels of the tick and are not
                // written by this one, so they are read through L1 (neighbouring writers share lines)
                const uint64_t d = (uint64_t)__ldg(&ldn[0]) | ((uint64_t)__ldg(&ldn[1]) << 16) |
                                   ((uint64_t)__ldg(&ldn[2]) << 32) | ((uint64_t)__ldg(S.frame + (size_t)p * 3) << 48) |
                                   ((uint64_t)__ldg(S.frame + (size_t)p * 3 + 1) << 56);
                ((uint64_t*)S.sD)[(size_t)s * npx + q] = d;
                S.sC[(size_t)s * npx + q] = __ldg(S.frame + (size_t)p * 3 + 2);
            } else {
                ((uint16_t*)S.sD)[(size_t)s * npx + q] = __ldg(&ldn[0]);
                S.sC[(size_t)s * npx + q] = __ldg(S.frame + p);
            }
            ++nw;
        };
        // the writes targeting q, in raster order of their writers, packed 12 bits each (window slot,
        // sample index, own write) into a register list, then executed by the warp together: a write
        // body per list position instead of one per window slot that any lane uses. More than five
        // writes (rare) take the slot loop.
        unsigned long long wlist = 0;
        int nwr = 0;
#pragma unroll
        for (int k = 0; k < 25; ++k) {
            const int dy = k / 5 - 2, dx = k % 5 - 2;
            const uint32_t w = it[(ly + 2 + dy) * IW + lx + 2 + dx];
            if (k == 12 && (w & kInValid) && (w & kInOwn)) {
                if (nwr < 5) wlist |= (unsigned long long)(2048u | (12u << 6) | in_sown(w)) << (12 * nwr);
                ++nwr;
            }
            if ((w & kNbMask) == (kInValid | ((uint32_t)(24 - k) << kInCodeShift) | (1u << kInNStShift))) {
                if (nwr < 5) wlist |= (unsigned long long)(((uint32_t)k << 6) | in_snb(w)) << (12 * nwr);
                ++nwr;
            }
        }
        const int nconv = nwr <= 5 ? nwr : 0;
        const int iters = __reduce_max_sync(__activemask(), (unsigned)nconv);
        for (int j = 0; j < iters; ++j) {
            if (j < nconv) {
                const uint32_t e = (uint32_t)(wlist >> (12 * j)) & 0xfffu;
                const int k = (int)((e >> 6) & 31u), sidx = (int)(e & 63u);
                const int p = (e & 2048u) ? q : (y + k / 5 - 2) * W + (x + k % 5 - 2);
                commit_write(p, sidx);
            }
        }
        if (nwr > 5) {
            for (int k = 0; k < 25; ++k) {
                const int dy = k / 5 - 2, dx = k % 5 - 2;
                const uint32_t w = it[(ly + 2 + dy) * IW + lx + 2 + dx];
                if (k == 12 && (w & kInValid) && (w & kInOwn)) commit_write(q, (int)in_sown(w));
                if ((w & kNbMask) == (kInValid | ((uint32_t)(24 - k) << kInCodeShift) | (1u << kInNStShift)))
                    commit_write((y + dy) * W + (x + dx), (int)in_snb(w));
            }
        }
        const uint32_t wq = it[(ly + 2) * IW + lx + 2];
        uint16_t kend = 0;
        ne = (int)in_e(wq);
        if (wq & kInValid) {
            if (wq & kInFG) kend = F.cooldown ? (uint16_t)(1 + ((wq & kInOwn) ? 1 : 0)) : 0;
            else kend = (uint16_t)(1 + ((wq & kInOwn) ? 1 : 0) + 2 + (in_nb_writes(wq) ? 1 : 0));
        }
        S.kctr[q] = kend;
        // blinks (:536-539)
        const uint8_t raw = (wq & kInFG) ? 255 : 0;
        const uint8_t cb = raw ^ lastRaw;
        S.blinks[q] = cb | lastRawBlink;
        S.lastRawBlink[q] = cb;
        S.lastRawFG[q] = raw;
        rawBit = raw != 0;
        // closing: erosion of the dilated mask (out-of-frame pixels never win)
        uint8_t v = 255;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int gx = x + dx, gy = y + dy;
                if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
                v &= dil[(ly + 1 + dy) * (kTileW + 2) + lx + 1 + dx];
            }
        closedBit = v != 0;
    }
    // each warp is one 32-pixel tile row: its ballots are the row's words of the raw and closed masks
    static_assert(kTileW == 32, "tile rows are bit-plane words");
    const unsigned rawW = __ballot_sync(0xffffffffu, rawBit), closedW = __ballot_sync(0xffffffffu, closedBit);
    if (lx == 0 && y < H) {
        const size_t o = (size_t)y * S.rowWords + tx;
        bit_plane(S, BP_RAW)[o] = rawW;
        bit_plane(S, BP_CLOSED)[o] = closedW;
    }
    block_add_stats(&S.ctl->st_writes, (unsigned long long)nw, &S.ctl->st_samples, (unsigned long long)ne);
}

// ------------------------------------------------------------------------------------------
// hole filling: cv::floodFill(closed, (0,0), 255) + bitwise_not (:541-543), rebuilt as union-find
// over the runs of 0-pixels of each row. The closed mask is 0 on the 2-pixel frame border (no ROI
// pixel lies there, and a 3x3 closing cannot reach it), so the flood-filled region is the
// 4-connected component of 0-pixels that contains that border ring. Every row's first and last
// run touch the ring and link straight to root 0; interior runs are united with the runs they
// overlap in the row above. Holes are the 0-pixels whose run's root is not 0.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int uf_find(int* L, int a, TickWork* w) {
    int n, it = 0;
    while ((n = __ldcg(&L[a])) != a) {
        a = n;
        if (++it > kUFLimit) {
            atomicOr(&w->err, ERR_UF_LIMIT);
            break;
        }
    }
    return a;
}
__device__ void uf_union(int* L, int a, int b, TickWork* w) {
    for (int it = 0; it < kUFLimit; ++it) {
        a = uf_find(L, a, w);
        b = uf_find(L, b, w);
        if (a == b) return;
        if (a < b) {
            const int old = atomicMin(&L[b], a);
            if (old == b) return;
            b = old;
        } else {
            const int old = atomicMin(&L[a], b);
            if (old == a) return;
            a = old;
        }
    }
    atomicOr(&w->err, ERR_UF_LIMIT);
}

// run start (x of the first pixel of the run of set bits) for each lane of a 32-pixel chunk
struct RunTracker {
    uint32_t carry;   // bit 31 of the previous chunk
    int prevStart;    // start of the run that reached the end of the previous chunk
    __device__ __forceinline__ void reset() {
        carry = 0;
        prevStart = -1;
    }
    // returns the run start of this lane (undefined when its bit is 0) and advances
    __device__ __forceinline__ int step(uint32_t ball, int x0, int lane) {
        const uint32_t starts = ball & ~((ball << 1) | carry);
        const uint32_t upto = starts & (0xffffffffu >> (31 - lane));
        const int rs = upto ? x0 + 31 - __clz(upto) : prevStart;
        const int rs31 = __shfl_sync(0xffffffffu, rs, 31);
        if (ball >> 31) prevStart = rs31;
        carry = ball >> 31;
        return rs;
    }
};

__device__ __forceinline__ int find_stream_by_row(const TickParams& P, int r) {
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.streams[mid].rowBase <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// bits of word w that lie inside a frame of width W
__device__ __forceinline__ uint32_t valid_bits(int w, int W) {
    const int n = W - 32 * w;
    return n >= 32 ? 0xffffffffu : (n <= 0 ? 0u : (1u << n) - 1u);
}

// runs pass: initializes the label of each run start (0 for runs touching the border ring)
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_runs(TickParams P) {
    const int gr = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W, H = S.H;
    const uint32_t* row = bit_plane(S, BP_CLOSED) + (size_t)y * S.rowWords;
    RunTracker rt;
    rt.reset();
    int last = -1;
    bool ringOk = true;
    for (int x0 = 0; x0 < W; x0 += 32) {
        const int x = x0 + lane;
        const uint32_t ball = ~__ldcg(&row[x0 >> 5]) & valid_bits(x0 >> 5, W);  // 0-pixels of the chunk
        const bool z = (ball >> lane) & 1u;
        if (x < W && (x < 2 || x >= W - 2 || y < 2 || y >= H - 2) && !z) ringOk = false;
        const uint32_t starts = ball & ~((ball << 1) | rt.carry);
        const int rs = rt.step(ball, x0, lane);
        if ((starts >> lane) & 1u) {
            const int idx = y * W + x;
            S.label[idx] = (x == 0 || y == 0 || y == H - 1) ? 0 : idx;
        }
        if (z) last = rs;
    }
    // the last run of the row reaches x = W-1, on the ring (held by the lane that read x = W-1)
    const int lastRun = __shfl_sync(0xffffffffu, last, (W - 1) & 31);
    if (lane == 0 && lastRun >= 0) S.label[y * W + lastRun] = 0;
    if (__any_sync(0xffffffffu, !ringOk) && lane == 0) atomicOr(&P.work->err, ERR_RING);
}

// vertical pass: unites each run with the runs it overlaps in the row above
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_vunion(TickParams P) {
    const int gr = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W;
    if (y == 0) return;
    const uint32_t* row = bit_plane(S, BP_CLOSED) + (size_t)y * S.rowWords;
    const uint32_t* up = row - S.rowWords;
    RunTracker rc, ru;
    rc.reset();
    ru.reset();
    uint32_t ovCarry = 0;
    for (int x0 = 0; x0 < W; x0 += 32) {
        const uint32_t vb = valid_bits(x0 >> 5, W);
        const uint32_t bc = ~__ldcg(&row[x0 >> 5]) & vb, bu = ~__ldcg(&up[x0 >> 5]) & vb;
        const int rsc = rc.step(bc, x0, lane), rsu = ru.step(bu, x0, lane);
        const uint32_t ov = bc & bu;
        const uint32_t segStarts = ov & ~((ov << 1) | ovCarry);
        ovCarry = ov >> 31;
        if ((segStarts >> lane) & 1u) uf_union(S.label, y * W + rsc, (y - 1) * W + rsu, P.work);
    }
}

// holes pass: the 0-pixels whose run is not connected to the ring
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_holes(TickParams P) {
    const int gr = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W;
    const uint32_t* row = bit_plane(S, BP_CLOSED) + (size_t)y * S.rowWords;
    uint32_t* holes = bit_plane(S, BP_HOLES) + (size_t)y * S.rowWords;
    // one root lookup per run: at the lane where the run starts; a run that continues from the
    // previous chunk keeps that chunk's answer
    uint32_t carry = 0;
    bool carryHole = false;
    for (int x0 = 0; x0 < W; x0 += 32) {
        const uint32_t ball = ~__ldcg(&row[x0 >> 5]) & valid_bits(x0 >> 5, W);
        const uint32_t starts = ball & ~((ball << 1) | carry);
        const bool isStart = (starts >> lane) & 1u;
        const bool h = isStart && uf_find(S.label, y * W + x0 + lane, P.work) != 0;
        const uint32_t upto = starts & (0xffffffffu >> (31 - lane));
        const int src = upto ? 31 - __clz(upto) : 0;
        const bool hs = __shfl_sync(0xffffffffu, h, src);
        const bool hole = ((ball >> lane) & 1u) && (upto ? hs : carryHole);
        const uint32_t hw = __ballot_sync(0xffffffffu, hole);
        if (lane == 0) holes[x0 >> 5] = hw;
        carryHole = (hw >> 31) & 1u;
        carry = ball >> 31;
    }
}

// word w of a bit-plane row with the pixels outside [0, W) set to fill (0 or ~0)
__device__ __forceinline__ uint32_t row_word(const uint32_t* row, int w, int RW, int W, uint32_t fill) {
    if (w < 0 || w >= RW) return fill;
    const uint32_t vb = valid_bits(w, W);
    return (__ldcg(&row[w]) & vb) | (fill & ~vb);
}

// 7-pixel horizontal AND (erode) or OR (dilate) of word w of a row; pixels outside the frame take
// the value that never wins
template <bool AND>
__device__ __forceinline__ uint32_t row_box7(const uint32_t* row, int w, int RW, int W) {
    const uint32_t fill = AND ? 0xffffffffu : 0u;
    const uint32_t L = row_word(row, w - 1, RW, W, fill), C = row_word(row, w, RW, W, fill),
                   R = row_word(row, w + 1, RW, W, fill);
    uint32_t v = C;
#pragma unroll
    for (int d = 1; d <= 3; ++d) {
        const uint32_t a = __funnelshift_r(C, R, d), b = __funnelshift_l(L, C, d);  // pixels x+d, x-d
        v = AND ? (v & a & b) : (v | a | b);
    }
    return v;
}

// 3-fold 3x3 erosion of the closed mask (a clipped 7x7 minimum) and mask |= holes | eroded (:544-546);
// one warp per row, one thread per 32-pixel word
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_combine(TickParams P) {
    const int gr = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W, H = S.H, RW = S.rowWords;
    const uint32_t* closed = bit_plane(S, BP_CLOSED);
    for (int w = lane; w < RW; w += 32) {
        uint32_t er = 0xffffffffu;
        for (int yy = max(0, y - 3); yy <= min(H - 1, y + 3); ++yy) er &= row_box7<true>(closed + (size_t)yy * RW, w, RW, W);
        const size_t o = (size_t)y * RW + w;
        bit_plane(S, BP_COMB)[o] = (__ldcg(&bit_plane(S, BP_RAW)[o]) | __ldcg(&bit_plane(S, BP_HOLES)[o]) | er) & valid_bits(w, W);
    }
}

// median, part 1: for each pixel, the number of set pixels of the combined mask in its row window
// [x - r, x + r] (replicate border: pixels left of 0 / right of W-1 repeat those two pixels); one
// block per row, four 32-pixel words per warp step
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_hcount(TickParams P) {
    const int gr = blockIdx.x, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W, RW = S.rowWords;
    const int r = S.ctl->median_k / 2;  // <= 15
    const uint32_t* row = bit_plane(S, BP_COMB) + (size_t)y * RW;
    const uint32_t lastFill = ((__ldcg(&row[(W - 1) >> 5]) >> ((W - 1) & 31)) & 1u) ? 0xffffffffu : 0u;
    const uint32_t firstFill = (__ldcg(&row[0]) & 1u) ? 0xffffffffu : 0u;
    const unsigned long long win = (2ull << (2 * r)) - 1ull;
    const int nw = blockDim.x >> 5;
    for (int w0 = (threadIdx.x >> 5) * 4; w0 < RW; w0 += 4 * nw) {
        // words w0-1 .. w0+4 first, then the four words' counts
        uint32_t v[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const int w = w0 - 1 + j;
            v[j] = w < 0 ? firstFill : row_word(row, w, RW, W, lastFill);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // bits 16..79 of the 96-bit row segment L | C | R: pixel x - r is bit 16 + lane - r
            const unsigned long long M =
                ((unsigned long long)v[j + 2] << 48) | ((unsigned long long)v[j + 1] << 16) | (v[j] >> 16);
            const int x = 32 * (w0 + j) + lane;
            if (x < W) S.hcount[(size_t)y * W + x] = (uint8_t)__popcll((M >> (16 + lane - r)) & win);
        }
    }
}

// median, part 2 (:547, :552-554): binary median blur (majority of the k x k window, replicate border)
// of the combined mask -> final mask, its row words, and the final-segmentation EMAs (addWeighted).
// One thread per pixel column of a 64-row segment, sliding the window sum down the rows.
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_median(TickParams P) {
    const int gs = blockIdx.y;
    if (gs >= P.totalSegs) return;
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.streams[mid].segBase <= gs) lo = mid;
        else hi = mid - 1;
    }
    const StreamDev& S = P.streams[lo];
    const int W = S.W, H = S.H, npx = S.npx;
    const int x0 = blockIdx.x * 256;
    if (x0 >= W) return;
    const int x = x0 + threadIdx.x, lane = threadIdx.x & 31;
    const bool in = x < W;
    const int y0 = (gs - S.segBase) * kMedSegRows, y1 = min(H, y0 + kMedSegRows);
    const int k = S.ctl->median_k, r = k / 2;
    const FrameK F = frame_consts(S);
    const float* fcur = S.fm + (size_t)F.cur * kNumFloatMaps * npx;
    float* fn = S.fm + (size_t)F.nxt * kNumFloatMaps * npx;
    const float aL = 1.0f - F.fLT, bL = S.ctl->bLT;
    const float aS = 1.0f - F.fST, bS = S.ctl->bST;
    const uint8_t* hc = S.hcount + (in ? x : 0);
    int sum = 0;
    if (in)
        for (int yy = y0 - r; yy <= y0 + r; ++yy) sum += __ldcg(&hc[(size_t)min(max(yy, 0), H - 1) * W]);
    uint32_t* fgRow = bit_plane(S, BP_FG) + (x0 >> 5) + (threadIdx.x >> 5);
    // four rows per step: every load of the step is issued before its stores
    for (int yb = y0; yb < y1; yb += 4) {
        int add[4], sub[4];
        float fl[4], fs[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int y = yb + j;
            add[j] = sub[j] = 0;
            fl[j] = fs[j] = 0.0f;
            if (in && y < y1) {
                const int q = y * W + x;
                add[j] = __ldcg(&hc[(size_t)min(y + r + 1, H - 1) * W]);
                sub[j] = __ldcg(&hc[(size_t)max(y - r, 0) * W]);
                fl[j] = fcur[FM_FIN_LT * npx + q];
                fs[j] = fcur[FM_FIN_ST * npx + q];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int y = yb + j;
            if (y >= y1) break;
            const bool fg = in && 2 * sum > k * k;
            const unsigned ball = __ballot_sync(0xffffffffu, fg);
            if (in) {
                const int q = y * W + x;
                const uint8_t fgv = fg ? 255 : 0;
                __stcg(&S.lastFG[q], fgv);
                if (S.maskOut) S.maskOut[q] = fgv;
                const float m = (float)fgv;
                fn[FM_FIN_LT * npx + q] = (fl[j] * aL + m * bL) + 0.0f;
                fn[FM_FIN_ST * npx + q] = (fs[j] * aS + m * bS) + 0.0f;
                sum += add[j] - sub[j];
            }
            if (lane == 0 && x < W) fgRow[(size_t)y * S.rowWords] = ball;
        }
    }
}

// 3-fold 3x3 dilation of the final mask (a clipped 7x7 maximum) and blink masking with the previous
// and the new inverted dilated masks (:548-551); one block per row, four 32-pixel words per warp step,
// one lane per pixel of each
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_dilate(TickParams P) {
    const int gr = blockIdx.x, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const StreamDev& S = P.streams[find_stream_by_row(P, gr)];
    const int y = gr - S.rowBase, W = S.W, H = S.H, RW = S.rowWords;
    const uint32_t* fgp = bit_plane(S, BP_FG);
    const int nw = blockDim.x >> 5;
    for (int w0 = (threadIdx.x >> 5) * 4; w0 < RW; w0 += 4 * nw) {
        // lane l < 28 dilates row y - 3 + l/4 of word w0 + l%4; an OR over the lanes of equal l%4
        const int j = lane & 3, yy = y - 3 + (lane >> 2);
        uint32_t d = 0;
        if (lane < 28 && yy >= 0 && yy < H && w0 + j < RW) d = row_box7<false>(fgp + (size_t)yy * RW, w0 + j, RW, W);
        d |= __shfl_xor_sync(0xffffffffu, d, 4);
        d |= __shfl_xor_sync(0xffffffffu, d, 8);
        d |= __shfl_xor_sync(0xffffffffu, d, 16);
        uint32_t dw[4];
        uint8_t bl[4], di[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            dw[i] = __shfl_sync(0xffffffffu, d, i);
            const int x = 32 * (w0 + i) + lane;
            bl[i] = di[i] = 0;
            if (x < W) {
                bl[i] = S.blinks[y * W + x];
                di[i] = S.dilInv[y * W + x];
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int x = 32 * (w0 + i) + lane;
            if (x < W) {
                const uint8_t inv = ((dw[i] >> lane) & 1u) ? 0 : 255;
                S.blinks[y * W + x] = (uint8_t)(bl[i] & di[i] & inv);
                S.dilInv[y * W + x] = inv;
            }
        }
    }
}

// frame-level epilogue of one stream (:555-611): LBSP threshold LUT adaptation, camera-motion
// analysis, automatic model reset decision and learning-rate caps
__device__ void stream_epilogue(const TickParams& P, const StreamDev& S) {
    StreamCtl* ctl = S.ctl;
    const float relThr = S.relThr;
    const unsigned int lbspOff = S.lbspOff;
    const unsigned long long nz = ctl->nz_acc;
    ctl->last_nz = nz;
    ctl->nz_acc = 0;
    const float ratio = __ull2float_rn(nz) / __ull2float_rn(ctl->n_rel);
    const float last = ctl->last_nz_ratio;
    if (ratio < 0.100f && last < 0.100f) {
        for (int t = 0; t <= 255; ++t) {
            const float v = ceilf((float)t * relThr / 4) + (float)lbspOff;
            const int lim = v > 255.0f ? 255 : (int)v;
            if ((int)ctl->lut[t] > lim) --ctl->lut[t];
        }
    } else if (ratio > 0.500f && last > 0.500f) {
        int lim = __float2int_rn((float)lbspOff + 255 * relThr);
        lim = lim < 0 ? 0 : lim > 255 ? 255 : lim;
        for (int t = 0; t <= 255; ++t)
            if ((int)ctl->lut[t] < lim) ++ctl->lut[t];
    }
    ctl->last_nz_ratio = ratio;
    ctl->refresh_pending = 0;
    ctl->ksent = 0;
    ctl->last_colordiff = 0;
    if (ctl->lr_scaling) {
        const unsigned long long tot = ctl->colordiff_acc;
        ctl->last_colordiff = tot;
        ctl->colordiff_acc = 0;
        const float cr = __ull2float_rn(tot) / (float)(S.dsW * S.dsH);
        const unsigned long long thr = (unsigned long long)(S.minColor / 2);
        if (ctl->auto_reset) {
            if (ctl->frames_since_reset > 1000ull) {
                ctl->auto_reset = 0;
            } else if (cr >= (float)thr && ctl->cooldown == 0ull) {
                ctl->frames_since_reset = 0;
                ctl->refresh_pending = 1;
                ctl->cooldown = (unsigned long long)(S.nmv / 4);
            } else {
                ++ctl->frames_since_reset;
            }
        } else if (cr >= (float)(thr * 2ull)) {
            ctl->frames_since_reset = 0;
            ctl->auto_reset = 1;
        }
        if (cr >= (float)(thr / 2ull)) {
            const int sh = ((int)(cr / 2)) & 31;
            const int lo = 2 >> sh, hi = 256 >> sh;
            ctl->t_lo = (float)(lo > 1 ? lo : 1);
            ctl->t_hi = (float)(hi > 1 ? hi : 1);
        } else {
            ctl->t_lo = 2.0f;
            ctl->t_hi = 256.0f;
        }
        if (ctl->cooldown > 0ull) --ctl->cooldown;
    }
}

// refreshModel (:80-105) of one pixel; lastBuf holds the latest colour/descriptor frame
template <int C>
__device__ void refresh_pixel(const StreamDev& S, int p, uint32_t frame, int start, int nref, int force, int lastBuf) {
    if (!S.roi[p]) return;
    if (!force && S.lastFG[p]) return;
    const int W = S.W, H = S.H, npx = S.npx, N = S.N;
    const int x0 = p % W, y0 = p / W;
    uint32_t k = S.kctr[p];
    DrawState ds;
    ds.blk = 0xffffffffu;
    const uint8_t* lc = S.lastCol + (size_t)lastBuf * npx * C;
    const uint16_t* ldd = S.lastDesc + (size_t)lastBuf * npx * C;
    for (int s = start; s < start + nref; ++s) {
        int r = 1 + (int)(draw_k(S.seed, frame, (uint32_t)p, k++, ds) % 512u);
        int sx = 0, sy = 0;
        for (int i = 0; i < 49; ++i) {
            r -= c_pat7[i];
            if (r <= 0) {
                sy = i / 7;
                sx = i % 7;
                break;
            }
        }
        sx += x0 - 3;
        sy += y0 - 3;
        clamp_xy(sx, sy, W, H);
        const int sp = sy * W + sx;
        if (!force && S.lastFG[sp]) continue;
        const int rs = s % N;
        if (C == 3) {
            const uint64_t d = (uint64_t)ldd[(size_t)sp * 3] | ((uint64_t)ldd[(size_t)sp * 3 + 1] << 16) |
                               ((uint64_t)ldd[(size_t)sp * 3 + 2] << 32) | ((uint64_t)lc[(size_t)sp * 3] << 48) |
                               ((uint64_t)lc[(size_t)sp * 3 + 1] << 56);
            ((uint64_t*)S.sD)[(size_t)rs * npx + p] = d;
            S.sC[(size_t)rs * npx + p] = lc[(size_t)sp * 3 + 2];
        } else {
            ((uint16_t*)S.sD)[(size_t)rs * npx + p] = ldd[sp];
            S.sC[(size_t)rs * npx + p] = lc[sp];
        }
    }
    S.kctr[p] = (uint16_t)k;
}

// ------------------------------------------------------------------------------------------
// the frame step: one kernel per phase, launched back to back over all streams of the batch (each
// kernel indexes the per-stream descriptor table); the repair loop is a cooperative kernel with
// grid barriers
// ------------------------------------------------------------------------------------------
#define LV_TILE_KERNEL_PROLOGUE                                              \
    const int t = blockIdx.x;                                               \
    if (t >= P.totalTiles) return;                                          \
    const int si = find_stream_by_tile(P, t);                               \
    const StreamDev& S = P.streams[si];                                     \
    const int lt = t - S.tileBase;

extern "C" __global__ void __launch_bounds__(kThreads, 5) lvbgs_k_eval(TickParams P) {
    __shared__ __align__(16) uint8_t smem[kTileRW<3> * (kTileH + 2 * kBorder) + 256];
    LV_TILE_KERNEL_PROLOGUE
    if (S.C == 3) phaseA_tile<3>(P, si, S, lt, smem);
    else phaseA_tile<1>(P, si, S, lt, smem);
}

// ------------------------------------------------------------------------------------------
// long sample scans: the pixels whose ordered scan did not settle within the first kScanCap samples
// (foreground pixels scan all N) continue here, one thread per pixel of the compacted list, from the
// saved scan state; then the rest of their evaluation. Spatially sparse long scans would otherwise
// keep whole warps of the evaluation waiting on a few lanes.
// ------------------------------------------------------------------------------------------
template <int C>
__device__ void longscan_item(const TickParams& P, unsigned int i) {
    const unsigned long long key = __ldcg(&P.rlist[0][i]);
    const unsigned long long sw = __ldcg(&P.rlist[1][i]);
    const int si = (int)(key >> 40), p = (int)(key & 0xffffffffffull);
    const StreamDev& S = P.streams[si];
    const FrameK F = frame_consts(S);
    const int W = S.W, x = p % W, y = p / W, npx = S.npx, N = S.N;
    ScanSt st;
    st.s = (int)(sw & 0xffu);
    st.nGood = (int)((sw >> 8) & 0xffu);
    const int g0 = (int)((sw >> 16) & 0xffu);
    st.g0 = g0 == 255 ? -1 : g0;
    st.minDesc = (uint32_t)((sw >> 32) & 0xffffu);
    st.minSum = (uint32_t)(sw >> 48);
    // a deferred scan has fewer than nreq good samples; with one, the minima are its distances
    st.g0d = st.minDesc;
    st.g0s = st.minSum;
    st.g1 = -1;
    st.g1d = st.g1s = 0;
    // samples s and s+1 with the feedback maps
    uint64_t dA = 0, dB = 0;
    uint32_t cA = 0, cB = 0;
    if (st.s < N) {
        dA = C == 3 ? ((const uint64_t*)S.sD)[(size_t)st.s * npx + p] : (uint64_t)((const uint16_t*)S.sD)[(size_t)st.s * npx + p];
        cA = S.sC[(size_t)st.s * npx + p];
    }
    if (st.s + 1 < N) {
        dB = C == 3 ? ((const uint64_t*)S.sD)[(size_t)(st.s + 1) * npx + p]
                    : (uint64_t)((const uint16_t*)S.sD)[(size_t)(st.s + 1) * npx + p];
        cB = S.sC[(size_t)(st.s + 1) * npx + p];
    }
    // the scan needs the thresholds only; the feedback maps of the tail are loaded after it, which
    // keeps the register peak (and so the occupancy) of this latency-bound kernel down
    const float* fc = S.fm + (size_t)F.cur * kNumFloatMaps * npx;
    const EvalThr th = eval_thresholds(S, fc[FM_R * npx + p], fc[FM_RAW_LT * npx + p], fc[FM_RAW_ST * npx + p],
                                       fc[FM_FIN_LT * npx + p], fc[FM_FIN_ST * npx + p],
                                       S.unst[(size_t)F.cur * npx + p]);
    uint32_t curr[C], intra[C];
    {
        uint32_t vals[C][4];
        const uint8_t* base = S.frame + (size_t)p * C;
        const uint8_t* lut = S.ctl->lut;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            gather_taps<C>(base, W * C, c, vals[c]);
            curr[c] = __ldg(base + c);
            intra[c] = lbsp_thr(vals[c], curr[c], lut[curr[c]]);
        }
        scan_samples<C, false>(S, lut, p, vals, curr, intra, th, nullptr, 0, 0ull, N, dA, cA, dB, cB, st);
    }
    record_scan(S, F, p, st);
    PixIn<C> in;
    load_pix<C>(S, F, p, in);
    __stcg(&S.intent[p], eval_tail<C>(S, F, x, y, p, in, curr, intra, th.uNew, st));
}

extern "C" __global__ void __launch_bounds__(256, 3) lvbgs_k_longscan(TickParams P) {
    const unsigned int n = min(ld_volatile(&P.work->lcount), P.listCap);
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int si = (int)(__ldcg(&P.rlist[0][i]) >> 40);
        if (P.streams[si].C == 3) longscan_item<3>(P, i);
        else longscan_item<1>(P, i);
    }
}

extern "C" __global__ void __launch_bounds__(kThreads) lvbgs_k_resolve(TickParams P, unsigned long long dsTotal,
                                                                       const unsigned long long* dsBase) {
    const int tileBlocks = (P.totalTiles + kResolveTiles - 1) / kResolveTiles;
    if ((int)blockIdx.x < tileBlocks) {
        phaseB_tiles(P, blockIdx.x * kResolveTiles);
        return;
    }
    const unsigned long long i = (unsigned long long)(blockIdx.x - tileBlocks) * blockDim.x + threadIdx.x;
    if (i >= dsTotal) return;
    int lo = 0, hi = P.nStreams - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (dsBase[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    ds_item(P.streams[lo], (int)(i - dsBase[lo]));
}

// repair to the raster-order fixed point (cooperative launch: all CTAs resident)
extern "C" __global__ void __launch_bounds__(kThreads) lvbgs_k_repair(TickParams P) {
    TickWork* w = P.work;
    if (blockIdx.x == 0 && threadIdx.x == 0 && w->nts < 40u) w->ts[w->nts++] = gtimer();  // phase profile
    if (P.dbgFault == LVBGS_FAULT_BARRIER_TIMEOUT) {
        // injected fault: every CTA but CTA 0 waits at a barrier CTA 0 never reaches; each wait gives
        // up after P.barrierNs and records ERR_BARRIER_TIMEOUT, and every CTA returns
        if (blockIdx.x != 0) grid_sync(w, P.barrierNs);
        return;
    }
    int iter = 0;
    for (;;) {
        const int par = iter & 1;
        const unsigned int n = ld_volatile(&w->dcount[par]);
        if (n == 0u) break;
        if (iter >= P.maxRepairIters) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&w->err, ERR_REPAIR_LIMIT);
            return;
        }
        const unsigned int nItems = n < P.listCap ? n : P.listCap;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            w->rcount[par ^ 1] = 0u;
            w->rematched += nItems;
            if (iter < 16) w->phase_ctr[iter] = nItems;
        }
        // items are fetched 32 at a time by each warp from a counter (not strided): per-item costs
        // vary widely, and every round waits for its slowest thread at the grid barrier
        const int lane = threadIdx.x & 31;
        for (;;) {
            unsigned int base = 0;
            if (lane == 0) base = atomicAdd(&w->fetchD[par], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= nItems) break;
            const unsigned int i = base + lane;
            if (i < nItems) {
                const unsigned long long item = __ldcg(&P.dlist[par][i]);
                const int si = (int)(item >> 40), q = (int)(item & 0xffffffffffull);
                const StreamDev& S = P.streams[si];
                const uint32_t stampNext = S.ctl->stamp_base + (uint32_t)iter + 2u;
                const bool counted = S.C == 3 ? rematch_item<3>(P, si, S, q, stampNext, par)
                                              : rematch_item<1>(P, si, S, q, stampNext, par);
                // re-match statistics: one atomic per stream among the lanes here
                const unsigned am = __activemask();
                const unsigned grp = __match_any_sync(am, counted ? si : -1 - (int)(threadIdx.x & 31));
                if (counted && (int)(threadIdx.x & 31) == __ffs(grp) - 1)
                    atomicAdd(&S.ctl->st_rematched, (unsigned long long)__popc(grp));
            }
        }
        if (!grid_sync(w, P.barrierNs)) return;
        const unsigned int nr0 = ld_volatile(&w->rcount[par]);
        const unsigned int nr = nr0 < P.listCap ? nr0 : P.listCap;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            w->dcount[par] = 0u;
            // the next round's counters (last used a round ago; visible after the next barrier)
            w->fetchD[par ^ 1] = 0u;
            w->fetchR[par ^ 1] = 0u;
        }
        for (;;) {
            unsigned int base = 0;
            if (lane == 0) base = atomicAdd(&w->fetchR[par], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= nr) break;
            const unsigned int i = base + lane;
            if (i < nr) {
                const unsigned long long item = __ldcg(&P.rlist[par][i]);
                const int si = (int)(item >> 40), p = (int)(item & 0xffffffffffull);
                const StreamDev& S = P.streams[si];
                reresolve_item(P, si, S, p, S.ctl->stamp_base + (uint32_t)iter + 2u, par);
            }
        }
        if (!grid_sync(w, P.barrierNs)) return;
        ++iter;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) w->iters = (unsigned)iter;
}

extern "C" __global__ void __launch_bounds__(kThreads) lvbgs_k_commit(TickParams P) {
    __shared__ __align__(16) uint8_t smem[(kTileW + 4) * (kTileH + 4) * 4 + (kTileW + 2) * (kTileH + 2)];
    LV_TILE_KERNEL_PROLOGUE
    if (S.C == 3) phaseF_tile<3>(P, S, lt, smem);
    else phaseF_tile<1>(P, S, lt, smem);
}



// frame-level epilogue of every stream (one thread per stream)
extern "C" __global__ void lvbgs_k_epilogue(TickParams P) {
    for (int si = blockIdx.x * blockDim.x + threadIdx.x; si < P.nStreams; si += gridDim.x * blockDim.x) {
        const StreamDev& S = P.streams[si];
        stream_epilogue(P, S);
        if (S.ctl->refresh_pending) {
            // nRefreshSampleStartPos = rand() % N, drawn with the frame-level (sentinel) counter (:86)
            DrawState ds;
            ds.blk = 0xffffffffu;
            const uint32_t f = (uint32_t)(S.ctl->frame_idx + 1ull);
            S.ctl->refresh_start = draw_k(S.seed, f, kSentinelPx, 0u, ds) % (uint32_t)S.N;
            S.ctl->ksent = 1;
            atomicExch(&P.work->anyReset, 1u);
        }
    }
}


// automatic model reset: refreshModel(0.1) and T(x) := 1 everywhere (:588-593); a small grid
// strides over the tiles of the streams that reset this frame
extern "C" __global__ void __launch_bounds__(kThreads) lvbgs_k_reset(TickParams P) {
    if (ld_volatile(&P.work->anyReset) == 0u) return;
    for (int t = blockIdx.x; t < P.totalTiles; t += gridDim.x) {
        const int si = find_stream_by_tile(P, t);
        const StreamDev& S = P.streams[si];
        if (!S.ctl->refresh_pending) continue;
        const int lt = t - S.tileBase;
        const int x = (lt % S.tilesX) * kTileW + threadIdx.x % kTileW;
        const int y = (lt / S.tilesX) * kTileH + threadIdx.x / kTileW;
        if (x >= S.W || y >= S.H) continue;
        const int p = y * S.W + x;
        const uint32_t f = (uint32_t)(S.ctl->frame_idx + 1ull);
        const int nxt = (int)((S.ctl->frame_idx + 1ull) & 1ull);
        const int nref = (int)(0.1f * (float)S.N);
        if (S.C == 3) refresh_pixel<3>(S, p, f, (int)S.ctl->refresh_start, nref, 0, nxt);
        else refresh_pixel<1>(S, p, f, (int)S.ctl->refresh_start, nref, 0, nxt);
        S.fm[(size_t)0 * kNumFloatMaps * S.npx + FM_T * S.npx + p] = 1.0f;
        S.fm[(size_t)1 * kNumFloatMaps * S.npx + FM_T * S.npx + p] = 1.0f;
    }
}

// closes the frame of every stream: frame index (and so the buffer parity), repair statistics
extern "C" __global__ void lvbgs_k_close(TickParams P) {
    const unsigned int its = P.work->iters;
    for (int si = blockIdx.x * blockDim.x + threadIdx.x; si < P.nStreams; si += gridDim.x * blockDim.x) {
        StreamCtl* ctl = P.streams[si].ctl;
        ctl->frame_idx += 1ull;
        ctl->st_rounds += its;
        ctl->stamp_base += its + 4u;
        frame_factors(ctl->frame_idx + 1ull, P.streams[si].nmv, &ctl->fLT, &ctl->fST, &ctl->bLT, &ctl->bST);
    }
}

// ------------------------------------------------------------------------------------------
// initialization, manual refresh, background images, LBSP extraction
// ------------------------------------------------------------------------------------------
// BackgroundSubtractorLBSP.cpp:21-65 + BackgroundSubtractorSuBSENSE.cpp:129-182 (map initial values)
extern "C" __global__ void lvbgs_init_maps(StreamDev S, const uint8_t* img, float tLo) {
    const int npx = S.npx;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
        const int C = S.C, x = p % S.W, y = p / S.W;
        for (int b = 0; b < 2; ++b) {
            float* f = S.fm + (size_t)b * kNumFloatMaps * npx;
            for (int m = 0; m < kNumFloatMaps; ++m) f[m * npx + p] = 0.0f;
            f[FM_T * npx + p] = tLo;
            f[FM_R * npx + p] = 1.0f;
            f[FM_V * npx + p] = 10.0f;
            S.unst[(size_t)b * npx + p] = 0;
        }
        const bool in = S.roi[p] != 0;
        const bool desc = in && x > kBorder && y > kBorder && x < S.W - kBorder && y < S.H - kBorder;
        for (int c = 0; c < C; ++c) {
            const uint8_t v = in ? img[(size_t)p * C + c] : 0;
            uint16_t d = 0;
            if (desc) {
                uint32_t vals[4];
                const uint8_t* base = img + (size_t)p * C;
                for (int j = 0; j < 4; ++j) {
                    uint32_t wv = 0;
                    for (int i = 0; i < 4; ++i) {
                        const int n = j * 4 + i;
                        wv |= (uint32_t)base[(c_lbsp_dy[n] * S.W + c_lbsp_dx[n]) * C + c] << (8 * i);
                    }
                    vals[j] = wv;
                }
                d = (uint16_t)lbsp_thr(vals, v, S.ctl->lut[v]);
            }
            for (int b = 0; b < 2; ++b) {
                S.lastCol[(size_t)b * npx * C + (size_t)p * C + c] = v;
                S.lastDesc[(size_t)b * npx * C + (size_t)p * C + c] = d;
            }
        }
        S.blinks[p] = 0;
        S.lastRawFG[p] = 0;
        S.lastFG[p] = 0;
        S.dilInv[p] = 0;
        S.lastRawBlink[p] = 0;
        S.kctr[p] = 0;
        S.stampD[p] = 0;
        S.stampR[p] = 0;
    }
}

// refreshModel(frac, force) outside a frame step (initialize(), or a user call)
extern "C" __global__ void lvbgs_refresh(StreamDev S, uint32_t frame, int start, int nref, int force, int lastBuf) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.npx; p += gridDim.x * blockDim.x) {
        if (S.C == 3) refresh_pixel<3>(S, p, frame, start, nref, force, lastBuf);
        else refresh_pixel<1>(S, p, frame, start, nref, force, lastBuf);
    }
}

// getBackgroundImage / getBackgroundDescriptorsImage (:614-649): float mean in sample order
extern "C" __global__ void lvbgs_background(StreamDev S, uint8_t* outCol, uint16_t* outDesc) {
    const int npx = S.npx, C = S.C, N = S.N;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
        for (int c = 0; c < C; ++c) {
            float acc = 0.0f, accd = 0.0f;
            for (int s = 0; s < N; ++s) {
                uint32_t col, d;
                if (C == 3) {
                    const uint64_t v = ((const uint64_t*)S.sD)[(size_t)s * npx + p];
                    col = c == 2 ? S.sC[(size_t)s * npx + p] : (uint32_t)(v >> (48 + 8 * c)) & 0xffu;
                    d = (uint32_t)(v >> (16 * c)) & 0xffffu;
                } else {
                    col = S.sC[(size_t)s * npx + p];
                    d = ((const uint16_t*)S.sD)[(size_t)s * npx + p];
                }
                acc += ((float)col) / (float)N;
                accd += ((float)d) / (float)N;
            }
            if (outCol) {
                int r = __float2int_rn(acc);
                outCol[(size_t)p * C + c] = (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
            }
            if (outDesc) {
                int r = __float2int_rn(accd);
                outDesc[(size_t)p * C + c] = (uint16_t)(r < 0 ? 0 : r > 65535 ? 65535 : r);
            }
        }
    }
}

// sample planes -> the reference's N sample images (inspection)
extern "C" __global__ void lvbgs_unpack_samples(StreamDev S, uint8_t* col, uint16_t* desc) {
    const size_t total = (size_t)S.N * S.npx;
    const int C = S.C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (C == 3) {
            const uint64_t v = ((const uint64_t*)S.sD)[i];
            for (int c = 0; c < 3; ++c) {
                col[i * 3 + c] = c == 2 ? S.sC[i] : (uint8_t)(v >> (48 + 8 * c));
                desc[i * 3 + c] = (uint16_t)(v >> (16 * c));
            }
        } else {
            col[i] = S.sC[i];
            desc[i] = ((const uint16_t*)S.sD)[i];
        }
    }
}

// the reference's N sample images -> sample planes (state restore)
extern "C" __global__ void lvbgs_pack_samples(StreamDev S, const uint8_t* col, const uint16_t* desc) {
    const size_t total = (size_t)S.N * S.npx;
    const int C = S.C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (C == 3) {
            ((uint64_t*)S.sD)[i] = (uint64_t)desc[i * 3] | ((uint64_t)desc[i * 3 + 1] << 16) |
                                   ((uint64_t)desc[i * 3 + 2] << 32) | ((uint64_t)col[i * 3] << 48) |
                                   ((uint64_t)col[i * 3 + 1] << 56);
            S.sC[i] = col[i * 3 + 2];
        } else {
            ((uint16_t*)S.sD)[i] = desc[i];
            S.sC[i] = col[i];
        }
    }
}

// LBSP::compute2 (LBSP.cpp:102-152): dense extraction, absolute (thr >= 0) or relative threshold
extern "C" __global__ void lvbgs_lbsp_dense(const uint8_t* img, int W, int H, int C, int absThr, float rel,
                                            unsigned int off, uint16_t* desc) {
    const int total = W * H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const int x = p % W, y = p / W;
        if (x < kBorder || y < kBorder || x >= W - kBorder || y >= H - kBorder) continue;
        for (int c = 0; c < C; ++c) {
            const uint8_t* base = img + (size_t)p * C;
            uint32_t vals[4];
            for (int j = 0; j < 4; ++j) {
                uint32_t wv = 0;
                for (int i = 0; i < 4; ++i) {
                    const int n = j * 4 + i;
                    wv |= (uint32_t)base[(c_lbsp_dy[n] * W + c_lbsp_dx[n]) * C + c] << (8 * i);
                }
                vals[j] = wv;
            }
            const uint32_t ref = base[c];
            uint32_t thr;
            if (absThr >= 0) {
                thr = absThr > 255 ? 255u : (uint32_t)absThr;
            } else {
                int r = __float2int_rn((float)ref * rel + (float)off);
                thr = (uint32_t)(r < 0 ? 0 : r > 255 ? 255 : r);
            }
            desc[(size_t)p * C + c] = (uint16_t)lbsp_thr(vals, ref, thr);
        }
    }
}

}  // namespace lvbgs
