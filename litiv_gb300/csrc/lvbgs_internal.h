// Internal definitions shared by the SuBSENSE kernels and the C-ABI layer.
//
// Device model layout (structure of arrays, one plane per quantity, coalesced per pixel):
//   fm[2][10][npx]   float feedback maps, double-buffered by frame parity: R, v, T, D_last,
//                    D_min LT/ST, raw-segmentation LT/ST, final-segmentation LT/ST
//                    (BackgroundSubtractorSuBSENSE.hpp:100-115)
//   unst[2][npx]     unstable-region flags (double-buffered)
//   lastCol[2][npx*C], lastDesc[2][npx*C]   last colour / LBSP descriptor frames
//   sD[N][npx]       sample descriptors: for C=3 one uint64 = desc0|desc1<<16|desc2<<32|B<<48|G<<56,
//                    for C=1 one uint16 descriptor
//   sC[N][npx]       sample colour byte: R for C=3, the intensity for C=1
//   (so one sample costs exactly 3*C bytes, the algorithmic minimum)
//   u8 maps: roi, blinks, last raw mask, last final mask, inverted dilated mask, last raw blinks,
//   plus per-frame scratch (closed mask, combined mask, union-find labels, intents, draw counters).
#pragma once
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define LV_HD __host__ __device__ __forceinline__
#else
#define LV_HD inline
#endif

#include "../../include/lvbgs.h"

namespace lvbgs {

// sets the library-level error message returned by lvbgs_last_error(NULL); returns st
lvbgs_status report_error(lvbgs_status st, const char* msg);

constexpr int kTileW = 32;  // one warp per tile row: coalesced 32-pixel rows
constexpr int kTileH = 8;
constexpr int kThreads = kTileW * kTileH;
constexpr int kBorder = 2;  // LBSP::PATCH_SIZE/2
constexpr int kMaxSamples = 64;
constexpr int kNumFloatMaps = 10;
enum FloatMap { FM_R = 0, FM_V, FM_T, FM_DLAST, FM_DMIN_LT, FM_DMIN_ST, FM_RAW_LT, FM_RAW_ST, FM_FIN_LT, FM_FIN_ST };
constexpr unsigned kPhilox0 = 0xD2511F53u, kPhilox1 = 0xCD9E8D57u, kWeyl0 = 0x9E3779B9u, kWeyl1 = 0xBB67AE85u;
constexpr uint32_t kSentinelPx = 0xFFFFFFFFu;

// Philox4x32-10 (Salmon et al., SC'11): the counter-based generator that replaces rand().
// Draw k of pixel p in frame t is block(ctr={k>>2,p,t,0}, key=seed)[k&3] & 0x7fffffff.
LV_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += kWeyl0;
            k1 += kWeyl1;
        }
        // one 32x32 -> 64-bit multiply each (a single wide multiply-add on the device)
        const uint64_t p0 = (uint64_t)kPhilox0 * x0, p1 = (uint64_t)kPhilox1 * x2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ x1 ^ k0, n2 = hi0 ^ x3 ^ k1;
        x0 = n0;
        x1 = lo1;
        x2 = n2;
        x3 = lo0;
    }
    c[0] = x0;
    c[1] = x1;
    c[2] = x2;
    c[3] = x3;
}

// rolling-average factors of frame f (BackgroundSubtractorSuBSENSE.cpp:198-199): 1/min(f, N_mv) and
// 1/min(f, N_mv/4), and the addWeighted mask weights (1.0/255)*factor of the final-segmentation
// averages (:553-554); computed once per frame instead of per pixel
LV_HD void frame_factors(unsigned long long f, int nmv, float* fLT, float* fST, float* bLT, float* bST) {
    const unsigned long long nlt = (unsigned long long)nmv, nst = (unsigned long long)(nmv / 4);
    *fLT = 1.0f / (float)(f < nlt ? f : nlt);
    *fST = 1.0f / (float)(f < nst ? f : nst);
    *bLT = (float)((1.0 / 255) * (double)*fLT);
    *bST = (float)((1.0 / 255) * (double)*fST);
}

// ---- per-pixel "intent" word: outcome of the pixel's evaluation in the current frame ----
// bit 0 valid (ROI pixel evaluated this frame), bit 1 foreground, bits 2-8 samples evaluated,
// bit 9 own-sample write, bits 10-15 own sample index, bits 16-20 neighbour code (dy+2)*5+(dx+2)
// of the clamped update target, bits 21-23 neighbour-update state, bits 24-29 neighbour sample.
constexpr uint32_t kInValid = 1u, kInFG = 2u, kInOwn = 1u << 9;
constexpr int kInEShift = 2, kInSOwnShift = 10, kInCodeShift = 16, kInNStShift = 21, kInSNbShift = 24;
// neighbour-update states
enum NbState : uint32_t {
    NB_NONE = 0,         // foreground pixel: no neighbour update
    NB_WRITE = 1,        // n_rand % (T or T/2+1) == 0: unconditional write
    NB_PENDING = 2,      // ghost test still to be evaluated against the target's maps
    NB_GHOST_WRITE = 3,  // ghost test passed
    NB_GHOST_NO = 4,     // ghost test failed
    NB_NO = 5            // neither condition can hold
};
LV_HD uint32_t in_e(uint32_t w) { return (w >> kInEShift) & 127u; }
LV_HD uint32_t in_sown(uint32_t w) { return (w >> kInSOwnShift) & 63u; }
LV_HD uint32_t in_code(uint32_t w) { return (w >> kInCodeShift) & 31u; }
LV_HD uint32_t in_nst(uint32_t w) { return (w >> kInNStShift) & 7u; }
LV_HD uint32_t in_snb(uint32_t w) { return (w >> kInSNbShift) & 63u; }
LV_HD bool in_nb_writes(uint32_t w) { return (w & kInValid) && (in_nst(w) == NB_WRITE || in_nst(w) == NB_GHOST_WRITE); }
LV_HD bool in_ghost(uint32_t w) {
    const uint32_t s = in_nst(w);
    return (w & kInValid) && (s == NB_PENDING || s == NB_GHOST_WRITE || s == NB_GHOST_NO);
}

// Frame-level state of one stream, resident on the device and updated by the kernel itself
// (BackgroundSubtractorSuBSENSE.cpp:555-611), so consecutive frames need no host round trip.
struct StreamCtl {
    unsigned long long frame_idx;  // apply() calls completed (m_nFrameIdx); parity = frame_idx & 1
    unsigned long long frames_since_reset, cooldown;
    int auto_reset, lr_scaling, use3x3, median_k;
    float t_lo, t_hi, last_nz_ratio, pad0;
    float fLT, fST, bLT, bST;  // rolling-average factors of the next frame and their addWeighted weights
    unsigned long long nz_acc, colordiff_acc;    // accumulators of the frame in flight
    unsigned long long last_nz, last_colordiff;  // values of the last completed frame
    unsigned long long st_samples, st_writes, st_rounds, st_rematched;
    unsigned long long n_rel, orig_roi;
    unsigned int refresh_pending, ksent;  // auto model reset decided this frame; sentinel draw counter
    unsigned int stamp_base, refresh_start;
    unsigned char lut[256];
};

// Per-stream descriptor read by the kernels (device memory, rewritten by the host per launch).
struct StreamDev {
    int W, H, C, npx;
    int tilesX, tilesY, tileBase, nTiles;
    int rowBase, rowWords;  // first row of this stream in the batch's row index space; bit-plane words per row
    int segBase, nSegs;     // first median column segment of this stream in the batch, and its count
    int dsW, dsH;  // size of the frame-level down-sampled frame (W/8, H/8)
    int N, nreq, minColor, descOff, stabColorOff, nmv;
    float relThr;
    unsigned int lbspOff;
    unsigned long long seed;
    unsigned long long nMagic;  // ceil(2^40 / N): fast exact draw % N
    // per-launch inputs
    const uint8_t* frame;  // dense device frame
    uint8_t* maskOut;      // device output mask (may be null)
    int lrMode;            // 0: per-pixel ceil(T(x)); 1: fixed value lrFixed
    int lrScaling;         // frame-level analysis enabled (host copy of StreamCtl::lr_scaling)
    unsigned long long lrFixed;
    // state
    float* fm;
    uint8_t* unst;
    uint8_t* lastCol;
    uint16_t* lastDesc;
    void* sD;
    uint8_t* sC;
    uint8_t* roi;
    uint8_t *blinks, *lastRawFG, *lastFG, *dilInv, *lastRawBlink;
    uint32_t* bits;   // mask bit planes (BP_*): rowWords words per row, bit b of word w = pixel 32w + b
    uint8_t* hcount;  // set pixels of the combined mask in each pixel's median row window
    int* label;
    uint32_t* intent;
    uint32_t *stampD, *stampR;
    uint4* goodRec;  // long scans of the frame: frame tag, stop position, good samples (index, distances)
    uint16_t* kctr;
    float *dsLT, *dsST;
    StreamCtl* ctl;
};

// Per-launch work area (reset before every launch).
struct TickWork {
    unsigned int bar_count, bar_gen, err, err_info;
    unsigned int phase_ctr[16];  // repair: re-matched items of rounds 0..15 (phase profile)
    unsigned int dcount[2], rcount[2];
    unsigned int done_ctas, iters;
    unsigned long long rematched;
    unsigned long long ts[40];  // %globaltimer after each grid barrier (CTA 0), for the phase profile
    unsigned int nts, anyReset;  // anyReset: some stream refreshes its model this frame
    unsigned int lcount, pad;    // long sample scans deferred by the evaluation (list in rlist[0..1])
    unsigned int fetchD[2], fetchR[2];  // repair: next item of each phase, by round parity (warp fetches)
};

// error codes reported in TickWork::err
enum : unsigned int { ERR_NONE = 0, ERR_BARRIER_TIMEOUT = 1, ERR_REPAIR_LIMIT = 2, ERR_UF_LIMIT = 4, ERR_RING = 8 };

struct TickParams {
    StreamDev* streams;
    int nStreams;
    int totalTiles;
    int totalRows;
    TickWork* work;
    unsigned long long* dlist[2];  // (stream << 40) | pixel
    unsigned long long* rlist[2];
    unsigned int listCap;
    int totalSegs, colBlocks;  // median: column segments of all streams; 256-pixel column blocks of the widest
    unsigned long long barrierNs;  // limit of one grid-barrier wait of the repair, then ERR_BARRIER_TIMEOUT
    int maxRepairIters;            // repair rounds before ERR_REPAIR_LIMIT
    int dbgFault;                  // injected fault (lvbgs_debug_inject_fault), 0: none
};
constexpr unsigned long long kBarrierNs = 2000000000ull;  // 2 s
constexpr unsigned long long kDebugBarrierNs = 2000000ull;  // 2 ms, for the injected barrier timeout
constexpr int kRepairIterLimit = 4096;

// mask bit planes of a stream (scratch of one frame step; bits beyond the frame width are 0)
enum { BP_CLOSED = 0, BP_RAW, BP_HOLES, BP_COMB, BP_FG, BP_COUNT };
constexpr int kMedSegRows = 32;  // rows of one median column segment
constexpr int kResolveTiles = 4;  // tiles per block of the ghost-resolution kernel
constexpr int kScanCap = 8;      // samples the evaluation scans per pixel before deferring to a long scan
__host__ __device__ __forceinline__ uint32_t* bit_plane(const StreamDev& S, int i) {
    return S.bits + (size_t)i * S.H * S.rowWords;
}
inline size_t bit_planes_bytes(int W, int H) { return (size_t)BP_COUNT * H * ((W + 31) / 32) * 4; }

// ---- cv::resize(src, dst, (dW, dH), INTER_AREA) of an 8-bit image, one output element ----
// When the source size is an integral multiple of the output (OpenCV's "area fast" case, e.g. the
// 1/8 down-sampling of frames whose sides are multiples of 8) the output is the block mean computed as
// round(sum * (1.f/area)), as before. Otherwise it is the exact area-weighted mean of the source
// pixels under the output pixel's footprint: in units of 1/dW (1/dH) a source pixel i spans
// [i*dW, (i+1)*dW) and output pixel x spans [x*W, (x+1)*W), so every overlap is an integer and the
// output is round(sum(ox * oy * src) / (W * H)) with ties to even, computed exactly in integers. The
// definition is written from the mathematics of the area relation (OpenCV documents INTER_AREA as
// "resampling using pixel area relation" and is not installed here); both the GPU and the oracle use it.
// get(i, j) returns the source value at column i, row j.
LV_HD uint8_t area_round_ties_even(unsigned long long num, unsigned long long den) {
    unsigned long long q = num / den;
    const unsigned long long r2 = (num % den) * 2ull;
    if (r2 > den || (r2 == den && (q & 1ull))) ++q;
    return (uint8_t)(q > 255ull ? 255ull : q);
}
template <typename Get>
LV_HD uint8_t area_resample(int W, int H, int dW, int dH, int x, int y, Get get) {
    if (W % dW == 0 && H % dH == 0) {
        const int sx = W / dW, sy = H / dH;
        int sum = 0;
        for (int j = 0; j < sy; ++j)
            for (int i = 0; i < sx; ++i) sum += get(x * sx + i, y * sy + j);
        const float v = (float)sum * (1.f / (float)(sx * sy));
#ifdef __CUDA_ARCH__
        const int r = __float2int_rn(v);
#else
        const int r = (int)nearbyintf(v);
#endif
        return (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
    }
    const long long x0 = (long long)x * W, x1 = x0 + W, y0 = (long long)y * H, y1 = y0 + H;
    const int i0 = (int)(x0 / dW), i1 = (int)((x1 + dW - 1) / dW);
    const int j0 = (int)(y0 / dH), j1 = (int)((y1 + dH - 1) / dH);
    unsigned long long num = 0;
    for (int j = j0; j < j1; ++j) {
        const long long a = (long long)j * dH, b = a + dH;
        const long long oy = (b < y1 ? b : y1) - (a > y0 ? a : y0);
        unsigned long long row = 0;
        for (int i = i0; i < i1; ++i) {
            const long long c = (long long)i * dW, d = c + dW;
            const long long ox = (d < x1 ? d : x1) - (c > x0 ? c : x0);
            row += (unsigned long long)ox * (unsigned long long)get(i, j);
        }
        num += row * (unsigned long long)oy;
    }
    return area_round_ties_even(num, (unsigned long long)W * (unsigned long long)H);
}

}  // namespace lvbgs
