// LOBSTER, ViBe and PBAS on the device: state of one stream and the host functions that run its frame
// steps (lobster.cu), called by the C-ABI layer for handles created with LVBGS_ALGO_LOBSTER / _VIBE / _PBAS.
// Both are sample-consensus models whose in-frame dependency is the same (a pixel's scan reads its own
// samples, which earlier pixels' neighbour updates may overwrite), so they share the frame step.
//
// Device layout (one allocation per stream, each array 256-byte aligned):
//   roi[npx], lastColor[npx*C], lastFG[npx], lastDesc[npx*C] (u16), kctr[npx] (u16, draws of the last
//   frame), samples sD[N][npx] / sC[N][npx] (the SuBSENSE packing: for C=3 one u64 = desc0 | desc1<<16 |
//   desc2<<32 | B<<48 | G<<56 and the R byte, for C=1 one u16 descriptor and the intensity),
//   ViBe keeps only its samples, sC[N][npx*C] (the reference's layout: C colour bytes per sample);
//   PBAS its colour and gradient samples sC / sG[N][npx*C], the R, T and D maps fm[2][3][npx] (by frame
//   parity), the frame's gradient image and the frame-level mean gradient distance;
//   scratch of a frame step: intent[npx] (u32), wD[npx] (the sample word a pixel writes), rawFG[npx],
//   two repair lists and their dedupe stamps, flags and counters, the staged frame and mask.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lvbgs_internal.h"

namespace lvbgs {

// the algorithm of a stream
enum { ALG_LOBSTER = 0, ALG_VIBE = 1, ALG_PBAS = 2 };

// flags of one frame step (device words)
enum { LOB_F_COUNT0 = 0, LOB_F_COUNT1, LOB_F_CONV, LOB_F_ROUNDS, LOB_F_ERR, LOB_F_WORDS = 8 };

// kernel parameters (by value)
struct LobDev {
    int alg;  // ALG_LOBSTER, ALG_VIBE or ALG_PBAS
    int W, H, C, N, nreq, npx;
    unsigned int descThr, colThr;  // m_nDescDistThreshold (LOBSTER), m_nColorDistThreshold (both)
    unsigned long long seed;
    unsigned long long nLR;  // ceil(learning rate), ~0 for an infinite rate
    uint32_t frameKey;       // apply() calls since initialize(): the generator's frame
    uint32_t stampBase;      // repair-list dedupe stamps of this frame step are stampBase + round + 1
    int medianK;
    unsigned int listCap;
    const uint8_t* frame;
    uint8_t* maskOut;
    uint8_t *roi, *lastColor, *lastFG, *rawFG, *lut;
    uint16_t *lastDesc, *kctr;
    void* sD;
    uint8_t* sC;
    uint32_t* intent;
    unsigned long long* wD;
    uint32_t *list0, *list1, *stamp;
    unsigned int* flags;
    unsigned long long* stats;  // samples evaluated, sample writes (cumulative); PBAS: bad samples' gradient sum, count
    // PBAS
    int cur;                // parity of the R, T, D maps the frame starts from
    int lrOverride;         // nLR is the override (otherwise ceil(T(x)) per pixel)
    float R0, updateRate;   // m_nDefaultColorDistThreshold, m_fDefaultUpdateRate
    uint8_t *sG, *grad, *blur;
    float *fm, *meanGrad, *badVals;
    uint32_t* badSum;
    uint8_t* badCnt;
    void* sumTr;  // three channels: the per-chunk transfers of the mean's exact float sum
};

struct LobState {
    LobDev d{};
    uint8_t* mem = nullptr;
    size_t bytes = 0;
    uint8_t* d_frame = nullptr;  // staging of host frames
    uint8_t* d_mask = nullptr;   // mask of the last frame step
    unsigned int* h_flags = nullptr;  // pinned copy of the flags
    cudaEvent_t done = nullptr;       // PBAS: the frame step's mask and flags are on the host
    cudaEvent_t meanDone = nullptr;   // PBAS: the frame step's mean gradient distance is written
    float pbasMean = 20.0f;           // PBAS: m_fFormerMeanGradDist across initialize() calls
    uint32_t ksent = 0;               // frame-level draws of the current frame (refreshModel's start)
    int lastRounds = 1;               // repair rounds of the last frame step
    unsigned long long frames = 0;
    size_t n_rel = 0, orig_roi = 0;
};

// allocates the stream's device state for a W x H x C frame and uploads the validated ROI (ViBe: every
// pixel) and the LBSP threshold LUT; the model itself is built by lob_init_model
lvbgs_status lob_setup(LobState& L, int alg, const lvbgs_params& prm, int W, int H, int C,
                       const std::vector<uint8_t>& roi, size_t orig, size_t fin, cudaStream_t st, std::string& err);
// initialize() after lob_setup, from dimg (a device frame); waits for the device. LOBSTER: last
// colour/descriptor frames, zero samples, then refreshModel(1.0, true); ViBe: every sample of every pixel
// from a 7x7 position of the frame; PBAS: the same for colour and gradient samples, and its maps
lvbgs_status lob_init_model(LobState& L, const uint8_t* dimg, cudaStream_t st, std::string& err);
// apply(): one frame step on dimg (device); the mask goes to dmask (device) and, when hostMask is not
// null, to host memory; waits for the device
lvbgs_status lob_apply(LobState& L, const uint8_t* dimg, uint8_t* dmask, uint8_t* hostMask, double lr,
                       cudaStream_t st, std::string& err);
// refreshModel(frac, force); waits for the device
lvbgs_status lob_refresh(LobState& L, float frac, int force, cudaStream_t st, std::string& err);
// getBackgroundImage (u8 [H*W*C]) or getBackgroundDescriptorsImage (u16 [H*W*C]) into host memory
lvbgs_status lob_background(LobState& L, void* hostOut, bool descriptors, cudaStream_t st, std::string& err);
// model maps in the reference's layout (LOBSTER: LVBGS_MAP_LAST_FG, _ROI, _LAST_COLOR, _LAST_DESC,
// _SAMPLE_COLOR, _SAMPLE_DESC, _LUT; ViBe: _SAMPLE_COLOR, _ROI; PBAS: _SAMPLE_COLOR, _SAMPLE_GRAD, _R,
// _T, _DMIN_LT (its D map), _GRAD, _MEAN_GRAD, _ROI); 0 bytes for the others
size_t lob_map_bytes(const LobState& L, int which);
lvbgs_status lob_get_map(LobState& L, int which, void* hostOut, size_t bytes, cudaStream_t st, std::string& err);
// samples evaluated and sample writes since initialize()
lvbgs_status lob_stats(LobState& L, unsigned long long out[2], cudaStream_t st, std::string& err);
void lob_release(LobState& L);

}  // namespace lvbgs
