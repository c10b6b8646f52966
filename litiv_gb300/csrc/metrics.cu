// Change-detection evaluation on the device: the pixel classification counters of
// lv::BinClassif::accumulate (modules/datasets/src/metrics.cpp:21-61) and the metrics of
// lv::BinClassifMetrics (modules/datasets/include/litiv/datasets/metrics.hpp:203-256), so that a
// foreground mask already on the device is scored against ground truth without a host round trip.
//
// Ground-truth codes (CDnet, metrics.hpp:23-27): 255 positive, 0 negative, 85 out of scope,
// 170 unknown, 50 shadow. A pixel is "don't care" when its ground truth is out of scope or unknown,
// or when a ROI is given and is 0 there; otherwise it is TP / FP / FN / TN by the mask (255 =
// positive, anything else negative) and the ground truth (255 = positive, anything else negative),
// and additionally a shadow error when the ground truth is shadow and the mask positive.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/lvbgs.h"
#include "lvbgs_internal.h"

namespace lvbgs {

enum { CL_TP = 0, CL_TN, CL_FP, CL_FN, CL_SE, CL_DC, CL_COUNT };

// four consecutive pixels per thread per step (grid-stride); per-warp then per-block sums, one
// 64-bit atomic per counter per block
extern "C" __global__ void __launch_bounds__(256) lvbgs_k_classif(const uint8_t* __restrict__ mask,
                                                                  const uint8_t* __restrict__ gt,
                                                                  const uint8_t* __restrict__ roi, size_t n,
                                                                  unsigned long long* counts) {
    unsigned int c[CL_COUNT] = {0, 0, 0, 0, 0, 0};
    const size_t stride = (size_t)gridDim.x * blockDim.x * 4;
    for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 4; i < n; i += stride) {
        const int m = n - i < 4 ? (int)(n - i) : 4;
        for (int k = 0; k < m; ++k) {
            const uint8_t g = __ldg(gt + i + k);
            const bool dc = g == 85 || g == 170 || (roi && __ldg(roi + i + k) == 0);
            if (dc) {
                ++c[CL_DC];
                continue;
            }
            const bool mp = __ldg(mask + i + k) == 255, gp = g == 255;
            c[mp ? (gp ? CL_TP : CL_FP) : (gp ? CL_FN : CL_TN)] += 1u;
            if (g == 50 && mp) ++c[CL_SE];
        }
    }
    __shared__ unsigned int s[CL_COUNT][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < CL_COUNT; ++j) {
        const unsigned int v = __reduce_add_sync(0xffffffffu, c[j]);
        if (lane == 0) s[j][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < CL_COUNT) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[threadIdx.x][w];
        if (t) atomicAdd(&counts[threadIdx.x], t);
    }
}

}  // namespace lvbgs

namespace {

bool on_device(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" lvbgs_status lvbgs_classif_accumulate(const uint8_t* fgmask, const uint8_t* gt, const uint8_t* roi,
                                                 int width, int height, uint64_t counts[6], int device_id,
                                                 void* cuda_stream) {
    using lvbgs::report_error;
    if (!fgmask || !counts || width <= 0 || height <= 0)
        return report_error(LVBGS_BAD_ARG, "classification: mask, counters and a non-empty size are required");
    const size_t n = (size_t)width * height;
    if (!gt) {
        // metrics.cpp:26-29: without ground truth every pixel is a "don't care"
        counts[lvbgs::CL_DC] += n;
        return LVBGS_OK;
    }
    if (cudaSetDevice(device_id) != cudaSuccess) {
        cudaGetLastError();
        return report_error(LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    }
    cudaStream_t st = (cudaStream_t)cuda_stream;
    // device staging: host inputs are copied (stream-ordered allocations), device inputs read in place
    const uint8_t* src[3] = {fgmask, gt, roi};
    const uint8_t* dptr[3] = {nullptr, nullptr, nullptr};
    uint8_t* tmp = nullptr;
    unsigned long long* dcounts = nullptr;
    size_t need = 256;  // the counters, then each staged input at a 256-byte boundary
    for (int i = 0; i < 3; ++i)
        if (src[i] && !on_device(src[i])) need += (n + 255) & ~(size_t)255;
    cudaError_t e = cudaMallocAsync((void**)&tmp, need, st);
    if (e == cudaSuccess) {
        dcounts = (unsigned long long*)tmp;
        size_t off = 256;
        e = cudaMemsetAsync(dcounts, 0, 6 * sizeof(unsigned long long), st);
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
            if (!src[i]) continue;
            if (on_device(src[i])) {
                dptr[i] = src[i];
                continue;
            }
            e = cudaMemcpyAsync(tmp + off, src[i], n, cudaMemcpyHostToDevice, st);
            dptr[i] = tmp + off;
            off += (n + 255) & ~(size_t)255;
        }
    }
    if (e == cudaSuccess) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_id);
        const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(sms, 1) * 8, (n + 1023) / 1024));
        lvbgs::lvbgs_k_classif<<<blocks, 256, 0, st>>>(dptr[0], dptr[1], dptr[2], n, dcounts);
        e = cudaGetLastError();
    }
    unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dcounts, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (tmp) cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return report_error(LVBGS_DEVICE_ERROR, cudaGetErrorString(e));
    }
    for (int i = 0; i < 6; ++i) counts[i] += h[i];
    return LVBGS_OK;
}

extern "C" lvbgs_status lvbgs_classif_metrics(const uint64_t counts[6], double out[8]) {
    if (!counts || !out) return lvbgs::report_error(LVBGS_BAD_ARG, "null argument");
    const double tp = (double)counts[0], tn = (double)counts[1], fp = (double)counts[2], fn = (double)counts[3];
    const uint64_t TP = counts[0], TN = counts[1], FP = counts[2], FN = counts[3];
    const uint64_t total = TP + TN + FP + FN;  // "don't care" excluded (metrics.hpp:46-48)
    const double recall = (TP + FN) > 0 ? tp / (double)(TP + FN) : 0.0;
    const double precision = (TP + FP) > 0 ? tp / (double)(TP + FP) : 0.0;
    out[0] = recall;
    out[1] = (TN + FP) > 0 ? tn / (double)(TN + FP) : 0.0;                   // specificity
    out[2] = (FP + TN) > 0 ? fp / (double)(FP + TN) : 0.0;                   // false positive rate
    out[3] = (TP + FN) > 0 ? fn / (double)(TP + FN) : 0.0;                   // false negative rate
    out[4] = total > 0 ? 100.0 * (double)(FN + FP) / (double)total : 0.0;    // percentage of bad classifications
    out[5] = precision;
    out[6] = (recall + precision) > 0 ? 2.0 * (recall * precision) / (recall + precision) : 0.0;  // F-measure
    // Matthews correlation coefficient: 0 when a marginal is empty
    const bool ok = (TP + FP) > 0 && (TP + FN) > 0 && (TN + FP) > 0 && (TN + FN) > 0;
    out[7] = ok ? ((tp * tn) - (double)(FP * FN)) / std::sqrt((tp + fp) * (double)(TP + FN) * (double)(TN + FP) *
                                                              (double)(TN + FN))
                : 0.0;
    return LVBGS_OK;
}
