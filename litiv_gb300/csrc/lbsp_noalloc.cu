// Dense LBSP extraction for callers that must not allocate device memory.
//
// lvbgs_lbsp_compute2() stages the caller's image and descriptor buffers in device memory it
// allocates per call. Code that runs where cudaMalloc/cudaFree are off limits -- a real-time
// capture thread with a no-allocation rule, or a host that shares the GPU under a fixed memory
// budget -- uses lvbgs_lbsp_compute2_noalloc() instead: the staging lives in one file-scope
// device array, reserved when the library is loaded, so a call allocates nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/lvbgs.h"
#include "lvbgs_internal.h"

namespace lvbgs {
extern "C" __global__ void lvbgs_lbsp_dense(const uint8_t* img, int W, int H, int C, int absThr, float rel,
                                            unsigned int off, uint16_t* desc);
}  // namespace lvbgs

namespace {

// Largest frame the entry point accepts: width*height*channels <= 8,388,608 elements (a 1920x1080
// BGR frame is 6,220,800). The array holds the image (one byte per element) followed, at the next
// 256-byte boundary, by the descriptors (two bytes per element): 24 MiB plus alignment, held on
// every GPU that loads the library until the process exits.
constexpr size_t kMaxElems = 8u << 20;
constexpr size_t kDescOffset = (kMaxElems + 255) & ~(size_t)255;
constexpr size_t kScratchBytes = kDescOffset + 2 * kMaxElems;

static __device__ __align__(256) unsigned char g_lbsp_scratch[kScratchBytes];

// device address of g_lbsp_scratch per device, fetched once with that device current
std::mutex g_mu;
std::vector<unsigned char*> g_addr;

cudaError_t scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_addr.size() <= device) g_addr.resize(device + 1, nullptr);
    if (!g_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_lbsp_scratch);
        if (e != cudaSuccess) return e;
        g_addr[device] = (unsigned char*)p;
    }
    *out = g_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" lvbgs_status lvbgs_lbsp_compute2_noalloc(const uint8_t* image, int W, int H, int C, long absThr,
                                                    float rel, size_t off, uint16_t* desc, int device_id,
                                                    void* cuda_stream) {
    using lvbgs::report_error;
    if (!image || !desc || W <= 0 || H <= 0) return report_error(LVBGS_BAD_ARG, "input image must be non-empty");
    if (C != 1 && C != 3) return report_error(LVBGS_BAD_TYPE, "input image must be of type 8UC1/8UC3");
    if (absThr < 0 && !(rel >= 0)) return report_error(LVBGS_BAD_ARG, "relative LBSP threshold must be non-negative");
    const size_t n = (size_t)W * H * C;
    if (n > kMaxElems)
        return report_error(LVBGS_BAD_SIZE,
                            "lvbgs_lbsp_compute2_noalloc: width*height*channels exceeds its fixed scratch of 8,388,608 "
                            "elements; use lvbgs_lbsp_compute2");
    if (cudaSetDevice(device_id) != cudaSuccess) return report_error(LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    unsigned char* base = nullptr;
    if (scratch_address(device_id, &base) != cudaSuccess) {
        cudaGetLastError();
        return report_error(LVBGS_DEVICE_ERROR, "cannot look up the no-allocation scratch array on this device");
    }
    uint8_t* dimg = base;
    uint16_t* ddesc = (uint16_t*)(base + kDescOffset);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    // the descriptors are staged too, so the 2-pixel border keeps the caller's content, as with
    // lvbgs_lbsp_compute2; nothing of the previous call's contents is read
    cudaError_t e = cudaMemcpyAsync(dimg, image, n, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ddesc, desc, n * 2, cudaMemcpyDefault, st);
    if (e == cudaSuccess) {
        const int thr = absThr < 0 ? -1 : (int)std::min<long>(absThr, 255);
        lvbgs::lvbgs_lbsp_dense<<<256, 256, 0, st>>>(dimg, W, H, C, thr, rel, (unsigned)off, ddesc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(desc, ddesc, n * 2, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return report_error(LVBGS_DEVICE_ERROR, cudaGetErrorString(e));
    }
    return LVBGS_OK;
}
