// Dense LBSP extraction for callers that must not allocate device memory.
//
// lvbgs_lbsp_compute2() stages the caller's image and descriptor buffers in device memory it
// allocates per call. Code that runs where cudaMalloc/cudaFree are off limits -- a real-time
// capture thread with a no-allocation rule, or a host that shares the GPU under a fixed memory
// budget -- uses lvbgs_lbsp_compute2_noalloc() instead: the staging lives in one file-scope
// device array, so a call allocates nothing once the array exists on the device. The CUDA runtime
// loads a module (and reserves its __device__ arrays) when the module is first used on a device
// (lazy loading, the default unless CUDA_MODULE_LOADING=EAGER), so the first call on a device --
// or any earlier use of this library there -- is what reserves the 24 MiB and loads the LBSP
// kernel; a caller under a no-allocation rule makes that first call during its set-up.
#include <cuda_runtime.h>

#include <algorithm>

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

// Device address of g_lbsp_scratch on the current device. In host code the array's name is only
// a host-side stand-in, so the address is looked up with the device current. It is looked up on
// every call (a host-side table lookup once the module is loaded; it allocates nothing), so a
// cudaDeviceReset() by the application, which unloads the module, leaves no stale address behind.
cudaError_t scratch_address(unsigned char** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_lbsp_scratch);
    if (e != cudaSuccess) return e;
    *out = (unsigned char*)p;
    return cudaSuccess;
}

// Makes `device` current for the life of the object and puts the caller's current device back.
struct DeviceGuard {
    int prev = -1, dev = -1;
    bool ok = false;
    explicit DeviceGuard(int device) : dev(device) {
        if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); prev = -1; }
        ok = prev == device || cudaSetDevice(device) == cudaSuccess;
        if (!ok) cudaGetLastError();
    }
    ~DeviceGuard() {
        if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
};

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
    DeviceGuard guard(device_id);
    if (!guard.ok) return report_error(LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (st) {
        int sdev = -1;
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return report_error(LVBGS_BAD_ARG, "lvbgs_lbsp_compute2_noalloc: invalid cuda_stream");
        }
        if (sdev != device_id)
            return report_error(LVBGS_BAD_ARG, "lvbgs_lbsp_compute2_noalloc: cuda_stream belongs to another device");
    }
    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) {
        cudaGetLastError();
        return report_error(LVBGS_DEVICE_ERROR, "cannot look up the no-allocation scratch array on this device");
    }
    uint8_t* dimg = base;
    uint16_t* ddesc = (uint16_t*)(base + kDescOffset);
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
