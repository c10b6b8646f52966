// LBSP thresholding on the device, shared by the SuBSENSE and LOBSTER kernels.
#pragma once
#include <stdint.h>

namespace lvbgs {

// LBSP::computeDescriptor_threshold (LBSP.hpp:193-202) on 16 packed taps (tap n in byte n & 3 of word
// n >> 2): bit n = |tap_n - ref| > thr
__device__ __forceinline__ uint32_t lbsp_thr(const uint32_t v[4], uint32_t ref, uint32_t thr) {
    const uint32_t r4 = ref * 0x01010101u, t4 = thr * 0x01010101u;
    uint32_t d = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t m = __vcmpgtu4(__vabsdiffu4(v[j], r4), t4);
        d |= (((m & 0x80808080u) * 0x00204081u) >> 28) << (4 * j);
    }
    return d;
}

}  // namespace lvbgs
