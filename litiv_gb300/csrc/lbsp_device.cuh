// LBSP thresholding on the device, shared by the SuBSENSE and LOBSTER kernels.
#pragma once
#include <stdint.h>

namespace lvbgs {

// bit 7 of each byte = (a > b) for the unsigned bytes of a and b, given nb = ~b and nbL = nb & 0x7f7f7f7f:
// a > b exactly when a + ~b carries out of the byte. The low seven bits of each byte are added without
// crossing into the next byte, and the carry out of bit 7 is the majority of a, ~b and that sum's bit 7.
// Bits 0-6 of each byte of the result are not defined.
__device__ __forceinline__ uint32_t bytes_gt(uint32_t a, uint32_t nb, uint32_t nbL) {
    const uint32_t s = (a & 0x7f7f7f7fu) + nbL;
    return (a & nb) | (a & s) | (nb & s);
}

// 8 descriptor bits from the byte masks of tap words 2k and 2k+1 (bit 7 of each byte): the bit of byte i
// of word 2k+j is moved to bit 8i + 3 + 4j, and the product with 2^21 + 2^14 + 2^7 + 1 shifts source byte
// i by 21 - 7i, so that byte 3 of the product holds tap 8k + 4j + i at bit 4j + i. No two partial products
// share a bit position (the other ones fall below bit 24 or above bit 31), so nothing carries into byte 3.
__device__ __forceinline__ uint32_t gather8(uint32_t m0, uint32_t m1) {
    return (((m0 & 0x80808080u) >> 4) | (m1 & 0x80808080u)) * 0x00204081u;
}

// LBSP::computeDescriptor_threshold (LBSP.hpp:193-202) on 16 packed taps (tap n in byte n & 3 of word
// n >> 2): bit n = |tap_n - ref| > thr. Bits 0-15 hold the descriptor; bits 16-31 are not defined (the
// callers mask them where they combine the descriptor with another one).
__device__ __forceinline__ uint32_t lbsp_thr_raw(const uint32_t v[4], uint32_t ref, uint32_t thr) {
    const uint32_t r4 = ref * 0x01010101u, nt4 = ~(thr * 0x01010101u), ntL = nt4 & 0x7f7f7f7fu;
    uint32_t m[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) m[j] = bytes_gt(__vabsdiffu4(v[j], r4), nt4, ntL);
    return __byte_perm(gather8(m[0], m[1]), gather8(m[2], m[3]), 0x0073);
}
__device__ __forceinline__ uint32_t lbsp_thr(const uint32_t v[4], uint32_t ref, uint32_t thr) {
    return lbsp_thr_raw(v, ref, thr) & 0xffffu;
}

}  // namespace lvbgs
