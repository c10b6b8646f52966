/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * Philox4x32-10 counter-based generator, written from the published description
 * (J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel Random Numbers: As Easy as
 * 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies, key bumped by the
 * Weyl constants between rounds.
 *
 * It replaces glibc rand() on the reference path. Every rand() call of the
 * reference (BackgroundSubtractorSuBSENSE.cpp:86,93,264-265,278-279,286-297,
 * 406-407,422-444) becomes draw k of pixel p in frame t:
 *     block = philox(ctr = {k>>2, p, t, 0}, key = {seed_lo, seed_hi})
 *     draw  = block[k & 3] & 0x7fffffff          (31 bits, like RAND_MAX)
 * The per-pixel draw counter k restarts at 0 for every frame (initialize() is
 * frame 0, the i-th apply() is frame i). Frame-level draws use p = 0xffffffff.
 */
#ifndef LV_ORACLE_PHILOX_H
#define LV_ORACLE_PHILOX_H
#include <stdint.h>

#define OPHILOX_M0 0xD2511F53u
#define OPHILOX_M1 0xCD9E8D57u
#define OPHILOX_W0 0x9E3779B9u
#define OPHILOX_W1 0xBB67AE85u
#define OPHILOX_SENTINEL_PX 0xFFFFFFFFu

static inline void ophilox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t x0 = ctr_in[0], x1 = ctr_in[1], x2 = ctr_in[2], x3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += OPHILOX_W0; k1 += OPHILOX_W1; }
        const uint64_t p0 = (uint64_t)OPHILOX_M0 * x0;
        const uint64_t p1 = (uint64_t)OPHILOX_M1 * x2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ x1 ^ k0;
        const uint32_t n2 = hi0 ^ x3 ^ k1;
        x0 = n0; x1 = lo1; x2 = n2; x3 = lo0;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

#endif
