/*
 * oracle/philox.h -- TEST INFRASTRUCTURE ONLY (part of the CPU oracle, never linked into
 * the product).
 *
 * Philox4x32-10 counter-based generator, written from the published description in
 * J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw, "Parallel Random Numbers: As Easy
 * as 1, 2, 3", SC'11: each round multiplies words 0 and 2 by the two round constants,
 * takes the 64-bit products apart into hi/lo halves and recombines them with the odd
 * words and the round key; the key is bumped by the two Weyl constants between rounds.
 * Pinned against the paper's known-answer vectors in tests/test_oracle_kat.py.
 *
 * Philox2x32-10 (same paper): two words, one multiplier; each round replaces (R0, R1) by
 * (hi(M * R0) ^ key ^ R1, lo(M * R0)) and bumps the single key word by the first Weyl
 * constant.
 */
#ifndef ORACLE_PHILOX_H
#define ORACLE_PHILOX_H

#include <stdint.h>

#define ORC_PHILOX_M0 0xD2511F53u
#define ORC_PHILOX_M1 0xCD9E8D57u
#define ORC_PHILOX_W0 0x9E3779B9u
#define ORC_PHILOX_W1 0xBB67AE85u

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                                     uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            k0 += ORC_PHILOX_W0;
            k1 += ORC_PHILOX_W1;
        }
        uint64_t prod0 = (uint64_t)ORC_PHILOX_M0 * (uint64_t)c0;
        uint64_t prod1 = (uint64_t)ORC_PHILOX_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(prod0 >> 32), lo0 = (uint32_t)prod0;
        uint32_t hi1 = (uint32_t)(prod1 >> 32), lo1 = (uint32_t)prod1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define ORC_PHILOX2_M0 0xD256D193u

static inline void orc_philox2x32_10(const uint32_t ctr_in[2], uint32_t key, uint32_t out[2]) {
    uint32_t r0 = ctr_in[0], r1 = ctr_in[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) key += ORC_PHILOX_W0;
        uint64_t prod = (uint64_t)ORC_PHILOX2_M0 * (uint64_t)r0;
        uint32_t n0 = (uint32_t)(prod >> 32) ^ key ^ r1;
        uint32_t n1 = (uint32_t)prod;
        r0 = n0; r1 = n1;
    }
    out[0] = r0; out[1] = r1;
}

#endif
