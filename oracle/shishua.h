/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product links this file.
 *
 * SHISHUA pseudo-random generator, written for this project from the public
 * SHISHUA design (espadrine/shishua, "shishua" full variant: four 256-bit state
 * lanes, a 256-bit counter, 128-byte output blocks, 13 initialisation rounds).
 * The reference does not vendor SHISHUA: its build clones upstream `master`
 * at build time (Makefile.am:157-159) and patches `prng_init` to be `inline`
 * (shishua_inline_patch.diff:7-8,18-19).  This header exposes exactly the API
 * that the reference's src/RNG.cpp binds:
 *     prng_state, prng_init(prng_state*, uint64_t seed[4]),
 *     prng_gen(prng_state*, uint8_t* buf, size_t bytes)
 * and includes <assert.h>/<string.h>, which RNG.cpp relies on transitively.
 *
 * Pinning: the 16 initialisation constants are the first 1024 bits of the
 * hexadecimal expansion of (sqrt(5)-1)/2; the last four of them also appear
 * verbatim in the reference patch context (shishua_inline_patch.diff:4,15),
 * and tests/test_oracle_rng.py recomputes all sixteen from their definition.
 * Upstream publishes no test vector that the reference repeats, so bit parity
 * with upstream's own output stream is NOT pinned beyond the constants.
 *
 * Layout: the state is four 256-bit lanes S0..S3, each held as four
 * little-endian 64-bit words.  One round, per 64-bit word k of each lane:
 *   S1 += C, S3 += C, C += (7,5,3,1)                      (counter stirring)
 *   U0 = S0>>1, U1 = S1>>3, U2 = S2>>1, U3 = S3>>3          (lossy shifts)
 *   T0 = rot32x5(S0), T1 = rot32x3(S1), T2 = rot32x5(S2), T3 = rot32x3(S3)
 *        (rot32xR: rotate the eight 32-bit halves of the lane so that 32-bit
 *         element i of the result is element (i+R) mod 8 of the input)
 *   S0 = T0+U0, S1 = T1+U1, S2 = T2+U2, S3 = T3+U3
 *   O0 = U0^T1, O1 = U2^T3, O2 = S0^S3, O3 = S2^S1          (output block)
 * prng_gen emits the pending output block, then runs one round.
 * prng_init XORs the seed into the constants and runs 13 rounds, each
 * followed by S = (O3, O2, O1, O0).
 */
#ifndef HEXO_ORACLE_SHISHUA_H
#define HEXO_ORACLE_SHISHUA_H

#include <assert.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

typedef struct prng_state {
    uint64_t state[16];   /* lane L, word k at state[4*L+k] */
    uint64_t output[16];  /* pending 128-byte block, same layout */
    uint64_t counter[4];
} prng_state;

/* 32-bit-element rotation of one 256-bit lane held as four 64-bit words:
 * result word k = high half of word (k+h) | low half of word (k+h+1) << 32,
 * with h = 2 for a rotation by five elements and h = 1 for three. */
static inline void hexo_sh_rot32(const uint64_t w[4], uint64_t r[4], unsigned h)
{
    for (unsigned k = 0; k < 4; ++k)
        r[k] = (w[(k + h) & 3u] >> 32) | (w[(k + h + 1u) & 3u] << 32);
}

static inline void hexo_sh_round(prng_state *s)
{
    static const uint64_t inc[4] = {7u, 5u, 3u, 1u};
    uint64_t *s0 = &s->state[0], *s1 = &s->state[4];
    uint64_t *s2 = &s->state[8], *s3 = &s->state[12];
    uint64_t u0[4], u1[4], u2[4], u3[4], t0[4], t1[4], t2[4], t3[4];
    for (unsigned k = 0; k < 4; ++k) {
        s1[k] += s->counter[k];
        s3[k] += s->counter[k];
        s->counter[k] += inc[k];
    }
    for (unsigned k = 0; k < 4; ++k) {
        u0[k] = s0[k] >> 1;
        u1[k] = s1[k] >> 3;
        u2[k] = s2[k] >> 1;
        u3[k] = s3[k] >> 3;
    }
    hexo_sh_rot32(s0, t0, 2u);
    hexo_sh_rot32(s1, t1, 1u);
    hexo_sh_rot32(s2, t2, 2u);
    hexo_sh_rot32(s3, t3, 1u);
    for (unsigned k = 0; k < 4; ++k) {
        s0[k] = t0[k] + u0[k];
        s1[k] = t1[k] + u1[k];
        s2[k] = t2[k] + u2[k];
        s3[k] = t3[k] + u3[k];
    }
    for (unsigned k = 0; k < 4; ++k) {
        s->output[k]      = u0[k] ^ t1[k];
        s->output[4 + k]  = u2[k] ^ t3[k];
        s->output[8 + k]  = s0[k] ^ s3[k];
        s->output[12 + k] = s2[k] ^ s1[k];
    }
}

static inline void hexo_sh_store_le64(uint8_t *dst, uint64_t v)
{
    for (unsigned b = 0; b < 8; ++b) dst[b] = (uint8_t)(v >> (8u * b));
}

/* Emits `size` bytes (a multiple of 128); buf may be NULL to skip blocks. */
static inline void prng_gen(prng_state *s, uint8_t *buf, size_t size)
{
    assert(size % 128 == 0 && "shishua emits whole 128-byte blocks");
    for (size_t off = 0; off < size; off += 128) {
        if (buf != NULL)
            for (unsigned j = 0; j < 16; ++j) hexo_sh_store_le64(buf + off + 8u * j, s->output[j]);
        hexo_sh_round(s);
    }
}

static inline void prng_init(prng_state *s, uint64_t seed[4])
{
    /* First 1024 bits of the hexadecimal expansion of (sqrt(5)-1)/2. */
    static const uint64_t phi[16] = {
        0x9E3779B97F4A7C15ull, 0xF39CC0605CEDC834ull, 0x1082276BF3A27251ull, 0xF86C6A11D0C18E95ull,
        0x2767F0B153D27B7Full, 0x0347045B5BF1827Full, 0x01886F0928403002ull, 0xC1D64BA40F335E36ull,
        0xF06AD7AE9717877Eull, 0x85839D6EFFBD7DC6ull, 0x64D325D1C5371682ull, 0xCADD0CCCFDFFBBE1ull,
        0x626E33B8D04B4331ull, 0xBBF73C790D94F79Dull, 0x471C4AB3ED3D82A5ull, 0xFEC507705E4AE6E5ull,
    };
    /* which seed word is XORed into the even words of each lane */
    static const unsigned seed_lo[4] = {0u, 2u, 2u, 0u};
    static const unsigned seed_hi[4] = {1u, 3u, 3u, 1u};
    memset(s, 0, sizeof(*s));
    for (unsigned lane = 0; lane < 4; ++lane) {
        s->state[4 * lane + 0] = phi[4 * lane + 0] ^ seed[seed_lo[lane]];
        s->state[4 * lane + 1] = phi[4 * lane + 1];
        s->state[4 * lane + 2] = phi[4 * lane + 2] ^ seed[seed_hi[lane]];
        s->state[4 * lane + 3] = phi[4 * lane + 3];
    }
    for (unsigned r = 0; r < 13; ++r) {
        hexo_sh_round(s);
        for (unsigned lane = 0; lane < 4; ++lane)
            for (unsigned k = 0; k < 4; ++k)
                s->state[4 * lane + k] = s->output[4 * (3 - lane) + k];
    }
}

#endif
