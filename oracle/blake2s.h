/*
 * ORACLE — test infrastructure only (see fields.h).
 *
 * BLAKE2s-256, unkeyed, written from RFC 7693 (sections 2.1-3.3). The
 * reference takes it from the `blake2` crate 0.10.6 (Cargo.lock:689-691) as
 * `Blake2s256` (crates/stwo/src/core/vcs/blake2_hash.rs:3,71-100). Streaming
 * semantics follow the RFC: a full 64-byte block is compressed only once more
 * input arrives, so the last block (full or partial) is the final one.
 */
#ifndef STWO_ORACLE_BLAKE2S_H
#define STWO_ORACLE_BLAKE2S_H

#include <stdint.h>
#include <string.h>

static const uint32_t B2S_IV[8] = {
    0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
    0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u,
};

static const uint8_t B2S_SIGMA[10][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15},
    {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4},
    {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13},
    {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11},
    {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5},
    {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0},
};

typedef struct {
    uint32_t h[8];
    uint64_t t;          /* bytes compressed so far */
    uint8_t buf[64];
    uint32_t buflen;
} b2s_state;

static inline uint32_t b2s_rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static inline void b2s_compress(uint32_t h[8], const uint32_t m[16], uint64_t t, int last) {
    uint32_t v[16];
    for (int i = 0; i < 8; i++) { v[i] = h[i]; v[i + 8] = B2S_IV[i]; }
    v[12] ^= (uint32_t)t;
    v[13] ^= (uint32_t)(t >> 32);
    if (last) v[14] = ~v[14];
#define B2S_G(a, b, c, d, x, y)                         \
    do {                                                \
        v[a] = v[a] + v[b] + (x); v[d] = b2s_rotr(v[d] ^ v[a], 16); \
        v[c] = v[c] + v[d];       v[b] = b2s_rotr(v[b] ^ v[c], 12); \
        v[a] = v[a] + v[b] + (y); v[d] = b2s_rotr(v[d] ^ v[a], 8);  \
        v[c] = v[c] + v[d];       v[b] = b2s_rotr(v[b] ^ v[c], 7);  \
    } while (0)
    for (int r = 0; r < 10; r++) {
        const uint8_t *s = B2S_SIGMA[r];
        B2S_G(0, 4, 8, 12, m[s[0]], m[s[1]]);
        B2S_G(1, 5, 9, 13, m[s[2]], m[s[3]]);
        B2S_G(2, 6, 10, 14, m[s[4]], m[s[5]]);
        B2S_G(3, 7, 11, 15, m[s[6]], m[s[7]]);
        B2S_G(0, 5, 10, 15, m[s[8]], m[s[9]]);
        B2S_G(1, 6, 11, 12, m[s[10]], m[s[11]]);
        B2S_G(2, 7, 8, 13, m[s[12]], m[s[13]]);
        B2S_G(3, 4, 9, 14, m[s[14]], m[s[15]]);
    }
#undef B2S_G
    for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

static inline void b2s_init(b2s_state *s) {
    for (int i = 0; i < 8; i++) s->h[i] = B2S_IV[i];
    s->h[0] ^= 0x01010000u ^ 32u;   /* depth 1, fanout 1, no key, 32-byte digest */
    s->t = 0;
    s->buflen = 0;
}

static inline void b2s_load_block(const uint8_t *b, uint32_t m[16]) {
    for (int i = 0; i < 16; i++)
        m[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) |
               ((uint32_t)b[4 * i + 2] << 16) | ((uint32_t)b[4 * i + 3] << 24);
}

static inline void b2s_update(b2s_state *s, const uint8_t *data, size_t len) {
    while (len > 0) {
        if (s->buflen == 64) {
            uint32_t m[16];
            b2s_load_block(s->buf, m);
            s->t += 64;
            b2s_compress(s->h, m, s->t, 0);
            s->buflen = 0;
        }
        size_t take = 64 - s->buflen;
        if (take > len) take = len;
        memcpy(s->buf + s->buflen, data, take);
        s->buflen += (uint32_t)take;
        data += take;
        len -= take;
    }
}

static inline void b2s_update_u32(b2s_state *s, uint32_t w) {
    uint8_t b[4] = {(uint8_t)w, (uint8_t)(w >> 8), (uint8_t)(w >> 16), (uint8_t)(w >> 24)};
    b2s_update(s, b, 4);
}

static inline void b2s_final(b2s_state *s, uint8_t out[32]) {
    uint32_t m[16];
    memset(s->buf + s->buflen, 0, 64 - s->buflen);
    b2s_load_block(s->buf, m);
    s->t += s->buflen;
    b2s_compress(s->h, m, s->t, 1);
    for (int i = 0; i < 8; i++) {
        out[4 * i] = (uint8_t)s->h[i];
        out[4 * i + 1] = (uint8_t)(s->h[i] >> 8);
        out[4 * i + 2] = (uint8_t)(s->h[i] >> 16);
        out[4 * i + 3] = (uint8_t)(s->h[i] >> 24);
    }
}

static inline void b2s_hash(const uint8_t *data, size_t len, uint8_t out[32]) {
    b2s_state s;
    b2s_init(&s);
    b2s_update(&s, data, len);
    b2s_final(&s, out);
}

#endif
