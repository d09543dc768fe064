/* Test infrastructure (oracle): the ChaCha20 block function of RFC 7539
 * (section 2.3), restated from the RFC, and the byte stream of SHELL's
 * ChaChaPrng built on it (prng/chacha_prng_util.cc:30-98): salt s gives
 * 8160 bytes (kChaChaOutputBytes, prng/chacha_prng_util.h:36) of ChaCha20
 * keystream under the 32-byte seed, nonce "salt" || s as 8 little-endian
 * bytes, block counter from 0; Rand8 takes the next byte, Rand64 the next 8
 * bytes little-endian.  Checked against RFC 7539's test vector and Python's
 * `cryptography` ChaCha20 in tests/test_oracle.py. */
#ifndef SHG_ORACLE_CHACHA20_H_
#define SHG_ORACLE_CHACHA20_H_

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#define SHG_CHACHA_SALT_BYTES 8160u

static inline uint32_t shg_rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

static inline uint32_t shg_load32_le(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
         ((uint32_t)p[3] << 24);
}

#define SHG_QR(a, b, c, d)                  \
  a += b; d ^= a; d = shg_rotl32(d, 16);    \
  c += d; b ^= c; b = shg_rotl32(b, 12);    \
  a += b; d ^= a; d = shg_rotl32(d, 8);     \
  c += d; b ^= c; b = shg_rotl32(b, 7);

/* One 64-byte keystream block (RFC 7539 section 2.3.2). */
static inline void shg_chacha20_block(const uint8_t key[32], uint32_t counter,
                                      const uint8_t nonce[12], uint8_t out[64]) {
  uint32_t s[16], x[16];
  s[0] = 0x61707865u; /* "expand 32-byte k" */
  s[1] = 0x3320646eu;
  s[2] = 0x79622d32u;
  s[3] = 0x6b206574u;
  for (int i = 0; i < 8; i++) s[4 + i] = shg_load32_le(key + 4 * i);
  s[12] = counter;
  for (int i = 0; i < 3; i++) s[13 + i] = shg_load32_le(nonce + 4 * i);
  memcpy(x, s, sizeof(x));
  for (int r = 0; r < 10; r++) {
    SHG_QR(x[0], x[4], x[8], x[12]) SHG_QR(x[1], x[5], x[9], x[13])
    SHG_QR(x[2], x[6], x[10], x[14]) SHG_QR(x[3], x[7], x[11], x[15])
    SHG_QR(x[0], x[5], x[10], x[15]) SHG_QR(x[1], x[6], x[11], x[12])
    SHG_QR(x[2], x[7], x[8], x[13]) SHG_QR(x[3], x[4], x[9], x[14])
  }
  for (int i = 0; i < 16; i++) {
    const uint32_t v = x[i] + s[i];
    out[4 * i] = (uint8_t)v;
    out[4 * i + 1] = (uint8_t)(v >> 8);
    out[4 * i + 2] = (uint8_t)(v >> 16);
    out[4 * i + 3] = (uint8_t)(v >> 24);
  }
}

/* out[i] = in[i] ^ keystream starting at block `counter` (RFC 7539 2.4). */
static inline void shg_chacha20_xor(uint8_t* out, const uint8_t* in, size_t len,
                                    const uint8_t key[32], const uint8_t nonce[12],
                                    uint32_t counter) {
  uint8_t block[64];
  for (size_t off = 0; off < len; off += 64, counter++) {
    shg_chacha20_block(key, counter, nonce, block);
    const size_t m = len - off < 64 ? len - off : 64;
    for (size_t i = 0; i < m; i++) out[off + i] = in[off + i] ^ block[i];
  }
}

/* Bytes [start, start + len) of the ChaChaPrng stream of `seed`. */
static inline void shg_chacha_prng_bytes(const uint8_t seed[32], uint64_t start, size_t len,
                                         uint8_t* out) {
  uint8_t block[64], nonce[12] = {'s', 'a', 'l', 't'};
  uint64_t salt_cached = ~(uint64_t)0;
  uint32_t block_cached = ~(uint32_t)0;
  for (size_t i = 0; i < len; i++) {
    const uint64_t b = start + i;
    const uint64_t salt = b / SHG_CHACHA_SALT_BYTES;
    const uint32_t off = (uint32_t)(b % SHG_CHACHA_SALT_BYTES);
    if (salt != salt_cached || off / 64 != block_cached) {
      for (int k = 0; k < 8; k++) nonce[4 + k] = (uint8_t)(salt >> (8 * k));
      shg_chacha20_block(seed, off / 64, nonce, block);
      salt_cached = salt;
      block_cached = off / 64;
    }
    out[i] = block[off % 64];
  }
}

#endif /* SHG_ORACLE_CHACHA20_H_ */
