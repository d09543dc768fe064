// Test infrastructure: link-time stand-ins for the two BoringSSL functions the
// reference's ChaCha PRNG calls.  CRYPTO_chacha_20 is RFC 7539 ChaCha20
// (oracle/chacha20.h, checked against the RFC's test vector and Python's
// `cryptography`); RAND_bytes fails, as seeds are always passed in.
#include <cstddef>
#include <cstdint>

#include "../chacha20.h"

extern "C" void CRYPTO_chacha_20(uint8_t* out, const uint8_t* in, size_t in_len,
                                 const uint8_t key[32], const uint8_t nonce[12],
                                 uint32_t counter) {
  shg_chacha20_xor(out, in, in_len, key, nonce, counter);
}

extern "C" int RAND_bytes(uint8_t*, size_t) { return 0; }
