// Test infrastructure: declaration of BoringSSL's CRYPTO_chacha_20 for the
// shim build of the reference's ChaCha PRNG (prng/chacha_prng_util.cc:51-54);
// the stand-in definition is oracle/ref/openssl_standin.cc.
#pragma once
#include <cstddef>
#include <cstdint>
extern "C" void CRYPTO_chacha_20(uint8_t* out, const uint8_t* in, size_t in_len,
                                 const uint8_t key[32], const uint8_t nonce[12],
                                 uint32_t counter);
