// Test infrastructure: declaration of RAND_bytes (prng/chacha_prng_util.cc:62);
// the stand-in reports failure, since the oracle never generates seeds.
#pragma once
#include <cstddef>
#include <cstdint>
extern "C" int RAND_bytes(uint8_t* buf, size_t len);
