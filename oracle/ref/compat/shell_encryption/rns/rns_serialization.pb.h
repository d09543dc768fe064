// Compat stand-in (test infrastructure) for shell_encryption/rns/rns_serialization.proto.
#pragma once
#include "shell_encryption/serialization.pb.h"
namespace rlwe {
class SerializedRnsPolynomial {
  SHG_PB_OPT(int32_t, log_n)
  SHG_PB_REP(std::string, coeff_vectors)
  SHG_PB_OPT(bool, is_ntt)
};
class SerializedRnsRlweCiphertext {
  SHG_PB_REP(SerializedRnsPolynomial, components)
  SHG_PB_OPT(int32_t, power_of_s)
  SHG_PB_OPT(double, error)
};
class SerializedRnsGaloisKey {
  SHG_PB_REP(SerializedRnsPolynomial, key_bs)
  SHG_PB_OPT(int32_t, power)
  SHG_PB_OPT(std::string, prng_seed)
  SHG_PB_OPT(PrngType, prng_type)
};
}  // namespace rlwe
