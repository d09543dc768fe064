// Compat stand-in (test infrastructure): plain structs with the accessor
// surface of the protobuf messages in shell_encryption/serialization.proto,
// enough for the reference sources to compile; no wire format.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#define SHG_PB_OPT(T, name)                                   \
 private:                                                     \
  T name##_{};                                                \
  bool has_##name##_ = false;                                 \
 public:                                                      \
  const T& name() const { return name##_; }                   \
  void set_##name(const T& v) { name##_ = v; has_##name##_ = true; } \
  T* mutable_##name() { has_##name##_ = true; return &name##_; } \
  bool has_##name() const { return has_##name##_; }

#define SHG_PB_REP(T, name)                                   \
 private:                                                     \
  std::vector<T> name##_;                                     \
 public:                                                      \
  const std::vector<T>& name() const { return name##_; }      \
  const T& name(int i) const { return name##_[i]; }           \
  T* mutable_##name(int i) { return &name##_[i]; }            \
  std::vector<T>* mutable_##name() { return &name##_; }       \
  int name##_size() const { return (int)name##_.size(); }     \
  T* add_##name() { name##_.emplace_back(); return &name##_.back(); } \
  void add_##name(const T& v) { name##_.push_back(v); }

namespace rlwe {
enum PrngType { PRNG_TYPE_INVALID = 0, PRNG_TYPE_HKDF = 1, PRNG_TYPE_CHACHA = 2 };
inline bool PrngType_IsValid(int v) { return v >= 0 && v <= 2; }
class SerializedNttPolynomial {
  SHG_PB_OPT(std::string, coeffs)
  SHG_PB_OPT(int32_t, num_coeffs)
};
class SerializedSymmetricRlweCiphertext {
  SHG_PB_REP(SerializedNttPolynomial, c)
  SHG_PB_OPT(int32_t, power_of_s)
  SHG_PB_OPT(double, error)
};
class SerializedRelinearizationKey {
  SHG_PB_REP(SerializedNttPolynomial, c)
  SHG_PB_OPT(int32_t, log_decomposition_modulus)
  SHG_PB_OPT(int32_t, num_parts)
  SHG_PB_OPT(std::string, prng_seed)
  SHG_PB_OPT(PrngType, prng_type)
  SHG_PB_OPT(int32_t, power_of_s)
};
class SerializedGaloisKey {
  SHG_PB_OPT(SerializedRelinearizationKey, key)
};
class SerializedPublicRlweKey {
  SHG_PB_OPT(std::string, prng_seed)
  SHG_PB_OPT(PrngType, prng_type)
  SHG_PB_OPT(SerializedNttPolynomial, b)
};
class SerializedAuxModRelinearizationKey {
  SHG_PB_REP(SerializedNttPolynomial, b)
  SHG_PB_OPT(int32_t, num_components)
  SHG_PB_OPT(std::string, prng_seed)
  SHG_PB_OPT(PrngType, prng_type)
  SHG_PB_OPT(int32_t, power_of_s)
};
class SerializedAuxModGaloisKey {
  SHG_PB_OPT(SerializedAuxModRelinearizationKey, key)
};
}  // namespace rlwe
