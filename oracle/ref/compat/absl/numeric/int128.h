// Compat stand-in (test infrastructure): absl::uint128 as the compiler's
// unsigned __int128 (ABSL_HAVE_INTRINSIC_INT128 stays undefined so the
// reference's duplicate __int128 specialisations are not compiled).
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <ostream>
#include <string>
namespace absl {
using uint128 = unsigned __int128;
using int128 = __int128;
inline constexpr uint64_t Uint128High64(uint128 v) { return (uint64_t)(v >> 64); }
inline constexpr uint64_t Uint128Low64(uint128 v) { return (uint64_t)v; }
inline constexpr uint128 MakeUint128(uint64_t hi, uint64_t lo) { return ((uint128)hi << 64) | lo; }
inline constexpr uint128 Uint128Max() { return ~(uint128)0; }
inline constexpr int128 MakeInt128(int64_t hi, uint64_t lo) { return (int128)(((uint128)(uint64_t)hi << 64) | lo); }
inline std::string U128ToString(uint128 v) {
  if (v == 0) return "0";
  std::string s;
  while (v) { s.insert(s.begin(), char('0' + (int)(v % 10))); v /= 10; }
  return s;
}
}  // namespace absl
inline std::ostream& operator<<(std::ostream& os, unsigned __int128 v) {
  return os << absl::U128ToString(v);
}
// Make the overload visible inside namespace rlwe, whose own operator<<
// (for uint256) would otherwise hide it.
namespace rlwe { using ::operator<<; }
