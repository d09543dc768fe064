// Compat stand-in (test infrastructure): StrCat via ostringstream.
#pragma once
#include <sstream>
#include <string>
#include "absl/numeric/int128.h"
namespace absl {
template <typename... Args>
std::string StrCat(const Args&... args) {
  std::ostringstream os;
  (os << ... << args);
  return os.str();
}
template <typename... Args>
void StrAppend(std::string* dst, const Args&... args) { *dst += StrCat(args...); }
}  // namespace absl
