// Compat stand-in (test infrastructure): StrFormat via snprintf.
#pragma once
#include <cstdio>
#include <string>
#include <type_traits>
namespace absl {
namespace compat_internal {
template <typename T> auto fmt_arg(const T& v) {
  if constexpr (std::is_same_v<T, std::string>) return v.c_str();
  else return v;
}
}  // namespace compat_internal
template <typename... Args>
std::string StrFormat(const char* fmt, const Args&... args) {
  char buf[1024];
  std::snprintf(buf, sizeof(buf), fmt, compat_internal::fmt_arg(args)...);
  return buf;
}
}  // namespace absl
