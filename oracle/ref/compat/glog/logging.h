// Compat stand-in (test infrastructure): CHECK / LOG macros that abort.
#pragma once
#include <cstdlib>
#include <iostream>
namespace compat_log {
struct Fatal {
  bool fatal;
  explicit Fatal(bool f) : fatal(f) {}
  ~Fatal() { if (fatal) { std::cerr << std::endl; std::abort(); } }
  template <typename T> Fatal& operator<<(const T& v) { if (fatal) std::cerr << v; return *this; }
};
}  // namespace compat_log
#define CHECK(c) compat_log::Fatal(!(c))
#define CHECK_EQ(a, b) CHECK((a) == (b))
#define CHECK_NE(a, b) CHECK((a) != (b))
#define CHECK_LT(a, b) CHECK((a) < (b))
#define CHECK_LE(a, b) CHECK((a) <= (b))
#define CHECK_GT(a, b) CHECK((a) > (b))
#define CHECK_GE(a, b) CHECK((a) >= (b))
#define CHECK_OK(s) CHECK((s).ok())
#define DCHECK(c) CHECK(c)
#define DCHECK_EQ(a, b) CHECK_EQ(a, b)
#define DCHECK_NE(a, b) CHECK_NE(a, b)
#define DCHECK_GT(a, b) CHECK_GT(a, b)
#define DCHECK_LT(a, b) CHECK_LT(a, b)
#define DCHECK_LE(a, b) CHECK_LE(a, b)
#define DCHECK_GE(a, b) CHECK_GE(a, b)
#define LOG(level) compat_log::Fatal(std::string(#level) == "FATAL")
