// Compat stand-in (test infrastructure).
#pragma once
#include <memory>
namespace absl {
template <typename T> std::unique_ptr<T> WrapUnique(T* p) { return std::unique_ptr<T>(p); }
}
