// Compat stand-in (test infrastructure).
#pragma once
#include <algorithm>
#include <numeric>
namespace absl {
template <typename C, typename T> T c_accumulate(const C& c, T init) { return std::accumulate(c.begin(), c.end(), init); }
template <typename C, typename T, typename Op> T c_accumulate(const C& c, T init, Op op) { return std::accumulate(c.begin(), c.end(), init, op); }
template <typename C, typename P> bool c_all_of(const C& c, P p) { return std::all_of(c.begin(), c.end(), p); }
template <typename C, typename P> bool c_any_of(const C& c, P p) { return std::any_of(c.begin(), c.end(), p); }
template <typename C, typename T> auto c_find(C& c, const T& v) { return std::find(c.begin(), c.end(), v); }
}  // namespace absl
