// Compat stand-in (test infrastructure): a minimal absl::Span<T>.
#pragma once
#include <array>
#include <cstddef>
#include <initializer_list>
#include <type_traits>
#include <vector>
namespace absl {
template <typename T>
class Span {
 public:
  using element_type = T;
  using value_type = std::remove_cv_t<T>;
  using pointer = T*;
  using iterator = T*;
  using const_iterator = const T*;
  constexpr Span() = default;
  constexpr Span(T* p, size_t n) : p_(p), n_(n) {}
  template <typename U, typename A,
            typename = std::enable_if_t<std::is_convertible_v<U*, T*>>>
  Span(std::vector<U, A>& v) : p_(v.data()), n_(v.size()) {}
  template <typename U, typename A,
            typename = std::enable_if_t<std::is_convertible_v<const U*, T*>>>
  Span(const std::vector<U, A>& v) : p_(v.data()), n_(v.size()) {}
  template <typename U, size_t N, typename = std::enable_if_t<std::is_convertible_v<U*, T*>>>
  Span(std::array<U, N>& a) : p_(a.data()), n_(N) {}
  template <typename U, size_t N, typename = std::enable_if_t<std::is_convertible_v<const U*, T*>>>
  Span(const std::array<U, N>& a) : p_(a.data()), n_(N) {}
  template <size_t N> constexpr Span(T (&a)[N]) : p_(a), n_(N) {}
  Span(std::initializer_list<value_type> il) : p_(il.begin()), n_(il.size()) {}
  template <typename U, typename = std::enable_if_t<std::is_convertible_v<U*, T*>>>
  constexpr Span(const Span<U>& o) : p_(o.data()), n_(o.size()) {}
  constexpr T* data() const { return p_; }
  constexpr size_t size() const { return n_; }
  constexpr size_t length() const { return n_; }
  constexpr bool empty() const { return n_ == 0; }
  constexpr T& operator[](size_t i) const { return p_[i]; }
  constexpr T& at(size_t i) const { return p_[i]; }
  constexpr T& front() const { return p_[0]; }
  constexpr T& back() const { return p_[n_ - 1]; }
  constexpr T* begin() const { return p_; }
  constexpr T* end() const { return p_ + n_; }
  constexpr Span first(size_t k) const { return Span(p_, k); }
  constexpr Span last(size_t k) const { return Span(p_ + n_ - k, k); }
  constexpr Span subspan(size_t pos, size_t len = static_cast<size_t>(-1)) const {
    size_t l = len > n_ - pos ? n_ - pos : len;
    return Span(p_ + pos, l);
  }
 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};
template <typename T> Span<T> MakeSpan(T* p, size_t n) { return Span<T>(p, n); }
template <typename C> auto MakeSpan(C& c) { return Span<std::remove_reference_t<decltype(*c.data())>>(c.data(), c.size()); }
template <typename C> auto MakeSpan(const C& c) { return Span<std::remove_reference_t<decltype(*c.data())>>(c.data(), c.size()); }
template <typename T> Span<const T> MakeConstSpan(T* p, size_t n) { return Span<const T>(p, n); }
template <typename C> auto MakeConstSpan(const C& c) { return Span<const std::remove_const_t<std::remove_reference_t<decltype(*c.data())>>>(c.data(), c.size()); }
}  // namespace absl
