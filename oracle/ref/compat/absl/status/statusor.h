// Compat stand-in (test infrastructure): a minimal absl::StatusOr<T>.
#pragma once
#include <cstdlib>
#include <optional>
#include <utility>
#include "absl/status/status.h"

namespace absl {
template <typename T>
class StatusOr {
 public:
  StatusOr() : status_(StatusCode::kUnknown, "") {}
  StatusOr(const Status& s) : status_(s) {}
  StatusOr(Status&& s) : status_(std::move(s)) {}
  StatusOr(const T& v) : value_(v) {}
  StatusOr(T&& v) : value_(std::move(v)) {}
  template <typename U, typename = std::enable_if_t<std::is_constructible_v<T, U&&> &&
                                                    !std::is_same_v<std::decay_t<U>, Status> &&
                                                    !std::is_same_v<std::decay_t<U>, StatusOr>>>
  StatusOr(U&& v) : value_(T(std::forward<U>(v))) {}
  template <typename U>
  StatusOr(StatusOr<U>&& o) : status_(o.status()) {
    if (o.ok()) value_.emplace(std::move(*o));
  }
  StatusOr(const StatusOr&) = default;
  StatusOr(StatusOr&&) = default;
  StatusOr& operator=(const StatusOr&) = default;
  StatusOr& operator=(StatusOr&&) = default;
  bool ok() const { return status_.ok(); }
  const Status& status() const { return status_; }
  const T& value() const& { check(); return *value_; }
  T& value() & { check(); return *value_; }
  T&& value() && { check(); return std::move(*value_); }
  const T& operator*() const& { return *value_; }
  T& operator*() & { return *value_; }
  T&& operator*() && { return std::move(*value_); }
  const T* operator->() const { return &*value_; }
  T* operator->() { return &*value_; }
 private:
  void check() const { if (!status_.ok()) std::abort(); }
  Status status_;
  std::optional<T> value_;
};
}  // namespace absl
