// Compat stand-in (test infrastructure): a minimal absl::Status for building
// the reference's hot-path sources in place.
#pragma once
// The reference relies on std headers reaching it through absl's own headers.
#include <algorithm>
#include <cmath>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <sstream>
#include <tuple>
#include <vector>
#include <ostream>
#include <string>
#include "absl/base/attributes.h"
#include "absl/memory/memory.h"
#include <string_view>
#include <utility>

namespace absl {
enum class StatusCode : int {
  kOk = 0, kCancelled = 1, kUnknown = 2, kInvalidArgument = 3, kDeadlineExceeded = 4,
  kNotFound = 5, kAlreadyExists = 6, kPermissionDenied = 7, kResourceExhausted = 8,
  kFailedPrecondition = 9, kAborted = 10, kOutOfRange = 11, kUnimplemented = 12,
  kInternal = 13, kUnavailable = 14, kDataLoss = 15, kUnauthenticated = 16,
};
class Status {
 public:
  Status() = default;
  Status(StatusCode c, std::string_view m) : code_(c), msg_(m) {}
  bool ok() const { return code_ == StatusCode::kOk; }
  StatusCode code() const { return code_; }
  std::string_view message() const { return msg_; }
  std::string ToString() const { return std::to_string((int)code_) + ": " + msg_; }
  void IgnoreError() const {}
  bool operator==(const Status& o) const { return code_ == o.code_ && msg_ == o.msg_; }
 private:
  StatusCode code_ = StatusCode::kOk;
  std::string msg_;
};
inline std::ostream& operator<<(std::ostream& os, const Status& s) { return os << s.ToString(); }
inline Status OkStatus() { return Status(); }
inline Status InvalidArgumentError(std::string_view m) { return Status(StatusCode::kInvalidArgument, m); }
inline Status InternalError(std::string_view m) { return Status(StatusCode::kInternal, m); }
inline Status UnknownError(std::string_view m) { return Status(StatusCode::kUnknown, m); }
inline Status FailedPreconditionError(std::string_view m) { return Status(StatusCode::kFailedPrecondition, m); }
inline Status OutOfRangeError(std::string_view m) { return Status(StatusCode::kOutOfRange, m); }
inline Status NotFoundError(std::string_view m) { return Status(StatusCode::kNotFound, m); }
inline Status UnimplementedError(std::string_view m) { return Status(StatusCode::kUnimplemented, m); }
inline Status ResourceExhaustedError(std::string_view m) { return Status(StatusCode::kResourceExhausted, m); }
inline Status AbortedError(std::string_view m) { return Status(StatusCode::kAborted, m); }
inline Status DataLossError(std::string_view m) { return Status(StatusCode::kDataLoss, m); }
inline bool IsInvalidArgument(const Status& s) { return s.code() == StatusCode::kInvalidArgument; }
}  // namespace absl
