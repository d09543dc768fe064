// Compat stand-in (test infrastructure).
#pragma once
#include <optional>
namespace absl { using std::optional; using std::nullopt; using std::make_optional; }
