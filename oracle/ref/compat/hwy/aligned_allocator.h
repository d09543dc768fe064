// Compat stand-in (test infrastructure): scalar build, no Highway.
#pragma once
#include <vector>
namespace hwy { template <typename T> using AlignedVector = std::vector<T>; }
