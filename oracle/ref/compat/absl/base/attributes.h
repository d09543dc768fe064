// Compat stand-in (test infrastructure): the attribute macros the reference uses.
#pragma once
#define ABSL_MUST_USE_RESULT
#define ABSL_DEPRECATED(msg) [[deprecated(msg)]]
#define ABSL_ATTRIBUTE_UNUSED __attribute__((unused))
#define ABSL_PREDICT_FALSE(x) (__builtin_expect(false || (x), false))
#define ABSL_PREDICT_TRUE(x) (__builtin_expect(false || (x), true))
