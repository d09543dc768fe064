// Test infrastructure: link-time stand-ins for the reference's HKDF PRNG seed
// generator and PRNG (referenced only by key-generation paths the driver never
// calls), which report an error.  The ChaCha PRNG is the reference's own code
// (prng/single_thread_chacha_prng.cc, prng/chacha_prng_util.cc) over the
// ChaCha20 stand-in of openssl_standin.cc.
#include <string>

#include "absl/status/status.h"
#include "absl/status/statusor.h"

namespace rlwe {
namespace internal {
absl::StatusOr<std::string> HkdfPrngGenerateKey() {
  return absl::UnimplementedError("PRNG seeding is not built into the oracle");
}
}  // namespace internal
}  // namespace rlwe

// Scalar restatement of the Highway batch kernels the lazy RNS polynomial
// links against (rns/rns_polynomial_hwy.h:31-85): raw products of Montgomery
// representations accumulated into double-width integers.
#include <memory>

#include "shell_encryption/montgomery.h"
#include "shell_encryption/prng/single_thread_chacha_prng.h"
#include "shell_encryption/prng/single_thread_hkdf_prng.h"
#include "shell_encryption/rns/rns_polynomial_hwy.h"

namespace rlwe {

absl::StatusOr<std::unique_ptr<SingleThreadHkdfPrng>> SingleThreadHkdfPrng::Create(
    absl::string_view) {
  return absl::UnimplementedError("PRNG seeding is not built into the oracle");
}

namespace internal {

template <typename Integer>
void BatchFusedMulAddMontgomeryRep(
    absl::Span<const MontgomeryInt<Integer>> a,
    absl::Span<const MontgomeryInt<Integer>> b,
    hwy::AlignedVector<typename BigInt<Integer>::value_type>& output) {
  using Big = typename BigInt<Integer>::value_type;
  for (size_t i = 0; i < a.size(); ++i)
    output[i] += static_cast<Big>(a[i].GetMontgomeryRepresentation()) *
                 b[i].GetMontgomeryRepresentation();
}

template <typename Integer>
void BatchFusedMulSumAddMontgomeryRep(
    absl::Span<const MontgomeryInt<Integer>> a,
    absl::Span<const MontgomeryInt<Integer>> b,
    absl::Span<const MontgomeryInt<Integer>> c,
    hwy::AlignedVector<typename BigInt<Integer>::value_type>& output) {
  using Big = typename BigInt<Integer>::value_type;
  for (size_t i = 0; i < a.size(); ++i)
    output[i] += (static_cast<Big>(a[i].GetMontgomeryRepresentation()) +
                  b[i].GetMontgomeryRepresentation()) *
                 c[i].GetMontgomeryRepresentation();
}

template <typename Integer>
void BatchFusedMulDifferenceAddMontgomeryRep(
    absl::Span<const MontgomeryInt<Integer>> a,
    absl::Span<const MontgomeryInt<Integer>> b,
    absl::Span<const MontgomeryInt<Integer>> c, Integer q,
    hwy::AlignedVector<typename BigInt<Integer>::value_type>& output) {
  using Big = typename BigInt<Integer>::value_type;
  for (size_t i = 0; i < a.size(); ++i)
    output[i] += (static_cast<Big>(a[i].GetMontgomeryRepresentation()) + q -
                  b[i].GetMontgomeryRepresentation()) *
                 c[i].GetMontgomeryRepresentation();
}

#define SHG_INST(T)                                                            \
  template void BatchFusedMulAddMontgomeryRep<T>(                              \
      absl::Span<const MontgomeryInt<T>>, absl::Span<const MontgomeryInt<T>>,  \
      hwy::AlignedVector<typename BigInt<T>::value_type>&);                    \
  template void BatchFusedMulSumAddMontgomeryRep<T>(                           \
      absl::Span<const MontgomeryInt<T>>, absl::Span<const MontgomeryInt<T>>,  \
      absl::Span<const MontgomeryInt<T>>,                                      \
      hwy::AlignedVector<typename BigInt<T>::value_type>&);                    \
  template void BatchFusedMulDifferenceAddMontgomeryRep<T>(                    \
      absl::Span<const MontgomeryInt<T>>, absl::Span<const MontgomeryInt<T>>,  \
      absl::Span<const MontgomeryInt<T>>, T,                                   \
      hwy::AlignedVector<typename BigInt<T>::value_type>&);
SHG_INST(Uint32)
SHG_INST(Uint64)
#undef SHG_INST

}  // namespace internal
}  // namespace rlwe
