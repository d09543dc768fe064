// The reference-side binding of the GPU path, compiled against SHELL's own
// headers (google/shell-encryption) and linked with the reference's compiled
// sources (oracle/_ref/libshellref.so, built from the reference in place by
// oracle/ref/Makefile) and libshellgpu.so.  It is the code a SHELL maintainer
// adds: real rlwe::RnsContext / RnsGadget / RnsRelinKey / RnsBgvCiphertext
// objects are handed to the C ABI (Coeffs() limbs as device buffers), and the
// GPU's RnsBgvCiphertext::operator* + RnsRelinKey::ApplyTo result is compared
// with SHELL's own.  Keys are built from components (key data, not key
// generation), which needs RnsRelinKey's private constructor, so the SHELL
// headers are included with member access opened for this file only.
//
// Without a CUDA device the reference half still runs and the C ABI must
// refuse the context cleanly; the test then prints "NO GPU" and exits 0.
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "absl/status/status.h"
#include "absl/status/statusor.h"

#define private public
#define protected public
#include "shell_encryption/montgomery.h"
#include "shell_encryption/rns/rns_bgv_ciphertext.h"
#include "shell_encryption/rns/rns_context.h"
#include "shell_encryption/rns/rns_error_params.h"
#include "shell_encryption/rns/rns_gadget.h"
#include "shell_encryption/rns/rns_polynomial.h"
#include "shell_encryption/rns/rns_relinearization_key.h"
#undef private
#undef protected

#include "shell_gpu.h"
#include "shell_gpu_runtime.h"

using M = rlwe::MontgomeryInt<uint64_t>;

namespace {

// --- the binding (what the integration guide shows) ------------------------

// One device context per rlwe::RnsContext: same log_n, moduli and t.
shg_context* MakeGpuContext(const rlwe::RnsContext<M>& ctx) {
  std::vector<uint64_t> qs;
  for (auto* m : ctx.MainPrimeModuli()) qs.push_back(m->Modulus());
  shg_context* g = nullptr;
  if (shg_context_create(ctx.LogN(), qs.data(), (int)qs.size(), ctx.PlaintextModulus(), &g))
    throw std::runtime_error(shg_last_error());
  return g;
}

// Appends an RnsPolynomial's limbs (Montgomery representations) to `out`.
void AppendCoeffs(const rlwe::RnsPolynomial<M>& p, std::vector<uint64_t>& out) {
  for (const auto& limb : p.Coeffs())
    for (const auto& x : limb) out.push_back(x.GetMontgomeryRepresentation());
}

// RnsRelinKey -> device key: GetKeyB() / GetKeyA() flattened [k][L][n].
shg_key* UploadRelinKey(shg_context* g, const rlwe::RnsRelinKey<M>& key,
                        const std::vector<int>& log_bs) {
  std::vector<uint64_t> b, a;
  for (const auto& p : key.GetKeyB()) AppendCoeffs(p, b);
  for (const auto& p : key.GetKeyA()) AppendCoeffs(p, a);
  shg_key* k = nullptr;
  if (shg_key_create(g, (int)log_bs.size(), log_bs.data(), /*power=*/1, b.data(), a.data(), &k))
    throw std::runtime_error(shg_last_error());
  return k;
}

// Ciphertexts -> one device buffer [count][2][L][n].
void* UploadCiphertexts(const std::vector<rlwe::RnsBgvCiphertext<M>>& cts) {
  std::vector<uint64_t> h;
  for (const auto& ct : cts)
    for (int c = 0; c < 2; ++c) AppendCoeffs(ct.Component(c).value(), h);
  void* d = nullptr;
  if (shg_device_alloc(h.size() * sizeof(uint64_t), &d) ||
      shg_memcpy_h2d(d, h.data(), h.size() * sizeof(uint64_t), nullptr))
    throw std::runtime_error(shg_last_error());
  return d;
}

// --- the test ----------------------------------------------------------------

uint64_t g_state = 0x9e3779b97f4a7c15ull;
uint64_t Next() {
  g_state ^= g_state << 13;
  g_state ^= g_state >> 7;
  g_state ^= g_state << 17;
  return g_state;
}

rlwe::RnsPolynomial<M> RandomNtt(int log_n,
                                 absl::Span<const rlwe::PrimeModulus<M>* const> moduli) {
  std::vector<std::vector<M>> limbs;
  for (auto* m : moduli) {
    std::vector<M> v;
    for (int i = 0; i < (1 << log_n); ++i) v.push_back(M(Next() % m->Modulus()));
    limbs.push_back(std::move(v));
  }
  return rlwe::RnsPolynomial<M>::Create(std::move(limbs), /*is_ntt=*/true).value();
}

}  // namespace

int main() {
  const int log_n = 10;
  const std::vector<uint64_t> qs = {35184371138561ull, 35184370941953ull, 35184370352129ull};
  const std::vector<int> log_bs = {20, 20, 20};
  const int L = (int)qs.size(), count = 2;
  auto ctx = rlwe::RnsContext<M>::Create(log_n, qs, {}, 65537).value();
  auto moduli = ctx.MainPrimeModuli();
  auto gadget =
      rlwe::RnsGadget<M>::Create(log_n, std::vector<size_t>(log_bs.begin(), log_bs.end()),
                                 ctx.MainPrimeModulusComplements(L - 1).value(),
                                 ctx.MainPrimeModulusCrtFactors(L - 1).value(), moduli)
          .value();
  std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
  for (int j = 0; j < gadget.Dimension(); ++j) {
    kbs.push_back(RandomNtt(log_n, moduli));
    kas.push_back(RandomNtt(log_n, moduli));
  }
  rlwe::RnsRelinKey<M> key(kas, kbs, &gadget, /*degree=*/2, moduli, "", rlwe::PRNG_TYPE_HKDF);
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, 16, 3.19).value();
  std::vector<rlwe::RnsBgvCiphertext<M>> xs, ys, want;
  for (int i = 0; i < count; ++i) {
    xs.emplace_back(std::vector<rlwe::RnsPolynomial<M>>{RandomNtt(log_n, moduli),
                                                        RandomNtt(log_n, moduli)},
                    moduli, 1, 1.0, &ep);
    ys.emplace_back(std::vector<rlwe::RnsPolynomial<M>>{RandomNtt(log_n, moduli),
                                                        RandomNtt(log_n, moduli)},
                    moduli, 1, 1.0, &ep);
    auto prod = xs[i] * ys[i];
    want.push_back(key.ApplyTo(prod.value()).value());
  }
  std::printf("reference: %d ct-mult+relin at n=2^%d, %d limbs\n", count, log_n, L);

  int devices = 0;
  if (shg_device_count(&devices) != SHG_OK || devices == 0) {
    shg_context* g = nullptr;
    const int rc = shg_context_create(log_n, qs.data(), L, 65537, &g);
    if (rc == SHG_OK) {
      std::printf("FAIL: context created without a device\n");
      return 1;
    }
    std::printf("NO GPU: shg_context_create -> %d (%s)\n", rc, shg_last_error());
    return 0;
  }
  shg_context* g = MakeGpuContext(ctx);
  shg_key* k = UploadRelinKey(g, key, log_bs);
  void* da = UploadCiphertexts(xs);
  void* db = UploadCiphertexts(ys);
  const size_t elems = (size_t)count * 2 * L << log_n;
  void* dout = nullptr;
  if (shg_device_alloc(elems * sizeof(uint64_t), &dout) ||
      shg_bgv_mul_relin(g, k, (uint64_t*)dout, (const uint64_t*)da, (const uint64_t*)db, count,
                        nullptr)) {
    std::printf("FAIL: %s\n", shg_last_error());
    return 1;
  }
  std::vector<uint64_t> got(elems), exp;
  shg_memcpy_d2h(got.data(), dout, elems * sizeof(uint64_t), nullptr);
  shg_stream_synchronize(nullptr);
  for (const auto& ct : want)
    for (int c = 0; c < 2; ++c) AppendCoeffs(ct.Component(c).value(), exp);
  shg_device_free(da);
  shg_device_free(db);
  shg_device_free(dout);
  shg_key_destroy(k);
  shg_context_destroy(g);
  if (got != exp) {
    std::printf("FAIL: GPU result differs from SHELL's\n");
    return 1;
  }
  std::printf("ALL OK: GPU ct-mult+relin equals SHELL's RnsBgvCiphertext::operator* + "
              "RnsRelinKey::ApplyTo\n");
  return 0;
}
