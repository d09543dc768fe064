// Test infrastructure: a C interface over google/shell-encryption's own
// hot-path classes, compiled in place from the reference sources (see
// oracle/ref/Makefile).  It lets the golden-vector generator run the real
// reference on seeded inputs; the product never links it.
//
// Keys are built from given components (key data, not key generation), which
// needs the private constructors of RnsRelinKey / RelinearizationKey /
// GaloisKey; the reference headers are therefore included with class
// member access opened up for this translation unit only.

// Standard headers first, with normal access control.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <optional>
#include <random>
#include <sstream>
#include <string>
#include <string_view>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "absl/numeric/int128.h"
#include "absl/status/status.h"
#include "absl/status/statusor.h"
#include "absl/strings/str_cat.h"
#include "absl/types/span.h"

#define private public
#define protected public
#include "shell_encryption/dft_transformations.h"
#include "shell_encryption/gadget.h"
#include "shell_encryption/galois_key.h"
#include "shell_encryption/montgomery.h"
#include "shell_encryption/ntt_parameters.h"
#include "shell_encryption/oblivious_expand.h"
#include "shell_encryption/polynomial.h"
#include "shell_encryption/relinearization_key.h"
#include "shell_encryption/rns/rns_bfv_ciphertext.h"
#include "shell_encryption/rns/rns_bgv_ciphertext.h"
#include "shell_encryption/rns/rns_context.h"
#include "shell_encryption/rns/rns_error_params.h"
#include "shell_encryption/rns/rns_gadget.h"
#include "shell_encryption/rns/rns_galois_key.h"
#include "shell_encryption/rns/rns_polynomial.h"
#include "shell_encryption/rns/rns_relinearization_key.h"
#include "shell_encryption/rns/rns_secret_key.h"
#include "shell_encryption/rns/error_distribution.h"
#include "shell_encryption/prng/single_thread_chacha_prng.h"
#include "shell_encryption/symmetric_encryption.h"
#undef private
#undef protected

using M = rlwe::MontgomeryInt<uint64_t>;
using Params = M::Params;

namespace {

thread_local std::string g_err;

int fail(const absl::Status& s) {
  g_err = std::string(s.message());
  return s.code() == absl::StatusCode::kOk ? 0 : (int)s.code();
}

struct Prime {
  std::unique_ptr<const Params> params;
  rlwe::NttParameters<M> ntt;
};

int make_prime(uint64_t q, int log_n, Prime* p) {
  auto params = Params::Create(q);
  if (!params.ok()) return fail(params.status());
  p->params = std::move(*params);
  auto ntt = rlwe::InitializeNttParameters<M>(log_n, p->params.get());
  if (!ntt.ok()) return fail(ntt.status());
  p->ntt = std::move(*ntt);
  return 0;
}

std::vector<M> to_vec(const uint64_t* a, size_t n) {
  std::vector<M> v;
  v.reserve(n);
  for (size_t i = 0; i < n; ++i) v.push_back(M(a[i]));
  return v;
}

void from_vec(const std::vector<M>& v, uint64_t* out) {
  for (size_t i = 0; i < v.size(); ++i) out[i] = v[i].GetMontgomeryRepresentation();
}

using Ctx = rlwe::RnsContext<M>;

std::unique_ptr<Ctx> make_ctx(int log_n, const uint64_t* qs, int L, uint64_t t,
                              int* st) {
  auto ctx = Ctx::Create(log_n, std::vector<uint64_t>(qs, qs + L), {}, t);
  if (!ctx.ok()) {
    *st = fail(ctx.status());
    return nullptr;
  }
  *st = 0;
  return std::make_unique<Ctx>(std::move(*ctx));
}

std::unique_ptr<Ctx> make_ctx_aux(int log_n, const uint64_t* qs, int L, const uint64_t* ps,
                                  int K, uint64_t t, int* st) {
  auto ctx = Ctx::Create(log_n, std::vector<uint64_t>(qs, qs + L),
                         std::vector<uint64_t>(ps, ps + K), t);
  if (!ctx.ok()) {
    *st = fail(ctx.status());
    return nullptr;
  }
  *st = 0;
  return std::make_unique<Ctx>(std::move(*ctx));
}

rlwe::RnsPolynomial<M> make_poly(const uint64_t* data, int L, int n, bool is_ntt) {
  std::vector<std::vector<M>> cv;
  for (int l = 0; l < L; ++l) cv.push_back(to_vec(data + (size_t)l * n, n));
  return rlwe::RnsPolynomial<M>(rlwe::RnsPolynomial<M>::Create(std::move(cv), is_ntt).value());
}

void store_poly(const rlwe::RnsPolynomial<M>& p, uint64_t* out) {
  const auto& cv = p.Coeffs();
  size_t n = cv[0].size();
  for (size_t l = 0; l < cv.size(); ++l) from_vec(cv[l], out + l * n);
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

// NttParameters tables (Montgomery reps) and constants of one prime.
int ref_prime_tables(uint64_t q, int log_n, uint64_t* fwd, uint64_t* inv,
                     uint64_t* n_inv) {
  Prime p;
  int st = make_prime(q, log_n, &p);
  if (st) return st;
  from_vec(p.ntt.psis_bitrev, fwd);
  from_vec(p.ntt.psis_inv_bitrev, inv);
  *n_inv = p.ntt.n_inv_ptr->GetMontgomeryRepresentation();
  return 0;
}

// ForwardNumberTheoreticTransform / InverseNumberTheoreticTransform on
// `count` vectors of n Montgomery residues, in place.
int ref_ntt(uint64_t q, int log_n, uint64_t* data, int count, int inverse) {
  Prime p;
  int st = make_prime(q, log_n, &p);
  if (st) return st;
  const int n = 1 << log_n;
  for (int c = 0; c < count; ++c) {
    std::vector<M> v = to_vec(data + (size_t)c * n, n);
    absl::Status s = inverse
                         ? rlwe::InverseNumberTheoreticTransform(v, p.ntt, *p.params)
                         : rlwe::ForwardNumberTheoreticTransform(v, p.ntt, *p.params);
    if (!s.ok()) return fail(s);
    from_vec(v, data + (size_t)c * n);
  }
  return 0;
}

// RnsPolynomial::Substitute.
int ref_rns_substitute(int log_n, const uint64_t* qs, int L, int power,
                       const uint64_t* in, uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  auto p = make_poly(in, L, 1 << log_n, true);
  auto r = p.Substitute(power, ctx->MainPrimeModuli());
  if (!r.ok()) return fail(r.status());
  store_poly(*r, out);
  return 0;
}

// RnsPolynomial::ModReduceLsb with ql_inv from MainPrimeModulusInverseResidues.
int ref_rns_modreduce_lsb(int log_n, const uint64_t* qs, int L, uint64_t t,
                          int is_ntt, const uint64_t* in, uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, t, &st);
  if (!ctx) return st;
  auto p = make_poly(in, L, 1 << log_n, is_ntt != 0);
  auto ql_inv = ctx->MainPrimeModulusInverseResidues()[L - 1].Prefix(L - 1);
  absl::Status s = p.ModReduceLsb(t, ql_inv, ctx->MainPrimeModuli());
  if (!s.ok()) return fail(s);
  store_poly(p, out);
  return 0;
}

// RnsBgvCiphertext::operator* followed by RnsRelinKey::ApplyTo, on `count`
// pairs a, b [count][2][L][n] with key components [k][L][n]; also returns the
// degree-2 product in prod [count][3][L][n] when prod is not null.
int ref_bgv_mul_relin(int log_n, const uint64_t* qs, int L, uint64_t t,
                      const int* log_bs, const uint64_t* key_b,
                      const uint64_t* key_a, const uint64_t* a,
                      const uint64_t* b, int count, uint64_t* prod,
                      uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, t, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  auto q_hats = ctx->MainPrimeModulusComplements(L - 1).value();
  auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(L - 1).value();
  auto gadget = rlwe::RnsGadget<M>::Create(
      log_n, std::vector<size_t>(log_bs, log_bs + L), q_hats, q_hat_invs, moduli);
  if (!gadget.ok()) return fail(gadget.status());
  const int k = gadget->Dimension();
  std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
  for (int j = 0; j < k; ++j) {
    kbs.push_back(make_poly(key_b + (size_t)j * P, L, n, true));
    kas.push_back(make_poly(key_a + (size_t)j * P, L, n, true));
  }
  rlwe::RnsRelinKey<M> key(std::move(kas), std::move(kbs), &*gadget,
                           /*degree=*/2, moduli, "", rlwe::PRNG_TYPE_HKDF);
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, 16, 3.19);
  if (!ep.ok()) return fail(ep.status());
  for (int c = 0; c < count; ++c) {
    std::vector<rlwe::RnsPolynomial<M>> ca, cb;
    for (int i = 0; i < 2; ++i) {
      ca.push_back(make_poly(a + ((size_t)c * 2 + i) * P, L, n, true));
      cb.push_back(make_poly(b + ((size_t)c * 2 + i) * P, L, n, true));
    }
    rlwe::RnsBgvCiphertext<M> x(std::move(ca), moduli, 1, 1.0, &*ep);
    rlwe::RnsBgvCiphertext<M> y(std::move(cb), moduli, 1, 1.0, &*ep);
    auto xy = x * y;
    if (!xy.ok()) return fail(xy.status());
    if (prod)
      for (int i = 0; i < 3; ++i)
        store_poly(xy->Component(i).value(), prod + ((size_t)c * 3 + i) * P);
    auto r = key.ApplyTo(*xy);
    if (!r.ok()) return fail(r.status());
    for (int i = 0; i < 2; ++i)
      store_poly(r->Component(i).value(), out + ((size_t)c * 2 + i) * P);
  }
  return 0;
}

// RnsBgvCiphertext::Substitute(power) then RnsGaloisKey::ApplyTo, with a key
// built by RnsGaloisKey::CreateFromKeyComponents.
int ref_bgv_rotate(int log_n, const uint64_t* qs, int L, const int* log_bs,
                   int power, const uint64_t* key_b, const uint64_t* key_a,
                   const uint64_t* ct, int count, uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  auto q_hats = ctx->MainPrimeModulusComplements(L - 1).value();
  auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(L - 1).value();
  auto gadget = rlwe::RnsGadget<M>::Create(
      log_n, std::vector<size_t>(log_bs, log_bs + L), q_hats, q_hat_invs, moduli);
  if (!gadget.ok()) return fail(gadget.status());
  const int k = gadget->Dimension();
  std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
  for (int j = 0; j < k; ++j) {
    kbs.push_back(make_poly(key_b + (size_t)j * P, L, n, true));
    kas.push_back(make_poly(key_a + (size_t)j * P, L, n, true));
  }
  auto key = rlwe::RnsGaloisKey<M>::CreateFromKeyComponents(
      std::move(kas), std::move(kbs), power, &*gadget, moduli, "",
      rlwe::PRNG_TYPE_HKDF);
  if (!key.ok()) return fail(key.status());
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, 16, 3.19);
  if (!ep.ok()) return fail(ep.status());
  for (int c = 0; c < count; ++c) {
    std::vector<rlwe::RnsPolynomial<M>> comps;
    for (int i = 0; i < 2; ++i)
      comps.push_back(make_poly(ct + ((size_t)c * 2 + i) * P, L, n, true));
    rlwe::RnsBgvCiphertext<M> x(std::move(comps), moduli, 1, 1.0, &*ep);
    auto sub = x.Substitute(power);
    if (!sub.ok()) return fail(sub.status());
    auto r = key->ApplyTo(*sub);
    if (!r.ok()) return fail(r.status());
    for (int i = 0; i < 2; ++i)
      store_poly(r->Component(i).value(), out + ((size_t)c * 2 + i) * P);
  }
  return 0;
}

// GaloisKeysObliviousExpander::ObliviousExpand of `count` ciphertexts [2][n]
// with keys[levels][2][dim][n] (row 0 = the "b" row, row 1 = the random row)
// for the substitution powers n/2^i + 1; out [count][2^levels][2][n].
int ref_oblivious_expand(uint64_t q, int log_n, int log_t, int levels, int log_b,
                         const uint64_t* keys, const uint64_t* ct, int count,
                         uint64_t* out) {
  Prime p;
  int st = make_prime(q, log_n, &p);
  if (st) return st;
  const int n = 1 << log_n;
  const int dim = rlwe::GadgetSize<M>(log_b, p.params.get());
  auto ep = rlwe::ErrorParams<M>::Create(log_t, 8, p.params.get(), &p.ntt);
  if (!ep.ok()) return fail(ep.status());
  auto dm = M::ImportInt((uint64_t)1 << log_b, p.params.get()).value();
  std::vector<rlwe::GaloisKey<M>> gks;
  for (int j = 0; j < levels; ++j) {
    std::vector<std::vector<rlwe::Polynomial<M>>> matrix(2);
    for (int row = 0; row < 2; ++row)
      for (int d = 0; d < dim; ++d)
        matrix[row].push_back(rlwe::Polynomial<M>(to_vec(
            keys + (((size_t)j * 2 + row) * dim + d) * n, n)));
    typename rlwe::RelinearizationKey<M>::RelinearizationKeyPart part(
        std::move(matrix), (uint64_t)log_b);
    rlwe::RelinearizationKey<M> rk((uint64_t)log_b, dm, p.params.get(), &p.ntt);
    rk.dimension_ = dim;
    rk.num_parts_ = 2;
    rk.substitution_power_ = (n >> j) + 1;
    rk.relinearization_key_.push_back(std::move(part));
    gks.push_back(rlwe::GaloisKey<M>(std::move(rk)));
  }
  auto exp = rlwe::GaloisKeysObliviousExpander<M>::Create(std::move(gks), log_t,
                                                          p.params.get(), &p.ntt);
  if (!exp.ok()) return fail(exp.status());
  for (int c = 0; c < count; ++c) {
    std::vector<rlwe::Polynomial<M>> comps;
    for (int i = 0; i < 2; ++i)
      comps.push_back(rlwe::Polynomial<M>(to_vec(ct + ((size_t)c * 2 + i) * n, n)));
    std::vector<rlwe::SymmetricRlweCiphertext<M>> in;
    in.emplace_back(std::move(comps), 1, 1.0, p.params.get(), &*ep);
    auto r = (*exp)->ObliviousExpand(std::move(in), levels, 1 << levels);
    if (!r.ok()) return fail(r.status());
    for (int i = 0; i < (1 << levels); ++i)
      for (int comp = 0; comp < 2; ++comp)
        from_vec((*r)[i].Component(comp).value().Coeffs(),
                 out + (((size_t)c << levels) + i) * 2 * n + (size_t)comp * n);
  }
  return 0;
}

// RnsGaloisKey::PrecomputeRandomPad then ApplyToWithRandomPad on `count`
// ciphertexts at the key's power with their c1 digits given: out
// [count][2][L][n] = the key-switched ciphertexts.
int ref_galois_random_pad(int log_n, const uint64_t* qs, int L, const int* log_bs,
                          int power, const uint64_t* key_b, const uint64_t* key_a,
                          const uint64_t* ct, const uint64_t* pad_digits, int count,
                          uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  auto q_hats = ctx->MainPrimeModulusComplements(L - 1).value();
  auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(L - 1).value();
  auto gadget = rlwe::RnsGadget<M>::Create(
      log_n, std::vector<size_t>(log_bs, log_bs + L), q_hats, q_hat_invs, moduli);
  if (!gadget.ok()) return fail(gadget.status());
  const int k = gadget->Dimension();
  std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
  for (int j = 0; j < k; ++j) {
    kbs.push_back(make_poly(key_b + (size_t)j * P, L, n, true));
    kas.push_back(make_poly(key_a + (size_t)j * P, L, n, true));
  }
  auto key = rlwe::RnsGaloisKey<M>::CreateFromKeyComponents(
      std::move(kas), std::move(kbs), power, &*gadget, moduli, "",
      rlwe::PRNG_TYPE_HKDF);
  if (!key.ok()) return fail(key.status());
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, 16, 3.19);
  if (!ep.ok()) return fail(ep.status());
  for (int c = 0; c < count; ++c) {
    std::vector<rlwe::RnsPolynomial<M>> comps;
    for (int i = 0; i < 2; ++i)
      comps.push_back(make_poly(ct + ((size_t)c * 2 + i) * P, L, n, true));
    rlwe::RnsBgvCiphertext<M> x(std::move(comps), moduli, power, 1.0, &*ep);
    std::vector<rlwe::RnsPolynomial<M>> digits;
    for (int j = 0; j < k; ++j)
      digits.push_back(make_poly(pad_digits + ((size_t)c * k + j) * P, L, n, true));
    auto pad = key->PrecomputeRandomPad(digits);
    if (!pad.ok()) return fail(pad.status());
    auto r = key->ApplyToWithRandomPad(x, digits, *pad);
    if (!r.ok()) return fail(r.status());
    for (int i = 0; i < 2; ++i)
      store_poly(r->Component(i).value(), out + ((size_t)c * 2 + i) * P);
  }
  return 0;
}

// The first `count` bytes (Rand8) of SingleThreadChaChaPrng::Create(seed).
int ref_prng_bytes(const uint8_t* seed, int count, uint8_t* out) {
  auto prng = rlwe::SingleThreadChaChaPrng::Create(
      std::string(reinterpret_cast<const char*>(seed), 32));
  if (!prng.ok()) return fail(prng.status());
  for (int i = 0; i < count; ++i) {
    auto b = (*prng)->Rand8();
    if (!b.ok()) return fail(b.status());
    out[i] = *b;
  }
  return 0;
}

// RnsPolynomial::SampleUniform then SampleError (rns/error_distribution.h)
// from one ChaCha PRNG of `seed`, as EncryptPolynomialBgv draws them;
// a_out, e_out [L][n] NTT form.
int ref_sample_uniform_error(int log_n, const uint64_t* qs, int L, int variance,
                             const uint8_t* seed, uint64_t* a_out, uint64_t* e_out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  auto moduli = ctx->MainPrimeModuli();
  auto prng = rlwe::SingleThreadChaChaPrng::Create(
      std::string(reinterpret_cast<const char*>(seed), 32));
  if (!prng.ok()) return fail(prng.status());
  auto a = rlwe::RnsPolynomial<M>::SampleUniform(log_n, prng->get(), moduli);
  if (!a.ok()) return fail(a.status());
  auto e = rlwe::SampleError<M>(log_n, variance, moduli, prng->get());
  if (!e.ok()) return fail(e.status());
  store_poly(*a, a_out);
  store_poly(*e, e_out);
  return 0;
}

struct PlainModulus {
  uint64_t t;
  uint64_t PlaintextModulus() const { return t; }
};

// RnsRlweSecretKey::EncryptPolynomialBgv (rns/rns_secret_key.h:188-231) of
// `count` NTT-form plaintexts, ciphertext c drawing its randomness from the
// ChaCha PRNG of seeds + 32 c: out [count][2][L][n].
int ref_encrypt_bgv(int log_n, const uint64_t* qs, int L, uint64_t t, int variance,
                    const uint64_t* key, const uint64_t* plaintexts, const uint8_t* seeds,
                    int count, uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, t, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  rlwe::RnsRlweSecretKey<M> sk(make_poly(key, L, n, true), moduli, variance);
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, 16, 3.19);
  if (!ep.ok()) return fail(ep.status());
  PlainModulus enc{t};
  for (int c = 0; c < count; ++c) {
    auto prng = rlwe::SingleThreadChaChaPrng::Create(
        std::string(reinterpret_cast<const char*>(seeds + 32 * c), 32));
    if (!prng.ok()) return fail(prng.status());
    auto ct = sk.EncryptPolynomialBgv(make_poly(plaintexts + (size_t)c * P, L, n, true), &enc,
                                      &*ep, prng->get());
    if (!ct.ok()) return fail(ct.status());
    for (int i = 0; i < 2; ++i)
      store_poly(ct->Component(i).value(), out + ((size_t)c * 2 + i) * P);
  }
  return 0;
}

// MontgomeryInt::SerializeVector of `count` Montgomery residues mod q into
// `out` (capacity `cap` bytes); *len receives the byte count.
int ref_serialize_vector(uint64_t q, const uint64_t* data, int count, uint8_t* out,
                         size_t cap, size_t* len) {
  auto params = M::Params::Create(q);
  if (!params.ok()) return fail(params.status());
  auto s = M::SerializeVector(to_vec(data, count), params->get());
  if (!s.ok()) return fail(s.status());
  if (s->size() > cap) {
    g_err = "output too small";
    return 3;
  }
  std::memcpy(out, s->data(), s->size());
  *len = s->size();
  return 0;
}

// MontgomeryInt::DeserializeVector of `count` values.
int ref_deserialize_vector(uint64_t q, const uint8_t* in, size_t len, int count,
                           uint64_t* out) {
  auto params = M::Params::Create(q);
  if (!params.ok()) return fail(params.status());
  auto v = M::DeserializeVector(
      count, std::string(reinterpret_cast<const char*>(in), len), params->get());
  if (!v.ok()) return fail(v.status());
  from_vec(*v, out);
  return 0;
}

// RNS basis conversions of one polynomial with the context's own tables
// (rns/rns_context.h:142-240): mode 0 SwitchRnsBasis main (q_0..q_level) ->
// aux; 1 SwitchRnsBasis aux -> main (every main prime); 2
// ScaleAndSwitchRnsBasis main (level) -> aux; 3 ApproxSwitchRnsBasis aux ->
// main (q_0..q_level); 4 ApproxSwitchRnsBasis main (level) -> aux.
int ref_switch_basis(int log_n, const uint64_t* qs, int L, const uint64_t* ps, int K,
                     int level, int mode, int is_ntt, int balanced, const uint64_t* in,
                     uint64_t* out) {
  int st;
  auto ctx = make_ctx_aux(log_n, qs, L, ps, K, 65537, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  auto main = ctx->MainPrimeModuli();
  main.resize(mode == 1 ? L : level + 1);
  auto aux = ctx->AuxPrimeModuli();
  const bool from_main = mode == 0 || mode == 2 || mode == 4;
  auto a = make_poly(in, from_main ? (int)main.size() : K, n, is_ntt != 0);
  absl::StatusOr<rlwe::RnsPolynomial<M>> r = absl::InternalError("mode");
  if (mode == 0) {
    auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(level).value();
    auto q_hat_mod_ps = ctx->MainPrimeModulusComplementResidues(level).value();
    auto q_mod_ps = ctx->MainLeveledModulusAuxResidues(level).value();
    r = a.SwitchRnsBasis(main, aux, q_hat_invs, q_hat_mod_ps, q_mod_ps.RnsRep());
  } else if (mode == 1) {
    r = a.SwitchRnsBasis(aux, main, ctx->AuxPrimeModulusCrtFactors(),
                         ctx->AuxPrimeModulusComplementResidues(), ctx->AuxModulusResidues());
  } else if (mode == 2) {
    auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(level).value();
    r = a.ScaleAndSwitchRnsBasis(main, aux, q_hat_invs,
                                 ctx->MainPrimeModulusInverseAuxResidues(),
                                 ctx->AuxModulusResidues());
  } else if (mode == 3) {
    r = a.ApproxSwitchRnsBasis(aux, main, ctx->AuxPrimeModulusCrtFactors(),
                               ctx->AuxPrimeModulusComplementResidues(), balanced != 0);
  } else if (mode == 4) {
    auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(level).value();
    auto q_hat_mod_ps = ctx->MainPrimeModulusComplementResidues(level).value();
    r = a.ApproxSwitchRnsBasis(main, aux, q_hat_invs, q_hat_mod_ps, balanced != 0);
  }
  if (!r.ok()) return fail(r.status());
  store_poly(*r, out);
  return 0;
}

// RnsPolynomial::ModReduceMsb with MainPrimeModulusInverseResidues()[L-1].
int ref_modreduce_msb(int log_n, const uint64_t* qs, int L, int is_ntt, const uint64_t* in,
                      uint64_t* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  auto moduli = ctx->MainPrimeModuli();
  auto a = make_poly(in, L, 1 << log_n, is_ntt != 0);
  auto ql_inv = ctx->MainPrimeModulusInverseResidues()[L - 1].Prefix(L - 1);
  auto s2 = a.ModReduceMsb(ql_inv, moduli);
  if (!s2.ok()) return fail(s2);
  store_poly(a, out);
  return 0;
}

// ScaleAndReduceRnsBasisInPlace (mode 0), ApproxModReduceLsb (1) and
// ApproxModReduceMsb (2) of (main mod Q, aux mod P) with the context's tables.
int ref_scale_reduce(int log_n, const uint64_t* qs, int L, const uint64_t* ps, int K,
                     uint64_t t, int mode, int is_ntt_main, const uint64_t* main_in,
                     int is_ntt_aux, const uint64_t* aux_in, uint64_t* out) {
  int st;
  auto ctx = make_ctx_aux(log_n, qs, L, ps, K, t, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  auto main = ctx->MainPrimeModuli();
  auto aux = ctx->AuxPrimeModuli();
  auto a = make_poly(main_in, L, n, is_ntt_main != 0);
  auto b = make_poly(aux_in, K, n, is_ntt_aux != 0);
  absl::Status s2;
  if (mode == 0) {
    s2 = a.ScaleAndReduceRnsBasisInPlace(
        std::move(b), t, main, aux, ctx->AuxPrimeModulusCrtFactors(),
        ctx->AuxPrimeModulusComplementResidues(), ctx->AuxModulusResidues(),
        ctx->AuxModulusInverseResidues());
  } else if (mode == 1) {
    s2 = a.ApproxModReduceLsb(std::move(b), main, aux, ctx->AuxModulusInverseResidues(),
                              ctx->AuxPrimeModulusCrtFactors(),
                              ctx->AuxPrimeModulusComplementResidues(),
                              ctx->PlaintextModulusInverseAuxResidues(),
                              ctx->AuxModulusPlaintextResidue(), t);
  } else {
    s2 = a.ApproxModReduceMsb(std::move(b), main, aux, ctx->AuxModulusInverseResidues(),
                              ctx->AuxPrimeModulusCrtFactors(),
                              ctx->AuxPrimeModulusComplementResidues());
  }
  if (!s2.ok()) return fail(s2);
  store_poly(a, out);
  return 0;
}

// RnsBfvCiphertext::operator* (Mul) of `count` pairs a, b [count][2][L][n]
// -> out [count][3][L][n]; op 1: AbsorbInPlace of a [count][len][L][n]
// with the plaintext b [L][n] -> out [count][len][L][n].
int ref_bfv(int log_n, const uint64_t* qs, int L, const uint64_t* ps, int K, uint64_t t,
            int op, int len, const uint64_t* a, const uint64_t* b, int count,
            uint64_t* out) {
  int st;
  auto ctx = make_ctx_aux(log_n, qs, L, ps, K, t, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, ctx->AuxPrimeModuli(), 16, 3.19);
  if (!ep.ok()) return fail(ep.status());
  for (int c = 0; c < count; ++c) {
    std::vector<rlwe::RnsPolynomial<M>> ca;
    const int la = op == 0 ? 2 : len;
    for (int i = 0; i < la; ++i) ca.push_back(make_poly(a + ((size_t)c * la + i) * P, L, n, true));
    rlwe::RnsBfvCiphertext<M> x(std::move(ca), moduli, 1, 1.0, &*ep, ctx.get());
    if (op == 0) {
      std::vector<rlwe::RnsPolynomial<M>> cb;
      for (int i = 0; i < 2; ++i) cb.push_back(make_poly(b + ((size_t)c * 2 + i) * P, L, n, true));
      rlwe::RnsBfvCiphertext<M> y(std::move(cb), moduli, 1, 1.0, &*ep, ctx.get());
      auto xy = x * y;
      if (!xy.ok()) return fail(xy.status());
      for (int i = 0; i < 3; ++i)
        store_poly(xy->Component(i).value(), out + ((size_t)c * 3 + i) * P);
    } else {
      auto s2 = x.AbsorbInPlace(make_poly(b, L, n, true));
      if (!s2.ok()) return fail(s2);
      for (int i = 0; i < la; ++i)
        store_poly(x.Component(i).value(), out + ((size_t)c * la + i) * P);
    }
  }
  return 0;
}

// RnsGaloisKey::Compose (rns/rns_galois_key.cc:349-406) of a key of power
// `power` with another key (same gadget) of power `power2`: composed rows
// out_b, out_a [k][L][n] and the composed power.
int ref_galois_compose(int log_n, const uint64_t* qs, int L, const int* log_bs, int power,
                       const uint64_t* key_b, const uint64_t* key_a, int power2,
                       const uint64_t* key2_b, const uint64_t* key2_a, uint64_t* out_b,
                       uint64_t* out_a, int* out_power) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  const size_t P = (size_t)L * n;
  auto moduli = ctx->MainPrimeModuli();
  auto q_hats = ctx->MainPrimeModulusComplements(L - 1).value();
  auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(L - 1).value();
  auto gadget = rlwe::RnsGadget<M>::Create(
      log_n, std::vector<size_t>(log_bs, log_bs + L), q_hats, q_hat_invs, moduli);
  if (!gadget.ok()) return fail(gadget.status());
  const int k = gadget->Dimension();
  auto make_key = [&](int pw, const uint64_t* kb, const uint64_t* ka) {
    std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
    for (int j = 0; j < k; ++j) {
      kbs.push_back(make_poly(kb + (size_t)j * P, L, n, true));
      kas.push_back(make_poly(ka + (size_t)j * P, L, n, true));
    }
    return rlwe::RnsGaloisKey<M>::CreateFromKeyComponents(
        std::move(kas), std::move(kbs), pw, &*gadget, moduli, "", rlwe::PRNG_TYPE_HKDF);
  };
  auto k1 = make_key(power, key_b, key_a);
  if (!k1.ok()) return fail(k1.status());
  auto k2 = make_key(power2, key2_b, key2_a);
  if (!k2.ok()) return fail(k2.status());
  auto c = k1->Compose(*k2);
  if (!c.ok()) return fail(c.status());
  for (int j = 0; j < k; ++j) {
    store_poly(c->key_bs_[j], out_b + (size_t)j * P);
    store_poly(c->key_as_[j], out_a + (size_t)j * P);
  }
  *out_power = c->power_;
  return 0;
}

// ObliviousExpander::ComputeNormalizer.
uint64_t ref_compute_normalizer(int k, int log_t) {
  return rlwe::ObliviousExpander<M>::ComputeNormalizer(k, log_t);
}

// The error bookkeeping of the reference's RNS ciphertexts: the constants of
// RnsErrorParams::Create(log_n, main moduli, {}, log_t, sigma)
// (rns/rns_error_params.h) and Error() after each operation of
// rns/rns_ciphertext.h, rns/rns_bgv_ciphertext.h and the key switches
// (rns/rns_relinearization_key.h:158-164, rns/rns_galois_key.h), starting
// from two degree-1 ciphertexts with errors e0 and e1 (zero data: the
// bookkeeping does not read it).  out: [0..3] B_plaintext,
// B_secretkey_encryption, B_publickey_encryption, B_scale;
// [4] BoundOnGadgetBasedKeySwitching(1, max log_b, k); [5] ct0 + ct1;
// [6] ct0 - ct1; [7] ct0 absorbing a plaintext; [8] ct0 absorbing `scalar`;
// [9] ct0 += ct1 * plaintext (FusedAbsorbAddInPlace); [10] ct0 * ct1;
// [11] the relinearized product; [12] ct0 after ModReduce;
// [13] ct0.Substitute(power); [14] that substitution Galois key-switched.
int ref_error_flow(int log_n, const uint64_t* qs, int L, const int* log_bs, int log_t,
                   double sigma, double e0, double e1, uint64_t scalar, int power,
                   double* out) {
  int st;
  auto ctx = make_ctx(log_n, qs, L, 65537, &st);
  if (!ctx) return st;
  const int n = 1 << log_n;
  auto moduli = ctx->MainPrimeModuli();
  auto ep = rlwe::RnsErrorParams<M>::Create(log_n, moduli, {}, log_t, sigma);
  if (!ep.ok()) return fail(ep.status());
  auto q_hats = ctx->MainPrimeModulusComplements(L - 1).value();
  auto q_hat_invs = ctx->MainPrimeModulusCrtFactors(L - 1).value();
  auto gadget = rlwe::RnsGadget<M>::Create(
      log_n, std::vector<size_t>(log_bs, log_bs + L), q_hats, q_hat_invs, moduli);
  if (!gadget.ok()) return fail(gadget.status());
  const int k = gadget->Dimension();
  std::vector<uint64_t> zeros((size_t)L * n, 0);
  auto zero = [&] { return make_poly(zeros.data(), L, n, true); };
  auto ct = [&](double e) {
    std::vector<rlwe::RnsPolynomial<M>> c{zero(), zero()};
    return rlwe::RnsBgvCiphertext<M>(std::move(c), moduli, 1, e, &*ep);
  };
  out[0] = ep->B_plaintext();
  out[1] = ep->B_secretkey_encryption();
  out[2] = ep->B_publickey_encryption();
  out[3] = ep->B_scale();
  out[4] = ep->BoundOnGadgetBasedKeySwitching(1, gadget->LogGadgetBase(), k);
  auto c0 = ct(e0), c1 = ct(e1);
  auto sum = c0 + c1;
  if (!sum.ok()) return fail(sum.status());
  out[5] = sum->Error();
  auto diff = c0 - c1;
  if (!diff.ok()) return fail(diff.status());
  out[6] = diff->Error();
  {
    auto x = ct(e0);
    if (absl::Status s = x.AbsorbInPlace(zero()); !s.ok()) return fail(s);
    out[7] = x.Error();
  }
  {
    auto x = ct(e0);
    if (absl::Status s = x.AbsorbInPlace(scalar); !s.ok()) return fail(s);
    out[8] = x.Error();
  }
  {
    auto x = ct(e0);
    if (absl::Status s = x.FusedAbsorbAddInPlace(c1, zero()); !s.ok()) return fail(s);
    out[9] = x.Error();
  }
  auto prod = c0 * c1;
  if (!prod.ok()) return fail(prod.status());
  out[10] = prod->Error();
  std::vector<rlwe::RnsPolynomial<M>> kas, kbs;
  for (int j = 0; j < k; ++j) {
    kbs.push_back(zero());
    kas.push_back(zero());
  }
  rlwe::RnsRelinKey<M> relin(kas, kbs, &*gadget, /*degree=*/2, moduli, "",
                             rlwe::PRNG_TYPE_HKDF);
  auto r = relin.ApplyTo(*prod);
  if (!r.ok()) return fail(r.status());
  out[11] = r->Error();
  {
    auto x = ct(e0);
    auto ql_inv = ctx->MainPrimeModulusInverseResidues()[L - 1].Prefix(L - 1);
    if (absl::Status s = x.ModReduce(65537, ql_inv); !s.ok()) return fail(s);
    out[12] = x.Error();
  }
  auto sub = c0.Substitute(power);
  if (!sub.ok()) return fail(sub.status());
  out[13] = sub->Error();
  auto gk = rlwe::RnsGaloisKey<M>::CreateFromKeyComponents(
      std::move(kas), std::move(kbs), power, &*gadget, moduli, "", rlwe::PRNG_TYPE_HKDF);
  if (!gk.ok()) return fail(gk.status());
  auto g = gk->ApplyTo(*sub);
  if (!g.ok()) return fail(g.status());
  out[14] = g->Error();
  return 0;
}

// The single-modulus symmetric flow (symmetric_encryption.h):
//  - the key: SymmetricRlweKey::Sample(log_n, variance, log_t) drawing from
//    SingleThreadChaChaPrng::Create(key_seed) (:634-649);
//  - message i (integers msgs[i][n] in [0, t)): plaintext ConvertToNtt of its
//    imported coefficients, then rlwe::Encrypt (:1006-1021) with the PRNG of
//    seeds[32 i..]; a second PRNG of the same seed replays what Encrypt draws
//    (SamplePolynomialFromPrng, then SampleFromErrorDistribution), giving the
//    injected-randomness inputs a [count][n] (NTT) and e [count][n]
//    (coefficient form) of internal::Encrypt (:940-963);
//  - pairs (i, half + i), half = count / 2: ct + ct (:111), ct * ct (:408),
//    and ct_i absorbing plaintext half + i (:214-226);
//  - Decrypt (:1138-1152) of every ciphertext, sum and product.
// Outputs (Montgomery representations, NTT form): s [n], pt [count][n],
// ct [count][2][n], sum [half][2][n], prod [half][3][n], absorb
// [half][2][n]; decryptions dec [count][n], dec_sum, dec_prod, dec_absorb
// [half][n]; err [4] = Error() of ct 0, sum 0, prod 0, absorb 0.
int ref_sym_c1(uint64_t q, int log_n, int log_t, int variance, const uint8_t* key_seed,
               const uint8_t* seeds, const uint64_t* msgs, int count, uint64_t* s_out,
               uint64_t* pt_out, uint64_t* a_out, uint64_t* e_out, uint64_t* ct_out,
               uint64_t* sum_out, uint64_t* prod_out, uint64_t* absorb_out,
               uint64_t* dec_out, uint64_t* dec_sum, uint64_t* dec_prod,
               uint64_t* dec_absorb, double* err) {
  Prime pr;
  if (int st = make_prime(q, log_n, &pr)) return st;
  const Params* params = pr.params.get();
  const size_t n = (size_t)1 << log_n;
  const int half = count / 2;
  auto seed_str = [](const uint8_t* s) {
    return std::string(reinterpret_cast<const char*>(s), 32);
  };
  auto key_prng = rlwe::SingleThreadChaChaPrng::Create(seed_str(key_seed));
  if (!key_prng.ok()) return fail(key_prng.status());
  auto key = rlwe::SymmetricRlweKey<M>::Sample(log_n, variance, log_t, params, &pr.ntt,
                                               key_prng->get());
  if (!key.ok()) return fail(key.status());
  auto ep = rlwe::ErrorParams<M>::Create(log_t, variance, params, &pr.ntt);
  if (!ep.ok()) return fail(ep.status());
  from_vec(key->Key().Coeffs(), s_out);
  std::vector<rlwe::Polynomial<M>> pts;
  std::vector<rlwe::SymmetricRlweCiphertext<M>> cts;
  for (int i = 0; i < count; ++i) {
    std::vector<M> coeffs;
    coeffs.reserve(n);
    for (size_t j = 0; j < n; ++j) {
      auto v = M::ImportInt(msgs[(size_t)i * n + j], params);
      if (!v.ok()) return fail(v.status());
      coeffs.push_back(*v);
    }
    pts.push_back(rlwe::Polynomial<M>::ConvertToNtt(std::move(coeffs), &pr.ntt, params));
    from_vec(pts.back().Coeffs(), pt_out + (size_t)i * n);
    auto replay = rlwe::SingleThreadChaChaPrng::Create(seed_str(seeds + 32 * (size_t)i));
    if (!replay.ok()) return fail(replay.status());
    auto a = rlwe::SamplePolynomialFromPrng<M>(n, replay->get(), params);
    if (!a.ok()) return fail(a.status());
    auto e = rlwe::SampleFromErrorDistribution<M>(n, variance, replay->get(), params);
    if (!e.ok()) return fail(e.status());
    from_vec(a->Coeffs(), a_out + (size_t)i * n);
    from_vec(*e, e_out + (size_t)i * n);
    auto prng = rlwe::SingleThreadChaChaPrng::Create(seed_str(seeds + 32 * (size_t)i));
    if (!prng.ok()) return fail(prng.status());
    auto ct = rlwe::Encrypt<M>(*key, pts.back(), &*ep, prng->get());
    if (!ct.ok()) return fail(ct.status());
    for (int c = 0; c < 2; ++c)
      from_vec(ct->Component(c)->Coeffs(), ct_out + ((size_t)i * 2 + c) * n);
    auto dec = rlwe::Decrypt<M>(*key, *ct);
    if (!dec.ok()) return fail(dec.status());
    std::copy(dec->begin(), dec->end(), dec_out + (size_t)i * n);
    cts.push_back(std::move(*ct));
  }
  for (int i = 0; i < half; ++i) {
    auto sum = cts[i] + cts[half + i];
    if (!sum.ok()) return fail(sum.status());
    auto prod = cts[i] * cts[half + i];
    if (!prod.ok()) return fail(prod.status());
    auto ab = cts[i] * pts[half + i];
    if (!ab.ok()) return fail(ab.status());
    for (int c = 0; c < 2; ++c) {
      from_vec(sum->Component(c)->Coeffs(), sum_out + ((size_t)i * 2 + c) * n);
      from_vec(ab->Component(c)->Coeffs(), absorb_out + ((size_t)i * 2 + c) * n);
    }
    for (int c = 0; c < 3; ++c)
      from_vec(prod->Component(c)->Coeffs(), prod_out + ((size_t)i * 3 + c) * n);
    auto d1 = rlwe::Decrypt<M>(*key, *sum);
    auto d2 = rlwe::Decrypt<M>(*key, *prod);
    auto d3 = rlwe::Decrypt<M>(*key, *ab);
    if (!d1.ok()) return fail(d1.status());
    if (!d2.ok()) return fail(d2.status());
    if (!d3.ok()) return fail(d3.status());
    std::copy(d1->begin(), d1->end(), dec_sum + (size_t)i * n);
    std::copy(d2->begin(), d2->end(), dec_prod + (size_t)i * n);
    std::copy(d3->begin(), d3->end(), dec_absorb + (size_t)i * n);
    if (i == 0) {
      err[0] = cts[0].Error();
      err[1] = sum->Error();
      err[2] = prod->Error();
      err[3] = ab->Error();
    }
  }
  return 0;
}

}  // extern "C"
