// Parity test of the C++ host classes (rlwe_gpu.h) on the GPU against the C
// oracle (oracle/shell_oracle.h, a restatement of the reference's CPU code
// pinned to it by tests/golden).  Written like the reference's own tests:
// rns/rns_polynomial_test.cc (NTT round trip, arithmetic, Substitute,
// ModReduceLsb), rns/rns_gadget_test.cc (Decompose),
// rns/rns_relinearization_key_test.cc, rns/rns_galois_key_test.cc,
// rns/rns_bgv_ciphertext_test.cc and oblivious_expand_test.cc, plus the
// reference's status messages on invalid calls.  Prints "ALL OK" and exits 0
// when every check passes.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "rlwe_gpu.h"
#include "shell_oracle.h"

using namespace rlwe_gpu;

namespace {

int g_failures = 0;
int g_checks = 0;

#define EXPECT(cond, what)                                            \
  do {                                                                \
    ++g_checks;                                                       \
    if (!(cond)) {                                                    \
      ++g_failures;                                                   \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, what);       \
    }                                                                 \
  } while (0)

#define ASSERT_OK_AND_ASSIGN(lhs, expr)                                          \
  auto RLWE_GPU_CONCAT_(_r_, __LINE__) = (expr);                                 \
  if (!RLWE_GPU_CONCAT_(_r_, __LINE__).ok()) {                                   \
    std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__,                           \
                RLWE_GPU_CONCAT_(_r_, __LINE__).status().ToString().c_str());    \
    ++g_failures;                                                                \
    return;                                                                      \
  }                                                                              \
  lhs = std::move(RLWE_GPU_CONCAT_(_r_, __LINE__)).value()

#define EXPECT_OK(expr)                                                    \
  do {                                                                     \
    Status _s = (expr);                                                    \
    ++g_checks;                                                            \
    if (!_s.ok()) {                                                        \
      ++g_failures;                                                        \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, _s.ToString().c_str()); \
    }                                                                      \
  } while (0)

void ExpectError(const Status& s, const std::string& msg, int line) {
  ++g_checks;
  if (s.ok() || s.code() != StatusCode::kInvalidArgument || s.message() != msg) {
    ++g_failures;
    std::printf("FAIL line %d: expected InvalidArgument \"%s\", got %s\n", line, msg.c_str(),
                s.ToString().c_str());
  }
}
#define EXPECT_ERROR(expr, msg) ExpectError((expr), (msg), __LINE__)

uint64_t SplitMix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// `count` polynomials of uniform residues over qs, flat [count][L][n].
std::vector<uint64_t> Uniform(uint64_t seed, const std::vector<uint64_t>& qs, int n,
                              int count) {
  std::vector<uint64_t> out((size_t)count * qs.size() * n);
  uint64_t s = seed;
  for (int c = 0; c < count; ++c)
    for (size_t l = 0; l < qs.size(); ++l)
      for (int i = 0; i < n; ++i)
        out[((size_t)c * qs.size() + l) * n + i] = SplitMix(s) % qs[l];
  return out;
}

std::vector<std::vector<uint64_t>> Limbs(const uint64_t* flat, int L, int n) {
  std::vector<std::vector<uint64_t>> v(L);
  for (int l = 0; l < L; ++l) v[l].assign(flat + (size_t)l * n, flat + (size_t)(l + 1) * n);
  return v;
}

std::vector<uint64_t> Flat(const std::vector<std::vector<uint64_t>>& limbs) {
  std::vector<uint64_t> out;
  for (const auto& l : limbs) out.insert(out.end(), l.begin(), l.end());
  return out;
}

std::vector<uint64_t> FlatCt(const RnsBgvCiphertext& ct) {
  std::vector<uint64_t> out;
  for (int c = 0; c < ct.Len(); ++c) {
    auto comp = ct.Component(c);
    auto f = Flat(comp->Coeffs());
    out.insert(out.end(), f.begin(), f.end());
  }
  return out;
}

const std::vector<uint64_t> kQ45 = {35184371138561ull, 35184370941953ull, 35184370352129ull,
                                    35184370155521ull, 35184369893377ull, 35184368877569ull};
const std::vector<uint64_t> kQ50 = {1125899904679937ull, 1125899903827969ull,
                                    1125899903500289ull};
const uint64_t kQ60 = 1152921504606830593ull;

void TestContextErrors() {
  auto bad = RnsContext::Create(10, {35184371138560ull}, {}, 65537);  // even
  EXPECT(!bad.ok(), "even modulus must be rejected");
  auto aux = RnsContext::Create(10, kQ45, {kQ50[0]}, 65537);
  EXPECT(aux.ok() && (*aux)->NumAuxPrimeModuli() == 1, "auxiliary primes are accepted");
  auto dup = RnsContext::Create(10, kQ45, {kQ45[2]}, 65537);
  EXPECT(!dup.ok(), "an auxiliary prime equal to a main prime is rejected");
}

void TestPolynomial(int log_n, const std::vector<uint64_t>& qs) {
  const int n = 1 << log_n, L = (int)qs.size();
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, qs, {}, 65537));
  const Moduli moduli = ctx->MainPrimeModuli();
  so_rns* orc = so_rns_create(log_n, qs.data(), L);
  auto a = Uniform(100 + log_n, qs, n, 1), b = Uniform(200 + log_n, qs, n, 1);

  // ConvertToNttForm / ConvertToCoeffForm (rns_polynomial_test.cc NTT round trip)
  RnsPolynomial pa;
  ASSERT_OK_AND_ASSIGN(pa, RnsPolynomial::Create(Limbs(a.data(), L, n), false));
  EXPECT_OK(pa.ConvertToNttForm(moduli));
  std::vector<uint64_t> want = a;
  so_rns_ntt_fwd(orc, want.data(), L);
  EXPECT(Flat(pa.Coeffs()) == want, "ConvertToNttForm equals the oracle");
  EXPECT_ERROR(pa.ConvertToNttForm(moduli), "Polynomial already in NTT form");
  EXPECT_OK(pa.ConvertToCoeffForm(moduli));
  EXPECT(Flat(pa.Coeffs()) == a, "NTT round trip");
  EXPECT_ERROR(pa.ConvertToCoeffForm(moduli), "Polynomial already in Coefficient form");
  EXPECT_OK(pa.ConvertToNttForm(moduli));

  RnsPolynomial pb;
  ASSERT_OK_AND_ASSIGN(pb, RnsPolynomial::Create(Limbs(b.data(), L, n), true));
  std::vector<uint64_t> wa = want, wb = b, w(a.size());
  // Add / Sub / Negate / Mul / FusedMulAdd against the per-prime oracle ops.
  auto per_limb = [&](auto fn) {
    for (int l = 0; l < L; ++l) fn(so_rns_prime(orc, l), (size_t)l * n);
  };
  RnsPolynomial r;
  ASSERT_OK_AND_ASSIGN(r, pa.Add(pb, moduli));
  per_limb([&](const so_prime* p, size_t o) { so_add(p, &wa[o], &wb[o], &w[o], n); });
  EXPECT(Flat(r.Coeffs()) == w, "Add");
  ASSERT_OK_AND_ASSIGN(r, pa.Sub(pb, moduli));
  per_limb([&](const so_prime* p, size_t o) { so_sub(p, &wa[o], &wb[o], &w[o], n); });
  EXPECT(Flat(r.Coeffs()) == w, "Sub");
  ASSERT_OK_AND_ASSIGN(r, pa.Negate(moduli));
  per_limb([&](const so_prime* p, size_t o) { so_neg(p, &wa[o], &w[o], n); });
  EXPECT(Flat(r.Coeffs()) == w, "Negate");
  ASSERT_OK_AND_ASSIGN(r, pa.Mul(pb, moduli));
  per_limb([&](const so_prime* p, size_t o) { so_mul(p, &wa[o], &wb[o], &w[o], n); });
  EXPECT(Flat(r.Coeffs()) == w, "Mul");
  std::vector<uint64_t> acc = w;
  EXPECT_OK(r.FusedMulAddInPlace(pa, pb, moduli));
  per_limb([&](const so_prime* p, size_t o) { so_fma(p, &acc[o], &wa[o], &wb[o], n); });
  EXPECT(Flat(r.Coeffs()) == acc, "FusedMulAddInPlace");

  // Invalid arguments keep the reference's messages.
  Moduli fewer(moduli.begin(), moduli.end() - 1);
  if (L > 1)
    EXPECT_ERROR(r.AddInPlace(pb, fewer),
                 "`moduli` must contain " + std::to_string(L) + " RNS moduli.");
  RnsPolynomial coeff;
  ASSERT_OK_AND_ASSIGN(coeff, RnsPolynomial::Create(Limbs(a.data(), L, n), false));
  EXPECT_ERROR(coeff.MulInPlace(pb, moduli), "RNS polynomial `this` must be in NTT form.");
  EXPECT_ERROR(pa.Substitute(4, moduli).status(),
               "Substitution power must be a non-negative odd integer less than 2*n.");

  // Substitute (rns_polynomial_test.cc Substitute in NTT form).
  for (int power : {3, 2 * n - 1}) {
    ASSERT_OK_AND_ASSIGN(r, pa.Substitute(power, moduli));
    so_rns_substitute(orc, L, power, wa.data(), w.data());
    EXPECT(Flat(r.Coeffs()) == w, "Substitute");
  }

  // ModReduceLsb in NTT and coefficient form.
  if (L > 1) {
    std::vector<uint64_t> ql_inv;
    ASSERT_OK_AND_ASSIGN(ql_inv, ctx->MainPrimeModulusInverseResidues(L - 1));
    for (int is_ntt : {1, 0}) {
      const std::vector<uint64_t>& src = is_ntt ? wa : a;
      RnsPolynomial m;
      ASSERT_OK_AND_ASSIGN(m, RnsPolynomial::Create(Limbs(src.data(), L, n), is_ntt));
      EXPECT_OK(m.ModReduceLsb(65537, ql_inv, moduli));
      std::vector<uint64_t> wm((size_t)(L - 1) * n);
      so_rns_modreduce_lsb(orc, L, 65537, is_ntt, src.data(), wm.data());
      EXPECT(m.NumModuli() == L - 1 && Flat(m.Coeffs()) == wm, "ModReduceLsb");
    }
    RnsPolynomial m;
    ASSERT_OK_AND_ASSIGN(m, RnsPolynomial::Create(Limbs(wa.data(), L, n), true));
    EXPECT_ERROR(m.ModReduceLsb(65537, std::vector<uint64_t>(L), moduli),
                 "`ql_inv` must be defined with respect to " + std::to_string(L - 1) +
                     " moduli.");
  }
  so_rns_destroy(orc);
}

void TestGadgetAndKeys(int log_n, const std::vector<uint64_t>& qs, std::vector<int> log_bs) {
  const int n = 1 << log_n, L = (int)qs.size();
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, qs, {}, 65537));
  const Moduli moduli = ctx->MainPrimeModuli();
  so_rns* orc = so_rns_create(log_n, qs.data(), L);
  RnsGadget gadget;
  ASSERT_OK_AND_ASSIGN(gadget, RnsGadget::Create(log_n, log_bs, moduli));
  const int k = gadget.Dimension();
  EXPECT(k == so_rns_gadget_dim(orc, L, log_bs.data()), "gadget dimension");

  // Decompose (rns_gadget_test.cc).
  auto x = Uniform(300 + log_n, qs, n, 1);
  RnsPolynomial px;
  ASSERT_OK_AND_ASSIGN(px, RnsPolynomial::Create(Limbs(x.data(), L, n), false));
  std::vector<RnsPolynomial> digits;
  ASSERT_OK_AND_ASSIGN(digits, gadget.Decompose(px, moduli));
  std::vector<uint64_t> wd((size_t)k * L * n);
  so_rns_decompose(orc, L, log_bs.data(), x.data(), wd.data());
  bool same = (int)digits.size() == k;
  for (int j = 0; same && j < k; ++j)
    same = Flat(digits[j].Coeffs()) ==
           std::vector<uint64_t>(wd.begin() + (size_t)j * L * n,
                                 wd.begin() + (size_t)(j + 1) * L * n);
  EXPECT(same, "Decompose");
  EXPECT_OK(px.ConvertToNttForm(moduli));
  EXPECT_ERROR(gadget.Decompose(px, moduli).status(), "`a` must be in coefficient form");

  // Keys from components; ct * ct then relinearize (rns_bgv_ciphertext_test.cc
  // + rns_relinearization_key_test.cc).
  auto kb = Uniform(400 + log_n, qs, n, k), ka = Uniform(500 + log_n, qs, n, k);
  std::vector<RnsPolynomial> key_bs, key_as;
  for (int j = 0; j < k; ++j) {
    RnsPolynomial pb, pa;
    ASSERT_OK_AND_ASSIGN(pb, RnsPolynomial::Create(Limbs(&kb[(size_t)j * L * n], L, n), true));
    ASSERT_OK_AND_ASSIGN(pa, RnsPolynomial::Create(Limbs(&ka[(size_t)j * L * n], L, n), true));
    key_bs.push_back(std::move(pb));
    key_as.push_back(std::move(pa));
  }
  RnsRelinKey relin;
  ASSERT_OK_AND_ASSIGN(relin, RnsRelinKey::CreateFromKeyComponents(key_bs, key_as, &gadget,
                                                                   moduli));
  EXPECT(relin.Dimension() == k, "relin key dimension");
  auto c = Uniform(600 + log_n, qs, n, 2), d = Uniform(700 + log_n, qs, n, 2);
  auto make_ct = [&](const std::vector<uint64_t>& flat, int power) {
    std::vector<RnsPolynomial> comps;
    for (int i = 0; i < 2; ++i)
      comps.push_back(*RnsPolynomial::Create(Limbs(&flat[(size_t)i * L * n], L, n), true));
    return RnsBgvCiphertext(std::move(comps), moduli, power, 1.0);
  };
  RnsBgvCiphertext ct1 = make_ct(c, 1), ct2 = make_ct(d, 1);
  RnsBgvCiphertext prod = ct1;
  ASSERT_OK_AND_ASSIGN(prod, ct1 * ct2);
  std::vector<uint64_t> w3((size_t)3 * L * n);
  so_rns_tensor(orc, L, c.data(), d.data(), w3.data());
  EXPECT(prod.Degree() == 2 && FlatCt(prod) == w3, "RnsBgvCiphertext operator*");
  RnsBgvCiphertext relined = prod;
  ASSERT_OK_AND_ASSIGN(relined, relin.ApplyTo(prod));
  std::vector<uint64_t> w2((size_t)2 * L * n);
  so_rns_relin(orc, L, log_bs.data(), w3.data(), kb.data(), ka.data(), w2.data());
  EXPECT(relined.Degree() == 1 && FlatCt(relined) == w2, "RnsRelinKey::ApplyTo");

  // Degree-3 product goes through the general FMA path.
  RnsBgvCiphertext cube = prod;
  ASSERT_OK_AND_ASSIGN(cube, prod * ct1);
  EXPECT(cube.Degree() == 3, "degree-3 product");
  EXPECT_ERROR(relin.ApplyTo(cube).status(),
               "`ciphertext` degree is larger than degree of this relinearization key, 2.");

  // Rotation: Substitute then the Galois key (rns_galois_key_test.cc).
  const int power = 5;
  RnsGaloisKey galois;
  ASSERT_OK_AND_ASSIGN(galois, RnsGaloisKey::CreateFromKeyComponents(key_as, key_bs, power,
                                                                     &gadget, moduli));
  EXPECT_ERROR(galois.ApplyTo(ct1).status(),
               "`ciphertext` does not have a matching substitution power.");
  RnsBgvCiphertext sub = ct1;
  ASSERT_OK_AND_ASSIGN(sub, ct1.Substitute(power));
  EXPECT(sub.PowerOfS() == power, "power of s after Substitute");
  RnsBgvCiphertext rot = sub;
  ASSERT_OK_AND_ASSIGN(rot, galois.ApplyTo(sub));
  std::vector<uint64_t> sc((size_t)2 * L * n), wr((size_t)2 * L * n);
  for (int i = 0; i < 2; ++i)
    so_rns_substitute(orc, L, power, &c[(size_t)i * L * n], &sc[(size_t)i * L * n]);
  so_rns_galois(orc, L, log_bs.data(), sc.data(), kb.data(), ka.data(), wr.data());
  EXPECT(rot.PowerOfS() == 1 && FlatCt(rot) == wr, "RnsGaloisKey::ApplyTo");

  // Random-pad path (rns_galois_key.cc:289-346): pad digits = NTT-form
  // gadget digits of the substituted ciphertext's c1.
  {
    RnsPolynomial c1;
    ASSERT_OK_AND_ASSIGN(c1, sub.Component(1));
    EXPECT_OK(c1.ConvertToCoeffForm(moduli));
    std::vector<RnsPolynomial> pad_digits;
    ASSERT_OK_AND_ASSIGN(pad_digits, gadget.Decompose(c1, moduli));
    for (auto& d : pad_digits) EXPECT_OK(d.ConvertToNttForm(moduli));
    RnsPolynomial pad_new;
    ASSERT_OK_AND_ASSIGN(pad_new, galois.PrecomputeRandomPad(pad_digits));
    RnsBgvCiphertext padded = sub;
    ASSERT_OK_AND_ASSIGN(padded, galois.ApplyToWithRandomPad(sub, pad_digits, pad_new));
    std::vector<uint64_t> flat_pad;
    for (auto& d : pad_digits) {
      auto f = Flat(d.Coeffs());
      flat_pad.insert(flat_pad.end(), f.begin(), f.end());
    }
    std::vector<uint64_t> wp((size_t)2 * L * n);
    so_rns_galois_pad(orc, L, k, sc.data(), flat_pad.data(), kb.data(), ka.data(), wp.data());
    EXPECT(FlatCt(padded) == wp, "ApplyToWithRandomPad equals the oracle");
    // with the pad being c1's own digits, the result is the plain key switch
    EXPECT(FlatCt(padded) == wr, "random-pad key switch equals ApplyTo");
  }

  // ModReduce drops the top prime of every component.
  if (L > 1) {
    std::vector<uint64_t> ql_inv;
    ASSERT_OK_AND_ASSIGN(ql_inv, ctx->MainPrimeModulusInverseResidues(L - 1));
    RnsBgvCiphertext m = relined;
    EXPECT_OK(m.ModReduce(65537, ql_inv));
    std::vector<uint64_t> wm((size_t)2 * (L - 1) * n);
    for (int i = 0; i < 2; ++i)
      so_rns_modreduce_lsb(orc, L, 65537, 1, &w2[(size_t)i * L * n],
                           &wm[(size_t)i * (L - 1) * n]);
    EXPECT(m.NumModuli() == L - 1 && FlatCt(m) == wm, "RnsBgvCiphertext::ModReduce");
  }
  so_rns_destroy(orc);
}

void TestSingleModulus(int log_n, int levels, int log_b) {
  const int n = 1 << log_n;
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, {kQ60}, {}, 65537));
  const PrimeModulus* m = ctx->MainPrimeModuli()[0];
  so_prime* p = so_prime_create(kQ60, log_n);
  const int dim = so_gadget_size(p, log_b);
  auto keys = Uniform(800 + log_n, {kQ60}, n, levels * 2 * dim);  // [levels][2][dim][n]
  std::vector<GaloisKey> gks;
  for (int j = 0; j < levels; ++j) {
    std::vector<Polynomial> k0, k1;
    for (int i = 0; i < dim; ++i) {
      const uint64_t* r0 = &keys[((size_t)(j * 2 + 0) * dim + i) * n];
      const uint64_t* r1 = &keys[((size_t)(j * 2 + 1) * dim + i) * n];
      k0.push_back(*RnsPolynomial::Create({std::vector<uint64_t>(r0, r0 + n)}, true));
      k1.push_back(*RnsPolynomial::Create({std::vector<uint64_t>(r1, r1 + n)}, true));
    }
    GaloisKey gk = *GaloisKey::CreateFromKeyComponents(k0, k1, (n >> j) + 1, log_b, m);
    gks.push_back(std::move(gk));
  }
  auto c = Uniform(900 + log_n, {kQ60}, n, 2);
  std::vector<Polynomial> comps;
  for (int i = 0; i < 2; ++i)
    comps.push_back(*RnsPolynomial::Create({std::vector<uint64_t>(c.begin() + i * n,
                                                                  c.begin() + (i + 1) * n)},
                                           true));
  SymmetricRlweCiphertext ct(std::move(comps), m, 1, 1.0);

  // GaloisKey::ApplyTo after Substitute (galois_key_test.cc).
  const int power = n + 1;
  SymmetricRlweCiphertext sub = ct;
  ASSERT_OK_AND_ASSIGN(sub, ct.Substitute(power));
  SymmetricRlweCiphertext sw = sub;
  ASSERT_OK_AND_ASSIGN(sw, gks[0].ApplyTo(sub));
  std::vector<uint64_t> sc(2 * (size_t)n), w(2 * (size_t)n);
  for (int i = 0; i < 2; ++i) so_substitute(p, power, &c[(size_t)i * n], &sc[(size_t)i * n]);
  so_galois_apply(p, log_b, dim, sc.data(), &keys[0], &keys[(size_t)dim * n], w.data());
  EXPECT(FlatCt(sw.rns()) == w, "GaloisKey::ApplyTo");
  EXPECT_ERROR(gks[0].ApplyTo(ct).status(),
               "Ciphertext PowerOfS: 1 doesn't match the key substitution power: " +
                   std::to_string(power));

  // ObliviousExpand (oblivious_expand_test.cc) with a truncated output.
  std::unique_ptr<GaloisKeysObliviousExpander> ex;
  ASSERT_OK_AND_ASSIGN(ex, GaloisKeysObliviousExpander::Create(gks, 16, m));
  const int out_len = (1 << levels) - 1;
  std::vector<SymmetricRlweCiphertext> expanded;
  ASSERT_OK_AND_ASSIGN(expanded, ex->ObliviousExpand({ct}, levels, out_len));
  std::vector<uint64_t> we(((size_t)2 << levels) * n);
  so_oblivious_expand(p, levels, log_b, keys.data(), c.data(), we.data());
  bool same = (int)expanded.size() == out_len;
  for (int i = 0; same && i < out_len; ++i)
    same = FlatCt(expanded[i].rns()) ==
           std::vector<uint64_t>(we.begin() + (size_t)i * 2 * n,
                                 we.begin() + (size_t)(i + 1) * 2 * n);
  EXPECT(same, "ObliviousExpand");
  EXPECT_ERROR(ex->ObliviousExpand({ct}, levels, (1 << levels) + 1).status(),
               "Output length must be at most " + std::to_string(1 << levels));
  so_prime_destroy(p);
}

// The single-modulus flow (symmetric_encryption_test.cc): encrypt with
// injected randomness, decrypt, ct + ct and ct * ct against the oracle.
void TestSymmetric() {
  const int log_n = 11, n = 1 << log_n;
  const uint64_t q = 576460752303415297ull, t = 65537;
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, {q}, {}, t));
  const PrimeModulus* m = ctx->MainPrimeModuli()[0];
  so_prime* p = so_prime_create(q, log_n);
  uint64_t st = 99;
  auto small = [&](int var) {  // centred binomial samples, imported
    std::vector<uint64_t> v(n);
    for (int i = 0; i < n; ++i) {
      int acc = 0;
      for (int b = 0; b < 2 * var; ++b) acc += (SplitMix(st) & 1) ? 1 : 0;
      const int64_t x = acc - var;
      v[i] = x < 0 ? q - (uint64_t)(-x) : (uint64_t)x;
    }
    so_import(p, v.data(), v.data(), n);
    return v;
  };
  std::vector<uint64_t> s = small(8);
  so_ntt_fwd(p, s.data());
  SymmetricRlweKey key = *SymmetricRlweKey::Create(*RnsPolynomial::Create({s}, true), m);
  std::vector<std::vector<uint64_t>> msgs(2, std::vector<uint64_t>(n));
  std::vector<SymmetricRlweCiphertext> cts;
  std::vector<std::vector<uint64_t>> want_cts;
  for (int c = 0; c < 2; ++c) {
    for (int i = 0; i < n; ++i) msgs[c][i] = SplitMix(st) % t;
    std::vector<uint64_t> mm = msgs[c];
    so_import(p, mm.data(), mm.data(), n);
    so_ntt_fwd(p, mm.data());
    std::vector<uint64_t> a = Uniform(4000 + c, {q}, n, 1), e = small(8);
    std::vector<uint64_t> w(2 * n);
    so_sym_encrypt(p, t, s.data(), a.data(), e.data(), mm.data(), w.data());
    want_cts.push_back(w);
    auto ct = key.Encrypt(*RnsPolynomial::Create({mm}, true), *RnsPolynomial::Create({a}, true),
                          *RnsPolynomial::Create({e}, false));
    EXPECT(ct.ok() && FlatCt(ct->rns()) == w, "SymmetricRlweKey::Encrypt");
    if (!ct.ok()) return;
    cts.push_back(*ct);
  }
  std::vector<uint64_t> dec;
  ASSERT_OK_AND_ASSIGN(dec, key.Decrypt(cts[0]));
  EXPECT(dec == msgs[0], "Decrypt(Encrypt(m)) == m");
  SymmetricRlweCiphertext sum = cts[0];
  ASSERT_OK_AND_ASSIGN(sum, cts[0] + cts[1]);
  ASSERT_OK_AND_ASSIGN(dec, key.Decrypt(sum));
  bool ok = true;
  for (int i = 0; i < n; ++i) ok &= dec[i] == (msgs[0][i] + msgs[1][i]) % t;
  EXPECT(ok, "Decrypt(ct1 + ct2) == m1 + m2");
  SymmetricRlweCiphertext prod = cts[0];
  ASSERT_OK_AND_ASSIGN(prod, cts[0] * cts[1]);
  ASSERT_OK_AND_ASSIGN(dec, key.Decrypt(prod));
  std::vector<uint64_t> want(n);
  auto fp = FlatCt(prod.rns());
  so_sym_decrypt(p, t, s.data(), fp.data(), 3, want.data());
  EXPECT(prod.Len() == 3 && dec == want, "Decrypt(ct1 * ct2) equals the oracle");
  so_prime_destroy(p);
}

// RnsRlweSecretKey::EncryptPolynomialBgv with the ChaCha PRNG on the device
// against the oracle's restatement (rns/rns_secret_key_test.cc's encryption
// cases), plus the reference's messages on bad seeds and plaintexts.
void TestRnsSecretKey(int log_n, const std::vector<uint64_t>& qs) {
  const int n = 1 << log_n, L = (int)qs.size();
  const uint64_t t = 65537;
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, qs, {}, t));
  const Moduli moduli = ctx->MainPrimeModuli();
  std::vector<uint64_t> s = Uniform(31, qs, n, 1);
  RnsRlweSecretKey key = *RnsRlweSecretKey::CreateFromKey(
      *RnsPolynomial::Create(Limbs(s.data(), L, n), true), moduli, 8);
  so_rns* r = so_rns_create(log_n, qs.data(), L);
  std::vector<RnsPolynomial> pts;
  std::vector<std::string> seeds;
  std::vector<std::vector<uint64_t>> want;
  for (int c = 0; c < 3; ++c) {
    std::vector<uint64_t> m = Uniform(500 + c, qs, n, 1);
    pts.push_back(*RnsPolynomial::Create(Limbs(m.data(), L, n), true));
    std::string seed(32, '\0');
    for (int i = 0; i < 32; ++i) seed[i] = (char)(i * 11 + c);
    seeds.push_back(seed);
    std::vector<uint64_t> w((size_t)2 * L * n);
    so_rns_encrypt_bgv(r, L, t, 8, s.data(), m.data(),
                       reinterpret_cast<const uint8_t*>(seed.data()), w.data());
    want.push_back(w);
  }
  RnsBgvCiphertext one = *key.EncryptPolynomialBgv(pts[1], seeds[1]);
  EXPECT(FlatCt(one) == want[1] && one.PowerOfS() == 1 && one.Len() == 2,
         "EncryptPolynomialBgv equals the oracle");
  std::vector<RnsBgvCiphertext> batch;
  ASSERT_OK_AND_ASSIGN(batch, key.EncryptPolynomialBgv(pts, seeds));
  bool ok = batch.size() == 3;
  for (int c = 0; ok && c < 3; ++c) ok &= FlatCt(batch[c]) == want[c];
  EXPECT(ok, "batched EncryptPolynomialBgv equals the oracle");
  EXPECT_ERROR(key.EncryptPolynomialBgv(pts[0], std::string(16, 'x')).status(),
               "Cannot create Prng with key of the wrong size. Real key length of 16 instead "
               "of expected key length of 32.");
  RnsPolynomial coeff = pts[0];
  EXPECT_OK(coeff.ConvertToCoeffForm(moduli));
  EXPECT_ERROR(key.EncryptPolynomialBgv(coeff, seeds[0]).status(),
               "`plaintext` must be in NTT form.");
  EXPECT_ERROR(RnsRlweSecretKey::CreateFromKey(pts[0], moduli, 0).status(),
               "`variance` must be positive.");
  EXPECT_ERROR(RnsRlweSecretKey::CreateFromKey(pts[0], moduli, 257).status(),
               "The variance, 257, must be at most 256.");
  so_rns_destroy(r);
}

// RnsBfvCiphertext (operator*, AbsorbInPlace, ModReduce) on a context with
// auxiliary primes, and RnsGaloisKey::Compose, against the oracle
// (rns/rns_bfv_ciphertext_test.cc, rns/rns_galois_key_test.cc).
void TestBfvAndCompose(int log_n, const std::vector<uint64_t>& qs,
                       const std::vector<uint64_t>& ps) {
  const int n = 1 << log_n, L = (int)qs.size(), K = (int)ps.size();
  const uint64_t t = 40961;
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, qs, ps, t));
  EXPECT(ctx->NumAuxPrimeModuli() == K, "AuxPrimeModuli");
  const Moduli moduli = ctx->MainPrimeModuli();
  std::vector<uint64_t> all = qs;
  all.insert(all.end(), ps.begin(), ps.end());
  so_rns* r = so_rns_create(log_n, all.data(), L + K);
  std::vector<int> aux(K);
  for (int j = 0; j < K; ++j) aux[j] = L + j;
  auto make_ct = [&](uint64_t seed) {
    std::vector<uint64_t> flat = Uniform(seed, qs, n, 2);
    std::vector<RnsPolynomial> comps;
    for (int c = 0; c < 2; ++c)
      comps.push_back(*RnsPolynomial::Create(Limbs(flat.data() + (size_t)c * L * n, L, n), true));
    return std::make_pair(RnsBfvCiphertext(RnsBgvCiphertext(comps, moduli, 1, 1.0), ctx.get()),
                          flat);
  };
  auto [x, fx] = make_ct(71);
  auto [y, fy] = make_ct(72);
  RnsBfvCiphertext prod = x;
  ASSERT_OK_AND_ASSIGN(prod, x * y);
  std::vector<uint64_t> want((size_t)3 * L * n);
  so_bfv_mul(r, L, aux.data(), K, t, fx.data(), fy.data(), want.data());
  EXPECT(prod.Len() == 3 && FlatCt(prod) == want, "RnsBfvCiphertext::operator*");
  std::vector<uint64_t> pt = Uniform(73, qs, n, 1);
  RnsBfvCiphertext absorbed = x;
  EXPECT_OK(absorbed.AbsorbInPlace(*RnsPolynomial::Create(Limbs(pt.data(), L, n), true)));
  want.assign((size_t)2 * L * n, 0);
  so_bfv_absorb(r, L, aux.data(), K, t, 2, fx.data(), pt.data(), want.data());
  EXPECT(FlatCt(absorbed) == want, "RnsBfvCiphertext::AbsorbInPlace");
  if (L > 1) {
    RnsBfvCiphertext red = x;
    EXPECT_OK(red.ModReduce());
    std::vector<uint64_t> w2;
    for (int c = 0; c < 2; ++c) {
      std::vector<uint64_t> o((size_t)(L - 1) * n);
      so_rns_modreduce_msb(r, L, 1, fx.data() + (size_t)c * L * n, o.data());
      w2.insert(w2.end(), o.begin(), o.end());
    }
    EXPECT(red.NumModuli() == L - 1 && FlatCt(red) == w2, "RnsBfvCiphertext::ModReduce");
  }
  // Compose of two Galois keys = rotating the second key's rows with the first
  std::vector<int> log_bs(L, 10);
  RnsGadget gadget = *RnsGadget::Create(log_n, log_bs, moduli);
  const int k = gadget.Dimension();
  std::vector<uint64_t> kb1 = Uniform(81, qs, n, k), ka1 = Uniform(82, qs, n, k);
  std::vector<uint64_t> kb2 = Uniform(83, qs, n, k), ka2 = Uniform(84, qs, n, k);
  auto rows = [&](const std::vector<uint64_t>& f) {
    std::vector<RnsPolynomial> v;
    for (int j = 0; j < k; ++j)
      v.push_back(*RnsPolynomial::Create(Limbs(f.data() + (size_t)j * L * n, L, n), true));
    return v;
  };
  RnsGaloisKey g1 = *RnsGaloisKey::CreateFromKeyComponents(rows(ka1), rows(kb1), 5, &gadget,
                                                           moduli);
  RnsGaloisKey g2 = *RnsGaloisKey::CreateFromKeyComponents(rows(ka2), rows(kb2), 3, &gadget,
                                                           moduli);
  RnsGaloisKey g12 = g1;
  ASSERT_OK_AND_ASSIGN(g12, g1.Compose(g2));
  EXPECT(g12.SubstitutionPower() == 15, "composed power");
  // apply the composed key and the oracle's composed rows to one ciphertext
  std::vector<uint64_t> cb((size_t)k * L * n), ca((size_t)k * L * n);
  for (int j = 0; j < k; ++j) {
    std::vector<uint64_t> row((size_t)2 * L * n), sub((size_t)2 * L * n), o((size_t)2 * L * n);
    std::copy(kb2.begin() + (size_t)j * L * n, kb2.begin() + (size_t)(j + 1) * L * n, row.begin());
    std::copy(ka2.begin() + (size_t)j * L * n, ka2.begin() + (size_t)(j + 1) * L * n,
              row.begin() + (size_t)L * n);
    so_rns_substitute(r, L, 5, row.data(), sub.data());
    so_rns_substitute(r, L, 5, row.data() + (size_t)L * n, sub.data() + (size_t)L * n);
    so_rns_galois(r, L, log_bs.data(), sub.data(), kb1.data(), ka1.data(), o.data());
    std::copy(o.begin(), o.begin() + (size_t)L * n, cb.begin() + (size_t)j * L * n);
    std::copy(o.begin() + (size_t)L * n, o.end(), ca.begin() + (size_t)j * L * n);
  }
  std::vector<uint64_t> got_b(cb.size()), got_a(ca.size());
  EXPECT_OK(Status(static_cast<StatusCode>(
                       shg_key_components(g12.handle(), got_b.data(), got_a.data())),
                   ""));
  EXPECT(got_b == cb && got_a == ca, "RnsGaloisKey::Compose rows");
  so_rns_destroy(r);
}

// Error() bookkeeping (rns/rns_ciphertext.h, rns/rns_bgv_ciphertext.h,
// rns/rns_relinearization_key.h:158-164, rns/rns_galois_key.h:284-290)
// against the reference's own values for the same parameters, read from
// `path` (one parameter set: "log_n log_t sigma e0 e1 scalar power L q... lb...",
// then "name value" lines; written by tests/test_host_api.py from the golden
// fixture).
void TestErrorBookkeeping(const char* path) {
  FILE* f = std::fopen(path, "r");
  EXPECT(f != nullptr, "error flow file");
  if (!f) return;
  int log_n, log_t, scalar, power, L;
  double sigma, e0, e1;
  if (std::fscanf(f, "%d %d %lf %lf %lf %d %d %d", &log_n, &log_t, &sigma, &e0, &e1, &scalar,
                  &power, &L) != 8) {
    EXPECT(false, "error flow header");
    std::fclose(f);
    return;
  }
  std::vector<uint64_t> qs(L);
  std::vector<int> log_bs(L);
  for (auto& q : qs) EXPECT(std::fscanf(f, "%llu", (unsigned long long*)&q) == 1, "q");
  for (auto& b : log_bs) EXPECT(std::fscanf(f, "%d", &b) == 1, "log_b");
  std::vector<std::pair<std::string, double>> want;
  char name[64];
  double v;
  while (std::fscanf(f, "%63s %lf", name, &v) == 2) want.emplace_back(name, v);
  std::fclose(f);
  auto expect_value = [&](const std::string& key, double got) {
    for (const auto& kv : want)
      if (kv.first == key) {
        ++g_checks;
        if (kv.second != got) {
          ++g_failures;
          std::printf("FAIL error %s: got %.17g want %.17g\n", key.c_str(), got, kv.second);
        }
        return;
      }
    EXPECT(false, ("missing expected value " + key).c_str());
  };
  const int n = 1 << log_n;
  std::unique_ptr<const RnsContext> ctx;
  ASSERT_OK_AND_ASSIGN(ctx, RnsContext::Create(log_n, qs, {}, 65537));
  const Moduli moduli = ctx->MainPrimeModuli();
  RnsErrorParams ep = *RnsErrorParams::Create(log_n, moduli, {}, log_t, sigma);
  RnsGadget gadget;
  ASSERT_OK_AND_ASSIGN(gadget, RnsGadget::Create(log_n, log_bs, moduli));
  const int k = gadget.Dimension();
  expect_value("B_plaintext", ep.B_plaintext());
  expect_value("B_secretkey_encryption", ep.B_secretkey_encryption());
  expect_value("B_publickey_encryption", ep.B_publickey_encryption());
  expect_value("B_scale", ep.B_scale());
  expect_value("gadget_key_switching_bound",
               ep.BoundOnGadgetBasedKeySwitching(1, gadget.LogGadgetBase(), k));
  auto poly = [&](int seed) {
    auto v = Uniform(seed, qs, n, 1);
    return *RnsPolynomial::Create(Limbs(v.data(), L, n), true);
  };
  auto ct = [&](double e, int seed) {
    return RnsBgvCiphertext({poly(seed), poly(seed + 1)}, moduli, 1, e, &ep);
  };
  RnsBgvCiphertext c0 = ct(e0, 900), c1 = ct(e1, 910);
  expect_value("add", (*(c0 + c1)).Error());
  expect_value("sub", (*(c0 - c1)).Error());
  {
    RnsBgvCiphertext x = ct(e0, 900);
    EXPECT_OK(x.AbsorbInPlace(poly(920)));
    expect_value("absorb", x.Error());
  }
  {
    RnsBgvCiphertext x = ct(e0, 900);
    EXPECT_OK(x.AbsorbInPlace((uint64_t)scalar));
    expect_value("absorb_scalar", x.Error());
  }
  {
    RnsBgvCiphertext x = ct(e0, 900);
    EXPECT_OK(x.FusedAbsorbAddInPlace(c1, poly(920)));
    expect_value("fused_absorb_add", x.Error());
  }
  RnsBgvCiphertext prod = *(c0 * c1);
  expect_value("mul", prod.Error());
  auto kb = Uniform(930, qs, n, k), ka = Uniform(940, qs, n, k);
  std::vector<RnsPolynomial> key_bs, key_as;
  for (int j = 0; j < k; ++j) {
    key_bs.push_back(*RnsPolynomial::Create(Limbs(&kb[(size_t)j * L * n], L, n), true));
    key_as.push_back(*RnsPolynomial::Create(Limbs(&ka[(size_t)j * L * n], L, n), true));
  }
  RnsRelinKey relin = *RnsRelinKey::CreateFromKeyComponents(key_bs, key_as, &gadget, moduli);
  expect_value("relin", (*relin.ApplyTo(prod)).Error());
  {
    RnsBgvCiphertext x = ct(e0, 900);
    EXPECT_OK(x.ModReduce(65537, *ctx->MainPrimeModulusInverseResidues(L - 1)));
    expect_value("mod_reduce", x.Error());
  }
  RnsBgvCiphertext sub = *c0.Substitute(power);
  expect_value("substitute", sub.Error());
  RnsGaloisKey galois =
      *RnsGaloisKey::CreateFromKeyComponents(key_as, key_bs, power, &gadget, moduli);
  expect_value("galois", (*galois.ApplyTo(sub)).Error());
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1) TestErrorBookkeeping(argv[1]);
  TestSymmetric();
  TestRnsSecretKey(10, {kQ45[0], kQ45[1]});
  TestRnsSecretKey(14, kQ45);
  TestBfvAndCompose(11, {8589905921ull, 8589852673ull, 8589844481ull},
                    {1073692673ull, 1073668097ull});
  TestBfvAndCompose(12, {kQ45[0], kQ45[1]}, {35184368320513ull, 35184368025601ull,
                                              35184367828993ull});
  TestContextErrors();
  TestPolynomial(4, {kQ45[0], kQ45[1]});
  TestPolynomial(11, kQ50);
  TestPolynomial(14, kQ45);
  TestPolynomial(15, {kQ50[0], kQ50[1]});
  TestGadgetAndKeys(10, {kQ45[0], kQ45[1], kQ45[2]}, {20, 20, 20});
  TestGadgetAndKeys(12, {kQ50[0], kQ50[1]}, {50, 16});
  TestGadgetAndKeys(14, kQ45, {20, 20, 20, 20, 20, 20});
  TestSingleModulus(8, 4, 8);
  TestSingleModulus(12, 3, 10);
  std::printf("%d checks, %d failures\n", g_checks, g_failures);
  if (g_failures == 0) std::printf("ALL OK\n");
  return g_failures == 0 ? 0 : 1;
}
