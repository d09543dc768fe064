// Implementation of the C++ host classes in rlwe_gpu.h over the C ABI.
// Validation messages follow the reference's (file:line at each method);
// every numeric operation is a libshellgpu.so call.
#include "rlwe_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include <utility>

namespace rlwe_gpu {
namespace {

shg_stream g_stream = nullptr;

Status FromCode(int code) {
  if (code == SHG_OK) return OkStatus();
  return Status(static_cast<StatusCode>(code), shg_last_error());
}

std::string ModuliMessage(int num) {
  return "`moduli` must contain " + std::to_string(num) + " RNS moduli.";
}

shg_context* ContextOf(const Moduli& moduli) {
  return moduli.empty() || !moduli[0] ? nullptr : moduli[0]->Context()->handle();
}

// The device context's primes must be the leading primes of the context, in
// order: that is how every RnsPolynomial of a ciphertext chain is defined
// (MainPrimeModuli() and its prefixes after ModReduce).
Status CheckPrefix(const Moduli& moduli) {
  for (size_t i = 0; i < moduli.size(); ++i) {
    if (!moduli[i] || moduli[i]->Index() != static_cast<int>(i) ||
        moduli[i]->Context() != moduli[0]->Context())
      return InvalidArgumentError(
          "`moduli` must be a prefix of one context's MainPrimeModuli().");
  }
  return OkStatus();
}

}  // namespace

std::string Status::ToString() const {
  if (ok()) return "OK";
  return "code " + std::to_string(static_cast<int>(code_)) + ": " + message_;
}

void SetStream(shg_stream stream) { g_stream = stream; }
shg_stream GetStream() { return g_stream; }

// ---------------------------------------------------------------------------
// DeviceArray
// ---------------------------------------------------------------------------

DeviceArray::DeviceArray(size_t elems) : elems_(elems) {
  void* p = nullptr;
  if (elems && shg_device_alloc(elems * sizeof(uint64_t), &p) != SHG_OK) elems_ = 0;
  ptr_ = static_cast<uint64_t*>(p);
}

DeviceArray::DeviceArray(const DeviceArray& other) : DeviceArray(other.elems_) {
  if (elems_)
    shg_memcpy_d2d(ptr_, other.ptr_, elems_ * sizeof(uint64_t), g_stream);
}

DeviceArray& DeviceArray::operator=(const DeviceArray& other) {
  if (this != &other) {
    DeviceArray tmp(other);
    *this = std::move(tmp);
  }
  return *this;
}

DeviceArray::DeviceArray(DeviceArray&& other) noexcept
    : ptr_(other.ptr_), elems_(other.elems_) {
  other.ptr_ = nullptr;
  other.elems_ = 0;
}

DeviceArray& DeviceArray::operator=(DeviceArray&& other) noexcept {
  if (this != &other) {
    if (ptr_) {
      shg_stream_synchronize(g_stream);
      shg_device_free(ptr_);
    }
    ptr_ = other.ptr_;
    elems_ = other.elems_;
    other.ptr_ = nullptr;
    other.elems_ = 0;
  }
  return *this;
}

DeviceArray::~DeviceArray() {
  if (ptr_) {
    shg_stream_synchronize(g_stream);
    shg_device_free(ptr_);
  }
}

Status DeviceArray::Upload(const uint64_t* host, size_t elems, size_t offset) {
  if (offset + elems > elems_) return InvalidArgumentError("upload out of range");
  if (!elems) return OkStatus();
  RLWE_GPU_RETURN_IF_ERROR(
      FromCode(shg_memcpy_h2d(ptr_ + offset, host, elems * sizeof(uint64_t), g_stream)));
  return FromCode(shg_stream_synchronize(g_stream));
}

Status DeviceArray::Download(uint64_t* host, size_t elems, size_t offset) const {
  if (offset + elems > elems_) return InvalidArgumentError("download out of range");
  if (!elems) return OkStatus();
  RLWE_GPU_RETURN_IF_ERROR(
      FromCode(shg_memcpy_d2h(host, ptr_ + offset, elems * sizeof(uint64_t), g_stream)));
  return FromCode(shg_stream_synchronize(g_stream));
}

// ---------------------------------------------------------------------------
// RnsContext
// ---------------------------------------------------------------------------

StatusOr<std::unique_ptr<const RnsContext>> RnsContext::Create(
    int log_n, std::vector<uint64_t> qs, std::vector<uint64_t> ps,
    uint64_t plaintext_modulus) {
  shg_context* h = nullptr;
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_context_create_with_aux(
      log_n, qs.data(), static_cast<int>(qs.size()), ps.data(), static_cast<int>(ps.size()),
      plaintext_modulus, &h)));
  std::unique_ptr<RnsContext> ctx(new RnsContext());
  ctx->h_ = h;
  ctx->log_n_ = log_n;
  ctx->t_ = plaintext_modulus;
  for (size_t i = 0; i < qs.size(); ++i)
    ctx->moduli_.push_back(std::unique_ptr<PrimeModulus>(
        new PrimeModulus(ctx.get(), static_cast<int>(i), qs[i])));
  for (size_t j = 0; j < ps.size(); ++j)
    ctx->aux_.push_back(std::unique_ptr<PrimeModulus>(
        new PrimeModulus(ctx.get(), static_cast<int>(qs.size() + j), ps[j])));
  return std::unique_ptr<const RnsContext>(std::move(ctx));
}

Moduli RnsContext::AuxPrimeModuli() const {
  Moduli out;
  for (const auto& m : aux_) out.push_back(m.get());
  return out;
}

RnsContext::~RnsContext() { shg_context_destroy(h_); }

Moduli RnsContext::MainPrimeModuli() const {
  Moduli out;
  for (const auto& m : moduli_) out.push_back(m.get());
  return out;
}

StatusOr<std::vector<uint64_t>> RnsContext::MainPrimeModulusInverseResidues(
    int level) const {
  std::vector<uint64_t> out(level > 0 ? level : 1);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_context_ql_inv(h_, level, out.data())));
  out.resize(level);
  return out;
}

// ---------------------------------------------------------------------------
// RnsPolynomial
// ---------------------------------------------------------------------------

StatusOr<RnsPolynomial> RnsPolynomial::Create(
    std::vector<std::vector<uint64_t>> coeff_vectors, bool is_ntt) {
  // rns/rns_polynomial.cc:35-60
  if (coeff_vectors.empty())
    return InvalidArgumentError("`coeff_vectors` cannot be empty.");
  const size_t num_coeffs = coeff_vectors[0].size();
  if (num_coeffs == 0 || (num_coeffs & (num_coeffs - 1)))
    return InvalidArgumentError(
        "`coeff_vectors` must contain vectors of length a power of two.");
  for (const auto& v : coeff_vectors)
    if (v.size() != num_coeffs)
      return InvalidArgumentError(
          "`coeff_vectors` must contain vectors of equal length.");
  int log_n = 0;
  while ((size_t(1) << log_n) < num_coeffs) ++log_n;
  RnsPolynomial p;
  p.data_ = DeviceArray(coeff_vectors.size() * num_coeffs);
  for (size_t i = 0; i < coeff_vectors.size(); ++i)
    RLWE_GPU_RETURN_IF_ERROR(
        p.data_.Upload(coeff_vectors[i].data(), num_coeffs, i * num_coeffs));
  p.log_n_ = log_n;
  p.num_moduli_ = static_cast<int>(coeff_vectors.size());
  p.is_ntt_ = is_ntt;
  return p;
}

StatusOr<RnsPolynomial> RnsPolynomial::CreateZero(int log_n, const Moduli& moduli,
                                                  bool is_ntt) {
  // rns/rns_polynomial.cc:63-83
  if (log_n <= 0) return InvalidArgumentError("`log_n` must be positive.");
  if (moduli.empty()) return InvalidArgumentError("`moduli` must not be empty.");
  RnsPolynomial p;
  p.data_ = DeviceArray(moduli.size() << log_n);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_memset_device(p.data_.data(), 0, p.data_.size() * sizeof(uint64_t), g_stream)));
  p.log_n_ = log_n;
  p.num_moduli_ = static_cast<int>(moduli.size());
  p.is_ntt_ = is_ntt;
  return p;
}

RnsPolynomial RnsPolynomial::FromDevice(DeviceArray data, int log_n, int num_moduli,
                                        bool is_ntt) {
  RnsPolynomial p;
  p.data_ = std::move(data);
  p.log_n_ = log_n;
  p.num_moduli_ = num_moduli;
  p.is_ntt_ = is_ntt;
  return p;
}

std::vector<std::vector<uint64_t>> RnsPolynomial::Coeffs() const {
  std::vector<std::vector<uint64_t>> out(num_moduli_,
                                         std::vector<uint64_t>(NumCoeffs()));
  for (int i = 0; i < num_moduli_; ++i)
    data_.Download(out[i].data(), NumCoeffs(), (size_t)i * NumCoeffs());
  return out;
}

Status RnsPolynomial::CheckModuli(const Moduli& moduli) const {
  if (static_cast<int>(moduli.size()) != num_moduli_)
    return InvalidArgumentError(ModuliMessage(num_moduli_));
  RLWE_GPU_RETURN_IF_ERROR(CheckPrefix(moduli));
  if (moduli[0]->Context()->LogN() != log_n_)
    return InvalidArgumentError("`moduli` belong to a context of another ring degree.");
  return OkStatus();
}

Status RnsPolynomial::CheckThat(const RnsPolynomial& that, const char* name) const {
  if (that.num_moduli_ != num_moduli_)
    return InvalidArgumentError(std::string("`") + name + "` must contain " +
                                std::to_string(num_moduli_) + " coefficient vectors.");
  if (that.log_n_ != log_n_)
    return InvalidArgumentError(std::string("`") + name + "` has a mismatched ring degree.");
  return OkStatus();
}

Status RnsPolynomial::ConvertToNttForm(const Moduli& moduli) {
  // rns/rns_polynomial.cc:171-188
  if (is_ntt_) return InvalidArgumentError("Polynomial already in NTT form");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_ntt_forward(ContextOf(moduli), data_.data(), 1, num_moduli_, g_stream)));
  is_ntt_ = true;
  return OkStatus();
}

Status RnsPolynomial::ConvertToCoeffForm(const Moduli& moduli) {
  // rns/rns_polynomial.cc:190-207
  if (!is_ntt_) return InvalidArgumentError("Polynomial already in Coefficient form");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_ntt_inverse(ContextOf(moduli), data_.data(), 1, num_moduli_, g_stream)));
  is_ntt_ = false;
  return OkStatus();
}

StatusOr<RnsPolynomial> RnsPolynomial::Negate(const Moduli& moduli) const {
  RnsPolynomial out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.NegateInPlace(moduli));
  return out;
}

Status RnsPolynomial::NegateInPlace(const Moduli& moduli) {
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  return FromCode(shg_poly_neg(ContextOf(moduli), data_.data(), data_.data(), 1,
                               num_moduli_, g_stream));
}

StatusOr<RnsPolynomial> RnsPolynomial::Add(const RnsPolynomial& that,
                                           const Moduli& moduli) const {
  RnsPolynomial out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.AddInPlace(that, moduli));
  return out;
}

Status RnsPolynomial::AddInPlace(const RnsPolynomial& that, const Moduli& moduli) {
  RLWE_GPU_RETURN_IF_ERROR(CheckThat(that, "that"));
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  return FromCode(shg_poly_add(ContextOf(moduli), data_.data(), data_.data(),
                               that.data_.data(), 1, num_moduli_, g_stream));
}

StatusOr<RnsPolynomial> RnsPolynomial::Sub(const RnsPolynomial& that,
                                           const Moduli& moduli) const {
  RnsPolynomial out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.SubInPlace(that, moduli));
  return out;
}

Status RnsPolynomial::SubInPlace(const RnsPolynomial& that, const Moduli& moduli) {
  RLWE_GPU_RETURN_IF_ERROR(CheckThat(that, "that"));
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  return FromCode(shg_poly_sub(ContextOf(moduli), data_.data(), data_.data(),
                               that.data_.data(), 1, num_moduli_, g_stream));
}

StatusOr<RnsPolynomial> RnsPolynomial::Mul(uint64_t scalar, const Moduli& moduli) const {
  RnsPolynomial out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.MulInPlace(scalar, moduli));
  return out;
}

Status RnsPolynomial::MulInPlace(uint64_t scalar, const Moduli& moduli) {
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  return FromCode(shg_poly_mul_integer(ContextOf(moduli), data_.data(), data_.data(),
                                       scalar, 1, num_moduli_, g_stream));
}

Status RnsPolynomial::MulInPlace(const std::vector<uint64_t>& scalar_mod_qs,
                                 const Moduli& moduli) {
  if (static_cast<int>(scalar_mod_qs.size()) != num_moduli_)
    return InvalidArgumentError("`scalar_mod_qs` must contain " +
                                std::to_string(num_moduli_) + " modular integers.");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  return FromCode(shg_poly_mul_rns_scalar(ContextOf(moduli), data_.data(), data_.data(),
                                          scalar_mod_qs.data(), 1, num_moduli_, g_stream));
}

StatusOr<RnsPolynomial> RnsPolynomial::Mul(const RnsPolynomial& that,
                                           const Moduli& moduli) const {
  RnsPolynomial out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.MulInPlace(that, moduli));
  return out;
}

Status RnsPolynomial::MulInPlace(const RnsPolynomial& that, const Moduli& moduli) {
  // rns/rns_polynomial.h:296-326
  RLWE_GPU_RETURN_IF_ERROR(CheckThat(that, "that"));
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  if (!is_ntt_) return InvalidArgumentError("RNS polynomial `this` must be in NTT form.");
  if (!that.is_ntt_)
    return InvalidArgumentError("RNS polynomial `that` must be in NTT form.");
  return FromCode(shg_poly_mul(ContextOf(moduli), data_.data(), data_.data(),
                               that.data_.data(), 1, num_moduli_, g_stream));
}

Status RnsPolynomial::FusedMulAddInPlace(const RnsPolynomial& a, const RnsPolynomial& b,
                                         const Moduli& moduli) {
  // rns/rns_polynomial.h:328-365
  RLWE_GPU_RETURN_IF_ERROR(CheckThat(a, "a"));
  RLWE_GPU_RETURN_IF_ERROR(CheckThat(b, "b"));
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  if (!is_ntt_) return InvalidArgumentError("RNS polynomial `this` must be in NTT form.");
  if (!a.is_ntt_) return InvalidArgumentError("RNS polynomial `a` must be in NTT form.");
  if (!b.is_ntt_) return InvalidArgumentError("RNS polynomial `b` must be in NTT form.");
  return FromCode(shg_poly_fma(ContextOf(moduli), data_.data(), a.data_.data(),
                               b.data_.data(), 1, num_moduli_, g_stream));
}

StatusOr<RnsPolynomial> RnsPolynomial::Substitute(int power, const Moduli& moduli) const {
  // rns/rns_polynomial.cc:209-227
  if (power < 0 || (power % 2) == 0 || power >= 2 * NumCoeffs())
    return InvalidArgumentError(
        "Substitution power must be a non-negative odd integer less than 2*n.");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  if (!is_ntt_) return InvalidArgumentError("RnsPolynomial must be in NTT form");
  RnsPolynomial out = FromDevice(DeviceArray(data_.size()), log_n_, num_moduli_, true);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_substitute(
      ContextOf(moduli), out.data_.data(), data_.data(), power, 1, num_moduli_, g_stream)));
  return out;
}

Status RnsPolynomial::ModReduceLsb(uint64_t t, const std::vector<uint64_t>& ql_inv,
                                   const Moduli& moduli) {
  // rns/rns_polynomial.cc:262-280
  if (static_cast<int>(moduli.size()) != num_moduli_)
    return InvalidArgumentError(ModuliMessage(num_moduli_));
  if (num_moduli_ <= 1)
    return InvalidArgumentError("ModReduceLsb cannot apply with only one prime modulus.");
  if (static_cast<int>(ql_inv.size()) != num_moduli_ - 1)
    return InvalidArgumentError("`ql_inv` must be defined with respect to " +
                                std::to_string(num_moduli_ - 1) + " moduli.");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  DeviceArray out((size_t)(num_moduli_ - 1) << log_n_);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_poly_modreduce_lsb(ContextOf(moduli), out.data(), data_.data(), t, ql_inv.data(),
                             is_ntt_ ? 1 : 0, 1, num_moduli_, g_stream)));
  data_ = std::move(out);
  --num_moduli_;
  return OkStatus();
}

Status RnsPolynomial::ModReduceMsb(const std::vector<uint64_t>& ql_inv, const Moduli& moduli) {
  // rns/rns_polynomial.cc:349-366
  if (static_cast<int>(moduli.size()) != num_moduli_)
    return InvalidArgumentError(ModuliMessage(num_moduli_));
  if (num_moduli_ <= 1)
    return InvalidArgumentError("ModReduceMsb cannot apply with only one prime modulus.");
  if (static_cast<int>(ql_inv.size()) != num_moduli_ - 1)
    return InvalidArgumentError("`ql_inv` must be defined with respect to " +
                                std::to_string(num_moduli_ - 1) + " moduli.");
  RLWE_GPU_RETURN_IF_ERROR(CheckModuli(moduli));
  DeviceArray out((size_t)(num_moduli_ - 1) << log_n_);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_modreduce_msb(ContextOf(moduli), out.data(),
                                                           data_.data(), ql_inv.data(),
                                                           is_ntt_ ? 1 : 0, 1, num_moduli_,
                                                           g_stream)));
  data_ = std::move(out);
  --num_moduli_;
  return OkStatus();
}

// ---------------------------------------------------------------------------
// RnsGadget
// ---------------------------------------------------------------------------

StatusOr<RnsGadget> RnsGadget::Create(int log_n, std::vector<int> log_bs,
                                      const Moduli& moduli) {
  // rns/rns_gadget.cc:42-70
  if (log_n <= 0) return InvalidArgumentError("`log_n` must be positive.");
  if (moduli.empty()) return InvalidArgumentError("`moduli` must not be empty.");
  if (log_bs.size() != moduli.size())
    return InvalidArgumentError("`log_bs` must contain " + std::to_string(moduli.size()) +
                                " elements.");
  RnsGadget g;
  g.log_n_ = log_n;
  for (size_t i = 0; i < moduli.size(); ++i) {
    if (log_bs[i] <= 0) return InvalidArgumentError("`log_bs` must contain positive integers.");
    int log_q = 0;
    while (log_q < 64 && (moduli[i]->Modulus() >> log_q)) ++log_q;
    g.dimension_ += (log_q + log_bs[i] - 1) / log_bs[i];  // GadgetSize (gadget.h:43-47)
  }
  g.log_bs_ = std::move(log_bs);
  return g;
}

StatusOr<std::vector<RnsPolynomial>> RnsGadget::Decompose(const RnsPolynomial& a,
                                                          const Moduli& moduli) const {
  // rns/rns_gadget.cc:108-120
  if (a.IsNttForm()) return InvalidArgumentError("`a` must be in coefficient form");
  const int num_moduli = static_cast<int>(moduli.size());
  if (a.NumModuli() != num_moduli)
    return InvalidArgumentError("`a` must be defined with respect to " +
                                std::to_string(num_moduli) + " RNS moduli.");
  if (static_cast<int>(log_bs_.size()) != num_moduli)
    return InvalidArgumentError("`moduli` must contain " + std::to_string(log_bs_.size()) +
                                " RNS moduli.");
  RLWE_GPU_RETURN_IF_ERROR(CheckPrefix(moduli));
  const size_t poly = (size_t)num_moduli << a.LogN();
  DeviceArray all(poly * dimension_);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_gadget_decompose(
      ContextOf(moduli), num_moduli, log_bs_.data(), all.data(), a.device_data(), 1,
      g_stream)));
  std::vector<RnsPolynomial> xs;
  xs.reserve(dimension_);
  for (int j = 0; j < dimension_; ++j) {
    DeviceArray one(poly);
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(
        one.data(), all.data() + j * poly, poly * sizeof(uint64_t), g_stream)));
    xs.push_back(RnsPolynomial::FromDevice(std::move(one), a.LogN(), num_moduli, false));
  }
  return xs;
}

int RnsGadget::LogGadgetBase() const {
  return log_bs_.empty() ? 0 : *std::max_element(log_bs_.begin(), log_bs_.end());
}

// ---------------------------------------------------------------------------
// RnsErrorParams (rns/rns_error_params.h).  Each bound keeps the reference's
// formula and evaluation order, so the doubles are the same.
// ---------------------------------------------------------------------------

StatusOr<RnsErrorParams> RnsErrorParams::Create(int log_n, const Moduli& main_moduli,
                                                const Moduli& aux_moduli,
                                                int log_plaintext_modulus, double sigma) {
  std::vector<uint64_t> qs, ps;
  for (const PrimeModulus* m : main_moduli) qs.push_back(m->Modulus());
  for (const PrimeModulus* m : aux_moduli) ps.push_back(m->Modulus());
  return Create(log_n, qs, ps, log_plaintext_modulus, sigma);
}

StatusOr<RnsErrorParams> RnsErrorParams::Create(int log_n, const std::vector<uint64_t>& main_qs,
                                                const std::vector<uint64_t>&,
                                                int log_plaintext_modulus, double sigma) {
  // rns/rns_error_params.h:46-62
  if (log_n <= 0) return InvalidArgumentError("`log_n` must be positive.");
  if (main_qs.empty()) return InvalidArgumentError("`main_moduli` must not be empty.");
  if (log_plaintext_modulus <= 0)
    return InvalidArgumentError("`log_plaintext_modulus` must be positive.");
  if (sigma <= 0) return InvalidArgumentError("`sigma` must be positive.");
  return RnsErrorParams(log_n, log_plaintext_modulus, sigma);
}

double RnsErrorParams::T2() const {
  // The reference's ExportDoubleT(): log_plaintext_modulus squared.
  return std::pow(log_t_, 2);
}

RnsErrorParams::RnsErrorParams(int log_n, int log_t, double sigma)
    : log_n_(log_n), log_t_(log_t), sigma_(sigma) {
  const int dimension = 1 << log_n;
  // rns/rns_error_params.h:127-167
  b_plaintext_ = T2() * std::sqrt(3.0 * dimension);
  b_secretkey_encryption_ = T2() * std::sqrt(dimension) * (std::sqrt(3.0) + 6.0 * sigma);
  b_publickey_encryption_ =
      T2() * (std::sqrt(dimension) * (6 * sigma + std::sqrt(3)) + 72 * dimension * sigma * sigma);
  b_scale_ = T2() * (std::sqrt(3.0 * dimension) + 8.0 * dimension * std::sqrt(1 / 3.0));
}

double RnsErrorParams::BoundOnGadgetBasedKeySwitching(int num_components, int log_gadget_base,
                                                      int num_digits) const {
  // rns/rns_error_params.h:84-91
  const int gadget_base = 1 << log_gadget_base;
  const int dimension = 1 << log_n_;
  return (8.0 / std::sqrt(3.0)) * T2() * num_digits * sigma_ * dimension * gadget_base *
         num_components;
}

namespace {

// The additive error of a gadget key switch with `key` on `num_components`
// components (rns/rns_relinearization_key.h:158-164, rns/rns_galois_key.h:
// 284-290); zero without error parameters.
double KeySwitchError(const RnsBgvCiphertext& ct, shg_key* key, int num_components) {
  if (!ct.ErrorParams()) return 0.0;
  int log_bs[64];
  const int L = shg_key_num_limbs(key);
  if (L <= 0 || L > 64 || shg_key_log_bs(key, log_bs, 64) != SHG_OK) return 0.0;
  int max_log_b = 0;
  for (int i = 0; i < L; ++i) max_log_b = std::max(max_log_b, log_bs[i]);
  return ct.ErrorParams()->BoundOnGadgetBasedKeySwitching(num_components, max_log_b,
                                                          shg_key_dimension(key));
}

}  // namespace

// ---------------------------------------------------------------------------
// RnsBgvCiphertext
// ---------------------------------------------------------------------------

RnsBgvCiphertext::RnsBgvCiphertext(std::vector<RnsPolynomial> components, Moduli moduli,
                                   int power_of_s, double error,
                                   const RnsErrorParams* error_params)
    : len_(static_cast<int>(components.size())),
      log_n_(components.empty() ? 0 : components[0].LogN()),
      moduli_(std::move(moduli)),
      power_of_s_(power_of_s),
      error_(error),
      error_params_(error_params) {
  const size_t elems = component_elems();
  data_ = DeviceArray(elems * len_);
  for (int i = 0; i < len_; ++i)
    shg_memcpy_d2d(data_.data() + i * elems, components[i].device_data(),
                   elems * sizeof(uint64_t), g_stream);
}

RnsBgvCiphertext RnsBgvCiphertext::FromDevice(DeviceArray data, int num_components,
                                              int log_n, Moduli moduli, int power_of_s,
                                              double error,
                                              const RnsErrorParams* error_params) {
  RnsBgvCiphertext ct;
  ct.error_params_ = error_params;
  ct.data_ = std::move(data);
  ct.len_ = num_components;
  ct.log_n_ = log_n;
  ct.moduli_ = std::move(moduli);
  ct.power_of_s_ = power_of_s;
  ct.error_ = error;
  return ct;
}

StatusOr<RnsPolynomial> RnsBgvCiphertext::Component(int index) const {
  // rns/rns_ciphertext.h:573-578
  if (index < 0 || index >= len_) return InvalidArgumentError("Index out of range.");
  const size_t elems = component_elems();
  DeviceArray one(elems);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(
      one.data(), data_.data() + index * elems, elems * sizeof(uint64_t), g_stream)));
  return RnsPolynomial::FromDevice(std::move(one), log_n_, NumModuli(), true);
}

Status RnsBgvCiphertext::CheckSameShape(const RnsBgvCiphertext& that,
                                        bool check_degree) const {
  // rns/rns_ciphertext.h:111-122
  if (check_degree && that.len_ != len_)
    return InvalidArgumentError("`that` has a mismatched degree.");
  if (that.Level() != Level()) return InvalidArgumentError("`that` has a mismatched level.");
  if (that.power_of_s_ != power_of_s_)
    return InvalidArgumentError("`that` is encrypted with a different key power.");
  return OkStatus();
}

Status RnsBgvCiphertext::AddInPlace(const RnsBgvCiphertext& that) {
  RLWE_GPU_RETURN_IF_ERROR(CheckSameShape(that, true));
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_add(ContextOf(moduli_), data_.data(),
                                                 data_.data(), that.data_.data(), len_,
                                                 NumModuli(), g_stream)));
  error_ += that.error_;
  return OkStatus();
}

Status RnsBgvCiphertext::SubInPlace(const RnsBgvCiphertext& that) {
  RLWE_GPU_RETURN_IF_ERROR(CheckSameShape(that, true));
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_sub(ContextOf(moduli_), data_.data(),
                                                 data_.data(), that.data_.data(), len_,
                                                 NumModuli(), g_stream)));
  error_ += that.error_;
  return OkStatus();
}

Status RnsBgvCiphertext::NegateInPlace() {
  return FromCode(shg_poly_neg(ContextOf(moduli_), data_.data(), data_.data(), len_,
                               NumModuli(), g_stream));
}

StatusOr<RnsBgvCiphertext> RnsBgvCiphertext::operator+(const RnsBgvCiphertext& that) const {
  RnsBgvCiphertext out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.AddInPlace(that));
  return out;
}

StatusOr<RnsBgvCiphertext> RnsBgvCiphertext::operator-(const RnsBgvCiphertext& that) const {
  RnsBgvCiphertext out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.SubInPlace(that));
  return out;
}

Status RnsBgvCiphertext::AbsorbInPlace(const RnsPolynomial& plaintext) {
  // rns/rns_ciphertext.h:208-217: every component times the plaintext.
  if (plaintext.NumModuli() != NumModuli())
    return InvalidArgumentError("`plaintext` has a mismatched level.");
  if (!plaintext.IsNttForm())
    return InvalidArgumentError("RNS polynomial `that` must be in NTT form.");
  const size_t elems = component_elems();
  for (int i = 0; i < len_; ++i)
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_mul(
        ContextOf(moduli_), data_.data() + i * elems, data_.data() + i * elems,
        plaintext.device_data(), 1, NumModuli(), g_stream)));
  if (error_params_) error_ *= error_params_->B_plaintext();
  return OkStatus();
}

Status RnsBgvCiphertext::AbsorbInPlace(uint64_t scalar) {
  // rns/rns_ciphertext.h:267-274: every component times the integer.
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_mul_integer(ContextOf(moduli_), data_.data(),
                                                         data_.data(), scalar, len_,
                                                         NumModuli(), g_stream)));
  // The scalar is represented as a value in [-scalar/2, scalar/2].
  error_ *= static_cast<double>(scalar) / 2;
  return OkStatus();
}

Status RnsBgvCiphertext::FusedAbsorbAddInPlace(const RnsBgvCiphertext& ctxt,
                                               const RnsPolynomial& ptxt) {
  // rns/rns_ciphertext.h:277-298
  if (Degree() != ctxt.Degree()) return InvalidArgumentError("`ctxt` has a mismatched degree.");
  if (Level() != ctxt.Level()) return InvalidArgumentError("`ctxt` has a mismatched level.");
  if (PowerOfS() != ctxt.PowerOfS())
    return InvalidArgumentError("`ctxt` has a mismatched key power.");
  if (ptxt.NumModuli() != NumModuli())
    return InvalidArgumentError("`ptxt` has a mismatched level.");
  if (!ptxt.IsNttForm()) return InvalidArgumentError("RNS polynomial `b` must be in NTT form.");
  const size_t elems = component_elems();
  for (int i = 0; i < len_; ++i)
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_fma(
        ContextOf(moduli_), data_.data() + i * elems, ctxt.data_.data() + i * elems,
        ptxt.device_data(), 1, NumModuli(), g_stream)));
  if (error_params_) error_ += ctxt.error_ * error_params_->B_plaintext();
  return OkStatus();
}

StatusOr<RnsBgvCiphertext> RnsBgvCiphertext::operator*(const RnsPolynomial& plaintext) const {
  RnsBgvCiphertext out = *this;
  RLWE_GPU_RETURN_IF_ERROR(out.AbsorbInPlace(plaintext));
  return out;
}

StatusOr<RnsBgvCiphertext> RnsBgvCiphertext::operator*(const RnsBgvCiphertext& that) const {
  // rns/rns_ciphertext.h:501-524: result[i + j] += c_i * d_j.
  if (Level() != that.Level()) return InvalidArgumentError("`that` has a mismatched level.");
  if (PowerOfS() != that.PowerOfS())
    return InvalidArgumentError("Ciphertexts must be encrypted with the same key power.");
  const int out_len = len_ + that.len_ - 1;
  const size_t elems = component_elems();
  DeviceArray out(elems * out_len);
  shg_context* ctx = ContextOf(moduli_);
  if (len_ == 2 && that.len_ == 2) {
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_ct_tensor(ctx, out.data(), data_.data(),
                                                    that.data_.data(), 1, NumModuli(),
                                                    g_stream)));
  } else {
    RLWE_GPU_RETURN_IF_ERROR(FromCode(
        shg_memset_device(out.data(), 0, out.size() * sizeof(uint64_t), g_stream)));
    for (int i = 0; i < len_; ++i)
      for (int j = 0; j < that.len_; ++j)
        RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_fma(
            ctx, out.data() + (i + j) * elems, data_.data() + i * elems,
            that.data_.data() + j * elems, 1, NumModuli(), g_stream)));
  }
  return FromDevice(std::move(out), out_len, log_n_, moduli_, power_of_s_,
                    error_ * that.error_, error_params_);
}

Status RnsBgvCiphertext::ModReduce(uint64_t t, const std::vector<uint64_t>& ql_inv) {
  // rns/rns_bgv_ciphertext.h:141-153
  if (moduli_.size() <= 1)
    return FailedPreconditionError(
        "Cannot perform ModReduce with insufficient number of prime moduli.");
  const int L = NumModuli();
  if (static_cast<int>(ql_inv.size()) != L - 1)
    return InvalidArgumentError("`ql_inv` must be defined with respect to " +
                                std::to_string(L - 1) + " moduli.");
  DeviceArray out((size_t)len_ * (L - 1) << log_n_);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_modreduce_lsb(
      ContextOf(moduli_), out.data(), data_.data(), t, ql_inv.data(), 1, len_, L,
      g_stream)));
  data_ = std::move(out);
  moduli_.pop_back();
  return OkStatus();
}

StatusOr<RnsBgvCiphertext> RnsBgvCiphertext::Substitute(int substitution_power) const {
  // rns/rns_bgv_ciphertext.h:155-170
  if (substitution_power < 0 || (substitution_power % 2) == 0 ||
      substitution_power >= 2 * NumCoeffs())
    return InvalidArgumentError(
        "Substitution power must be a non-negative odd integer less than 2*n.");
  DeviceArray out(data_.size());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_substitute(
      ContextOf(moduli_), out.data(), data_.data(), substitution_power, len_, NumModuli(),
      g_stream)));
  const int power = (int)(((int64_t)power_of_s_ * substitution_power) % (2 * NumCoeffs()));
  return FromDevice(std::move(out), len_, log_n_, moduli_, power, error_, error_params_);
}

// ---------------------------------------------------------------------------
// Keys
// ---------------------------------------------------------------------------

namespace {

// Uploads key components ([k][L][n] each) into a device key.
StatusOr<std::shared_ptr<shg_key>> MakeKey(const std::vector<RnsPolynomial>& bs,
                                           const std::vector<RnsPolynomial>& as,
                                           int power, const RnsGadget* gadget,
                                           const Moduli& moduli) {
  if (gadget == nullptr) return InvalidArgumentError("`gadget` must not be null.");
  if (static_cast<int>(as.size()) != gadget->Dimension() ||
      static_cast<int>(bs.size()) != gadget->Dimension())
    return InvalidArgumentError(
        "`key_as` and `key_bs` must have the same length as the gadget dimension.");
  RLWE_GPU_RETURN_IF_ERROR(CheckPrefix(moduli));
  if (moduli.empty()) return InvalidArgumentError("`moduli` must not be empty.");
  const int L = static_cast<int>(moduli.size());
  const int log_n = moduli[0]->Context()->LogN();
  const size_t poly = (size_t)L << log_n;
  std::vector<uint64_t> hb(poly * bs.size()), ha(poly * as.size());
  for (size_t j = 0; j < bs.size(); ++j) {
    if (bs[j].NumModuli() != L || as[j].NumModuli() != L || bs[j].LogN() != log_n ||
        as[j].LogN() != log_n || !bs[j].IsNttForm() || !as[j].IsNttForm())
      return InvalidArgumentError(
          "key components must be NTT-form polynomials over `moduli`.");
    auto cb = bs[j].Coeffs(), ca = as[j].Coeffs();
    for (int l = 0; l < L; ++l) {
      std::copy(cb[l].begin(), cb[l].end(), hb.begin() + j * poly + ((size_t)l << log_n));
      std::copy(ca[l].begin(), ca[l].end(), ha.begin() + j * poly + ((size_t)l << log_n));
    }
  }
  shg_key* k = nullptr;
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_key_create(ContextOf(moduli), L,
                                                   gadget->LogGadgetBases().data(), power,
                                                   hb.data(), ha.data(), &k)));
  return std::shared_ptr<shg_key>(k, [](shg_key* p) { shg_key_destroy(p); });
}

}  // namespace

StatusOr<RnsRelinKey> RnsRelinKey::CreateFromKeyComponents(
    const std::vector<RnsPolynomial>& key_bs, const std::vector<RnsPolynomial>& key_as,
    const RnsGadget* gadget, Moduli moduli) {
  RnsRelinKey key;
  RLWE_GPU_ASSIGN_OR_RETURN(key.key_, MakeKey(key_bs, key_as, 1, gadget, moduli));
  key.moduli_ = std::move(moduli);
  return key;
}

int RnsRelinKey::Dimension() const { return shg_key_dimension(key_.get()); }

StatusOr<RnsBgvCiphertext> RnsRelinKey::ApplyTo(const RnsBgvCiphertext& ct) const {
  // rns/rns_relinearization_key.cc:184-203 (degree-2 key)
  if (ct.Degree() > 2)
    return InvalidArgumentError(
        "`ciphertext` degree is larger than degree of this relinearization key, 2.");
  if (ct.NumModuli() != static_cast<int>(moduli_.size()))
    return InvalidArgumentError("`ciphertext` does not have a matching RNS moduli set.");
  if (ct.PowerOfS() != 1)
    return InvalidArgumentError(
        "Relinearization key can only apply to a ciphertext of power 1.");
  if (ct.Degree() < 2) return ct;
  DeviceArray out(2 * ct.component_elems());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_relin_apply(ContextOf(moduli_), key_.get(),
                                                    out.data(), ct.device_data(), 1,
                                                    g_stream)));
  // ErrorAfterApplication (rns/rns_relinearization_key.h:158-164)
  const double error = ct.Error() + KeySwitchError(ct, key_.get(), ct.Degree() - 1);
  return RnsBgvCiphertext::FromDevice(std::move(out), 2, ct.LogN(), moduli_, 1, error,
                                      ct.ErrorParams());
}

// ---------------------------------------------------------------------------
// RnsBfvCiphertext
// ---------------------------------------------------------------------------

StatusOr<RnsBfvCiphertext> RnsBfvCiphertext::operator*(const RnsBfvCiphertext& that) const {
  // rns/rns_bfv_ciphertext.cc:100-108
  if (Level() != that.Level()) return InvalidArgumentError("`that` has a mismatched level.");
  if (PowerOfS() != that.PowerOfS())
    return InvalidArgumentError("Ciphertexts must be encrypted with the same key power.");
  if (Len() != 2 || that.Len() != 2)
    return InvalidArgumentError("the device BFV product takes two-component ciphertexts");
  if (!context_ || context_->NumAuxPrimeModuli() == 0)
    return InvalidArgumentError("the context has no auxiliary prime moduli");
  DeviceArray out(3 * component_elems());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_bfv_mul(context_->handle(), out.data(), device_data(),
                                                that.device_data(), 1, NumModuli(),
                                                g_stream)));
  return RnsBfvCiphertext(
      FromDevice(std::move(out), 3, LogN(), moduli(), PowerOfS(), Error() * that.Error()),
      context_);
}

Status RnsBfvCiphertext::AbsorbInPlace(const RnsPolynomial& plaintext) {
  // rns/rns_bfv_ciphertext.cc:33-98
  if (!plaintext.IsNttForm()) return InvalidArgumentError("`plaintext` must be in NTT form.");
  if (plaintext.NumModuli() != NumModuli() || plaintext.LogN() != LogN())
    return InvalidArgumentError("`plaintext` has a mismatched level.");
  if (!context_ || context_->NumAuxPrimeModuli() == 0)
    return InvalidArgumentError("the context has no auxiliary prime moduli");
  DeviceArray out(data_.size());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_bfv_absorb(context_->handle(), out.data(),
                                                   data_.data(), plaintext.device_data(), len_,
                                                   1, NumModuli(), g_stream)));
  data_ = std::move(out);
  return OkStatus();
}

Status RnsBfvCiphertext::ModReduce() {
  // rns/rns_bfv_ciphertext.h:184-200
  if (moduli_.size() <= 1)
    return FailedPreconditionError(
        "Cannot perform ModReduce with insufficient number of prime moduli.");
  const int L = NumModuli();
  RLWE_GPU_ASSIGN_OR_RETURN(std::vector<uint64_t> ql_inv,
                            context_->MainPrimeModulusInverseResidues(L - 1));
  DeviceArray out((size_t)len_ * (L - 1) << log_n_);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_poly_modreduce_msb(
      context_->handle(), out.data(), data_.data(), ql_inv.data(), 1, len_, L, g_stream)));
  data_ = std::move(out);
  moduli_.pop_back();
  return OkStatus();
}

StatusOr<RnsGaloisKey> RnsGaloisKey::Compose(const RnsGaloisKey& other_key) const {
  shg_key* k = nullptr;
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_galois_key_compose(ContextOf(moduli_), key_.get(), other_key.key_.get(), &k)));
  RnsGaloisKey key;
  key.key_ = std::shared_ptr<shg_key>(k, [](shg_key* p) { shg_key_destroy(p); });
  key.moduli_ = moduli_;
  key.power_ = shg_key_power(k);
  return key;
}

StatusOr<RnsGaloisKey> RnsGaloisKey::CreateFromKeyComponents(
    const std::vector<RnsPolynomial>& key_as, const std::vector<RnsPolynomial>& key_bs,
    int power, const RnsGadget* gadget, Moduli moduli) {
  RnsGaloisKey key;
  RLWE_GPU_ASSIGN_OR_RETURN(key.key_, MakeKey(key_bs, key_as, power, gadget, moduli));
  key.moduli_ = std::move(moduli);
  key.power_ = power;
  return key;
}

int RnsGaloisKey::Dimension() const { return shg_key_dimension(key_.get()); }

StatusOr<RnsBgvCiphertext> RnsGaloisKey::ApplyTo(const RnsBgvCiphertext& ct) const {
  // rns/rns_galois_key.cc:238-252
  if (ct.PowerOfS() != power_)
    return InvalidArgumentError("`ciphertext` does not have a matching substitution power.");
  if (ct.NumModuli() != static_cast<int>(moduli_.size()))
    return InvalidArgumentError("`ciphertext` does not have a matching RNS moduli set.");
  if (ct.Degree() != 1)
    return InvalidArgumentError("Galois key can only apply to a ciphertext of degree 1.");
  DeviceArray out(2 * ct.component_elems());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_galois_apply(ContextOf(moduli_), key_.get(),
                                                     out.data(), ct.device_data(), 1,
                                                     g_stream)));
  // ErrorAfterApplication (rns/rns_galois_key.h:284-290)
  const double error = ct.Error() + KeySwitchError(ct, key_.get(), 1);
  return RnsBgvCiphertext::FromDevice(std::move(out), 2, ct.LogN(), moduli_, 1, error,
                                      ct.ErrorParams());
}

StatusOr<DeviceArray> RnsGaloisKey::PackDigits(
    const std::vector<RnsPolynomial>& digits) const {
  if (static_cast<int>(digits.size()) != Dimension())
    return InvalidArgumentError("`ciphertext_pad_digits` has incorrect size");
  const int L = static_cast<int>(moduli_.size());
  const size_t poly = (size_t)L << moduli_[0]->Context()->LogN();
  DeviceArray all(poly * digits.size());
  for (size_t j = 0; j < digits.size(); ++j) {
    if (digits[j].NumModuli() != L || !digits[j].IsNttForm())
      return InvalidArgumentError("`ciphertext_pad_digits` must be in NTT form");
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(all.data() + j * poly,
                                                     digits[j].device_data(),
                                                     poly * sizeof(uint64_t), g_stream)));
  }
  return all;
}

StatusOr<RnsPolynomial> RnsGaloisKey::PrecomputeRandomPad(
    const std::vector<RnsPolynomial>& ciphertext_pad_digits) const {
  DeviceArray pad;
  RLWE_GPU_ASSIGN_OR_RETURN(pad, PackDigits(ciphertext_pad_digits));
  const int L = static_cast<int>(moduli_.size());
  const int log_n = moduli_[0]->Context()->LogN();
  DeviceArray out((size_t)L << log_n);
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_galois_precompute_pad(
      ContextOf(moduli_), key_.get(), out.data(), pad.data(), 1, g_stream)));
  return RnsPolynomial::FromDevice(std::move(out), log_n, L, true);
}

StatusOr<RnsBgvCiphertext> RnsGaloisKey::ApplyToWithRandomPad(
    const RnsBgvCiphertext& ct, const std::vector<RnsPolynomial>& ciphertext_pad_digits,
    const RnsPolynomial& ciphertext_pad_new) const {
  // rns/rns_galois_key.cc:313-330
  if (ct.PowerOfS() != power_)
    return InvalidArgumentError("`ciphertext` does not have a matching substitution power.");
  if (ct.NumModuli() != static_cast<int>(moduli_.size()))
    return InvalidArgumentError("`ciphertext` does not have a matching RNS moduli set.");
  if (ct.Degree() > 1)
    return InvalidArgumentError("Galois key can only apply to a ciphertext of degree 1.");
  DeviceArray pad;
  RLWE_GPU_ASSIGN_OR_RETURN(pad, PackDigits(ciphertext_pad_digits));
  DeviceArray out(2 * ct.component_elems());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_galois_apply_with_pad(
      ContextOf(moduli_), key_.get(), out.data(), ct.device_data(), pad.data(),
      ciphertext_pad_new.device_data(), 1, g_stream)));
  const double error = ct.Error() + KeySwitchError(ct, key_.get(), 1);
  return RnsBgvCiphertext::FromDevice(std::move(out), 2, ct.LogN(), moduli_, 1, error,
                                      ct.ErrorParams());
}

// ---------------------------------------------------------------------------
// Single modulus
// ---------------------------------------------------------------------------

SymmetricRlweCiphertext::SymmetricRlweCiphertext(std::vector<Polynomial> components,
                                                 const PrimeModulus* modulus,
                                                 int power_of_s, double error)
    : ct_(std::move(components), Moduli{modulus}, power_of_s, error), modulus_(modulus) {}

SymmetricRlweCiphertext SymmetricRlweCiphertext::FromDevice(DeviceArray data,
                                                            int num_components, int log_n,
                                                            const PrimeModulus* modulus,
                                                            int power_of_s, double error) {
  return SymmetricRlweCiphertext(
      RnsBgvCiphertext::FromDevice(std::move(data), num_components, log_n,
                                   Moduli{modulus}, power_of_s, error),
      modulus);
}

StatusOr<SymmetricRlweCiphertext> SymmetricRlweCiphertext::operator+(
    const SymmetricRlweCiphertext& that) const {
  RLWE_GPU_ASSIGN_OR_RETURN(RnsBgvCiphertext r, ct_ + that.ct_);
  return SymmetricRlweCiphertext(std::move(r), modulus_);
}

StatusOr<SymmetricRlweCiphertext> SymmetricRlweCiphertext::operator-(
    const SymmetricRlweCiphertext& that) const {
  RLWE_GPU_ASSIGN_OR_RETURN(RnsBgvCiphertext r, ct_ - that.ct_);
  return SymmetricRlweCiphertext(std::move(r), modulus_);
}

StatusOr<SymmetricRlweCiphertext> SymmetricRlweCiphertext::operator*(
    const SymmetricRlweCiphertext& that) const {
  RLWE_GPU_ASSIGN_OR_RETURN(RnsBgvCiphertext r, ct_ * that.ct_);
  return SymmetricRlweCiphertext(std::move(r), modulus_);
}

Status SymmetricRlweCiphertext::AbsorbInPlace(const Polynomial& plaintext) {
  return ct_.AbsorbInPlace(plaintext);
}

StatusOr<SymmetricRlweCiphertext> SymmetricRlweCiphertext::Substitute(
    int substitution_power) const {
  RLWE_GPU_ASSIGN_OR_RETURN(RnsBgvCiphertext r, ct_.Substitute(substitution_power));
  return SymmetricRlweCiphertext(std::move(r), modulus_);
}

StatusOr<SymmetricRlweKey> SymmetricRlweKey::Create(Polynomial key,
                                                    const PrimeModulus* modulus) {
  if (!modulus) return InvalidArgumentError("`modulus` must not be null.");
  if (modulus->Context()->NumMainPrimeModuli() != 1)
    return InvalidArgumentError("symmetric encryption needs a one-prime context");
  if (key.NumModuli() != 1 || key.LogN() != modulus->Context()->LogN() || !key.IsNttForm())
    return InvalidArgumentError("the key must be one NTT-form polynomial of the ring");
  return SymmetricRlweKey(std::move(key), modulus);
}

StatusOr<RnsRlweSecretKey> RnsRlweSecretKey::CreateFromKey(RnsPolynomial key, Moduli moduli,
                                                           int variance) {
  if (moduli.empty()) return InvalidArgumentError("`moduli` must not be empty.");
  if (key.NumModuli() != (int)moduli.size())
    return InvalidArgumentError("`key` must have one limb per modulus.");
  if (!key.IsNttForm()) return InvalidArgumentError("`key` must be in NTT form.");
  if (variance <= 0) return InvalidArgumentError("`variance` must be positive.");
  if (variance > 256)
    return InvalidArgumentError("The variance, " + std::to_string(variance) +
                                ", must be at most 256.");
  return RnsRlweSecretKey(std::move(key), std::move(moduli), variance);
}

StatusOr<std::vector<RnsBgvCiphertext>> RnsRlweSecretKey::EncryptPolynomialBgv(
    const std::vector<RnsPolynomial>& plaintexts, const std::vector<std::string>& prng_seeds,
    double error_bound) const {
  if (plaintexts.size() != prng_seeds.size())
    return InvalidArgumentError("one PRNG seed per plaintext is needed");
  const int L = key_.NumModuli(), log_n = key_.LogN();
  const size_t limb_elems = (size_t)L << log_n, count = plaintexts.size();
  for (const RnsPolynomial& pt : plaintexts) {
    if (!pt.IsNttForm()) return InvalidArgumentError("`plaintext` must be in NTT form.");
    if (pt.NumModuli() != L || pt.LogN() != log_n)
      return InvalidArgumentError("`plaintext` must have the key's ring and moduli");
  }
  std::vector<uint64_t> seed_words(count * 4);
  for (size_t i = 0; i < count; ++i) {
    if (prng_seeds[i].size() != 32)
      return InvalidArgumentError(
          "Cannot create Prng with key of the wrong size. Real key length of " +
          std::to_string(prng_seeds[i].size()) + " instead of expected key length of 32.");
    std::memcpy(&seed_words[i * 4], prng_seeds[i].data(), 32);
  }
  std::vector<RnsBgvCiphertext> out;
  if (count == 0) return out;
  DeviceArray seeds(count * 4), pts(count * limb_elems), cts(count * 2 * limb_elems);
  RLWE_GPU_RETURN_IF_ERROR(seeds.Upload(seed_words.data(), seed_words.size()));
  shg_context* h = moduli_[0]->Context()->handle();
  for (size_t i = 0; i < count; ++i)
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(pts.data() + i * limb_elems,
                                                      plaintexts[i].device_data(),
                                                      limb_elems * 8, g_stream)));
  RLWE_GPU_RETURN_IF_ERROR(FromCode(
      shg_bgv_encrypt(h, cts.data(), key_.device_data(), pts.data(),
                      reinterpret_cast<const uint8_t*>(seeds.data()), L, (int)count, variance_,
                      g_stream)));
  out.reserve(count);
  for (size_t i = 0; i < count; ++i) {
    DeviceArray one(2 * limb_elems);
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(one.data(), cts.data() + i * 2 * limb_elems,
                                                      2 * limb_elems * 8, g_stream)));
    out.push_back(RnsBgvCiphertext::FromDevice(std::move(one), 2, log_n, moduli_, 1,
                                               error_bound));
  }
  return out;
}

StatusOr<RnsBgvCiphertext> RnsRlweSecretKey::EncryptPolynomialBgv(
    const RnsPolynomial& plaintext, const std::string& prng_seed, double error_bound) const {
  RLWE_GPU_ASSIGN_OR_RETURN(std::vector<RnsBgvCiphertext> cts,
                            EncryptPolynomialBgv(std::vector<RnsPolynomial>{plaintext},
                                                 std::vector<std::string>{prng_seed},
                                                 error_bound));
  return std::move(cts[0]);
}

StatusOr<SymmetricRlweCiphertext> SymmetricRlweKey::Encrypt(const Polynomial& plaintext,
                                                            const Polynomial& a,
                                                            const Polynomial& e) const {
  for (const Polynomial* q : {&plaintext, &a, &e})
    if (q->NumModuli() != 1 || q->LogN() != key_.LogN())
      return InvalidArgumentError("operands must be polynomials of the key's ring");
  if (!plaintext.IsNttForm() || !a.IsNttForm() || e.IsNttForm())
    return InvalidArgumentError(
        "`plaintext` and `a` must be in NTT form, `e` in coefficient form");
  DeviceArray out((size_t)2 << key_.LogN());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_symmetric_encrypt(
      modulus_->Context()->handle(), out.data(), key_.device_data(), a.device_data(),
      e.device_data(), plaintext.device_data(), 1, g_stream)));
  return SymmetricRlweCiphertext::FromDevice(std::move(out), 2, key_.LogN(), modulus_, 1, 0.0);
}

StatusOr<std::vector<uint64_t>> SymmetricRlweKey::Decrypt(
    const SymmetricRlweCiphertext& ciphertext) const {
  const RnsBgvCiphertext& ct = ciphertext.rns();
  if (ct.LogN() != key_.LogN() || ct.NumModuli() != 1)
    return InvalidArgumentError("ciphertext of another ring");
  DeviceArray out((size_t)1 << key_.LogN());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_symmetric_decrypt(
      modulus_->Context()->handle(), out.data(), key_.device_data(), ct.device_data(),
      ct.Len(), 1, g_stream)));
  std::vector<uint64_t> m((size_t)1 << key_.LogN());
  RLWE_GPU_RETURN_IF_ERROR(out.Download(m.data(), m.size()));
  return m;
}

StatusOr<GaloisKey> GaloisKey::CreateFromKeyComponents(const std::vector<Polynomial>& key_0,
                                                       const std::vector<Polynomial>& key_1,
                                                       int substitution_power, int log_b,
                                                       const PrimeModulus* modulus) {
  if (!modulus) return InvalidArgumentError("`modulus` must not be null.");
  const Moduli moduli{modulus};
  RLWE_GPU_ASSIGN_OR_RETURN(
      RnsGadget gadget,
      RnsGadget::Create(modulus->Context()->LogN(), std::vector<int>{log_b}, moduli));
  RLWE_GPU_ASSIGN_OR_RETURN(
      RnsGaloisKey key, RnsGaloisKey::CreateFromKeyComponents(key_1, key_0, substitution_power,
                                                              &gadget, moduli));
  return GaloisKey(std::move(key));
}

StatusOr<SymmetricRlweCiphertext> GaloisKey::ApplyTo(const SymmetricRlweCiphertext& ct) const {
  // galois_key.h:52-75 -> RelinearizationKey::ApplyTo (relinearization_key.cc:
  // 288-344), power != 1 adds only c0.
  if (ct.PowerOfS() != key_.SubstitutionPower())
    return InvalidArgumentError("Ciphertext PowerOfS: " + std::to_string(ct.PowerOfS()) +
                                " doesn't match the key substitution power: " +
                                std::to_string(key_.SubstitutionPower()));
  RLWE_GPU_ASSIGN_OR_RETURN(RnsBgvCiphertext r, key_.ApplyTo(ct.ct_));
  return SymmetricRlweCiphertext(std::move(r), ct.modulus_);
}

StatusOr<std::unique_ptr<GaloisKeysObliviousExpander>> GaloisKeysObliviousExpander::Create(
    std::vector<GaloisKey> galois_keys, int log_t, const PrimeModulus* modulus) {
  // oblivious_expand.h:237-258
  if (!modulus) return InvalidArgumentError("Parameters are null.");
  const int n = modulus->Context()->NumCoeffs();
  for (size_t i = 0; i < galois_keys.size(); ++i)
    if (galois_keys[i].SubstitutionPower() != (n >> i) + 1)
      return InvalidArgumentError(
          "Substitution power of the i'th GaloisKey must be (N / (2 ^ i)) + 1");
  return std::unique_ptr<GaloisKeysObliviousExpander>(
      new GaloisKeysObliviousExpander(std::move(galois_keys), log_t, modulus));
}

StatusOr<std::vector<SymmetricRlweCiphertext>> GaloisKeysObliviousExpander::ObliviousExpand(
    std::vector<SymmetricRlweCiphertext> ciphertexts, int levels_of_expand,
    int output_length) {
  // oblivious_expand.h:95-138
  if (output_length < 0) return InvalidArgumentError("Output length must be at least 0");
  if (levels_of_expand < 0 || levels_of_expand >= 32)
    return InvalidArgumentError("The number of levels of expansion must fall within [0, 32)");
  if (static_cast<int>(ciphertexts.size()) == output_length) return ciphertexts;
  const int64_t max_length = (int64_t)ciphertexts.size() << levels_of_expand;
  if (output_length > max_length)
    return InvalidArgumentError("Output length must be at most " + std::to_string(max_length));
  if (levels_of_expand > static_cast<int>(keys_.size()))
    return InvalidArgumentError("Not enough Galois keys for the levels of expansion");
  const int log_n = modulus_->Context()->LogN();
  const size_t ct_elems = (size_t)2 << log_n;
  const int count = static_cast<int>(ciphertexts.size());
  DeviceArray in(ct_elems * count);
  for (int i = 0; i < count; ++i) {
    const RnsBgvCiphertext& c = ciphertexts[i].rns();
    if (c.Len() != 2 || c.LogN() != log_n)
      return InvalidArgumentError("ciphertexts must be degree-1 over the expander's ring");
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(
        in.data() + i * ct_elems, c.device_data(), ct_elems * sizeof(uint64_t), g_stream)));
  }
  const size_t per = (size_t)1 << levels_of_expand;
  DeviceArray out(ct_elems * per * count);
  std::vector<const shg_key*> hs;
  for (int j = 0; j < levels_of_expand; ++j) hs.push_back(keys_[j].handle());
  RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_oblivious_expand(
      modulus_->Context()->handle(), hs.data(), levels_of_expand, out.data(), in.data(),
      count, g_stream)));
  std::vector<SymmetricRlweCiphertext> result;
  result.reserve(output_length);
  for (int64_t m = 0; m < output_length; ++m) {
    DeviceArray one(ct_elems);
    RLWE_GPU_RETURN_IF_ERROR(FromCode(shg_memcpy_d2d(one.data(), out.data() + m * ct_elems,
                                                     ct_elems * sizeof(uint64_t), g_stream)));
    result.push_back(SymmetricRlweCiphertext::FromDevice(std::move(one), 2, log_n, modulus_,
                                                         1, 0.0));
  }
  return result;
}

}  // namespace rlwe_gpu
