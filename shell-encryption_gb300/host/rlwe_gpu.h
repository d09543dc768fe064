// C++ host classes over the C ABI of libshellgpu.so (include/shell_gpu.h).
//
// They mirror the names, argument order, value semantics and absl::Status
// behaviour of google/shell-encryption's RNS and single-modulus API for the
// polynomial hot path, so calling code ports by switching its includes and
// namespace:
//
//   rlwe::RnsContext<ModularInt>          -> rlwe_gpu::RnsContext
//   rlwe::PrimeModulus<ModularInt>        -> rlwe_gpu::PrimeModulus
//   rlwe::RnsPolynomial<ModularInt>       -> rlwe_gpu::RnsPolynomial
//   rlwe::RnsGadget<ModularInt>           -> rlwe_gpu::RnsGadget
//   rlwe::RnsRlweCiphertext / RnsBgvCiphertext -> rlwe_gpu::RnsBgvCiphertext
//   rlwe::RnsRelinKey / RnsGaloisKey      -> rlwe_gpu::RnsRelinKey / RnsGaloisKey
//   rlwe::Polynomial, SymmetricRlweCiphertext, GaloisKey,
//   GaloisKeysObliviousExpander           -> same names in rlwe_gpu
//
// Storage is device memory: a polynomial's limbs live in HBM as uint64
// residues in the reference's MontgomeryInt<uint64> representation (x * 2^64
// mod q, canonical), so Coeffs() equals the reference's Coeffs() bit for bit.
// Where the reference passes ModularInt values, these classes take those
// values' Montgomery representations as uint64_t.  Every operation runs CUDA
// kernels of libshellgpu.so; nothing computes on the host.  Operations are
// queued on one stream (SetStream, default the legacy default stream) and
// Coeffs() waits for them.  Keys and ciphertexts arrive as data: sampling,
// encryption and key generation stay with the caller.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <string>
#include <utility>
#include <vector>

#include "shell_gpu.h"
#include "shell_gpu_runtime.h"

namespace rlwe_gpu {

// ---------------------------------------------------------------------------
// absl::Status / absl::StatusOr counterparts (codes are absl::StatusCode).
// ---------------------------------------------------------------------------

enum class StatusCode : int {
  kOk = 0,
  kInvalidArgument = 3,
  kResourceExhausted = 8,
  kFailedPrecondition = 9,
  kInternal = 13,
};

class Status {
 public:
  Status() = default;
  Status(StatusCode code, std::string message)
      : code_(code), message_(std::move(message)) {}
  bool ok() const { return code_ == StatusCode::kOk; }
  StatusCode code() const { return code_; }
  const std::string& message() const { return message_; }
  std::string ToString() const;

 private:
  StatusCode code_ = StatusCode::kOk;
  std::string message_;
};

inline Status OkStatus() { return Status(); }
inline Status InvalidArgumentError(std::string m) {
  return Status(StatusCode::kInvalidArgument, std::move(m));
}
inline Status FailedPreconditionError(std::string m) {
  return Status(StatusCode::kFailedPrecondition, std::move(m));
}
inline Status InternalError(std::string m) {
  return Status(StatusCode::kInternal, std::move(m));
}

template <typename T>
class StatusOr {
 public:
  StatusOr(Status status) : status_(std::move(status)) {  // NOLINT
    if (status_.ok()) status_ = InternalError("StatusOr built from OkStatus");
  }
  StatusOr(T value) : value_(std::move(value)) {}  // NOLINT
  bool ok() const { return status_.ok(); }
  const Status& status() const { return status_; }
  T& value() & { return *value_; }
  const T& value() const& { return *value_; }
  T&& value() && { return std::move(*value_); }
  T& operator*() & { return *value_; }
  const T& operator*() const& { return *value_; }
  T* operator->() { return &*value_; }
  const T* operator->() const { return &*value_; }

 private:
  Status status_;
  std::optional<T> value_;
};

#define RLWE_GPU_CONCAT_INNER_(a, b) a##b
#define RLWE_GPU_CONCAT_(a, b) RLWE_GPU_CONCAT_INNER_(a, b)
#define RLWE_GPU_RETURN_IF_ERROR(expr)            \
  do {                                            \
    ::rlwe_gpu::Status _st = (expr);              \
    if (!_st.ok()) return _st;                    \
  } while (0)
#define RLWE_GPU_ASSIGN_OR_RETURN_IMPL_(tmp, lhs, expr) \
  auto tmp = (expr);                                   \
  if (!tmp.ok()) return tmp.status();                  \
  lhs = std::move(tmp).value()
#define RLWE_GPU_ASSIGN_OR_RETURN(lhs, expr) \
  RLWE_GPU_ASSIGN_OR_RETURN_IMPL_(RLWE_GPU_CONCAT_(_sor_, __LINE__), lhs, expr)

// Stream every class below queues its work on (nullptr = legacy default).
void SetStream(shg_stream stream);
shg_stream GetStream();

// ---------------------------------------------------------------------------
// Device memory with value semantics (copies are device-to-device).
// ---------------------------------------------------------------------------

class DeviceArray {
 public:
  DeviceArray() = default;
  explicit DeviceArray(size_t elems);
  DeviceArray(const DeviceArray& other);
  DeviceArray& operator=(const DeviceArray& other);
  DeviceArray(DeviceArray&& other) noexcept;
  DeviceArray& operator=(DeviceArray&& other) noexcept;
  ~DeviceArray();
  uint64_t* data() const { return ptr_; }
  size_t size() const { return elems_; }
  Status Upload(const uint64_t* host, size_t elems, size_t offset = 0);
  Status Download(uint64_t* host, size_t elems, size_t offset = 0) const;

 private:
  uint64_t* ptr_ = nullptr;
  size_t elems_ = 0;
};

// ---------------------------------------------------------------------------
// RnsContext / PrimeModulus (rns/rns_context.h, rns/rns_modulus.h).
// ---------------------------------------------------------------------------

class RnsContext;

// One prime of a context: rlwe::PrimeModulus's role (ModParams + NttParams),
// here the index of the prime inside its device-resident context.
class PrimeModulus {
 public:
  uint64_t Modulus() const { return q_; }
  int Index() const { return index_; }
  const RnsContext* Context() const { return ctx_; }

 private:
  friend class RnsContext;
  PrimeModulus(const RnsContext* ctx, int index, uint64_t q)
      : ctx_(ctx), index_(index), q_(q) {}
  const RnsContext* ctx_;
  int index_;
  uint64_t q_;
};

using Moduli = std::vector<const PrimeModulus*>;

class RnsContext {
 public:
  // RnsContext::Create(log_n, qs, ps, plaintext_modulus)
  // (rns/rns_context.h:62-72); auxiliary primes `ps` serve the BFV basis
  // extension (RnsBfvCiphertext).
  static StatusOr<std::unique_ptr<const RnsContext>> Create(
      int log_n, std::vector<uint64_t> qs, std::vector<uint64_t> ps,
      uint64_t plaintext_modulus);
  ~RnsContext();
  RnsContext(const RnsContext&) = delete;
  RnsContext& operator=(const RnsContext&) = delete;

  int LogN() const { return log_n_; }
  int NumCoeffs() const { return 1 << log_n_; }
  int NumMainPrimeModuli() const { return static_cast<int>(moduli_.size()); }
  uint64_t PlaintextModulus() const { return t_; }
  Moduli MainPrimeModuli() const;
  int NumAuxPrimeModuli() const { return static_cast<int>(aux_.size()); }
  Moduli AuxPrimeModuli() const;
  // MainPrimeModulusInverseResidues()[level].Prefix(level): Montgomery
  // residues of q_level^{-1} mod q_j, j < level (rns/rns_context.h:145-147),
  // the `ql_inv` argument of ModReduceLsb / ModReduce.
  StatusOr<std::vector<uint64_t>> MainPrimeModulusInverseResidues(int level) const;
  shg_context* handle() const { return h_; }

 private:
  RnsContext() = default;
  shg_context* h_ = nullptr;
  int log_n_ = 0;
  uint64_t t_ = 0;
  std::vector<std::unique_ptr<PrimeModulus>> moduli_;
  std::vector<std::unique_ptr<PrimeModulus>> aux_;
};

// ---------------------------------------------------------------------------
// RnsPolynomial (rns/rns_polynomial.h).
// ---------------------------------------------------------------------------

class RnsPolynomial {
 public:
  // RnsPolynomial::Create(coeff_vectors, is_ntt): Montgomery residues, one
  // vector per prime (rns/rns_polynomial.cc:35-60).
  static StatusOr<RnsPolynomial> Create(std::vector<std::vector<uint64_t>> coeff_vectors,
                                        bool is_ntt);
  // CreateZero (rns/rns_polynomial.cc:63-83).
  static StatusOr<RnsPolynomial> CreateZero(int log_n, const Moduli& moduli,
                                            bool is_ntt = true);
  // Wraps `num_moduli` limbs of n coefficients already on the device.
  static RnsPolynomial FromDevice(DeviceArray data, int log_n, int num_moduli,
                                  bool is_ntt);

  int LogN() const { return log_n_; }
  int NumCoeffs() const { return 1 << log_n_; }
  int NumModuli() const { return num_moduli_; }
  bool IsNttForm() const { return is_ntt_; }
  // Downloads the limbs (waits for queued work).
  std::vector<std::vector<uint64_t>> Coeffs() const;

  Status ConvertToNttForm(const Moduli& moduli);
  Status ConvertToCoeffForm(const Moduli& moduli);

  StatusOr<RnsPolynomial> Negate(const Moduli& moduli) const;
  Status NegateInPlace(const Moduli& moduli);
  StatusOr<RnsPolynomial> Add(const RnsPolynomial& that, const Moduli& moduli) const;
  Status AddInPlace(const RnsPolynomial& that, const Moduli& moduli);
  StatusOr<RnsPolynomial> Sub(const RnsPolynomial& that, const Moduli& moduli) const;
  Status SubInPlace(const RnsPolynomial& that, const Moduli& moduli);
  // Mul / MulInPlace by an integer scalar (rns/rns_polynomial.h:205-227).
  StatusOr<RnsPolynomial> Mul(uint64_t scalar, const Moduli& moduli) const;
  Status MulInPlace(uint64_t scalar, const Moduli& moduli);
  // MulInPlace(Span<const ModularInt> scalar_mod_qs): Montgomery residues of
  // the scalar, one per prime (rns/rns_polynomial.h:236-262).
  Status MulInPlace(const std::vector<uint64_t>& scalar_mod_qs, const Moduli& moduli);
  StatusOr<RnsPolynomial> Mul(const RnsPolynomial& that, const Moduli& moduli) const;
  Status MulInPlace(const RnsPolynomial& that, const Moduli& moduli);
  Status FusedMulAddInPlace(const RnsPolynomial& a, const RnsPolynomial& b,
                            const Moduli& moduli);
  // Substitute(power, moduli) (rns/rns_polynomial.cc:209-260).
  StatusOr<RnsPolynomial> Substitute(int power, const Moduli& moduli) const;
  // ModReduceLsb(t, ql_inv, moduli) (rns/rns_polynomial.cc:262-344).
  Status ModReduceLsb(uint64_t t, const std::vector<uint64_t>& ql_inv,
                      const Moduli& moduli);
  // ModReduceMsb(ql_inv, moduli) (rns/rns_polynomial.cc:349-417).
  Status ModReduceMsb(const std::vector<uint64_t>& ql_inv, const Moduli& moduli);

  uint64_t* device_data() const { return data_.data(); }

 private:
  Status CheckModuli(const Moduli& moduli) const;
  Status CheckThat(const RnsPolynomial& that, const char* name) const;
  DeviceArray data_;
  int log_n_ = 0;
  int num_moduli_ = 0;
  bool is_ntt_ = true;
};

// ---------------------------------------------------------------------------
// RnsGadget (rns/rns_gadget.h).
// ---------------------------------------------------------------------------

class RnsGadget {
 public:
  // RnsGadget::Create(log_n, log_bs, q_hats, q_hat_invs, moduli)
  // (rns/rns_gadget.cc:42-102).  The gadget vector g itself is only needed to
  // generate keys, which stays with the caller, so only the digit structure
  // (log_bs) is kept.
  static StatusOr<RnsGadget> Create(int log_n, std::vector<int> log_bs,
                                    const Moduli& moduli);
  int Dimension() const { return dimension_; }
  // The largest per-limb base exponent (rns/rns_gadget.h:91-94).
  int LogGadgetBase() const;
  const std::vector<int>& LogGadgetBases() const { return log_bs_; }
  // Decompose(a, moduli): k polynomials in coefficient form
  // (rns/rns_gadget.cc:108-153).
  StatusOr<std::vector<RnsPolynomial>> Decompose(const RnsPolynomial& a,
                                                 const Moduli& moduli) const;

 private:
  int log_n_ = 0;
  int dimension_ = 0;
  std::vector<int> log_bs_;
};

// rlwe::RnsErrorParams (rns/rns_error_params.h): the heuristic error bounds
// that RNS ciphertexts carry, as host-side doubles with the reference's
// constants and evaluation order (so Error() values equal the reference's).
// The plaintext-modulus factor is the reference's ExportDoubleT(), the square
// of log_plaintext_modulus.
class RnsErrorParams {
 public:
  // RnsErrorParams::Create(log_n, main_moduli, aux_moduli,
  // log_plaintext_modulus, sigma) (rns/rns_error_params.h:46-82), with the
  // reference's status messages.
  static StatusOr<RnsErrorParams> Create(int log_n, const Moduli& main_moduli,
                                         const Moduli& aux_moduli, int log_plaintext_modulus,
                                         double sigma);
  // The same from the primes themselves (no device context needed).
  static StatusOr<RnsErrorParams> Create(int log_n, const std::vector<uint64_t>& main_qs,
                                         const std::vector<uint64_t>& aux_qs,
                                         int log_plaintext_modulus, double sigma);
  // Error added by a gadget key switch of `num_components` components
  // (rns/rns_error_params.h:84-91).
  double BoundOnGadgetBasedKeySwitching(int num_components, int log_gadget_base,
                                        int num_digits) const;
  double B_plaintext() const { return b_plaintext_; }
  double B_secretkey_encryption() const { return b_secretkey_encryption_; }
  double B_publickey_encryption() const { return b_publickey_encryption_; }
  double B_scale() const { return b_scale_; }

 private:
  RnsErrorParams(int log_n, int log_t, double sigma);
  double T2() const;
  int log_n_ = 0;
  int log_t_ = 0;
  double sigma_ = 0;
  double b_plaintext_ = 0, b_secretkey_encryption_ = 0, b_publickey_encryption_ = 0,
         b_scale_ = 0;
};

// ---------------------------------------------------------------------------
// RnsRlweCiphertext / RnsBgvCiphertext (rns/rns_ciphertext.h,
// rns/rns_bgv_ciphertext.h).  Components are stored contiguously on the
// device ([degree + 1][num_moduli][n]) so batched kernels take them as is.
// ---------------------------------------------------------------------------

class RnsBgvCiphertext {
 public:
  // `error_params` (borrowed, may be null) drives the Error() bookkeeping of
  // the operations below as in the reference; without it Error() changes
  // only under +, -, * and the key switches' additive terms are skipped.
  RnsBgvCiphertext(std::vector<RnsPolynomial> components, Moduli moduli,
                   int power_of_s, double error,
                   const RnsErrorParams* error_params = nullptr);
  static RnsBgvCiphertext FromDevice(DeviceArray data, int num_components, int log_n,
                                     Moduli moduli, int power_of_s, double error,
                                     const RnsErrorParams* error_params = nullptr);

  int Len() const { return len_; }
  int Degree() const { return len_ - 1; }
  int Level() const { return static_cast<int>(moduli_.size()) - 1; }
  int LogN() const { return log_n_; }
  int NumCoeffs() const { return 1 << log_n_; }
  int NumModuli() const { return static_cast<int>(moduli_.size()); }
  int PowerOfS() const { return power_of_s_; }
  double Error() const { return error_; }
  void SetError(double error) { error_ = error; }
  const RnsErrorParams* ErrorParams() const { return error_params_; }
  const Moduli& moduli() const { return moduli_; }
  StatusOr<RnsPolynomial> Component(int index) const;

  Status AddInPlace(const RnsBgvCiphertext& that);
  Status SubInPlace(const RnsBgvCiphertext& that);
  Status NegateInPlace();
  StatusOr<RnsBgvCiphertext> operator+(const RnsBgvCiphertext& that) const;
  StatusOr<RnsBgvCiphertext> operator-(const RnsBgvCiphertext& that) const;
  // AbsorbInPlace(plaintext): every component times an NTT-form plaintext;
  // Error() times B_plaintext (rns/rns_ciphertext.h:208-214).
  Status AbsorbInPlace(const RnsPolynomial& plaintext);
  // AbsorbInPlace(scalar): every component times the integer; Error() times
  // scalar / 2 (rns/rns_ciphertext.h:267-274).
  Status AbsorbInPlace(uint64_t scalar);
  // FusedAbsorbAddInPlace(ctxt, ptxt): this += ctxt * ptxt; Error() plus
  // ctxt.Error() * B_plaintext (rns/rns_ciphertext.h:277-298).
  Status FusedAbsorbAddInPlace(const RnsBgvCiphertext& ctxt, const RnsPolynomial& ptxt);
  StatusOr<RnsBgvCiphertext> operator*(const RnsPolynomial& plaintext) const;
  // RnsRlweCiphertext::Mul (rns/rns_ciphertext.h:501-524).
  StatusOr<RnsBgvCiphertext> operator*(const RnsBgvCiphertext& that) const;
  // ModReduce(t, ql_inv) (rns/rns_bgv_ciphertext.h:141-153).
  Status ModReduce(uint64_t t, const std::vector<uint64_t>& ql_inv);
  // Substitute(power) (rns/rns_bgv_ciphertext.h:155-170).
  StatusOr<RnsBgvCiphertext> Substitute(int substitution_power) const;

  uint64_t* device_data() const { return data_.data(); }
  size_t component_elems() const { return (size_t)moduli_.size() << log_n_; }

 protected:
  RnsBgvCiphertext() = default;
  Status CheckSameShape(const RnsBgvCiphertext& that, bool check_degree) const;
  DeviceArray data_;
  int len_ = 0;
  int log_n_ = 0;
  Moduli moduli_;
  int power_of_s_ = 1;
  double error_ = 0;
  const RnsErrorParams* error_params_ = nullptr;
};
using RnsRlweCiphertext = RnsBgvCiphertext;

// rlwe::RnsBfvCiphertext (rns/rns_bfv_ciphertext.h): an RNS ciphertext whose
// products extend to the context's auxiliary primes.  Addition, subtraction,
// negation and Substitute are the base class's.
class RnsBfvCiphertext : public RnsBgvCiphertext {
 public:
  RnsBfvCiphertext(RnsBgvCiphertext ct, const RnsContext* context)
      : RnsBgvCiphertext(std::move(ct)), context_(context) {}
  // Mul (rns/rns_bfv_ciphertext.cc:100-205).
  StatusOr<RnsBfvCiphertext> operator*(const RnsBfvCiphertext& that) const;
  // AbsorbInPlace(plaintext) (rns/rns_bfv_ciphertext.cc:33-98).
  Status AbsorbInPlace(const RnsPolynomial& plaintext);
  // ModReduce() (rns/rns_bfv_ciphertext.h:184-200): ModReduceMsb of every
  // component with MainPrimeModulusInverseResidues()[level].
  Status ModReduce();
  const RnsContext* Context() const { return context_; }

 private:
  const RnsContext* context_;
};

// Gadget key for relinearization (power 1) or a Galois automorphism, held on
// the device in the layout the key-switch kernels read.
class RnsRelinKey {
 public:
  // Builds the key from its components: key_bs[j], key_as[j] in NTT form
  // (the reference's GetKeyB() / GetKeyA(), rns/rns_relinearization_key.h:
  // 99-104), for degree-2 ciphertexts.
  static StatusOr<RnsRelinKey> CreateFromKeyComponents(
      const std::vector<RnsPolynomial>& key_bs, const std::vector<RnsPolynomial>& key_as,
      const RnsGadget* gadget, Moduli moduli);
  // ApplyTo (rns/rns_relinearization_key.h:82-92, .cc:184-232).
  StatusOr<RnsBgvCiphertext> ApplyTo(const RnsBgvCiphertext& ciphertext) const;
  int Dimension() const;
  shg_key* handle() const { return key_.get(); }

 private:
  std::shared_ptr<shg_key> key_;
  Moduli moduli_;
};

class RnsGaloisKey {
 public:
  // CreateFromKeyComponents(key_as, key_bs, power, gadget, moduli)
  // (rns/rns_galois_key.cc:183-202).
  static StatusOr<RnsGaloisKey> CreateFromKeyComponents(
      const std::vector<RnsPolynomial>& key_as, const std::vector<RnsPolynomial>& key_bs,
      int power, const RnsGadget* gadget, Moduli moduli);
  // ApplyTo on a ciphertext whose power of s equals the key's
  // (rns/rns_galois_key.h:146-156, .cc:238-287).
  StatusOr<RnsBgvCiphertext> ApplyTo(const RnsBgvCiphertext& ciphertext) const;
  // PrecomputeRandomPad(ciphertext_pad_digits) (rns/rns_galois_key.cc:
  // 289-306): the key-switched "a" part from the NTT-form gadget digits of a
  // ciphertext's c1.
  StatusOr<RnsPolynomial> PrecomputeRandomPad(
      const std::vector<RnsPolynomial>& ciphertext_pad_digits) const;
  // ApplyToWithRandomPad(ciphertext, pad digits, pad_new)
  // (rns/rns_galois_key.h:177-192).
  StatusOr<RnsBgvCiphertext> ApplyToWithRandomPad(
      const RnsBgvCiphertext& ciphertext,
      const std::vector<RnsPolynomial>& ciphertext_pad_digits,
      const RnsPolynomial& ciphertext_pad_new) const;
  // Compose(other_key) (rns/rns_galois_key.cc:349-406): the key for the
  // product of the two substitution powers.
  StatusOr<RnsGaloisKey> Compose(const RnsGaloisKey& other_key) const;
  int SubstitutionPower() const { return power_; }
  int Dimension() const;
  shg_key* handle() const { return key_.get(); }

 private:
  StatusOr<DeviceArray> PackDigits(const std::vector<RnsPolynomial>& digits) const;
  std::shared_ptr<shg_key> key_;
  Moduli moduli_;
  int power_ = 1;
};

// ---------------------------------------------------------------------------
// Single-modulus counterparts (polynomial.h, symmetric_encryption.h,
// galois_key.h, oblivious_expand.h): a one-prime RnsContext.
// ---------------------------------------------------------------------------

// rlwe::Polynomial<ModularInt> over one prime.
using Polynomial = RnsPolynomial;

class SymmetricRlweCiphertext {
 public:
  SymmetricRlweCiphertext(std::vector<Polynomial> components, const PrimeModulus* modulus,
                          int power_of_s, double error);
  static SymmetricRlweCiphertext FromDevice(DeviceArray data, int num_components,
                                            int log_n, const PrimeModulus* modulus,
                                            int power_of_s, double error);
  int Len() const { return ct_.Len(); }
  int PowerOfS() const { return ct_.PowerOfS(); }
  int LogN() const { return ct_.LogN(); }
  StatusOr<Polynomial> Component(int index) const { return ct_.Component(index); }
  StatusOr<SymmetricRlweCiphertext> operator+(const SymmetricRlweCiphertext& that) const;
  StatusOr<SymmetricRlweCiphertext> operator-(const SymmetricRlweCiphertext& that) const;
  StatusOr<SymmetricRlweCiphertext> operator*(const SymmetricRlweCiphertext& that) const;
  Status AbsorbInPlace(const Polynomial& plaintext);
  StatusOr<SymmetricRlweCiphertext> Substitute(int substitution_power) const;
  const RnsBgvCiphertext& rns() const { return ct_; }
  const PrimeModulus* modulus() const { return modulus_; }

 private:
  friend class GaloisKey;
  friend class GaloisKeysObliviousExpander;
  explicit SymmetricRlweCiphertext(RnsBgvCiphertext ct, const PrimeModulus* m)
      : ct_(std::move(ct)), modulus_(m) {}
  RnsBgvCiphertext ct_;
  const PrimeModulus* modulus_;
};

// rlwe::RnsRlweSecretKey (rns/rns_secret_key.h): the secret key s in NTT form
// over `moduli` and the error variance.  Key sampling stays with the caller;
// encryption draws its randomness on the device from SHELL's ChaCha PRNG.
class RnsRlweSecretKey {
 public:
  // `key` in NTT form with one limb per modulus; 1 <= variance <= 256.
  static StatusOr<RnsRlweSecretKey> CreateFromKey(RnsPolynomial key, Moduli moduli,
                                                  int variance);
  // EncryptPolynomialBgv(plaintext, encoder, error_params, prng)
  // (rns/rns_secret_key.h:188-231) with prng = SingleThreadChaChaPrng::Create
  // (prng_seed) (32 bytes) and t the context's plaintext modulus; the result
  // carries `error_bound` (error_params->B_secretkey_encryption()).
  StatusOr<RnsBgvCiphertext> EncryptPolynomialBgv(const RnsPolynomial& plaintext,
                                                  const std::string& prng_seed,
                                                  double error_bound = 0) const;
  // The same for a batch: plaintext i with prng_seeds[i], one launch set.
  StatusOr<std::vector<RnsBgvCiphertext>> EncryptPolynomialBgv(
      const std::vector<RnsPolynomial>& plaintexts, const std::vector<std::string>& prng_seeds,
      double error_bound = 0) const;
  const RnsPolynomial& Key() const { return key_; }
  const Moduli& moduli() const { return moduli_; }
  int Variance() const { return variance_; }

 private:
  RnsRlweSecretKey(RnsPolynomial key, Moduli moduli, int variance)
      : key_(std::move(key)), moduli_(std::move(moduli)), variance_(variance) {}
  RnsPolynomial key_;
  Moduli moduli_;
  int variance_;
};

// rlwe::SymmetricRlweKey over a one-prime context: the key polynomial s (NTT
// form) and the context's plaintext modulus t (SymmetricRlweKey::Sample's
// t = 2^log_t + 1 when the context was created with it).
class SymmetricRlweKey {
 public:
  static StatusOr<SymmetricRlweKey> Create(Polynomial key, const PrimeModulus* modulus);
  // rlwe::Encrypt with the randomness injected as in internal::Encrypt
  // (symmetric_encryption.h:940-963, 1006-1021): `a` uniform (NTT form), `e`
  // error samples (coefficient form), `plaintext` in NTT form.
  StatusOr<SymmetricRlweCiphertext> Encrypt(const Polynomial& plaintext, const Polynomial& a,
                                            const Polynomial& e) const;
  // rlwe::Decrypt (symmetric_encryption.h:1138-1152): message coefficients
  // in [0, t).
  StatusOr<std::vector<uint64_t>> Decrypt(const SymmetricRlweCiphertext& ciphertext) const;
  const Polynomial& Key() const { return key_; }

 private:
  SymmetricRlweKey(Polynomial key, const PrimeModulus* m) : key_(std::move(key)), modulus_(m) {}
  Polynomial key_;
  const PrimeModulus* modulus_;
};

// rlwe::GaloisKey: a single-modulus key-switching key for X -> X^power with
// gadget base 2^log_b; key_0[i], key_1[i] are the rows of the key part
// (relinearization_key.cc:99-141) in NTT form.
class GaloisKey {
 public:
  static StatusOr<GaloisKey> CreateFromKeyComponents(const std::vector<Polynomial>& key_0,
                                                     const std::vector<Polynomial>& key_1,
                                                     int substitution_power, int log_b,
                                                     const PrimeModulus* modulus);
  // ApplyTo(ciphertext) (galois_key.h:52-75): ciphertext already substituted
  // to the key's power.
  StatusOr<SymmetricRlweCiphertext> ApplyTo(const SymmetricRlweCiphertext& ct) const;
  int SubstitutionPower() const { return key_.SubstitutionPower(); }
  shg_key* handle() const { return key_.handle(); }

 private:
  explicit GaloisKey(RnsGaloisKey key) : key_(std::move(key)) {}
  RnsGaloisKey key_;
};

// GaloisKeysObliviousExpander (oblivious_expand.h:233-291): key i has
// substitution power n / 2^i + 1.
class GaloisKeysObliviousExpander {
 public:
  static StatusOr<std::unique_ptr<GaloisKeysObliviousExpander>> Create(
      std::vector<GaloisKey> galois_keys, int log_t, const PrimeModulus* modulus);
  // ObliviousExpand(ciphertexts, levels_of_expand, output_length)
  // (oblivious_expand.h:95-138).
  StatusOr<std::vector<SymmetricRlweCiphertext>> ObliviousExpand(
      std::vector<SymmetricRlweCiphertext> ciphertexts, int levels_of_expand,
      int output_length);

 private:
  GaloisKeysObliviousExpander(std::vector<GaloisKey> keys, int log_t,
                              const PrimeModulus* modulus)
      : keys_(std::move(keys)), log_t_(log_t), modulus_(modulus) {}
  std::vector<GaloisKey> keys_;
  int log_t_;
  const PrimeModulus* modulus_;
};

}  // namespace rlwe_gpu
