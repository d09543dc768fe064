/*
 * shell_gpu.h — C ABI of the GB300 RLWE polynomial hot path.
 *
 * A drop-in device backend for google/shell-encryption's RNS polynomial,
 * ciphertext and key-switching calls.  Every entry point takes plain pointers
 * and sizes; polynomial data are DEVICE pointers to uint64 residues in SHELL's
 * MontgomeryInt<uint64> representation (x * 2^64 mod q), laid out as
 *
 *   poly        [num_limbs][n]                 limb l is modulo q_l
 *   ciphertext  [num_components][num_limbs][n]
 *   batches     [count][...]                   contiguous
 *
 * so results compare bit-for-bit (memcmp) with the reference's
 * RnsPolynomial::Coeffs() / Polynomial::Coeffs().  Calls are asynchronous on
 * the given stream (0 = legacy default stream); argument validation happens
 * on the host before any launch and mirrors the reference's absl::Status
 * checks.  Return values are absl::StatusCode numbers (0 = OK,
 * 3 = INVALID_ARGUMENT, 9 = FAILED_PRECONDITION, 8 = RESOURCE_EXHAUSTED,
 * 13 = INTERNAL); shg_last_error() returns the message of the calling
 * thread's last failure.  Batched calls of one context share its device
 * scratch: issue them on one stream, or order their streams with events.
 *
 * Reference interfaces cited below are paths inside google/shell-encryption.
 */
#ifndef SHELL_GPU_H_
#define SHELL_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shg_context shg_context;  /* RNS context resident on the GPU */
typedef struct shg_key shg_key;          /* gadget key-switching key */
typedef void* shg_stream;                /* a cudaStream_t */

enum {
  SHG_OK = 0,
  SHG_INVALID_ARGUMENT = 3,
  SHG_RESOURCE_EXHAUSTED = 8,
  SHG_FAILED_PRECONDITION = 9,
  SHG_INTERNAL = 13,
};

/* Message of this thread's most recent failed call ("" if none). */
const char* shg_last_error(void);

/* ---------------------------------------------------------------------------
 * Context
 * ------------------------------------------------------------------------- */

/* RnsContext<MontgomeryInt<uint64>>::Create(log_n, qs, {}, t)
 * (shell_encryption/rns/rns_context.h:62-72, rns/rns_context.cc:22-76):
 * validates every prime like MontgomeryIntParams::Create (montgomery.cc:44-59)
 * and InitializeNttParameters (ntt_parameters.h:183-235), derives psi with the
 * reference's smallest-t search and uploads twiddle and CRT tables. */
int shg_context_create(int log_n, const uint64_t* qs, int num_qs,
                       uint64_t plaintext_modulus, shg_context** out);
/* RnsContext::Create(log_n, qs, ps, t) with auxiliary primes ps (the BFV
 * basis extension, rns/rns_context.cc:22-76): main limbs are q_0..q_{L-1};
 * the auxiliary primes get their own NTT tables and the CRT constants of
 * GenerateCrtConstantsForAuxModulus (:317-377).  Every prime is validated
 * as in shg_context_create, and all must be distinct. */
int shg_context_create_with_aux(int log_n, const uint64_t* qs, int num_qs, const uint64_t* ps,
                                int num_ps, uint64_t plaintext_modulus, shg_context** out);
int shg_context_num_aux_moduli(const shg_context* ctx);
void shg_context_destroy(shg_context* ctx);
int shg_context_log_n(const shg_context* ctx);
int shg_context_num_moduli(const shg_context* ctx);

/* Host copy of limb i's Montgomery parameters (montgomery.h:77-202):
 * out[0..9] = q, log_q, inv_modulus, r_mod_q, r_mod_q_barrett, inv_r,
 * inv_r_barrett, barrett_numerator, psi (plain), n_inv (Montgomery). */
int shg_context_prime_info(const shg_context* ctx, int i, uint64_t out[10]);
/* Host copies of NttParameters::psis_bitrev / psis_inv_bitrev for limb i
 * (Montgomery reps, n each) (ntt_parameters.h:117-157). */
int shg_context_ntt_tables(const shg_context* ctx, int i, uint64_t* psis_bitrev,
                           uint64_t* psis_inv_bitrev);
/* MainPrimeModulusInverseResidues()[level].Prefix(level): q_level^{-1} mod q_j
 * for j < level, Montgomery reps (rns/rns_context.h:145-147). */
int shg_context_ql_inv(const shg_context* ctx, int level, uint64_t* out);

/* ---------------------------------------------------------------------------
 * RnsPolynomial operations.  `polys` hold `count` polynomials of `num_limbs`
 * limbs each (limb l modulo q_l, num_limbs <= num_moduli).
 * ------------------------------------------------------------------------- */

/* RnsPolynomial::ConvertToNttForm (rns/rns_polynomial.cc:171-188) /
 * ForwardNumberTheoreticTransform (dft_transformations.h:158-176). In place. */
int shg_ntt_forward(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                    shg_stream stream);
/* RnsPolynomial::ConvertToCoeffForm (rns/rns_polynomial.cc:190-207) /
 * InverseNumberTheoreticTransform (dft_transformations.h:181-201). In place. */
int shg_ntt_inverse(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                    shg_stream stream);

/* RnsPolynomial::Add / Sub / Negate / Mul(poly) / FusedMulAddInPlace
 * (rns/rns_polynomial.h:150-365) -> MontgomeryInt Batch* ops
 * (montgomery.cc:229-440).  out may alias an input.  fma: acc += a * b. */
int shg_poly_add(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream stream);
int shg_poly_sub(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream stream);
int shg_poly_neg(shg_context* ctx, uint64_t* out, const uint64_t* a, int count,
                 int num_limbs, shg_stream stream);
int shg_poly_mul(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream stream);
int shg_poly_fma(shg_context* ctx, uint64_t* acc, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream stream);
/* RnsPolynomial::MulInPlace(RnsInt / Span<ModularInt>) with a per-limb
 * Montgomery-form scalar (host array, num_limbs entries)
 * (rns/rns_polynomial.h:236-262). */
int shg_poly_mul_rns_scalar(shg_context* ctx, uint64_t* out, const uint64_t* a,
                            const uint64_t* scalar_mont, int count,
                            int num_limbs, shg_stream stream);
/* RnsPolynomial::MulInPlace(Integer scalar) (rns/rns_polynomial.h:214-227). */
int shg_poly_mul_integer(shg_context* ctx, uint64_t* out, const uint64_t* a,
                         uint64_t scalar, int count, int num_limbs,
                         shg_stream stream);
/* RnsPolynomial::Substitute (rns/rns_polynomial.cc:209-260); NTT form; out
 * must not alias in. */
int shg_poly_substitute(shg_context* ctx, uint64_t* out, const uint64_t* in,
                        int power, int count, int num_limbs, shg_stream stream);
/* RnsPolynomial::ModReduceLsb (rns/rns_polynomial.cc:262-344): in
 * [count][num_limbs][n] -> out [count][num_limbs-1][n]; ql_inv holds the
 * num_limbs-1 Montgomery residues of q_{num_limbs-1}^{-1} (host array);
 * is_ntt selects the input form. */
int shg_poly_modreduce_lsb(shg_context* ctx, uint64_t* out, const uint64_t* in,
                           uint64_t t, const uint64_t* ql_inv, int is_ntt,
                           int count, int num_limbs, shg_stream stream);

/* RnsGadget::Decompose (rns/rns_gadget.cc:108-153) with the gadget of
 * log_bs[num_limbs] (rns/rns_gadget.cc:42-102): in [count][num_limbs][n]
 * (coefficient form) -> out [count][k][num_limbs][n] (coefficient form),
 * k = sum_i GadgetSize(log q_i, log_bs[i]) (gadget.h:43-47).  out must not
 * alias in. */
int shg_gadget_decompose(shg_context* ctx, int num_limbs, const int* log_bs,
                         uint64_t* out, const uint64_t* in, int count,
                         shg_stream stream);

/* Wire format: RnsPolynomial::Serialize / Deserialize (rns/rns_polynomial.h:
 * 99-140) limb by limb, each limb MontgomeryInt::SerializeVector /
 * DeserializeVector (montgomery.cc:142-215): the n Montgomery residues as a
 * little-endian bit stream of log q_l bits each (value i at stream bits
 * [i*b, i*b + b), bit j in byte j/8 at position j%8), ceil(n*b/8) bytes.
 * A serialized polynomial is its limbs' streams back to back
 * (shg_poly_serialized_bytes bytes); batches are polynomials back to back.
 * Device buffers; for n >= 64 the serialized buffer must be 8-byte aligned.
 * Deserialization, like the reference's, does not range-check values. */
size_t shg_poly_serialized_bytes(const shg_context* ctx, int num_limbs);
int shg_poly_serialize(shg_context* ctx, uint8_t* out, const uint64_t* polys,
                       int count, int num_limbs, shg_stream stream);
int shg_poly_deserialize(shg_context* ctx, uint64_t* polys, const uint8_t* in,
                         int count, int num_limbs, shg_stream stream);

/* ---------------------------------------------------------------------------
 * Ciphertexts
 * ------------------------------------------------------------------------- */

/* RnsRlweCiphertext::Mul / RnsBgvCiphertext::operator* for degree-1 inputs
 * (rns/rns_ciphertext.h:501-524, rns/rns_bgv_ciphertext.h:134-139):
 * a, b [count][2][L][n] -> out [count][3][L][n]. */
int shg_ct_tensor(shg_context* ctx, uint64_t* out, const uint64_t* a,
                  const uint64_t* b, int count, int num_limbs,
                  shg_stream stream);

/* ---------------------------------------------------------------------------
 * Gadget key switching (relinearization and Galois keys)
 * ------------------------------------------------------------------------- */

/* Uploads a gadget key: key_b, key_a [k][num_limbs][n] host or device arrays in NTT
 * form (Montgomery reps) with the RnsGadget of log_bs[num_limbs]
 * (rns/rns_gadget.cc:42-102).  `power` is the key's substitution power: 1
 * for an RnsRelinKey (GetKeyB/GetKeyA, rns/rns_relinearization_key.h:99-104),
 * the Galois power for an RnsGaloisKey (CreateFromKeyComponents,
 * rns/rns_galois_key.cc:183-202).  A single-modulus RelinearizationKey /
 * GaloisKey part is the num_limbs == 1 case (relinearization_key.cc:99-141;
 * galois_key.h:43-111). */
int shg_key_create(shg_context* ctx, int num_limbs, const int* log_bs,
                   int power, const uint64_t* key_b, const uint64_t* key_a,
                   shg_key** out);
void shg_key_destroy(shg_key* key);
int shg_key_dimension(const shg_key* key);
/* Number of limbs, substitution power (1 = relinearization key) and owning
 * context of a key. */
int shg_key_num_limbs(const shg_key* key);
/* The key's gadget base exponents (num_limbs entries into log_bs[max]). */
int shg_key_log_bs(const shg_key* key, int* log_bs, int max);
int shg_key_power(const shg_key* key);
shg_context* shg_key_context(const shg_key* key);
/* Device bytes held by the key. */
size_t shg_key_device_bytes(const shg_key* key);

/* RnsRelinKey::ApplyTo for degree-2 ciphertexts
 * (rns/rns_relinearization_key.h:82-92, .cc:184-232):
 * ct [count][3][L][n] (NTT) -> out [count][2][L][n].  out may not alias ct. */
int shg_relin_apply(shg_context* ctx, const shg_key* key, uint64_t* out,
                    const uint64_t* ct, int count, shg_stream stream);
/* Allocation-free variant of shg_relin_apply; it has no counterpart in the
 * reference.  It is for callers that may not allocate device memory during a
 * call (memory handed out by an external pool or arena, a device budget owned
 * by another component, or a latency-critical path where an allocation's
 * implicit synchronization would stall other streams).  Its scratch is a
 * fixed 32 MiB array inside the library's device image (held on every GPU
 * that loads the library until the process exits); the call allocates and
 * frees nothing.  Inputs, outputs and results are those of shg_relin_apply.
 * Limit: one ciphertext's scratch, n * num_limbs * (1 + gadget dimension) * 8
 * bytes, must fit in 32 MiB (n = 2^14 with 6 limbs and dimension 18 needs
 * 14.9 MiB); larger shapes return SHG_INVALID_ARGUMENT.  Batches larger than
 * the scratch are processed in chunks.  The first call on each device looks
 * up the array's device address (with that device current) and should come
 * before any stream capture; that first call may also be what loads the
 * library's device image (the 32 MiB array included) onto the device, so
 * make one warm-up call before entering a region where nothing may
 * allocate.  The looked-up address is kept for the life of the process and
 * is valid only until the device is reset (cudaDeviceReset, or the primary
 * context torn down and created again); do not call this entry point after
 * such a reset.  With the library's per-kernel profiling switched on
 * (shg_profile_start) every launch creates CUDA events.  All calls on a
 * device share the one array, so calls whose work overlaps on the GPU
 * (different streams, or host threads) race: serialize them on one stream. */
int shg_relin_apply_noalloc(shg_context* ctx, const shg_key* key, uint64_t* out,
                            const uint64_t* ct, int count, shg_stream stream);

/* RnsGaloisKey::ApplyTo (rns/rns_galois_key.h:146-156, .cc:238-287) on
 * ciphertexts already substituted to the key's power: ct [count][2][L][n]
 * -> out [count][2][L][n]. */
int shg_galois_apply(shg_context* ctx, const shg_key* key, uint64_t* out,
                     const uint64_t* ct, int count, shg_stream stream);

/* The key's rows key_b, key_a [k][L][n] as given to shg_key_create (the
 * reference's GetKeyB / GetKeyA, rns/rns_galois_key.h:152-158), into host or
 * device memory. */
int shg_key_components(const shg_key* key, uint64_t* key_b, uint64_t* key_a);

/* RnsGaloisKey::Compose (rns/rns_galois_key.h:214, .cc:349-406): the key for
 * X -> X^(power * other.power) from `key` and `other` (same moduli and
 * gadget dimension): each row (b_i, a_i) of `other`, substituted by key's
 * power and key-switched with `key`.  *out is a new key with other's gadget.
 * CreatePadOfComposedKey (.cc:408-434) is shg_galois_precompute_pad with the
 * first key and the second key's a-row digits; ComposeWithPads (.cc:436-471)
 * is shg_poly_substitute of the b rows followed by shg_galois_apply_with_pad. */
int shg_galois_key_compose(shg_context* ctx, const shg_key* key, const shg_key* other,
                           shg_key** out);

/* RnsGaloisKey::PrecomputeRandomPad (rns/rns_galois_key.h:170-175,
 * .cc:289-306): pad_digits [count][k][L][n] = the gadget digits of each
 * ciphertext's "a" part (c1) in NTT form -> out [count][L][n] =
 * sum_j pad_j * key_a_j, the key-switched "a" part. */
int shg_galois_precompute_pad(shg_context* ctx, const shg_key* galois_key,
                              uint64_t* out, const uint64_t* pad_digits, int count,
                              shg_stream stream);
/* RnsGaloisKey::ApplyToWithRandomPad (rns/rns_galois_key.h:177-192,
 * .cc:308-346): ct [count][2][L][n] at the key's power, its c1 digits
 * pad_digits and the precomputed pad_new [count][L][n] -> out
 * [count][2][L][n] = (c0 + sum_j pad_j * key_b_j, pad_new). */
int shg_galois_apply_with_pad(shg_context* ctx, const shg_key* galois_key,
                              uint64_t* out, const uint64_t* ct,
                              const uint64_t* pad_digits, const uint64_t* pad_new,
                              int count, shg_stream stream);

/* Batched fused form of RnsBgvCiphertext::operator* followed by
 * RnsRelinKey::ApplyTo (rns/rns_bgv_ciphertext.h:134-139 +
 * rns/rns_relinearization_key.cc:184-232): a, b [count][2][L][n] ->
 * out [count][2][L][n], bit-identical to calling both per ciphertext. */
int shg_bgv_mul_relin(shg_context* ctx, const shg_key* relin_key, uint64_t* out,
                      const uint64_t* a, const uint64_t* b, int count,
                      shg_stream stream);
/* Batches whose members bring their own keys (different clients): member i
 * of shg_bgv_mul_relin_multikey / shg_bgv_rotate_multikey uses keys[i], and
 * query q of shg_pir_expand_absorb_multikey uses keys[q * levels + j] at
 * level j.  All keys of one call share the context, limbs, gadget and
 * substitution power (per level for the expansion); results equal one call
 * per key.  The key tables are staged from host memory, so these calls are
 * not for stream capture. */
int shg_bgv_mul_relin_multikey(shg_context* ctx, const shg_key* const* relin_keys,
                               uint64_t* out, const uint64_t* a, const uint64_t* b,
                               int count, shg_stream stream);
int shg_bgv_rotate_multikey(shg_context* ctx, const shg_key* const* galois_keys,
                            uint64_t* out, const uint64_t* ct, int count,
                            shg_stream stream);
int shg_pir_expand_absorb_multikey(shg_context* ctx, const shg_key* const* keys,
                                   int levels, const uint64_t* db, int num_items,
                                   uint64_t* out, const uint64_t* ct, int count,
                                   shg_stream stream);

/* shg_bgv_mul_relin on HOST buffers (a, b, out in host memory, page-locked
 * for full speed): the batch is split into pieces whose host->device copies
 * (a and b on two streams), ct-mult+relin and device->host copy run on four
 * streams through a ring of device staging slots, so transfers overlap
 * computation (shape: shg_context_set_host_pipeline).  Ordered after prior work on `stream`; `stream` is
 * ordered after the last copy back (synchronize it before reading out). */
int shg_bgv_mul_relin_host(shg_context* ctx, const shg_key* relin_key,
                           uint64_t* out, const uint64_t* a, const uint64_t* b,
                           int count, shg_stream stream);
/* shg_bgv_mul_relin_host on serialized ciphertexts (the wire format above:
 * each ciphertext is its two polynomials' streams, 2 *
 * shg_poly_serialized_bytes(ctx, L) bytes, ciphertexts back to back in host
 * memory): the packed bytes cross the host link and are deserialized and
 * re-serialized on the device.  n >= 64. */
int shg_bgv_mul_relin_host_serialized(shg_context* ctx, const shg_key* relin_key,
                                      uint8_t* out, const uint8_t* a, const uint8_t* b,
                                      int count, shg_stream stream);

/* RnsBgvCiphertext::Substitute(power) then RnsGaloisKey::ApplyTo
 * (rns/rns_bgv_ciphertext.h:161-174): ct [count][2][L][n] -> out. */
int shg_bgv_rotate(shg_context* ctx, const shg_key* galois_key, uint64_t* out,
                   const uint64_t* ct, int count, shg_stream stream);

/* ---------------------------------------------------------------------------
 * RNS basis conversion and BFV, on a context with auxiliary primes.
 * `num_limbs` main limbs q_0..q_{num_limbs-1} (the ciphertext's level + 1)
 * and all K auxiliary primes p_0..p_{K-1}; main polys [count][num_limbs][n],
 * auxiliary polys [count][K][n].  The reference evaluates round(sum_i v_i /
 * q_i) in double precision inside SwitchRnsBasis; the kernels reproduce that
 * value exactly.
 * ------------------------------------------------------------------------- */

/* RnsPolynomial::SwitchRnsBasis (rns/rns_polynomial.cc:419-525), coefficient
 * form in and out: direction 0 main -> aux with the tables of
 * MainPrimeModulusCrtFactors / MainPrimeModulusComplementResidues /
 * MainLeveledModulusAuxResidues(level), direction 1 aux -> main with
 * AuxPrimeModulusCrtFactors / AuxPrimeModulusComplementResidues /
 * AuxModulusResidues (rns/rns_context.h:142-200). */
int shg_poly_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                              int direction, int num_limbs, int count, shg_stream stream);
/* ScaleAndSwitchRnsBasis main -> aux (rns/rns_polynomial.cc:527-640):
 * round(P/Q a) mod P, coefficient form. */
int shg_poly_scale_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                                    int num_limbs, int count, shg_stream stream);
/* ApproxSwitchRnsBasis (rns/rns_polynomial.cc:653-724): input in NTT form when
 * is_ntt, output coefficient form; balanced: ConvertModulusBalanced. */
int shg_poly_approx_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                                     int direction, int num_limbs, int is_ntt, int balanced,
                                     int count, shg_stream stream);
/* RnsPolynomial::ModReduceMsb (rns/rns_polynomial.cc:349-417): in
 * [count][num_limbs][n] -> out [count][num_limbs-1][n] = round(a / q_l),
 * ql_inv as for shg_poly_modreduce_lsb.  Works on any context. */
int shg_poly_modreduce_msb(shg_context* ctx, uint64_t* out, const uint64_t* in,
                           const uint64_t* ql_inv, int is_ntt, int count, int num_limbs,
                           shg_stream stream);
/* ScaleAndReduceRnsBasisInPlace (rns/rns_polynomial.h:458-490): (main mod Q,
 * aux mod P) -> out = (t main - SwitchRnsBasis(t aux)) / P mod Q, in main's
 * form. */
int shg_poly_scale_reduce_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* main,
                                    const uint64_t* aux, uint64_t t, int is_ntt_main,
                                    int is_ntt_aux, int num_limbs, int count,
                                    shg_stream stream);
/* ApproxModReduceLsb (lsb = 1, rns/rns_polynomial.cc:726-791) or
 * ApproxModReduceMsb (lsb = 0, :793-852) of (main mod Q, aux mod P): out
 * [count][num_limbs][n] in NTT form. */
int shg_poly_approx_modreduce(shg_context* ctx, uint64_t* out, const uint64_t* main,
                              const uint64_t* aux, int lsb, uint64_t t, int is_ntt_main,
                              int is_ntt_aux, int num_limbs, int count, shg_stream stream);
/* RnsBfvCiphertext::operator* (Mul, rns/rns_bfv_ciphertext.cc:100-205) for
 * `count` pairs: a, b [count][2][num_limbs][n] (NTT form) -> out
 * [count][3][num_limbs][n]; t = the context's plaintext modulus. */
int shg_bfv_mul(shg_context* ctx, uint64_t* out, const uint64_t* a, const uint64_t* b,
                int count, int num_limbs, shg_stream stream);
/* RnsBfvCiphertext::AbsorbInPlace (rns/rns_bfv_ciphertext.cc:33-98):
 * ct [count][len][num_limbs][n] times the NTT-form plaintext [num_limbs][n]
 * -> out (same shape). */
int shg_bfv_absorb(shg_context* ctx, uint64_t* out, const uint64_t* ct,
                   const uint64_t* plaintext, int len, int count, int num_limbs,
                   shg_stream stream);

/* ---------------------------------------------------------------------------
 * Encryption randomness from SHELL's ChaCha PRNG, sampled on the device.
 * Ciphertext c uses the stream of SingleThreadChaChaPrng::Create(seed)
 * (prng/single_thread_chacha_prng.h:35-80, prng/chacha_prng_util.cc:30-98)
 * with seed = seeds[32c .. 32c+31] (device bytes), so results equal the
 * reference's for the same seeds.
 * ------------------------------------------------------------------------- */

/* RnsPolynomial::SampleUniform (rns/rns_polynomial.h:74-77, 638-667) then
 * SampleError (rns/error_distribution.h:40-60) from one stream per seed:
 * a, e [count][num_limbs][n], both NTT form.  1 <= variance <= 256. */
int shg_sample_uniform_error(shg_context* ctx, uint64_t* a, uint64_t* e,
                             const uint8_t* seeds, int num_limbs, int count, int variance,
                             shg_stream stream);

/* RnsRlweSecretKey::EncryptPolynomialBgv (rns/rns_secret_key.h:70-74,
 * 188-231) for `count` plaintexts, the PRNG of ciphertext c seeded with
 * seeds[c]: key s [num_limbs][n], plaintexts m [count][num_limbs][n] (NTT
 * form) -> out [count][2][num_limbs][n] = (e * t + m + a * s, -a) with a, e
 * as shg_sample_uniform_error draws them and t the context's plaintext
 * modulus.  1 <= variance <= 256. */
int shg_bgv_encrypt(shg_context* ctx, uint64_t* out, const uint64_t* key,
                    const uint64_t* plaintexts, const uint8_t* seeds, int num_limbs,
                    int count, int variance, shg_stream stream);

/* ---------------------------------------------------------------------------
 * Single-modulus symmetric RLWE, on a one-prime context (t = the context's
 * plaintext modulus)
 * ------------------------------------------------------------------------- */

/* Encrypt (symmetric_encryption.h:1006-1021) with the randomness injected as
 * in internal::Encrypt (symmetric_encryption.h:940-963): key s [n] (NTT
 * form), a [count][n] (uniform, NTT form), e [count][n] (error samples,
 * coefficient form), m [count][n] (plaintexts, NTT form), all Montgomery ->
 * out [count][2][n] = (NTT(e) * t + m + a * s, -a).  Sampling stays with the
 * caller. */
int shg_symmetric_encrypt(shg_context* ctx, uint64_t* out, const uint64_t* s,
                          const uint64_t* a, const uint64_t* e, const uint64_t* m,
                          int count, shg_stream stream);
/* Decrypt (symmetric_encryption.h:1138-1152: ExtractErrorAndMessage then
 * RemoveError): ct [count][len][n] (NTT form) -> out [count][n] plaintext
 * integers in [0, t). */
int shg_symmetric_decrypt(shg_context* ctx, uint64_t* out, const uint64_t* s,
                          const uint64_t* ct, int len, int count, shg_stream stream);

/* ---------------------------------------------------------------------------
 * Single-modulus oblivious expansion (PIR), on a one-prime context
 * ------------------------------------------------------------------------- */

/* GaloisKeysObliviousExpander::ObliviousExpand for `count` query ciphertexts
 * (oblivious_expand.h:95-138, 173-227, 273-282): keys[levels] with powers
 * n/2^i + 1, ct [count][2][n] -> out [count][2^levels][2][n]. */
int shg_oblivious_expand(shg_context* ctx, const shg_key* const* keys,
                         int levels, uint64_t* out, const uint64_t* ct,
                         int count, shg_stream stream);
/* PIR server step: GaloisKeysObliviousExpander::ObliviousExpand of every
 * query to num_items ciphertexts (oblivious_expand.h:95-138, 173-227), then
 * sum_i expanded_i * db[i] with SymmetricRlweCiphertext::FusedAbsorbAddInPlace
 * (symmetric_encryption.h:250-275).  keys as for shg_oblivious_expand,
 * db [num_items][n] (NTT form, device), 1 <= num_items <= 2^levels,
 * ct [count][2][n] -> out [count][2][n].  Equals shg_oblivious_expand
 * followed by shg_absorb_sum over each query's first num_items ciphertexts,
 * without holding all expanded ciphertexts at once (queries go through in
 * groups that share 1 GiB of scratch). */
int shg_pir_expand_absorb(shg_context* ctx, const shg_key* const* keys,
                          int levels, const uint64_t* db, int num_items,
                          uint64_t* out, const uint64_t* ct, int count,
                          shg_stream stream);
/* Sum_i cts[i] * db[i] via SymmetricRlweCiphertext::FusedAbsorbAddInPlace
 * (symmetric_encryption.h:250-275): cts [count][num_items][2][n],
 * db [num_items][n] -> out [count][2][n]. */
int shg_absorb_sum(shg_context* ctx, uint64_t* out, const uint64_t* cts,
                   const uint64_t* db, int num_items, int count,
                   shg_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* SHELL_GPU_H_ */
