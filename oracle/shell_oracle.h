/*
 * CPU oracle for the SHELL RLWE polynomial hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of google/shell-encryption's CPU algorithms for
 * the path the GPU library accelerates (Montgomery arithmetic, negacyclic NTT,
 * RNS pointwise ops, Substitute, BGV ModReduceLsb, gadget decomposition and
 * key switching, oblivious expansion).  Every function cites the reference
 * file:line it restates.  Residues are stored exactly as SHELL stores them:
 * MontgomeryInt<uint64> representations x*2^64 mod q, canonical in [0, q).
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark may load this library, and only as the checker / the timed CPU
 * baseline.  The GPU product never links or calls it.
 *
 * Parity pin: the results of this restatement are checked bit-for-bit against
 * outputs of the reference's own C++ code (compiled in place by
 * oracle/ref/Makefile where the reference sources are present), recorded as
 * golden fixtures under tests/golden/.
 */
#ifndef SHELL_ORACLE_H_
#define SHELL_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One prime modulus with its Montgomery and NTT parameters at a ring degree. */
typedef struct so_prime so_prime;
/* An RNS context: a chain of primes q_0..q_{L-1} at one ring degree. */
typedef struct so_rns so_rns;

/* ---- prime / Montgomery / NTT parameters ---------------------------------- */
so_prime* so_prime_create(uint64_t q, int log_n);
void so_prime_destroy(so_prime* p);
/* out[0..9] = q, log_q, inv_modulus, r_mod_q, r_mod_q_barrett, inv_r,
 *             inv_r_barrett, barrett_numerator, psi (plain), n_inv (Montgomery) */
void so_prime_info(const so_prime* p, uint64_t out[10]);
/* Montgomery representations of psis_bitrev[i], psis_inv_bitrev[i] (n each). */
void so_prime_tables(const so_prime* p, uint64_t* psis_bitrev,
                     uint64_t* psis_inv_bitrev);

/* ---- element-wise modular ops over `cnt` residues ------------------------- */
void so_import(const so_prime* p, const uint64_t* in, uint64_t* out, size_t cnt);
void so_export(const so_prime* p, const uint64_t* in, uint64_t* out, size_t cnt);
void so_add(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt);
void so_sub(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt);
void so_neg(const so_prime* p, const uint64_t* a, uint64_t* out, size_t cnt);
void so_mul(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt);
/* acc += a*b (Montgomery FusedMulAddInPlace) */
void so_fma(const so_prime* p, uint64_t* acc, const uint64_t* a,
            const uint64_t* b, size_t cnt);
/* out = a * s for one Montgomery-form scalar s */
void so_mul_scalar(const so_prime* p, const uint64_t* a, uint64_t s,
                   uint64_t* out, size_t cnt);

/* ---- NTT ------------------------------------------------------------------ */
void so_ntt_fwd(const so_prime* p, uint64_t* a);
void so_ntt_inv(const so_prime* p, uint64_t* a);
/* 0 on success, 3 (invalid argument) on a bad power */
int so_substitute(const so_prime* p, int power, const uint64_t* in,
                  uint64_t* out);

/* ---- RNS context ---------------------------------------------------------- */
so_rns* so_rns_create(int log_n, const uint64_t* qs, int num_qs);
void so_rns_destroy(so_rns* r);
const so_prime* so_rns_prime(const so_rns* r, int i);
/* q_l^{-1} mod q_j for j < level (Montgomery reps): ql_inv of ModReduce */
void so_rns_ql_inv(const so_rns* r, int level, uint64_t* out);
/* Qhat_i mod q_i and Qhat_i^{-1} mod q_i at `level` (Montgomery reps) */
void so_rns_complements(const so_rns* r, int level, uint64_t* q_hats,
                        uint64_t* q_hat_invs);
/* gadget dimension for log_bs[0..L-1] */
int so_rns_gadget_dim(const so_rns* r, int L, const int* log_bs);
/* gadget vector entries g[k][L] (Montgomery reps, 0 outside limb i) */
void so_rns_gadget_vector(const so_rns* r, int L, const int* log_bs,
                          uint64_t* g);

/* Polys are [L][n] contiguous; ciphertexts [deg+1][L][n]. */
void so_rns_ntt_fwd(const so_rns* r, uint64_t* poly, int L);
void so_rns_ntt_inv(const so_rns* r, uint64_t* poly, int L);
int so_rns_substitute(const so_rns* r, int L, int power, const uint64_t* in,
                      uint64_t* out);
/* Gadget decomposition of a coefficient-form poly: out [k][L][n] coeff form. */
void so_rns_decompose(const so_rns* r, int L, const int* log_bs,
                      const uint64_t* a, uint64_t* out);
/* (r0,r1,r2) = (a0,a1) (x) (b0,b1); inputs [2][L][n], output [3][L][n]. */
void so_rns_tensor(const so_rns* r, int L, const uint64_t* a, const uint64_t* b,
                   uint64_t* out);
/* Relinearize a degree-2 ct [3][L][n] (NTT form) with key_b/key_a [k][L][n];
 * out [2][L][n]. */
void so_rns_relin(const so_rns* r, int L, const int* log_bs, const uint64_t* ct,
                  const uint64_t* key_b, const uint64_t* key_a, uint64_t* out);
/* Galois key switch of a degree-1 ct [2][L][n]; out [2][L][n]. */
void so_rns_galois(const so_rns* r, int L, const int* log_bs,
                   const uint64_t* ct, const uint64_t* key_b,
                   const uint64_t* key_a, uint64_t* out);
/* BGV ModReduceLsb of one poly [L][n] -> [L-1][n]; is_ntt selects the form. */
int so_rns_modreduce_lsb(const so_rns* r, int L, uint64_t t, int is_ntt,
                         const uint64_t* in, uint64_t* out);
/* ct*ct followed by relinearization, `count` independent pairs on `threads`
 * host threads.  a, b: [count][2][L][n]; out [count][2][L][n]. */
void so_rns_mul_relin_batch(const so_rns* r, int L, const int* log_bs,
                            const uint64_t* a, const uint64_t* b,
                            const uint64_t* key_b, const uint64_t* key_a,
                            uint64_t* out, int count, int threads);

/* ChaChaPrng stream bytes [start, start + len) of a 32-byte seed. */
void so_chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                       uint8_t out[64]);
void so_prng_bytes(const uint8_t seed[32], uint64_t start, size_t len, uint8_t* out);
/* SampleUniform then SampleError from the PRNG of seed: a, e [L][n] NTT. */
void so_rns_sample_uniform_error(const so_rns* r, int L, int variance, const uint8_t seed[32],
                                 uint64_t* a, uint64_t* e);
/* EncryptPolynomialBgv: key, m [L][n] NTT; out [2][L][n]. */
void so_rns_encrypt_bgv(const so_rns* r, int L, uint64_t t, int variance, const uint64_t* key,
                        const uint64_t* m, const uint8_t seed[32], uint64_t* out);

/* RnsGaloisKey with a precomputed random pad: ct [2][L][n] at the key's
 * power, pad [k][L][n] = the NTT-form gadget digits of c1; out [2][L][n]. */
void so_rns_galois_pad(const so_rns* r, int L, int k, const uint64_t* ct,
                       const uint64_t* pad, const uint64_t* key_b, const uint64_t* key_a,
                       uint64_t* out);

/* ---- single-modulus key switching / oblivious expansion ------------------- */
int so_gadget_size(const so_prime* p, int log_b);
/* ApplyPartTo: (out0, out1) = sum_i NTT(digit_i(c)) * (k0[i], k1[i]).
 * c in NTT form; k0, k1 [dim][n]. */
void so_keyswitch_part(const so_prime* p, int log_b, int dim, const uint64_t* c,
                       const uint64_t* k0, const uint64_t* k1, uint64_t* out0,
                       uint64_t* out1);
/* GaloisKey::ApplyTo on a substituted ct (c0,c1): out = part(c1) + (c0, 0). */
void so_galois_apply(const so_prime* p, int log_b, int dim, const uint64_t* ct,
                     const uint64_t* k0, const uint64_t* k1, uint64_t* out);
/* GaloisKeysObliviousExpander::ObliviousExpand of one ct [2][n] with `levels`
 * keys keys[levels][2][dim][n]; out [2^levels][2][n]. */
int so_oblivious_expand(const so_prime* p, int levels, int log_b,
                        const uint64_t* keys, const uint64_t* ct,
                        uint64_t* out);
/* out[2][n] = sum_i cts[i] * db[i] (FusedAbsorbAddInPlace chain). */
void so_absorb_sum(const so_prime* p, int count, const uint64_t* cts,
                   const uint64_t* db, uint64_t* out);
/* Symmetric RLWE encryption with injected randomness a (uniform, NTT form)
 * and e (error, coefficient form): out [2][n] = (NTT(e)*t + m + a*s, -a). */
void so_sym_encrypt(const so_prime* p, uint64_t t, const uint64_t* s, const uint64_t* a,
                    const uint64_t* e, const uint64_t* m, uint64_t* out);
/* SymmetricRlweKey::Sample from the PRNG of seed: s [n] NTT form. */
void so_sym_key_sample(const so_prime* p, int variance, const uint8_t seed[32], uint64_t* s);
/* rlwe::Encrypt drawing a, then e, from the PRNG of seed: out [2][n]. */
void so_sym_encrypt_prng(const so_prime* p, uint64_t t, int variance, const uint64_t* s,
                         const uint64_t* m, const uint8_t seed[32], uint64_t* out);
/* Decrypt a ciphertext of `len` components [len][n]: out [n] in [0, t). */
void so_sym_decrypt(const so_prime* p, uint64_t t, const uint64_t* s, const uint64_t* ct,
                    int len, uint64_t* out);
/* MontgomeryInt::SerializeVector / DeserializeVector bit streams of `count`
 * values of one prime; serialize returns the byte count. */
size_t so_serialize_vector(const so_prime* p, const uint64_t* in, size_t count,
                           uint8_t* out);
void so_deserialize_vector(const so_prime* p, const uint8_t* in, size_t count,
                           uint64_t* out);
/* ObliviousExpander::ComputeNormalizer */
uint64_t so_compute_normalizer(int k, int log_t);

/* ---- RNS basis conversion and BFV: the so_rns holds the main primes first
 * and the auxiliary primes after them; index lists name its primes. -------- */
/* SwitchRnsBasis: in [ns][n] over src[] (coefficient form) -> out [nd][n]. */
void so_rns_switch_basis(const so_rns* r, const int* src, int ns, const int* dst, int nd,
                         const uint64_t* in, uint64_t* out);
/* ScaleAndSwitchRnsBasis: round(P/Q * a) mod P, Q = prod src, P = prod dst. */
void so_rns_scale_switch_basis(const so_rns* r, const int* src, int ns, const int* dst,
                               int nd, const uint64_t* in, uint64_t* out);
/* ApproxSwitchRnsBasis; is_ntt: input in NTT form; output coefficient form. */
void so_rns_approx_switch_basis(const so_rns* r, const int* src, int ns, const int* dst,
                                int nd, int is_ntt, int balanced, const uint64_t* in,
                                uint64_t* out);
/* ModReduceMsb: in [L][n] over q_0..q_{L-1} -> out [L-1][n]; 3 if L <= 1. */
int so_rns_modreduce_msb(const so_rns* r, int L, int is_ntt, const uint64_t* in,
                         uint64_t* out);
/* ScaleAndReduceRnsBasisInPlace: main [nm][n] over q_0.., aux [na][n] over aux[]. */
void so_rns_scale_reduce(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                         int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                         const uint64_t* aux_in, uint64_t* out);
/* ApproxModReduceLsb / ApproxModReduceMsb: out [nm][n] NTT form. */
void so_rns_approx_modreduce_lsb(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                                 int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                                 const uint64_t* aux_in, uint64_t* out);
void so_rns_approx_modreduce_msb(const so_rns* r, int nm, const int* aux, int na,
                                 int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                                 const uint64_t* aux_in, uint64_t* out);
/* RnsBfvCiphertext::Mul: a, b [2][nm][n] NTT form -> out [3][nm][n]. */
void so_bfv_mul(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                const uint64_t* a, const uint64_t* b, uint64_t* out);
/* RnsBfvCiphertext::AbsorbInPlace: ct [len][nm][n], pt [nm][n] NTT -> out. */
void so_bfv_absorb(const so_rns* r, int nm, const int* aux, int na, uint64_t t, int len,
                   const uint64_t* ct, const uint64_t* pt, uint64_t* out);

#ifdef __cplusplus
}
#endif
#endif  /* SHELL_ORACLE_H_ */
