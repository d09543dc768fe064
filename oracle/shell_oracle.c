/*
 * CPU oracle for the SHELL RLWE polynomial hot path — TEST INFRASTRUCTURE ONLY.
 * Plain-C restatement of google/shell-encryption's CPU algorithms; each
 * function names the reference file:line it follows.  Only tests, the smoke
 * check and the benchmark's CPU-baseline leg use it.
 */
#include "shell_oracle.h"
#include "chacha20.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

struct so_prime {
  /* MontgomeryIntParams<uint64> (montgomery.h:77-202) */
  uint64_t q;
  int log_q;
  uint64_t inv_modulus;      /* R*inv_r - q*inv_modulus = 1 */
  uint64_t r_mod_q;          /* 2^64 mod q */
  uint64_t r_mod_q_barrett;  /* floor(r_mod_q * 2^64 / q) */
  uint64_t inv_r;            /* 2^-64 mod q */
  uint64_t inv_r_barrett;    /* floor(inv_r * 2^64 / q) */
  uint64_t barrett_num;      /* floor(2^64 / q) */
  /* NttParameters (ntt_parameters.h:160-235) */
  int log_n, n;
  uint64_t psi;              /* plain value of the primitive 2n-th root */
  uint64_t n_inv;            /* Montgomery rep of n^{-1} */
  uint64_t* psis_bitrev;     /* Montgomery reps, n */
  uint64_t* psis_bitrev_c;   /* GetConstant(): plain value */
  uint64_t* psis_bitrev_cb;  /* GetConstant(): barrett */
  uint64_t* psis_inv_bitrev;
  uint64_t* psis_inv_bitrev_c;
  uint64_t* psis_inv_bitrev_cb;
  uint32_t* bitrevs;
};

struct so_rns {
  int log_n, L;
  so_prime** primes;
  /* prime_q_invs_[i][j] = q_i^{-1} mod q_j, 1 when i == j
   * (rns/rns_context.cc:169-200), Montgomery reps */
  uint64_t* q_invs;
  /* prime_qs_[i][j] = q_i mod q_j, 0 when i == j */
  uint64_t* q_mods;
};

/* ---------------------------------------------------------------------------
 * Montgomery arithmetic (montgomery.h / montgomery.cc)
 * ------------------------------------------------------------------------- */

static int bit_length(uint64_t x) {  /* bits_util.h BitLength */
  int b = 0;
  while (x) { b++; x >>= 1; }
  return b;
}

/* ToMontgomeryInt: Shoup multiply by r_mod_q (montgomery.cc:27-40). */
static inline uint64_t mont_import(const so_prime* p, uint64_t x) {
  uint64_t hi = (uint64_t)(((u128)p->r_mod_q_barrett * x) >> 64);
  uint64_t r = x * p->r_mod_q - hi * p->q;
  return r >= p->q ? r - p->q : r;
}

/* ExportInt (montgomery.h:156-164). */
static inline uint64_t mont_export(const so_prime* p, uint64_t x) {
  uint64_t hi = (uint64_t)(((u128)p->inv_r_barrett * x) >> 64);
  uint64_t r = x * p->inv_r - hi * p->q;
  return r >= p->q ? r - p->q : r;
}

/* MulInPlace: REDC (montgomery.h:318-336). */
static inline uint64_t mont_mul(const so_prime* p, uint64_t a, uint64_t b) {
  u128 prod = (u128)a * b;
  uint64_t u = (uint64_t)prod * p->inv_modulus;
  u128 t = prod + (u128)p->q * u;
  uint64_t r = (uint64_t)(t >> 64);
  return r >= p->q ? r - p->q : r;
}

/* FusedMulAddInPlace (montgomery.h:446-465). */
static inline uint64_t mont_fma(const so_prime* p, uint64_t acc, uint64_t a,
                                uint64_t b) {
  u128 t = (u128)p->r_mod_q * acc + (u128)a * b;
  uint64_t u = (uint64_t)t * p->inv_modulus;
  t += (u128)p->q * u;
  uint64_t r = (uint64_t)(t >> 64);
  return r >= p->q ? r - p->q : r;
}

/* MulConstantInPlace (montgomery.h:362-372); input may be in [0, 4q). */
static inline uint64_t mul_const(const so_prime* p, uint64_t x, uint64_t c,
                                 uint64_t cb) {
  uint64_t hi = (uint64_t)(((u128)cb * x) >> 64);
  uint64_t r = x * c - hi * p->q;
  return r >= p->q ? r - p->q : r;
}

/* BarrettReduce (montgomery.h:126-133); input < 4q. */
static inline uint64_t barrett(const so_prime* p, uint64_t x) {
  uint64_t hi = (uint64_t)(((u128)p->barrett_num * x) >> 64);
  uint64_t r = x - hi * p->q;
  return r >= p->q ? r - p->q : r;
}

/* AddInPlace / SubInPlace / NegateInPlace (montgomery.h:383-415). */
static inline uint64_t mont_add(const so_prime* p, uint64_t a, uint64_t b) {
  return barrett(p, a + b);
}
static inline uint64_t mont_sub(const so_prime* p, uint64_t a, uint64_t b) {
  return barrett(p, a + (p->q - b));
}
static inline uint64_t mont_neg(const so_prime* p, uint64_t a) {
  return p->q - a;
}

/* ModExp on Montgomery reps (montgomery.cc:472-492). */
static uint64_t mont_pow(const so_prime* p, uint64_t base, uint64_t e) {
  uint64_t result = p->r_mod_q;  /* ImportOne */
  while (e > 0) {
    if (e & 1) result = mont_mul(p, result, base);
    base = mont_mul(p, base, base);
    e >>= 1;
  }
  return result;
}

/* GetConstant (montgomery.cc:221-227). */
static void get_constant(const so_prime* p, uint64_t m, uint64_t* c,
                         uint64_t* cb) {
  *c = mont_export(p, m);
  *cb = (uint64_t)(((u128)(*c) << 64) / p->q);
}

/* Bitrev (ntt_parameters.cc:21-31). */
static uint32_t bitrev(uint32_t x, int log_n) {
  uint32_t out = 0;
  for (int i = 0; i < log_n; i++) {
    out = (out << 1) | (x & 1);
    x >>= 1;
  }
  return out;
}

/* MontgomeryIntParams::Create and constructor (montgomery.cc:44-92,
 * montgomery.h:179-193), InitializeNttParameters (ntt_parameters.h:183-235). */
so_prime* so_prime_create(uint64_t q, int log_n) {
  if ((q >> 62) != 0 || (q & 1) == 0) return NULL;
  if (log_n <= 0 || log_n > 15) return NULL;
  uint64_t two_n = (uint64_t)1 << (log_n + 1);
  if (q % two_n != 1) return NULL;
  so_prime* p = (so_prime*)calloc(1, sizeof(so_prime));
  p->q = q;
  p->log_q = bit_length(q);
  /* Inverses via the halving loop of montgomery.cc:61-92: x*2^64 - y*q = 1 */
  u128 x = 1, y = 0;
  const u128 R = (u128)1 << 64;
  for (int i = 64; i > 0; i--) {
    if (x & 1) { x += q; y += R; }
    x >>= 1;
    y >>= 1;
  }
  p->inv_r = (uint64_t)x;
  p->inv_modulus = (uint64_t)y;
  p->r_mod_q = (uint64_t)(R % q);
  p->r_mod_q_barrett = (uint64_t)(((u128)p->r_mod_q << 64) / q);
  p->inv_r_barrett = (uint64_t)(((u128)p->inv_r << 64) / q);
  p->barrett_num = (uint64_t)(R / q);

  int n = 1 << log_n;
  p->log_n = log_n;
  p->n = n;
  /* n^{-1}: ImportInt(n).MultiplicativeInverse() (ntt_parameters.h:207-210,
   * montgomery.cc:494-498) */
  p->n_inv = mont_pow(p, mont_import(p, (uint64_t)n), q - 2);

  /* PrimitiveNthRootOfUnity(log_n + 1) (ntt_parameters.h:41-71): first t >= 2
   * with (t^k)^{n} != 1 where k = (q-1)/2n. */
  uint64_t k = (q - 1) / two_n;
  uint64_t one = p->r_mod_q;
  uint64_t psi_m = 0;
  for (uint64_t t = 2; t < q; t++) {
    uint64_t cand = mont_pow(p, mont_import(p, t), k);
    if (mont_pow(p, cand, (uint64_t)n) != one) { psi_m = cand; break; }
  }
  p->psi = mont_export(p, psi_m);

  p->bitrevs = (uint32_t*)malloc(sizeof(uint32_t) * n);
  for (int i = 0; i < n; i++) p->bitrevs[i] = bitrev((uint32_t)i, log_n);

  /* NttPsis: row[i] = psi^i (ntt_parameters.h:79-92). */
  uint64_t* row = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < n; i++) row[i] = mont_pow(p, psi_m, (uint64_t)i);
  /* NttPsisBitrev (ntt_parameters.h:117-127). */
  p->psis_bitrev = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < n; i++) p->psis_bitrev[i] = row[p->bitrevs[i]];
  /* NttPsisInvBitrev (ntt_parameters.h:131-157): reverse row[1..n-1],
   * bit-reverse, then multiply row[0] by psi^{-1} = -row[1] and the others by
   * row[1] (= -psi^{-1}). */
  uint64_t* rev = (uint64_t*)malloc(sizeof(uint64_t) * n);
  rev[0] = row[0];
  for (int i = 1; i < n; i++) rev[i] = row[n - i];
  uint64_t psi_inv = mont_neg(p, rev[1 % n]);
  uint64_t neg_psi_inv = rev[1 % n];
  if (n == 1) { psi_inv = 0; neg_psi_inv = 0; }
  p->psis_inv_bitrev = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < n; i++) p->psis_inv_bitrev[i] = rev[p->bitrevs[i]];
  p->psis_inv_bitrev[0] = mont_mul(p, p->psis_inv_bitrev[0], psi_inv);
  for (int i = 1; i < n; i++)
    p->psis_inv_bitrev[i] = mont_mul(p, p->psis_inv_bitrev[i], neg_psi_inv);
  free(rev);
  free(row);

  p->psis_bitrev_c = (uint64_t*)malloc(sizeof(uint64_t) * n);
  p->psis_bitrev_cb = (uint64_t*)malloc(sizeof(uint64_t) * n);
  p->psis_inv_bitrev_c = (uint64_t*)malloc(sizeof(uint64_t) * n);
  p->psis_inv_bitrev_cb = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < n; i++) {
    get_constant(p, p->psis_bitrev[i], &p->psis_bitrev_c[i],
                 &p->psis_bitrev_cb[i]);
    get_constant(p, p->psis_inv_bitrev[i], &p->psis_inv_bitrev_c[i],
                 &p->psis_inv_bitrev_cb[i]);
  }
  return p;
}

void so_prime_destroy(so_prime* p) {
  if (!p) return;
  free(p->psis_bitrev); free(p->psis_bitrev_c); free(p->psis_bitrev_cb);
  free(p->psis_inv_bitrev); free(p->psis_inv_bitrev_c);
  free(p->psis_inv_bitrev_cb); free(p->bitrevs);
  free(p);
}

void so_prime_info(const so_prime* p, uint64_t out[10]) {
  out[0] = p->q; out[1] = (uint64_t)p->log_q; out[2] = p->inv_modulus;
  out[3] = p->r_mod_q; out[4] = p->r_mod_q_barrett; out[5] = p->inv_r;
  out[6] = p->inv_r_barrett; out[7] = p->barrett_num; out[8] = p->psi;
  out[9] = p->n_inv;
}

void so_prime_tables(const so_prime* p, uint64_t* fwd, uint64_t* inv) {
  memcpy(fwd, p->psis_bitrev, sizeof(uint64_t) * p->n);
  memcpy(inv, p->psis_inv_bitrev, sizeof(uint64_t) * p->n);
}

void so_import(const so_prime* p, const uint64_t* in, uint64_t* out,
               size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_import(p, in[i]);
}
void so_export(const so_prime* p, const uint64_t* in, uint64_t* out,
               size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_export(p, in[i]);
}
void so_add(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_add(p, a[i], b[i]);
}
void so_sub(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_sub(p, a[i], b[i]);
}
void so_neg(const so_prime* p, const uint64_t* a, uint64_t* out, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_neg(p, a[i]);
}
void so_mul(const so_prime* p, const uint64_t* a, const uint64_t* b,
            uint64_t* out, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_mul(p, a[i], b[i]);
}
void so_fma(const so_prime* p, uint64_t* acc, const uint64_t* a,
            const uint64_t* b, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) acc[i] = mont_fma(p, acc[i], a[i], b[i]);
}
void so_mul_scalar(const so_prime* p, const uint64_t* a, uint64_t s,
                   uint64_t* out, size_t cnt) {
  for (size_t i = 0; i < cnt; i++) out[i] = mont_mul(p, a[i], s);
}

/* ---------------------------------------------------------------------------
 * NTT (dft_transformations.h)
 * ------------------------------------------------------------------------- */

/* IterativeCooleyTukey (dft_transformations.h:59-100). */
void so_ntt_fwd(const so_prime* p, uint64_t* a) {
  int index_psi = 1;
  const int n = p->n;
  for (int i = p->log_n - 1; i >= 0; i--) {
    const int half_m = 1 << i;
    const int m = half_m << 1;
    for (int k = 0; k < n; k += m) {
      const uint64_t c = p->psis_bitrev_c[index_psi];
      const uint64_t cb = p->psis_bitrev_cb[index_psi];
      for (int j = 0; j < half_m; j++) {
        uint64_t t = mul_const(p, a[k + j + half_m], c, cb);
        uint64_t u = a[k + j];
        if (i & 1) {  /* lazy layer: LazyAdd / LazySub */
          a[k + j] = a[k + j] + t;
          a[k + j + half_m] = u + (p->q - t);
        } else {
          a[k + j] = mont_add(p, a[k + j], t);
          a[k + j + half_m] = mont_sub(p, u, t);
        }
      }
      index_psi++;
    }
  }
}

/* IterativeGentlemanSande + normalisation (dft_transformations.h:118-153,
 * 181-201). */
void so_ntt_inv(const so_prime* p, uint64_t* a) {
  int index_psi_inv = 0;
  const int n = p->n;
  for (int i = 0; i < p->log_n; i++) {
    const int half_m = 1 << i;
    const int m = half_m << 1;
    for (int k = 0; k < n; k += m) {
      const uint64_t c = p->psis_inv_bitrev_c[index_psi_inv];
      const uint64_t cb = p->psis_inv_bitrev_cb[index_psi_inv];
      for (int j = 0; j < half_m; j++) {
        uint64_t t = a[k + j + half_m];
        uint64_t u = a[k + j];
        a[k + j] = mont_add(p, a[k + j], t);
        a[k + j + half_m] = mul_const(p, u + (p->q - t), c, cb);
      }
      index_psi_inv++;
    }
  }
  for (int i = 0; i < n; i++) a[i] = mont_mul(p, a[i], p->n_inv);
}

/* Polynomial::Substitute (polynomial.h:226-260) and
 * RnsPolynomial::Substitute (rns/rns_polynomial.cc:209-260). */
int so_substitute(const so_prime* p, int power, const uint64_t* in,
                  uint64_t* out) {
  const int n = p->n;
  if (power < 0 || (power % 2) == 0 || power >= 2 * n) return 3;
  int psi_power_index = (power - 1) / 2;
  for (int j = 0; j < n; j++) {
    out[p->bitrevs[j]] = in[p->bitrevs[psi_power_index]];
    psi_power_index = (psi_power_index + power) % n;
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * RNS context (rns/rns_context.cc)
 * ------------------------------------------------------------------------- */

so_rns* so_rns_create(int log_n, const uint64_t* qs, int num_qs) {
  so_rns* r = (so_rns*)calloc(1, sizeof(so_rns));
  r->log_n = log_n;
  r->L = num_qs;
  r->primes = (so_prime**)calloc(num_qs, sizeof(so_prime*));
  for (int i = 0; i < num_qs; i++) {
    r->primes[i] = so_prime_create(qs[i], log_n);
    if (!r->primes[i]) { so_rns_destroy(r); return NULL; }
  }
  /* GenerateCrtConstantsForMainModulus (rns/rns_context.cc:169-200). */
  r->q_invs = (uint64_t*)calloc((size_t)num_qs * num_qs, sizeof(uint64_t));
  r->q_mods = (uint64_t*)calloc((size_t)num_qs * num_qs, sizeof(uint64_t));
  for (int i = 0; i < num_qs; i++) {
    for (int j = 0; j < num_qs; j++) {
      const so_prime* pj = r->primes[j];
      if (i == j) {
        r->q_mods[i * num_qs + j] = 0;
        r->q_invs[i * num_qs + j] = pj->r_mod_q;
      } else {
        uint64_t qi_mod_qj = mont_import(pj, qs[i]);
        r->q_mods[i * num_qs + j] = qi_mod_qj;
        r->q_invs[i * num_qs + j] = mont_pow(pj, qi_mod_qj, pj->q - 2);
      }
    }
  }
  return r;
}

void so_rns_destroy(so_rns* r) {
  if (!r) return;
  for (int i = 0; i < r->L; i++) so_prime_destroy(r->primes[i]);
  free(r->primes); free(r->q_invs); free(r->q_mods);
  free(r);
}

const so_prime* so_rns_prime(const so_rns* r, int i) { return r->primes[i]; }

/* MainPrimeModulusInverseResidues()[level].Prefix(level)
 * (rns/rns_context.h:145-147, rns/rns_integer.h:37-40). */
void so_rns_ql_inv(const so_rns* r, int level, uint64_t* out) {
  for (int j = 0; j < level; j++) out[j] = r->q_invs[level * r->L + j];
}

/* MainPrimeModulusComplements / MainPrimeModulusCrtFactors
 * (rns/rns_context.cc:234-282). */
void so_rns_complements(const so_rns* r, int level, uint64_t* q_hats,
                        uint64_t* q_hat_invs) {
  for (int i = 0; i <= level; i++) {
    const so_prime* pi = r->primes[i];
    uint64_t h = pi->r_mod_q, hi = pi->r_mod_q;
    for (int j = 0; j <= level; j++) {
      if (j == i) continue;
      h = mont_mul(pi, h, r->q_mods[j * r->L + i]);
      hi = mont_mul(pi, hi, r->q_invs[j * r->L + i]);
    }
    q_hats[i] = h;
    q_hat_invs[i] = hi;
  }
}

/* GadgetSize (gadget.h:43-47). */
static int gadget_size(const so_prime* p, int log_b) {
  return (p->log_q + (log_b - 1)) / log_b;
}

int so_rns_gadget_dim(const so_rns* r, int L, const int* log_bs) {
  int k = 0;
  for (int i = 0; i < L; i++) k += gadget_size(r->primes[i], log_bs[i]);
  return k;
}

/* RnsGadget::Create (rns/rns_gadget.cc:42-102), with q_hats / q_hat_invs at
 * level L-1. */
void so_rns_gadget_vector(const so_rns* r, int L, const int* log_bs,
                          uint64_t* g) {
  uint64_t* qh = (uint64_t*)malloc(sizeof(uint64_t) * L);
  uint64_t* qhi = (uint64_t*)malloc(sizeof(uint64_t) * L);
  so_rns_complements(r, L - 1, qh, qhi);
  int row = 0;
  for (int i = 0; i < L; i++) {
    const so_prime* pi = r->primes[i];
    uint64_t bi = mont_import(pi, (uint64_t)1 << log_bs[i]);
    uint64_t cur = mont_mul(pi, qh[i], qhi[i]);
    int ki = gadget_size(pi, log_bs[i]);
    for (int j = 0; j < ki; j++) {
      for (int l = 0; l < L; l++) g[(size_t)row * L + l] = (l == i) ? cur : 0;
      row++;
      cur = mont_mul(pi, cur, bi);
    }
  }
  free(qh);
  free(qhi);
}

void so_rns_ntt_fwd(const so_rns* r, uint64_t* poly, int L) {
  const size_t n = (size_t)1 << r->log_n;
  for (int i = 0; i < L; i++) so_ntt_fwd(r->primes[i], poly + i * n);
}

void so_rns_ntt_inv(const so_rns* r, uint64_t* poly, int L) {
  const size_t n = (size_t)1 << r->log_n;
  for (int i = 0; i < L; i++) so_ntt_inv(r->primes[i], poly + i * n);
}

int so_rns_substitute(const so_rns* r, int L, int power, const uint64_t* in,
                      uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  for (int i = 0; i < L; i++) {
    int st = so_substitute(r->primes[i], power, in + i * n, out + i * n);
    if (st) return st;
  }
  return 0;
}

/* ConvertModulusBalanced of one exported value x (modulus_conversion.h:30-83):
 * x > floor(q/2) denotes x - q.  Returns the Montgomery rep mod p. */
static inline uint64_t convert_balanced(const so_prime* from,
                                        const so_prime* to, uint64_t x) {
  if (from->q == to->q) return mont_import(to, x);
  uint64_t xp = mont_import(to, x);
  if (x > (from->q >> 1)) {
    if (to->q > from->q) {
      uint64_t diff = mont_import(to, to->q - from->q);
      xp = mont_add(to, xp, diff);
    } else {
      uint64_t diff = mont_import(to, from->q - to->q);
      xp = mont_sub(to, xp, diff);
    }
  }
  return xp;
}

/* RnsGadget::Decompose (rns/rns_gadget.cc:108-153) with BaseDecompose
 * (gadget.h:52-79): digits LSB first, each lifted (balanced) to every limb. */
void so_rns_decompose(const so_rns* r, int L, const int* log_bs,
                      const uint64_t* a, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  int row = 0;
  uint64_t* x = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < L; i++) {
    const so_prime* pi = r->primes[i];
    int ki = gadget_size(pi, log_bs[i]);
    uint64_t mask = ((uint64_t)1 << log_bs[i]) - 1;
    for (size_t c = 0; c < n; c++) x[c] = mont_export(pi, a[i * n + c]);
    for (int d = 0; d < ki; d++) {
      uint64_t* dst = out + (size_t)row * L * n;
      for (size_t c = 0; c < n; c++) {
        uint64_t digit_m = mont_import(pi, x[c] & mask);
        uint64_t digit = mont_export(pi, digit_m);
        for (int l = 0; l < L; l++) {
          dst[l * n + c] =
              (l == i) ? digit_m : convert_balanced(pi, r->primes[l], digit);
        }
        x[c] >>= log_bs[i];
      }
      row++;
    }
  }
  free(x);
}

/* RnsRlweCiphertext::Mul (rns/rns_ciphertext.h:501-524) for 2x2 components. */
void so_rns_tensor(const so_rns* r, int L, const uint64_t* a, const uint64_t* b,
                   uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  const size_t P = (size_t)L * n;
  memset(out, 0, sizeof(uint64_t) * 3 * P);
  for (int i = 0; i < 2; i++) {
    for (int j = 0; j < 2; j++) {
      for (int l = 0; l < L; l++) {
        so_fma(r->primes[l], out + (i + j) * P + l * n, a + i * P + l * n,
               b + j * P + l * n, n);
      }
    }
  }
}

static void rns_fma_poly(const so_rns* r, int L, uint64_t* acc,
                         const uint64_t* a, const uint64_t* b) {
  const size_t n = (size_t)1 << r->log_n;
  for (int l = 0; l < L; l++)
    so_fma(r->primes[l], acc + l * n, a + l * n, b + l * n, n);
}

/* Key-switch core shared by relinearization and Galois keys:
 * acc0 += sum_j NTT(g^{-1}(c))_j * key_b[j], acc1 += ... * key_a[j]. */
static void rns_keyswitch_accumulate(const so_rns* r, int L, const int* log_bs,
                                     const uint64_t* c_ntt,
                                     const uint64_t* key_b,
                                     const uint64_t* key_a, uint64_t* acc0,
                                     uint64_t* acc1) {
  const size_t n = (size_t)1 << r->log_n;
  const size_t P = (size_t)L * n;
  int k = so_rns_gadget_dim(r, L, log_bs);
  uint64_t* coeff = (uint64_t*)malloc(sizeof(uint64_t) * P);
  memcpy(coeff, c_ntt, sizeof(uint64_t) * P);
  so_rns_ntt_inv(r, coeff, L);  /* ConvertToCoeffForm */
  uint64_t* digits = (uint64_t*)malloc(sizeof(uint64_t) * P * k);
  so_rns_decompose(r, L, log_bs, coeff, digits);
  for (int j = 0; j < k; j++) {
    uint64_t* dj = digits + (size_t)j * P;
    so_rns_ntt_fwd(r, dj, L);
    rns_fma_poly(r, L, acc0, dj, key_b + (size_t)j * P);
    rns_fma_poly(r, L, acc1, dj, key_a + (size_t)j * P);
  }
  free(digits);
  free(coeff);
}

/* RnsRelinKey::ApplyToRlweCiphertext for a degree-2 ciphertext
 * (rns/rns_relinearization_key.cc:184-232); key index (i-2)*l + j = j. */
void so_rns_relin(const so_rns* r, int L, const int* log_bs, const uint64_t* ct,
                  const uint64_t* key_b, const uint64_t* key_a, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  const size_t P = (size_t)L * n;
  memcpy(out, ct, sizeof(uint64_t) * 2 * P);
  rns_keyswitch_accumulate(r, L, log_bs, ct + 2 * P, key_b, key_a, out,
                           out + P);
}

/* RnsGaloisKey::ApplyToRlweCiphertext (rns/rns_galois_key.cc:238-287). */
void so_rns_galois(const so_rns* r, int L, const int* log_bs,
                   const uint64_t* ct, const uint64_t* key_b,
                   const uint64_t* key_a, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  const size_t P = (size_t)L * n;
  memset(out, 0, sizeof(uint64_t) * 2 * P);
  rns_keyswitch_accumulate(r, L, log_bs, ct + P, key_b, key_a, out, out + P);
  for (int l = 0; l < L; l++)
    so_add(r->primes[l], out + l * n, ct + l * n, out + l * n, n);
}

/* RnsPolynomial::ModReduceLsb (rns/rns_polynomial.cc:262-344). */
int so_rns_modreduce_lsb(const so_rns* r, int L, uint64_t t, int is_ntt,
                         const uint64_t* in, uint64_t* out) {
  if (L <= 1) return 3;
  const size_t n = (size_t)1 << r->log_n;
  const int Lr = L - 1;
  const so_prime* pl = r->primes[L - 1];
  uint64_t rr = pl->q % t;
  uint64_t kk = (pl->q - rr) / t;
  uint64_t k_mod_ql = mont_import(pl, kk);
  uint64_t* delta = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (size_t c = 0; c < n; c++)
    delta[c] = mont_mul(pl, in[(size_t)(L - 1) * n + c], k_mod_ql);
  uint64_t* ql_inv = (uint64_t*)malloc(sizeof(uint64_t) * (Lr > 0 ? Lr : 1));
  so_rns_ql_inv(r, L - 1, ql_inv);
  /* r * a (mod Q/ql) */
  for (int i = 0; i < Lr; i++) {
    uint64_t r_m = mont_import(r->primes[i], rr);
    so_mul_scalar(r->primes[i], in + i * n, r_m, out + i * n, n);
  }
  if (is_ntt) so_ntt_inv(pl, delta);
  uint64_t* dq = (uint64_t*)malloc(sizeof(uint64_t) * n);
  for (int i = 0; i < Lr; i++) {
    const so_prime* pi = r->primes[i];
    for (size_t c = 0; c < n; c++)
      dq[c] = convert_balanced(pl, pi, mont_export(pl, delta[c]));
    if (is_ntt) so_ntt_fwd(pi, dq);
    uint64_t t_m = mont_import(pi, t);
    for (size_t c = 0; c < n; c++) {
      uint64_t d = mont_mul(pi, dq[c], t_m);
      uint64_t v = mont_add(pi, out[i * n + c], d);
      out[i * n + c] = mont_mul(pi, v, ql_inv[i]);
    }
  }
  free(dq);
  free(ql_inv);
  free(delta);
  return 0;
}

typedef struct {
  const so_rns* r;
  int L;
  const int* log_bs;
  const uint64_t *a, *b, *key_b, *key_a;
  uint64_t* out;
  int begin, end;
} mul_relin_job;

static void* mul_relin_worker(void* arg) {
  mul_relin_job* job = (mul_relin_job*)arg;
  const size_t n = (size_t)1 << job->r->log_n;
  const size_t P = (size_t)job->L * n;
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * 3 * P);
  for (int c = job->begin; c < job->end; c++) {
    so_rns_tensor(job->r, job->L, job->a + (size_t)c * 2 * P,
                  job->b + (size_t)c * 2 * P, tmp);
    so_rns_relin(job->r, job->L, job->log_bs, tmp, job->key_b, job->key_a,
                 job->out + (size_t)c * 2 * P);
  }
  free(tmp);
  return NULL;
}

void so_rns_mul_relin_batch(const so_rns* r, int L, const int* log_bs,
                            const uint64_t* a, const uint64_t* b,
                            const uint64_t* key_b, const uint64_t* key_a,
                            uint64_t* out, int count, int threads) {
  if (threads < 1) threads = 1;
  if (threads > count) threads = count > 0 ? count : 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
  mul_relin_job* jobs = (mul_relin_job*)malloc(sizeof(mul_relin_job) * threads);
  for (int t = 0; t < threads; t++) {
    jobs[t] = (mul_relin_job){r, L, log_bs, a, b, key_b, key_a, out,
                              (int)((long)count * t / threads),
                              (int)((long)count * (t + 1) / threads)};
    pthread_create(&th[t], NULL, mul_relin_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
}

/* ---------------------------------------------------------------------------
 * Single-modulus key switching and oblivious expansion
 * ------------------------------------------------------------------------- */

int so_gadget_size(const so_prime* p, int log_b) { return gadget_size(p, log_b); }

/* RelinearizationKeyPart::ApplyPartTo + MatrixMultiply
 * (relinearization_key.cc:76-96, 143-162); BaseDecompose (gadget.h:52-79)
 * imports the digits into the same modulus. */
void so_keyswitch_part(const so_prime* p, int log_b, int dim, const uint64_t* c,
                       const uint64_t* k0, const uint64_t* k1, uint64_t* out0,
                       uint64_t* out1) {
  const size_t n = (size_t)p->n;
  uint64_t* x = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint64_t* d = (uint64_t*)malloc(sizeof(uint64_t) * n);
  memcpy(x, c, sizeof(uint64_t) * n);
  so_ntt_inv(p, x);
  for (size_t i = 0; i < n; i++) x[i] = mont_export(p, x[i]);
  uint64_t mask = ((uint64_t)1 << log_b) - 1;
  memset(out0, 0, sizeof(uint64_t) * n);
  memset(out1, 0, sizeof(uint64_t) * n);
  for (int j = 0; j < dim; j++) {
    for (size_t i = 0; i < n; i++) {
      d[i] = mont_import(p, x[i] & mask);
      x[i] >>= log_b;
    }
    so_ntt_fwd(p, d);
    so_fma(p, out0, d, k0 + (size_t)j * n, n);
    so_fma(p, out1, d, k1 + (size_t)j * n, n);
  }
  free(d);
  free(x);
}

/* RelinearizationKey::ApplyTo for a Galois key (num_parts 2, target s)
 * (relinearization_key.cc:288-344): part(c1) + (c0, 0). */
void so_galois_apply(const so_prime* p, int log_b, int dim, const uint64_t* ct,
                     const uint64_t* k0, const uint64_t* k1, uint64_t* out) {
  const size_t n = (size_t)p->n;
  so_keyswitch_part(p, log_b, dim, ct + n, k0, k1, out, out + n);
  so_add(p, out, ct, out, n);
}

/* ObliviousExpander::ExpandCiphertext with GaloisKeysObliviousExpander's
 * SubstitutionWithKeys (oblivious_expand.h:173-227, 273-282). */
int so_oblivious_expand(const so_prime* p, int levels, int log_b,
                        const uint64_t* keys, const uint64_t* ct,
                        uint64_t* out) {
  const size_t n = (size_t)p->n;
  const int dim = gadget_size(p, log_b);
  const size_t key_sz = (size_t)2 * dim * n;
  if (levels < 0 || levels >= 32) return 3;
  if ((n >> levels) == 0) return 3;
  memcpy(out, ct, sizeof(uint64_t) * 2 * n);
  uint64_t* monomial = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint64_t* sub = (uint64_t*)malloc(sizeof(uint64_t) * 2 * n);
  uint64_t* ks = (uint64_t*)malloc(sizeof(uint64_t) * 2 * n);
  for (int j = 0; j < levels; j++) {
    memset(monomial, 0, sizeof(uint64_t) * n);
    monomial[n - ((size_t)1 << j)] = mont_neg(p, p->r_mod_q);  /* -x^{N-2^j} */
    so_ntt_fwd(p, monomial);
    int power = (int)(n >> j) + 1;
    const uint64_t* key = keys + (size_t)j * key_sz;
    for (int k = 0; k < (1 << j); k++) {
      uint64_t* c = out + (size_t)k * 2 * n;
      uint64_t* c_hi = out + ((size_t)k + ((size_t)1 << j)) * 2 * n;
      so_substitute(p, power, c, sub);
      so_substitute(p, power, c + n, sub + n);
      so_galois_apply(p, log_b, dim, sub, key, key + (size_t)dim * n, ks);
      /* result[k + 2^j] = (c - sub) * monomial */
      for (int comp = 0; comp < 2; comp++) {
        so_sub(p, c + comp * n, ks + comp * n, c_hi + comp * n, n);
        so_mul(p, c_hi + comp * n, monomial, c_hi + comp * n, n);
      }
      /* result[k] += sub */
      so_add(p, c, ks, c, 2 * n);
    }
  }
  free(ks);
  free(sub);
  free(monomial);
  return 0;
}

/* SymmetricRlweCiphertext::FusedAbsorbAddInPlace chain
 * (symmetric_encryption.h:250-275). */
void so_absorb_sum(const so_prime* p, int count, const uint64_t* cts,
                   const uint64_t* db, uint64_t* out) {
  const size_t n = (size_t)p->n;
  memset(out, 0, sizeof(uint64_t) * 2 * n);
  for (int i = 0; i < count; i++) {
    const uint64_t* c = cts + (size_t)i * 2 * n;
    so_fma(p, out, c, db + (size_t)i * n, n);
    so_fma(p, out + n, c + n, db + (size_t)i * n, n);
  }
}

/* internal::Encrypt with the randomness injected (symmetric_encryption.h:
 * 940-963) and c1 = -a (symmetric_encryption.h:1006-1021):
 * c0 = NTT(e) * t + m + a * s, c1 = -a.  s, a, m in NTT form, e in
 * coefficient form, all Montgomery; t = the plaintext modulus (an integer,
 * imported like SymmetricRlweKey's t_mod).  out [2][n]. */
void so_sym_encrypt(const so_prime* p, uint64_t t, const uint64_t* s, const uint64_t* a,
                    const uint64_t* e, const uint64_t* m, uint64_t* out) {
  const size_t n = (size_t)p->n;
  uint64_t* c0 = out;
  memcpy(c0, e, n * sizeof(uint64_t));
  so_ntt_fwd(p, c0);
  const uint64_t t_mont = mont_import(p, t % p->q);
  for (size_t i = 0; i < n; i++) c0[i] = mont_mul(p, c0[i], t_mont);
  so_add(p, c0, m, c0, n);
  so_fma(p, c0, a, s, n);
  so_neg(p, a, out + n, n);
}

/* Decrypt (symmetric_encryption.h:1138-1152): ExtractErrorAndMessage
 * (sum_i c_i * s^i in NTT form, inverse NTT; :966-1000) then RemoveError
 * (ExportInt, values above floor(q/2) minus q mod t, then mod t; :1084-1110).
 * ct [len][n] NTT form; out [n] integers in [0, t). */
void so_sym_decrypt(const so_prime* p, uint64_t t, const uint64_t* s, const uint64_t* ct,
                    int len, uint64_t* out) {
  const size_t n = (size_t)p->n;
  uint64_t* acc = (uint64_t*)calloc(n, sizeof(uint64_t));
  uint64_t* pw = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t* ci = (uint64_t*)malloc(n * sizeof(uint64_t));
  memcpy(pw, s, n * sizeof(uint64_t));
  for (int i = 0; i < len; i++) {
    memcpy(ci, ct + (size_t)i * n, n * sizeof(uint64_t));
    if (i > 1) so_mul(p, pw, s, pw, n);
    if (i > 0) so_mul(p, ci, pw, ci, n);
    so_add(p, acc, ci, acc, n);
  }
  so_ntt_inv(p, acc);
  const uint64_t q = p->q, q_mod_t = q % t;
  for (size_t i = 0; i < n; i++) {
    uint64_t x = mont_export(p, acc[i]);
    if (x > (q >> 1)) x -= q_mod_t;
    out[i] = x % t;
  }
  free(acc);
  free(pw);
  free(ci);
}

/* RnsGaloisKey::PrecomputeRandomPad (rns/rns_galois_key.cc:289-306) and
 * ApplyToRlweCiphertextWithRandomPad (:308-346): with the gadget digits of
 * c1 given in NTT form (pad [k][L][n]), out [2][L][n] =
 * (c0 + sum_j pad_j * key_b_j, sum_j pad_j * key_a_j). */
void so_rns_galois_pad(const so_rns* r, int L, int k, const uint64_t* ct,
                       const uint64_t* pad, const uint64_t* key_b, const uint64_t* key_a,
                       uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n, P = (size_t)L * n;
  memcpy(out, ct, P * sizeof(uint64_t));
  memset(out + P, 0, P * sizeof(uint64_t));
  for (int j = 0; j < k; j++)
    for (int l = 0; l < L; l++) {
      const so_prime* p = r->primes[l];
      const size_t o = (size_t)j * P + (size_t)l * n;
      so_fma(p, out + (size_t)l * n, pad + o, key_b + o, n);
      so_fma(p, out + P + (size_t)l * n, pad + o, key_a + o, n);
    }
}

/* ---- ChaCha PRNG, samplers and BGV encryption -------------------------- */

/* One ChaCha20 keystream block (RFC 7539 section 2.3.2). */
void so_chacha20_block(const uint8_t key[32], uint32_t counter, const uint8_t nonce[12],
                       uint8_t out[64]) {
  shg_chacha20_block(key, counter, nonce, out);
}

void so_prng_bytes(const uint8_t seed[32], uint64_t start, size_t len, uint8_t* out) {
  shg_chacha_prng_bytes(seed, start, len, out);
}

static uint64_t prng_rand64(const uint8_t seed[32], uint64_t* pos) {
  uint8_t b[8];
  shg_chacha_prng_bytes(seed, *pos, 8, b);
  *pos += 8;
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)b[i] << (8 * i);
  return v;
}

static uint8_t prng_rand8(const uint8_t seed[32], uint64_t* pos) {
  uint8_t b;
  shg_chacha_prng_bytes(seed, *pos, 1, &b);
  *pos += 1;
  return b;
}

static int popcount64(uint64_t x) {
  int c = 0;
  while (x) {
    x &= x - 1;
    c++;
  }
  return c;
}

/* One coefficient of SampleFromErrorDistribution (sample_error.h:43-100):
 * the centred binomial sum over 2 * variance bit pairs (64 pairs per two
 * Rand64, 8 per two Rand8, the rest from two masked Rand8), mod q. */
static uint64_t cbd_mod_q(const so_prime* p, int variance, const uint8_t seed[32],
                          uint64_t* pos) {
  uint64_t c = p->q;
  int k = 2 * variance;
  while (k > 0) {
    if (k >= 64) {
      c += popcount64(prng_rand64(seed, pos));
      c -= popcount64(prng_rand64(seed, pos));
      k -= 64;
    } else if (k >= 8) {
      c += popcount64(prng_rand8(seed, pos));
      c -= popcount64(prng_rand8(seed, pos));
      k -= 8;
    } else {
      const uint8_t m = (uint8_t)((1u << k) - 1);
      c += popcount64(prng_rand8(seed, pos) & m);
      c -= popcount64(prng_rand8(seed, pos) & m);
      break;
    }
  }
  return c >= p->q ? c - p->q : c;
}

/* RnsPolynomial::SampleUniform (rns/rns_polynomial.h:638-667): limb by limb,
 * each coefficient the first 8-byte candidate (Rand64, masked to log q bits)
 * below q (MontgomeryInt::ImportRandom, montgomery.h:261-272, 629-655); the
 * value is taken as the Montgomery representation.  Then SampleError
 * (rns/error_distribution.h:40-60): centred binomial coefficients of
 * variance `variance` mod q_0 (SampleFromErrorDistribution,
 * sample_error.h:43-100), lifted balanced to every limb and put in NTT form.
 * Both from the PRNG stream of `seed` starting at *pos. */
static void sample_uniform_error(const so_rns* r, int L, int variance, const uint8_t seed[32],
                                 uint64_t* pos, uint64_t* a, uint64_t* e) {
  const size_t n = (size_t)1 << r->log_n;
  for (int l = 0; l < L; l++) {
    const so_prime* p = r->primes[l];
    const uint64_t mask = p->log_q >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << p->log_q) - 1);
    for (size_t j = 0; j < n; j++) {
      uint64_t v;
      do {
        v = prng_rand64(seed, pos) & mask;
      } while (v >= p->q);
      a[(size_t)l * n + j] = v;
    }
  }
  const so_prime* p0 = r->primes[0];
  for (size_t j = 0; j < n; j++) {
    const uint64_t c = cbd_mod_q(p0, variance, seed, pos);
    /* ConvertModulusBalanced (modulus_conversion.h:30-157) of c (mod q0) */
    for (int l = 0; l < L; l++) {
      const so_prime* p = r->primes[l];
      uint64_t v;
      if (c > (p0->q >> 1))
        v = p->q - ((p0->q - c) % p->q);
      else
        v = c % p->q;
      if (v == p->q) v = 0;
      e[(size_t)l * n + j] = mont_import(p, v);
    }
  }
  for (int l = 0; l < L; l++) so_ntt_fwd(r->primes[l], e + (size_t)l * n);
}

void so_rns_sample_uniform_error(const so_rns* r, int L, int variance, const uint8_t seed[32],
                                 uint64_t* a, uint64_t* e) {
  uint64_t pos = 0;
  sample_uniform_error(r, L, variance, seed, &pos, a, e);
}

/* RnsRlweSecretKey::EncryptPolynomialBgv (rns/rns_secret_key.h:188-231):
 * a, e drawn from the PRNG of `seed`, c0 = e * t + m + a * s, c1 = -a.
 * key, m [L][n] NTT form; out [2][L][n]. */
void so_rns_encrypt_bgv(const so_rns* r, int L, uint64_t t, int variance, const uint64_t* key,
                        const uint64_t* m, const uint8_t seed[32], uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n, P = (size_t)L * n;
  uint64_t* a = (uint64_t*)malloc(P * sizeof(uint64_t));
  uint64_t pos = 0;
  sample_uniform_error(r, L, variance, seed, &pos, a, out);
  for (int l = 0; l < L; l++) {
    const so_prime* p = r->primes[l];
    const uint64_t tm = mont_import(p, t % p->q);
    uint64_t* c0 = out + (size_t)l * n;
    for (size_t j = 0; j < n; j++) c0[j] = mont_mul(p, c0[j], tm);
    so_add(p, c0, m + (size_t)l * n, c0, n);
    so_fma(p, c0, a + (size_t)l * n, key + (size_t)l * n, n);
    so_neg(p, a + (size_t)l * n, out + P + (size_t)l * n, n);
  }
  free(a);
}

/* SymmetricRlweKey::Sample (symmetric_encryption.h:634-649): n error
 * coefficients (SampleFromErrorDistribution) from the start of the PRNG
 * stream of `seed`, imported and put in NTT form -> s [n]. */
void so_sym_key_sample(const so_prime* p, int variance, const uint8_t seed[32], uint64_t* s) {
  const size_t n = (size_t)p->n;
  uint64_t pos = 0;
  for (size_t j = 0; j < n; j++) s[j] = mont_import(p, cbd_mod_q(p, variance, seed, &pos));
  so_ntt_fwd(p, s);
}

/* rlwe::Encrypt (symmetric_encryption.h:1006-1021) with the PRNG of `seed`:
 * a = SamplePolynomialFromPrng (polynomial.h:361-381; ImportRandom per
 * coefficient, taken as NTT-form values), then internal::Encrypt's error
 * (SampleFromErrorDistribution), c0 = NTT(e) t + m + a s, c1 = -a.
 * s, m [n] NTT form; out [2][n]. */
void so_sym_encrypt_prng(const so_prime* p, uint64_t t, int variance, const uint64_t* s,
                         const uint64_t* m, const uint8_t seed[32], uint64_t* out) {
  const size_t n = (size_t)p->n;
  uint64_t* a = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t* e = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t pos = 0;
  const uint64_t mask = p->log_q >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << p->log_q) - 1);
  for (size_t j = 0; j < n; j++) {
    uint64_t v;
    do {
      v = prng_rand64(seed, &pos) & mask;
    } while (v >= p->q);
    a[j] = v;
  }
  for (size_t j = 0; j < n; j++) e[j] = mont_import(p, cbd_mod_q(p, variance, seed, &pos));
  so_sym_encrypt(p, t, s, a, e, m, out);
  free(a);
  free(e);
}

/* MontgomeryInt::SerializeVector (montgomery.cc:142-166) through
 * TranscribeBits (transcription.h:43-118): the log_q-bit Montgomery
 * representations as one little-endian bit stream -- value i fills stream
 * bits [i*b, i*b + b) from its least significant bit, stream bit j is bit
 * j % 8 of byte j / 8.  Returns ceil(count * b / 8), the bytes written. */
size_t so_serialize_vector(const so_prime* p, const uint64_t* in, size_t count,
                           uint8_t* out) {
  const int b = p->log_q;
  const size_t bytes = (count * (size_t)b + 7) / 8;
  memset(out, 0, bytes);
  for (size_t i = 0; i < count; i++)
    for (int k = 0; k < b; k++) {
      const size_t pos = i * (size_t)b + (size_t)k;
      out[pos >> 3] |= (uint8_t)(((in[i] >> k) & 1u) << (pos & 7));
    }
  return bytes;
}

/* MontgomeryInt::DeserializeVector (montgomery.cc:186-215): the inverse bit
 * stream; values are taken as Montgomery representations unchecked, as the
 * reference does. */
void so_deserialize_vector(const so_prime* p, const uint8_t* in, size_t count,
                           uint64_t* out) {
  const int b = p->log_q;
  for (size_t i = 0; i < count; i++) {
    uint64_t v = 0;
    for (int k = 0; k < b; k++) {
      const size_t pos = i * (size_t)b + (size_t)k;
      v |= (uint64_t)((in[pos >> 3] >> (pos & 7)) & 1u) << k;
    }
    out[i] = v;
  }
}

/* ObliviousExpander::ComputeNormalizer (oblivious_expand.h:143-157). */
uint64_t so_compute_normalizer(int k, int log_t) {
  int log_t_minus_r = log_t - (k % log_t);
  int pp = k / log_t;
  if (pp % 2 == 0)
    return (((uint64_t)1 << log_t) + 1) - ((uint64_t)1 << log_t_minus_r);
  return (uint64_t)1 << log_t_minus_r;
}

/* ---------------------------------------------------------------------------
 * RNS basis conversion and BFV (rns/rns_polynomial.cc:349-852,
 * rns/rns_polynomial.h:458-490, rns/rns_bfv_ciphertext.cc:33-205).  The
 * so_rns holds the main primes first and the auxiliary primes after them;
 * index lists name primes of that context.
 * ------------------------------------------------------------------------- */

/* prod_{k != skip} primes[idx[k]] mod p (Montgomery rep). */
static uint64_t prod_mod(const so_rns* r, const int* idx, int cnt, int skip,
                         const so_prime* p) {
  uint64_t acc = p->r_mod_q;
  for (int k = 0; k < cnt; k++)
    if (k != skip) acc = mont_mul(p, acc, mont_import(p, r->primes[idx[k]]->q));
  return acc;
}

static uint64_t mont_inverse(const so_prime* p, uint64_t x) {
  return mont_pow(p, x, p->q - 2);
}

/* SwitchRnsBasis (rns/rns_polynomial.cc:419-525) when scale == 0, and
 * ScaleAndSwitchRnsBasis (:527-640) when scale == 1, for Q = prod src and
 * P = prod dst:
 *   s_i = a_i * [P mod q_i if scale] * (Q/q_i)^-1 mod q_i,
 *   u = round(sum_i (double)s_i / (double)q_i), summed in order i = 0..,
 *   out_j = sum_i s_i * (Q/q_i mod p_j) - u * (Q mod p_j)         (scale 0)
 *   out_j = sum_i s_i * (-q_i^-1 mod p_j) + u                      (scale 1).
 * in [ns][n] and out [nd][n] coefficient form. */
static void switch_basis(const so_rns* r, const int* src, int ns, const int* dst, int nd,
                         int scale, const uint64_t* in, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  uint64_t* s = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)ns * n);
  double* us = (double*)calloc(n, sizeof(double));
  for (int i = 0; i < ns; i++) {
    const so_prime* qi = r->primes[src[i]];
    const uint64_t qhat_inv = mont_inverse(qi, prod_mod(r, src, ns, i, qi));
    const uint64_t pmod = scale ? prod_mod(r, dst, nd, -1, qi) : 0;
    const double qd = (double)qi->q;
    for (size_t k = 0; k < n; k++) {
      uint64_t x = in[(size_t)i * n + k];
      if (scale) x = mont_mul(qi, x, pmod);
      x = mont_mul(qi, x, qhat_inv);
      s[(size_t)i * n + k] = x;
      us[k] += (double)mont_export(qi, x) / qd;
    }
  }
  for (int j = 0; j < nd; j++) {
    const so_prime* pj = r->primes[dst[j]];
    uint64_t* o = out + (size_t)j * n;
    for (size_t k = 0; k < n; k++) o[k] = 0;
    for (int i = 0; i < ns; i++) {
      const so_prime* qi = r->primes[src[i]];
      uint64_t w;
      if (scale)
        w = mont_neg(pj, mont_inverse(pj, mont_import(pj, qi->q)));
      else
        w = prod_mod(r, src, ns, i, pj);
      for (size_t k = 0; k < n; k++) {
        const uint64_t v = mont_import(pj, mont_export(qi, s[(size_t)i * n + k]));
        o[k] = mont_add(pj, o[k], mont_mul(pj, v, w));
      }
    }
    const uint64_t qmod = prod_mod(r, src, ns, -1, pj);
    for (size_t k = 0; k < n; k++) {
      const uint64_t u = (uint64_t)round(us[k]);
      const uint64_t um = mont_import(pj, u);
      o[k] = scale ? mont_add(pj, o[k], um) : mont_sub(pj, o[k], mont_mul(pj, um, qmod));
    }
  }
  free(s);
  free(us);
}

void so_rns_switch_basis(const so_rns* r, const int* src, int ns, const int* dst, int nd,
                         const uint64_t* in, uint64_t* out) {
  switch_basis(r, src, ns, dst, nd, 0, in, out);
}

void so_rns_scale_switch_basis(const so_rns* r, const int* src, int ns, const int* dst,
                               int nd, const uint64_t* in, uint64_t* out) {
  switch_basis(r, src, ns, dst, nd, 1, in, out);
}

/* ApproxSwitchRnsBasis (rns/rns_polynomial.cc:653-724): a_i * (Q/q_i)^-1 mod
 * q_i (then iNTT when is_ntt), converted to every p_j (balanced or not),
 * times Q/q_i mod p_j, summed.  Output coefficient form. */
void so_rns_approx_switch_basis(const so_rns* r, const int* src, int ns, const int* dst,
                                int nd, int is_ntt, int balanced, const uint64_t* in,
                                uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * n);
  memset(out, 0, sizeof(uint64_t) * (size_t)nd * n);
  for (int i = 0; i < ns; i++) {
    const so_prime* qi = r->primes[src[i]];
    const uint64_t qhat_inv = mont_inverse(qi, prod_mod(r, src, ns, i, qi));
    for (size_t k = 0; k < n; k++) a[k] = mont_mul(qi, in[(size_t)i * n + k], qhat_inv);
    if (is_ntt) so_ntt_inv(qi, a);
    for (int j = 0; j < nd; j++) {
      const so_prime* pj = r->primes[dst[j]];
      const uint64_t w = prod_mod(r, src, ns, i, pj);
      uint64_t* o = out + (size_t)j * n;
      for (size_t k = 0; k < n; k++) {
        const uint64_t x = mont_export(qi, a[k]);
        const uint64_t v = balanced ? convert_balanced(qi, pj, x)
                                    : (qi->q == pj->q ? a[k] : mont_import(pj, x));
        o[k] = mont_add(pj, o[k], mont_mul(pj, v, w));
      }
    }
  }
  free(a);
}

/* ModReduceMsb (rns/rns_polynomial.cc:349-417): round(a / q_{L-1}) mod
 * q_0..q_{L-2}: the last limb (iNTT when is_ntt), lifted balanced to every
 * other limb (NTT when is_ntt), subtracted, times q_{L-1}^-1.  in [L][n] ->
 * out [L-1][n].  3 when L <= 1. */
int so_rns_modreduce_msb(const so_rns* r, int L, int is_ntt, const uint64_t* in,
                         uint64_t* out) {
  if (L <= 1) return 3;
  const size_t n = (size_t)1 << r->log_n;
  const so_prime* ql = r->primes[L - 1];
  uint64_t* last = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint64_t* d = (uint64_t*)malloc(sizeof(uint64_t) * n);
  memcpy(last, in + (size_t)(L - 1) * n, sizeof(uint64_t) * n);
  if (is_ntt) so_ntt_inv(ql, last);
  for (int i = 0; i < L - 1; i++) {
    const so_prime* qi = r->primes[i];
    for (size_t k = 0; k < n; k++) d[k] = convert_balanced(ql, qi, mont_export(ql, last[k]));
    if (is_ntt) so_ntt_fwd(qi, d);
    const uint64_t ql_inv = r->q_invs[(size_t)(L - 1) * r->L + i];
    for (size_t k = 0; k < n; k++)
      out[(size_t)i * n + k] = mont_mul(qi, mont_sub(qi, in[(size_t)i * n + k], d[k]), ql_inv);
  }
  free(last);
  free(d);
  return 0;
}

static void seq_idx(int* idx, int first, int cnt) {
  for (int k = 0; k < cnt; k++) idx[k] = first + k;
}

/* RnsPolynomial::MulInPlace(Int scalar) (rns/rns_polynomial.h:243-259). */
static void mul_int(const so_rns* r, const int* idx, int cnt, uint64_t* poly, uint64_t c) {
  const size_t n = (size_t)1 << r->log_n;
  for (int i = 0; i < cnt; i++) {
    const so_prime* p = r->primes[idx[i]];
    const uint64_t cm = mont_import(p, c);
    for (size_t k = 0; k < n; k++) poly[(size_t)i * n + k] = mont_mul(p, poly[(size_t)i * n + k], cm);
  }
}

static void ntt_idx(const so_rns* r, const int* idx, int cnt, uint64_t* poly, int inverse) {
  const size_t n = (size_t)1 << r->log_n;
  for (int i = 0; i < cnt; i++) {
    if (inverse)
      so_ntt_inv(r->primes[idx[i]], poly + (size_t)i * n);
    else
      so_ntt_fwd(r->primes[idx[i]], poly + (size_t)i * n);
  }
}

/* ScaleAndReduceRnsBasisInPlace (rns/rns_polynomial.h:458-490): main
 * [nm][n] over q_0..q_{nm-1} and aux [na][n] over aux[]:
 * out = (t * main - SwitchRnsBasis(t * aux, aux -> main)) * P^-1 mod Q, in
 * main's form.  Note the reference's SwitchRnsBasis takes P mod q_i for
 * every main prime of the context, so it needs nm == the context's count. */
void so_rns_scale_reduce(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                         int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                         const uint64_t* aux_in, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  int* mi = (int*)calloc(nm, sizeof(int));
  seq_idx(mi, 0, nm);
  uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)na * n);
  uint64_t* delta = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)nm * n);
  memcpy(out, main_in, sizeof(uint64_t) * (size_t)nm * n);
  memcpy(a, aux_in, sizeof(uint64_t) * (size_t)na * n);
  mul_int(r, mi, nm, out, t);
  mul_int(r, aux, na, a, t);
  if (is_ntt_aux) ntt_idx(r, aux, na, a, 1);
  switch_basis(r, aux, na, mi, nm, 0, a, delta);
  if (is_ntt_main) ntt_idx(r, mi, nm, delta, 0);
  for (int i = 0; i < nm; i++) {
    const so_prime* qi = r->primes[i];
    const uint64_t pinv = mont_inverse(qi, prod_mod(r, aux, na, -1, qi));
    for (size_t k = 0; k < n; k++) {
      uint64_t* o = out + (size_t)i * n + k;
      *o = mont_mul(qi, mont_sub(qi, *o, delta[(size_t)i * n + k]), pinv);
    }
  }
  free(mi);
  free(a);
  free(delta);
}

/* ApproxModReduceLsb (rns/rns_polynomial.cc:726-791) when lsb, else
 * ApproxModReduceMsb (:793-852): out [nm][n] NTT form. */
static void approx_modreduce(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                             int lsb, int is_ntt_main, const uint64_t* main_in,
                             int is_ntt_aux, const uint64_t* aux_in, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n;
  int* mi = (int*)calloc(nm, sizeof(int));
  seq_idx(mi, 0, nm);
  uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)na * n);
  uint64_t* delta = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)nm * n);
  memcpy(a, aux_in, sizeof(uint64_t) * (size_t)na * n);
  uint64_t p_mod_t = 0;
  if (lsb) {
    /* P mod t over the integers (rns/rns_context.cc GeneratePlaintextModulusConstants) */
    u128 pm = 1 % t;
    for (int j = 0; j < na; j++) pm = (pm * (r->primes[aux[j]]->q % t)) % t;
    p_mod_t = (uint64_t)pm;
    for (int j = 0; j < na; j++) {
      const so_prime* pj = r->primes[aux[j]];
      const uint64_t rr = mont_import(pj, p_mod_t);
      const uint64_t tinv = mont_neg(pj, mont_inverse(pj, mont_import(pj, t)));
      uint64_t* row = a + (size_t)j * n;
      for (size_t k = 0; k < n; k++) row[k] = mont_mul(pj, mont_mul(pj, row[k], rr), tinv);
    }
  }
  so_rns_approx_switch_basis(r, aux, na, mi, nm, is_ntt_aux, lsb, a, delta);
  ntt_idx(r, mi, nm, delta, 0);
  if (lsb) mul_int(r, mi, nm, delta, t);
  memcpy(out, main_in, sizeof(uint64_t) * (size_t)nm * n);
  if (!is_ntt_main) ntt_idx(r, mi, nm, out, 0);
  if (lsb) mul_int(r, mi, nm, out, p_mod_t);
  for (int i = 0; i < nm; i++) {
    const so_prime* qi = r->primes[i];
    const uint64_t pinv = mont_inverse(qi, prod_mod(r, aux, na, -1, qi));
    for (size_t k = 0; k < n; k++) {
      uint64_t* o = out + (size_t)i * n + k;
      const uint64_t dv = delta[(size_t)i * n + k];
      *o = mont_mul(qi, lsb ? mont_add(qi, *o, dv) : mont_sub(qi, *o, dv), pinv);
    }
  }
  free(mi);
  free(a);
  free(delta);
}

void so_rns_approx_modreduce_lsb(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                                 int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                                 const uint64_t* aux_in, uint64_t* out) {
  approx_modreduce(r, nm, aux, na, t, 1, is_ntt_main, main_in, is_ntt_aux, aux_in, out);
}

void so_rns_approx_modreduce_msb(const so_rns* r, int nm, const int* aux, int na,
                                 int is_ntt_main, const uint64_t* main_in, int is_ntt_aux,
                                 const uint64_t* aux_in, uint64_t* out) {
  approx_modreduce(r, nm, aux, na, 0, 0, is_ntt_main, main_in, is_ntt_aux, aux_in, out);
}

/* RnsBfvCiphertext::Mul (rns/rns_bfv_ciphertext.cc:100-205), after Kim et
 * al.: b_j -> coefficient form -> SwitchRnsBasis to P -> NTT; a_i ->
 * coefficient form -> ScaleAndSwitchRnsBasis to P (round(P/Q a_i)) ->
 * SwitchRnsBasis back to Q -> NTT both; the tensor product mod Q and mod P;
 * each component ScaleAndReduceRnsBasisInPlace'd by t.  a, b [2][nm][n]
 * NTT form over q_0..q_{nm-1} -> out [3][nm][n]. */
void so_bfv_mul(const so_rns* r, int nm, const int* aux, int na, uint64_t t,
                const uint64_t* a, const uint64_t* b, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n, Pm = (size_t)nm * n, Pa = (size_t)na * n;
  int* mi = (int*)calloc(nm, sizeof(int));
  seq_idx(mi, 0, nm);
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * Pm);
  uint64_t* b_aux = (uint64_t*)malloc(sizeof(uint64_t) * 2 * Pa);
  uint64_t* a_aux = (uint64_t*)malloc(sizeof(uint64_t) * 2 * Pa);
  uint64_t* a_main = (uint64_t*)malloc(sizeof(uint64_t) * 2 * Pm);
  uint64_t* t_main = (uint64_t*)calloc(3 * Pm, sizeof(uint64_t));
  uint64_t* t_aux = (uint64_t*)calloc(3 * Pa, sizeof(uint64_t));
  for (int j = 0; j < 2; j++) {
    memcpy(tmp, b + j * Pm, sizeof(uint64_t) * Pm);
    ntt_idx(r, mi, nm, tmp, 1);
    switch_basis(r, mi, nm, aux, na, 0, tmp, b_aux + j * Pa);
    ntt_idx(r, aux, na, b_aux + j * Pa, 0);
  }
  for (int i = 0; i < 2; i++) {
    memcpy(tmp, a + i * Pm, sizeof(uint64_t) * Pm);
    ntt_idx(r, mi, nm, tmp, 1);
    switch_basis(r, mi, nm, aux, na, 1, tmp, a_aux + i * Pa);
    switch_basis(r, aux, na, mi, nm, 0, a_aux + i * Pa, a_main + i * Pm);
    ntt_idx(r, mi, nm, a_main + i * Pm, 0);
    ntt_idx(r, aux, na, a_aux + i * Pa, 0);
  }
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      for (int l = 0; l < nm; l++)
        so_fma(r->primes[l], t_main + (i + j) * Pm + l * n, a_main + i * Pm + l * n,
               b + j * Pm + l * n, n);
      for (int l = 0; l < na; l++)
        so_fma(r->primes[aux[l]], t_aux + (i + j) * Pa + l * n, a_aux + i * Pa + l * n,
               b_aux + j * Pa + l * n, n);
    }
  for (int k = 0; k < 3; k++)
    so_rns_scale_reduce(r, nm, aux, na, t, 1, t_main + k * Pm, 1, t_aux + k * Pa,
                        out + k * Pm);
  free(mi); free(tmp); free(b_aux); free(a_aux); free(a_main); free(t_main); free(t_aux);
}

/* RnsBfvCiphertext::AbsorbInPlace (rns/rns_bfv_ciphertext.cc:33-98): the
 * plaintext (NTT form) is switched to P as for the second factor of Mul;
 * each component is scaled to P, switched back, multiplied by the plaintext
 * mod Q and mod P and scale-reduced by t.  ct [len][nm][n] -> out. */
void so_bfv_absorb(const so_rns* r, int nm, const int* aux, int na, uint64_t t, int len,
                   const uint64_t* ct, const uint64_t* pt, uint64_t* out) {
  const size_t n = (size_t)1 << r->log_n, Pm = (size_t)nm * n, Pa = (size_t)na * n;
  int* mi = (int*)calloc(nm, sizeof(int));
  seq_idx(mi, 0, nm);
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * Pm);
  uint64_t* pt_aux = (uint64_t*)malloc(sizeof(uint64_t) * Pa);
  uint64_t* c_aux = (uint64_t*)malloc(sizeof(uint64_t) * Pa);
  uint64_t* c_main = (uint64_t*)malloc(sizeof(uint64_t) * Pm);
  memcpy(tmp, pt, sizeof(uint64_t) * Pm);
  ntt_idx(r, mi, nm, tmp, 1);
  switch_basis(r, mi, nm, aux, na, 0, tmp, pt_aux);
  ntt_idx(r, aux, na, pt_aux, 0);
  for (int c = 0; c < len; c++) {
    memcpy(tmp, ct + c * Pm, sizeof(uint64_t) * Pm);
    ntt_idx(r, mi, nm, tmp, 1);
    switch_basis(r, mi, nm, aux, na, 1, tmp, c_aux);
    switch_basis(r, aux, na, mi, nm, 0, c_aux, c_main);
    ntt_idx(r, mi, nm, c_main, 0);
    for (int l = 0; l < nm; l++)
      so_mul(r->primes[l], c_main + l * n, pt + l * n, c_main + l * n, n);
    ntt_idx(r, aux, na, c_aux, 0);
    for (int l = 0; l < na; l++)
      so_mul(r->primes[aux[l]], c_aux + l * n, pt_aux + l * n, c_aux + l * n, n);
    so_rns_scale_reduce(r, nm, aux, na, t, 1, c_main, 1, c_aux, out + c * Pm);
  }
  free(mi); free(tmp); free(pt_aux); free(c_aux); free(c_main);
}
