// C ABI of the GB300 RLWE hot path: host-side validation (mirroring the
// reference's absl::Status checks), parameter derivation and kernel
// orchestration.  No CPU fallback: every operation runs on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/shell_gpu.h"
#include "../../include/shell_gpu_runtime.h"
#include "kernels.cuh"

using shg::CtMap;
using shg::CtxDev;
using shg::DigitDesc;
using shg::PrimeDev;
using shg::ScalarPack;
using shg::Tw;
typedef unsigned __int128 u128;

namespace {

thread_local std::string t_last_error;

int fail(int code, const std::string& msg) {
  t_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(SHG_INTERNAL, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SHG_CUDA(call)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);  \
  } while (0)

// ---- host modular arithmetic (parameter setup only) -----------------------
uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) {
  return (uint64_t)(((u128)a * b) % q);
}
uint64_t powmod(uint64_t b, uint64_t e, uint64_t q) {
  uint64_t r = 1 % q;
  b %= q;
  while (e) {
    if (e & 1) r = mulmod(r, b, q);
    b = mulmod(b, b, q);
    e >>= 1;
  }
  return r;
}
uint64_t to_mont(uint64_t x, uint64_t q) {
  return (uint64_t)(((u128)(x % q) << 64) % q);
}
uint64_t from_mont(uint64_t xm, uint64_t q, uint64_t inv_r) {
  return mulmod(xm, inv_r, q);
}
uint64_t shoup_of(uint64_t w, uint64_t q) {
  return (uint64_t)(((u128)w << 64) / q);
}
int bit_length(uint64_t x) {
  int b = 0;
  while (x) {
    ++b;
    x >>= 1;
  }
  return b;
}
uint32_t bitrev(uint32_t x, int bits) {
  uint32_t r = 0;
  for (int i = 0; i < bits; ++i) {
    r = (r << 1) | (x & 1);
    x >>= 1;
  }
  return r;
}

// Everything the host keeps about one prime at the context's ring degree.
struct HostPrime {
  uint64_t q = 0;
  int log_q = 0;
  uint64_t inv_modulus = 0, r_mod_q = 0, r_mod_q_barrett = 0, inv_r = 0,
           inv_r_barrett = 0, barrett_num = 0;
  uint64_t psi = 0;      // plain
  uint64_t n_inv = 0;    // plain
  std::vector<uint64_t> fwd, inv;  // plain twiddles (psi^{brv i}, psi^{-(brv i + 1)})
};

// Validations of MontgomeryIntParams::Create (montgomery.cc:44-59) and
// InitializeNttParameters (ntt_parameters.h:183-203).
int make_prime(uint64_t q, int log_n, HostPrime* hp) {
  if ((q >> 62) != 0)
    return fail(SHG_INVALID_ARGUMENT, "The modulus should be less than 2^62.");
  if ((q & 1) == 0) return fail(SHG_INVALID_ARGUMENT, "The modulus should be odd.");
  const uint64_t two_n = (uint64_t)1 << (log_n + 1);
  if (q % two_n != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "modulus is not 1 mod 2n for logn, " + std::to_string(log_n));
  const int n = 1 << log_n;
  hp->q = q;
  hp->log_q = bit_length(q);
  const u128 R = (u128)1 << 64;
  hp->r_mod_q = (uint64_t)(R % q);
  hp->inv_r = powmod(hp->r_mod_q, q - 2, q);  // R^{-1} (q prime)
  // inv_modulus = -q^{-1} mod 2^64 via Newton iteration.
  uint64_t inv = q;
  for (int i = 0; i < 6; ++i) inv *= 2 - q * inv;
  hp->inv_modulus = (uint64_t)0 - inv;
  hp->r_mod_q_barrett = shoup_of(hp->r_mod_q, q);
  hp->inv_r_barrett = shoup_of(hp->inv_r, q);
  hp->barrett_num = (uint64_t)(R / q);
  // n^{-1} = n^{q-2} as MultiplicativeInverse does (montgomery.cc:494-498).
  hp->n_inv = powmod((uint64_t)n, q - 2, q);
  // psi: the first t >= 2 whose t^{(q-1)/2n} has order exactly 2n
  // (PrimitiveNthRootOfUnity, ntt_parameters.h:41-71).
  const uint64_t k = (q - 1) / two_n;
  uint64_t psi = 0;
  for (uint64_t t = 2; t < q; ++t) {
    uint64_t cand = powmod(t, k, q);
    if (powmod(cand, (uint64_t)n, q) != 1) {
      psi = cand;
      break;
    }
  }
  if (psi == 0)
    return fail(SHG_INTERNAL, "Loop in PrimitiveNthRootOfUnity terminated.");
  hp->psi = psi;
  const uint64_t psi_inv = powmod(psi, q - 2, q);
  std::vector<uint64_t> pw(n + 1), pwi(n + 1);
  pw[0] = 1;
  pwi[0] = 1;
  for (int e = 1; e <= n; ++e) {
    pw[e] = mulmod(pw[e - 1], psi, q);
    pwi[e] = mulmod(pwi[e - 1], psi_inv, q);
  }
  hp->fwd.resize(n);
  hp->inv.resize(n);
  for (int i = 0; i < n; ++i) {
    const uint32_t b = bitrev((uint32_t)i, log_n);
    hp->fwd[i] = pw[b];        // psis_bitrev[i]
    hp->inv[i] = pwi[b + 1];   // psis_inv_bitrev[i] (ntt_parameters.h:131-157)
  }
  return SHG_OK;
}

}  // namespace

namespace shg {
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace shg

// ---------------------------------------------------------------------------
// Context and key objects
// ---------------------------------------------------------------------------

struct shg_context {
  int log_n = 0, n = 0, L = 0;
  int K = 0;  // auxiliary primes (BFV basis extension), after the L main ones
  // Basis-conversion tables (BasisConv) by slot, see conv_slot(); K > 0 only.
  shg::BasisConv* d_conv = nullptr;
  std::vector<uint8_t> conv_fast;  // per table: takes the specialised kernel
  uint64_t t = 0;
  int device = 0;
  int sms = 152;  // multiprocessors of `device`
  std::vector<HostPrime> hp;
  PrimeDev* d_primes = nullptr;
  Tw* d_tw_fwd = nullptr;
  Tw* d_tw_inv = nullptr;
  uint64_t* d_qmod = nullptr;
  std::vector<uint64_t> qmod;  // [L][L] q_i mod q_j
  uint64_t* ws = nullptr;      // scratch for batched pipelines
  size_t ws_bytes = 0;
  int chunk_cts = 0;
  int small_q = 0;  // all moduli below 2^58
  int narrow_q = 0;  // all moduli below 2^45
  int ntt4_min = 13;  // four-step transforms from this log_n up (measured faster
                      // for every operation from n = 2^13; mixed at 2^12)
  int ntt4_plain_min = 12;  // plain forward / inverse NTTs: four-step from 2^12
                            // (8-10 % faster there) unless the threshold is set
                            // above 13
  int ks_fused = 1;   // fused digit row phase + key inner product
  int ks_lanes = 2;      // streams the batched key-switch chunks rotate over (1..4)
  // Host pipeline shape, measured fastest on a GB300 for 1024 pairs at
  // n = 2^14, L = 6 (18.2 ms against 22.3 ms with fixed pieces of 128):
  int host_piece = 32;  // ciphertexts per piece
  int host_slots = 4;   // device staging slots in flight
  int host_ramp = 2;    // first/last pieces start at piece >> ramp (0: none)
  std::mutex mu;
  // Host-buffer pipeline: device staging slots and three streams.
  uint64_t* io = nullptr;
  size_t io_bytes = 0;
  cudaStream_t io_streams[3] = {nullptr, nullptr, nullptr};  // copy in, compute, copy out
  // Second stream of the batched key switch (chunks alternate between the
  // caller's stream and this one) with its fork / join events.
  static constexpr int kMaxKsLanes = 4;
  cudaStream_t ks_side[kMaxKsLanes - 1] = {};
  cudaEvent_t ks_fork = nullptr;
  cudaEvent_t ks_join[kMaxKsLanes - 1] = {};
  // Key-switch lanes of the host-buffer pipeline.
  cudaStream_t io_lanes[kMaxKsLanes] = {};
  std::mutex io_mu;

  CtxDev dev() const {
    return CtxDev{log_n, n, L, d_primes, d_tw_fwd, d_tw_inv, d_qmod, small_q, ntt4_min,
                  ks_fused, sms, ntt4_plain_min, narrow_q};
  }
  // The auxiliary primes as a context of their own (NTTs and pointwise ops
  // over aux limbs); there is no cross-prime table in this view.
  CtxDev aux_dev() const {
    return CtxDev{log_n, n, K, d_primes + L, d_tw_fwd + (size_t)L * n,
                  d_tw_inv + (size_t)L * n, nullptr, small_q, ntt4_min, ks_fused, sms,
                  ntt4_plain_min, narrow_q};
  }
  int ensure_ws(size_t bytes) {
    if (bytes <= ws_bytes) return SHG_OK;
    if (ws) {
      SHG_CUDA(cudaDeviceSynchronize());
      cudaFree(ws);
      ws = nullptr;
      ws_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ws, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(SHG_RESOURCE_EXHAUSTED,
                  "cannot reserve " + std::to_string(bytes) +
                      " bytes of device scratch: " + cudaGetErrorString(e));
    }
    ws_bytes = bytes;
    return SHG_OK;
  }
};

struct shg_key {
  shg_context* ctx = nullptr;
  int L = 0, k = 0, power = 1;
  std::vector<int> log_bs;
  DigitDesc* d_digits = nullptr;
  uint64_t* kb = nullptr;  // [k][L][n], premultiplied by 2^64 mod q
  uint64_t* ka = nullptr;
  int need_lift = 0;
  int digit_flags = 0;  // shg::digit_flags(need_lift, largest log_b)
  int chunk = 1;       // digits per REDC for canonical digit transforms
  int chunk_lazy = 1;  // the same for lazily reduced ones (below 62 q)
  size_t bytes = 0;
};

namespace {

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int check_ptrs(std::initializer_list<const void*> ps) {
  for (const void* p : ps) {
    if (p == nullptr) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
    if (!aligned16(p))
      return fail(SHG_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
  }
  return SHG_OK;
}

int check_limbs(const shg_context* ctx, int count, int num_limbs) {
  if (ctx == nullptr) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (num_limbs <= 0 || num_limbs > ctx->L)
    return fail(SHG_INVALID_ARGUMENT,
                "`moduli` must contain " + std::to_string(num_limbs) +
                    " RNS moduli.");
  return SHG_OK;
}

// Serialized layout of a polynomial of num_limbs limbs (the wire format of
// shg_poly_serialize).
shg::SerLayout ser_layout(const shg_context* ctx, int num_limbs) {
  shg::SerLayout lay{};
  lay.offset[0] = 0;
  for (int l = 0; l < num_limbs; ++l) {
    lay.bits[l] = ctx->hp[l].log_q;
    lay.offset[l + 1] = lay.offset[l] + ((size_t)ctx->n * lay.bits[l] + 7) / 8;
  }
  return lay;
}

int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return SHG_OK;
}

// Cts per pipeline chunk, bounded by the scratch budget.
int chunk_for(shg_context* ctx, size_t per_ct_bytes, int count) {
  int c = ctx->chunk_cts > 0 ? ctx->chunk_cts : 16;
  const size_t budget = (size_t)1 << 30;  // 1 GiB default scratch ceiling
  const size_t cap = std::max<size_t>(1, budget / std::max<size_t>(per_ct_bytes, 1));
  if ((size_t)c > cap) c = (int)cap;
  if (c > count) c = count;
  return std::max(c, 1);
}

// ---- RNS basis conversion tables (BFV) --------------------------------------
//
// Slots of ctx->d_conv for a main prefix q_0..q_l (l = level) and all K
// auxiliary primes p_0..p_{K-1}:
//   l           SwitchRnsBasis main -> aux (MainPrimeModulusCrtFactors(l),
//               MainPrimeModulusComplementResidues(l), MainLeveledModulusAuxResidues(l))
//   L + l       ScaleAndSwitchRnsBasis main -> aux (times P mod q_i,
//               -q_i^-1 mod p_j, MainPrimeModulusInverseAuxResidues)
//   2L + 2l + b ApproxSwitchRnsBasis main -> aux, b = balanced
//   4L + l      SwitchRnsBasis aux -> main q_0..q_l (AuxPrimeModulusCrtFactors,
//               AuxPrimeModulusComplementResidues, AuxModulusResidues)
//   5L + 2l + b ApproxSwitchRnsBasis aux -> main q_0..q_l
//   7L + l      slot 4L + l with the source first multiplied by the context's t
//               (ScaleAndReduceRnsBasisInPlace's t * polynomial_aux)
// (rns/rns_context.cc:169-317 define the tables; every value here is the
// same residue computed directly.)
enum ConvKind { CONV_SWITCH_UP = 0, CONV_SCALE_UP = 1, CONV_APPROX_UP = 2, CONV_SWITCH_DOWN = 4,
                CONV_APPROX_DOWN = 5, CONV_SWITCH_DOWN_T = 7 };

int conv_slot(const shg_context* ctx, int kind, int level, int balanced = 0) {
  const int L = ctx->L;
  switch (kind) {
    case CONV_SWITCH_UP: return level;
    case CONV_SCALE_UP: return L + level;
    case CONV_APPROX_UP: return 2 * L + 2 * level + balanced;
    case CONV_SWITCH_DOWN: return 4 * L + level;
    case CONV_APPROX_DOWN: return 5 * L + 2 * level + balanced;
    default: return 7 * L + level;
  }
}

// prod_{k in [k0, k1), k != skip} hp[k].q mod q (plain).
uint64_t prod_mod(const shg_context* ctx, int k0, int k1, int skip, uint64_t q) {
  uint64_t acc = 1 % q;
  for (int k = k0; k < k1; ++k)
    if (k != skip) acc = mulmod(acc, ctx->hp[k].q % q, q);
  return acc;
}

uint64_t invmod(uint64_t x, uint64_t q) { return powmod(x, q - 2, q); }

// Table for sources [s0, s0 + ns) -> destinations [d0, d0 + nd) of the
// context's prime array.  mode 0 switch, 1 scale and switch, 2 approximate;
// `pre` is a plain factor applied to every source value first.
shg::BasisConv make_conv(const shg_context* ctx, int s0, int ns, int d0, int nd, int mode,
                         int balanced, uint64_t pre) {
  shg::BasisConv bc;
  memset(&bc, 0, sizeof(bc));
  bc.ns = ns;
  bc.nd = nd;
  bc.src0 = s0;
  bc.dst0 = d0;
  bc.mode = mode;
  bc.balanced = balanced;
  // REDC of a 128-bit sum needs it below p * 2^64: sum_i v_i + u < 2^64 per chunk
  u128 bound = 64;
  bc.chunk = 0;
  for (int i = 0; i < ns; ++i) {
    bound += ctx->hp[s0 + i].q;
    if (bound >= ((u128)1 << 64)) break;
    ++bc.chunk;
  }
  if (bc.chunk < 1) bc.chunk = 1;
  for (int i = 0; i < ns; ++i) {
    const uint64_t q = ctx->hp[s0 + i].q;
    uint64_t m = invmod(prod_mod(ctx, s0, s0 + ns, s0 + i, q), q);  // (Q/q_i)^-1
    if (mode == 1) m = mulmod(m, prod_mod(ctx, d0, d0 + nd, -1, q), q);  // * P
    m = mulmod(m, pre % q, q);
    bc.smul[i] = m;
    const u128 two64 = (u128)1 << 64;
    bc.rinv[i] = (uint64_t)(two64 / q);
    bc.rho[i] = (uint64_t)((((u128)(uint64_t)(two64 % q)) << 64) / q);
    bc.qd[i] = (double)q;
  }
  for (int j = 0; j < nd; ++j) {
    const uint64_t p = ctx->hp[d0 + j].q;
    for (int i = 0; i < ns; ++i) {
      const uint64_t qi = ctx->hp[s0 + i].q;
      uint64_t w;
      if (mode == 1)
        w = (p - invmod(qi % p, p)) % p;  // -q_i^-1 mod p_j
      else
        w = prod_mod(ctx, s0, s0 + ns, s0 + i, p);  // (Q/q_i) mod p_j
      const uint64_t wm = to_mont(w, p);
      bc.w[i * nd + j] = wm;
      bc.ws[i * nd + j] = shoup_of(wm, p);
      bc.wq[i * nd + j] = mulmod(qi % p, wm, p);
      bc.w2[i * nd + j] = to_mont(wm, p);
    }
    // mode 0: -u * (Q mod p_j); mode 1: + u (as a Montgomery rep)
    const uint64_t z = mode == 1 ? 1 % p : (p - prod_mod(ctx, s0, s0 + ns, -1, p)) % p;
    bc.z2[j] = to_mont(to_mont(z, p), p);
  }
  return bc;
}

std::vector<shg::BasisConv> make_conv_tables(const shg_context* ctx) {
  const int L = ctx->L, K = ctx->K;
  std::vector<shg::BasisConv> t((size_t)8 * L);
  for (int l = 0; l < L; ++l) {
    const int m = l + 1;
    t[conv_slot(ctx, CONV_SWITCH_UP, l)] = make_conv(ctx, 0, m, L, K, 0, 0, 1);
    t[conv_slot(ctx, CONV_SCALE_UP, l)] = make_conv(ctx, 0, m, L, K, 1, 0, 1);
    for (int b = 0; b < 2; ++b) {
      t[conv_slot(ctx, CONV_APPROX_UP, l, b)] = make_conv(ctx, 0, m, L, K, 2, b, 1);
      t[conv_slot(ctx, CONV_APPROX_DOWN, l, b)] = make_conv(ctx, L, K, 0, m, 2, b, 1);
    }
    t[conv_slot(ctx, CONV_SWITCH_DOWN, l)] = make_conv(ctx, L, K, 0, m, 0, 0, 1);
    t[conv_slot(ctx, CONV_SWITCH_DOWN_T, l)] = make_conv(ctx, L, K, 0, m, 0, 0, ctx->t);
  }
  return t;
}

}  // namespace

extern "C" {

const char* shg_last_error(void) { return t_last_error.c_str(); }

int shg_context_create(int log_n, const uint64_t* qs, int num_qs,
                       uint64_t plaintext_modulus, shg_context** out) {
  return shg_context_create_with_aux(log_n, qs, num_qs, nullptr, 0, plaintext_modulus, out);
}

int shg_context_create_with_aux(int log_n, const uint64_t* qs, int num_qs, const uint64_t* ps,
                                int num_ps, uint64_t plaintext_modulus, shg_context** out) {
  if (out == nullptr) return fail(SHG_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  if (plaintext_modulus == 0)
    return fail(SHG_INVALID_ARGUMENT, "`plaintext_modulus` must be positive.");
  if (log_n <= 0) return fail(SHG_INVALID_ARGUMENT, "`log_n` must be positive.");
  if (log_n > 15)
    return fail(SHG_INVALID_ARGUMENT,
                "log_n, " + std::to_string(log_n) + ", must be less than 15.");
  if (qs == nullptr || num_qs <= 0 || num_qs > shg::kMaxLimbs)
    return fail(SHG_INVALID_ARGUMENT,
                "`qs` must hold between 1 and " + std::to_string(shg::kMaxLimbs) +
                    " prime moduli");
  if (num_ps < 0 || num_ps > shg::kMaxLimbs || (num_ps > 0 && ps == nullptr))
    return fail(SHG_INVALID_ARGUMENT, "`ps` must hold at most " +
                                          std::to_string(shg::kMaxLimbs) + " prime moduli");
  std::vector<uint64_t> all(qs, qs + num_qs);
  if (num_ps > 0) all.insert(all.end(), ps, ps + num_ps);
  for (size_t i = 0; i < all.size(); ++i)
    for (size_t j = 0; j < i; ++j)
      if (all[i] == all[j])
        return fail(SHG_INVALID_ARGUMENT, "the prime moduli must be distinct");
  shg_context* ctx = new shg_context();
  ctx->log_n = log_n;
  ctx->n = 1 << log_n;
  ctx->L = num_qs;
  ctx->K = num_ps;
  ctx->t = plaintext_modulus;
  cudaGetDevice(&ctx->device);
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int NP = num_qs + num_ps;  // main primes, then auxiliary ones
  ctx->hp.resize(NP);
  for (int i = 0; i < NP; ++i) {
    int st = make_prime(all[i], log_n, &ctx->hp[i]);
    if (st != SHG_OK) {
      delete ctx;
      return st;
    }
  }
  const int n = ctx->n, L = num_qs;
  std::vector<PrimeDev> pd(NP);
  std::vector<Tw> twf((size_t)NP * n), twi((size_t)NP * n);
  for (int i = 0; i < NP; ++i) {
    const HostPrime& h = ctx->hp[i];
    PrimeDev& d = pd[i];
    memset(&d, 0, sizeof(d));
    d.q = h.q;
    d.two_q = 2 * h.q;
    d.inv_modulus = h.inv_modulus;
    d.r_mod_q = h.r_mod_q;
    d.r_mod_q_shoup = shoup_of(h.r_mod_q, h.q);
    d.inv_r = h.inv_r;
    d.inv_r_shoup = shoup_of(h.inv_r, h.q);
    d.n_inv = h.n_inv;
    d.n_inv_shoup = shoup_of(h.n_inv, h.q);
    d.n_inv_r = mulmod(h.n_inv, h.inv_r, h.q);
    d.n_inv_r_shoup = shoup_of(d.n_inv_r, h.q);
    d.half_q = h.q >> 1;
    d.log_q = (uint64_t)h.log_q;
    d.barrett = h.barrett_num;
    for (int j = 0; j < n; ++j) {
      twf[(size_t)i * n + j] = Tw{h.fwd[j], shoup_of(h.fwd[j], h.q)};
      twi[(size_t)i * n + j] = Tw{h.inv[j], shoup_of(h.inv[j], h.q)};
    }
  }
  ctx->small_q = 1;
  ctx->narrow_q = 1;
  for (int i = 0; i < NP; ++i) {
    if ((all[i] >> 58) != 0) ctx->small_q = 0;
    if ((all[i] >> 45) != 0) ctx->narrow_q = 0;
  }
  ctx->qmod.resize((size_t)L * L);
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) ctx->qmod[(size_t)i * L + j] = qs[i] % qs[j];
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_primes, sizeof(PrimeDev) * NP);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_tw_fwd, sizeof(Tw) * NP * n);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_tw_inv, sizeof(Tw) * NP * n);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_qmod, sizeof(uint64_t) * L * L);
  if (e == cudaSuccess)
    e = cudaMemcpy(ctx->d_primes, pd.data(), sizeof(PrimeDev) * NP,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(ctx->d_tw_fwd, twf.data(), sizeof(Tw) * NP * n,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(ctx->d_tw_inv, twi.data(), sizeof(Tw) * NP * n,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_ps > 0) {
    std::vector<shg::BasisConv> tables = make_conv_tables(ctx);
    ctx->conv_fast.resize(tables.size());
    for (size_t i = 0; i < tables.size(); ++i) {
      const shg::BasisConv& b = tables[i];
      ctx->conv_fast[i] = !b.balanced && b.ns >= 1 && b.ns <= 8 && b.chunk >= b.ns;
    }
    e = cudaMalloc(&ctx->d_conv, sizeof(shg::BasisConv) * tables.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(ctx->d_conv, tables.data(), sizeof(shg::BasisConv) * tables.size(),
                     cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(ctx->d_qmod, ctx->qmod.data(), sizeof(uint64_t) * L * L,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    shg_context_destroy(ctx);
    return cuda_fail(e, "context upload");
  }
  *out = ctx;
  return SHG_OK;
}

void shg_context_destroy(shg_context* ctx) {
  if (!ctx) return;
  cudaFree(ctx->d_conv);
  cudaFree(ctx->d_primes);
  cudaFree(ctx->d_tw_fwd);
  cudaFree(ctx->d_tw_inv);
  cudaFree(ctx->d_qmod);
  cudaFree(ctx->ws);
  cudaFree(ctx->io);
  for (cudaStream_t s : ctx->io_streams)
    if (s) cudaStreamDestroy(s);
  for (cudaStream_t s : ctx->io_lanes)
    if (s) cudaStreamDestroy(s);
  for (int i = 0; i < shg_context::kMaxKsLanes - 1; ++i) {
    if (ctx->ks_side[i]) cudaStreamDestroy(ctx->ks_side[i]);
    if (ctx->ks_join[i]) cudaEventDestroy(ctx->ks_join[i]);
  }
  if (ctx->ks_fork) cudaEventDestroy(ctx->ks_fork);
  delete ctx;
}

int shg_context_log_n(const shg_context* ctx) { return ctx ? ctx->log_n : -1; }
int shg_context_num_moduli(const shg_context* ctx) { return ctx ? ctx->L : -1; }

int shg_context_prime_info(const shg_context* ctx, int i, uint64_t out[10]) {
  if (!ctx || i < 0 || i >= ctx->L || !out)
    return fail(SHG_INVALID_ARGUMENT, "bad prime index");
  const HostPrime& h = ctx->hp[i];
  out[0] = h.q;
  out[1] = (uint64_t)h.log_q;
  out[2] = h.inv_modulus;
  out[3] = h.r_mod_q;
  out[4] = h.r_mod_q_barrett;
  out[5] = h.inv_r;
  out[6] = h.inv_r_barrett;
  out[7] = h.barrett_num;
  out[8] = h.psi;
  out[9] = to_mont(h.n_inv, h.q);
  return SHG_OK;
}

int shg_context_ntt_tables(const shg_context* ctx, int i, uint64_t* fwd,
                           uint64_t* inv) {
  if (!ctx || i < 0 || i >= ctx->L || !fwd || !inv)
    return fail(SHG_INVALID_ARGUMENT, "bad prime index");
  const HostPrime& h = ctx->hp[i];
  for (int j = 0; j < ctx->n; ++j) {
    fwd[j] = to_mont(h.fwd[j], h.q);
    inv[j] = to_mont(h.inv[j], h.q);
  }
  return SHG_OK;
}

int shg_context_ql_inv(const shg_context* ctx, int level, uint64_t* out) {
  if (!ctx || level < 0 || level >= ctx->L || (!out && level > 0))
    return fail(SHG_INVALID_ARGUMENT,
                "`level` must be non-negative and at most " +
                    std::to_string(ctx ? ctx->L - 1 : 0));
  const uint64_t ql = ctx->hp[level].q;
  for (int j = 0; j < level; ++j) {
    const uint64_t qj = ctx->hp[j].q;
    out[j] = to_mont(powmod(ql % qj, qj - 2, qj), qj);
  }
  return SHG_OK;
}

// ---------------------------------------------------------------------------
// Polynomial operations
// ---------------------------------------------------------------------------

int shg_ntt_forward(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                    shg_stream stream) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({polys}))) return st;
  shg::launch_ntt_fwd(ctx->dev(), polys, polys, count * num_limbs, num_limbs,
                      (cudaStream_t)stream);
  return launch_status("ntt_forward");
}

int shg_ntt_inverse(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                    shg_stream stream) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({polys}))) return st;
  shg::launch_ntt_inv(ctx->dev(), polys, polys, count * num_limbs, num_limbs, 0,
                      (cudaStream_t)stream);
  return launch_status("ntt_inverse");
}

static int pointwise(shg_context* ctx, shg::PwOp op, uint64_t* out,
                     const uint64_t* a, const uint64_t* b,
                     const ScalarPack& sc, int count, int num_limbs,
                     shg_stream stream) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, a}))) return st;
  if (b && (st = check_ptrs({b}))) return st;
  shg::launch_pointwise(ctx->dev(), op, out, a, b, sc, count, num_limbs,
                        (cudaStream_t)stream);
  return launch_status("pointwise");
}

int shg_poly_add(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream s) {
  if (!b) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  return pointwise(ctx, shg::PW_ADD, out, a, b, ScalarPack{}, count, num_limbs, s);
}
int shg_poly_sub(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream s) {
  if (!b) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  return pointwise(ctx, shg::PW_SUB, out, a, b, ScalarPack{}, count, num_limbs, s);
}
int shg_poly_neg(shg_context* ctx, uint64_t* out, const uint64_t* a, int count,
                 int num_limbs, shg_stream s) {
  return pointwise(ctx, shg::PW_NEG, out, a, nullptr, ScalarPack{}, count,
                   num_limbs, s);
}
int shg_poly_mul(shg_context* ctx, uint64_t* out, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream s) {
  if (!b) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  return pointwise(ctx, shg::PW_MUL, out, a, b, ScalarPack{}, count, num_limbs, s);
}
int shg_poly_fma(shg_context* ctx, uint64_t* acc, const uint64_t* a,
                 const uint64_t* b, int count, int num_limbs, shg_stream s) {
  if (!b) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  return pointwise(ctx, shg::PW_FMA, acc, a, b, ScalarPack{}, count, num_limbs, s);
}
int shg_poly_mul_rns_scalar(shg_context* ctx, uint64_t* out, const uint64_t* a,
                            const uint64_t* scalar_mont, int count,
                            int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (!scalar_mont) return fail(SHG_INVALID_ARGUMENT, "null scalar array");
  ScalarPack sc{};
  for (int l = 0; l < num_limbs; ++l) sc.v[l] = scalar_mont[l];
  return pointwise(ctx, shg::PW_MUL_MONT, out, a, nullptr, sc, count, num_limbs, s);
}
int shg_poly_mul_integer(shg_context* ctx, uint64_t* out, const uint64_t* a,
                         uint64_t scalar, int count, int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  ScalarPack sc{};
  for (int l = 0; l < num_limbs; ++l) {
    const uint64_t q = ctx->hp[l].q;
    const uint64_t w = scalar % q;
    sc.v[2 * l] = w;
    sc.v[2 * l + 1] = shoup_of(w, q);
  }
  return pointwise(ctx, shg::PW_MUL_SHOUP, out, a, nullptr, sc, count, num_limbs, s);
}

int shg_poly_substitute(shg_context* ctx, uint64_t* out, const uint64_t* in,
                        int power, int count, int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (power < 0 || (power % 2) == 0 || power >= 2 * ctx->n)
    return fail(SHG_INVALID_ARGUMENT,
                "Substitution power must be a non-negative odd integer less "
                "than 2*n.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  if (out == in) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `in`");
  shg::launch_substitute(ctx->dev(), out, in, power, count, num_limbs,
                         (cudaStream_t)s);
  return launch_status("substitute");
}

int shg_gadget_decompose(shg_context* ctx, int num_limbs, const int* log_bs,
                         uint64_t* out, const uint64_t* in, int count,
                         shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (!log_bs)
    return fail(SHG_INVALID_ARGUMENT,
                "`log_bs` must contain " + std::to_string(num_limbs) + " elements.");
  shg::GadgetBases gb{};
  int k = 0;
  for (int i = 0; i < num_limbs; ++i) {
    if (log_bs[i] <= 0 || log_bs[i] >= 63)
      return fail(SHG_INVALID_ARGUMENT, "log_b must lie in [1, 62]");
    gb.log_b[i] = log_bs[i];
    k += (ctx->hp[i].log_q + log_bs[i] - 1) / log_bs[i];  // GadgetSize (gadget.h:43-47)
  }
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  if (out == in) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `in`");
  shg::launch_decompose(ctx->dev(), out, in, gb, k, count, num_limbs,
                        (cudaStream_t)s);
  return launch_status("gadget decompose");
}

}  // extern "C"

namespace {

// ModReduceLsb (msb = 0, rns/rns_polynomial.cc:262-344) and ModReduceMsb
// (msb = 1, :349-417) share one pipeline: the top limb times k (iNTT and
// ExportInt folded in), lifted balanced to every other limb (NTT), then
// out_i = in_i * c1 + delta_i * c2 with (k, c1, c2) = ((q_l - r) / t,
// r * ql_inv, t * ql_inv) for Lsb (r = q_l mod t) and (1, ql_inv, -ql_inv)
// for Msb.
int modreduce_impl(shg_context* ctx, uint64_t* out, const uint64_t* in, uint64_t t,
                   const uint64_t* ql_inv, int is_ntt, int count, int num_limbs, shg_stream s,
                   int msb) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (num_limbs <= 1)
    return fail(SHG_INVALID_ARGUMENT,
                msb ? "ModReduceMsb cannot apply with only one prime modulus."
                    : "ModReduceLsb cannot apply with only one prime modulus.");
  if (!ql_inv)
    return fail(SHG_INVALID_ARGUMENT,
                "`ql_inv` must be defined with respect to " +
                    std::to_string(num_limbs - 1) + " moduli.");
  if (!msb && t == 0) return fail(SHG_INVALID_ARGUMENT, "`t` must be positive.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  {
    const size_t in_bytes = (size_t)count * num_limbs * ctx->n * sizeof(uint64_t);
    const size_t out_bytes = (size_t)count * (num_limbs - 1) * ctx->n * sizeof(uint64_t);
    const uintptr_t i0 = (uintptr_t)in, o0 = (uintptr_t)out;
    if (o0 < i0 + in_bytes && i0 < o0 + out_bytes)
      return fail(SHG_INVALID_ARGUMENT, "`out` must not overlap `in`");
  }
  const int Lr = num_limbs - 1;
  const HostPrime& hl = ctx->hp[Lr];
  const uint64_t r = msb ? 1 : hl.q % t;
  const uint64_t k = msb ? 1 : (hl.q - r) / t;
  ScalarPack sc{};
  for (int i = 0; i < Lr; ++i) {
    const HostPrime& h = ctx->hp[i];
    const uint64_t qlinv_plain = from_mont(ql_inv[i], h.q, h.inv_r);
    // out = (in * r + delta * t) * ql^{-1} (Lsb) or (in - delta) * ql^{-1}
    // (Msb); in and out are Montgomery, delta is produced in plain form,
    // hence c2 carries an extra 2^64.
    const uint64_t c1 = mulmod(r % h.q, qlinv_plain, h.q);
    const uint64_t tm = msb ? (h.q - 1) : t % h.q;
    const uint64_t c2 = mulmod(mulmod(tm, h.r_mod_q, h.q), qlinv_plain, h.q);
    sc.v[4 * i] = c1;
    sc.v[4 * i + 1] = shoup_of(c1, h.q);
    sc.v[4 * i + 2] = c2;
    sc.v[4 * i + 3] = shoup_of(c2, h.q);
  }
  if (is_ntt) {
    // Scale of the top-limb inverse NTT: k * n^{-1} * 2^-64 mod q_l.
    const uint64_t kp = mulmod(mulmod(k % hl.q, hl.n_inv, hl.q), hl.inv_r, hl.q);
    std::lock_guard<std::mutex> lock(ctx->mu);
    const size_t need = (size_t)count * ctx->n * sizeof(uint64_t);
    if ((st = ctx->ensure_ws(need))) return st;
    shg::launch_modreduce_ntt(ctx->dev(), out, ctx->ws, in, kp,
                              shoup_of(kp, hl.q), sc, count, num_limbs,
                              (cudaStream_t)s);
  } else {
    const uint64_t kp = mulmod(k % hl.q, hl.inv_r, hl.q);
    shg::launch_modreduce_coeff(ctx->dev(), out, in, kp, shoup_of(kp, hl.q), sc,
                                count, num_limbs, (cudaStream_t)s);
  }
  return launch_status(msb ? "modreduce_msb" : "modreduce_lsb");
}

}  // namespace

extern "C" {

int shg_poly_modreduce_lsb(shg_context* ctx, uint64_t* out, const uint64_t* in,
                           uint64_t t, const uint64_t* ql_inv, int is_ntt,
                           int count, int num_limbs, shg_stream s) {
  return modreduce_impl(ctx, out, in, t, ql_inv, is_ntt, count, num_limbs, s, 0);
}

int shg_poly_modreduce_msb(shg_context* ctx, uint64_t* out, const uint64_t* in,
                           const uint64_t* ql_inv, int is_ntt, int count, int num_limbs,
                           shg_stream s) {
  return modreduce_impl(ctx, out, in, 0, ql_inv, is_ntt, count, num_limbs, s, 1);
}

int shg_ct_tensor(shg_context* ctx, uint64_t* out, const uint64_t* a,
                  const uint64_t* b, int count, int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, a, b}))) return st;
  shg::launch_tensor(ctx->dev(), out, a, b, count, num_limbs, (cudaStream_t)s);
  return launch_status("ct_tensor");
}

// ---------------------------------------------------------------------------
// Keys and key switching
// ---------------------------------------------------------------------------

int shg_key_create(shg_context* ctx, int num_limbs, const int* log_bs,
                   int power, const uint64_t* key_b, const uint64_t* key_a,
                   shg_key** out) {
  if (!out) return fail(SHG_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  int st = check_limbs(ctx, 1, num_limbs);
  if (st) return st;
  if (!log_bs)
    return fail(SHG_INVALID_ARGUMENT,
                "`log_bs` must contain " + std::to_string(num_limbs) + " elements.");
  if (!key_b || !key_a) return fail(SHG_INVALID_ARGUMENT, "null key component");
  if (power <= 0 || (power % 2) == 0 || power >= 2 * ctx->n)
    return fail(SHG_INVALID_ARGUMENT,
                "key power must be a positive odd integer less than 2*n");
  shg_key* key = new shg_key();
  key->ctx = ctx;
  key->L = num_limbs;
  key->power = power;
  std::vector<DigitDesc> dd;
  uint64_t qmax = 0;
  for (int i = 0; i < num_limbs; ++i) {
    const int b = log_bs[i];
    const HostPrime& h = ctx->hp[i];
    if (b <= 0 || b >= 63) {
      delete key;
      return fail(SHG_INVALID_ARGUMENT, "log_b must lie in [1, 62]");
    }
    key->log_bs.push_back(b);
    const int dims = (h.log_q + (b - 1)) / b;  // GadgetSize (gadget.h:43-47)
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    for (int d = 0; d < dims; ++d) dd.push_back(DigitDesc{i, d * b, mask});
    if (mask > (h.q >> 1)) key->need_lift = 1;
    for (int j = 0; j < num_limbs; ++j)
      if (mask >= ctx->hp[j].q) key->need_lift = 1;
    qmax = std::max(qmax, h.q);
  }
  key->k = (int)dd.size();
  key->digit_flags =
      shg::digit_flags(key->need_lift, *std::max_element(key->log_bs.begin(), key->log_bs.end()));
  key->chunk = (int)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)key->k, (~(uint64_t)0) / qmax));
  // The fused row kernel keeps the digit transforms lazily reduced when every
  // prime is below 2^58: values below 62 q (inputs below 2q, at most 4q of
  // growth in each of up to 15 levels), so a REDC of `chunk_lazy` products
  // stays below q * 2^64.
  key->chunk_lazy = (qmax >> 58) ? key->chunk
                                 : (int)std::max<uint64_t>(
                                       1, std::min<uint64_t>((uint64_t)key->k,
                                                             (~(uint64_t)0) / (62 * qmax)));
  const size_t elems = (size_t)key->k * num_limbs * ctx->n;
  key->bytes = 2 * elems * sizeof(uint64_t) + dd.size() * sizeof(DigitDesc);
  cudaError_t e = cudaMalloc(&key->kb, elems * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMalloc(&key->ka, elems * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMalloc(&key->d_digits, dd.size() * sizeof(DigitDesc));
  if (e == cudaSuccess)
    e = cudaMemcpy(key->kb, key_b, elems * sizeof(uint64_t), cudaMemcpyDefault);
  if (e == cudaSuccess)
    e = cudaMemcpy(key->ka, key_a, elems * sizeof(uint64_t), cudaMemcpyDefault);
  if (e == cudaSuccess)
    e = cudaMemcpy(key->d_digits, dd.data(), dd.size() * sizeof(DigitDesc),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaGetLastError();
    shg_key_destroy(key);
    return fail(SHG_RESOURCE_EXHAUSTED,
                std::string("key upload failed: ") + cudaGetErrorString(e));
  }
  // Key form: multiply by 2^64 mod q so that REDC of (plain digit NTT) x
  // (key) yields the Montgomery representation of their product.
  ScalarPack sc{};
  for (int l = 0; l < num_limbs; ++l) {
    sc.v[2 * l] = ctx->hp[l].r_mod_q;
    sc.v[2 * l + 1] = shoup_of(ctx->hp[l].r_mod_q, ctx->hp[l].q);
  }
  shg::launch_pointwise(ctx->dev(), shg::PW_MUL_SHOUP, key->kb, key->kb, nullptr,
                        sc, key->k, num_limbs, 0);
  shg::launch_pointwise(ctx->dev(), shg::PW_MUL_SHOUP, key->ka, key->ka, nullptr,
                        sc, key->k, num_limbs, 0);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    shg_key_destroy(key);
    return cuda_fail(e, "key conversion");
  }
  *out = key;
  return SHG_OK;
}

void shg_key_destroy(shg_key* key) {
  if (!key) return;
  cudaFree(key->kb);
  cudaFree(key->ka);
  cudaFree(key->d_digits);
  delete key;
}

int shg_key_num_limbs(const shg_key* key) { return key ? key->L : 0; }
int shg_key_log_bs(const shg_key* key, int* log_bs, int max) {
  if (!key || !log_bs) return fail(SHG_INVALID_ARGUMENT, "null argument");
  if (max < key->L) return fail(SHG_INVALID_ARGUMENT, "`log_bs` array too short");
  for (int i = 0; i < key->L; ++i) log_bs[i] = key->log_bs[i];
  return SHG_OK;
}
int shg_key_power(const shg_key* key) { return key ? key->power : 0; }
shg_context* shg_key_context(const shg_key* key) { return key ? key->ctx : nullptr; }
int shg_key_dimension(const shg_key* key) { return key ? key->k : -1; }
size_t shg_key_device_bytes(const shg_key* key) { return key ? key->bytes : 0; }

namespace {

// Shared key-switch pipeline: X = export(iNTT(component)), D = NTT(digits),
// out = base + <D, key>.
struct KsArgs {
  const uint64_t* ct;  // source ciphertexts
  int ncomp;           // components per source ciphertext
  int comp;            // component to decompose
  int subst_power;     // > 0: substitute first (Galois rotation)
  int base1_zero;      // Galois: c1' has no base term
};

int upload_key_table(const shg_key* const* keys, int count, int stride, int offset,
                     const uint64_t** dst, shg::KeyTable* out, cudaStream_t s);

// Gadget key switch of component a.comp of `count` ciphertexts; with `keys`,
// member i uses keys[i] (same gadget shape as `key`).
int keyswitch(shg_context* ctx, const shg_key* key, uint64_t* out,
              const KsArgs& a, int count, cudaStream_t s,
              const shg_key* const* keys = nullptr) {
  const int L = key->L, n = ctx->n, k = key->k;
  const size_t Ln = (size_t)L * n;
  const size_t per_ct = (Ln + (size_t)k * Ln) * sizeof(uint64_t);
  const int C = chunk_for(ctx, per_ct, count);
  const size_t tab_bytes = keys ? 2 * (size_t)count * sizeof(void*) : 0;
  std::lock_guard<std::mutex> lock(ctx->mu);
  int st = ctx->ensure_ws(per_ct * C + tab_bytes);
  if (st) return st;
  uint64_t* X = ctx->ws;
  uint64_t* D = X + (size_t)C * Ln;
  shg::KeyTable table;
  if (keys &&
      (st = upload_key_table(keys, count, 1, 0,
                             reinterpret_cast<const uint64_t**>(D + (size_t)C * k * Ln),
                             &table, s)))
    return st;
  const CtxDev dv = ctx->dev();
  for (int c0 = 0; c0 < count; c0 += C) {
    const int cc = std::min(C, count - c0);
    const uint64_t* src = a.ct + (size_t)c0 * a.ncomp * Ln;
    shg::launch_intt_export(dv, X, src, a.ncomp, a.comp, a.subst_power,
                            CtMap::identity(), cc, L, s);
    shg::KeyTable kt;
    if (keys) kt = shg::KeyTable{table.kb + c0, table.ka + c0, 0, count - c0};
    shg::launch_keyswitch(dv, D, X, key->d_digits, k, key->digit_flags, key->chunk, key->chunk_lazy,
                          key->kb, key->ka, out + (size_t)c0 * 2 * Ln, src,
                          (size_t)a.ncomp * Ln, CtMap::identity(), a.base1_zero,
                          a.subst_power, cc, L, s, kt);
  }
  return launch_status("keyswitch");
}

int check_key(const shg_context* ctx, const shg_key* key) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (!key) return fail(SHG_INVALID_ARGUMENT, "null key");
  if (key->ctx != ctx)
    return fail(SHG_INVALID_ARGUMENT,
                "`ciphertext` does not have a matching RNS moduli set.");
  return SHG_OK;
}

// keys[i * stride] for i < count must share the first key's context, limbs,
// gadget (log_bs) and substitution power.
int check_same_shape(const shg_context* ctx, const shg_key* const* keys, int count,
                     int stride) {
  if (!keys) return fail(SHG_INVALID_ARGUMENT, "null key list");
  int st = check_key(ctx, keys[0]);
  if (st) return st;
  const shg_key* k0 = keys[0];
  for (int i = 1; i < count; ++i) {
    const shg_key* k = keys[(size_t)i * stride];
    if ((st = check_key(ctx, k))) return st;
    if (k->L != k0->L || k->log_bs != k0->log_bs || k->power != k0->power)
      return fail(SHG_INVALID_ARGUMENT,
                  "keys of one batch must share their moduli, gadget and power");
  }
  return SHG_OK;
}

// Device tables of kb / ka pointers for keys[i * stride + offset], i < count,
// written into `dst` (2 * count pointers of device scratch).  The source is
// pageable host memory, so the call is not graph-capturable.
int upload_key_table(const shg_key* const* keys, int count, int stride, int offset,
                     const uint64_t** dst, shg::KeyTable* out, cudaStream_t s) {
  std::vector<const uint64_t*> h(2 * (size_t)count);
  for (int i = 0; i < count; ++i) {
    const shg_key* k = keys[(size_t)i * stride + offset];
    h[i] = k->kb;
    h[count + i] = k->ka;
  }
  SHG_CUDA(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(void*), cudaMemcpyHostToDevice,
                           s));
  *out = shg::KeyTable{dst, dst + count, 0, count};
  return SHG_OK;
}

// RnsBgvCiphertext::operator* then RnsRelinKey::ApplyTo over a batch; with
// `keys`, member i uses keys[i] (same gadget shape as `key`).
int mul_relin_impl(shg_context* ctx, const shg_key* key, const shg_key* const* keys,
                   uint64_t* out, const uint64_t* a, const uint64_t* b, int count,
                   cudaStream_t s) {
  int st;
  const int L = key->L, n = ctx->n, k = key->k;
  const size_t Ln = (size_t)L * n;
  // Phase 1 over the whole batch (one launch fills the GPU): tensor product
  // and the exported coefficients X of every degree-2 component.  Phase 2 in
  // chunks of the digit NTTs D and the key inner product.
  const size_t x_bytes = (size_t)count * Ln * sizeof(uint64_t);
  const size_t d_per_ct = (size_t)k * Ln * sizeof(uint64_t);
  // 16 ciphertexts per chunk measured fastest at n = 2^14, L = 6 (the digit
  // kernel's grid is then ~13.8 K CTAs).
  int C = ctx->chunk_cts > 0 ? ctx->chunk_cts
                             : (int)std::max<size_t>(1, ((size_t)256 << 20) / d_per_ct);
  C = std::min(C, 16);
  C = std::max(1, std::min(C, count));
  const size_t tab_bytes = keys ? 2 * (size_t)count * sizeof(void*) : 0;
  std::lock_guard<std::mutex> lock(ctx->mu);
  // Chunks rotate over the caller's stream and up to three more (ks_lanes in
  // all), each lane with its own digit scratch, so one chunk's kernels fill
  // another's tail.  The extra streams are created outside any stream
  // capture (the first call).
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  SHG_CUDA(cudaStreamIsCapturing(s, &cap));
  if (!ctx->ks_fork && cap == cudaStreamCaptureStatusNone) {
    SHG_CUDA(cudaEventCreateWithFlags(&ctx->ks_fork, cudaEventDisableTiming));
    for (int i = 0; i < shg_context::kMaxKsLanes - 1; ++i) {
      SHG_CUDA(cudaStreamCreateWithFlags(&ctx->ks_side[i], cudaStreamNonBlocking));
      SHG_CUDA(cudaEventCreateWithFlags(&ctx->ks_join[i], cudaEventDisableTiming));
    }
  }
  const int nchunks = (count + C - 1) / C;
  const int lanes = ctx->ks_fork ? std::max(1, std::min(ctx->ks_lanes, nchunks)) : 1;
  if ((st = ctx->ensure_ws(x_bytes + lanes * d_per_ct * C + tab_bytes))) return st;
  uint64_t* X = ctx->ws;
  uint64_t* D0 = X + (size_t)count * Ln;
  shg::KeyTable kt;
  if (keys &&
      (st = upload_key_table(keys, count, 1, 0,
                             reinterpret_cast<const uint64_t**>(D0 + (size_t)lanes * C * k * Ln),
                             &kt, s)))
    return st;
  const CtxDev dv = ctx->dev();
  shg::launch_tensor_intt(dv, out, X, a, b, count, L, s);
  if (lanes > 1) {
    SHG_CUDA(cudaEventRecord(ctx->ks_fork, s));
    for (int i = 0; i + 1 < lanes; ++i)
      SHG_CUDA(cudaStreamWaitEvent(ctx->ks_side[i], ctx->ks_fork, 0));
  }
  for (int i = 0; i < nchunks; ++i) {
    const int c0 = i * C, cc = std::min(C, count - c0);
    const int lane = i % lanes;
    cudaStream_t ls = lane ? ctx->ks_side[lane - 1] : s;
    uint64_t* o = out + (size_t)c0 * 2 * Ln;
    shg::KeyTable kc;
    if (keys) kc = shg::KeyTable{kt.kb + c0, kt.ka + c0, 0, count - c0};
    shg::launch_keyswitch(dv, D0 + (size_t)lane * C * k * Ln, X + (size_t)c0 * Ln,
                          key->d_digits, k, key->digit_flags, key->chunk, key->chunk_lazy,
                          key->kb, key->ka, o, o, 2 * Ln, CtMap::identity(), 0, 0, cc, L, ls,
                          kc);
  }
  for (int i = 0; i + 1 < lanes; ++i) {
    SHG_CUDA(cudaEventRecord(ctx->ks_join[i], ctx->ks_side[i]));
    SHG_CUDA(cudaStreamWaitEvent(s, ctx->ks_join[i], 0));
  }
  return launch_status("bgv_mul_relin");
}

}  // namespace

int shg_relin_apply(shg_context* ctx, const shg_key* key, uint64_t* out,
                    const uint64_t* ct, int count, shg_stream s) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (key->power != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "Relinearization key can only apply to a ciphertext of power 1.");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  return keyswitch(ctx, key, out, KsArgs{ct, 3, 2, 0, 0}, count, (cudaStream_t)s);
}

int shg_galois_apply(shg_context* ctx, const shg_key* key, uint64_t* out,
                     const uint64_t* ct, int count, shg_stream s) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  return keyswitch(ctx, key, out, KsArgs{ct, 2, 1, 0, 1}, count, (cudaStream_t)s);
}

}  // extern "C"

namespace {
// Host-buffer ct-mult+relin pipeline.  wire: a, b, out hold serialized
// ciphertexts (shg_poly_serialize layout, two polynomials each), which cross
// the host link packed and are (de)serialized on the device.
int mul_relin_host_impl(shg_context* ctx, const shg_key* key, void* out_v, const void* a_v,
                        const void* b_v, int count, shg_stream stream, bool wire) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (key->power != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "Relinearization key can only apply to a ciphertext of power 1.");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if (!out_v || !a_v || !b_v) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  const size_t ct_elems = 2 * (size_t)key->L * ctx->n;
  const size_t ct_bytes = ct_elems * sizeof(uint64_t);
  const shg::SerLayout lay = ser_layout(ctx, key->L);
  // Bytes of one ciphertext on the host side (packed when wire), rounded to
  // 16 so every staged piece stays aligned.
  const size_t host_ct = wire ? 2 * (size_t)lay.offset[key->L] : ct_bytes;
  const size_t host_ct_pad = (host_ct + 15) / 16 * 16;
  const uint8_t* a = static_cast<const uint8_t*>(a_v);
  const uint8_t* b = static_cast<const uint8_t*>(b_v);
  uint8_t* out = static_cast<uint8_t*>(out_v);
  // Pieces of host_piece ciphertexts through host_slots staging slots of
  // (a, b, out, exported degree-2 component) plus, when wire, their packed
  // forms; a and b come in on one copy stream.  The compute stream runs each
  // piece's tensor product and export; the piece's key-switch chunks go to
  // the pipeline's own lanes (chunks rotate over them across pieces), so the
  // next piece's tensor product starts while the lanes still work, and a
  // piece's copy-out waits for the lanes that ran its chunks.
  const int L = key->L, k = key->k;
  const size_t Ln = (size_t)L * ctx->n;
  const int P = std::min(count, ctx->host_piece);
  const int S = ctx->host_slots;
  const size_t packed = wire ? 3 * (size_t)P * host_ct_pad : 0;
  const size_t slot = 3 * (size_t)P * ct_bytes + (size_t)P * Ln * sizeof(uint64_t) + packed;
  const size_t d_per_ct = (size_t)k * Ln * sizeof(uint64_t);
  int C = ctx->chunk_cts > 0 ? ctx->chunk_cts
                             : (int)std::max<size_t>(1, ((size_t)256 << 20) / d_per_ct);
  C = std::max(1, std::min({C, 16, P}));
  const int lanes = std::max(1, std::min(ctx->ks_lanes, (int)shg_context::kMaxKsLanes));
  std::lock_guard<std::mutex> io_lock(ctx->io_mu);
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (ctx->io_bytes < S * slot) {
    SHG_CUDA(cudaDeviceSynchronize());
    cudaFree(ctx->io);
    ctx->io = nullptr;
    ctx->io_bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->io, S * slot);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(SHG_RESOURCE_EXHAUSTED, "cannot reserve host-pipeline staging");
    }
    ctx->io_bytes = S * slot;
  }
  if ((st = ctx->ensure_ws((size_t)lanes * C * d_per_ct))) return st;
  uint64_t* D0 = ctx->ws;
  for (cudaStream_t& s : ctx->io_streams)
    if (!s) SHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  for (int i = 0; i < lanes; ++i)
    if (!ctx->io_lanes[i]) SHG_CUDA(cudaStreamCreateWithFlags(&ctx->io_lanes[i], cudaStreamNonBlocking));
  // One copy-in stream for both operands: two concurrent host-to-device
  // streams measured 1.5 % slower end to end (18.12 against 17.86 ms per 1024
  // pairs) on the same link.
  cudaStream_t s_in = ctx->io_streams[0], s_comp = ctx->io_streams[1],
               s_out = ctx->io_streams[2];
  cudaStream_t user = (cudaStream_t)stream;
  // Piece schedule: full pieces of P in the middle; when ramping, the
  // pipeline fills and drains through pieces of P >> ramp, doubling, at both
  // ends, so the first copy-in and the last compute + copy-out are short.
  std::vector<int> sizes;
  {
    const int ramp = ctx->host_ramp;
    std::vector<int> back;
    int rem = count;
    for (int r = 0; rem > 0; ++r) {
      const int sz =
          ramp ? (int)std::min<long long>(P, (long long)std::max(1, P >> ramp) << std::min(r, 20))
               : P;
      const int f = std::min(sz, rem);
      sizes.push_back(f);
      rem -= f;
      if (rem == 0 || !ramp) continue;
      const int bk = std::min(sz, rem);
      back.push_back(bk);
      rem -= bk;
    }
    sizes.insert(sizes.end(), back.rbegin(), back.rend());
  }
  const int pieces = (int)sizes.size();
  // Every event of the call goes back on every return path (an event still
  // pending when destroyed is released once it completes).
  struct Events {
    std::vector<cudaEvent_t> v;
    ~Events() {
      for (cudaEvent_t e : v) cudaEventDestroy(e);
    }
  } evs;
  auto event = [&](cudaEvent_t* e) -> int {
    SHG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    evs.v.push_back(*e);
    return SHG_OK;
  };
  cudaEvent_t start;
  if ((st = event(&start))) return st;
  SHG_CUDA(cudaEventRecord(start, user));
  SHG_CUDA(cudaStreamWaitEvent(s_in, start, 0));
  std::vector<cudaEvent_t> loaded(pieces), tensored(pieces), stored(pieces);
  for (int i = 0; i < pieces && st == SHG_OK; ++i) {
    if ((st = event(&loaded[i])) || (st = event(&tensored[i]))) break;
    st = event(&stored[i]);
  }
  if (st) return st;
  const CtxDev dv = ctx->dev();
  int c0 = 0, chunk_no = 0;
  for (int i = 0; i < pieces; c0 += sizes[i], ++i) {
    const int cc = sizes[i];
    uint64_t* da = ctx->io + (size_t)(i % S) * (slot / sizeof(uint64_t));
    uint64_t* db = da + (size_t)P * ct_elems;
    uint64_t* dout = db + (size_t)P * ct_elems;
    uint64_t* dx = dout + (size_t)P * ct_elems;
    uint8_t* pa = reinterpret_cast<uint8_t*>(dx + (size_t)P * Ln);
    uint8_t* pb = pa + (size_t)P * host_ct_pad;
    uint8_t* pout = pb + (size_t)P * host_ct_pad;
    // Slot reuse: piece i-S must have been copied back (its tensor product
    // and key switch finished reading the slot before that).
    if (i >= S) SHG_CUDA(cudaStreamWaitEvent(s_in, stored[i - S], 0));
    if (wire) {
      // Packed ciphertexts are host_ct bytes each, back to back.
      SHG_CUDA(cudaMemcpyAsync(pa, a + (size_t)c0 * host_ct, cc * host_ct,
                               cudaMemcpyHostToDevice, s_in));
      SHG_CUDA(cudaMemcpyAsync(pb, b + (size_t)c0 * host_ct, cc * host_ct,
                               cudaMemcpyHostToDevice, s_in));
    } else {
      SHG_CUDA(cudaMemcpyAsync(da, a + (size_t)c0 * ct_bytes, cc * ct_bytes,
                               cudaMemcpyHostToDevice, s_in));
      SHG_CUDA(cudaMemcpyAsync(db, b + (size_t)c0 * ct_bytes, cc * ct_bytes,
                               cudaMemcpyHostToDevice, s_in));
    }
    SHG_CUDA(cudaEventRecord(loaded[i], s_in));
    SHG_CUDA(cudaStreamWaitEvent(s_comp, loaded[i], 0));
    if (wire) {
      shg::launch_deserialize(dv, da, pa, lay, 2 * cc, L, s_comp);
      shg::launch_deserialize(dv, db, pb, lay, 2 * cc, L, s_comp);
    }
    shg::launch_tensor_intt(dv, dout, dx, da, db, cc, L, s_comp);
    SHG_CUDA(cudaEventRecord(tensored[i], s_comp));
    bool used[shg_context::kMaxKsLanes] = {};
    for (int j = 0; j < cc; j += C, ++chunk_no) {
      const int lane = chunk_no % lanes, nc = std::min(C, cc - j);
      cudaStream_t ls = ctx->io_lanes[lane];
      if (!used[lane]) SHG_CUDA(cudaStreamWaitEvent(ls, tensored[i], 0));
      used[lane] = true;
      uint64_t* o = dout + (size_t)j * 2 * Ln;
      shg::launch_keyswitch(dv, D0 + (size_t)lane * C * k * Ln, dx + (size_t)j * Ln,
                            key->d_digits, k, key->digit_flags, key->chunk, key->chunk_lazy,
                            key->kb, key->ka, o, o, 2 * Ln, CtMap::identity(), 0, 0, nc, L, ls,
                            shg::KeyTable{});
    }
    for (int lane = 0; lane < lanes; ++lane) {
      if (!used[lane]) continue;
      cudaEvent_t done;
      if ((st = event(&done))) break;
      SHG_CUDA(cudaEventRecord(done, ctx->io_lanes[lane]));
      SHG_CUDA(cudaStreamWaitEvent(s_out, done, 0));
    }
    if (st) break;
    if (wire) {
      shg::launch_serialize(dv, pout, dout, lay, 2 * cc, L, s_out);
      SHG_CUDA(cudaMemcpyAsync(out + (size_t)c0 * host_ct, pout, cc * host_ct,
                               cudaMemcpyDeviceToHost, s_out));
    } else {
      SHG_CUDA(cudaMemcpyAsync(out + (size_t)c0 * ct_bytes, dout, cc * ct_bytes,
                               cudaMemcpyDeviceToHost, s_out));
    }
    SHG_CUDA(cudaEventRecord(stored[i], s_out));
  }
  if (st == SHG_OK) st = launch_status("bgv_mul_relin_host");
  if (st == SHG_OK) SHG_CUDA(cudaStreamWaitEvent(user, stored[pieces - 1], 0));
  return st;
}
}  // namespace

extern "C" {

int shg_bgv_mul_relin_host(shg_context* ctx, const shg_key* key, uint64_t* out,
                           const uint64_t* a, const uint64_t* b, int count,
                           shg_stream stream) {
  return mul_relin_host_impl(ctx, key, out, a, b, count, stream, false);
}

int shg_bgv_mul_relin_host_serialized(shg_context* ctx, const shg_key* key, uint8_t* out,
                                      const uint8_t* a, const uint8_t* b, int count,
                                      shg_stream stream) {
  if (ctx && ctx->n < 64)
    return fail(SHG_INVALID_ARGUMENT, "the serialized pipeline needs n >= 64");
  return mul_relin_host_impl(ctx, key, out, a, b, count, stream, true);
}

int shg_bgv_rotate(shg_context* ctx, const shg_key* key, uint64_t* out,
                   const uint64_t* ct, int count, shg_stream s) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  return keyswitch(ctx, key, out, KsArgs{ct, 2, 1, key->power, 1}, count,
                   (cudaStream_t)s);
}

int shg_key_components(const shg_key* key, uint64_t* key_b, uint64_t* key_a) {
  if (!key || !key_b || !key_a) return fail(SHG_INVALID_ARGUMENT, "null argument");
  shg_context* ctx = key->ctx;
  const size_t elems = (size_t)key->k * key->L * ctx->n;
  uint64_t* tmp = nullptr;
  cudaError_t e = cudaMalloc(&tmp, elems * sizeof(uint64_t));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SHG_RESOURCE_EXHAUSTED, "cannot reserve scratch for the key rows");
  }
  ScalarPack sc{};
  for (int l = 0; l < key->L; ++l) {
    sc.v[2 * l] = ctx->hp[l].inv_r;  // undo the 2^64 premultiplication
    sc.v[2 * l + 1] = shoup_of(ctx->hp[l].inv_r, ctx->hp[l].q);
  }
  for (int c = 0; c < 2 && e == cudaSuccess; ++c) {
    shg::launch_pointwise(ctx->dev(), shg::PW_MUL_SHOUP, tmp, c ? key->ka : key->kb, nullptr,
                          sc, key->k, key->L, 0);
    e = cudaMemcpy(c ? key_a : key_b, tmp, elems * sizeof(uint64_t), cudaMemcpyDefault);
  }
  cudaFree(tmp);
  return e == cudaSuccess ? SHG_OK : cuda_fail(e, "key_components");
}

int shg_galois_key_compose(shg_context* ctx, const shg_key* key, const shg_key* other,
                           shg_key** out) {
  if (!out) return fail(SHG_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  int st = check_key(ctx, key);
  if (st) return st;
  if ((st = check_key(ctx, other))) return st;
  if (key->L != other->L || key->k != other->k)
    return fail(SHG_INVALID_ARGUMENT, "the keys must share moduli and gadget dimension");
  const int L = key->L, k = key->k;
  const size_t Ln = (size_t)L * ctx->n, bytes = Ln * sizeof(uint64_t);
  // The other key's rows as k ciphertexts (b_i, a_i), un-premultiplied.
  uint64_t *ct = nullptr, *res = nullptr;
  cudaError_t e = cudaMalloc(&ct, 2 * k * bytes);
  if (e == cudaSuccess) e = cudaMalloc(&res, 2 * k * bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(ct);
    return fail(SHG_RESOURCE_EXHAUSTED, "cannot reserve scratch for key composition");
  }
  ScalarPack sc{};
  for (int l = 0; l < L; ++l) {
    sc.v[2 * l] = ctx->hp[l].inv_r;
    sc.v[2 * l + 1] = shoup_of(ctx->hp[l].inv_r, ctx->hp[l].q);
  }
  for (int i = 0; i < k && st == SHG_OK; ++i) {
    shg::launch_pointwise(ctx->dev(), shg::PW_MUL_SHOUP, ct + (size_t)2 * i * Ln,
                          other->kb + (size_t)i * Ln, nullptr, sc, 1, L, 0);
    shg::launch_pointwise(ctx->dev(), shg::PW_MUL_SHOUP, ct + (size_t)(2 * i + 1) * Ln,
                          other->ka + (size_t)i * Ln, nullptr, sc, 1, L, 0);
  }
  // RnsGaloisKey::Compose (rns/rns_galois_key.cc:349-406) substitutes each
  // row by this key's power and key-switches its a part with this key: the
  // rotation of that ciphertext.
  st = launch_status("galois_key_compose");
  if (st == SHG_OK)
    st = keyswitch(ctx, key, res, KsArgs{ct, 2, 1, key->power, 1}, k, (cudaStream_t)0);
  if (st == SHG_OK) {
    e = cudaMemcpy2D(ct, bytes, res, 2 * bytes, bytes, k, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy2D(ct + (size_t)k * Ln, bytes, res + Ln, 2 * bytes, bytes, k,
                       cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) st = cuda_fail(e, "galois_key_compose");
  }
  if (st == SHG_OK) {
    const int power = (int)(((int64_t)key->power * other->power) % (2 * ctx->n));
    st = shg_key_create(ctx, L, other->log_bs.data(), power, ct, ct + (size_t)k * Ln, out);
  }
  cudaFree(ct);
  cudaFree(res);
  return st;
}

int shg_galois_precompute_pad(shg_context* ctx, const shg_key* key, uint64_t* out,
                              const uint64_t* pad_digits, int count, shg_stream s) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, pad_digits}))) return st;
  shg::launch_pad_inner(ctx->dev(), out, pad_digits, key->ka, key->k, key->chunk, nullptr,
                        nullptr, 0, count, key->L, (cudaStream_t)s);
  return launch_status("galois_precompute_pad");
}

int shg_galois_apply_with_pad(shg_context* ctx, const shg_key* key, uint64_t* out,
                              const uint64_t* ct, const uint64_t* pad_digits,
                              const uint64_t* pad_new, int count, shg_stream s) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct, pad_digits, pad_new}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  shg::launch_pad_inner(ctx->dev(), out, pad_digits, key->kb, key->k, key->chunk, ct, pad_new,
                        1, count, key->L, (cudaStream_t)s);
  return launch_status("galois_apply_with_pad");
}

int shg_bgv_rotate_multikey(shg_context* ctx, const shg_key* const* keys, uint64_t* out,
                            const uint64_t* ct, int count, shg_stream s) {
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  int st = check_same_shape(ctx, keys, count, 1);
  if (st) return st;
  if ((st = check_ptrs({out, ct}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  return keyswitch(ctx, keys[0], out, KsArgs{ct, 2, 1, keys[0]->power, 1}, count,
                   (cudaStream_t)s, keys);
}

int shg_bgv_mul_relin(shg_context* ctx, const shg_key* key, uint64_t* out,
                      const uint64_t* a, const uint64_t* b, int count,
                      shg_stream stream) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (key->power != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "Relinearization key can only apply to a ciphertext of power 1.");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, a, b}))) return st;
  return mul_relin_impl(ctx, key, nullptr, out, a, b, count, (cudaStream_t)stream);
}

int shg_bgv_mul_relin_multikey(shg_context* ctx, const shg_key* const* keys,
                               uint64_t* out, const uint64_t* a, const uint64_t* b,
                               int count, shg_stream stream) {
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  int st = check_same_shape(ctx, keys, count, 1);
  if (st) return st;
  if (keys[0]->power != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "Relinearization key can only apply to a ciphertext of power 1.");
  if ((st = check_ptrs({out, a, b}))) return st;
  return mul_relin_impl(ctx, keys[0], keys, out, a, b, count, (cudaStream_t)stream);
}

}  // extern "C"

namespace {

// Argument checks shared by the expansion entry points
// (oblivious_expand.h:95-138, 237-258).
int check_expand(const shg_context* ctx, const shg_key* const* keys, int levels,
                 int count) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (levels < 0 || levels >= 32)
    return fail(SHG_INVALID_ARGUMENT,
                "The number of levels of expansion must fall within [0, 32)");
  if ((1 << std::min(levels, 30)) > ctx->n)
    return fail(SHG_INVALID_ARGUMENT, "levels of expansion exceed log n");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  for (int j = 0; j < levels; ++j) {
    if (!keys || !keys[j]) return fail(SHG_INVALID_ARGUMENT, "null Galois key");
    if (keys[j]->ctx != ctx || keys[j]->L != 1)
      return fail(SHG_INVALID_ARGUMENT, "Galois key does not match the context");
    if (keys[j]->power != (ctx->n >> j) + 1)
      return fail(SHG_INVALID_ARGUMENT,
                  "Substitution power of the i'th GaloisKey must be (N / (2 ^ "
                  "i)) + 1");
  }
  return SHG_OK;
}

// Scratch of one expansion pass: the level monomials, then X, D and KS for
// C members at a time.  A chunk holds whole queries, so it must fit the
// 2^(levels-1) members one query contributes at the last level.
struct ExpandPlan {
  int C = 1;
  size_t mono_bytes = 0, per_member = 0;
  size_t bytes() const { return mono_bytes + per_member * C; }
};

ExpandPlan plan_expand(const shg_context* ctx, const shg_key* const* keys, int levels,
                       int count) {
  ExpandPlan p;
  const int n = ctx->n;
  const int kmax = levels ? keys[0]->k : 0;
  p.per_member = ((size_t)n + (size_t)kmax * n + 2 * (size_t)n) * sizeof(uint64_t);
  p.mono_bytes = (size_t)levels * n * sizeof(uint64_t);
  const int members_max = std::max(1, count << std::max(levels - 1, 0));
  p.C = std::max(1 << std::max(levels - 1, 0),
                 (int)std::min<size_t>((size_t)members_max, ((size_t)256 << 20) / p.per_member));
  return p;
}

// ExpandCiphertext over `count` queries already placed at slot 0 of their
// [2^levels][2][n] blocks in `out` (oblivious_expand.h:173-227): level j
// substitutes every member by n/2^j + 1, key-switches it and combines
// (c + ks, (c - ks) * -x^{n - 2^j}) into slots p and p + 2^j.  `ws` is the
// plan's scratch, the monomials first.
// `tables` (optional): per level j, device tables of the count queries' key
// pointers (query q uses entry q): every query brings its own keys.
int run_expand(shg_context* ctx, const shg_key* const* keys, int levels, uint64_t* out,
               int count, const ExpandPlan& plan, uint64_t* ws, cudaStream_t s,
               const shg::KeyTable* tables = nullptr) {
  if (levels == 0 || count == 0) return SHG_OK;
  const int n = ctx->n;
  const int C = plan.C;
  const int kmax = keys[0]->k;
  const size_t per_query = ((size_t)2 * n) << levels;
  uint64_t* mono = ws;
  uint64_t* X = mono + (size_t)levels * n;
  uint64_t* D = X + (size_t)C * n;
  uint64_t* KS = D + (size_t)C * kmax * n;
  // Monomials -x^{n - 2^j} in NTT form (oblivious_expand.h:197-200), built
  // on the stream so the whole expansion can be captured in a graph.
  shg::launch_monomials(ctx->dev(), mono, levels, ctx->hp[0].q - ctx->hp[0].r_mod_q, s);
  shg::launch_ntt_fwd(ctx->dev(), mono, mono, levels, 1, s);
  const CtxDev dv = ctx->dev();
  for (int j = 0; j < levels; ++j) {
    const shg_key* key = keys[j];
    const int power = (n >> j) + 1;
    const CtMap map{j, levels};
    // Members of a level are processed in chunks of whole queries.
    const int q_per_chunk = std::max(1, C >> j);
    for (int q0 = 0; q0 < count; q0 += q_per_chunk) {
      const int qc = std::min(q_per_chunk, count - q0);
      const int mc = qc << j;
      uint64_t* blk = out + (size_t)q0 * per_query;
      shg::launch_intt_export(dv, X, blk, 2, 1, power, map, mc, 1, s);
      shg::KeyTable kt;
      if (tables)
        kt = shg::KeyTable{tables[j].kb + q0, tables[j].ka + q0, j,
                           tables[j].entries ? tables[j].entries - q0 : 0};
      shg::launch_keyswitch(dv, D, X, key->d_digits, key->k, key->digit_flags,
                            key->chunk, key->chunk_lazy, key->kb, key->ka, KS, blk, 2 * (size_t)n,
                            map, 1, power, mc, 1, s, kt);
      shg::launch_expand_combine(dv, blk, KS, mono + (size_t)j * n, map, 1 << j,
                                 mc, s);
    }
  }
  return SHG_OK;
}

int absorb_chunk(const shg_context* ctx) {
  const uint64_t q = ctx->hp[0].q;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(1u << 20, (~(uint64_t)0) / q));
}

// PIR server step over `count` queries; per_query_keys: keys is
// [count][levels] (query q's level-j key at keys[q * levels + j]), else one
// key list [levels] for every query.
int pir_impl(shg_context* ctx, const shg_key* const* keys, bool per_query_keys, int levels,
             const uint64_t* db, int num_items, uint64_t* out, const uint64_t* ct, int count,
             cudaStream_t s) {
  int st = check_expand(ctx, keys, levels, count);
  if (st) return st;
  if (num_items < 1 || num_items > (1 << levels))
    return fail(SHG_INVALID_ARGUMENT,
                "Output length must be at most " + std::to_string(1 << levels));
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct, db}))) return st;
  if (per_query_keys)
    for (int j = 0; j < levels; ++j)
      if ((st = check_same_shape(ctx, keys + j, count, levels))) return st;
  const int n = ctx->n;
  const size_t per_query_elems = ((size_t)2 * n) << levels;
  // Queries per group: their expanded blocks (2^levels ciphertexts each) share
  // a 1 GiB scratch region and are absorbed before the next group starts.
  const int group = (int)std::max<size_t>(
      1, std::min<size_t>((size_t)count, ((size_t)1 << 30) / (per_query_elems * 8)));
  const ExpandPlan plan = plan_expand(ctx, keys, levels, group);
  const size_t blocks_bytes = (size_t)group * per_query_elems * sizeof(uint64_t);
  const size_t tab_bytes = per_query_keys ? 2 * (size_t)levels * count * sizeof(void*) : 0;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(plan.bytes() + blocks_bytes + tab_bytes))) return st;
  uint64_t* blocks = ctx->ws + plan.bytes() / sizeof(uint64_t);
  std::vector<shg::KeyTable> tables(per_query_keys ? levels : 0);
  if (per_query_keys) {
    const uint64_t** tab = reinterpret_cast<const uint64_t**>(
        blocks + (size_t)group * per_query_elems);
    for (int j = 0; j < levels; ++j)
      if ((st = upload_key_table(keys, count, levels, j, tab + 2 * (size_t)j * count,
                                 &tables[j], s)))
        return st;
  }
  const shg_key* const* level_keys = keys;  // per-level shape (first query's keys)
  for (int g0 = 0; g0 < count; g0 += group) {
    const int gc = std::min(group, count - g0);
    // Slot 0 of every block <- its query; the strided copy is one call.
    SHG_CUDA(cudaMemcpy2DAsync(blocks, per_query_elems * sizeof(uint64_t),
                               ct + (size_t)g0 * 2 * n, 2 * n * sizeof(uint64_t),
                               2 * n * sizeof(uint64_t), gc, cudaMemcpyDeviceToDevice, s));
    std::vector<shg::KeyTable> gt(tables.size());
    for (size_t j = 0; j < tables.size(); ++j)
      gt[j] = shg::KeyTable{tables[j].kb + g0, tables[j].ka + g0, 0,
                            tables[j].entries ? tables[j].entries - g0 : 0};
    if ((st = run_expand(ctx, level_keys, levels, blocks, gc, plan, ctx->ws, s,
                         per_query_keys ? gt.data() : nullptr)))
      return st;
    shg::launch_absorb_sum(ctx->dev(), out + (size_t)g0 * 2 * n, blocks, db, num_items,
                           (size_t)1 << levels, absorb_chunk(ctx), gc, s);
  }
  return launch_status("pir_expand_absorb");
}

}  // namespace

extern "C" {

int shg_oblivious_expand(shg_context* ctx, const shg_key* const* keys,
                         int levels, uint64_t* out, const uint64_t* ct,
                         int count, shg_stream stream) {
  int st = check_expand(ctx, keys, levels, count);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = ctx->n;
  const size_t per_query = ((size_t)2 * n) << levels;
  // Place each query at slot 0 of its output block.
  for (int qi = 0; qi < count; ++qi) {
    SHG_CUDA(cudaMemcpyAsync(out + (size_t)qi * per_query, ct + (size_t)qi * 2 * n,
                             2 * n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  }
  if (levels == 0) return SHG_OK;
  const ExpandPlan plan = plan_expand(ctx, keys, levels, count);
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(plan.bytes()))) return st;
  if ((st = run_expand(ctx, keys, levels, out, count, plan, ctx->ws, s))) return st;
  return launch_status("oblivious_expand");
}

int shg_pir_expand_absorb(shg_context* ctx, const shg_key* const* keys, int levels,
                          const uint64_t* db, int num_items, uint64_t* out,
                          const uint64_t* ct, int count, shg_stream stream) {
  return pir_impl(ctx, keys, false, levels, db, num_items, out, ct, count,
                  (cudaStream_t)stream);
}

int shg_pir_expand_absorb_multikey(shg_context* ctx, const shg_key* const* keys, int levels,
                                   const uint64_t* db, int num_items, uint64_t* out,
                                   const uint64_t* ct, int count, shg_stream stream) {
  return pir_impl(ctx, keys, true, levels, db, num_items, out, ct, count,
                  (cudaStream_t)stream);
}

size_t shg_poly_serialized_bytes(const shg_context* ctx, int num_limbs) {
  if (!ctx || num_limbs <= 0 || num_limbs > ctx->L) return 0;
  return (size_t)ser_layout(ctx, num_limbs).offset[num_limbs];
}

int shg_poly_serialize(shg_context* ctx, uint8_t* out, const uint64_t* polys, int count,
                       int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if (!out) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  if ((st = check_ptrs({polys}))) return st;
  if (ctx->n >= 64 && ((uintptr_t)out & 7))
    return fail(SHG_INVALID_ARGUMENT, "serialized buffers must be 8-byte aligned");
  shg::launch_serialize(ctx->dev(), out, polys, ser_layout(ctx, num_limbs), count, num_limbs,
                        (cudaStream_t)s);
  return launch_status("serialize");
}

int shg_poly_deserialize(shg_context* ctx, uint64_t* polys, const uint8_t* in, int count,
                         int num_limbs, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if (!in) return fail(SHG_INVALID_ARGUMENT, "null buffer pointer");
  if ((st = check_ptrs({polys}))) return st;
  if (ctx->n >= 64 && ((uintptr_t)in & 7))
    return fail(SHG_INVALID_ARGUMENT, "serialized buffers must be 8-byte aligned");
  shg::launch_deserialize(ctx->dev(), polys, in, ser_layout(ctx, num_limbs), count, num_limbs,
                          (cudaStream_t)s);
  return launch_status("deserialize");
}

int shg_symmetric_encrypt(shg_context* ctx, uint64_t* out, const uint64_t* s_ntt,
                          const uint64_t* a, const uint64_t* e, const uint64_t* m, int count,
                          shg_stream stream) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (ctx->L != 1)
    return fail(SHG_INVALID_ARGUMENT, "symmetric encryption needs a one-prime context");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  int st = check_ptrs({out, s_ntt, a, e, m});
  if (st) return st;
  const HostPrime& h = ctx->hp[0];
  if (ctx->t == 0 || ctx->t >= h.q)
    return fail(SHG_INVALID_ARGUMENT, "the plaintext modulus must lie in [1, q)");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t elems = (size_t)count * ctx->n;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(elems * sizeof(uint64_t)))) return st;
  // c0 = e, in NTT form (Polynomial::ConvertToNtt of the error samples).
  SHG_CUDA(cudaMemcpyAsync(ctx->ws, e, elems * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  shg::launch_ntt_fwd(ctx->dev(), ctx->ws, ctx->ws, count, 1, s);
  shg::launch_sym_encrypt(ctx->dev(), out, ctx->ws, a, m, s_ntt, to_mont(ctx->t, h.q), count,
                          s);
  return launch_status("symmetric_encrypt");
}

int shg_symmetric_decrypt(shg_context* ctx, uint64_t* out, const uint64_t* s_ntt,
                          const uint64_t* ct, int len, int count, shg_stream stream) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (ctx->L != 1)
    return fail(SHG_INVALID_ARGUMENT, "symmetric encryption needs a one-prime context");
  if (ctx->t == 0) return fail(SHG_INVALID_ARGUMENT, "t is zero");
  if (count < 0 || len < 1)
    return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative and `len` positive.");
  if (count == 0) return SHG_OK;
  int st = check_ptrs({out, s_ntt, ct});
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t elems = (size_t)count * ctx->n;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(elems * sizeof(uint64_t)))) return st;
  shg::launch_sym_dot(ctx->dev(), ctx->ws, ct, s_ntt, len, count, s);
  // InverseNtt + ExportInt in one scaled inverse transform, then RemoveError.
  shg::launch_ntt_inv(ctx->dev(), ctx->ws, ctx->ws, count, 1, 1, s);
  shg::launch_remove_error(ctx->dev(), out, ctx->ws, ctx->hp[0].q, ctx->t, count, s);
  return launch_status("symmetric_decrypt");
}

int shg_absorb_sum(shg_context* ctx, uint64_t* out, const uint64_t* cts,
                   const uint64_t* db, int num_items, int count,
                   shg_stream stream) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  if (count < 0 || num_items < 0)
    return fail(SHG_INVALID_ARGUMENT, "sizes must be non-negative");
  if (count == 0) return SHG_OK;
  int st = check_ptrs({out, cts, db});
  if (st) return st;
  shg::launch_absorb_sum(ctx->dev(), out, cts, db, num_items, (size_t)num_items,
                         absorb_chunk(ctx), count, (cudaStream_t)stream);
  return launch_status("absorb_sum");
}

// ---------------------------------------------------------------------------
// Runtime plumbing
// ---------------------------------------------------------------------------

int shg_device_count(int* count) {
  SHG_CUDA(cudaGetDeviceCount(count));
  return SHG_OK;
}
int shg_set_device(int device) {
  SHG_CUDA(cudaSetDevice(device));
  return SHG_OK;
}
int shg_device_alloc(size_t bytes, void** out) {
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SHG_RESOURCE_EXHAUSTED, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return SHG_OK;
}
int shg_device_free(void* ptr) {
  SHG_CUDA(cudaFree(ptr));
  return SHG_OK;
}
int shg_host_alloc(size_t bytes, void** out) {
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SHG_RESOURCE_EXHAUSTED, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
  }
  return SHG_OK;
}
int shg_host_free(void* ptr) {
  SHG_CUDA(cudaFreeHost(ptr));
  return SHG_OK;
}
int shg_memcpy_h2d(void* dst, const void* src, size_t bytes, shg_stream s) {
  SHG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)s));
  return SHG_OK;
}
int shg_memcpy_d2h(void* dst, const void* src, size_t bytes, shg_stream s) {
  SHG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)s));
  return SHG_OK;
}
int shg_memcpy_d2d(void* dst, const void* src, size_t bytes, shg_stream s) {
  SHG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)s));
  return SHG_OK;
}
int shg_memset_device(void* dst, int value, size_t bytes, shg_stream s) {
  SHG_CUDA(cudaMemsetAsync(dst, value, bytes, (cudaStream_t)s));
  return SHG_OK;
}
int shg_stream_create(shg_stream* out) {
  cudaStream_t s;
  SHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *out = (shg_stream)s;
  return SHG_OK;
}
int shg_stream_destroy(shg_stream s) {
  SHG_CUDA(cudaStreamDestroy((cudaStream_t)s));
  return SHG_OK;
}
int shg_stream_synchronize(shg_stream s) {
  SHG_CUDA(cudaStreamSynchronize((cudaStream_t)s));
  return SHG_OK;
}
int shg_device_synchronize(void) {
  SHG_CUDA(cudaDeviceSynchronize());
  return SHG_OK;
}
int shg_event_create(void** out) {
  cudaEvent_t e;
  SHG_CUDA(cudaEventCreate(&e));
  *out = (void*)e;
  return SHG_OK;
}
int shg_event_destroy(void* ev) {
  SHG_CUDA(cudaEventDestroy((cudaEvent_t)ev));
  return SHG_OK;
}
int shg_event_record(void* ev, shg_stream s) {
  SHG_CUDA(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)s));
  return SHG_OK;
}
int shg_event_elapsed_ms(void* a, void* b, float* ms) {
  SHG_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b));
  return SHG_OK;
}
int shg_graph_capture_begin(shg_stream s) {
  SHG_CUDA(cudaStreamBeginCapture((cudaStream_t)s, cudaStreamCaptureModeThreadLocal));
  return SHG_OK;
}
int shg_graph_capture_end(shg_stream s, void** exec) {
  cudaGraph_t g;
  SHG_CUDA(cudaStreamEndCapture((cudaStream_t)s, &g));
  cudaGraphExec_t ge;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  *exec = (void*)ge;
  return SHG_OK;
}
int shg_graph_launch(void* exec, shg_stream s) {
  SHG_CUDA(cudaGraphLaunch((cudaGraphExec_t)exec, (cudaStream_t)s));
  return SHG_OK;
}
int shg_graph_destroy(void* exec) {
  SHG_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)exec));
  return SHG_OK;
}
uint64_t shg_launch_count(void) { return shg::g_launch_count.load(); }

int shg_measure_butterfly_rate(double* per_second) {
  if (!per_second) return fail(SHG_INVALID_ARGUMENT, "null argument");
  if (shg::measure_butterfly_rate(per_second) != 0)
    return fail(SHG_INTERNAL, std::string("butterfly probe failed: ") +
                                  cudaGetErrorString(cudaGetLastError()));
  return SHG_OK;
}

namespace {
struct ProfTotal {
  std::string name;
  double ms = 0;
  uint64_t launches = 0;
};
std::vector<ProfTotal> g_prof_totals;
}  // namespace

int shg_profile_start(void) {
  std::lock_guard<std::mutex> lock(shg::g_prof_mu);
  for (auto& e : shg::g_prof_pending) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  shg::g_prof_pending.clear();
  g_prof_totals.clear();
  shg::g_prof_on = true;
  return SHG_OK;
}

int shg_profile_stop(void) {
  shg::g_prof_on = false;
  SHG_CUDA(cudaDeviceSynchronize());
  std::lock_guard<std::mutex> lock(shg::g_prof_mu);
  for (auto& e : shg::g_prof_pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, e.a, e.b);
    auto it = std::find_if(g_prof_totals.begin(), g_prof_totals.end(),
                           [&](const ProfTotal& t) { return t.name == e.name; });
    if (it == g_prof_totals.end()) {
      g_prof_totals.push_back(ProfTotal{e.name, 0, 0});
      it = g_prof_totals.end() - 1;
    }
    it->ms += ms;
    it->launches += 1;
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  shg::g_prof_pending.clear();
  return SHG_OK;
}

int shg_profile_query(const char* kernel, double* total_ms, uint64_t* launches) {
  if (!kernel || !total_ms || !launches)
    return fail(SHG_INVALID_ARGUMENT, "null argument");
  *total_ms = 0;
  *launches = 0;
  for (const auto& t : g_prof_totals) {
    if (t.name == kernel) {
      *total_ms = t.ms;
      *launches = t.launches;
    }
  }
  return SHG_OK;
}
int shg_context_reserve(shg_context* ctx, size_t bytes) {
  if (!ctx) return fail(SHG_INVALID_ARGUMENT, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  return ctx->ensure_ws(bytes);
}
int shg_context_set_chunk(shg_context* ctx, int cts) {
  if (!ctx || cts < 0) return fail(SHG_INVALID_ARGUMENT, "bad chunk size");
  ctx->chunk_cts = cts;
  return SHG_OK;
}
int shg_context_set_four_step_min(shg_context* ctx, int log_n) {
  if (!ctx || log_n < 12 || log_n > 16)
    return fail(SHG_INVALID_ARGUMENT, "four-step threshold must lie in [12, 16]");
  ctx->ntt4_min = log_n;
  ctx->ntt4_plain_min = log_n <= 13 ? 12 : log_n;
  return SHG_OK;
}
int shg_debug_status(unsigned* first_failure) {
  if (!first_failure) return fail(SHG_INVALID_ARGUMENT, "null argument");
  const unsigned a = shg::take_debug_word_kernels();
  const unsigned b = shg::take_debug_word_ntt4();
  *first_failure = a ? a : b;
  return SHG_OK;
}

int shg_context_set_ks_lanes(shg_context* ctx, int lanes) {
  if (!ctx || lanes < 1 || lanes > shg_context::kMaxKsLanes)
    return fail(SHG_INVALID_ARGUMENT, "key-switch lanes must be 1 to 4");
  ctx->ks_lanes = lanes;
  return SHG_OK;
}
int shg_context_set_host_pipeline(shg_context* ctx, int piece_cts, int slots) {
  if (!ctx || piece_cts < 1 || slots < 2 || slots > 8)
    return fail(SHG_INVALID_ARGUMENT, "piece must be positive and slots in [2, 8]");
  ctx->host_piece = piece_cts;
  ctx->host_slots = slots;
  return SHG_OK;
}

int shg_context_set_host_ramp(shg_context* ctx, int ramp) {
  if (!ctx || ramp < 0 || ramp > 16)
    return fail(SHG_INVALID_ARGUMENT, "ramp must be in [0, 16]");
  ctx->host_ramp = ramp;
  return SHG_OK;
}
int shg_context_get_tuning(const shg_context* ctx, int* chunk, int* four_step_min,
                           int* ks_fused) {
  if (!ctx || !chunk || !four_step_min || !ks_fused)
    return fail(SHG_INVALID_ARGUMENT, "null argument");
  *chunk = ctx->chunk_cts;
  *four_step_min = ctx->ntt4_min;
  *ks_fused = ctx->ks_fused;
  return SHG_OK;
}
int shg_poly_fill_uniform(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                          uint64_t seed, shg_stream s) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({polys}))) return st;
  shg::launch_fill_uniform(ctx->dev(), polys, seed, count, num_limbs, (cudaStream_t)s);
  return launch_status("fill_uniform");
}
// SampleError's variance bounds (rns/error_distribution.h:44-49,
// sample_error.h:47-50, kMaxVariance = 256 in constants.h).
static int check_variance(int variance) {
  if (variance <= 0) return fail(SHG_INVALID_ARGUMENT, "`variance` must be positive.");
  if (variance > 256)
    return fail(SHG_INVALID_ARGUMENT, "The variance, " + std::to_string(variance) +
                                          ", must be at most 256.");
  return SHG_OK;
}

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

int shg_sample_uniform_error(shg_context* ctx, uint64_t* a, uint64_t* e,
                             const uint8_t* seeds, int num_limbs, int count, int variance,
                             shg_stream stream) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if ((st = check_variance(variance))) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({a, e, seeds}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = num_limbs;
  const size_t Ln = (size_t)L * ctx->n;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(round256((size_t)count * ctx->n * sizeof(int32_t))))) return st;
  int32_t* err = reinterpret_cast<int32_t*>(ctx->ws);
  const shg::CtxDev dev = ctx->dev();
  shg::launch_sample_uniform_error(dev, a, Ln, 0, err, seeds, L, variance, count, s);
  shg::launch_error_lift(dev, e, err, count, L, s);
  shg::launch_ntt_fwd(dev, e, e, count * L, L, s);
  return launch_status("sample_uniform_error");
}

int shg_bgv_encrypt(shg_context* ctx, uint64_t* out, const uint64_t* key,
                    const uint64_t* plaintexts, const uint8_t* seeds, int num_limbs,
                    int count, int variance, shg_stream stream) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if ((st = check_variance(variance))) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, key, plaintexts, seeds}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = num_limbs;
  const size_t n = ctx->n, Ln = (size_t)L * n;
  shg::ScalarPack tm{};
  for (int l = 0; l < L; ++l) tm.v[l] = to_mont(ctx->t % ctx->hp[l].q, ctx->hp[l].q);
  const bool four = ctx->log_n >= 12 && (ctx->log_n >= ctx->ntt4_min || ctx->log_n > 14);
  // Transform chunks as large as 1 GiB of scratch allows (or the context's
  // chunk setting): whole-batch launches measured faster (n = 2^14, six
  // limbs, 1024 ciphertexts: 1.50 ms) than L2-sized 42-ciphertext chunks
  // (2.03 ms), whose launches leave the GPU part idle.
  const size_t per_ct = Ln * sizeof(uint64_t);
  const size_t want = ctx->chunk_cts > 0 ? (size_t)ctx->chunk_cts
                                         : std::max<size_t>(1, ((size_t)1 << 30) / per_ct);
  const int C = (int)std::max<size_t>(1, std::min<size_t>((size_t)count, want));
  const size_t err_bytes = round256((size_t)count * n * sizeof(int32_t));
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(err_bytes + (size_t)C * per_ct))) return st;
  int32_t* err = reinterpret_cast<int32_t*>(ctx->ws);
  uint64_t* buf = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(ctx->ws) + err_bytes);
  const shg::CtxDev dev = ctx->dev();
  // c1 = -a straight from the sampler; the error waits in err.
  shg::launch_sample_uniform_error(dev, out + Ln, 2 * Ln, 1, err, seeds, L, variance, count,
                                   s);
  for (int c0 = 0; c0 < count; c0 += C) {
    const int cc = std::min(C, count - c0);
    uint64_t* o = out + (size_t)c0 * 2 * Ln;
    const uint64_t* m = plaintexts + (size_t)c0 * Ln;
    const int32_t* e = err + (size_t)c0 * n;
    if (four) {
      shg::launch4_bgv_encrypt(dev, o, e, m, key, tm, buf, cc, L, s);
    } else {
      shg::launch_error_lift(dev, buf, e, cc, L, s);
      shg::launch_ntt_fwd(dev, buf, buf, cc * L, L, s);
      shg::launch_bgv_enc_combine(dev, o, buf, m, key, tm, cc, L, s);
    }
  }
  return launch_status("bgv_encrypt");
}

// ---------------------------------------------------------------------------
// RNS basis conversion and BFV (auxiliary primes)
// ---------------------------------------------------------------------------

int shg_context_num_aux_moduli(const shg_context* ctx) { return ctx ? ctx->K : 0; }

static int check_aux(shg_context* ctx, int count, int num_limbs) {
  int st = check_limbs(ctx, count, num_limbs);
  if (st) return st;
  if (ctx->K == 0)
    return fail(SHG_INVALID_ARGUMENT, "the context has no auxiliary prime moduli");
  return SHG_OK;
}

static shg::ConvRef conv(const shg_context* ctx, int kind, int level, int balanced = 0) {
  const int slot = conv_slot(ctx, kind, level, balanced);
  return shg::ConvRef{ctx->d_conv + slot, ctx->conv_fast[slot]};
}

int shg_poly_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                              int direction, int num_limbs, int count, shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (direction != 0 && direction != 1)
    return fail(SHG_INVALID_ARGUMENT, "`direction` must be 0 (main to aux) or 1 (aux to main)");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  const size_t n = ctx->n, m = (size_t)num_limbs * n, a = (size_t)ctx->K * n;
  const int l = num_limbs - 1;
  if (direction == 0)
    shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SWITCH_UP, l), num_limbs, ctx->K, in,
                             m, out, a, count, ctx->log_n, (cudaStream_t)stream);
  else
    shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SWITCH_DOWN, l), ctx->K, num_limbs,
                             in, a, out, m, count, ctx->log_n, (cudaStream_t)stream);
  return launch_status("switch_rns_basis");
}

int shg_poly_scale_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                                    int num_limbs, int count, shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  const size_t n = ctx->n;
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SCALE_UP, num_limbs - 1), num_limbs,
                           ctx->K, in, (size_t)num_limbs * n, out, (size_t)ctx->K * n, count,
                           ctx->log_n, (cudaStream_t)stream);
  return launch_status("scale_switch_rns_basis");
}

int shg_poly_approx_switch_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* in,
                                     int direction, int num_limbs, int is_ntt, int balanced,
                                     int count, shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (direction != 0 && direction != 1)
    return fail(SHG_INVALID_ARGUMENT, "`direction` must be 0 (main to aux) or 1 (aux to main)");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, in}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n = ctx->n, m = (size_t)num_limbs * n, a = (size_t)ctx->K * n;
  const int l = num_limbs - 1, ns = direction == 0 ? num_limbs : ctx->K;
  const size_t in_elems = direction == 0 ? m : a;
  std::lock_guard<std::mutex> lock(ctx->mu);
  const uint64_t* src = in;
  if (is_ntt) {
    // ApproxSwitchRnsBasis's inverse NTT after the (Q/q_i)^-1 factor; the
    // two commute, so the inputs are transformed first.
    if ((st = ctx->ensure_ws((size_t)count * in_elems * sizeof(uint64_t)))) return st;
    const shg::CtxDev view = direction == 0 ? ctx->dev() : ctx->aux_dev();
    shg::launch_ntt_inv(view, in, ctx->ws, count * ns, ns, 0, s);
    src = ctx->ws;
  }
  if (direction == 0)
    shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_APPROX_UP, l, balanced != 0),
                             num_limbs, ctx->K, src, m, out, a, count, ctx->log_n, s);
  else
    shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_APPROX_DOWN, l, balanced != 0),
                             ctx->K, num_limbs, src, a, out, m, count, ctx->log_n, s);
  return launch_status("approx_switch_rns_basis");
}

// P^-1 mod q_i (plain), P = the product of the auxiliary primes.
static uint64_t p_inv_mod(const shg_context* ctx, int i) {
  const uint64_t q = ctx->hp[i].q;
  return invmod(prod_mod(ctx, ctx->L, ctx->L + ctx->K, -1, q), q);
}

// out_i = main_i * c_i - delta_i * d_i (sign 1) or + (sign 0), c, d plain.
static void combine(shg_context* ctx, uint64_t* out, const uint64_t* main_ntt,
                    const uint64_t* delta, const uint64_t* c, const uint64_t* d, int sign,
                    int count, int Lm, cudaStream_t s) {
  shg::ScalarPack cd{};
  for (int i = 0; i < Lm; ++i) {
    const uint64_t q = ctx->hp[i].q;
    cd.v[2 * i] = to_mont(c[i], q);
    cd.v[2 * i + 1] = to_mont(d[i], q);
  }
  shg::launch_lin2(ctx->dev(), out, main_ntt, delta, cd, sign, count, Lm, s);
}

// aux [count][K][n] times a plain factor per aux prime into dst.
static void scale_aux(shg_context* ctx, uint64_t* dst, const uint64_t* aux,
                      const std::vector<uint64_t>& f, int count, cudaStream_t s) {
  shg::ScalarPack sc{};
  for (int j = 0; j < ctx->K; ++j) {
    const uint64_t p = ctx->hp[ctx->L + j].q;
    sc.v[2 * j] = f[j] % p;
    sc.v[2 * j + 1] = shoup_of(sc.v[2 * j], p);
  }
  shg::launch_pointwise(ctx->aux_dev(), shg::PW_MUL_SHOUP, dst, aux, nullptr, sc, count,
                        ctx->K, s);
}

int shg_poly_scale_reduce_rns_basis(shg_context* ctx, uint64_t* out, const uint64_t* main,
                                    const uint64_t* aux, uint64_t t, int is_ntt_main,
                                    int is_ntt_aux, int num_limbs, int count,
                                    shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (t == 0) return fail(SHG_INVALID_ARGUMENT, "`t` must be positive.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, main, aux}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int Lm = num_limbs, K = ctx->K, l = Lm - 1;
  const size_t n = ctx->n, a_elems = (size_t)count * K * n, m_elems = (size_t)count * Lm * n;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws((a_elems + m_elems) * sizeof(uint64_t)))) return st;
  uint64_t* aux_c = ctx->ws;
  uint64_t* delta = ctx->ws + a_elems;
  const shg::CtxDev aux_view = ctx->aux_dev();
  shg::ConvRef bc;
  if (t == ctx->t) {  // t folded into the conversion's source factor
    if (is_ntt_aux) shg::launch_ntt_inv(aux_view, aux, aux_c, count * K, K, 0, s);
    bc = conv(ctx, CONV_SWITCH_DOWN_T, l);
  } else {
    scale_aux(ctx, aux_c, aux, std::vector<uint64_t>(K, t), count, s);
    if (is_ntt_aux) shg::launch_ntt_inv(aux_view, aux_c, aux_c, count * K, K, 0, s);
    bc = conv(ctx, CONV_SWITCH_DOWN, l);
  }
  shg::launch_switch_basis(ctx->d_primes, bc, K, Lm,
                           (is_ntt_aux || t != ctx->t) ? aux_c : aux, (size_t)K * n, delta,
                           (size_t)Lm * n, count, ctx->log_n, s);
  if (is_ntt_main) shg::launch_ntt_fwd(ctx->dev(), delta, delta, count * Lm, Lm, s);
  std::vector<uint64_t> c(Lm), d(Lm);
  for (int i = 0; i < Lm; ++i) {
    d[i] = p_inv_mod(ctx, i);
    c[i] = mulmod(t % ctx->hp[i].q, d[i], ctx->hp[i].q);
  }
  combine(ctx, out, main, delta, c.data(), d.data(), 1, count, Lm, s);
  return launch_status("scale_reduce_rns_basis");
}

int shg_poly_approx_modreduce(shg_context* ctx, uint64_t* out, const uint64_t* main,
                              const uint64_t* aux, int lsb, uint64_t t, int is_ntt_main,
                              int is_ntt_aux, int num_limbs, int count, shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (lsb && t == 0) return fail(SHG_INVALID_ARGUMENT, "`t` must be positive.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, main, aux}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int Lm = num_limbs, K = ctx->K, l = Lm - 1;
  const size_t n = ctx->n, a_elems = (size_t)count * K * n, m_elems = (size_t)count * Lm * n;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws((a_elems + 2 * m_elems) * sizeof(uint64_t)))) return st;
  uint64_t* aux_c = ctx->ws;
  uint64_t* delta = ctx->ws + a_elems;
  uint64_t* main_c = delta + m_elems;
  const shg::CtxDev aux_view = ctx->aux_dev();
  uint64_t p_mod_t = 0;
  const uint64_t* src = aux;
  if (lsb) {
    // P mod t over the integers; aux times p_mod_t * (-t^-1) mod p_j
    // (ApproxModReduceLsb, rns/rns_polynomial.cc:769-779)
    u128 pm = 1 % t;
    for (int j = 0; j < K; ++j) pm = pm * (ctx->hp[ctx->L + j].q % t) % t;
    p_mod_t = (uint64_t)pm;
    std::vector<uint64_t> f(K);
    for (int j = 0; j < K; ++j) {
      const uint64_t p = ctx->hp[ctx->L + j].q;
      f[j] = mulmod(p_mod_t % p, (p - invmod(t % p, p)) % p, p);
    }
    scale_aux(ctx, aux_c, aux, f, count, s);
    src = aux_c;
  }
  if (is_ntt_aux) {
    shg::launch_ntt_inv(aux_view, src, aux_c, count * K, K, 0, s);
    src = aux_c;
  }
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_APPROX_DOWN, l, lsb ? 1 : 0), K, Lm,
                           src, (size_t)K * n, delta, (size_t)Lm * n, count, ctx->log_n, s);
  shg::launch_ntt_fwd(ctx->dev(), delta, delta, count * Lm, Lm, s);
  const uint64_t* m = main;
  if (!is_ntt_main) {
    shg::launch_ntt_fwd(ctx->dev(), main, main_c, count * Lm, Lm, s);
    m = main_c;
  }
  std::vector<uint64_t> c(Lm), d(Lm);
  for (int i = 0; i < Lm; ++i) {
    const uint64_t q = ctx->hp[i].q, pinv = p_inv_mod(ctx, i);
    c[i] = lsb ? mulmod(p_mod_t % q, pinv, q) : pinv;
    d[i] = lsb ? mulmod(t % q, pinv, q) : pinv;
  }
  combine(ctx, out, m, delta, c.data(), d.data(), lsb ? 0 : 1, count, Lm, s);
  return launch_status("approx_modreduce");
}

// Ciphertext components x [count][Lm][n] (NTT form) -> the ScaleAndSwitch /
// Switch round trip of RnsBfvCiphertext::Mul (rns/rns_bfv_ciphertext.cc:161-179):
// x_aux = ScaleAndSwitchRnsBasis(x) = round(P/Q x) mod P and x_main =
// SwitchRnsBasis(x_aux) = the same integer mod Q, both returned in NTT form.
// X: [count][Lm][n] scratch.
static void bfv_scale_up(shg_context* ctx, const uint64_t* x, uint64_t* X, uint64_t* x_aux,
                         uint64_t* x_main, int count, int Lm, cudaStream_t s) {
  const size_t n = ctx->n;
  const int K = ctx->K, l = Lm - 1;
  shg::launch_ntt_inv(ctx->dev(), x, X, count * Lm, Lm, 0, s);
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SCALE_UP, l), Lm, K, X,
                           (size_t)Lm * n, x_aux, (size_t)K * n, count, ctx->log_n, s);
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SWITCH_DOWN, l), K, Lm, x_aux,
                           (size_t)K * n, x_main, (size_t)Lm * n, count, ctx->log_n, s);
  shg::launch_ntt_fwd(ctx->dev(), x_main, x_main, count * Lm, Lm, s);
  shg::launch_ntt_fwd(ctx->aux_dev(), x_aux, x_aux, count * K, K, s);
}

// NTT-form x [count][Lm][n] -> its SwitchRnsBasis to the auxiliary primes in
// NTT form [count][K][n]; X: [count][Lm][n] scratch.
static void bfv_switch_up(shg_context* ctx, const uint64_t* x, uint64_t* X, uint64_t* x_aux,
                          int count, int Lm, cudaStream_t s) {
  const size_t n = ctx->n;
  const int K = ctx->K;
  shg::launch_ntt_inv(ctx->dev(), x, X, count * Lm, Lm, 0, s);
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SWITCH_UP, Lm - 1), Lm, K, X,
                           (size_t)Lm * n, x_aux, (size_t)K * n, count, ctx->log_n, s);
  shg::launch_ntt_fwd(ctx->aux_dev(), x_aux, x_aux, count * K, K, s);
}

// ScaleAndReduceRnsBasisInPlace with the context's t of (t_main, t_aux) [count]
// (NTT form both) into out; t_aux is consumed, D [count][Lm][n] scratch.
static void bfv_scale_reduce(shg_context* ctx, uint64_t* out, const uint64_t* t_main,
                             uint64_t* t_aux, uint64_t* D, int count, int Lm, cudaStream_t s) {
  const size_t n = ctx->n;
  const int K = ctx->K;
  shg::launch_ntt_inv(ctx->aux_dev(), t_aux, t_aux, count * K, K, 0, s);
  shg::launch_switch_basis(ctx->d_primes, conv(ctx, CONV_SWITCH_DOWN_T, Lm - 1), K, Lm, t_aux,
                           (size_t)K * n, D, (size_t)Lm * n, count, ctx->log_n, s);
  shg::launch_ntt_fwd(ctx->dev(), D, D, count * Lm, Lm, s);
  std::vector<uint64_t> c(Lm), d(Lm);
  for (int i = 0; i < Lm; ++i) {
    d[i] = p_inv_mod(ctx, i);
    c[i] = mulmod(ctx->t % ctx->hp[i].q, d[i], ctx->hp[i].q);
  }
  combine(ctx, out, t_main, D, c.data(), d.data(), 1, count, Lm, s);
}

int shg_bfv_mul(shg_context* ctx, uint64_t* out, const uint64_t* a, const uint64_t* b,
                int count, int num_limbs, shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, a, b}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int Lm = num_limbs, K = ctx->K;
  const size_t n = ctx->n, pm = (size_t)Lm * n, pa = (size_t)K * n;
  // per ciphertext: X [4][Lm] (a, b coefficient forms; later the deltas),
  // b_aux [2][K], a_aux [2][K], a_main [2][Lm], t_main [3][Lm], t_aux [3][K]
  const size_t per_ct = (9 * pm + 7 * pa) * sizeof(uint64_t);
  const size_t want = ctx->chunk_cts > 0 ? (size_t)ctx->chunk_cts
                                         : std::max<size_t>(1, ((size_t)1 << 30) / per_ct);
  const int C = (int)std::min<size_t>((size_t)count, want);
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws((size_t)C * per_ct))) return st;
  uint64_t* X = ctx->ws;
  uint64_t* b_aux = X + (size_t)C * 4 * pm;
  uint64_t* a_aux = b_aux + (size_t)C * 2 * pa;
  uint64_t* a_main = a_aux + (size_t)C * 2 * pa;
  uint64_t* t_main = a_main + (size_t)C * 2 * pm;
  uint64_t* t_aux = t_main + (size_t)C * 3 * pm;
  for (int c0 = 0; c0 < count; c0 += C) {
    const int cc = std::min(C, count - c0);
    const uint64_t* ac = a + (size_t)c0 * 2 * pm;
    const uint64_t* bc = b + (size_t)c0 * 2 * pm;
    // Q/t * b_j (mod P): b -> coefficient form -> SwitchRnsBasis -> NTT
    bfv_switch_up(ctx, bc, X, b_aux, cc * 2, Lm, s);
    // P/t * a_i (mod P) and (mod Q)
    bfv_scale_up(ctx, ac, X, a_aux, a_main, cc * 2, Lm, s);
    // the tensor product mod Q and mod P
    shg::launch_tensor(ctx->dev(), t_main, a_main, bc, cc, Lm, s);
    shg::launch_tensor(ctx->aux_dev(), t_aux, a_aux, b_aux, cc, K, s);
    // Q/t * tensor (mod Q)
    bfv_scale_reduce(ctx, out + (size_t)c0 * 3 * pm, t_main, t_aux, X, cc * 3, Lm, s);
  }
  return launch_status("bfv_mul");
}

int shg_bfv_absorb(shg_context* ctx, uint64_t* out, const uint64_t* ct,
                   const uint64_t* plaintext, int len, int count, int num_limbs,
                   shg_stream stream) {
  int st = check_aux(ctx, count, num_limbs);
  if (st) return st;
  if (len < 1) return fail(SHG_INVALID_ARGUMENT, "`len` must be positive.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct, plaintext}))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int Lm = num_limbs, K = ctx->K;
  const size_t n = ctx->n, pm = (size_t)Lm * n, pa = (size_t)K * n;
  const int members = count * len;
  // pt_aux [K]; per component: X [Lm], c_aux [K], c_main [Lm]
  const size_t per = (2 * pm + pa) * sizeof(uint64_t);
  const size_t want = ctx->chunk_cts > 0 ? (size_t)ctx->chunk_cts * len
                                         : std::max<size_t>(1, ((size_t)1 << 30) / per);
  const int C = (int)std::min<size_t>((size_t)members, want);
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((st = ctx->ensure_ws(pa * sizeof(uint64_t) + (size_t)C * per))) return st;
  uint64_t* pt_aux = ctx->ws;
  uint64_t* X = pt_aux + pa;
  uint64_t* c_aux = X + (size_t)C * pm;
  uint64_t* c_main = c_aux + (size_t)C * pa;
  // Q/t * plaintext (mod P) (rns/rns_bfv_ciphertext.cc:48-56)
  bfv_switch_up(ctx, plaintext, X, pt_aux, 1, Lm, s);
  for (int m0 = 0; m0 < members; m0 += C) {
    const int mc = std::min(C, members - m0);
    bfv_scale_up(ctx, ct + (size_t)m0 * pm, X, c_aux, c_main, mc, Lm, s);
    shg::ScalarPack none{};
    shg::launch_pointwise(ctx->dev(), shg::PW_MUL_BCAST, c_main, c_main, plaintext, none, mc,
                          Lm, s);
    shg::launch_pointwise(ctx->aux_dev(), shg::PW_MUL_BCAST, c_aux, c_aux, pt_aux, none, mc, K,
                          s);
    bfv_scale_reduce(ctx, out + (size_t)m0 * pm, c_main, c_aux, X, mc, Lm, s);
  }
  return launch_status("bfv_absorb");
}

int shg_context_set_ks_fused(shg_context* ctx, int on) {
  if (!ctx || (on != 0 && on != 1))
    return fail(SHG_INVALID_ARGUMENT, "fused key switch switch must be 0 or 1");
  ctx->ks_fused = on;
  return SHG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free relinearization.
//
// Some callers of this library cannot allocate device memory while they run:
// a host process whose GPU memory is handed out by an external pool or arena
// manager that forbids cudaMalloc, code running while another component holds
// the whole device budget, or a real-time request path where an allocation's
// implicit device synchronization would stall other streams.  For them,
// shg_relin_apply_noalloc runs the same key-switch kernels as
// shg_relin_apply, but its scratch lives in the fixed array below, which is
// part of the library's device image: every GPU that loads the library holds
// these bytes until the process exits, and no call allocates or frees.
// ---------------------------------------------------------------------------

// Scratch of the allocation-free entry point: the exported source limbs and
// the NTT'd digits of one chunk of ciphertexts.  Both are completely
// overwritten before they are read, so nothing needs clearing between calls.
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB
static __device__ __align__(256) uint64_t
    g_noalloc_scratch[kNoAllocScratchBytes / sizeof(uint64_t)];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint64_t* g_noalloc_dev_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// `g_noalloc_scratch` only names a host-side shadow, so the address must come
// from cudaGetSymbolAddress, taken once per device while that device is
// current (this is the set-up done by the first call on each device).
int noalloc_scratch(int device, uint64_t** out) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return fail(SHG_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_dev_ptr[device] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
    g_noalloc_dev_ptr[device] = static_cast<uint64_t*>(p);
  }
  *out = g_noalloc_dev_ptr[device];
  return SHG_OK;
}

}  // namespace

extern "C" int shg_relin_apply_noalloc(shg_context* ctx, const shg_key* key,
                                       uint64_t* out, const uint64_t* ct,
                                       int count, shg_stream stream) {
  int st = check_key(ctx, key);
  if (st) return st;
  if (key->power != 1)
    return fail(SHG_INVALID_ARGUMENT,
                "Relinearization key can only apply to a ciphertext of power 1.");
  if (count < 0) return fail(SHG_INVALID_ARGUMENT, "`count` must be non-negative.");
  if (count == 0) return SHG_OK;
  if ((st = check_ptrs({out, ct}))) return st;
  if (out == ct) return fail(SHG_INVALID_ARGUMENT, "`out` must not alias `ct`");
  int device = -1;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device != ctx->device)
    return fail(SHG_FAILED_PRECONDITION,
                "call shg_relin_apply_noalloc with the context's device current");
  const int L = key->L, n = ctx->n, k = key->k;
  const size_t Ln = (size_t)L * n;
  const size_t per_ct = (Ln + (size_t)k * Ln) * sizeof(uint64_t);
  if (per_ct > kNoAllocScratchBytes)
    return fail(SHG_INVALID_ARGUMENT,
                "shg_relin_apply_noalloc: one ciphertext needs " +
                    std::to_string(per_ct) +
                    " bytes of scratch (n * limbs * (1 + gadget dimension) * 8) "
                    "but the fixed scratch holds " +
                    std::to_string(kNoAllocScratchBytes) + " bytes");
  uint64_t* scratch = nullptr;
  if ((st = noalloc_scratch(device, &scratch))) return st;
  const int C = (int)std::min<size_t>((size_t)count, kNoAllocScratchBytes / per_ct);
  uint64_t* X = scratch;
  uint64_t* D = X + (size_t)C * Ln;
  cudaStream_t s = (cudaStream_t)stream;
  const CtxDev dv = ctx->dev();
  for (int c0 = 0; c0 < count; c0 += C) {
    const int cc = std::min(C, count - c0);
    const uint64_t* src = ct + (size_t)c0 * 3 * Ln;
    shg::launch_intt_export(dv, X, src, 3, 2, 0, CtMap::identity(), cc, L, s);
    shg::launch_keyswitch(dv, D, X, key->d_digits, k, key->digit_flags, key->chunk, key->chunk_lazy,
                          key->kb, key->ka, out + (size_t)c0 * 2 * Ln, src, 3 * Ln,
                          CtMap::identity(), 0, 0, cc, L, s);
  }
  return launch_status("relin_apply_noalloc");
}
