// CUDA kernels of the RLWE polynomial hot path (sm_103a).
//
// Every kernel reads and writes residues in SHELL's Montgomery representation
// and returns canonical values, so results are bit-identical to the
// reference CPU path; see the per-kernel comments for the reference
// functions each one replaces.
#include "kernels.cuh"

namespace shg {

std::atomic<uint64_t> g_launch_count{0};
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<ProfEntry> g_prof_pending;

namespace {


template <int LOG_N>
struct Cfg {
  using C = NttCore<LOG_N>;
  static constexpr int N = C::N;
  static constexpr int E = C::E;
  static constexpr int T = C::T;
  static constexpr int LPC = T >= 256 ? 1 : 256 / T;  // limbs per CTA
  static constexpr int THREADS = T * LPC;
  static constexpr int SMEM = LPC * N * 8;
};

template <class K>
void set_smem(K kernel, int smem) {
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         smem);
  }
}

template <int E>
__device__ __forceinline__ void load_contig(uint64_t (&x)[E],
                                            const uint64_t* p) {
#pragma unroll
  for (int k = 0; k < E; k += 2) {
    ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p + k);
    x[k] = v.x;
    x[k + 1] = v.y;
  }
}

template <int E>
__device__ __forceinline__ void store_contig(uint64_t* p,
                                             const uint64_t (&x)[E]) {
#pragma unroll
  for (int k = 0; k < E; k += 2) {
    *reinterpret_cast<ulonglong2*>(p + k) = make_ulonglong2(x[k], x[k + 1]);
  }
}

// Source position of NTT-domain slot `pos` under X -> X^power
// (rns/rns_polynomial.cc:236-256): out[brv(j)] = in[brv((power-1)/2 +
// j*power mod n)].
template <int LOG_N>
__device__ __forceinline__ int subst_src(int pos, int power) {
  const unsigned j = __brev((unsigned)pos) >> (32 - LOG_N);
  const unsigned t =
      ((unsigned)((power - 1) >> 1) + j * (unsigned)power) & ((1u << LOG_N) - 1);
  return (int)(__brev(t) >> (32 - LOG_N));
}

__device__ __forceinline__ int subst_src_rt(int pos, int power, int log_n) {
  const unsigned j = __brev((unsigned)pos) >> (32 - log_n);
  const unsigned t =
      ((unsigned)((power - 1) >> 1) + j * (unsigned)power) & ((1u << log_n) - 1);
  return (int)(__brev(t) >> (32 - log_n));
}

// Canonical residues at the end of a forward transform.
template <bool LAZY, int E>
__device__ __forceinline__ void finish_forward(uint64_t (&x)[E], uint64_t q,
                                               uint64_t two_q, uint64_t bar) {
#pragma unroll
  for (int k = 0; k < E; ++k)
    x[k] = LAZY ? reduce_full(x[k], q, bar) : reduce_4q(x[k], q, two_q);
}

// --------------------------------------------------------------------------
// Forward / inverse NTT (ForwardNumberTheoreticTransform /
// InverseNumberTheoreticTransform, dft_transformations.h:158-201).
// --------------------------------------------------------------------------

template <int LOG_N, bool LAZY>
__device__ __forceinline__ void ntt_fwd_body(const uint64_t* in, uint64_t* out, int num, int L,
                                             const CtxDev& c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const int l = g % L;
  const uint64_t q = c.primes[l].q, two_q = c.primes[l].two_q;
  const uint64_t* src = in + (size_t)g * C::N;
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; ++k) x[k] = src[C::fwd_in_idx(tid, k)];
  C::template forward<LAZY>(x, tid, smem + sub * C::N,
                            c.tw_fwd + (size_t)l * C::N, 1, q, two_q);
  finish_forward<LAZY, C::E>(x, q, two_q, c.primes[l].barrett);
  if (active) store_contig(out + (size_t)g * C::N + C::fwd_out_idx(tid, 0), x);
}

// The body stays a separate inlined function: written directly in the kernel
// the same code measured 7 % slower at n = 2^12 (a different register
// allocation).
template <int LOG_N, bool LAZY>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_ntt_fwd(const uint64_t* in, uint64_t* out, int num, int L, CtxDev c) {
  ntt_fwd_body<LOG_N, LAZY>(in, out, num, L, c);
}

// scale_mode: 0 -> x n^{-1}; 1 -> x n^{-1} 2^-64 (iNTT fused with ExportInt);
// 2 -> x (sw, swp) given by the caller.
template <int LOG_N, bool WIDE>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_ntt_inv(const uint64_t* in, uint64_t* out, int num, int L, int in_first,
              int in_stride, int scale_mode, uint64_t sw, uint64_t swp,
              CtxDev c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const size_t src_limb = (size_t)in_first + (size_t)g * in_stride;
  const int l = (int)(src_limb % (size_t)L);
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  uint64_t x[C::E];
  load_contig(x, in + src_limb * C::N + C::inv_in_idx(tid, 0));
  C::template inverse<WIDE>(x, tid, smem + sub * C::N, c.tw_inv + (size_t)l * C::N, C::N, 0, q,
             two_q);
  if (scale_mode == 0) {
    sw = P->n_inv;
    swp = P->n_inv_shoup;
  } else if (scale_mode == 1) {
    sw = P->n_inv_r;
    swp = P->n_inv_r_shoup;
  }
  if (active) {
    uint64_t* dst = out + (size_t)g * C::N;
#pragma unroll
    for (int k = 0; k < C::E; ++k)
      dst[C::inv_out_idx(tid, k)] = shoup(x[k], sw, swp, q);
  }
}

// --------------------------------------------------------------------------
// Fused kernels built on the NTT core.
// --------------------------------------------------------------------------

// RnsRlweCiphertext::Mul (rns/rns_ciphertext.h:501-524) for degree-1 inputs,
// fused with ConvertToCoeffForm + ExportInt of the degree-2 component as
// RnsRelinKey::ApplyToRlweCiphertext needs it (rns_relinearization_key.cc:
// 215-218, rns_gadget.cc:130-134).  One CTA per (ciphertext, limb).
template <int LOG_N, bool WIDE>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_tensor_intt(uint64_t* out01, uint64_t* X, const uint64_t* a,
                  const uint64_t* b, int num, int L, CtxDev c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const int ct = g / L, l = g % L;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q, qinv = P->inv_modulus;
  const size_t Ln = (size_t)L * C::N;
  const size_t off = (size_t)ct * 2 * Ln + (size_t)l * C::N + C::inv_in_idx(tid, 0);
  // Two coefficients at a time keeps the live register set at the 16
  // degree-2 values plus one vector of each input.
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; k += 2) {
    const ulonglong2 va0 = *reinterpret_cast<const ulonglong2*>(a + off + k);
    const ulonglong2 va1 = *reinterpret_cast<const ulonglong2*>(a + off + Ln + k);
    const ulonglong2 vb0 = *reinterpret_cast<const ulonglong2*>(b + off + k);
    const ulonglong2 vb1 = *reinterpret_cast<const ulonglong2*>(b + off + Ln + k);
    ulonglong2 r0, r1, r2;
    tensor3_pair(va0, va1, vb0, vb1, q, qinv, r0, r1, r2);
    x[k] = r2.x;  // the degree-2 component
    x[k + 1] = r2.y;
    if (active) {
      *reinterpret_cast<ulonglong2*>(out01 + off + k) = r0;
      *reinterpret_cast<ulonglong2*>(out01 + off + Ln + k) = r1;
    }
  }
  C::template inverse<WIDE>(x, tid, smem + sub * C::N, c.tw_inv + (size_t)l * C::N, C::N, 0,
             q, two_q);
  if (active) {
    uint64_t* dst = X + (size_t)g * C::N;
#pragma unroll
    for (int k = 0; k < C::E; ++k)
      dst[C::inv_out_idx(tid, k)] = shoup(x[k], P->n_inv_r, P->n_inv_r_shoup, q);
  }
}

// ConvertToCoeffForm + ExportInt of one component (optionally substituted
// first), as the key-switch input (rns_galois_key.cc:257-263,
// relinearization_key.cc:148-150).
template <int LOG_N, bool WIDE>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_intt_export(uint64_t* X, const uint64_t* ct, int ncomp, int comp,
                  int subst_power, CtMap map, int num, int L, CtxDev c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const int p = g / L, l = g % L;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t* src =
      ct + (map(p) * ncomp + comp) * (size_t)L * C::N + (size_t)l * C::N;
  uint64_t x[C::E];
  if (subst_power > 0) {
#pragma unroll
    for (int k = 0; k < C::E; ++k)
      x[k] = src[dbg_index(subst_src<LOG_N>(C::inv_in_idx(tid, k), subst_power), C::N, kDbgSubst)];
  } else {
    load_contig(x, src + C::inv_in_idx(tid, 0));
  }
  C::template inverse<WIDE>(x, tid, smem + sub * C::N, c.tw_inv + (size_t)l * C::N, C::N, 0, q,
             two_q);
  if (active) {
    uint64_t* dst = X + (size_t)g * C::N;
#pragma unroll
    for (int k = 0; k < C::E; ++k)
      dst[C::inv_out_idx(tid, k)] = shoup(x[k], P->n_inv_r, P->n_inv_r_shoup, q);
  }
}

// RnsGadget::Decompose (rns/rns_gadget.cc:108-153, BaseDecompose gadget.h:
// 52-79, ConvertModulusBalanced modulus_conversion.h:30-83) fused with the
// per-digit ConvertToNttForm of the key-switch loop
// (rns_relinearization_key.cc:219-226).  One CTA per (ct, digit, out limb).
// The NTT runs on the plain digits; the key is premultiplied by 2^64 so the
// inner product's REDC restores Montgomery form.
// SMALL_IN: digits of at most 32 bits without the lift (need_lift = 0), so
// the first butterfly level takes the 32-bit-operand product.
template <int LOG_N, bool LAZY, bool SMALL_IN = false>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_digit_ntt(uint64_t* D, const uint64_t* X, const DigitDesc* digits, int k,
                int need_lift, int num, int L, CtxDev c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const int j = dbg_index(g % L, c.L, kDbgLimb);
  const int pd = g / L;
  const int idx = pd % k, p = pd / k;
  DigitDesc dd = digits[idx];
  dd.src_limb = dbg_index(dd.src_limb, L, kDbgDigit);
  const PrimeDev* P = c.primes + j;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t* src = X + ((size_t)p * L + dd.src_limb) * C::N;
  uint64_t x[C::E];
  if (!need_lift) {
#pragma unroll
    for (int kk = 0; kk < C::E; ++kk)
      x[kk] = (src[C::fwd_in_idx(tid, kk)] >> dd.shift) & dd.mask;
  } else {
    const PrimeDev* Pi = c.primes + dd.src_limb;
    const uint64_t half_qi = Pi->half_q;
    const uint64_t qi_mod_qj = c.qmod[dd.src_limb * c.L + j];
    const uint64_t bar = P->barrett;
#pragma unroll
    for (int kk = 0; kk < C::E; ++kk) {
      uint64_t v = (src[C::fwd_in_idx(tid, kk)] >> dd.shift) & dd.mask;
      const bool neg = v > half_qi;
      v = reduce_2q(v - mulhi64(v, bar) * q, q);  // v mod q_j
      if (neg && dd.src_limb != j) v += q - qi_mod_qj;
      x[kk] = v;
    }
  }
  C::template forward_m<LAZY, true, typename C::SwzMap, SMALL_IN>(
      x, tid, typename C::SwzMap{smem + sub * C::N}, c.tw_fwd + (size_t)j * C::N, 1, q, two_q);
  // LAZY: D stays below 62 q; the key inner product takes it as it is.
  if constexpr (!LAZY) finish_forward<LAZY, C::E>(x, q, two_q, P->barrett);
  if (active) store_contig(D + (size_t)g * C::N + C::fwd_out_idx(tid, 0), x);
}

// RnsPolynomial::ModReduceLsb, NTT form, second half (rns/rns_polynomial.cc:
// 302-323): balanced lift of the top limb's plain coefficients Y to q_i,
// forward NTT, and out_i = in_i * c1_i + delta_i * c2_i.
template <int LOG_N, bool LAZY>
__global__ void __launch_bounds__(Cfg<LOG_N>::THREADS)
    k_modreduce_lift(uint64_t* out, const uint64_t* Y, const uint64_t* in,
                     ScalarPack sc, int num, int L, CtxDev c) {
  using C = NttCore<LOG_N>;
  using G = Cfg<LOG_N>;
  extern __shared__ uint64_t smem[];
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  int g = blockIdx.x * G::LPC + sub;
  const bool active = g < num;
  if (!active) g = num - 1;
  const int Lr = L - 1;
  const int i = g % Lr, p = g / Lr;
  const PrimeDev* P = c.primes + i;
  const PrimeDev* Pl = c.primes + Lr;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t half_ql = Pl->half_q;
  const uint64_t ql_mod_qi = c.qmod[Lr * c.L + i];
  const uint64_t bar = P->barrett;
  const uint64_t* src = Y + (size_t)p * C::N;
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; ++k) {
    uint64_t y = src[C::fwd_in_idx(tid, k)];
    const bool neg = y > half_ql;
    y = reduce_2q(y - mulhi64(y, bar) * q, q);
    if (neg) y += q - ql_mod_qi;
    x[k] = y;
  }
  C::template forward<LAZY>(x, tid, smem + sub * C::N,
                            c.tw_fwd + (size_t)i * C::N, 1, q, two_q);
  finish_forward<LAZY, C::E>(x, q, two_q, bar);
  const uint64_t c1 = sc.v[4 * i], c1p = sc.v[4 * i + 1];
  const uint64_t c2 = sc.v[4 * i + 2], c2p = sc.v[4 * i + 3];
  const size_t off = ((size_t)p * L + i) * C::N + C::fwd_out_idx(tid, 0);
  uint64_t a[C::E];
  load_contig(a, in + off);
#pragma unroll
  for (int k = 0; k < C::E; ++k) {
    x[k] = reduce_2q_full(shoup(a[k], c1, c1p, q) + shoup(x[k], c2, c2p, q), q);
  }
  if (active)
    store_contig(out + ((size_t)p * Lr + i) * C::N + C::fwd_out_idx(tid, 0), x);
}

// --------------------------------------------------------------------------
// Element-wise kernels.
// --------------------------------------------------------------------------

__global__ void k_pointwise(PwOp op, uint64_t* out, const uint64_t* a,
                            const uint64_t* b, ScalarPack sc, size_t total,
                            int log_n, int L, CtxDev c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x * 2;
  for (size_t e = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
       e < total; e += stride) {
    const int l = (int)((e >> log_n) % (size_t)L);
    const PrimeDev* P = c.primes + l;
    const uint64_t q = P->q;
    const ulonglong2 va = *reinterpret_cast<const ulonglong2*>(a + e);
    ulonglong2 r;
    switch (op) {
      case PW_ADD: {
        const ulonglong2 vb = *reinterpret_cast<const ulonglong2*>(b + e);
        r.x = add_mod(va.x, vb.x, q);
        r.y = add_mod(va.y, vb.y, q);
        break;
      }
      case PW_SUB: {
        const ulonglong2 vb = *reinterpret_cast<const ulonglong2*>(b + e);
        r.x = sub_mod(va.x, vb.x, q);
        r.y = sub_mod(va.y, vb.y, q);
        break;
      }
      case PW_NEG:
        r.x = neg_mod(va.x, q);
        r.y = neg_mod(va.y, q);
        break;
      case PW_MUL: {
        const ulonglong2 vb = *reinterpret_cast<const ulonglong2*>(b + e);
        r.x = mont_mul(va.x, vb.x, q, P->inv_modulus);
        r.y = mont_mul(va.y, vb.y, q, P->inv_modulus);
        break;
      }
      case PW_FMA: {
        // acc (out) += a * b  (FusedMulAddInPlace, montgomery.h:446-465)
        const ulonglong2 vb = *reinterpret_cast<const ulonglong2*>(b + e);
        const ulonglong2 acc = *reinterpret_cast<const ulonglong2*>(out + e);
        r.x = add_mod(acc.x, mont_mul(va.x, vb.x, q, P->inv_modulus), q);
        r.y = add_mod(acc.y, mont_mul(va.y, vb.y, q, P->inv_modulus), q);
        break;
      }
      case PW_MUL_BCAST: {
        const ulonglong2 vb =
            *reinterpret_cast<const ulonglong2*>(b + (e % ((size_t)L << log_n)));
        r.x = mont_mul(va.x, vb.x, q, P->inv_modulus);
        r.y = mont_mul(va.y, vb.y, q, P->inv_modulus);
        break;
      }
      case PW_MUL_MONT: {
        const uint64_t s = sc.v[l];
        r.x = mont_mul(va.x, s, q, P->inv_modulus);
        r.y = mont_mul(va.y, s, q, P->inv_modulus);
        break;
      }
      case PW_MUL_SHOUP:
      default: {
        const uint64_t w = sc.v[2 * l], wp = sc.v[2 * l + 1];
        r.x = shoup(va.x, w, wp, q);
        r.y = shoup(va.y, w, wp, q);
        break;
      }
    }
    *reinterpret_cast<ulonglong2*>(out + e) = r;
  }
}

__global__ void k_substitute(uint64_t* out, const uint64_t* in, int power,
                             size_t total, int log_n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t nmask = ((size_t)1 << log_n) - 1;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const int pos = (int)(e & nmask);
    out[e] = in[(e & ~nmask) |
               (size_t)dbg_index(subst_src_rt(pos, power, log_n), 1LL << log_n, kDbgSubst)];
  }
}

__global__ void k_tensor(uint64_t* out, const uint64_t* a, const uint64_t* b,
                         size_t total /* count*L*n */, int log_n, int L,
                         CtxDev c) {
  const size_t Ln = (size_t)L << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t ct = e / Ln, r = e % Ln;
    const int l = (int)(r >> log_n);
    const PrimeDev* P = c.primes + l;
    const uint64_t q = P->q, qinv = P->inv_modulus;
    const uint64_t a0 = a[ct * 2 * Ln + r], a1 = a[ct * 2 * Ln + Ln + r];
    const uint64_t b0 = b[ct * 2 * Ln + r], b1 = b[ct * 2 * Ln + Ln + r];
    uint64_t c0, c1, c2;
    tensor3(a0, a1, b0, b1, q, qinv, c0, c1, c2);
    out[ct * 3 * Ln + r] = c0;
    out[ct * 3 * Ln + Ln + r] = c1;
    out[ct * 3 * Ln + 2 * Ln + r] = c2;
  }
}

// Key inner product of the gadget key switch (rns_relinearization_key.cc:
// 219-226, rns_galois_key.cc:265-283, relinearization_key.cc:76-96): 128-bit
// lazy accumulation of raw products, one REDC per `chunk` terms.
__global__ void k_ks_inner(uint64_t* out, const uint64_t* D, const uint64_t* kb,
                           const uint64_t* ka, int k, int chunk,
                           const uint64_t* base, size_t base_ct_elems,
                           CtMap map, int base1_zero, int subst_power,
                           int p0, int log_n, int L, KeyTable kt, CtxDev c) {
  // blockIdx.y: ciphertext p0 + y; x covers its L * n slots.
  const int Ln = L << log_n;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= Ln) return;
  const size_t p = (size_t)p0 + blockIdx.y;
  if (kt.kb) {
    const size_t e = dbg_index(p >> kt.shift, kt.entries ? kt.entries : (1LL << 62), kDbgKeyTable);
    kb = kt.kb[e];
    ka = kt.ka[e];
  }
  const int l = r >> log_n;
  const int pos = r & ((1 << log_n) - 1);
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, qinv = P->inv_modulus;
  const uint64_t* dp = D + p * (size_t)k * Ln + r;
  const uint64_t* pb = kb + r;
  const uint64_t* pa = ka + r;
  uint64_t s0 = 0, s1 = 0;
  for (int j0 = 0; j0 < k; j0 += chunk) {
    const int j1 = min(k, j0 + chunk);
    uint64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
#pragma unroll 4
    for (int j = j0; j < j1; ++j) {
      const uint64_t d = *dp;
      mac128(lo0, hi0, d, __ldg(pb));
      mac128(lo1, hi1, d, __ldg(pa));
      dp += Ln;
      pb += Ln;
      pa += Ln;
    }
    s0 = add_mod(s0, redc128(lo0, hi0, q, qinv), q);
    s1 = add_mod(s1, redc128(lo1, hi1, q, qinv), q);
  }
  const uint64_t* bp = base + map(p) * base_ct_elems + ((size_t)l << log_n);
  const int pos0 = subst_power > 0
                       ? dbg_index(subst_src_rt(pos, subst_power, log_n), 1LL << log_n, kDbgSubst)
                       : pos;
  const uint64_t b0 = bp[pos0];
  const uint64_t b1 = base1_zero ? 0 : bp[(size_t)Ln + pos];
  out[p * 2 * Ln + r] = add_mod(b0, s0, q);
  out[p * 2 * Ln + Ln + r] = add_mod(b1, s1, q);
}

// RnsGaloisKey with a precomputed random pad (rns/rns_galois_key.cc:289-346):
// the digits pad [count][k][L][n] are Montgomery NTT polynomials, so the
// products with the stored keys (premultiplied by 2^64) need one REDC per
// chunk and one more for the Montgomery scaling: the lazy 128-bit sum of
// LazyRnsPolynomial and its export give the same canonical value.
// mode 0 (PrecomputeRandomPad): out [count][L][n] = sum_j pad_j * key_a_j.
// mode 1 (ApplyToRlweCiphertextWithRandomPad): out [count][2][L][n] =
// (c0 + sum_j pad_j * key_b_j, pad_new).
__global__ void k_pad_inner(uint64_t* out, const uint64_t* pad, const uint64_t* key,
                            int k, int chunk, const uint64_t* ct, const uint64_t* pad_new,
                            int mode, int log_n, int L, CtxDev c) {
  const int Ln = L << log_n;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= Ln) return;
  const size_t p = blockIdx.y;
  const int l = r >> log_n;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, qinv = P->inv_modulus;
  const uint64_t* dp = pad + p * (size_t)k * Ln + r;
  const uint64_t* kp = key + r;
  uint64_t s = 0;
  for (int j0 = 0; j0 < k; j0 += chunk) {
    const int j1 = min(k, j0 + chunk);
    uint64_t lo = 0, hi = 0;
    for (int j = j0; j < j1; ++j) {
      mac128(lo, hi, *dp, __ldg(kp));
      dp += Ln;
      kp += Ln;
    }
    s = add_mod(s, redc128(lo, hi, q, qinv), q);
  }
  s = redc128(s, 0, q, qinv);
  if (mode == 0) {
    out[p * Ln + r] = s;
  } else {
    out[p * 2 * Ln + r] = add_mod(ct[p * 2 * Ln + r], s, q);
    out[p * 2 * Ln + Ln + r] = pad_new[p * Ln + r];
  }
}

// RnsGadget::Decompose (rns/rns_gadget.cc:108-153) of coefficient-form
// polys: digit d of limb i's exported residue (BaseDecompose, gadget.h:
// 50-79), imported to limb i as is and to every other limb l through
// ConvertModulusBalanced (modulus_conversion.h:30-157: values above
// floor(q_i/2) stand for value - q_i).  out [count][k][L][n], Montgomery
// form, coefficient domain.
__global__ void k_decompose(uint64_t* out, const uint64_t* in, GadgetBases gb,
                            int k, size_t total /* count*k*L*n */, int log_n,
                            int L, CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const size_t Ln = (size_t)L * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e / ((size_t)k * Ln), r = e % ((size_t)k * Ln);
    const int di = (int)(r / Ln);
    const size_t rem = r % Ln;
    const int l = (int)(rem >> log_n);
    const size_t pos = rem & (n - 1);
    int i = 0, d = di;
    for (; i < L; ++i) {
      const int dims = ((int)c.primes[i].log_q + gb.log_b[i] - 1) / gb.log_b[i];
      if (d < dims) break;
      d -= dims;
    }
    const PrimeDev* Pi = c.primes + i;
    const PrimeDev* Pl = c.primes + l;
    const int b = gb.log_b[i];
    const uint64_t x = shoup(in[(p * L + i) * n + pos], Pi->inv_r, Pi->inv_r_shoup, Pi->q);
    uint64_t v = (x >> (d * b)) & ((uint64_t(1) << b) - 1);
    if (l != i) {
      const bool neg = v > Pi->half_q;
      v = reduce_full(v, Pl->q, Pl->barrett);
      if (neg) v = reduce_2q(v + (Pl->q - c.qmod[i * c.L + l]), Pl->q);
    }
    out[e] = shoup(v, Pl->r_mod_q, Pl->r_mod_q_shoup, Pl->q);
  }
}

// ModReduceLsb, coefficient form (rns/rns_polynomial.cc:324-342).
__global__ void k_modreduce_coeff(uint64_t* out, const uint64_t* in,
                                  uint64_t k_plain, uint64_t k_shoup,
                                  ScalarPack sc, size_t total /*count*(L-1)*n*/,
                                  int log_n, int L, CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const int Lr = L - 1;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const PrimeDev* Pl = c.primes + Lr;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e / ((size_t)Lr * n), r = e % ((size_t)Lr * n);
    const int i = (int)(r >> log_n);
    const size_t pos = r & (n - 1);
    const PrimeDev* P = c.primes + i;
    const uint64_t q = P->q;
    // plain value of (a_l * k) mod q_l
    uint64_t y = shoup(in[(p * L + Lr) * n + pos], k_plain, k_shoup, Pl->q);
    const bool neg = y > Pl->half_q;
    y = reduce_2q(y - mulhi64(y, P->barrett) * q, q);
    if (neg) y = reduce_2q(y + q - c.qmod[Lr * c.L + i], q);
    const uint64_t a = in[(p * L + i) * n + pos];
    out[e] = reduce_2q_full(shoup(a, sc.v[4 * i], sc.v[4 * i + 1], q) +
                                shoup(y, sc.v[4 * i + 2], sc.v[4 * i + 3], q),
                            q);
  }
}

// ExpandCiphertext's per-level update (oblivious_expand.h:216-223).
__global__ void k_expand_combine(uint64_t* base, const uint64_t* ks,
                                 const uint64_t* mono, CtMap map, int half,
                                 size_t total /* count*2*n */, int log_n,
                                 CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uint64_t q = c.primes[0].q, qinv = c.primes[0].inv_modulus;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e / (2 * n), r = e % (2 * n);
    uint64_t* cp = base + map(p) * 2 * n + r;
    uint64_t* hp = cp + (size_t)half * 2 * n;
    const uint64_t cv = *cp, kv = ks[e];
    *hp = mont_mul(sub_mod(cv, kv, q), mono[r & (n - 1)], q, qinv);
    *cp = add_mod(cv, kv, q);
  }
}

// Monomials -x^{n - 2^j}, j < levels, in coefficient form
// (oblivious_expand.h:197-200): row j is zero but for coefficient n - 2^j,
// which is `minus_one` (the Montgomery form of -1).
__global__ void k_monomials(uint64_t* mono, int levels, int log_n,
                            uint64_t minus_one) {
  const size_t n = (size_t)1 << log_n;
  const size_t total = (size_t)levels * n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const int j = (int)(e >> log_n);
    const size_t i = e & (n - 1);
    mono[e] = i == n - ((size_t)1 << j) ? minus_one : 0;
  }
}

// MontgomeryInt::DeserializeVector (montgomery.cc:186-215) of every limb:
// value i of a limb stream is stream bits [i*b, i*b + b) (TranscribeBits,
// transcription.h:43-118, least significant bit first).  WORDS: every limb
// stream starts on an 8-byte boundary (n * b a multiple of 64), so a value is
// read from at most two aligned 64-bit words; otherwise bytes are gathered.
template <bool WORDS>
__global__ void k_deserialize(uint64_t* polys, const uint8_t* in, SerLayout lay,
                              size_t total /* count*L*n */, int log_n, int L) {
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t pl = e >> log_n, i = e & (n - 1);
    const size_t p = pl / L;
    const int l = (int)(pl % L);
    const int b = lay.bits[l];
    const uint8_t* stream = in + p * lay.offset[L] + lay.offset[l];
    const size_t bit = i * (size_t)b;
    const uint64_t mask = b == 64 ? ~0ull : ((1ull << b) - 1);
    uint64_t v;
    if (WORDS) {
      const uint64_t* w = reinterpret_cast<const uint64_t*>(stream);
      const size_t w0 = bit >> 6;
      const int o = (int)(bit & 63);
      v = w[w0] >> o;
      if (o + b > 64) v |= w[w0 + 1] << (64 - o);
    } else {
      const size_t byte0 = bit >> 3;
      const int o = (int)(bit & 7);
      const int nbytes = (o + b + 7) >> 3;
      unsigned __int128 acc = 0;
      for (int k = 0; k < nbytes; ++k)
        acc |= (unsigned __int128)stream[byte0 + k] << (8 * k);
      v = (uint64_t)(acc >> o);
    }
    polys[e] = v & mask;
  }
}

// MontgomeryInt::SerializeVector (montgomery.cc:142-166) of every limb: one
// thread per output unit (a 64-bit word, or a byte without WORDS) ORs in the
// parts of the values that overlap it.
template <bool WORDS>
__global__ void k_serialize(uint8_t* out, const uint64_t* polys, SerLayout lay,
                            size_t units_per_poly, size_t total /* count*units */,
                            int log_n, int L) {
  const size_t n = (size_t)1 << log_n;
  const int U = WORDS ? 64 : 8;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e / units_per_poly, u = e % units_per_poly;
    // limb of this unit: offsets are multiples of the unit
    int l = 0;
    while (l + 1 < L && (size_t)lay.offset[l + 1] * 8 / U <= u) ++l;
    const int b = lay.bits[l];
    const size_t bit0 = (u - (size_t)lay.offset[l] * 8 / U) * U;  // stream bit of the unit
    const uint64_t* vals = polys + (p * L + l) * n;
    const size_t stream_bits = n * (size_t)b;
    uint64_t acc = 0;
    for (size_t i = bit0 / b; i < n && i * (size_t)b < bit0 + U && i * (size_t)b < stream_bits;
         ++i) {
      const long long sh = (long long)(i * (size_t)b) - (long long)bit0;  // value bit 0 in the unit
      const uint64_t v = vals[i] & (b == 64 ? ~0ull : ((1ull << b) - 1));
      if (sh >= 0)
        acc |= sh < 64 ? v << sh : 0;
      else
        acc |= v >> (-sh);
    }
    if (WORDS) {
      reinterpret_cast<uint64_t*>(out)[e] = acc;
    } else {
      out[e] = (uint8_t)acc;
    }
  }
}

// Symmetric RLWE encryption combine (symmetric_encryption.h:940-963,
// 1006-1021) on limb 0: out [count][2][n] = (e_ntt * t + m + a * s, -a).
__global__ void k_sym_encrypt(uint64_t* out, const uint64_t* e_ntt, const uint64_t* a,
                              const uint64_t* m, const uint64_t* sk, uint64_t t_mont,
                              size_t total /* count*n */, int log_n, CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uint64_t q = c.primes[0].q, qinv = c.primes[0].inv_modulus;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e >> log_n, i = e & (n - 1);
    uint64_t c0 = mont_mul(e_ntt[e], t_mont, q, qinv);
    c0 = add_mod(c0, m[e], q);
    c0 = add_mod(c0, mont_mul(a[e], sk[i], q, qinv), q);
    out[p * 2 * n + i] = c0;
    out[p * 2 * n + n + i] = neg_mod(a[e], q);
  }
}

// ExtractErrorAndMessage's dot product (symmetric_encryption.h:966-1000) on
// limb 0: acc [count][n] = sum_i ct[count][i] * s^i, NTT form.
__global__ void k_sym_dot(uint64_t* acc, const uint64_t* ct, const uint64_t* sk, int len,
                          size_t total /* count*n */, int log_n, CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uint64_t q = c.primes[0].q, qinv = c.primes[0].inv_modulus;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t p = e >> log_n, i = e & (n - 1);
    const uint64_t* cp = ct + p * (size_t)len * n + i;
    const uint64_t s = sk[i];
    uint64_t sum = cp[0], pw = s;
    for (int j = 1; j < len; ++j) {
      sum = add_mod(sum, mont_mul(cp[(size_t)j * n], pw, q, qinv), q);
      if (j + 1 < len) pw = mont_mul(pw, s, q, qinv);
    }
    acc[e] = sum;
  }
}

// RemoveError (symmetric_encryption.h:1084-1110) on exported coefficients:
// values above floor(q/2) stand for value - q; the message is that mod t.
__global__ void k_remove_error(uint64_t* out, const uint64_t* x, size_t total, uint64_t q,
                               uint64_t t, uint64_t q_mod_t) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    uint64_t v = x[e];
    if (v > (q >> 1)) v -= q_mod_t;
    out[e] = v % t;
  }
}

// Seeded uniform residues: element e of [count][L][n] is splitmix64 output
// e + 1 of state `seed`, reduced mod its limb's prime.
__global__ void k_fill_uniform(uint64_t* out, uint64_t seed, size_t total,
                               int log_n, int L, CtxDev c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    uint64_t z = seed + (uint64_t)(e + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int l = (int)((e >> log_n) % (size_t)L);
    out[e] = z % c.primes[l].q;
  }
}

// Operand gather / result scatter of the batch executor: `count` blocks of
// `elems` uint64 (a multiple of 2, 16-byte aligned) between a contiguous
// buffer and a device table of block pointers.
__global__ void k_gather(uint64_t* dst, const uint64_t* const* srcs, size_t elems,
                         size_t total /* count*elems/2 */) {
  const size_t half = elems / 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t b = e / half, i = e % half;
    reinterpret_cast<ulonglong2*>(dst)[e] =
        reinterpret_cast<const ulonglong2*>(srcs[b])[i];
  }
}

__global__ void k_scatter(uint64_t* const* dsts, const uint64_t* src, size_t elems,
                          size_t total /* count*elems/2 */) {
  const size_t half = elems / 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t b = e / half, i = e % half;
    reinterpret_cast<ulonglong2*>(dsts[b])[i] =
        reinterpret_cast<const ulonglong2*>(src)[e];
  }
}

// FusedAbsorbAddInPlace chain (symmetric_encryption.h:250-275).
__global__ void k_absorb_sum(uint64_t* out, const uint64_t* cts,
                             const uint64_t* db, int num_items,
                             size_t item_stride, int chunk,
                             size_t total /* count*2*n */, int log_n,
                             CtxDev c) {
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uint64_t q = c.primes[0].q, qinv = c.primes[0].inv_modulus;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += stride) {
    const size_t qi = e / (2 * n), r = e % (2 * n);
    const size_t pos = r & (n - 1);
    const uint64_t* cp = cts + qi * item_stride * 2 * n + r;
    uint64_t s = 0;
    for (int i0 = 0; i0 < num_items; i0 += chunk) {
      const int i1 = min(num_items, i0 + chunk);
      uint64_t lo = 0, hi = 0;
      for (int i = i0; i < i1; ++i)
        mac128(lo, hi, cp[(size_t)i * 2 * n], __ldg(db + (size_t)i * n + pos));
      s = add_mod(s, redc128(lo, hi, q, qinv), q);
    }
    out[e] = s;
  }
}

}  // namespace

int grid_for(size_t work, int threads) {
  size_t blocks = (work + threads - 1) / threads;
  const size_t cap = 152 * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

namespace {

// Runtime log_n -> template dispatch for CTA-resident transforms.
#define SHG_DISPATCH_LOGN(log_n, F)                                  \
  switch (log_n) {                                                   \
    case 1: F(1); break;                                             \
    case 2: F(2); break;                                             \
    case 3: F(3); break;                                             \
    case 4: F(4); break;                                             \
    case 5: F(5); break;                                             \
    case 6: F(6); break;                                             \
    case 7: F(7); break;                                             \
    case 8: F(8); break;                                             \
    case 9: F(9); break;                                             \
    case 10: F(10); break;                                           \
    case 11: F(11); break;                                           \
    case 12: F(12); break;                                           \
    case 13: F(13); break;                                           \
    case 14: F(14); break;                                           \
    default: break;                                                  \
  }

// Transforms of n >= 2^ntt4_min (always n = 2^15) run as two four-step
// phase kernels (ntt4.cu); smaller ones as one CTA-resident kernel.
bool use_ntt4(const CtxDev& c) { return c.log_n >= c.ntt4_min || c.log_n > 14; }
bool use_ntt4_plain(const CtxDev& c) {
  return c.log_n >= 12 && (c.log_n >= c.ntt4_plain_min || c.log_n > 14);
}

template <int LOG_N>
int blocks_for(int num) {
  return (num + Cfg<LOG_N>::LPC - 1) / Cfg<LOG_N>::LPC;
}

}  // namespace

void launch_ntt_fwd(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                    int L, cudaStream_t s) {
  if (num <= 0) return;
  LaunchScope scope_("ntt_fwd", s);
  if (use_ntt4_plain(c)) {
    g_launch_count++;  // second phase kernel
    launch4_ntt_fwd(c, in, out, num, L, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_ntt_fwd<LN, true> : k_ntt_fwd<LN, false>;  \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        in, out, num, L, c);                                                  \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

// plain: a plain inverse NTT call (the plain-NTT threshold applies).
static void launch_ntt_inv_scaled(const CtxDev& c, const uint64_t* in,
                                  uint64_t* out, int num, int L, int in_first,
                                  int in_stride, int mode, uint64_t sw,
                                  uint64_t swp, cudaStream_t s, bool plain = false) {
  if (num <= 0) return;
  LaunchScope scope_("ntt_inv", s);
  if (plain ? use_ntt4_plain(c) : use_ntt4(c)) {
    g_launch_count++;  // second phase kernel
    launch4_ntt_inv(c, in, out, num, L, in_first, in_stride, mode, sw, swp, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_ntt_inv<LN, true> : k_ntt_inv<LN, false>;                                                \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        in, out, num, L, in_first, in_stride, mode, sw, swp, c);              \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

void launch_ntt_inv(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                    int L, int scale_export, cudaStream_t s) {
  launch_ntt_inv_scaled(c, in, out, num, L, 0, 1, scale_export ? 1 : 0, 0, 0,
                        s, /*plain=*/true);
}

void launch_pointwise(const CtxDev& c, PwOp op, uint64_t* out, const uint64_t* a,
                      const uint64_t* b, const ScalarPack& sc, int count, int L,
                      cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("pointwise", s);
  k_pointwise<<<grid_for(total / 2, 256), 256, 0, s>>>(op, out, a, b, sc, total,
                                                       c.log_n, L, c);
}

void launch_substitute(const CtxDev& c, uint64_t* out, const uint64_t* in,
                       int power, int count, int L, cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("substitute", s);
  k_substitute<<<grid_for(total, 256), 256, 0, s>>>(out, in, power, total,
                                                    c.log_n);
}

void launch_tensor(const CtxDev& c, uint64_t* out, const uint64_t* a,
                   const uint64_t* b, int count, int L, cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("tensor", s);
  k_tensor<<<grid_for(total, 256), 256, 0, s>>>(out, a, b, total, c.log_n, L,
                                                c);
}

void launch_tensor_intt(const CtxDev& c, uint64_t* out01, uint64_t* X,
                        const uint64_t* a, const uint64_t* b, int count, int L,
                        cudaStream_t s) {
  const int num = count * L;
  if (num <= 0) return;
  LaunchScope scope_("tensor_intt", s);
  if (use_ntt4(c)) {
    g_launch_count++;  // second phase kernel
    launch4_tensor_intt(c, out01, X, a, b, count, L, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_tensor_intt<LN, true> : k_tensor_intt<LN, false>;                                            \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        out01, X, a, b, num, L, c);                                           \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

void launch_intt_export(const CtxDev& c, uint64_t* X, const uint64_t* ct,
                        int ncomp, int comp, int subst_power, CtMap map,
                        int count, int L, cudaStream_t s) {
  const int num = count * L;
  if (num <= 0) return;
  LaunchScope scope_("intt_export", s);
  if (use_ntt4(c)) {
    g_launch_count++;  // second phase kernel
    launch4_intt_export(c, X, ct, ncomp, comp, subst_power, map, count, L, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_intt_export<LN, true> : k_intt_export<LN, false>;                                            \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        X, ct, ncomp, comp, subst_power, map, num, L, c);                     \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

void launch_digit_ntt(const CtxDev& c, uint64_t* D, const uint64_t* X,
                      const DigitDesc* digits, int k, int digit_flags, int count,
                      int L, cudaStream_t s) {
  const int num = count * k * L;
  if (num <= 0) return;
  const int need_lift = digit_flags & 1;
  LaunchScope scope_("digit_ntt", s);
  if (use_ntt4(c)) {
    g_launch_count++;  // second phase kernel
    launch4_digit_ntt(c, D, X, digits, k, digit_flags, count, L, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_digit_ntt<LN, true> : k_digit_ntt<LN, false>;  \
    if (digit_flags == 0)                                                     \
      kern = c.small_q ? k_digit_ntt<LN, true, true> : k_digit_ntt<LN, false, true>; \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        D, X, digits, k, need_lift, num, L, c);                               \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

void launch_ks_inner(const CtxDev& c, uint64_t* out, const uint64_t* D,
                     const uint64_t* kb, const uint64_t* ka, int k, int chunk,
                     const uint64_t* base, size_t base_ct_elems, CtMap map,
                     int base1_zero, int subst_power, int count, int L,
                     cudaStream_t s, const KeyTable& kt) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("ks_inner", s);
  // One slot of one ciphertext per thread: blocking several ciphertexts per
  // thread to reuse key loads measured slower (lower occupancy, fewer loads
  // in flight).  Grid: x over the L * n slots, y over ciphertexts.
  const int Ln = L << c.log_n;
  const dim3 block(256);
  for (int p0 = 0; p0 < count; p0 += 65535) {
    const dim3 grid((Ln + 255) / 256, std::min(count - p0, 65535));
    k_ks_inner<<<grid, block, 0, s>>>(out, D, kb, ka, k, chunk, base, base_ct_elems,
                                      map, base1_zero, subst_power, p0, c.log_n, L, kt,
                                      c);
  }
}

void launch_keyswitch(const CtxDev& c, uint64_t* D, const uint64_t* X,
                      const DigitDesc* digits, int k, int digit_flags, int chunk,
                      int chunk_lazy,
                      const uint64_t* kb, const uint64_t* ka, uint64_t* out,
                      const uint64_t* base, size_t base_ct_elems, CtMap map,
                      int base1_zero, int subst_power, int count, int L,
                      cudaStream_t s, const KeyTable& kt) {
  if (count <= 0) return;
  const int need_lift = digit_flags & 1;
  if (use_ntt4(c) && c.ks_fused && ks4_rows_per_cta(k) > 0) {
    {
      LaunchScope scope_("digit_cols", s);
      launch4_digit_cols(c, D, X, digits, k, digit_flags, count, L, s);
    }
    LaunchScope scope_("ks_rows", s);
    // small primes: the row kernel skips the final reduction (chunk_lazy)
    launch4_ks_rows(c, D, k, c.small_q ? chunk_lazy : chunk, kb, ka, out, base,
                    base_ct_elems, map,
                    base1_zero, subst_power, count, L, s, kt);
    return;
  }
  // The digit transforms come out lazily reduced for small primes (below
  // 62 q), which chunk_lazy covers; canonical ones are covered a fortiori.
  launch_digit_ntt(c, D, X, digits, k, digit_flags, count, L, s);
  launch_ks_inner(c, out, D, kb, ka, k, c.small_q ? chunk_lazy : chunk, base, base_ct_elems,
                  map,
                  base1_zero, subst_power, count, L, s, kt);
}

void launch_modreduce_ntt(const CtxDev& c, uint64_t* out, uint64_t* Y,
                          const uint64_t* in, uint64_t k_plain,
                          uint64_t k_shoup, const ScalarPack& sc, int count,
                          int L, cudaStream_t s) {
  if (count <= 0) return;
  // Stage 1 (rns_polynomial.cc:286-306): the top limb of every poly (limb
  // L-1, stride L limbs), multiplied by k, inverse NTT and ExportInt, all
  // folded into one scale k * n^{-1} * 2^-64 -> Y [count][n] plain.
  launch_ntt_inv_scaled(c, in, Y, count, L, L - 1, L, 2, k_plain, k_shoup, s);
  // Stage 2: lift, forward NTT, combine.
  LaunchScope scope_("modreduce_lift", s);
  if (use_ntt4(c)) {
    g_launch_count++;  // second phase kernel
    launch4_modreduce_lift(c, out, Y, in, sc, count, L, s);
    return;
  }
#define F(LN)                                                                 \
  {                                                                           \
    auto kern = c.small_q ? k_modreduce_lift<LN, true> : k_modreduce_lift<LN, false>;  \
    set_smem(kern, Cfg<LN>::SMEM);                                            \
    const int num = count * (L - 1);                                          \
    kern<<<blocks_for<LN>(num), Cfg<LN>::THREADS, Cfg<LN>::SMEM, s>>>(        \
        out, Y, in, sc, num, L, c);                                           \
  }
  SHG_DISPATCH_LOGN(c.log_n, F)
#undef F
}

void launch_modreduce_coeff(const CtxDev& c, uint64_t* out, const uint64_t* in,
                            uint64_t k_plain, uint64_t k_shoup,
                            const ScalarPack& sc, int count, int L,
                            cudaStream_t s) {
  const size_t total = (size_t)count * (L - 1) * c.n;
  if (total == 0) return;
  LaunchScope scope_("modreduce_coeff", s);
  k_modreduce_coeff<<<grid_for(total, 256), 256, 0, s>>>(
      out, in, k_plain, k_shoup, sc, total, c.log_n, L, c);
}

void launch_pad_inner(const CtxDev& c, uint64_t* out, const uint64_t* pad,
                      const uint64_t* key, int k, int chunk, const uint64_t* ct,
                      const uint64_t* pad_new, int mode, int count, int L, cudaStream_t s) {
  if (count <= 0) return;
  LaunchScope scope_("pad_inner", s);
  const int Ln = L << c.log_n;
  for (int p0 = 0; p0 < count; p0 += 65535) {
    const int cc = std::min(count - p0, 65535);
    const dim3 grid((Ln + 255) / 256, cc);
    const size_t o_out = (size_t)p0 * (mode == 0 ? 1 : 2) * Ln;
    k_pad_inner<<<grid, 256, 0, s>>>(out + o_out, pad + (size_t)p0 * k * Ln, key, k, chunk,
                                     ct ? ct + (size_t)p0 * 2 * Ln : nullptr,
                                     pad_new ? pad_new + (size_t)p0 * Ln : nullptr, mode,
                                     c.log_n, L, c);
  }
}

void launch_decompose(const CtxDev& c, uint64_t* out, const uint64_t* in,
                      const GadgetBases& gb, int k, int count, int L,
                      cudaStream_t s) {
  const size_t total = (size_t)count * k * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("decompose", s);
  k_decompose<<<grid_for(total, 256), 256, 0, s>>>(out, in, gb, k, total,
                                                   c.log_n, L, c);
}

void launch_expand_combine(const CtxDev& c, uint64_t* base, const uint64_t* ks,
                           const uint64_t* mono, CtMap map, int half,
                           int count, cudaStream_t s) {
  const size_t total = (size_t)count * 2 * c.n;
  if (total == 0) return;
  LaunchScope scope_("expand_combine", s);
  k_expand_combine<<<grid_for(total, 256), 256, 0, s>>>(base, ks, mono, map,
                                                        half, total, c.log_n, c);
}

void launch_deserialize(const CtxDev& c, uint64_t* polys, const uint8_t* in,
                        const SerLayout& lay, int count, int L, cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("deserialize", s);
  if (lay.offset[L] % 8 == 0 && c.n >= 64)
    k_deserialize<true><<<grid_for(total, 256), 256, 0, s>>>(polys, in, lay, total, c.log_n, L);
  else
    k_deserialize<false><<<grid_for(total, 256), 256, 0, s>>>(polys, in, lay, total, c.log_n, L);
}

void launch_serialize(const CtxDev& c, uint8_t* out, const uint64_t* polys,
                      const SerLayout& lay, int count, int L, cudaStream_t s) {
  if (count <= 0) return;
  LaunchScope scope_("serialize", s);
  if (lay.offset[L] % 8 == 0 && c.n >= 64) {
    const size_t units = lay.offset[L] / 8, total = units * count;
    k_serialize<true><<<grid_for(total, 256), 256, 0, s>>>(out, polys, lay, units, total,
                                                           c.log_n, L);
  } else {
    const size_t units = lay.offset[L], total = units * count;
    k_serialize<false><<<grid_for(total, 256), 256, 0, s>>>(out, polys, lay, units, total,
                                                            c.log_n, L);
  }
}

void launch_sym_encrypt(const CtxDev& c, uint64_t* out, const uint64_t* e_ntt,
                        const uint64_t* a, const uint64_t* m, const uint64_t* sk,
                        uint64_t t_mont, int count, cudaStream_t s) {
  const size_t total = (size_t)count * c.n;
  if (total == 0) return;
  LaunchScope scope_("sym_encrypt", s);
  k_sym_encrypt<<<grid_for(total, 256), 256, 0, s>>>(out, e_ntt, a, m, sk, t_mont, total,
                                                     c.log_n, c);
}

void launch_sym_dot(const CtxDev& c, uint64_t* acc, const uint64_t* ct, const uint64_t* sk,
                    int len, int count, cudaStream_t s) {
  const size_t total = (size_t)count * c.n;
  if (total == 0) return;
  LaunchScope scope_("sym_dot", s);
  k_sym_dot<<<grid_for(total, 256), 256, 0, s>>>(acc, ct, sk, len, total, c.log_n, c);
}

void launch_remove_error(const CtxDev& c, uint64_t* out, const uint64_t* x, uint64_t q,
                         uint64_t t, int count, cudaStream_t s) {
  const size_t total = (size_t)count * c.n;
  if (total == 0) return;
  LaunchScope scope_("remove_error", s);
  k_remove_error<<<grid_for(total, 256), 256, 0, s>>>(out, x, total, q, t, q % t);
}

void launch_fill_uniform(const CtxDev& c, uint64_t* out, uint64_t seed, int count,
                         int L, cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("fill_uniform", s);
  k_fill_uniform<<<grid_for(total, 256), 256, 0, s>>>(out, seed, total, c.log_n, L, c);
}

void launch_gather(uint64_t* dst, const uint64_t* const* srcs, size_t elems, int count,
                   cudaStream_t s) {
  const size_t total = (size_t)count * (elems / 2);
  if (total == 0) return;
  LaunchScope scope_("gather", s);
  k_gather<<<grid_for(total, 256), 256, 0, s>>>(dst, srcs, elems, total);
}

void launch_scatter(uint64_t* const* dsts, const uint64_t* src, size_t elems, int count,
                    cudaStream_t s) {
  const size_t total = (size_t)count * (elems / 2);
  if (total == 0) return;
  LaunchScope scope_("scatter", s);
  k_scatter<<<grid_for(total, 256), 256, 0, s>>>(dsts, src, elems, total);
}

void launch_monomials(const CtxDev& c, uint64_t* mono, int levels,
                      uint64_t minus_one, cudaStream_t s) {
  const size_t total = (size_t)levels * c.n;
  if (total == 0) return;
  LaunchScope scope_("monomials", s);
  k_monomials<<<grid_for(total, 256), 256, 0, s>>>(mono, levels, c.log_n, minus_one);
}

void launch_absorb_sum(const CtxDev& c, uint64_t* out, const uint64_t* cts,
                       const uint64_t* db, int num_items, size_t item_stride,
                       int chunk, int count, cudaStream_t s) {
  const size_t total = (size_t)count * 2 * c.n;
  if (total == 0) return;
  LaunchScope scope_("absorb_sum", s);
  k_absorb_sum<<<grid_for(total, 256), 256, 0, s>>>(
      out, cts, db, num_items, item_stride, chunk, total, c.log_n, c);
}

// Integer ceiling of the transforms: the NTT's lazy Cooley-Tukey butterfly
// (bf_ct_lazy) on register-resident values with one fixed twiddle, ILP
// independent pairs per thread, no memory traffic.  The values wrap mod 2^64;
// only the instruction stream matters.
namespace {
template <int ILP>
__global__ void __launch_bounds__(256)
    k_butterfly_probe(uint64_t* sink, Tw w, uint64_t q, int iters) {
  const uint64_t two_q = 2 * q;
  uint64_t x[2 * ILP];
#pragma unroll
  for (int i = 0; i < 2 * ILP; ++i)
    x[i] = (uint64_t)(blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) bf_ct_lazy(x[2 * i], x[2 * i + 1], w, q, two_q);
  }
  uint64_t acc = 0;
#pragma unroll
  for (int i = 0; i < 2 * ILP; ++i) acc ^= x[i];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}
}  // namespace

int measure_butterfly_rate(double* per_second) {
  constexpr int kIlp = 8, kThreads = 256, kIters = 8192;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -1;
  const int blocks = sms * 8;
  uint64_t* sink = nullptr;
  if (cudaMalloc(&sink, (size_t)blocks * kThreads * 8) != cudaSuccess) return -1;
  // 45-bit prime of the ct-mult workload and an arbitrary twiddle below it.
  const uint64_t q = 35184371138561ull, wv = 1234567890123ull;
  const Tw w{wv, (uint64_t)(((unsigned __int128)wv << 64) / q)};
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_butterfly_probe<kIlp><<<blocks, kThreads>>>(sink, w, q, 64);
  cudaEventRecord(a);
  k_butterfly_probe<kIlp><<<blocks, kThreads>>>(sink, w, q, kIters);
  cudaEventRecord(b);
  g_launch_count += 2;
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess || ms <= 0) return -1;
  *per_second = (double)blocks * kThreads * kIlp * kIters / (ms * 1e-3);
  return 0;
}

unsigned take_debug_word_kernels() {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_shg_dbg, sizeof(v)) != cudaSuccess) return 0;
  if (v) cudaMemcpyToSymbol(g_shg_dbg, &z, sizeof(z));
  return v;
}

}  // namespace shg
