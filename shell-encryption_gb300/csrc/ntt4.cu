// Four-step NTT kernels (n = 2^12 .. 2^15) and the fused operations built on
// them.  Phase kernels take a source policy (how transform g's inputs are
// produced) and a sink policy (where its outputs go); see ntt4.cuh.
#include "ntt4.cuh"

#include <type_traits>

namespace shg {
namespace {

template <class K>
void set_smem4(K kernel, int smem) {
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

// Pulls the 128-byte line at p into L2 ahead of its use.
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <bool LAZY, int E>
__device__ __forceinline__ void finish_fwd(uint64_t (&x)[E], uint64_t q,
                                           uint64_t two_q, uint64_t bar) {
#pragma unroll
  for (int k = 0; k < E; ++k)
    x[k] = LAZY ? reduce_full(x[k], q, bar) : reduce_4q(x[k], q, two_q);
}

// ---------------------------------------------------------------------------
// Forward phase-1 sources: element `idx` of transform g (column loads).
// ---------------------------------------------------------------------------

template <int LOG_N>
struct FwdSrcPlain {
  const uint64_t* p;
  struct H {
    const uint64_t* base;
    __device__ __forceinline__ uint64_t operator()(int i) const { return base[i]; }
  };
  __device__ H bind(int g, int, const CtxDev&) const {
    return H{p + ((size_t)g << LOG_N)};
  }
};

// RnsGadget::Decompose's digit of the exported source limb, balanced-lifted
// to the output limb when needed (rns/rns_gadget.cc:108-153).
template <int LOG_N>
struct FwdSrcDigit {
  const uint64_t* X;
  const DigitDesc* digits;
  int k, L, need_lift;
  struct H {
    const uint64_t* base;
    int shift, lift;
    uint64_t mask, half_qi, q, bar, add;
    __device__ __forceinline__ uint64_t operator()(int i) const {
      uint64_t v = (base[i] >> shift) & mask;
      if (lift) {
        const bool neg = v > half_qi;
        v = reduce_2q(v - mulhi64(v, bar) * q, q);
        if (neg) v += add;
      }
      return v;
    }
  };
  __device__ H bind(int g, int j, const CtxDev& c) const {
    const int pd = g / L;
    const int di = pd % k, p = pd / k;
    DigitDesc dd = digits[di];
    dd.src_limb = dbg_index(dd.src_limb, L, kDbgDigit);
    H h;
    h.base = X + (((size_t)p * L + dd.src_limb) << LOG_N);
    h.shift = dd.shift;
    h.mask = dd.mask;
    h.lift = need_lift;
    h.half_qi = c.primes[dd.src_limb].half_q;
    h.q = c.primes[j].q;
    h.bar = c.primes[j].barrett;
    h.add = dd.src_limb != j ? h.q - c.qmod[dd.src_limb * c.L + j] : 0;
    return h;
  }
};

// ModReduceLsb: balanced lift of the top limb's plain coefficients to q_i
// (rns/rns_polynomial.cc:307-313).
template <int LOG_N>
struct FwdSrcModLift {
  const uint64_t* Y;
  int Lr;
  struct H {
    const uint64_t* base;
    uint64_t half_ql, q, bar, add;
    __device__ __forceinline__ uint64_t operator()(int i) const {
      uint64_t y = base[i];
      const bool neg = y > half_ql;
      y = reduce_2q(y - mulhi64(y, bar) * q, q);
      if (neg) y += add;
      return y;
    }
  };
  __device__ H bind(int g, int i, const CtxDev& c) const {
    H h;
    h.base = Y + ((size_t)(g / Lr) << LOG_N);
    h.half_ql = c.primes[Lr].half_q;
    h.q = c.primes[i].q;
    h.bar = c.primes[i].barrett;
    h.add = h.q - c.qmod[Lr * c.L + i];
    return h;
  }
};

// Encryption error (SampleError, rns/error_distribution.h:40-60): the signed
// centred-binomial coefficient of ciphertext g / L, lifted balanced to limb
// i and put in Montgomery form.
template <int LOG_N>
struct FwdSrcError {
  const int32_t* err;
  int L;
  struct H {
    const int32_t* base;
    uint64_t q, r, rp;
    __device__ __forceinline__ uint64_t operator()(int i) const {
      const int e = base[i];
      const uint64_t u = shoup((uint64_t)(e < 0 ? -e : e), r, rp, q);
      return (e < 0 && u) ? q - u : u;
    }
  };
  __device__ H bind(int g, int i, const CtxDev& c) const {
    return H{err + ((size_t)(g / L) << LOG_N), c.primes[i].q, c.primes[i].r_mod_q,
             c.primes[i].r_mod_q_shoup};
  }
};

// ---------------------------------------------------------------------------
// Forward phase-2 sinks: the values at i, i + 1 of transform g -- canonical,
// or below 62 q (lazy, small primes) for sinks with kTakesLazy.
// ---------------------------------------------------------------------------

template <int LOG_N>
struct FwdDstPlain {
  static constexpr bool kTakesLazy = false;  // writes canonical residues
  uint64_t* p;
  struct H {
    uint64_t* base;
    __device__ __forceinline__ void pair(int i, uint64_t x0, uint64_t x1) const {
      *reinterpret_cast<ulonglong2*>(base + i) = make_ulonglong2(x0, x1);
    }
  };
  __device__ H bind(int g, int, const CtxDev&) const { return H{p + ((size_t)g << LOG_N)}; }
  __device__ void prefetch(int, int, int) const {}
};

// ModReduceLsb combine: out_i = in_i * c1 + delta_i * c2
// (rns/rns_polynomial.cc:314-323).
template <int LOG_N>
struct FwdDstModCombine {
  // Shoup products take any 64-bit x, so lazily reduced values need no
  // final reduction first.
  static constexpr bool kTakesLazy = true;
  uint64_t* out;
  const uint64_t* in;
  int L;
  ScalarPack sc;
  struct H {
    uint64_t* o;
    const uint64_t* a;
    uint64_t q, c1, c1p, c2, c2p;
    __device__ __forceinline__ void pair(int i, uint64_t x0, uint64_t x1) const {
      const ulonglong2 av = *reinterpret_cast<const ulonglong2*>(a + i);
      ulonglong2 r;
      r.x = reduce_2q_full(shoup(av.x, c1, c1p, q) + shoup(x0, c2, c2p, q), q);
      r.y = reduce_2q_full(shoup(av.y, c1, c1p, q) + shoup(x1, c2, c2p, q), q);
      *reinterpret_cast<ulonglong2*>(o + i) = r;
    }
  };
  __device__ H bind(int g, int i, const CtxDev& c) const {
    const int Lr = L - 1;
    const int p = g / Lr;
    H h;
    h.o = out + ((size_t)g << LOG_N);
    h.a = in + (((size_t)p * L + i) << LOG_N);
    h.q = c.primes[i].q;
    h.c1 = sc.v[4 * i];
    h.c1p = sc.v[4 * i + 1];
    h.c2 = sc.v[4 * i + 2];
    h.c2p = sc.v[4 * i + 3];
    return h;
  }
  // The 16 values of limb i of `in` that the sink reads at i0.
  __device__ void prefetch(int g, int i, int i0) const {
    prefetch_l2(in + ((((size_t)(g / (L - 1)) * L + i) << LOG_N) + i0));
  }
};

// EncryptPolynomialBgv combine (rns/rns_secret_key.h:216-226): with x the
// NTT of the error, c0 = x * t + m + a * s where c1 already holds -a;
// out [count][2][L][n], m [count][L][n], key [L][n], tm.v[i] = t (Montgomery).
template <int LOG_N>
struct FwdDstBgvEnc {
  // REDC(x * t) needs x * t < q 2^64, true for lazily reduced x < 62 q (62 q < 2^64).
  static constexpr bool kTakesLazy = true;
  uint64_t* out;
  const uint64_t* m;
  const uint64_t* key;
  int L;
  ScalarPack tm;
  struct H {
    uint64_t* o;
    const uint64_t* mm;
    const uint64_t* s;
    uint64_t q, qinv, t;
    int c1_off;
    __device__ __forceinline__ void pair(int i, uint64_t x0, uint64_t x1) const {
      const ulonglong2 mv = *reinterpret_cast<const ulonglong2*>(mm + i);
      const ulonglong2 sv = *reinterpret_cast<const ulonglong2*>(s + i);
      const ulonglong2 c1 = *reinterpret_cast<const ulonglong2*>(o + c1_off + i);
      ulonglong2 r;
      r.x = add_mod(add_mod(mont_mul(x0, t, q, qinv), mv.x, q),
                    mont_mul(q - c1.x, sv.x, q, qinv), q);
      r.y = add_mod(add_mod(mont_mul(x1, t, q, qinv), mv.y, q),
                    mont_mul(q - c1.y, sv.y, q, qinv), q);
      *reinterpret_cast<ulonglong2*>(o + i) = r;
    }
  };
  __device__ H bind(int g, int i, const CtxDev& c) const {
    const int p = g / L;
    H h;
    h.o = out + (((size_t)p * 2 * L + i) << LOG_N);
    h.mm = m + ((size_t)g << LOG_N);
    h.s = key + ((size_t)i << LOG_N);
    h.q = c.primes[i].q;
    h.qinv = c.primes[i].inv_modulus;
    h.t = tm.v[i];
    h.c1_off = L << LOG_N;
    return h;
  }
  // Plaintext and c1 lines the sink reads at i0, fetched while the row
  // transform runs.
  __device__ void prefetch(int g, int i, int i0) const {
    prefetch_l2(m + ((size_t)g << LOG_N) + i0);
    prefetch_l2(out + ((((size_t)(g / L) * 2 + 1) * L + i) << LOG_N) + i0);
  }
};

// ---------------------------------------------------------------------------
// Inverse phase-1 sources: the values at i, i + 1 of transform g (rows).
// ---------------------------------------------------------------------------

template <int LOG_N>
struct InvSrcPlain {
  const uint64_t* p;
  int first, stride;  // source limb of transform g: first + g * stride
  struct H {
    const uint64_t* base;
    __device__ __forceinline__ ulonglong2 pair(int i) const {
      return *reinterpret_cast<const ulonglong2*>(base + i);
    }
  };
  __device__ H bind(int g, int, const CtxDev&) const {
    return H{p + (((size_t)first + (size_t)g * stride) << LOG_N)};
  }
};

// One component of ciphertext map(p), optionally read through the NTT-domain
// substitution X -> X^power (rns/rns_polynomial.cc:236-256).
template <int LOG_N>
struct InvSrcComponent {
  const uint64_t* ct;
  int ncomp, comp, power, L;
  CtMap map;
  struct H {
    const uint64_t* base;
    int power;
    __device__ __forceinline__ uint64_t at(int i) const {
      const unsigned j = __brev((unsigned)i) >> (32 - LOG_N);
      const unsigned t = ((unsigned)((power - 1) >> 1) + j * (unsigned)power) &
                         ((1u << LOG_N) - 1);
      return base[dbg_index(__brev(t) >> (32 - LOG_N), 1LL << LOG_N, kDbgSubst)];
    }
    __device__ __forceinline__ ulonglong2 pair(int i) const {
      if (power > 0) return make_ulonglong2(at(i), at(i + 1));
      return *reinterpret_cast<const ulonglong2*>(base + i);
    }
  };
  __device__ H bind(int g, int l, const CtxDev&) const {
    const int p = g / L;
    return H{ct + (((map(p) * ncomp + comp) * (size_t)L + l) << LOG_N), power};
  }
};

// RnsRlweCiphertext::Mul for degree-1 inputs (rns/rns_ciphertext.h:501-524):
// writes (c0, c1) of the product and yields its degree-2 component.
template <int LOG_N>
struct InvSrcTensor {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* out01;
  int L;
  struct H {
    const uint64_t *a0, *b0;
    uint64_t* o0;
    size_t Ln;
    uint64_t q, qinv;
    __device__ __forceinline__ ulonglong2 pair(int i) const {
      const ulonglong2 va0 = *reinterpret_cast<const ulonglong2*>(a0 + i);
      const ulonglong2 va1 = *reinterpret_cast<const ulonglong2*>(a0 + Ln + i);
      const ulonglong2 vb0 = *reinterpret_cast<const ulonglong2*>(b0 + i);
      const ulonglong2 vb1 = *reinterpret_cast<const ulonglong2*>(b0 + Ln + i);
      ulonglong2 r0, r1, r2;
      tensor3_pair(va0, va1, vb0, vb1, q, qinv, r0, r1, r2);
      *reinterpret_cast<ulonglong2*>(o0 + i) = r0;
      *reinterpret_cast<ulonglong2*>(o0 + Ln + i) = r1;
      return r2;
    }
  };
  __device__ H bind(int g, int l, const CtxDev& c) const {
    const int ct = g / L;
    H h;
    h.Ln = (size_t)L << LOG_N;
    const size_t off = (size_t)ct * 2 * h.Ln + ((size_t)l << LOG_N);
    h.a0 = a + off;
    h.b0 = b + off;
    h.o0 = out01 + off;
    h.q = c.primes[l].q;
    h.qinv = c.primes[l].inv_modulus;
    return h;
  }
};

// ---------------------------------------------------------------------------
// Inverse phase-2 sink: scaled value at idx of transform g (column stores).
// mode 0: x n^{-1}; 1: x n^{-1} 2^-64 (ExportInt folded); 2: x (sw, swp).
// ---------------------------------------------------------------------------

template <int LOG_N>
struct InvDstScale {
  uint64_t* p;
  int mode;
  uint64_t sw, swp;
  struct H {
    uint64_t* base;
    uint64_t w, wp, q;
    __device__ __forceinline__ void operator()(int i, uint64_t x) const {
      base[i] = shoup(x, w, wp, q);
    }
  };
  __device__ H bind(int g, int l, const CtxDev& c) const {
    const PrimeDev* P = c.primes + l;
    H h;
    h.base = p + ((size_t)g << LOG_N);
    h.q = P->q;
    h.w = mode == 0 ? P->n_inv : (mode == 1 ? P->n_inv_r : sw);
    h.wp = mode == 0 ? P->n_inv_shoup : (mode == 1 ? P->n_inv_r_shoup : swp);
    return h;
  }
};

// ---------------------------------------------------------------------------
// Phase kernels.
// ---------------------------------------------------------------------------

// Occupancy for at most 72 registers per thread (seven 128-thread CTAs at
// n = 2^14): left to itself the compiler spends up to 128 on some sources.
// SMALL_IN: every source value is below 2^32 (digits of at most 32 bits
// without the lift), so the first butterfly level takes the 32-bit-operand
// product.
template <int LOG_N, bool LAZY, class Src, bool SMALL_IN = false>
__global__ void __launch_bounds__(Ntt4<LOG_N>::COL_THREADS,
                                  65536 / (Ntt4<LOG_N>::COL_THREADS * 72))
    k4_fwd_cols(Src src, PrimeMap pm, uint64_t* buf, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::CC;
  extern __shared__ uint64_t smem[];
  const int g = blockIdx.x / S::COL_TILES, tile = blockIdx.x % S::COL_TILES;
  const int j = threadIdx.x % S::COLS, t = threadIdx.x / S::COLS;
  const int col = tile * S::COLS + j;
  const int l = dbg_index(pm(g), c.L, kDbgLimb);
  const uint64_t q = c.primes[l].q, two_q = c.primes[l].two_q;
  const auto h = src.bind(g, l, c);
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; ++k) x[k] = h((C::fwd_in_idx(t, k) << S::B) | col);
  C::template forward_m<LAZY, true, typename C::ColMap, SMALL_IN>(
      x, t, typename C::ColMap{smem, S::COLS, j}, c.tw_fwd + ((size_t)l << LOG_N), 1, q, two_q);
  uint64_t* dst = buf + ((size_t)g << LOG_N);
#pragma unroll
  for (int k = 0; k < C::E; ++k) dst[(C::fwd_out_idx(t, k) << S::B) | col] = x[k];
}

// Digit extraction and column phase of one gadget digit for every output
// limb: the CTA takes 16 columns of digit j of ciphertext p, extracts the
// digit once from the exported source limb (rns/rns_gadget.cc:108-153) and
// runs the column phase of its transform modulo each prime in turn (the
// digit is the same integer for every limb; the balanced lift, when the
// gadget needs it, is applied per limb).  D [count][k][L][n] as
// k4_fwd_cols<FwdSrcDigit> writes it.  DT = uint32_t is the form for digits
// of at most 32 bits without the lift (need_lift is ignored there).
template <int LOG_N, bool LAZY, class DT>
__global__ void __launch_bounds__(Ntt4<LOG_N>::COL_THREADS,
                                  (sizeof(DT) == 4 ? 6 : 5) * 128 / Ntt4<LOG_N>::COL_THREADS)
    k4_digit_cols_all(const uint64_t* X, const DigitDesc* digits, int k, int L, int need_lift,
                      uint64_t* D, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::CC;
  extern __shared__ uint64_t smem[];
  const int pj = blockIdx.x / S::COL_TILES, tile = blockIdx.x % S::COL_TILES;
  const int j = pj % k;
  const size_t p = (size_t)(pj / k);
  const int jc = threadIdx.x % S::COLS, t = threadIdx.x / S::COLS;
  const int col = tile * S::COLS + jc;
  DigitDesc dd = digits[j];
  dd.src_limb = dbg_index(dd.src_limb, L, kDbgDigit);
  const uint64_t* src = X + ((p * L + dd.src_limb) << LOG_N);
  // DT = uint32_t holds digits of at most 32 bits in half the registers.
  DT dv[C::E];
#pragma unroll
  for (int e = 0; e < C::E; ++e)
    dv[e] = (DT)((src[(C::fwd_in_idx(t, e) << S::B) | col] >> dd.shift) & dd.mask);
  const uint64_t half_qi = c.primes[dd.src_limb].half_q;
#pragma unroll 1
  for (int l = 0; l < L; ++l) {
    const PrimeDev* P = c.primes + l;
    const uint64_t q = P->q, two_q = P->two_q;
    uint64_t x[C::E];
    if (sizeof(DT) == 4 || !need_lift) {
#pragma unroll
      for (int e = 0; e < C::E; ++e) x[e] = dv[e];
    } else {
      const uint64_t bar = P->barrett;
      const uint64_t add = dd.src_limb != l ? q - c.qmod[dd.src_limb * c.L + l] : 0;
#pragma unroll
      for (int e = 0; e < C::E; ++e) {
        uint64_t v = dv[e];
        const bool neg = v > half_qi;
        v = reduce_2q(v - mulhi64(v, bar) * q, q);
        x[e] = neg ? v + add : v;
      }
    }
    // 32-bit digits without the lift (the only launch of the 32-bit form)
    // enter the first level below 2^32.
    C::template forward_m<LAZY, true, typename C::ColMap, sizeof(DT) == 4>(
        x, t, typename C::ColMap{smem, S::COLS, jc}, c.tw_fwd + ((size_t)l << LOG_N), 1, q,
        two_q);
    uint64_t* dst = D + (((p * k + j) * L + l) << LOG_N);
#pragma unroll
    for (int e = 0; e < C::E; ++e) dst[(C::fwd_out_idx(t, e) << S::B) | col] = x[e];
  }
}

// The CTA takes row `row` of ROWS transforms that share a prime (transform g
// has limb g mod pm.L for every forward use), so the sub-rows read the same
// twiddles and the loads hit in L1.
template <int LOG_N, bool LAZY, class Dst>
__global__ void __launch_bounds__(Ntt4<LOG_N>::ROW_THREADS)
    k4_fwd_rows(const uint64_t* buf, Dst dst, PrimeMap pm, int num, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::RC;
  extern __shared__ uint64_t smem[];
  const int rows = 1 << S::A;
  const int per_class = num / pm.L;
  const int groups = (per_class + S::ROWS - 1) / S::ROWS;
  const int row = blockIdx.x % rows;
  const int cg = blockIdx.x / rows;
  const int l = dbg_index(cg / groups, c.L, kDbgLimb), grp = cg % groups;
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  const int m = grp * S::ROWS + sub;
  const bool active = m < per_class;
  const int g = l + pm.L * (active ? m : per_class - 1);
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t* src = buf + ((size_t)g << LOG_N) + ((size_t)row << S::B);
  if (active) dst.prefetch(g, l, (row << S::B) | C::fwd_out_idx(tid, 0));
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; ++k) x[k] = src[C::fwd_in_idx(tid, k)];
  C::template forward_m<LAZY>(x, tid, RowMap<S::B>{smem, sub},
                              c.tw_fwd + ((size_t)l << LOG_N), (1 << S::A) + row, q,
                              two_q);
  if constexpr (!(LAZY && Dst::kTakesLazy)) finish_fwd<LAZY>(x, q, two_q, P->barrett);
  // Thread tid holds elements 16 tid .. 16 tid + 15 of its sub-row.  They
  // go through shared memory (pair slots XOR-swizzled by tid, so neither
  // side has bank conflicts) and each warp then hands whole sub-rows to the
  // sink, 32 consecutive pairs per access.
  static_assert(C::T == 8 && (1 << S::B) == 128 && C::fwd_clo(C::P - 1) == 0,
                "row epilogue assumes 8 threads x 16 consecutive values per row");
  __syncthreads();
  ulonglong2* t2 = reinterpret_cast<ulonglong2*>(smem);
#pragma unroll
  for (int p = 0; p < 8; ++p)
    t2[sub * 64 + tid * 8 + ((p ^ tid) & 7)] = make_ulonglong2(x[2 * p], x[2 * p + 1]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int s2 = warp; s2 < S::ROWS; s2 += S::ROW_THREADS / 32) {
    const int m2 = grp * S::ROWS + s2;
    if (m2 >= per_class) break;
    const auto h = dst.bind(l + pm.L * m2, l, c);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int pp = half * 32 + lane, tq = pp >> 3;
      const ulonglong2 v = t2[s2 * 64 + tq * 8 + ((pp ^ tq) & 7)];
      h.pair((row << S::B) + 2 * pp, v.x, v.y);
    }
  }
}

// Forward row phase of all k gadget digits of (ciphertext p, limb l), fused
// with the key inner product and base add of the key switch
// (rns_relinearization_key.cc:219-226, rns_galois_key.cc:265-283,
// relinearization_key.cc:76-96).  The CTA runs rows tile*R .. tile*R+R-1 of
// the k digit transforms (sub-row r*k + j: row r, digit j; they share the
// prime and the row, so they read the same twiddles), parks the NTT values in
// shared memory (canonical, or lazily reduced below 62 q when LAZY), and then
// each thread produces output slots:
//   out0 = base0 + REDC(sum_j D_j * kb_j), out1 = base1 + REDC(sum_j D_j * ka_j)
// with 128-bit lazy accumulation, one REDC per `chunk` digits.  The digit
// transforms never go back to memory.  Arguments as in launch_ks_inner.
// 72 registers let three 288-thread CTAs (k = 18 digits, 2 rows) share an
// SM; 96 allowed only two.
constexpr int kKsRowsMaxThreads = 512;

template <int LOG_N, bool LAZY>
__global__ void __maxnreg__(72)
    k4_ks_rows(const uint64_t* buf, int k, int R, int chunk, const uint64_t* kb,
               const uint64_t* ka, uint64_t* out, const uint64_t* base,
               size_t base_ct_elems, CtMap map, int base1_zero, int subst_power,
               int L, KeyTable kt, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::RC;
  extern __shared__ uint64_t smem[];
  const int tiles = (1 << S::A) / R;
  const int tile = blockIdx.x % tiles;
  const int pl = blockIdx.x / tiles;
  const int l = dbg_index(pl % L, c.L, kDbgLimb);
  const size_t p = (size_t)(pl / L);
  if (kt.kb) {
    const size_t e = dbg_index(p >> kt.shift, kt.entries ? kt.entries : (1LL << 62), kDbgKeyTable);
    kb = kt.kb[e];
    ka = kt.ka[e];
  }
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  const int r = sub / k, j = sub % k;
  const int row = tile * R + r;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t* src =
      buf + (((p * k + j) * L + l) << LOG_N) + ((size_t)row << S::B);
  uint64_t x[C::E];
#pragma unroll
  for (int e = 0; e < C::E; ++e) x[e] = src[C::fwd_in_idx(tid, e)];
  // the split Shoup product: the fused one spills at this register cap
  C::template forward_m<LAZY, false>(x, tid, RowMap<S::B>{smem, sub},
                                     c.tw_fwd + ((size_t)l << LOG_N), (1 << S::A) + row, q,
                                     two_q);
  // LAZY (every prime below 2^58): the digit values stay below 62 q, which
  // the inner product's 128-bit sums and REDC take as they are (chunk_lazy
  // digits per REDC); otherwise reduce to canonical first.
  if constexpr (!LAZY) finish_fwd<LAZY>(x, q, two_q, P->barrett);
  __syncthreads();  // every sub-row is done with its exchange tile
  {
    const RowMap<S::B> park{smem, sub};
    const int i0 = C::fwd_out_idx(tid, 0);
#pragma unroll
    for (int e = 0; e < C::E; ++e) park(i0 + e) = x[e];
  }
  __syncthreads();
  const size_t n = (size_t)1 << LOG_N, Ln = (size_t)L * n;
  const uint64_t qinv = P->inv_modulus;
  for (int o = threadIdx.x; o < (R << S::B); o += blockDim.x) {
    const int rr = o >> S::B, e = o & ((1 << S::B) - 1);
    const int pos = ((tile * R + rr) << S::B) | e;
    const size_t kr = (size_t)l * n + pos;
    // Digit jj of this slot sits in sub-row rr*k + jj at RowMap's swizzled
    // column: the 16-element swizzle of e, flipped on bit 3 for odd rows.
    const uint64_t* drow = smem + ((size_t)(rr * k) << S::B);
    const int col_even = (e ^ ((e >> 4) & 15)) ^ (((rr * k) & 1) << 3);
    const uint64_t* pb = kb + kr;
    const uint64_t* pa = ka + kr;
    uint64_t s0 = 0, s1 = 0;
    for (int j0 = 0; j0 < k; j0 += chunk) {
      const int j1 = min(k, j0 + chunk);
      uint64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
#pragma unroll 6
      for (int jj = j0; jj < j1; ++jj) {
        const uint64_t d = drow[(jj << S::B) + (col_even ^ ((jj & 1) << 3))];
        mac128(lo0, hi0, d, __ldg(pb));
        mac128(lo1, hi1, d, __ldg(pa));
        pb += Ln;
        pa += Ln;
      }
      s0 = add_mod(s0, redc128(lo0, hi0, q, qinv), q);
      s1 = add_mod(s1, redc128(lo1, hi1, q, qinv), q);
    }
    const uint64_t* bp = base + map(p) * base_ct_elems + (size_t)l * n;
    int pos0 = pos;
    if (subst_power > 0) {
      const unsigned jb = __brev((unsigned)pos) >> (32 - LOG_N);
      const unsigned t = ((unsigned)((subst_power - 1) >> 1) + jb * (unsigned)subst_power) &
                         ((1u << LOG_N) - 1);
      pos0 = dbg_index((int)(__brev(t) >> (32 - LOG_N)), 1LL << LOG_N, kDbgSubst);
    }
    const uint64_t b0 = bp[pos0];
    const uint64_t b1 = base1_zero ? 0 : bp[Ln + pos];
    out[p * 2 * Ln + kr] = add_mod(b0, s0, q);
    out[p * 2 * Ln + Ln + kr] = add_mod(b1, s1, q);
  }
}

// Sub-row tile of the 8-value row core: NttCore<7, 3>'s own swizzle (index
// bits 3..6 XORed into bits 0..3) on each 128-element sub-row; a half-warp
// is one sub-row, so every exchange and the parked reads are conflict-free.
template <int B>
struct RowMap8 {
  uint64_t* sm;
  int sub;
  __device__ __forceinline__ uint64_t& operator()(int i) const {
    return sm[(sub << B) + (i ^ ((i >> 3) & 15))];
  }
};

// k4_ks_rows with 8 values per thread (16 threads per 128-element row, one
// row of all k digits per CTA).  Half the register array of the 16-value
// core: 56 registers, so four 288-thread CTAs (k = 18) share an SM, and the
// butterflies keep the fused PTX Shoup products (three-term quotient when
// LAZY) without spilling.  The inner product takes one key
// component of one coefficient per thread.  Requires k * 16 threads to be
// whole warps (k even) and at most kKsRowsMaxThreads.
template <int LOG_N, bool LAZY>
__global__ void __maxnreg__(56)
    k4_ks_rows8(const uint64_t* buf, int k, int chunk, const uint64_t* kb,
                const uint64_t* ka, uint64_t* out, const uint64_t* base,
                size_t base_ct_elems, CtMap map, int base1_zero, int subst_power,
                int L, KeyTable kt, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = NttCore<S::B, 3>;
  extern __shared__ uint64_t smem[];
  constexpr int rows = 1 << S::A;
  const int row = blockIdx.x % rows;
  const int pl = blockIdx.x / rows;
  const int l = dbg_index(pl % L, c.L, kDbgLimb);
  const size_t p = (size_t)(pl / L);
  if (kt.kb) {
    const size_t e = dbg_index(p >> kt.shift, kt.entries ? kt.entries : (1LL << 62), kDbgKeyTable);
    kb = kt.kb[e];
    ka = kt.ka[e];
  }
  const int j = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const uint64_t* src =
      buf + (((p * k + j) * L + l) << LOG_N) + ((size_t)row << S::B);
  uint64_t x[C::E];
#pragma unroll
  for (int e = 0; e < C::E; ++e) x[e] = src[C::fwd_in_idx(tid, e)];
  C::template forward_m<LAZY>(x, tid, RowMap8<S::B>{smem, j},
                              c.tw_fwd + ((size_t)l << LOG_N), (1 << S::A) + row, q, two_q);
  // LAZY: the digit values stay below 62 q for the inner product (chunk_lazy)
  if constexpr (!LAZY) finish_fwd<LAZY>(x, q, two_q, P->barrett);
  {
    const RowMap8<S::B> park{smem, j};
    const int i0 = C::fwd_out_idx(tid, 0);
#pragma unroll
    for (int e = 0; e < C::E; ++e) park(i0 + e) = x[e];
  }
  __syncthreads();
  const size_t n = (size_t)1 << LOG_N, Ln = (size_t)L * n;
  const uint64_t qinv = P->inv_modulus;
  for (int o = threadIdx.x; o < (2 << S::B); o += blockDim.x) {
    const int comp = o >> S::B, e = o & ((1 << S::B) - 1);
    const int pos = (row << S::B) | e;
    const size_t kr = (size_t)l * n + pos;
    const uint64_t* d = smem + (e ^ ((e >> 3) & 15));
    const uint64_t* pk = (comp ? ka : kb) + kr;
    uint64_t acc = 0;
    for (int j0 = 0; j0 < k; j0 += chunk) {
      const int j1 = min(k, j0 + chunk);
      uint64_t lo = 0, hi = 0;
#pragma unroll 6
      for (int jj = j0; jj < j1; ++jj) {
        mac128(lo, hi, d[jj << S::B], __ldg(pk));
        pk += Ln;
      }
      acc = add_mod(acc, redc128(lo, hi, q, qinv), q);
    }
    const uint64_t* bp = base + map(p) * base_ct_elems + (size_t)l * n;
    uint64_t b;
    if (comp == 0) {
      int pos0 = pos;
      if (subst_power > 0) {
        const unsigned jb = __brev((unsigned)pos) >> (32 - LOG_N);
        const unsigned t = ((unsigned)((subst_power - 1) >> 1) + jb * (unsigned)subst_power) &
                           ((1u << LOG_N) - 1);
        pos0 = dbg_index((int)(__brev(t) >> (32 - LOG_N)), 1LL << LOG_N, kDbgSubst);
      }
      b = bp[pos0];
    } else {
      b = base1_zero ? 0 : bp[Ln + pos];
    }
    out[p * 2 * Ln + comp * Ln + kr] = add_mod(b, acc, q);
  }
}

// Rows (warps) per CTA of k4_ks_rows_warp, and digits each warp transforms
// together (1, 2, 3, 4, 6 digits: 57.2, 60.8, 62.3, 62.6, 62.2 k ct-mult+relin/s;
// with the 32-bit first digit level, 3 and 4 digits: 64.23 and 64.52 k/s).
constexpr int kKsWarpRows = 4;
constexpr int kKsWarpDigits = 4;

// The key switch's row phase with one warp per row of one (ciphertext,
// limb): its 32 threads run that row of every digit transform (4 values per
// thread, NttCore<7, 2>: four passes, exchanges in the warp's own swizzled
// shared tiles with warp-level synchronisation only), DPI digits at a time,
// and keep the key inner product of their 4 consecutive output slots in
// registers (two components, 128-bit sums).  The digit values are never
// parked, no CTA-wide barrier is taken, each digit's key values are loaded
// before its transform, and key rows and the base are read 16 bytes at a
// time.  For a chunk covering every digit (chunk >= k), as lazily reduced
// digits of primes below 2^58 give at up to a few dozen digits.  W rows
// (warps) per CTA, at least MB CTAs per SM.  Against k4_ks_rows8 (one row of
// all digits per CTA, values parked in shared memory, CTA barriers) it shares
// the SMs far better with the next chunk's column kernel on the other
// key-switch stream (ct-mult+relin 53.4 k -> 56.1 k/s one digit at a time,
// 62.3 k/s three at a time).
// NARROW (every prime below 2^45): the inner product's multiply-accumulates
// drop the zero high word of the high partial product (mac128_narrow).
template <int LOG_N, bool LAZY, int W, int MB, int DPI, bool NARROW = false>
__global__ void __launch_bounds__(32 * W, MB)
    k4_ks_rows_warp(const uint64_t* buf, int k, const uint64_t* kb, const uint64_t* ka,
                    uint64_t* out, const uint64_t* base, size_t base_ct_elems, CtMap map,
                    int base1_zero, int subst_power, int L, KeyTable kt, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = NttCore<S::B, 2>;
  static_assert(C::T == 32 && C::E == 4 && C::P == 4, "32 threads x 4 values per row");
  extern __shared__ uint64_t smem[];
  constexpr int tiles = (1 << S::A) / W;
  const int tile = blockIdx.x % tiles;
  const int pl = blockIdx.x / tiles;
  const int l = dbg_index(pl % L, c.L, kDbgLimb);
  const size_t p = (size_t)(pl / L);
  if (kt.kb) {
    const size_t e = dbg_index(p >> kt.shift, kt.entries ? kt.entries : (1LL << 62), kDbgKeyTable);
    kb = kt.kb[e];
    ka = kt.ka[e];
  }
  const int warp = threadIdx.x >> 5, tid = threadIdx.x & 31;
  const int row = tile * W + warp;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const size_t n = (size_t)1 << LOG_N, Ln = (size_t)L * n;
  const Tw* tw0 = c.tw_fwd + ((size_t)l << LOG_N);
  const int tm = (1 << S::A) + row;
  const typename C::SwzMap m{smem + ((size_t)warp * DPI << S::B)};
  // this thread's output slots after the last pass: 4 consecutive positions
  const int pos0 = (row << S::B) | C::fwd_out_idx(tid, 0);
  const size_t kr0 = (size_t)l * n + pos0;
  const uint64_t* src = buf + (((p * k) * L + l) << LOG_N) + ((size_t)row << S::B);
  uint64_t lo0[4], hi0[4], lo1[4], hi1[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) lo0[e] = hi0[e] = lo1[e] = hi1[e] = 0;
  // DPI digits at a time, interleaved: their transforms use the same
  // twiddles and tile offsets (tile d at d KB above the first), so the index
  // work is shared and each level has DPI times the independent butterflies;
  // of the last k mod DPI digits, two go together and the rest one by one.
  auto digits = [&](int j, auto dn) {
    constexpr int D = decltype(dn)::value;
    const Tw* tw;
    asm volatile("mov.b64 %0, %1;" : "=l"(tw) : "l"(tw0));
    uint64_t x[D][4];
    ulonglong2 kv[D][4];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const uint64_t* sd = src + (size_t)(j + d) * Ln;
#pragma unroll
      for (int e = 0; e < 4; ++e) x[d][e] = sd[C::fwd_in_idx(tid, e)];
      const ulonglong2* b2 = reinterpret_cast<const ulonglong2*>(kb + kr0 + (size_t)(j + d) * Ln);
      const ulonglong2* a2 = reinterpret_cast<const ulonglong2*>(ka + kr0 + (size_t)(j + d) * Ln);
      kv[d][0] = __ldg(b2);
      kv[d][1] = __ldg(b2 + 1);
      kv[d][2] = __ldg(a2);
      kv[d][3] = __ldg(a2 + 1);
    }
    static_for<0, C::P>([&](auto pp) {
      constexpr int ps = decltype(pp)::value;
#pragma unroll
      for (int d = 0; d < D; ++d) C::template fwd_pass<ps, LAZY>(x[d], tid, tw, tm, q, two_q);
      if constexpr (ps + 1 < C::P) {
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int e = 0; e < 4; ++e) (&m(C::idx(tid, e, C::fwd_clo(ps))))[d << S::B] = x[d][e];
        __syncwarp();
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int e = 0; e < 4; ++e) x[d][e] = (&m(C::idx(tid, e, C::fwd_clo(ps + 1))))[d << S::B];
        __syncwarp();  // every read is done before the tile is rewritten
      }
    });
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if constexpr (!LAZY) finish_fwd<LAZY>(x[d], q, two_q, P->barrett);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const ulonglong2 vb = kv[d][h], va = kv[d][2 + h];
        auto mac = [](uint64_t& lo, uint64_t& hi, uint64_t a, uint64_t b) {
          if constexpr (NARROW && LAZY) {
            mac128_narrow(lo, hi, a, b);
          } else {
            mac128(lo, hi, a, b);
          }
        };
        mac(lo0[2 * h], hi0[2 * h], x[d][2 * h], vb.x);
        mac(lo0[2 * h + 1], hi0[2 * h + 1], x[d][2 * h + 1], vb.y);
        mac(lo1[2 * h], hi1[2 * h], x[d][2 * h], va.x);
        mac(lo1[2 * h + 1], hi1[2 * h + 1], x[d][2 * h + 1], va.y);
      }
    }
  };
  int j = 0;
  if constexpr (DPI > 1) {
#pragma unroll 1
    for (; j + DPI <= k; j += DPI) digits(j, std::integral_constant<int, DPI>{});
  }
  if constexpr (DPI > 2) {
    if (j + 2 <= k) {
      digits(j, std::integral_constant<int, 2>{});
      j += 2;
    }
  }
#pragma unroll 1
  for (; j < k; ++j) digits(j, std::integral_constant<int, 1>{});
  const uint64_t qinv = P->inv_modulus;
  const uint64_t* bp = base + map(p) * base_ct_elems + (size_t)l * n;
  uint64_t* o0 = out + p * 2 * Ln + kr0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    uint64_t b0[2], b1[2];
    if (subst_power > 0) {
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int pos = pos0 + 2 * h + t;
        const unsigned jb = __brev((unsigned)pos) >> (32 - LOG_N);
        const unsigned tt = ((unsigned)((subst_power - 1) >> 1) + jb * (unsigned)subst_power) &
                            ((1u << LOG_N) - 1);
        b0[t] = bp[dbg_index(__brev(tt) >> (32 - LOG_N), 1LL << LOG_N, kDbgSubst)];
      }
    } else {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(bp + pos0 + 2 * h);
      b0[0] = v.x;
      b0[1] = v.y;
    }
    if (base1_zero) {
      b1[0] = b1[1] = 0;
    } else {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(bp + Ln + pos0 + 2 * h);
      b1[0] = v.x;
      b1[1] = v.y;
    }
    ulonglong2 r0, r1;
    r0.x = add_mod(b0[0], redc128(lo0[2 * h], hi0[2 * h], q, qinv), q);
    r0.y = add_mod(b0[1], redc128(lo0[2 * h + 1], hi0[2 * h + 1], q, qinv), q);
    r1.x = add_mod(b1[0], redc128(lo1[2 * h], hi1[2 * h], q, qinv), q);
    r1.y = add_mod(b1[1], redc128(lo1[2 * h + 1], hi1[2 * h + 1], q, qinv), q);
    *reinterpret_cast<ulonglong2*>(o0 + 2 * h) = r0;
    *reinterpret_cast<ulonglong2*>(o0 + Ln + 2 * h) = r1;
  }
}

// Row phases with one warp per row of DPI transforms that share a prime
// (same twiddles; 4 values per thread per transform, NttCore<7, 2>, four
// passes exchanged through the warp's own swizzled tiles with warp-level
// synchronisation only).  A thread's 4 values are consecutive at the
// forward phase's end and the inverse phase's start, so the sink and source
// move 16-byte pairs and every warp access covers whole rows.  Work item w =
// blockIdx.x * W + warp: row w mod 2^A of the group of DPI transforms
// (w / 2^A) -- prime class first, as in k4_fwd_rows.
template <int LOG_N, bool LAZY, class Dst, int W, int DPI>
__global__ void __launch_bounds__(32 * W)
    k4_fwd_rows_warp(const uint64_t* buf, Dst dst, PrimeMap pm, int num, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = NttCore<S::B, 2>;
  static_assert(C::T == 32 && C::E == 4 && C::P == 4, "32 threads x 4 values per row");
  static_assert((1 << S::A) % W == 0, "whole CTAs of rows");
  extern __shared__ uint64_t smem[];
  constexpr int rows = 1 << S::A;
  const int warp = threadIdx.x >> 5, tid = threadIdx.x & 31;
  const int w = blockIdx.x * W + warp;
  const int per_class = num / pm.L;
  const int groups = (per_class + DPI - 1) / DPI;
  const int row = w % rows;
  const int cg = w / rows;
  const int l = dbg_index(cg / groups, c.L, kDbgLimb), grp = cg % groups;
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const Tw* tw = c.tw_fwd + ((size_t)l << LOG_N);
  const int tm = (1 << S::A) + row;
  const typename C::SwzMap m{smem + ((size_t)warp * DPI << S::B)};
  const int pos0 = (row << S::B) | C::fwd_out_idx(tid, 0);
  uint64_t x[DPI][4];
  int g[DPI];
#pragma unroll
  for (int d = 0; d < DPI; ++d) {
    const int mm = min(grp * DPI + d, per_class - 1);
    g[d] = l + pm.L * mm;
    if (grp * DPI + d < per_class) dst.prefetch(g[d], l, pos0);
    const uint64_t* src = buf + ((size_t)g[d] << LOG_N) + ((size_t)row << S::B);
#pragma unroll
    for (int e = 0; e < 4; ++e) x[d][e] = src[C::fwd_in_idx(tid, e)];
  }
  static_for<0, C::P>([&](auto pp) {
    constexpr int ps = decltype(pp)::value;
#pragma unroll
    for (int d = 0; d < DPI; ++d) C::template fwd_pass<ps, LAZY>(x[d], tid, tw, tm, q, two_q);
    if constexpr (ps + 1 < C::P) {
#pragma unroll
      for (int d = 0; d < DPI; ++d)
#pragma unroll
        for (int e = 0; e < 4; ++e) (&m(C::idx(tid, e, C::fwd_clo(ps))))[d << S::B] = x[d][e];
      __syncwarp();
#pragma unroll
      for (int d = 0; d < DPI; ++d)
#pragma unroll
        for (int e = 0; e < 4; ++e) x[d][e] = (&m(C::idx(tid, e, C::fwd_clo(ps + 1))))[d << S::B];
      __syncwarp();
    }
  });
#pragma unroll
  for (int d = 0; d < DPI; ++d) {
    if constexpr (!(LAZY && Dst::kTakesLazy)) finish_fwd<LAZY>(x[d], q, two_q, P->barrett);
    if (grp * DPI + d < per_class) {
      const auto h = dst.bind(g[d], l, c);
      h.pair(pos0, x[d][0], x[d][1]);
      h.pair(pos0 + 2, x[d][2], x[d][3]);
    }
  }
}

template <int LOG_N, bool WIDE, class Src, int W, int DPI>
__global__ void __launch_bounds__(32 * W)
    k4_inv_rows_warp(Src src, PrimeMap pm, uint64_t* buf, int num, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = NttCore<S::B, 2>;
  static_assert(C::T == 32 && C::E == 4 && C::P == 4, "32 threads x 4 values per row");
  static_assert((1 << S::A) % W == 0, "whole CTAs of rows");
  extern __shared__ uint64_t smem[];
  constexpr int rows = 1 << S::A;
  const int warp = threadIdx.x >> 5, tid = threadIdx.x & 31;
  const int w = blockIdx.x * W + warp;
  // transforms g = cls + L m share limb pm(cls) for any PrimeMap (num is a
  // multiple of L); the warp takes DPI of one class
  const int per_class = num / pm.L;
  const int groups = (per_class + DPI - 1) / DPI;
  const int row = w % rows;
  const int cg = w / rows;
  const int cls = cg / groups, grp = cg % groups;
  const int l = dbg_index(pm(cls), c.L, kDbgLimb);
  const PrimeDev* P = c.primes + l;
  const uint64_t q = P->q, two_q = P->two_q;
  const Tw* tw = c.tw_inv + ((size_t)l << LOG_N);
  const typename C::SwzMap m{smem + ((size_t)warp * DPI << S::B)};
  const int pos0 = (row << S::B) | C::inv_in_idx(tid, 0);
  uint64_t x[DPI][4];
  int g[DPI];
#pragma unroll
  for (int d = 0; d < DPI; ++d) {
    g[d] = cls + pm.L * min(grp * DPI + d, per_class - 1);
    const auto h = src.bind(g[d], l, c);
    const ulonglong2 v0 = h.pair(pos0), v1 = h.pair(pos0 + 2);
    x[d][0] = v0.x;
    x[d][1] = v0.y;
    x[d][2] = v1.x;
    x[d][3] = v1.y;
  }
  static_for<0, C::P>([&](auto pp) {
    constexpr int ps = decltype(pp)::value;
#pragma unroll
    for (int d = 0; d < DPI; ++d)
      C::template inv_pass<ps, WIDE>(x[d], tid, tw, S::N, 0, row, q, two_q);
    if constexpr (ps + 1 < C::P) {
#pragma unroll
      for (int d = 0; d < DPI; ++d)
#pragma unroll
        for (int e = 0; e < 4; ++e) (&m(C::idx(tid, e, C::inv_clo(ps))))[d << S::B] = x[d][e];
      __syncwarp();
#pragma unroll
      for (int d = 0; d < DPI; ++d)
#pragma unroll
        for (int e = 0; e < 4; ++e) x[d][e] = (&m(C::idx(tid, e, C::inv_clo(ps + 1))))[d << S::B];
      __syncwarp();
    }
  });
#pragma unroll
  for (int d = 0; d < DPI; ++d) {
    if (grp * DPI + d >= per_class) continue;
    uint64_t* dstp = buf + ((size_t)g[d] << LOG_N) + ((size_t)row << S::B);
#pragma unroll
    for (int e = 0; e < 4; ++e) dstp[C::inv_out_idx(tid, e)] = x[d][e];
  }
}

template <int LOG_N, bool WIDE, class Src>
__global__ void __launch_bounds__(Ntt4<LOG_N>::ROW_THREADS)
    k4_inv_rows(Src src, PrimeMap pm, uint64_t* buf, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::RC;
  extern __shared__ uint64_t smem[];
  const int g = blockIdx.x / S::ROW_TILES, tile = blockIdx.x % S::ROW_TILES;
  const int sub = threadIdx.x / C::T, tid = threadIdx.x % C::T;
  const int row = tile * S::ROWS + sub;
  const int l = dbg_index(pm(g), c.L, kDbgLimb);
  const uint64_t q = c.primes[l].q, two_q = c.primes[l].two_q;
  // Whole sub-rows come in warp by warp, 32 consecutive pairs per access,
  // through shared memory (pair slots XOR-swizzled, as in k4_fwd_rows'
  // epilogue); thread tid then takes elements 16 tid .. 16 tid + 15.
  static_assert(C::T == 8 && (1 << S::B) == 128 && C::inv_clo(0) == 0,
                "row prologue assumes 8 threads x 16 consecutive values per row");
  ulonglong2* t2 = reinterpret_cast<ulonglong2*>(smem);
  {
    const auto h = src.bind(g, l, c);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int s2 = warp; s2 < S::ROWS; s2 += S::ROW_THREADS / 32) {
      const int row2 = tile * S::ROWS + s2;
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int pp = half * 32 + lane, tq = pp >> 3;
        t2[s2 * 64 + tq * 8 + ((pp ^ tq) & 7)] = h.pair((row2 << S::B) + 2 * pp);
      }
    }
  }
  __syncthreads();
  uint64_t x[C::E];
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const ulonglong2 v = t2[sub * 64 + tid * 8 + ((p ^ tid) & 7)];
    x[2 * p] = v.x;
    x[2 * p + 1] = v.y;
  }
  __syncthreads();  // the tile is the transform's exchange space next
  C::template inverse_m<WIDE>(x, tid, RowMap<S::B>{smem, sub}, c.tw_inv + ((size_t)l << LOG_N),
               S::N, 0, row, q, two_q);
  uint64_t* dst = buf + ((size_t)g << LOG_N) + ((size_t)row << S::B);
#pragma unroll
  for (int k = 0; k < C::E; ++k) dst[C::inv_out_idx(tid, k)] = x[k];
}

template <int LOG_N, bool WIDE, class Dst>
__global__ void __launch_bounds__(Ntt4<LOG_N>::COL_THREADS)
    k4_inv_cols(const uint64_t* buf, Dst dst, PrimeMap pm, CtxDev c) {
  using S = Ntt4<LOG_N>;
  using C = typename S::CC;
  extern __shared__ uint64_t smem[];
  const int g = blockIdx.x / S::COL_TILES, tile = blockIdx.x % S::COL_TILES;
  const int j = threadIdx.x % S::COLS, t = threadIdx.x / S::COLS;
  const int col = tile * S::COLS + j;
  const int l = dbg_index(pm(g), c.L, kDbgLimb);
  const uint64_t q = c.primes[l].q, two_q = c.primes[l].two_q;
  const uint64_t* src = buf + ((size_t)g << LOG_N);
  uint64_t x[C::E];
#pragma unroll
  for (int k = 0; k < C::E; ++k) x[k] = src[(C::inv_in_idx(t, k) << S::B) | col];
  C::template inverse_m<WIDE>(x, t, typename C::ColMap{smem, S::COLS, j},
               c.tw_inv + ((size_t)l << LOG_N), S::N, S::B, 0, q, two_q);
  const auto h = dst.bind(g, l, c);
#pragma unroll
  for (int k = 0; k < C::E; ++k) h((C::inv_out_idx(t, k) << S::B) | col, x[k]);
}

// Forward row phase grid: (prime class, group of ROWS transforms, row).
// Every forward caller passes PrimeMap{0, 1, L} with num a multiple of L.
template <int LOG_N>
int row_blocks(int num, PrimeMap pm) {
  using S = Ntt4<LOG_N>;
  const int per_class = num / pm.L;
  const int groups = (per_class + S::ROWS - 1) / S::ROWS;
  return pm.L * groups * (1 << S::A);
}

// Row-phase choice (measured on a GB300, n = 2^14 and 2^15): the warp-per-row
// kernels, three transforms of one prime per warp, are 2-3 % faster for the
// plain sink and for the plain and component sources; the CTA-per-row
// kernels stay faster for the fused sinks (encryption, ModReduce), whose
// loads want 32 consecutive pairs per warp access, and for the tensor
// source.
constexpr int kRowsWarpW = 4, kRowsWarpDpi = 3;

template <int LOG_N, class Src, class Dst>
void fwd4(const CtxDev& c, const Src& src, const Dst& dst, PrimeMap pm,
          uint64_t* buf, int num, cudaStream_t s, bool small_in = false) {
  using S = Ntt4<LOG_N>;
  // column kernel; small_in: every source value below 2^32
  auto cols = [&](auto lazy) {
    constexpr bool LZ = decltype(lazy)::value;
    auto k1 = k4_fwd_cols<LOG_N, LZ, Src>;
    if constexpr (std::is_same_v<Src, FwdSrcDigit<LOG_N>>) {
      if (small_in) k1 = k4_fwd_cols<LOG_N, LZ, Src, true>;
    }
    set_smem4(k1, S::COL_SMEM);
    k1<<<num * S::COL_TILES, S::COL_THREADS, S::COL_SMEM, s>>>(src, pm, buf, c);
  };
  if (c.small_q)
    cols(std::true_type{});
  else
    cols(std::false_type{});
  if constexpr (std::is_same_v<Dst, FwdDstPlain<LOG_N>>) {
    constexpr int W = kRowsWarpW, DPI = kRowsWarpDpi;
    const int groups = (num / pm.L + DPI - 1) / DPI;
    const int blocks = pm.L * groups * (1 << S::A) / W;
    auto k2 = c.small_q ? k4_fwd_rows_warp<LOG_N, true, Dst, W, DPI>
                        : k4_fwd_rows_warp<LOG_N, false, Dst, W, DPI>;
    set_smem4(k2, W * DPI * (1 << S::B) * 8);
    k2<<<blocks, 32 * W, W * DPI * (1 << S::B) * 8, s>>>(buf, dst, pm, num, c);
  } else {
    auto k2 = c.small_q ? k4_fwd_rows<LOG_N, true, Dst> : k4_fwd_rows<LOG_N, false, Dst>;
    set_smem4(k2, S::ROW_SMEM);
    k2<<<row_blocks<LOG_N>(num, pm), S::ROW_THREADS, S::ROW_SMEM, s>>>(buf, dst, pm,
                                                                      num, c);
  }
}

template <int LOG_N, class Src, class Dst>
void inv4(const CtxDev& c, const Src& src, const Dst& dst, PrimeMap pm,
          uint64_t* buf, int num, cudaStream_t s) {
  using S = Ntt4<LOG_N>;
  auto k2 = c.small_q ? k4_inv_cols<LOG_N, true, Dst> : k4_inv_cols<LOG_N, false, Dst>;
  set_smem4(k2, S::COL_SMEM);
  constexpr bool warp_rows = std::is_same_v<Src, InvSrcPlain<LOG_N>> ||
                             std::is_same_v<Src, InvSrcComponent<LOG_N>>;
  if (warp_rows && num % pm.L == 0) {
    constexpr int W = kRowsWarpW, DPI = kRowsWarpDpi;
    const int groups = pm.L * ((num / pm.L + DPI - 1) / DPI);
    auto k1 = c.small_q ? k4_inv_rows_warp<LOG_N, true, Src, W, DPI>
                        : k4_inv_rows_warp<LOG_N, false, Src, W, DPI>;
    set_smem4(k1, W * DPI * (1 << S::B) * 8);
    k1<<<groups * (1 << S::A) / W, 32 * W, W * DPI * (1 << S::B) * 8, s>>>(src, pm, buf, num, c);
  } else {
    auto k1 = c.small_q ? k4_inv_rows<LOG_N, true, Src> : k4_inv_rows<LOG_N, false, Src>;
    set_smem4(k1, S::ROW_SMEM);
    k1<<<num * S::ROW_TILES, S::ROW_THREADS, S::ROW_SMEM, s>>>(src, pm, buf, c);
  }
  k2<<<num * S::COL_TILES, S::COL_THREADS, S::COL_SMEM, s>>>(buf, dst, pm, c);
}

#define SHG_DISPATCH4(log_n, F) \
  switch (log_n) {              \
    case 12: F(12); break;      \
    case 13: F(13); break;      \
    case 14: F(14); break;      \
    case 15: F(15); break;      \
    default: break;             \
  }

}  // namespace

void launch4_ntt_fwd(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                     int L, cudaStream_t s) {
#define F(LN) fwd4<LN>(c, FwdSrcPlain<LN>{in}, FwdDstPlain<LN>{out}, PrimeMap{0, 1, L}, out, num, s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_ntt_inv(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                     int L, int in_first, int in_stride, int mode, uint64_t sw,
                     uint64_t swp, cudaStream_t s) {
#define F(LN)                                                                    \
  inv4<LN>(c, InvSrcPlain<LN>{in, in_first, in_stride},                         \
           InvDstScale<LN>{out, mode, sw, swp}, PrimeMap{in_first, in_stride, L}, \
           out, num, s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_tensor_intt(const CtxDev& c, uint64_t* out01, uint64_t* X,
                         const uint64_t* a, const uint64_t* b, int count, int L,
                         cudaStream_t s) {
#define F(LN)                                                                  \
  inv4<LN>(c, InvSrcTensor<LN>{a, b, out01, L}, InvDstScale<LN>{X, 1, 0, 0},  \
           PrimeMap{0, 1, L}, X, count * L, s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_intt_export(const CtxDev& c, uint64_t* X, const uint64_t* ct,
                         int ncomp, int comp, int subst_power, CtMap map,
                         int count, int L, cudaStream_t s) {
#define F(LN)                                                                  \
  inv4<LN>(c, InvSrcComponent<LN>{ct, ncomp, comp, subst_power, L, map},      \
           InvDstScale<LN>{X, 1, 0, 0}, PrimeMap{0, 1, L}, X, count * L, s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_digit_ntt(const CtxDev& c, uint64_t* D, const uint64_t* X,
                       const DigitDesc* digits, int k, int digit_flags, int count,
                       int L, cudaStream_t s) {
  const int need_lift = digit_flags & 1;
#define F(LN)                                                                  \
  fwd4<LN>(c, FwdSrcDigit<LN>{X, digits, k, L, need_lift}, FwdDstPlain<LN>{D}, \
           PrimeMap{0, 1, L}, D, count * k * L, s, digit_flags == 0)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

int ks4_rows_per_cta(int k) {
  constexpr int T = NttCore<kNtt4RowBits, 4>::T;
  for (int R = 1; R <= 4; R *= 2)
    if ((R * k * T) % 32 == 0 && R * k * T <= kKsRowsMaxThreads) return R;
  return k >= 1 && k * T <= kKsRowsMaxThreads ? 1 : 0;
}

void launch4_digit_cols(const CtxDev& c, uint64_t* D, const uint64_t* X,
                        const DigitDesc* digits, int k, int digit_flags, int count,
                        int L, cudaStream_t s) {
  // Digits of at most 32 bits without the balanced lift (every gadget base up
  // to 2^32 below the primes' halves): one CTA per digit tile for all limbs,
  // when that still gives two full waves of CTAs (six per SM); a handful of
  // ciphertexts (one-call-per-op use) keeps one CTA per digit and limb.
  if (digit_flags == 0 &&
      (long long)count * k * Ntt4<14>::COL_TILES >= 2LL * 6 * c.sms) {  // tiles: any n
#define F(LN)                                                                   \
  {                                                                             \
    using S = Ntt4<LN>;                                                         \
    auto k1 = c.small_q ? k4_digit_cols_all<LN, true, uint32_t>                 \
                        : k4_digit_cols_all<LN, false, uint32_t>;               \
    set_smem4(k1, S::COL_SMEM);                                                 \
    k1<<<count * k * S::COL_TILES, S::COL_THREADS, S::COL_SMEM, s>>>(X, digits, k, L, 0, D, c); \
  }
    SHG_DISPATCH4(c.log_n, F)
#undef F
    return;
  }
  const int need_lift = digit_flags & 1;
#define F(LN)                                                                   \
  {                                                                             \
    using S = Ntt4<LN>;                                                         \
    const FwdSrcDigit<LN> src{X, digits, k, L, need_lift};                      \
    auto k1 = c.small_q ? k4_fwd_cols<LN, true, FwdSrcDigit<LN>>                \
                        : k4_fwd_cols<LN, false, FwdSrcDigit<LN>>;              \
    if (digit_flags == 0)                                                       \
      k1 = c.small_q ? k4_fwd_cols<LN, true, FwdSrcDigit<LN>, true>             \
                     : k4_fwd_cols<LN, false, FwdSrcDigit<LN>, true>;           \
    set_smem4(k1, S::COL_SMEM);                                                 \
    k1<<<count * k * L * S::COL_TILES, S::COL_THREADS, S::COL_SMEM, s>>>(       \
        src, PrimeMap{0, 1, L}, D, c);                                          \
  }
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_ks_rows(const CtxDev& c, const uint64_t* D, int k, int chunk,
                     const uint64_t* kb, const uint64_t* ka, uint64_t* out,
                     const uint64_t* base, size_t base_ct_elems, CtMap map,
                     int base1_zero, int subst_power, int count, int L,
                     cudaStream_t s, const KeyTable& kt) {
  // One REDC covers every digit (lazily reduced digits of primes below 2^58
  // at the usual digit counts, canonical ones of larger primes at up to
  // floor(2^64 / q) digits): one warp per row, all digits in turn.
  // ... and the launch still gives two full waves of CTAs (five per SM); a
  // handful of ciphertexts keeps the row kernels below, which spread one
  // row's digits over a CTA.
  const bool fits_rows8 = k % 2 == 0 && k * 16 <= kKsRowsMaxThreads;
  if (chunk >= k && (!fits_rows8 || (long long)count * L * ((1 << (c.log_n - 7)) / kKsWarpRows) >=
                                        2LL * 5 * c.sms)) {
#define F(LN)                                                                   \
  {                                                                             \
    auto kern = c.small_q ? k4_ks_rows_warp<LN, true, kKsWarpRows, 4, kKsWarpDigits>   \
                          : k4_ks_rows_warp<LN, false, kKsWarpRows, 4, kKsWarpDigits>; \
    if (c.narrow_q) kern = k4_ks_rows_warp<LN, true, kKsWarpRows, 4, kKsWarpDigits, true>; \
    const int smem = kKsWarpRows * kKsWarpDigits * 128 * 8;                     \
    set_smem4(kern, smem);                                                      \
    kern<<<count * L * ((1 << (LN - 7)) / kKsWarpRows), 32 * kKsWarpRows, smem, s>>>( \
        D, k, kb, ka, out, base, base_ct_elems, map, base1_zero, subst_power, L, kt, c); \
  }
    SHG_DISPATCH4(c.log_n, F)
#undef F
    return;
  }
  if (k % 2 == 0 && k * 16 <= kKsRowsMaxThreads) {
#define F(LN)                                                                   \
  {                                                                             \
    using S = Ntt4<LN>;                                                         \
    auto kern = c.small_q ? k4_ks_rows8<LN, true> : k4_ks_rows8<LN, false>;     \
    const int smem = k * (1 << S::B) * 8;                                       \
    set_smem4(kern, smem);                                                      \
    kern<<<count * L * (1 << S::A), k * 16, smem, s>>>(                         \
        D, k, chunk, kb, ka, out, base, base_ct_elems, map, base1_zero,         \
        subst_power, L, kt, c);                                                 \
  }
    SHG_DISPATCH4(c.log_n, F)
#undef F
    return;
  }
  const int R = ks4_rows_per_cta(k);
#define F(LN)                                                                   \
  {                                                                             \
    using S = Ntt4<LN>;                                                         \
    auto kern = c.small_q ? k4_ks_rows<LN, true> : k4_ks_rows<LN, false>;       \
    const int threads = R * k * S::RC::T;                                       \
    const int smem = R * k * (1 << S::B) * 8;                                   \
    set_smem4(kern, smem);                                                      \
    kern<<<count * L * ((1 << S::A) / R), threads, smem, s>>>(                  \
        D, k, R, chunk, kb, ka, out, base, base_ct_elems, map, base1_zero,      \
        subst_power, L, kt, c);                                                 \
  }
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_modreduce_lift(const CtxDev& c, uint64_t* out, const uint64_t* Y,
                            const uint64_t* in, const ScalarPack& sc, int count,
                            int L, cudaStream_t s) {
#define F(LN)                                                                  \
  fwd4<LN>(c, FwdSrcModLift<LN>{Y, L - 1}, FwdDstModCombine<LN>{out, in, L, sc}, \
           PrimeMap{0, 1, L - 1}, out, count * (L - 1), s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

void launch4_bgv_encrypt(const CtxDev& c, uint64_t* out, const int32_t* err,
                         const uint64_t* m, const uint64_t* key, const ScalarPack& tm,
                         uint64_t* buf, int count, int L, cudaStream_t s) {
  if (count <= 0) return;
  LaunchScope scope_("bgv_encrypt_ntt", s);
  g_launch_count++;  // second phase kernel
#define F(LN)                                                                       \
  fwd4<LN>(c, FwdSrcError<LN>{err, L}, FwdDstBgvEnc<LN>{out, m, key, L, tm},         \
           PrimeMap{0, 1, L}, buf, count * L, s)
  SHG_DISPATCH4(c.log_n, F)
#undef F
}

unsigned take_debug_word_ntt4() {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_shg_dbg, sizeof(v)) != cudaSuccess) return 0;
  if (v) cudaMemcpyToSymbol(g_shg_dbg, &z, sizeof(z));
  return v;
}

}  // namespace shg
