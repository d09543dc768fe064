// Negacyclic NTT core for one CTA-resident limb (n = 2^LOG_N <= 2^14).
//
// The transform is the same linear map as SHELL's IterativeCooleyTukey
// (dft_transformations.h:59-100): psi is the reference's primitive 2n-th root
// (ntt_parameters.h:41-71), twiddles are psi^{brv(i)} (ntt_parameters.h:
// 117-127) and the output is in bit-reversed evaluation order.  The inverse is
// the exact inverse map, consuming the reference's psis_inv_bitrev table in
// the order of IterativeGentlemanSande (dft_transformations.h:118-153).
//
// GPU organisation: each thread holds E = 16 coefficients in registers and
// runs up to four butterfly levels on them per pass; passes exchange through
// a swizzled shared-memory tile.  Butterflies are Harvey-style with Shoup
// twiddles: forward values stay in [0, 4q), inverse values in [0, 2q), and the
// final pass reduces to canonical residues.
#pragma once
#include <stdint.h>

#include <type_traits>

#include "modarith.cuh"

namespace shg {

template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

struct Tw {
  uint64_t w;   // plain twiddle value
  uint64_t wp;  // floor(w * 2^64 / q)
};

__device__ __forceinline__ Tw load_tw(const Tw* p) {
  ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
  return Tw{v.x, v.y};
}

// Cooley-Tukey butterfly, inputs/outputs in [0, 4q).
template <bool FUSED = true>
__device__ __forceinline__ void bf_ct(uint64_t& X, uint64_t& Y, Tw w,
                                      uint64_t q, uint64_t two_q) {
  uint64_t x = X >= two_q ? X - two_q : X;
  uint64_t t = FUSED ? shoup_lazy(Y, w.w, w.wp, q) : shoup_lazy_split(Y, w.w, w.wp, q);
  X = x + t;
  Y = x - t + two_q;
}

// Cooley-Tukey butterfly without any per-level reduction.  FUSED: the Shoup
// product with the three-term quotient (shoup_lazy4, below 4q for every 64-bit
// input), Y' = X - t + 4q; otherwise the exact split product (below 2q),
// Y' = X - t + 2q.  Either way a level grows the bound by at most 4q: inputs
// below 2q stay below (4 log n + 2) q <= 62 q after the at most 15 levels of
// n <= 2^15, which fits 64 bits for q < 2^58 (the path's 45- and 50-bit
// primes); the final pass (or a sink that takes lazy values) reduces.
template <bool FUSED = true>
__device__ __forceinline__ void bf_ct_lazy(uint64_t& X, uint64_t& Y, Tw w,
                                           uint64_t q, uint64_t two_q) {
  uint64_t x = X;
  if constexpr (FUSED) {
    const uint64_t t = shoup_lazy4(Y, w.w, w.wp, q);
    X = x + t;
    Y = x - t + 2 * two_q;
  } else {
    const uint64_t t = shoup_lazy_split(Y, w.w, w.wp, q);
    X = x + t;
    Y = x - t + two_q;
  }
}

// First-level butterfly on raw inputs below 2^32 for the exact path (bf_ct's
// ranges): the 32-bit-operand product is below 3q, one conditional
// subtraction brings it below 2q.
__device__ __forceinline__ void bf_ct_x32(uint64_t& X, uint64_t& Y, Tw w, uint64_t q,
                                          uint64_t two_q) {
  const uint64_t x = X;  // below 2^32 < 2q
  uint64_t t = shoup_lazy_x32((uint32_t)Y, w.w, w.wp, q);
  t = t >= two_q ? t - q : t;
  X = x + t;
  Y = x - t + two_q;
}

// First-level lazy butterfly on raw inputs below 2^32 (Y's product from
// shoup_lazy_x32, below 3q; the outputs stay within bf_ct_lazy's ranges).
__device__ __forceinline__ void bf_ct_lazy_x32(uint64_t& X, uint64_t& Y, Tw w, uint64_t q,
                                               uint64_t two_q) {
  const uint64_t x = X;
  const uint64_t t = shoup_lazy_x32((uint32_t)Y, w.w, w.wp, q);
  X = x + t;
  Y = x - t + 2 * two_q;
}

// x mod q for any x < 2^64 with bar = floor(2^64 / q).
__device__ __forceinline__ uint64_t reduce_full(uint64_t x, uint64_t q,
                                                uint64_t bar) {
  return reduce_2q(x - mulhi64(x, bar) * q, q);
}

// Gentleman-Sande butterfly, inputs/outputs in [0, 2q) with the exact Shoup
// product; WIDE (primes below 2^58, so 8q < 2^64): inputs/outputs in [0, 4q)
// with the three-term quotient (shoup_lazy4, below 4q), the same one
// conditional subtraction, of 4q.
template <bool WIDE = false>
__device__ __forceinline__ void bf_gs(uint64_t& X, uint64_t& Y, Tw w,
                                      uint64_t q, uint64_t two_q) {
  if constexpr (WIDE) {
    const uint64_t four_q = 2 * two_q;
    uint64_t s = X + Y;
    s = s >= four_q ? s - four_q : s;
    const uint64_t d = X - Y + four_q;
    X = s;
    Y = shoup_lazy4(d, w.w, w.wp, q);
  } else {
    uint64_t s = X + Y;
    s = s >= two_q ? s - two_q : s;
    uint64_t d = X - Y + two_q;
    X = s;
    Y = shoup_lazy(d, w.w, w.wp, q);
  }
}

// Coefficients per thread: 16, or 32 at n = 2^14 (512 threads, so a thread
// may use 128 registers and the transform needs one exchange less).
__host__ __device__ constexpr int default_elog(int log_n) {
  return log_n < 4 ? log_n : (log_n == 14 ? 5 : 4);
}

template <int LOG_N, int ELOG_ = default_elog(LOG_N)>
struct NttCore {
  static_assert(LOG_N >= 1 && LOG_N <= 14, "CTA-resident NTT handles n <= 2^14");
  static constexpr int N = 1 << LOG_N;
  static constexpr int ELOG = ELOG_;

  // Shared-memory swizzle: XOR the low 4 index bits with bits ELOG..ELOG+3,
  // which makes every pass's per-register access pattern bank-conflict free
  // (each half-warp of 8-byte accesses hits 16 distinct bank pairs).
  __device__ __forceinline__ static int swz(int i) {
    return i ^ ((i >> ELOG) & 15);
  }
  static constexpr int E = 1 << ELOG;
  static constexpr int T = N / E;  // threads per limb
  static constexpr int P = (LOG_N + ELOG - 1) / ELOG;  // passes

  // Pass p covers R(p) butterfly levels.  Its registers span the contiguous
  // index-bit range [clo, clo + ELOG); within that range the butterfly bits
  // start at local bit plo.
  __host__ __device__ static constexpr int R(int p) {
    return (LOG_N - p * ELOG) < ELOG ? (LOG_N - p * ELOG) : ELOG;
  }
  // Forward: top bits first; the short last pass sits at bits [0, R) with the
  // remaining register bits above it.
  __host__ __device__ static constexpr int fwd_clo(int p) {
    return p == P - 1 ? 0 : LOG_N - p * ELOG - ELOG;
  }
  __host__ __device__ static constexpr int fwd_plo(int) { return 0; }
  // Inverse: bottom bits first; the short last pass sits at the top bits
  // with the remaining register bits below it.
  __host__ __device__ static constexpr int inv_clo(int p) {
    return p == P - 1 ? LOG_N - ELOG : p * ELOG;
  }
  __host__ __device__ static constexpr int inv_plo(int p) {
    return p == P - 1 ? ELOG - R(p) : 0;
  }

  __device__ __forceinline__ static int idx(int tid, int k, int clo) {
    return (tid & ((1 << clo) - 1)) | (k << clo) | ((tid >> clo) << (clo + ELOG));
  }
  // Register layouts at the boundaries.
  __device__ __forceinline__ static int fwd_in_idx(int tid, int k) {
    return idx(tid, k, fwd_clo(0));
  }
  __device__ __forceinline__ static int fwd_out_idx(int tid, int k) {
    return idx(tid, k, fwd_clo(P - 1));
  }
  __device__ __forceinline__ static int inv_in_idx(int tid, int k) {
    return idx(tid, k, inv_clo(0));
  }
  __device__ __forceinline__ static int inv_out_idx(int tid, int k) {
    return idx(tid, k, inv_clo(P - 1));
  }

  // One forward pass on registers.  tw is the limb's psi_bitrev table; stage s
  // reads tw[tw_mult * 2^s + (i >> (b+1))] (tw_mult = 1 for a full transform;
  // 2 + h for half h of a 2n transform whose first level ran elsewhere).
  // LAZY selects bf_ct_lazy (valid when q < 2^58, see above); FUSED the
  // butterflies' Shoup product form.
  // SMALL_IN (pass 0 only): every input is below 2^32, so the first level's
  // products take the 32-bit-operand butterflies (bf_ct_lazy_x32 / bf_ct_x32).
  template <int p, bool LAZY, bool FUSED = true, bool SMALL_IN = false>
  __device__ __forceinline__ static void fwd_pass(uint64_t (&x)[E], int tid,
                                                  const Tw* __restrict__ tw,
                                                  int tw_mult, uint64_t q,
                                                  uint64_t two_q) {
    constexpr int clo = fwd_clo(p);
    constexpr int plo = fwd_plo(p);
    constexpr int RR = R(p);
    const int tid_high = tid >> clo;
    static_for<0, RR>([&](auto ii) {
      constexpr int lb = plo + RR - 1 - decltype(ii)::value;  // high to low
      constexpr int b = clo + lb;
      constexpr int s = LOG_N - 1 - b;
      const int base = tw_mult * (1 << s) + (tid_high << (ELOG - lb - 1));
      static_for<0, (E >> (lb + 1))>([&](auto uu) {
        constexpr int u = decltype(uu)::value;
        const Tw w = load_tw(tw + base + u);
        static_for<0, (1 << lb)>([&](auto ll) {
          constexpr int k0 = (u << (lb + 1)) | decltype(ll)::value;
          constexpr int k1 = k0 | (1 << lb);
          if constexpr (SMALL_IN && p == 0 && decltype(ii)::value == 0) {
            if constexpr (LAZY) {
              bf_ct_lazy_x32(x[k0], x[k1], w, q, two_q);
            } else {
              bf_ct_x32(x[k0], x[k1], w, q, two_q);
            }
          } else if constexpr (LAZY) {
            bf_ct_lazy<FUSED>(x[k0], x[k1], w, q, two_q);
          } else {
            bf_ct<FUSED>(x[k0], x[k1], w, q, two_q);
          }
        });
      });
    });
  }

  // One inverse pass.  Layer b (local bit) reads
  //   tw[nfull - nfull / 2^(b + bit_off) + (row << (LOG_N - b - 1)) + (i >> (b+1))]
  // which is the reference's IterativeGentlemanSande order for a full
  // transform (bit_off = 0, row = 0), for row r of a transform whose low
  // LOG_N bits form the rows (bit_off = 0, row = r), and for the columns of
  // one whose low bit_off bits were done first (row = 0).
  template <int p, bool WIDE = false>
  __device__ __forceinline__ static void inv_pass(uint64_t (&x)[E], int tid,
                                                  const Tw* __restrict__ tw,
                                                  int nfull, int bit_off,
                                                  int row, uint64_t q,
                                                  uint64_t two_q) {
    constexpr int clo = inv_clo(p);
    constexpr int plo = inv_plo(p);
    constexpr int RR = R(p);
    const int tid_high = tid >> clo;
    static_for<0, RR>([&](auto ii) {
      constexpr int lb = plo + decltype(ii)::value;  // low to high
      constexpr int b = clo + lb;
      const int base = nfull - (nfull >> (b + bit_off)) +
                       (row << (LOG_N - b - 1)) + (tid_high << (ELOG - lb - 1));
      static_for<0, (E >> (lb + 1))>([&](auto uu) {
        constexpr int u = decltype(uu)::value;
        const Tw w = load_tw(tw + base + u);
        static_for<0, (1 << lb)>([&](auto ll) {
          constexpr int k0 = (u << (lb + 1)) | decltype(ll)::value;
          constexpr int k1 = k0 | (1 << lb);
          bf_gs<WIDE>(x[k0], x[k1], w, q, two_q);
        });
      });
    });
  }

  // Shared-memory position maps for the register exchanges: one transform
  // per shared tile (swizzled), or CB interleaved column transforms (element
  // i of column j at i * CB + j, conflict-free without a swizzle).
  struct SwzMap {
    uint64_t* sm;
    __device__ __forceinline__ uint64_t& operator()(int i) const { return sm[swz(i)]; }
  };
  struct ColMap {
    uint64_t* sm;
    int cb, j;
    __device__ __forceinline__ uint64_t& operator()(int i) const { return sm[i * cb + j]; }
  };

  // Register exchange through shared memory from layout clo_a to clo_b.
  template <class Map>
  __device__ __forceinline__ static void exchange(uint64_t (&x)[E], int tid,
                                                  const Map& m, int clo_a,
                                                  int clo_b) {
#pragma unroll
    for (int k = 0; k < E; ++k) m(idx(tid, k, clo_a)) = x[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < E; ++k) x[k] = m(idx(tid, k, clo_b));
    __syncthreads();
  }

  // Full forward transform on registers (input in fwd_in layout, values in
  // [0, 4q) -- below 2q for LAZY; output in fwd_out layout, values in [0, 4q),
  // or below (4 LOG_N + 2) q for LAZY).
  template <bool LAZY = false, bool FUSED = true, class Map = SwzMap, bool SMALL_IN = false>
  __device__ __forceinline__ static void forward_m(uint64_t (&x)[E], int tid,
                                                   const Map& m,
                                                   const Tw* __restrict__ tw,
                                                   int tw_mult, uint64_t q,
                                                   uint64_t two_q) {
    static_for<0, P>([&](auto pp) {
      constexpr int p = decltype(pp)::value;
      fwd_pass<p, LAZY, FUSED, SMALL_IN>(x, tid, tw, tw_mult, q, two_q);
      if constexpr (p + 1 < P) exchange(x, tid, m, fwd_clo(p), fwd_clo(p + 1));
    });
  }
  template <bool LAZY = false>
  __device__ __forceinline__ static void forward(uint64_t (&x)[E], int tid,
                                                 uint64_t* sm,
                                                 const Tw* __restrict__ tw,
                                                 int tw_mult, uint64_t q,
                                                 uint64_t two_q) {
    forward_m<LAZY>(x, tid, SwzMap{sm}, tw, tw_mult, q, two_q);
  }

  // Full inverse transform without the n^{-1} scaling (input in inv_in
  // layout, values in [0, 2q); output in inv_out layout, values in [0, 2q);
  // WIDE: [0, 4q) both, for primes below 2^58).  Every caller finishes with
  // an exact Shoup product (the n^{-1} scaling), which takes any 64-bit value;
  // a caller that stores the output without that product must reduce it
  // (below 4q with WIDE, below 2q otherwise).
  template <bool WIDE = false, class Map = SwzMap>
  __device__ __forceinline__ static void inverse_m(uint64_t (&x)[E], int tid,
                                                   const Map& m,
                                                   const Tw* __restrict__ tw,
                                                   int nfull, int bit_off,
                                                   int row, uint64_t q,
                                                   uint64_t two_q) {
    static_for<0, P>([&](auto pp) {
      constexpr int p = decltype(pp)::value;
      inv_pass<p, WIDE>(x, tid, tw, nfull, bit_off, row, q, two_q);
      if constexpr (p + 1 < P) exchange(x, tid, m, inv_clo(p), inv_clo(p + 1));
    });
  }
  template <bool WIDE = false>
  __device__ __forceinline__ static void inverse(uint64_t (&x)[E], int tid,
                                                 uint64_t* sm,
                                                 const Tw* __restrict__ tw,
                                                 int nfull, int row, uint64_t q,
                                                 uint64_t two_q) {
    inverse_m<WIDE>(x, tid, SwzMap{sm}, tw, nfull, 0, row, q, two_q);
  }
};

}  // namespace shg
