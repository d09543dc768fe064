// Four-step organisation of the negacyclic NTT for n = 2^12 .. 2^15.
//
// The transform index splits into A high "row" bits and B = 7 low "column"
// bits.  The forward transform's first A levels pair elements that differ
// only in row bits, so they run as independent length-2^A transforms down
// each column; the last B levels run along each row of 2^B contiguous
// elements.  The inverse runs rows first, then columns.  Both phases keep
// the reference's twiddle order exactly (see NttCore's tw_mult / bit_off /
// row parameters), so results equal the single-pass transform bit for bit.
//
// Each phase is a kernel with small CTAs (16 columns or 16 rows, 16 KB or
// 32 KB of shared memory), so several CTAs share an SM and overlap each
// other's memory and barrier phases; the intermediate goes through a dense
// [transform][n] buffer (normally the operation's own output, so L2).
#pragma once
#include "kernels.cuh"

namespace shg {

constexpr int kNtt4RowBits = 7;

template <int LOG_N>
struct Ntt4 {
  static constexpr int B = kNtt4RowBits;  // bits along a row
  static constexpr int A = LOG_N - B;     // bits down a column
  static constexpr int N = 1 << LOG_N;
  using CC = NttCore<A, 4>;  // column transforms, 16 values per thread
  using RC = NttCore<B, 4>;  // row transforms, 16 values per thread
  static constexpr int COLS = 16;  // columns per CTA
  static constexpr int ROWS = 16;  // rows per CTA
  static constexpr int COL_THREADS = CC::T * COLS;
  static constexpr int ROW_THREADS = RC::T * ROWS;
  static constexpr int COL_SMEM = COLS * (1 << A) * 8;
  static constexpr int ROW_SMEM = ROWS * (1 << B) * 8;
  static constexpr int COL_TILES = (1 << B) / COLS;
  static constexpr int ROW_TILES = (1 << A) / ROWS;
};

// Limb of transform g: (first + g * stride) mod L.
struct PrimeMap {
  int first, stride, L;
  __device__ __forceinline__ int operator()(int g) const {
    return (int)(((size_t)first + (size_t)g * stride) % (size_t)L);
  }
};

// Shared tile of ROWS rows: row `sub` at sub * 2^B with its 16-element
// swizzle flipped on bit 3 for odd rows, so the two rows of a half-warp land
// on disjoint bank pairs in both register layouts.
template <int B>
struct RowMap {
  uint64_t* sm;
  int sub;
  __device__ __forceinline__ uint64_t& operator()(int i) const {
    const int s = (i ^ ((i >> 4) & 15)) ^ ((sub & 1) << 3);
    return sm[(sub << B) + s];
  }
};

}  // namespace shg
