// Device-side 64-bit modular arithmetic for residues mod q < 2^62.
//
// Stored residues follow SHELL's MontgomeryInt<uint64> convention
// (montgomery.h:226-300): a value x is held as x * 2^64 mod q, canonical in
// [0, q).  Internally the kernels use Harvey-style lazy ranges ([0, 2q) or
// [0, 4q)) and Shoup constant multiplication; every value that leaves a
// kernel is canonical, so outputs are bit-identical to the reference.
#pragma once
#include <stdint.h>

namespace shg {

// Per-prime constants, resident in device memory (one entry per RNS limb).
struct PrimeDev {
  uint64_t q;
  uint64_t two_q;
  uint64_t inv_modulus;    // -q^{-1} mod 2^64 (montgomery.h inv_modulus)
  uint64_t r_mod_q;        // 2^64 mod q  (Montgomery one)
  uint64_t r_mod_q_shoup;  // floor(r_mod_q * 2^64 / q)
  uint64_t inv_r;          // 2^-64 mod q
  uint64_t inv_r_shoup;
  uint64_t n_inv;          // n^{-1} mod q (plain)
  uint64_t n_inv_shoup;
  uint64_t n_inv_r;        // n^{-1} * 2^-64 mod q (iNTT fused with export)
  uint64_t n_inv_r_shoup;
  uint64_t half_q;         // floor(q / 2): balanced-lift threshold
  uint64_t log_q;
  uint64_t barrett;        // floor(2^64 / q): x mod q for any 64-bit x
  uint64_t pad[2];
};
static_assert(sizeof(PrimeDev) == 128, "PrimeDev is one cache line");

// High 64 bits of a * b from the four 32x32 partial products on carry
// chains (inline PTX).
__device__ __forceinline__ uint64_t mulhi64(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 al, ah, bl, bh, c1, c2, c3;\n\t"
      "mov.b64 {al, ah}, %1;\n\t"
      "mov.b64 {bl, bh}, %2;\n\t"
      "mul.hi.u32 c1, al, bl;\n\t"
      "mad.lo.cc.u32 c1, al, bh, c1;\n\t"
      "madc.hi.u32 c2, al, bh, 0;\n\t"
      "mad.lo.cc.u32 c1, ah, bl, c1;\n\t"
      "madc.hi.cc.u32 c2, ah, bl, c2;\n\t"
      "addc.u32 c3, 0, 0;\n\t"
      "mad.lo.cc.u32 c2, ah, bh, c2;\n\t"
      "madc.hi.u32 c3, ah, bh, c3;\n\t"
      "mov.b64 %0, {c2, c3};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}

// x * w mod q using the Shoup constant wp = floor(w * 2^64 / q).
// Valid for any x < 2^64 and w < q; result in [0, 2q).  One carry chain
// forms Q = floor(x * wp / 2^64); then x * w + Q * (2^64 - q) mod 2^64 comes
// from two widening multiply-adds for the low products and four 32-bit
// multiply-adds into the high word, instead of two 64-bit products and a
// 64-bit subtraction.
__device__ __forceinline__ uint64_t shoup_lazy(uint64_t x, uint64_t w,
                                               uint64_t wp, uint64_t q) {
  const uint64_t nq = 0 - q;  // loop-invariant: the compiler hoists it
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 xl, xh, wl, wh, pl, ph, nl, nh, c1, c2, c3, rl, rh;\n\t"
      ".reg .u64 t;\n\t"
      "mov.b64 {xl, xh}, %1;\n\t"
      "mov.b64 {wl, wh}, %2;\n\t"
      "mov.b64 {pl, ph}, %3;\n\t"
      "mov.b64 {nl, nh}, %4;\n\t"
      "mul.hi.u32 c1, xl, pl;\n\t"
      "mad.lo.cc.u32 c1, xl, ph, c1;\n\t"
      "madc.hi.u32 c2, xl, ph, 0;\n\t"
      "mad.lo.cc.u32 c1, xh, pl, c1;\n\t"
      "madc.hi.cc.u32 c2, xh, pl, c2;\n\t"
      "addc.u32 c3, 0, 0;\n\t"
      "mad.lo.cc.u32 c2, xh, ph, c2;\n\t"
      "madc.hi.u32 c3, xh, ph, c3;\n\t"
      "mul.wide.u32 t, xl, wl;\n\t"
      "mad.wide.u32 t, c2, nl, t;\n\t"
      "mov.b64 {rl, rh}, t;\n\t"
      "mad.lo.u32 rh, xl, wh, rh;\n\t"
      "mad.lo.u32 rh, xh, wl, rh;\n\t"
      "mad.lo.u32 rh, c2, nh, rh;\n\t"
      "mad.lo.u32 rh, c3, nl, rh;\n\t"
      "mov.b64 %0, {rl, rh};\n\t"
      "}"
      : "=l"(r)
      : "l"(x), "l"(w), "l"(wp), "l"(nq));
  return r;
}

// x * w mod q up to 4q, for the lazily reduced forward butterflies.  The
// quotient keeps three of the four partial products of x * wp:
//   Q' = xh * ph + hi32(xh * pl) + hi32(xl * ph)
// (x = xh 2^32 + xl, wp = ph 2^32 + pl).  The dropped terms lo32(xh * pl),
// lo32(xl * ph) and hi32(xl * pl) are each below 2^32, so together they carry
// at most 2 into bit 64: floor(x * wp / 2^64) - 2 <= Q' <= floor(x * wp / 2^64),
// and x * w - Q' q = (Shoup's remainder in [0, 2q)) + (0, 1 or 2) q lies in
// [0, 4q).  Four multiplies fewer than shoup_lazy.
__device__ __forceinline__ uint64_t shoup_lazy4(uint64_t x, uint64_t w,
                                                uint64_t wp, uint64_t q) {
  const uint64_t nq = 0 - q;
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 xl, xh, wl, wh, pl, ph, nl, nh, h1, h2, ql, qh, rl, rh;\n\t"
      ".reg .u64 t, qq;\n\t"
      "mov.b64 {xl, xh}, %1;\n\t"
      "mov.b64 {wl, wh}, %2;\n\t"
      "mov.b64 {pl, ph}, %3;\n\t"
      "mov.b64 {nl, nh}, %4;\n\t"
      "mul.hi.u32 h1, xh, pl;\n\t"
      "mul.hi.u32 h2, xl, ph;\n\t"
      "add.cc.u32 h1, h1, h2;\n\t"
      "addc.u32 h2, 0, 0;\n\t"
      "mov.b64 t, {h1, h2};\n\t"
      "mad.wide.u32 qq, xh, ph, t;\n\t"
      "mov.b64 {ql, qh}, qq;\n\t"
      "mul.wide.u32 t, xl, wl;\n\t"
      "mad.wide.u32 t, ql, nl, t;\n\t"
      "mov.b64 {rl, rh}, t;\n\t"
      "mad.lo.u32 rh, xl, wh, rh;\n\t"
      "mad.lo.u32 rh, xh, wl, rh;\n\t"
      "mad.lo.u32 rh, ql, nh, rh;\n\t"
      "mad.lo.u32 rh, qh, nl, rh;\n\t"
      "mov.b64 %0, {rl, rh};\n\t"
      "}"
      : "=l"(r)
      : "l"(x), "l"(w), "l"(wp), "l"(nq));
  return r;
}

// x * w mod q up to 3q for a 32-bit x (the raw gadget digits at a digit
// transform's first level).  With wp = ph 2^32 + pl the quotient
// floor(x * wp / 2^64) = floor((x ph + x pl / 2^32) / 2^32) is at most one
// above Q' = hi32(x * ph), so x * w - Q' q is Shoup's remainder in [0, 2q)
// plus 0 or q.  Five multiplies instead of shoup_lazy4's nine.
__device__ __forceinline__ uint64_t shoup_lazy_x32(uint32_t x, uint64_t w, uint64_t wp,
                                                   uint64_t q) {
  const uint64_t nq = 0 - q;
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 wl, wh, pl, ph, nl, nh, qq, rl, rh;\n\t"
      ".reg .u64 t;\n\t"
      "mov.b64 {wl, wh}, %2;\n\t"
      "mov.b64 {pl, ph}, %3;\n\t"
      "mov.b64 {nl, nh}, %4;\n\t"
      "mul.hi.u32 qq, %1, ph;\n\t"
      "mul.wide.u32 t, %1, wl;\n\t"
      "mad.wide.u32 t, qq, nl, t;\n\t"
      "mov.b64 {rl, rh}, t;\n\t"
      "mad.lo.u32 rh, %1, wh, rh;\n\t"
      "mad.lo.u32 rh, qq, nh, rh;\n\t"
      "mov.b64 %0, {rl, rh};\n\t"
      "}"
      : "=l"(r)
      : "r"(x), "l"(w), "l"(wp), "l"(nq));
  return r;
}

// The same product from two 64-bit products and a subtraction: the compiler
// schedules it with fewer live registers, which a kernel at a tight register
// cap needs (the fused form keeps -q and all 32-bit halves live).
__device__ __forceinline__ uint64_t shoup_lazy_split(uint64_t x, uint64_t w,
                                                     uint64_t wp, uint64_t q) {
  return x * w - mulhi64(x, wp) * q;
}

__device__ __forceinline__ uint64_t reduce_2q(uint64_t x, uint64_t q) {
  return x >= q ? x - q : x;
}

__device__ __forceinline__ uint64_t reduce_4q(uint64_t x, uint64_t q,
                                              uint64_t two_q) {
  x = x >= two_q ? x - two_q : x;
  return x >= q ? x - q : x;
}

__device__ __forceinline__ uint64_t shoup(uint64_t x, uint64_t w, uint64_t wp,
                                          uint64_t q) {
  return reduce_2q(shoup_lazy(x, w, wp, q), q);
}

// Montgomery product a*b*2^-64 mod q (REDC, montgomery.h:318-336); a*b < q*2^64.
// The low halves of a*b and u*q sum to 0 mod 2^64, so the carry into the high
// half is (lo != 0).
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b,
                                             uint64_t q, uint64_t qinv) {
  uint64_t lo = a * b;
  uint64_t hi = mulhi64(a, b);
  uint64_t u = lo * qinv;
  uint64_t r = hi + mulhi64(u, q) + (lo != 0);
  return reduce_2q(r, q);
}

// REDC of a 128-bit accumulator (hi:lo) < q * 2^64.
__device__ __forceinline__ uint64_t redc128(uint64_t lo, uint64_t hi,
                                            uint64_t q, uint64_t qinv) {
  uint64_t u = lo * qinv;
  uint64_t r = hi + mulhi64(u, q) + (lo != 0);
  return reduce_2q(r, q);
}

// 128-bit multiply-accumulate: (hi:lo) += a*b (the caller keeps the sum
// below 2^128).  The four 32x32 partial products go straight into the
// accumulator's 32-bit limbs with three carry chains.
__device__ __forceinline__ void mac128(uint64_t& lo, uint64_t& hi, uint64_t a,
                                       uint64_t b) {
  asm("{\n\t"
      ".reg .u32 al, ah, bl, bh, c0, c1, c2, c3;\n\t"
      "mov.b64 {al, ah}, %2;\n\t"
      "mov.b64 {bl, bh}, %3;\n\t"
      "mov.b64 {c0, c1}, %0;\n\t"
      "mov.b64 {c2, c3}, %1;\n\t"
      "mad.lo.cc.u32 c0, al, bl, c0;\n\t"
      "madc.hi.cc.u32 c1, al, bl, c1;\n\t"
      "madc.lo.cc.u32 c2, ah, bh, c2;\n\t"
      "madc.hi.u32 c3, ah, bh, c3;\n\t"
      "mad.lo.cc.u32 c1, al, bh, c1;\n\t"
      "madc.hi.cc.u32 c2, al, bh, c2;\n\t"
      "addc.u32 c3, c3, 0;\n\t"
      "mad.lo.cc.u32 c1, ah, bl, c1;\n\t"
      "madc.hi.cc.u32 c2, ah, bl, c2;\n\t"
      "addc.u32 c3, c3, 0;\n\t"
      "mov.b64 %0, {c0, c1};\n\t"
      "mov.b64 %1, {c2, c3};\n\t"
      "}"
      : "+l"(lo), "+l"(hi)
      : "l"(a), "l"(b));
}

// The three products of a ciphertext tensor: c0 = a0 b0, c1 = a0 b1 + a1 b0,
// c2 = a1 b1, each times 2^-64 mod q (Montgomery), canonical.  c1 comes from
// Karatsuba's (a0 + a1)(b0 + b1) - a0 b0 - a1 b1 on exact 128-bit products:
// three 128-bit products and three REDCs (54 multiplies) instead of two
// Montgomery products, two multiply-accumulates and a REDC (66).  Inputs below q.
__device__ __forceinline__ void tensor3(uint64_t a0, uint64_t a1, uint64_t b0, uint64_t b1,
                                        uint64_t q, uint64_t qinv, uint64_t& c0,
                                        uint64_t& c1, uint64_t& c2) {
  uint64_t p0l = 0, p0h = 0, p2l = 0, p2h = 0, sl = 0, sh = 0;
  mac128(p0l, p0h, a0, b0);
  mac128(p2l, p2h, a1, b1);
  mac128(sl, sh, a0 + a1, b0 + b1);
  // s - p0 - p2 = a0 b1 + a1 b0, exact (no borrow out of 128 bits)
  uint64_t l = sl - p0l;
  uint64_t h = sh - p0h - (sl < p0l);
  const uint64_t l2 = l - p2l;
  h = h - p2h - (l < p2l);
  c0 = redc128(p0l, p0h, q, qinv);
  c1 = redc128(l2, h, q, qinv);
  c2 = redc128(p2l, p2h, q, qinv);
}

// tensor3 of two adjacent coefficients.
__device__ __forceinline__ void tensor3_pair(const ulonglong2& a0, const ulonglong2& a1,
                                             const ulonglong2& b0, const ulonglong2& b1,
                                             uint64_t q, uint64_t qinv, ulonglong2& c0,
                                             ulonglong2& c1, ulonglong2& c2) {
  uint64_t x0, x1, x2, y0, y1, y2;
  tensor3(a0.x, a1.x, b0.x, b1.x, q, qinv, x0, x1, x2);
  tensor3(a0.y, a1.y, b0.y, b1.y, q, qinv, y0, y1, y2);
  c0 = make_ulonglong2(x0, y0);
  c1 = make_ulonglong2(x1, y1);
  c2 = make_ulonglong2(x2, y2);
}

// mac128 when the high partial product fits 32 bits: hi32(a) * hi32(b) <
// 2^32, so its high word is zero and one multiply becomes a carry add.  That
// holds for the key inner product when every prime is below 2^45: lazy digit
// transforms below 62 q give hi32(a) <= 507903, canonical key values
// hi32(b) <= 8191, and 507903 * 8191 < 2^32.
__device__ __forceinline__ void mac128_narrow(uint64_t& lo, uint64_t& hi, uint64_t a,
                                              uint64_t b) {
  asm("{\n\t"
      ".reg .u32 al, ah, bl, bh, c0, c1, c2, c3;\n\t"
      "mov.b64 {al, ah}, %2;\n\t"
      "mov.b64 {bl, bh}, %3;\n\t"
      "mov.b64 {c0, c1}, %0;\n\t"
      "mov.b64 {c2, c3}, %1;\n\t"
      "mad.lo.cc.u32 c0, al, bl, c0;\n\t"
      "madc.hi.cc.u32 c1, al, bl, c1;\n\t"
      "madc.lo.cc.u32 c2, ah, bh, c2;\n\t"
      "addc.u32 c3, c3, 0;\n\t"
      "mad.lo.cc.u32 c1, al, bh, c1;\n\t"
      "madc.hi.cc.u32 c2, al, bh, c2;\n\t"
      "addc.u32 c3, c3, 0;\n\t"
      "mad.lo.cc.u32 c1, ah, bl, c1;\n\t"
      "madc.hi.cc.u32 c2, ah, bl, c2;\n\t"
      "addc.u32 c3, c3, 0;\n\t"
      "mov.b64 %0, {c0, c1};\n\t"
      "mov.b64 %1, {c2, c3};\n\t"
      "}"
      : "+l"(lo), "+l"(hi)
      : "l"(a), "l"(b));
}

// Inputs may be any value in [0, q] (SHELL's NegateInPlace maps 0 to q,
// montgomery.h:405-408); results are canonical like the reference's Barrett
// AddInPlace / SubInPlace (montgomery.h:383-415).
__device__ __forceinline__ uint64_t reduce_2q_full(uint64_t x, uint64_t q) {
  x = x >= q ? x - q : x;
  return x >= q ? x - q : x;
}

__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b,
                                            uint64_t q) {
  return reduce_2q_full(a + b, q);
}

__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b,
                                            uint64_t q) {
  return reduce_2q_full(a + (q - b), q);
}

// NegateInPlace (montgomery.h:405-408): q - a, which is q (not 0) for a == 0.
__device__ __forceinline__ uint64_t neg_mod(uint64_t a, uint64_t q) {
  return q - a;
}

}  // namespace shg
