// RNS basis conversion kernels for the BFV path (rns/rns_polynomial.cc:349-852,
// rns/rns_polynomial.h:458-490, rns/rns_bfv_ciphertext.cc:33-205).
//
// SwitchRnsBasis and ScaleAndSwitchRnsBasis need u = round(sum_i v_i / q_i),
// which the reference evaluates in IEEE double precision (one correctly
// rounded division and addition per source limb, in limb order).  FP64 is
// slow on this part, so each coefficient first computes the sum in 64.64
// fixed point (v_i * 2^64 / q_i from a precomputed reciprocal, at most two
// units low per term).  The double evaluation errs by at most
// (ns + ns^2) * 2^-53 < 2^-42 for ns <= 32 and the fixed-point sum by less
// than 2^-57, so whenever the fixed-point fraction is more than 2^-32 away
// from one half both round to the same integer; the remaining coefficients
// (probability about 2^-31) redo the reference's double evaluation exactly.
#include "kernels.cuh"

namespace shg {
namespace {

constexpr int kConvThreads = 256;

// u of one coefficient; v[i] are the exported source values.
template <int MAXS>
__device__ __forceinline__ uint64_t round_sum(const uint64_t (&v)[MAXS], const BasisConv& bc,
                                              int ns) {
  uint64_t lo = 0, hi = 0;
#pragma unroll
  for (int i = 0; i < MAXS; ++i) {
    if (i < ns) {
      const uint64_t f = v[i] * bc.rinv[i] + __umul64hi(v[i], bc.rho[i]);
      lo += f;
      hi += lo < f;
    }
  }
  // |fraction - 1/2| <= 2^-32: evaluate exactly as the reference does
  if (lo - ((1ull << 63) - (1ull << 32)) <= (1ull << 33)) {
    double us = 0.0;
#pragma unroll
    for (int i = 0; i < MAXS; ++i)
      if (i < ns) us += __ull2double_rn(v[i]) / bc.qd[i];
    return (uint64_t)round(us);
  }
  return hi + (lo >> 63);
}

// One coefficient per thread: the ns source values are exported once and
// kept in registers, then every destination limb is produced in turn.
template <int MAXS>
__global__ void __launch_bounds__(kConvThreads)
    k_switch_basis(const BasisConv* __restrict__ bcp, const PrimeDev* __restrict__ primes,
                   const uint64_t* __restrict__ in, size_t in_stride,
                   uint64_t* __restrict__ out, size_t out_stride, size_t total, int log_n) {
  const BasisConv& bc = *bcp;
  const int ns = bc.ns, nd = bc.nd, mode = bc.mode, balanced = bc.balanced, chunk = bc.chunk;
  const PrimeDev* src = primes + bc.src0;
  const PrimeDev* dst = primes + bc.dst0;
  const size_t n = (size_t)1 << log_n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const size_t p = e >> log_n, k = e & (n - 1);
    const uint64_t* x = in + p * in_stride + k;
    uint64_t v[MAXS];
#pragma unroll
    for (int i = 0; i < MAXS; ++i) {
      v[i] = 0;
      // ExportInt(x_i * S_i) in one REDC
      if (i < ns) v[i] = mont_mul(x[(size_t)i << log_n], bc.smul[i], src[i].q, src[i].inv_modulus);
    }
    const uint64_t u = mode == 2 ? 0 : round_sum<MAXS>(v, bc, ns);
    uint64_t* o = out + p * out_stride + k;
    if (!balanced) {
      for (int j = 0; j < nd; ++j) {
        const uint64_t q = dst[j].q, qinv = dst[j].inv_modulus;
        const uint64_t* w2 = bc.w2 + j;
        uint64_t lo = 0, hi = 0, acc = 0;
        int left = chunk;
#pragma unroll
        for (int i = 0; i < MAXS; ++i) {
          if (i < ns) {
            mac128(lo, hi, v[i], w2[i * nd]);
            if (--left == 0 && i + 1 < ns) {
              acc = add_mod(acc, redc128(lo, hi, q, qinv), q);
              lo = hi = 0;
              left = chunk;
            }
          }
        }
        if (mode != 2) mac128(lo, hi, u, bc.z2[j]);
        o[(size_t)j << log_n] = add_mod(acc, redc128(lo, hi, q, qinv), q);
      }
    } else {
      for (int j = 0; j < nd; ++j) {
        const uint64_t q = dst[j].q;
        uint64_t acc = 0;
#pragma unroll
        for (int i = 0; i < MAXS; ++i) {
          if (i < ns) {
            uint64_t t = shoup(v[i], bc.w[i * nd + j], bc.ws[i * nd + j], q);
            if (v[i] > src[i].half_q) t = sub_mod(t, bc.wq[i * nd + j], q);
            acc = add_mod(acc, t, q);
          }
        }
        o[(size_t)j << log_n] = acc;
      }
    }
  }
}

// out = a * c_l - b * d_l (sign 1) or a * c_l + b * d_l (sign 0), per limb l.
__global__ void k_lin2(uint64_t* out, const uint64_t* a, const uint64_t* b, ScalarPack cd,
                       int sign, size_t total, int log_n, int L, CtxDev c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int l = (int)((e >> log_n) % (size_t)L);
    const PrimeDev& P = c.primes[l];
    const uint64_t x = mont_mul(a[e], cd.v[2 * l], P.q, P.inv_modulus);
    const uint64_t y = mont_mul(b[e], cd.v[2 * l + 1], P.q, P.inv_modulus);
    out[e] = sign ? sub_mod(x, y, P.q) : add_mod(x, y, P.q);
  }
}

}  // namespace

void launch_switch_basis(const PrimeDev* primes, const BasisConv* bc, int ns, int nd,
                         const uint64_t* in, size_t in_stride, uint64_t* out,
                         size_t out_stride, int count, int log_n, cudaStream_t s) {
  const size_t total = (size_t)count << log_n;
  if (total == 0 || nd == 0) return;
  LaunchScope scope_("switch_basis", s);
  const int grid = grid_for(total, kConvThreads);
  if (ns <= 4)
    k_switch_basis<4><<<grid, kConvThreads, 0, s>>>(bc, primes, in, in_stride, out,
                                                    out_stride, total, log_n);
  else if (ns <= 8)
    k_switch_basis<8><<<grid, kConvThreads, 0, s>>>(bc, primes, in, in_stride, out,
                                                    out_stride, total, log_n);
  else if (ns <= 16)
    k_switch_basis<16><<<grid, kConvThreads, 0, s>>>(bc, primes, in, in_stride, out,
                                                     out_stride, total, log_n);
  else
    k_switch_basis<kMaxLimbs><<<grid, kConvThreads, 0, s>>>(bc, primes, in, in_stride, out,
                                                            out_stride, total, log_n);
}

void launch_lin2(const CtxDev& c, uint64_t* out, const uint64_t* a, const uint64_t* b,
                 const ScalarPack& cd, int sign, int count, int L, cudaStream_t s) {
  const size_t total = (size_t)count * L << c.log_n;
  if (total == 0) return;
  LaunchScope scope_("lin2", s);
  k_lin2<<<grid_for(total, 256), 256, 0, s>>>(out, a, b, cd, sign, total, c.log_n, L, c);
}

}  // namespace shg
