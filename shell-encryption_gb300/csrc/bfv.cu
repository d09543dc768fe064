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

// u of one coefficient; v[i] are the exported source values, rinv / rho the
// 64.64 reciprocals of the source primes and qd the primes as doubles.
template <int MAXS>
__device__ __forceinline__ uint64_t round_sum(const uint64_t (&v)[MAXS], const uint64_t* rinv,
                                              const uint64_t* rho, const double* qd, int ns) {
  uint64_t lo = 0, hi = 0;
#pragma unroll
  for (int i = 0; i < MAXS; ++i) {
    if (i < ns) {
      const uint64_t f = v[i] * rinv[i] + __umul64hi(v[i], rho[i]);
      lo += f;
      hi += lo < f;
    }
  }
  // |fraction - 1/2| <= 2^-32: evaluate exactly as the reference does
  if (lo - ((1ull << 63) - (1ull << 32)) <= (1ull << 33)) {
    double us = 0.0;
#pragma unroll
    for (int i = 0; i < MAXS; ++i)
      if (i < ns) us += __ull2double_rn(v[i]) / qd[i];
    return (uint64_t)round(us);
  }
  return hi + (lo >> 63);
}

// Fast path of the conversion: exactly NS (<= 8) source limbs, one 128-bit
// accumulation per destination value (the host sets `fast` only when every
// sum_i v_i w_ij + u z_j stays below p_j 2^64), unbalanced.  Each thread
// converts coefficients k and k + n/2 of one member, so every table value
// read from shared memory serves two independent carry chains.
template <int NS>
__global__ void __launch_bounds__(kConvThreads, NS >= 8 ? 2 : 3)
    k_switch_basis_ns(const BasisConv* __restrict__ bcp, const PrimeDev* __restrict__ primes,
                      const uint64_t* __restrict__ in, size_t in_stride,
                      uint64_t* __restrict__ out, size_t out_stride, size_t total_half,
                      int log_n) {
  extern __shared__ uint64_t tab[];
  const BasisConv& bc = *bcp;
  const int nd = bc.nd;
  const bool with_u = bc.mode != 2;
  // [0, 5 NS): per source limb S_i, q_i, q_i^-1 mod 2^64, rinv_i, rho_i;
  // then per destination limb p_j, p_j^-1, z_j and w_ij at w[j * NS + i].
  uint64_t* s_mul = tab;
  uint64_t* s_q = tab + NS;
  uint64_t* s_qinv = tab + 2 * NS;
  uint64_t* s_rinv = tab + 3 * NS;
  uint64_t* s_rho = tab + 4 * NS;
  uint64_t* d_q = tab + 5 * NS;
  uint64_t* d_qinv = d_q + nd;
  uint64_t* d_z = d_qinv + nd;
  uint64_t* d_w = d_z + nd;
  {
    const PrimeDev* src = primes + bc.src0;
    const PrimeDev* dst = primes + bc.dst0;
    if (threadIdx.x < NS) {
      const int i = threadIdx.x;
      s_mul[i] = bc.smul[i];
      s_q[i] = src[i].q;
      s_qinv[i] = src[i].inv_modulus;
      s_rinv[i] = bc.rinv[i];
      s_rho[i] = bc.rho[i];
    }
    for (int j = threadIdx.x; j < nd; j += blockDim.x) {
      d_q[j] = dst[j].q;
      d_qinv[j] = dst[j].inv_modulus;
      d_z[j] = bc.z2[j];
    }
    for (int t = threadIdx.x; t < NS * nd; t += blockDim.x)
      d_w[t] = bc.w2[(t % NS) * nd + t / NS];
  }
  __syncthreads();
  const size_t half = (size_t)1 << (log_n - 1);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total_half; e += stride) {
    const size_t p = e >> (log_n - 1), k = e & (half - 1);
    const uint64_t* x = in + p * in_stride + k;
    uint64_t v0[NS], v1[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      // ExportInt(x_i * S_i) in one REDC
      const uint64_t a = x[(size_t)i << log_n], b = x[((size_t)i << log_n) + half];
      const uint64_t m = s_mul[i], q = s_q[i], qinv = s_qinv[i];
      v0[i] = mont_mul(a, m, q, qinv);
      v1[i] = mont_mul(b, m, q, qinv);
    }
    uint64_t u0 = 0, u1 = 0;
    if (with_u) {
      u0 = round_sum<NS>(v0, s_rinv, s_rho, bc.qd, NS);
      u1 = round_sum<NS>(v1, s_rinv, s_rho, bc.qd, NS);
    }
    uint64_t* o = out + p * out_stride + k;
    for (int j = 0; j < nd; ++j) {
      const uint64_t* w = d_w + j * NS;
      uint64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const uint64_t wi = w[i];
        mac128(lo0, hi0, v0[i], wi);
        mac128(lo1, hi1, v1[i], wi);
      }
      if (with_u) {
        const uint64_t z = d_z[j];
        mac128(lo0, hi0, u0, z);
        mac128(lo1, hi1, u1, z);
      }
      const uint64_t q = d_q[j], qinv = d_qinv[j];
      o[(size_t)j << log_n] = redc128(lo0, hi0, q, qinv);
      o[((size_t)j << log_n) + half] = redc128(lo1, hi1, q, qinv);
    }
  }
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
    const uint64_t u = mode == 2 ? 0 : round_sum<MAXS>(v, bc.rinv, bc.rho, bc.qd, ns);
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

void launch_switch_basis(const PrimeDev* primes, ConvRef conv, int ns, int nd,
                         const uint64_t* in, size_t in_stride, uint64_t* out,
                         size_t out_stride, int count, int log_n, cudaStream_t s) {
  const size_t total = (size_t)count << log_n;
  if (total == 0 || nd == 0) return;
  LaunchScope scope_("switch_basis", s);
  const BasisConv* bc = conv.bc;
  if (conv.fast && log_n >= 1 && ns >= 1 && ns <= 8) {
    const size_t smem = sizeof(uint64_t) * (5 * ns + (3 + ns) * (size_t)nd);
    const int grid = grid_for(total / 2, kConvThreads);
#define SHG_SWITCH_NS(NS)                                                                   \
  case NS:                                                                                  \
    k_switch_basis_ns<NS><<<grid, kConvThreads, smem, s>>>(bc, primes, in, in_stride, out, \
                                                           out_stride, total / 2, log_n);   \
    return;
    switch (ns) {
      SHG_SWITCH_NS(1)
      SHG_SWITCH_NS(2)
      SHG_SWITCH_NS(3)
      SHG_SWITCH_NS(4)
      SHG_SWITCH_NS(5)
      SHG_SWITCH_NS(6)
      SHG_SWITCH_NS(7)
      SHG_SWITCH_NS(8)
    }
#undef SHG_SWITCH_NS
  }
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
