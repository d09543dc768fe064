// On-device sampling of BGV encryption randomness from SHELL's ChaCha PRNG.
//
// SingleThreadChaChaPrng (prng/single_thread_chacha_prng.cc,
// prng/chacha_prng_util.cc:30-98) expands a 32-byte seed into a byte stream:
// salt s contributes 8160 bytes (kChaChaOutputBytes) of ChaCha20 keystream
// (RFC 7539) under the seed as key, nonce "salt" || s as 8 little-endian
// bytes and block counter 0, 1, ...; Rand64 takes the next 8 bytes little
// endian, Rand8 the next byte.  8160 = 127 * 64 + 32, so block 127 of every
// salt is cut to 32 bytes, and 8-byte words never straddle a block.
//
// RnsRlweSecretKey::EncryptPolynomialBgv (rns/rns_secret_key.h:188-231)
// draws, from one such stream per ciphertext,
//   a = RnsPolynomial::SampleUniform (rns/rns_polynomial.h:638-667): limb by
//       limb, each coefficient the first Rand64 masked to log q bits that is
//       below q (MontgomeryInt::ImportRandom), taken as the Montgomery value;
//   e = SampleError (rns/error_distribution.h:40-60): centred binomial
//       coefficients of variance v (SampleFromErrorDistribution,
//       sample_error.h:43-100; k = 2v bit pairs, 16 bytes per 64 pairs, 2
//       bytes per 8 and 2 for the rest), lifted balanced to every limb.
// The uniform part is a sequential rejection scan, so one CTA owns one
// ciphertext's stream: each pass generates one ChaCha block per thread,
// block-scans the accepted words and writes them in stream order.  The error
// coefficients then sit at fixed byte offsets after the uniform part and are
// produced in parallel from keystream staged in shared memory.
#include "kernels.cuh"

namespace shg {
namespace {

constexpr int kSaltWords = 1020;   // 8160 bytes of keystream per salt
constexpr int kSaltBytes = 8160;

__device__ __forceinline__ uint32_t rotl32(uint32_t v, int c) {
  return __funnelshift_l(v, v, c);
}

#define SHG_QUARTER(a, b, c, d) \
  a += b; d ^= a; d = rotl32(d, 16); \
  c += d; b ^= c; b = rotl32(b, 12); \
  a += b; d ^= a; d = rotl32(d, 8);  \
  c += d; b ^= c; b = rotl32(b, 7);

// ChaCha20 block (RFC 7539 section 2.3) of the seed `key` for keystream
// block `blk` of salt `salt`: nonce words ("salt", salt lo, salt hi).
__device__ __forceinline__ void chacha_block(const uint32_t (&key)[8], uint32_t blk,
                                             uint64_t salt, uint32_t (&x)[16]) {
  uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                    key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                    blk, 0x746c6173u /* "salt" */, (uint32_t)salt,
                    (uint32_t)(salt >> 32)};
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = s[i];
#pragma unroll 2
  for (int r = 0; r < 10; ++r) {
    SHG_QUARTER(x[0], x[4], x[8], x[12])
    SHG_QUARTER(x[1], x[5], x[9], x[13])
    SHG_QUARTER(x[2], x[6], x[10], x[14])
    SHG_QUARTER(x[3], x[7], x[11], x[15])
    SHG_QUARTER(x[0], x[5], x[10], x[15])
    SHG_QUARTER(x[1], x[6], x[11], x[12])
    SHG_QUARTER(x[2], x[7], x[8], x[13])
    SHG_QUARTER(x[3], x[4], x[9], x[14])
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] += s[i];
}
#undef SHG_QUARTER

// Global keystream block g = salt * 128 + b (b < 128) covers stream words
// [word0(g), word0(g) + (b == 127 ? 4 : 8)).
__device__ __forceinline__ uint64_t word0(uint64_t g) {
  return (g >> 7) * kSaltWords + (g & 127) * 8;
}
__device__ __forceinline__ uint64_t block_of_word(uint64_t w) {
  return (w / kSaltWords) * 128 + (w % kSaltWords) / 8;
}
__device__ __forceinline__ uint64_t block_of_byte(uint64_t b) {
  return (b / kSaltBytes) * 128 + (b % kSaltBytes) / 64;
}

// Bytes of stream one error coefficient takes for k = 2 * variance pairs.
__host__ __device__ __forceinline__ int error_bytes(int k) {
  return 16 * (k / 64) + 2 * ((k % 64) / 8) + ((k % 8) ? 2 : 0);
}

// Exclusive block-wide prefix sum of v over THREADS threads; *total gets
// the sum.
template <int THREADS>
__device__ __forceinline__ int block_scan(int v, int* warp_sums, int* total) {
  constexpr int W = THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < W ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < W; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < W) warp_sums[lane] = w;
  }
  __syncthreads();
  const int before = wid ? warp_sums[wid - 1] : 0;
  *total = warp_sums[W - 1];
  return before + x - v;
}

// Staging slot of accepted word r: the low four bits XORed with the next
// four, so eight words per thread at consecutive ranks (the usual case) and
// the in-order copy-out both run without shared-memory bank conflicts.
__device__ __forceinline__ int stage_slot(int r) { return r ^ ((r >> 4) & 15); }

// One CTA of THREADS threads per ciphertext p.  a (uniform, Montgomery
// values; negated when `negate`, i.e. written as c1 = -a) goes to
// a_dst + p * a_stride as [L][n]; the signed error coefficients to err [p][n].
template <int THREADS>
__global__ void __launch_bounds__(THREADS)
    k_sample_uniform_error(uint64_t* a_dst, size_t a_stride, int negate, int32_t* err,
                           const uint8_t* seeds, int L, int variance, int log_n, CtxDev c) {
  constexpr int kStageWords = THREADS * 8;
  __shared__ uint64_t stage[kStageWords];  // accepted words / error keystream bytes
  __shared__ int warp_sums[THREADS / 32];
  __shared__ unsigned long long s_stop;
  const int p = blockIdx.x, tid = threadIdx.x;
  const int n = 1 << log_n;
  uint32_t key[8];
  {
    const uint4* sp = reinterpret_cast<const uint4*>(seeds + (size_t)p * 32);
    const uint4 k0 = sp[0], k1 = sp[1];
    key[0] = k0.x; key[1] = k0.y; key[2] = k0.z; key[3] = k0.w;
    key[4] = k1.x; key[5] = k1.y; key[6] = k1.z; key[7] = k1.w;
  }
  uint64_t pos = 0;  // next candidate word of the stream
  for (int l = 0; l < L; ++l) {
    const PrimeDev& P = c.primes[l];
    const uint64_t q = P.q;
    const uint64_t mask = P.log_q >= 64 ? ~0ull : ((1ull << P.log_q) - 1);
    uint64_t* dst = a_dst + (size_t)p * a_stride + ((size_t)l << log_n);
    int accepted = 0;
    while (accepted < n) {
      const int need = n - accepted;
      // Blocks this pass: what `need` words take without rejections, plus
      // one for a start inside a block and one for a short block; a pass
      // that falls short is followed by another.
      const int nb = min(THREADS, need / 8 + 2);
      const uint64_t g0 = block_of_word(pos);
      const uint64_t g = g0 + tid;
      const uint64_t w0 = word0(g);
      uint64_t v[8];
      unsigned ok = 0;
      if (tid < nb) {
        uint32_t x[16];
        chacha_block(key, (uint32_t)(g & 127), g >> 7, x);
        // words before `pos` (only in block g0) and past a short block's end
        // are not candidates
        const int first = tid == 0 ? (int)(pos - w0) : 0;
        const int nw = (g & 127) == 127 ? 4 : 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          v[k] = ((uint64_t)x[2 * k + 1] << 32 | x[2 * k]) & mask;
          if (k >= first && k < nw && v[k] < q) ok |= 1u << k;
        }
      }
      int total;
      int r = block_scan<THREADS>(__popc(ok), warp_sums, &total);
      const int take = min(total, need);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (ok >> k & 1u) {
          if (r < need) stage[stage_slot(r)] = v[k];
          if (r == need - 1) s_stop = w0 + k + 1;
          ++r;
        }
      }
      __syncthreads();
      for (int i = tid; i < take; i += THREADS) {
        const uint64_t a = stage[stage_slot(i)];
        dst[accepted + i] = negate ? q - a : a;
      }
      pos = total >= need ? s_stop : word0(g0 + nb);
      accepted += take;
      __syncthreads();  // stage and s_stop are rewritten by the next pass
    }
  }

  // Error coefficients: coefficient j takes stream bytes
  // [e0 + j * B, e0 + (j + 1) * B), e0 = 8 * pos.
  const int k2 = 2 * variance;
  const int B = error_bytes(k2);
  const int per_pass = (kStageWords * 8) / B;
  uint8_t* bytes = reinterpret_cast<uint8_t*>(stage);
  const uint64_t e0 = pos * 8;
  for (int j0 = 0; j0 < n; j0 += per_pass) {
    const int J = min(per_pass, n - j0);
    const uint64_t r0 = e0 + (uint64_t)j0 * B, r1 = r0 + (uint64_t)J * B;
    const uint64_t gb0 = block_of_byte(r0), gb1 = block_of_byte(r1 - 1);
    for (uint64_t g = gb0 + tid; g <= gb1; g += THREADS) {
      uint32_t x[16];
      chacha_block(key, (uint32_t)(g & 127), g >> 7, x);
      const uint64_t b0 = (g >> 7) * kSaltBytes + (g & 127) * 64;
      const int len = (g & 127) == 127 ? 32 : 64;
      const uint64_t lo = max(b0, r0), hi = min(b0 + len, r1);
      if (((lo | hi) & 3) == 0 && ((b0 - r0) & 3) == 0) {
        // whole 32-bit words (block starts are 32-byte aligned)
        uint32_t* words = reinterpret_cast<uint32_t*>(bytes);
        for (uint64_t b = lo; b < hi; b += 4) words[(b - r0) >> 2] = x[(b - b0) >> 2];
      } else {
        for (uint64_t b = lo; b < hi; ++b) {
          const uint32_t w = x[(b - b0) >> 2];
          bytes[b - r0] = (uint8_t)(w >> (8 * ((b - b0) & 3)));
        }
      }
    }
    __syncthreads();
    for (int j = tid; j < J; j += THREADS) {
      const uint8_t* cb = bytes + (size_t)j * B;
      int val = 0, kk = k2;
      while (kk > 0) {
        if (kk >= 64) {
          uint64_t plus = 0, minus = 0;
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            plus |= (uint64_t)cb[i] << (8 * i);
            minus |= (uint64_t)cb[8 + i] << (8 * i);
          }
          val += __popcll(plus) - __popcll(minus);
          cb += 16;
          kk -= 64;
        } else if (kk >= 8) {
          val += __popc(cb[0]) - __popc(cb[1]);
          cb += 2;
          kk -= 8;
        } else {
          const unsigned m = (1u << kk) - 1;
          val += __popc(cb[0] & m) - __popc(cb[1] & m);
          break;
        }
      }
      err[((size_t)p << log_n) + j0 + j] = val;
    }
    __syncthreads();
  }
}

// Signed error e (|e| < q) as the Montgomery value of e mod q: the balanced
// lift of ConvertBalancedFromPolynomialCoeffs (rns/rns_polynomial.h).
__device__ __forceinline__ uint64_t error_mont(int e, const PrimeDev& P) {
  const uint64_t u =
      shoup((uint64_t)(e < 0 ? -e : e), P.r_mod_q, P.r_mod_q_shoup, P.q);
  return (e < 0 && u) ? P.q - u : u;
}

// out [count][L][n] <- the Montgomery lift of err [count][n] to each limb.
__global__ void k_error_lift(uint64_t* out, const int32_t* err, size_t total, int log_n,
                             int L, CtxDev c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const size_t j = e & (((size_t)1 << log_n) - 1);
    const size_t pl = e >> log_n;
    const int l = (int)(pl % L);
    const size_t p = pl / L;
    out[e] = error_mont(err[(p << log_n) + j], c.primes[l]);
  }
}

// EncryptPolynomialBgv combine per ciphertext p, limb l:
//   c0 = e * t + m + a * s with a = -c1 (c1 already holds -a), s = key.
// e_ntt [count][L][n]; out [count][2][L][n]; tm.v[l] = t in Montgomery form.
__global__ void k_bgv_enc_combine(uint64_t* out, const uint64_t* e_ntt, const uint64_t* m,
                                  const uint64_t* key, ScalarPack tm, size_t total, int log_n,
                                  int L, CtxDev c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t n = (size_t)1 << log_n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const size_t j = e & (n - 1), pl = e >> log_n;
    const int l = (int)(pl % L);
    const size_t p = pl / L;
    const PrimeDev& P = c.primes[l];
    const uint64_t q = P.q, qinv = P.inv_modulus;
    uint64_t* o = out + (p * 2 * L + l) * n + j;
    const uint64_t a = q - o[(size_t)L * n];
    uint64_t c0 = mont_mul(e_ntt[e], tm.v[l], q, qinv);
    c0 = add_mod(c0, m[e], q);
    c0 = add_mod(c0, mont_mul(a, key[((size_t)l << log_n) + j], q, qinv), q);
    *o = c0;
  }
}

}  // namespace

int sample_error_bytes(int variance) { return error_bytes(2 * variance); }

void launch_sample_uniform_error(const CtxDev& c, uint64_t* a_dst, size_t a_stride,
                                 int negate, int32_t* err, const uint8_t* seeds, int L,
                                 int variance, int count, cudaStream_t s) {
  if (count <= 0) return;
  LaunchScope scope_("sample_uniform_error", s);
  // 256-thread CTAs: four per SM (64 registers each), so 1024 ciphertexts
  // take 1.7 waves of 608 slots rather than 3.4 waves of 304.
  constexpr int T = 256;
  k_sample_uniform_error<T><<<count, T, 0, s>>>(a_dst, a_stride, negate, err, seeds, L,
                                                variance, c.log_n, c);
}

void launch_error_lift(const CtxDev& c, uint64_t* out, const int32_t* err, int count, int L,
                       cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("error_lift", s);
  k_error_lift<<<grid_for(total, 256), 256, 0, s>>>(out, err, total, c.log_n, L, c);
}

void launch_bgv_enc_combine(const CtxDev& c, uint64_t* out, const uint64_t* e_ntt,
                            const uint64_t* m, const uint64_t* key, const ScalarPack& tm,
                            int count, int L, cudaStream_t s) {
  const size_t total = (size_t)count * L * c.n;
  if (total == 0) return;
  LaunchScope scope_("bgv_enc_combine", s);
  k_bgv_enc_combine<<<grid_for(total, 256), 256, 0, s>>>(out, e_ntt, m, key, tm, total,
                                                         c.log_n, L, c);
}

}  // namespace shg
