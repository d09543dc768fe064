// Internal interface between the C ABI (capi.cu) and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "modarith.cuh"
#include "ntt.cuh"

namespace shg {

constexpr int kMaxLimbs = 32;

// Device view of a context: per-limb constants and twiddle tables.
struct CtxDev {
  int log_n;
  int n;
  int L;                      // number of moduli in the context
  const PrimeDev* primes;     // [L]
  const Tw* tw_fwd;           // [L][n]  plain psi^{brv(i)} + Shoup constant
  const Tw* tw_inv;           // [L][n]  plain psis_inv_bitrev + Shoup constant
  const uint64_t* qmod;       // [L][L]  q_i mod q_j (plain), row i
  // Every q < 2^58: forward NTTs skip per-level reductions (values below 62 q)
  // and inverse NTTs run the WIDE butterflies, whose outputs lie in [0, 4q).
  // Every inverse consumer ends with an exact Shoup scaling (which takes any
  // 64-bit value); one that stores inverse output without it must reduce it.
  int small_q;
  int ntt4_min;               // log_n from which transforms use the four-step kernels
  int ks_fused;               // four-step key switch: digit row phase fused with the inner product
  int sms;                    // multiprocessors of the context's device (launch-shape choices)
  int ntt4_plain_min;         // the same threshold for plain forward / inverse NTTs
  int narrow_q;               // every q below 2^45 (implies small_q)
};

// Per-digit description of a gadget key (RnsGadget::Decompose order,
// rns/rns_gadget.cc:108-153: prime-major, least significant digit first).
struct DigitDesc {
  int src_limb;   // limb i whose residue is decomposed
  int shift;      // d * log_b_i
  uint64_t mask;  // 2^log_b_i - 1
};

// Per-member keys of a batched key switch: member p of a launch uses the key
// at kb[p >> shift], ka[p >> shift] (device tables of key base pointers, all
// keys of one gadget shape).  kb == nullptr: every member uses the launch's
// single key.
struct KeyTable {
  const uint64_t* const* kb = nullptr;
  const uint64_t* const* ka = nullptr;
  int shift = 0;
  int entries = 0;  // table entries from kb / ka on (debug builds check p >> shift)
};

// Gadget base exponents per limb (RnsGadget log_bs), passed by value.
struct GadgetBases {
  int log_b[kMaxLimbs];
};

// Small per-limb constant arrays passed by value.
struct ScalarPack {
  uint64_t v[4 * kMaxLimbs];
};

// Ciphertext addressing for batches whose members are not contiguous
// (oblivious expansion): member p lives at index
//   ((p >> grp_log) << stride_log) | (p & (2^grp_log - 1)).
struct CtMap {
  int grp_log;
  int stride_log;
  __host__ __device__ static CtMap identity() { return CtMap{30, 30}; }
  __host__ __device__ __forceinline__ size_t operator()(size_t p) const {
    return ((p >> grp_log) << stride_log) | (p & ((size_t(1) << grp_log) - 1));
  }
};

// Debug builds (compiled with SHG_DEBUG) check computed indices before they
// address memory -- substitution gathers, key-table members, gadget digit
// descriptors, limb indices.  An index outside [0, bound) records its check's
// tag in this translation unit's debug word (the first failure wins) and is
// replaced by 0, so the access stays inside its buffer and nothing traps;
// shg_debug_status() reads and clears the words.  Release builds compile the
// checks away.
enum DbgTag : unsigned {
  kDbgSubst = 1,     // NTT-domain substitution gather position
  kDbgKeyTable = 2,  // per-member key table entry
  kDbgDigit = 3,     // gadget digit descriptor / its source limb
  kDbgLimb = 4,      // limb (prime) index of a transform
};
static __device__ unsigned g_shg_dbg;
template <class I>
__device__ __forceinline__ I dbg_index(I idx, long long bound, unsigned tag) {
#ifdef SHG_DEBUG
  if ((long long)idx < 0 || (long long)idx >= bound) {
    atomicCAS(&g_shg_dbg, 0u, tag);
    return 0;
  }
#else
  (void)bound;
  (void)tag;
#endif
  return idx;
}
// The debug words of kernels.cu and ntt4.cu on the current device, cleared
// after reading (0: no check failed).
unsigned take_debug_word_kernels();
unsigned take_debug_word_ntt4();

// Number of kernels this library has launched (host-side counter).
extern std::atomic<uint64_t> g_launch_count;

// Optional per-kernel timing: while g_prof_on is set every launch is
// bracketed by a pair of CUDA events recorded on its stream.
struct ProfEntry {
  const char* name;
  cudaEvent_t a, b;
};
extern std::atomic<bool> g_prof_on;
extern std::mutex g_prof_mu;
extern std::vector<ProfEntry> g_prof_pending;

// Counts every launch and names it as an NVTX range (visible in Nsight
// timelines; a no-op without an attached tool); with profiling on, brackets
// it with CUDA events on the launch stream (these also work inside stream
// capture).
struct LaunchScope {
  const char* name;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  LaunchScope(const char* n, cudaStream_t st) : name(n), s(st) {
    nvtxRangePushA(n);
    g_launch_count++;
    if (g_prof_on.load()) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
  }
  ~LaunchScope() {
    nvtxRangePop();
    if (a) {
      cudaEventRecord(b, s);
      std::lock_guard<std::mutex> lock(g_prof_mu);
      g_prof_pending.push_back(ProfEntry{name, a, b});
    }
  }
};

// Blocks for a grid-stride loop over `work` items (at most 16 per SM).
int grid_for(size_t work, int threads);

// `num` limb transforms; limb index of transform g is g % L.
void launch_ntt_fwd(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                    int L, cudaStream_t s);
// scale_export = 1 folds ExportInt into the n^{-1} scaling (plain output).
void launch_ntt_inv(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                    int L, int scale_export, cudaStream_t s);

enum PwOp {
  PW_ADD = 0,
  PW_SUB,
  PW_NEG,
  PW_MUL,         // REDC(a, b)
  PW_FMA,         // out += REDC(a, b)
  PW_MUL_MONT,    // REDC(a, scalar_l)      v[l] = Montgomery scalar
  PW_MUL_SHOUP,   // a * w_l mod q          v[2l], v[2l+1] = w, Shoup(w)
  PW_MUL_BCAST,   // REDC(a, b) with one b [L][n] for every member of a
};
void launch_pointwise(const CtxDev& c, PwOp op, uint64_t* out, const uint64_t* a,
                      const uint64_t* b, const ScalarPack& sc, int count, int L,
                      cudaStream_t s);

void launch_substitute(const CtxDev& c, uint64_t* out, const uint64_t* in,
                       int power, int count, int L, cudaStream_t s);

// out [count][3][L][n] = a (x) b.
void launch_tensor(const CtxDev& c, uint64_t* out, const uint64_t* a,
                   const uint64_t* b, int count, int L, cudaStream_t s);

// Fused tensor product + inverse NTT of the degree-2 part:
// out01 [count][2][L][n] <- (a0*b0, a0*b1 + a1*b0); X [count][L][n] <- plain
// coefficients of a1*b1.
void launch_tensor_intt(const CtxDev& c, uint64_t* out01, uint64_t* X,
                        const uint64_t* a, const uint64_t* b, int count, int L,
                        cudaStream_t s);

// Inverse NTT + export of component `comp` of ciphertexts with `ncomp`
// components (member p at map(p)); X [count][L][n] plain coefficients.  If
// subst_power > 0 the component is substituted (NTT-domain gather) first.
void launch_intt_export(const CtxDev& c, uint64_t* X, const uint64_t* ct,
                        int ncomp, int comp, int subst_power, CtMap map,
                        int count, int L, cudaStream_t s);

// Digit decomposition + forward NTT: D [count][k][L][n] (NTT values of the
// plain digits: canonical, or below 62 q when every prime is below 2^58) from
// X [count][L][n].
void launch_digit_ntt(const CtxDev& c, uint64_t* D, const uint64_t* X,
                      const DigitDesc* digits, int k, int digit_flags, int count,
                      int L, cudaStream_t s);

// Key inner product, per ciphertext p and limb:
//   out0 = base0 + REDC(sum_j D_j * kb_j), out1 = base1 + REDC(sum_j D_j * ka_j)
// kb/ka hold the key premultiplied by 2^64 mod q (so REDC lands in Montgomery
// form); `chunk` products are summed per REDC (chunk * q < 2^64).
// out [count][2][L][n]; base component c of member p lives at
// base + map(p) * base_ct_elems + c * L * n; base1_zero drops base1.  If
// subst_power > 0, base0 is read through that substitution.
void launch_ks_inner(const CtxDev& c, uint64_t* out, const uint64_t* D,
                     const uint64_t* kb, const uint64_t* ka, int k, int chunk,
                     const uint64_t* base, size_t base_ct_elems, CtMap map,
                     int base1_zero, int subst_power, int count, int L,
                     cudaStream_t s, const KeyTable& kt = KeyTable{});

// Gadget key switch core: digit decomposition + NTT of every digit + key
// inner product + base add (launch_digit_ntt then launch_ks_inner).
// D: [count][k][L][n] scratch.  digit_flags (digit_flags() below): bit 0 the
// digits need the balanced lift, bit 1 some digit is wider than 32 bits.
inline int digit_flags(int need_lift, int max_log_b) {
  return (need_lift ? 1 : 0) | (max_log_b > 32 ? 2 : 0);
}
void launch_keyswitch(const CtxDev& c, uint64_t* D, const uint64_t* X,
                      const DigitDesc* digits, int k, int digit_flags, int chunk,
                      int chunk_lazy,
                      const uint64_t* kb, const uint64_t* ka, uint64_t* out,
                      const uint64_t* base, size_t base_ct_elems, CtMap map,
                      int base1_zero, int subst_power, int count, int L,
                      cudaStream_t s, const KeyTable& kt = KeyTable{});

// ModReduceLsb (NTT form): Y [count][n] scratch; out [count][L-1][n].
// sc.v[4i..4i+3] = (c1, Shoup(c1), c2, Shoup(c2)) for output limb i with
// out = in_i * c1 + delta_i * c2.  (k_plain, k_shoup) multiply the top limb.
void launch_modreduce_ntt(const CtxDev& c, uint64_t* out, uint64_t* Y,
                          const uint64_t* in, uint64_t k_plain,
                          uint64_t k_shoup, const ScalarPack& sc, int count,
                          int L, cudaStream_t s);
void launch_modreduce_coeff(const CtxDev& c, uint64_t* out, const uint64_t* in,
                            uint64_t k_plain, uint64_t k_shoup,
                            const ScalarPack& sc, int count, int L,
                            cudaStream_t s);

// Galois key with a precomputed random pad: mode 0 out [count][L][n] =
// sum_j pad_j * key_j (key = the stored key_a); mode 1 out [count][2][L][n] =
// (c0 + sum_j pad_j * key_j, pad_new) (key = the stored key_b).
void launch_pad_inner(const CtxDev& c, uint64_t* out, const uint64_t* pad,
                      const uint64_t* key, int k, int chunk, const uint64_t* ct,
                      const uint64_t* pad_new, int mode, int count, int L, cudaStream_t s);

// RnsGadget::Decompose: in [count][L][n] coefficient form -> out
// [count][k][L][n] coefficient form (k = sum_i GadgetSize(log q_i, log_b_i)).
void launch_decompose(const CtxDev& c, uint64_t* out, const uint64_t* in,
                      const GadgetBases& gb, int k, int count, int L,
                      cudaStream_t s);

// Oblivious-expand level combine for members p (ciphertext at map(p) of
// `base`, partner at map(p) + half): hi = (c - ks[p]) * mono; c = c + ks[p].
void launch_expand_combine(const CtxDev& c, uint64_t* base, const uint64_t* ks,
                           const uint64_t* mono, CtMap map, int half,
                           int count, cudaStream_t s);

// One RNS basis conversion between two prime sets of a context
// (RnsPolynomial::SwitchRnsBasis, ScaleAndSwitchRnsBasis, ApproxSwitchRnsBasis,
// rns/rns_polynomial.cc:419-724), kept in device memory.  Source limb i's
// exported value is v_i = ExportInt(x_i * S_i) = REDC(x_i * smul_i) with smul_i
// the plain value S_i; destination j gets sum_i ImportInt(v_i) * W_ij mod p_j
// (W_ij a Montgomery rep), then
//   mode 0: minus u * (Q mod p_j),  mode 1: plus u,  mode 2: nothing,
// with u = round(sum_i v_i / q_i) as the reference computes it in double
// precision.  Unbalanced conversions accumulate v_i * w2[i][j] (w2 = W * 2^64
// mod p_j) and u * z2[j] in 128 bits, `chunk` source limbs per REDC, so one
// REDC per chunk lands on the Montgomery rep of the sum.  balanced (mode 2):
// v_i > q_i / 2 stands for v_i - q_i; that path multiplies with Shoup
// constants (w, ws) and corrects by wq[i][j] = q_i * W_ij mod p_j.
struct BasisConv {
  int ns, nd;          // source / destination prime counts
  int src0, dst0;      // first prime index of each set in the context
  int mode, balanced;
  int chunk, pad_;     // source limbs per 128-bit accumulation
  uint64_t smul[kMaxLimbs];     // plain multiplier S_i of source limb i
  uint64_t rinv[kMaxLimbs];     // floor(2^64 / q_i)
  uint64_t rho[kMaxLimbs];      // floor(frac(2^64 / q_i) * 2^64)
  double qd[kMaxLimbs];         // (double) q_i
  uint64_t z2[kMaxLimbs];       // per destination: u's coefficient times 2^64 mod p_j
  // [i * nd + j], ns * nd entries used
  uint64_t w2[kMaxLimbs * kMaxLimbs];
  uint64_t w[kMaxLimbs * kMaxLimbs], ws[kMaxLimbs * kMaxLimbs], wq[kMaxLimbs * kMaxLimbs];
};

// out [count][nd][n] (member p at out + p * out_stride) <- the conversion of
// in [count][ns][n] (coefficient form, member p at in + p * in_stride);
// `primes` = the context's full prime array.
// A conversion table on the device; `fast` when it is unbalanced, has at
// most 8 source limbs and needs one 128-bit accumulation per output value
// (chunk >= ns), which a kernel specialised on the source count handles.
struct ConvRef {
  const BasisConv* bc;
  int fast;
};

void launch_switch_basis(const PrimeDev* primes, ConvRef conv, int ns, int nd,
                         const uint64_t* in, size_t in_stride, uint64_t* out,
                         size_t out_stride, int count, int log_n, cudaStream_t s);

// out_i = (a_i * c[i] - b_i * d[i]) mod q_i over [count][L][n] with c, d
// Montgomery scalars per limb (ScaleAndReduce / ModReduceMsb combines).
void launch_lin2(const CtxDev& c, uint64_t* out, const uint64_t* a, const uint64_t* b,
                 const ScalarPack& cd, int sign, int count, int L, cudaStream_t s);

// Serialized polynomial layout (MontgomeryInt::SerializeVector per limb):
// limb l is an n * bits[l] bit little-endian stream of the Montgomery
// residues, starting at byte offset[l] of the polynomial; a polynomial takes
// offset[L] bytes.
struct SerLayout {
  int bits[kMaxLimbs];
  unsigned long long offset[kMaxLimbs + 1];
};
void launch_deserialize(const CtxDev& c, uint64_t* polys, const uint8_t* in,
                        const SerLayout& lay, int count, int L, cudaStream_t s);
void launch_serialize(const CtxDev& c, uint8_t* out, const uint64_t* polys,
                      const SerLayout& lay, int count, int L, cudaStream_t s);

// Symmetric RLWE on limb 0: encryption combine out [count][2][n] =
// (e_ntt * t + m + a * s, -a); decryption dot product acc [count][n] =
// sum_i ct[count][i] * s^i; RemoveError of exported coefficients.
void launch_sym_encrypt(const CtxDev& c, uint64_t* out, const uint64_t* e_ntt,
                        const uint64_t* a, const uint64_t* m, const uint64_t* sk,
                        uint64_t t_mont, int count, cudaStream_t s);
void launch_sym_dot(const CtxDev& c, uint64_t* acc, const uint64_t* ct, const uint64_t* sk,
                    int len, int count, cudaStream_t s);
void launch_remove_error(const CtxDev& c, uint64_t* out, const uint64_t* x, uint64_t q,
                         uint64_t t, int count, cudaStream_t s);

// Seeded uniform residues [count][L][n] (splitmix64, reduced per limb).
void launch_fill_uniform(const CtxDev& c, uint64_t* out, uint64_t seed, int count,
                         int L, cudaStream_t s);
// dst [count][elems] <- srcs[b][elems]; dsts[b][elems] <- src [count][elems].
// elems even, every block 16-byte aligned; srcs / dsts are device tables.
void launch_gather(uint64_t* dst, const uint64_t* const* srcs, size_t elems, int count,
                   cudaStream_t s);
void launch_scatter(uint64_t* const* dsts, const uint64_t* src, size_t elems, int count,
                    cudaStream_t s);
// Sets this thread's last-error message (the C ABI's shg_last_error) and
// returns `code`.
int set_error(int code, const std::string& msg);

// BGV encryption randomness from the ChaCha PRNG of seeds [count][32]
// (RnsPolynomial::SampleUniform then SampleError): ciphertext p's uniform
// polynomial (negated when `negate`) goes to a_dst + p * a_stride as [L][n],
// its signed error coefficients to err [count][n].
void launch_sample_uniform_error(const CtxDev& c, uint64_t* a_dst, size_t a_stride,
                                 int negate, int32_t* err, const uint8_t* seeds, int L,
                                 int variance, int count, cudaStream_t s);
// Stream bytes one error coefficient of this variance takes.
int sample_error_bytes(int variance);
// out [count][L][n] <- err [count][n] lifted to every limb (Montgomery).
void launch_error_lift(const CtxDev& c, uint64_t* out, const int32_t* err, int count, int L,
                       cudaStream_t s);
// out [count][2][L][n]: c0 <- e_ntt * t + m + (-c1) * key (c1 holds -a).
void launch_bgv_enc_combine(const CtxDev& c, uint64_t* out, const uint64_t* e_ntt,
                            const uint64_t* m, const uint64_t* key, const ScalarPack& tm,
                            int count, int L, cudaStream_t s);

// mono [levels][n] <- -x^{n - 2^j} in coefficient form (minus_one = the
// Montgomery form of -1).
void launch_monomials(const CtxDev& c, uint64_t* mono, int levels,
                      uint64_t minus_one, cudaStream_t s);

// out [count][2][n] = sum_{i < num_items} cts[count][i][2][n] * db[i][n],
// query p's items starting at cts + p * item_stride * 2n.
void launch_absorb_sum(const CtxDev& c, uint64_t* out, const uint64_t* cts,
                       const uint64_t* db, int num_items, size_t item_stride,
                       int chunk, int count, cudaStream_t s);

// Butterflies per second of the NTT's lazy butterfly on register-resident
// values (the integer ceiling of every transform kernel) on the current
// device; 0 on success.
int measure_butterfly_rate(double* per_second);

// Four-step variants (ntt4.cu), n = 2^12 .. 2^15; same semantics as the
// launchers above.
void launch4_ntt_fwd(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                     int L, cudaStream_t s);
void launch4_ntt_inv(const CtxDev& c, const uint64_t* in, uint64_t* out, int num,
                     int L, int in_first, int in_stride, int mode, uint64_t sw,
                     uint64_t swp, cudaStream_t s);
void launch4_tensor_intt(const CtxDev& c, uint64_t* out01, uint64_t* X,
                         const uint64_t* a, const uint64_t* b, int count, int L,
                         cudaStream_t s);
void launch4_intt_export(const CtxDev& c, uint64_t* X, const uint64_t* ct,
                         int ncomp, int comp, int subst_power, CtMap map,
                         int count, int L, cudaStream_t s);
void launch4_digit_ntt(const CtxDev& c, uint64_t* D, const uint64_t* X,
                       const DigitDesc* digits, int k, int digit_flags, int count,
                       int L, cudaStream_t s);
void launch4_modreduce_lift(const CtxDev& c, uint64_t* out, const uint64_t* Y,
                            const uint64_t* in, const ScalarPack& sc, int count,
                            int L, cudaStream_t s);

// Fused four-step encryption tail: NTT of the lifted error err [count][n]
// with the combine of launch_bgv_enc_combine as its sink; buf [count][L][n].
void launch4_bgv_encrypt(const CtxDev& c, uint64_t* out, const int32_t* err,
                         const uint64_t* m, const uint64_t* key, const ScalarPack& tm,
                         uint64_t* buf, int count, int L, cudaStream_t s);

// Fused four-step key switch: launch4_digit_cols runs the digit extraction and
// column phase of every digit transform into D [count][k][L][n];
// launch4_ks_rows runs the row phase of all digits of each (ciphertext, limb)
// together with the key inner product and base add (launch_ks_inner's
// arguments and output).  ks4_rows_per_cta(k) is the number of rows one CTA
// of launch4_ks_rows takes, 0 if k digits do not fit one CTA.
int ks4_rows_per_cta(int k);
void launch4_digit_cols(const CtxDev& c, uint64_t* D, const uint64_t* X,
                        const DigitDesc* digits, int k, int digit_flags, int count,
                        int L, cudaStream_t s);
void launch4_ks_rows(const CtxDev& c, const uint64_t* D, int k, int chunk,
                     const uint64_t* kb, const uint64_t* ka, uint64_t* out,
                     const uint64_t* base, size_t base_ct_elems, CtMap map,
                     int base1_zero, int subst_power, int count, int L,
                     cudaStream_t s, const KeyTable& kt = KeyTable{});

}  // namespace shg
