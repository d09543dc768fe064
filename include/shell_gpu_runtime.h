/*
 * shell_gpu_runtime.h — device-memory, stream, event and graph plumbing for
 * callers of shell_gpu.h that do not link the CUDA runtime themselves (the
 * Python tests and benchmark use these through ctypes).  These have no
 * counterpart in google/shell-encryption, which is CPU-only.
 */
#ifndef SHELL_GPU_RUNTIME_H_
#define SHELL_GPU_RUNTIME_H_

#include <stddef.h>
#include <stdint.h>

#include "shell_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

int shg_device_count(int* count);
int shg_set_device(int device);
int shg_device_alloc(size_t bytes, void** out);
int shg_device_free(void* ptr);
int shg_host_alloc(size_t bytes, void** out); /* page-locked */
int shg_host_free(void* ptr);
int shg_memcpy_h2d(void* dst, const void* src, size_t bytes, shg_stream stream);
int shg_memcpy_d2h(void* dst, const void* src, size_t bytes, shg_stream stream);
int shg_memcpy_d2d(void* dst, const void* src, size_t bytes, shg_stream stream);
int shg_memset_device(void* dst, int value, size_t bytes, shg_stream stream);
int shg_stream_create(shg_stream* out);
int shg_stream_destroy(shg_stream stream);
int shg_stream_synchronize(shg_stream stream);
int shg_device_synchronize(void);
int shg_event_create(void** out);
int shg_event_destroy(void* event);
int shg_event_record(void* event, shg_stream stream);
int shg_event_elapsed_ms(void* start, void* stop, float* ms);
/* Stream capture into a CUDA graph and replay. */
int shg_graph_capture_begin(shg_stream stream);
int shg_graph_capture_end(shg_stream stream, void** graph_exec);
int shg_graph_launch(void* graph_exec, shg_stream stream);
int shg_graph_destroy(void* graph_exec);
/* Number of kernels launched by this library so far (host-side count of
 * launch calls; graph replays are not counted). */
uint64_t shg_launch_count(void);
/* Per-kernel timing: between start and stop every launch of this library is
 * bracketed by CUDA events on its own stream; stop synchronizes the device
 * and accumulates.  query returns the total milliseconds and launch count of
 * one kernel family ("ntt_fwd", "ntt_inv", "digit_ntt", "ks_inner",
 * "tensor_intt", "intt_export", "pointwise", ...). */
/* Butterflies per second of the NTT's lazy Cooley-Tukey butterfly on
 * register-resident values, measured on the current device (about 0.1 s of
 * GPU time): the integer-pipe ceiling of every transform kernel. */
int shg_measure_butterfly_rate(double* per_second);
int shg_profile_start(void);
int shg_profile_stop(void);
int shg_profile_query(const char* kernel, double* total_ms, uint64_t* launches);
/* Reserve scratch space for batched calls up front (so a later call can be
 * captured into a graph without allocating). */
int shg_context_reserve(shg_context* ctx, size_t bytes);
/* Ciphertexts per internal chunk of the batched key-switch pipeline
 * (0 = default). */
int shg_context_set_chunk(shg_context* ctx, int cts_per_chunk);
/* Transforms of n >= 2^log_n use the two-kernel four-step NTT, log_n in
 * [12, 16] (13 = default; 12 also moves n = 2^12 off the one-CTA-per-limb
 * kernels; 14 or more keeps smaller n on them; n = 2^15 always uses the
 * four-step kernels).  Plain shg_ntt_forward / shg_ntt_inverse calls use the
 * four-step kernels from n = 2^12 at 12 and 13, and follow higher values. */
int shg_context_set_four_step_min(shg_context* ctx, int log_n);
/* 1 (default): four-step key switches run the digit row phase and the key
 * inner product as one kernel; 0: separate row phase, digit NTTs written to
 * scratch, then the inner product.  Results are identical. */
int shg_context_set_ks_fused(shg_context* ctx, int on);
/* Index checks of a debug build (no counterpart in the reference; the
 * library compiled with SHG_DEBUG, see __graft_entry__.build_debug).  Debug
 * kernels check computed indices before they address memory (substitution
 * gathers, per-member key tables, gadget digit descriptors, limb indices);
 * a failing check records its tag (1 substitution, 2 key table, 3 digit,
 * 4 limb), the index is replaced by 0 so nothing faults, and the call goes
 * on.  Reads and clears the current device's records: *first_failure = 0 when
 * no check failed.  A release build always reports 0. */
int shg_debug_status(unsigned* first_failure);
/* Streams the chunks of a batched ct-mult+relin rotate over, 1 to 4 (2 =
 * default: the caller's stream and a second one, so one chunk fills the
 * other's tail; 1 = the caller's stream only, e.g. to time kernels one at a
 * time).  Each lane holds its own chunk of digit scratch. */
int shg_context_set_ks_lanes(shg_context* ctx, int lanes);
/* shg_bgv_mul_relin_host pipeline shape: ciphertexts per piece (default 32)
 * and device staging slots in flight (default 4, at most 8). */
int shg_context_set_host_pipeline(shg_context* ctx, int piece_cts, int slots);
/* shg_bgv_mul_relin_host piece ramp: with ramp r > 0 the first and last
 * pieces hold piece_cts >> r ciphertexts, doubling towards the middle, so the
 * pipeline fills and drains in short steps; 0 = every piece full (default 2,
 * at most 16). */
int shg_context_set_host_ramp(shg_context* ctx, int ramp);
/* Current values of the three settings above (chunk 0 = default). */
int shg_context_get_tuning(const shg_context* ctx, int* chunk_cts, int* four_step_min,
                           int* ks_fused);
/* Seeded synthetic data: polys [count][num_limbs][n] <- uniform residues,
 * element e = splitmix64 output e + 1 of state `seed` mod its limb's prime
 * (the generator of the test suite's oracle.uniform_limbs). */
int shg_poly_fill_uniform(shg_context* ctx, uint64_t* polys, int count, int num_limbs,
                          uint64_t seed, shg_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* SHELL_GPU_RUNTIME_H_ */
