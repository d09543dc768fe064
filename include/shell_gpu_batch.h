/*
 * shell_gpu_batch.h — uneven-batch executor and autotuner.
 *
 * The reference runs one operation per call (RnsBgvCiphertext::operator* +
 * RnsRelinKey::ApplyTo, RnsBgvCiphertext::Substitute + RnsGaloisKey::ApplyTo,
 * RnsBgvCiphertext::ModReduce; rns/rns_bgv_ciphertext.h:134-170,
 * rns/rns_relinearization_key.cc:184-232, rns/rns_galois_key.cc:238-287).
 * A batch queues many such operations over ciphertexts of different ring
 * degrees, limb counts and keys, each at its own device address, and runs
 * them together: operations are grouped by (context, kind, key, shape); each
 * group's operands are gathered into contiguous scratch by one kernel, run
 * through the batched entry point (shg_bgv_mul_relin, shg_bgv_rotate,
 * shg_poly_modreduce_lsb) with the group's tuned settings, and scattered back
 * by one kernel.  Results are bit-identical to one call per operation.
 *
 * shg_batch_run plans on its first call after operations were added
 * (allocates scratch, uploads pointer tables, synchronizes); later calls only
 * enqueue work, so a second call can be captured into a CUDA graph
 * (shg_graph_capture_begin / _end) and replayed.
 *
 * The autotuner times candidate settings for each group — the transform
 * organisation (one CTA per limb, or the two-phase four-step kernels, for
 * n = 2^12 .. 2^14), the fused or separate key-switch row phase, and the
 * ciphertexts per internal chunk — on the group's own operands, and records
 * the fastest in a process-wide table keyed by (log n, limbs, gadget
 * dimension, kind, count rounded up to a power of two).  shg_batch_run
 * applies the table's entry to each group (and restores the context's
 * settings after it).
 */
#ifndef SHELL_GPU_BATCH_H_
#define SHELL_GPU_BATCH_H_

#include "shell_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shg_batch shg_batch;

enum {
  SHG_OP_MUL_RELIN = 0, /* out = relin(a * b); a, b, out [2][L][n] */
  SHG_OP_ROTATE = 1,    /* out = galois(substitute(ct)); ct, out [2][L][n] */
  SHG_OP_MODREDUCE = 2, /* out [c][L-1][n] = ModReduce(in [c][L][n]) */
};

int shg_batch_create(shg_batch** out);
void shg_batch_destroy(shg_batch* batch);
/* Drops every queued operation (and the plan). */
int shg_batch_clear(shg_batch* batch);
int shg_batch_size(const shg_batch* batch);

/* Queue one operation; every pointer is a 16-byte aligned device pointer to
 * one ciphertext in the layouts above.  The operation's limb count is the
 * key's (mul_relin, rotate) or num_limbs (modreduce). */
int shg_batch_add_mul_relin(shg_batch* batch, shg_context* ctx,
                            const shg_key* relin_key, uint64_t* out,
                            const uint64_t* a, const uint64_t* b);
int shg_batch_add_rotate(shg_batch* batch, shg_context* ctx,
                         const shg_key* galois_key, uint64_t* out,
                         const uint64_t* ct);
/* ql_inv: host array of the num_limbs-1 Montgomery residues of
 * q_{num_limbs-1}^{-1} (shg_context_ql_inv), copied at the call. */
int shg_batch_add_modreduce(shg_batch* batch, shg_context* ctx, uint64_t* out,
                            const uint64_t* in, int num_components,
                            int num_limbs, uint64_t t, const uint64_t* ql_inv);

/* Runs every queued operation on `stream` (see above). */
int shg_batch_run(shg_batch* batch, shg_stream stream);
/* Number of groups of the current plan (0 before the first run). */
int shg_batch_num_groups(const shg_batch* batch);

/* Tunes every group of the batch: `reps` timed runs per candidate after one
 * warm-up run; results go to the process-wide table.  Runs the operations
 * (outputs are written; inputs must not alias outputs). */
int shg_batch_autotune(shg_batch* batch, int reps, shg_stream stream);

/* The tuning table: entries as text lines
 *   log_n num_limbs dimension kind count_bucket chunk four_step_min ks_fused ms */
int shg_tuning_clear(void);
int shg_tuning_size(void);
int shg_tuning_save(const char* path);
int shg_tuning_load(const char* path);
/* Entry for one group shape; SHG_FAILED_PRECONDITION if there is none. */
int shg_tuning_lookup(int log_n, int num_limbs, int dimension, int kind, int count,
                      int* chunk, int* four_step_min, int* ks_fused);

#ifdef __cplusplus
}
#endif
#endif /* SHELL_GPU_BATCH_H_ */
