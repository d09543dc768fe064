/*
 * shell_gpu_serve.h — request-serving loop with continuous batching.
 *
 * A server owns one host thread that admits requests (ct-mult+relin,
 * rotation, PIR expand+absorb — the reference's RnsBgvCiphertext::operator*
 * + RnsRelinKey::ApplyTo, RnsBgvCiphertext::Substitute +
 * RnsGaloisKey::ApplyTo, and GaloisKeysObliviousExpander::ObliviousExpand +
 * FusedAbsorbAddInPlace) as they arrive, while earlier batches run:
 *
 *  - admission by HBM footprint: a request enters only while the device
 *    bytes of all admitted, unfinished requests' operands stay within
 *    hbm_budget_bytes (first come, first served);
 *  - continuous batching: admitted requests wait in groups of identical
 *    (context, operation, key); a group launches as soon as its context's
 *    stream is idle, or when it holds max_batch requests, or when its oldest
 *    request has waited max_wait_us, so requests that arrive while others
 *    are on the GPU join the next batch;
 *  - overlap: each context runs on one of num_streams streams (its scratch is
 *    per context), so batches of different parameter sets overlap;
 *  - a batch copies its requests' host inputs into stream-ordered device
 *    memory, runs one batched call and copies each result back to its host
 *    output.
 *
 * Keys and contexts are created by the caller and stay resident; requests
 * name them.  Results are bit-identical to one call per request.  Waits are
 * bounded: shg_server_wait returns SHG_DEADLINE_EXCEEDED after its timeout.
 */
#ifndef SHELL_GPU_SERVE_H_
#define SHELL_GPU_SERVE_H_

#include "shell_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { SHG_DEADLINE_EXCEEDED = 4 };

enum {
  SHG_REQ_MUL_RELIN = 0,     /* in_a, in_b, out: [2][L][n] host */
  SHG_REQ_ROTATE = 1,        /* in_a, out: [2][L][n] host; key = Galois key */
  SHG_REQ_EXPAND_ABSORB = 2, /* in_a, out: [2][n] host; keys/levels/db/num_items */
};

typedef struct shg_server shg_server;

typedef struct {
  size_t hbm_budget_bytes; /* device bytes of admitted requests' operands */
  int max_batch;           /* requests per launch (1 = one call per request) */
  int max_wait_us;         /* partial-batch deadline when the stream is busy */
  int num_streams;         /* concurrent streams (contexts are spread over them) */
} shg_server_config;

typedef struct {
  int kind;
  shg_context* ctx;
  const shg_key* key;          /* relinearization or Galois key */
  const shg_key* const* keys;  /* expand: one Galois key per level */
  int levels;                  /* expand */
  const uint64_t* db;          /* expand: device [num_items][n], NTT form */
  int num_items;               /* expand */
  const uint64_t* in_a;        /* host */
  const uint64_t* in_b;        /* host (mul_relin) */
  uint64_t* out;               /* host */
} shg_request;

typedef struct {
  uint64_t submitted, completed, failed, batches;
  double mean_batch;             /* requests per launched batch */
  size_t peak_bytes_in_flight;   /* admitted operand bytes, high-water mark */
  uint64_t admission_waits;      /* times the head request did not fit */
} shg_server_stats;

int shg_server_create(const shg_server_config* config, shg_server** out);
/* Finishes every submitted request, then stops the thread and frees. */
void shg_server_destroy(shg_server* server);
/* Queues a request (host buffers must stay valid until it completes; page-
 * locked memory lets the copies run asynchronously). */
int shg_server_submit(shg_server* server, const shg_request* request, uint64_t* ticket);
/* *done = 1 once the request finished; its status is the return value then. */
int shg_server_poll(shg_server* server, uint64_t ticket, int* done);
/* Waits at most timeout_us for the request; SHG_DEADLINE_EXCEEDED if it is
 * still running, else its status. */
int shg_server_wait(shg_server* server, uint64_t ticket, int64_t timeout_us);
/* Microseconds from submission to admission, to launch and to completion. */
int shg_server_latency(shg_server* server, uint64_t ticket, double* admit_us,
                       double* launch_us, double* done_us);
int shg_server_get_stats(shg_server* server, shg_server_stats* out);
/* Open-loop load generator: submits requests[i] when arrival_us[i]
 * (non-decreasing, from the call's start) has passed, on the calling
 * thread, and returns after the last submission; tickets[i] receives each
 * ticket. */
int shg_server_replay(shg_server* server, const shg_request* requests,
                      const double* arrival_us, int count, uint64_t* tickets);

#ifdef __cplusplus
}
#endif
#endif /* SHELL_GPU_SERVE_H_ */
