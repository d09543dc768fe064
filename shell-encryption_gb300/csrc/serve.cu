// Request-serving loop with continuous batching (include/shell_gpu_serve.h).
//
// One server thread owns every CUDA call of the server: it admits submitted
// requests in arrival order while the operand bytes of admitted, unfinished
// requests fit the HBM budget, groups them by (context, operation, key),
// launches a group's batch as soon as the group's stream is idle (or the
// group is full, or its oldest request has waited max_wait_us), and retires
// batches by polling their completion events.  Device operands come from a
// stream-ordered memory pool owned by the server, so allocation never
// synchronizes the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/shell_gpu.h"
#include "../../include/shell_gpu_runtime.h"
#include "../../include/shell_gpu_serve.h"
#include "kernels.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  shg_request r{};
  size_t in_elems = 0, out_elems = 0, bytes = 0;
  int status = SHG_OK;
  bool done = false;
  Clock::time_point t_submit, t_admit, t_launch, t_done;
};

// Requests batch together when they share context, operation and the shape
// of their keys (limbs, gadget, power) -- not the keys themselves: a batch of
// different clients' requests runs through the multi-key entry points.
struct GroupKey {
  shg_context* ctx;
  int kind;
  int power, levels, num_items;
  const uint64_t* db;
  std::vector<int> log_bs;
  bool operator<(const GroupKey& o) const {
    return std::tie(ctx, kind, power, levels, num_items, db, log_bs) <
           std::tie(o.ctx, o.kind, o.power, o.levels, o.num_items, o.db, o.log_bs);
  }
};

GroupKey group_of(const shg_request& r) {
  GroupKey g{r.ctx, r.kind, 0, 0, 0, nullptr, {}};
  const shg_key* k = r.kind == SHG_REQ_EXPAND_ABSORB ? (r.levels ? r.keys[0] : nullptr) : r.key;
  if (k) {
    g.power = shg_key_power(k);
    g.log_bs.resize(shg_key_num_limbs(k));
    shg_key_log_bs(k, g.log_bs.data(), (int)g.log_bs.size());
  }
  if (r.kind == SHG_REQ_EXPAND_ABSORB) {
    g.levels = r.levels;
    g.num_items = r.num_items;
    g.db = r.db;
  }
  return g;
}

struct Batch {
  int stream = 0;
  std::vector<uint64_t> reqs;
  cudaEvent_t done = nullptr;
  size_t bytes = 0;
};

double us_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::micro>(b - a).count();
}

}  // namespace

struct shg_server {
  shg_server_config cfg{};
  std::mutex mu;  // requests, pending, stats
  std::condition_variable cv_work, cv_done;
  std::deque<Req> reqs;
  std::deque<uint64_t> pending;  // submitted, not admitted
  bool stopping = false;
  std::thread thread;
  // Owned by the server thread:
  std::map<GroupKey, std::deque<uint64_t>> ready;  // admitted, not launched
  std::vector<Batch> inflight;
  std::vector<int> inflight_per_stream;
  std::map<shg_context*, int> ctx_stream;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> free_events;
  cudaMemPool_t pool = nullptr;
  size_t bytes_in_flight = 0;
  // Stats (under mu).
  shg_server_stats stats{};
  uint64_t batched_requests = 0;

  void loop();
  bool admit(Clock::time_point now);
  bool launch_ready(Clock::time_point now);
  bool retire(Clock::time_point now);
  void launch(const GroupKey& gk, std::deque<uint64_t>& q, int stream);
  void finish(const std::vector<uint64_t>& ids, int status, Clock::time_point now);
};

namespace {

int validate(const shg_request* r, size_t* in_elems, size_t* out_elems, size_t* bytes) {
  if (!r) return shg::set_error(SHG_INVALID_ARGUMENT, "null request");
  if (!r->ctx) return shg::set_error(SHG_INVALID_ARGUMENT, "null context");
  if (!r->in_a || !r->out || (r->kind == SHG_REQ_MUL_RELIN && !r->in_b))
    return shg::set_error(SHG_INVALID_ARGUMENT, "null host buffer");
  const size_t n = (size_t)1 << shg_context_log_n(r->ctx);
  switch (r->kind) {
    case SHG_REQ_MUL_RELIN:
    case SHG_REQ_ROTATE: {
      if (!r->key || shg_key_context(r->key) != r->ctx)
        return shg::set_error(SHG_INVALID_ARGUMENT, "key does not belong to the context");
      const bool relin = shg_key_power(r->key) == 1;
      if (relin != (r->kind == SHG_REQ_MUL_RELIN))
        return shg::set_error(SHG_INVALID_ARGUMENT,
                              relin ? "rotation needs a Galois key (power != 1)"
                                    : "Relinearization key can only apply to a ciphertext "
                                      "of power 1.");
      *in_elems = *out_elems = 2 * (size_t)shg_key_num_limbs(r->key) * n;
      *bytes = (*in_elems * (r->kind == SHG_REQ_MUL_RELIN ? 2 : 1) + *out_elems) * 8;
      return SHG_OK;
    }
    case SHG_REQ_EXPAND_ABSORB:
      if (!r->keys || !r->db || r->levels < 0 || r->levels >= 31 || r->num_items < 1 ||
          r->num_items > (1 << r->levels))
        return shg::set_error(SHG_INVALID_ARGUMENT, "bad expansion request");
      *in_elems = *out_elems = 2 * n;
      *bytes = (*in_elems + *out_elems) * 8;
      return SHG_OK;
    default:
      return shg::set_error(SHG_INVALID_ARGUMENT, "unknown request kind");
  }
}

}  // namespace

void shg_server::finish(const std::vector<uint64_t>& ids, int status, Clock::time_point now) {
  std::lock_guard<std::mutex> lock(mu);
  for (uint64_t id : ids) {
    Req& q = reqs[id];
    q.status = status;
    q.done = true;
    q.t_done = now;
    bytes_in_flight -= q.bytes;
    if (status == SHG_OK)
      ++stats.completed;
    else
      ++stats.failed;
  }
  cv_done.notify_all();
}

bool shg_server::admit(Clock::time_point now) {
  bool any = false;
  std::lock_guard<std::mutex> lock(mu);
  while (!pending.empty()) {
    Req& q = reqs[pending.front()];
    if (bytes_in_flight + q.bytes > cfg.hbm_budget_bytes) {
      ++stats.admission_waits;
      break;
    }
    bytes_in_flight += q.bytes;
    stats.peak_bytes_in_flight = std::max(stats.peak_bytes_in_flight, bytes_in_flight);
    q.t_admit = now;
    ready[group_of(q.r)].push_back(pending.front());
    pending.pop_front();
    any = true;
  }
  return any;
}

void shg_server::launch(const GroupKey& gk, std::deque<uint64_t>& q, int stream) {
  const int m = std::min<int>((int)q.size(), std::max(1, cfg.max_batch));
  Batch b;
  b.stream = stream;
  for (int i = 0; i < m; ++i) {
    b.reqs.push_back(q.front());
    q.pop_front();
  }
  cudaStream_t s = streams[stream];
  const Clock::time_point now = Clock::now();
  // Element addresses of the request deque are stable (it only grows at the
  // back); its index structure is not, so look them up under the lock.
  std::vector<const shg_request*> rq(m);
  size_t in_e, out_e;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < m; ++i) {
      Req& q = reqs[b.reqs[i]];
      q.t_launch = now;
      b.bytes += q.bytes;
      rq[i] = &q.r;
    }
    in_e = reqs[b.reqs[0]].in_elems;
    out_e = reqs[b.reqs[0]].out_elems;
    ++stats.batches;
    batched_requests += m;
  }
  const shg_request* r0 = rq[0];
  const bool two_inputs = gk.kind == SHG_REQ_MUL_RELIN;
  const size_t elems = (size_t)m * (in_e * (two_inputs ? 2 : 1) + out_e);
  uint64_t* dev = nullptr;
  int st = SHG_OK;
  cudaError_t e = cudaMallocFromPoolAsync((void**)&dev, elems * 8, pool, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    finish(b.reqs, SHG_RESOURCE_EXHAUSTED, Clock::now());
    return;
  }
  uint64_t* da = dev;
  uint64_t* db = two_inputs ? dev + (size_t)m * in_e : nullptr;
  uint64_t* dout = dev + (size_t)m * in_e * (two_inputs ? 2 : 1);
  for (int i = 0; i < m && e == cudaSuccess; ++i) {
    e = cudaMemcpyAsync(da + i * in_e, rq[i]->in_a, in_e * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && two_inputs)
      e = cudaMemcpyAsync(db + i * in_e, rq[i]->in_b, in_e * 8, cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess) {
    // One key for the whole batch when every request names the same one;
    // otherwise per-request keys through the multi-key entry points.
    bool same = true;
    for (int i = 1; i < m && same; ++i)
      same = gk.kind == SHG_REQ_EXPAND_ABSORB ? rq[i]->keys == r0->keys : rq[i]->key == r0->key;
    std::vector<const shg_key*> keys;
    if (!same) {
      if (gk.kind == SHG_REQ_EXPAND_ABSORB) {
        keys.reserve((size_t)m * r0->levels);
        for (int i = 0; i < m; ++i)
          keys.insert(keys.end(), rq[i]->keys, rq[i]->keys + r0->levels);
      } else {
        for (int i = 0; i < m; ++i) keys.push_back(rq[i]->key);
      }
    }
    switch (gk.kind) {
      case SHG_REQ_MUL_RELIN:
        st = same ? shg_bgv_mul_relin(gk.ctx, r0->key, dout, da, db, m, s)
                  : shg_bgv_mul_relin_multikey(gk.ctx, keys.data(), dout, da, db, m, s);
        break;
      case SHG_REQ_ROTATE:
        st = same ? shg_bgv_rotate(gk.ctx, r0->key, dout, da, m, s)
                  : shg_bgv_rotate_multikey(gk.ctx, keys.data(), dout, da, m, s);
        break;
      default:
        st = same ? shg_pir_expand_absorb(gk.ctx, r0->keys, r0->levels, r0->db, r0->num_items,
                                          dout, da, m, s)
                  : shg_pir_expand_absorb_multikey(gk.ctx, keys.data(), r0->levels, r0->db,
                                                   r0->num_items, dout, da, m, s);
        break;
    }
  }
  for (int i = 0; i < m && e == cudaSuccess && st == SHG_OK; ++i)
    e = cudaMemcpyAsync(rq[i]->out, dout + i * out_e, out_e * 8, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(dev, s);
  if (e != cudaSuccess || st != SHG_OK) {
    cudaGetLastError();
    cudaStreamSynchronize(s);
    finish(b.reqs, st != SHG_OK ? st : SHG_INTERNAL, Clock::now());
    return;
  }
  if (free_events.empty()) {
    cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
  } else {
    b.done = free_events.back();
    free_events.pop_back();
  }
  cudaEventRecord(b.done, s);
  ++inflight_per_stream[stream];
  inflight.push_back(std::move(b));
}

bool shg_server::launch_ready(Clock::time_point now) {
  bool any = false;
  for (auto it = ready.begin(); it != ready.end();) {
    auto& q = it->second;
    if (q.empty()) {
      it = ready.erase(it);
      continue;
    }
    auto cs = ctx_stream.find(it->first.ctx);
    if (cs == ctx_stream.end())
      cs = ctx_stream.emplace(it->first.ctx, (int)ctx_stream.size() % (int)streams.size()).first;
    const int stream = cs->second;
    double oldest_us;
    {
      std::lock_guard<std::mutex> lock(mu);
      oldest_us = us_between(reqs[q.front()].t_admit, now);
    }
    const bool idle = inflight_per_stream[stream] == 0;
    if (idle || (int)q.size() >= std::max(1, cfg.max_batch) || oldest_us >= cfg.max_wait_us) {
      launch(it->first, q, stream);
      any = true;
    }
    ++it;
  }
  return any;
}

bool shg_server::retire(Clock::time_point now) {
  bool any = false;
  for (size_t i = 0; i < inflight.size();) {
    Batch& b = inflight[i];
    const cudaError_t e = cudaEventQuery(b.done);
    if (e == cudaErrorNotReady) {
      ++i;
      continue;
    }
    finish(b.reqs, e == cudaSuccess ? SHG_OK : SHG_INTERNAL, now);
    if (e != cudaSuccess) cudaGetLastError();
    --inflight_per_stream[b.stream];
    free_events.push_back(b.done);
    inflight[i] = std::move(inflight.back());
    inflight.pop_back();
    any = true;
  }
  return any;
}

void shg_server::loop() {
  for (;;) {
    const Clock::time_point now = Clock::now();
    bool progress = retire(now);
    progress |= admit(now);
    progress |= launch_ready(now);
    bool idle;
    {
      std::unique_lock<std::mutex> lock(mu);
      idle = pending.empty() && ready.empty() && inflight.empty();
      if (idle && stopping) break;
      if (idle) {
        cv_work.wait_for(lock, std::chrono::milliseconds(2));
        continue;
      }
    }
    if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(5));
  }
}

extern "C" {

int shg_server_create(const shg_server_config* cfg, shg_server** out) {
  if (!cfg || !out) return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  if (cfg->hbm_budget_bytes == 0 || cfg->max_batch < 1 || cfg->max_wait_us < 0 ||
      cfg->num_streams < 1 || cfg->num_streams > 64)
    return shg::set_error(SHG_INVALID_ARGUMENT, "bad server configuration");
  shg_server* sv = new shg_server();
  sv->cfg = *cfg;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaError_t e = cudaMemPoolCreate(&sv->pool, &props);
  if (e == cudaSuccess) {
    uint64_t keep = cfg->hbm_budget_bytes;  // cached bytes kept across batches
    e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < cfg->num_streams && e == cudaSuccess; ++i) {
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) sv->streams.push_back(s);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (cudaStream_t s : sv->streams) cudaStreamDestroy(s);
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    delete sv;
    return shg::set_error(SHG_INTERNAL, std::string("server setup: ") + cudaGetErrorString(e));
  }
  sv->inflight_per_stream.assign(cfg->num_streams, 0);
  sv->thread = std::thread([sv, dev] {
    cudaSetDevice(dev);
    sv->loop();
  });
  *out = sv;
  return SHG_OK;
}

void shg_server_destroy(shg_server* sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->stopping = true;
  }
  sv->cv_work.notify_all();
  sv->thread.join();
  for (cudaEvent_t e : sv->free_events) cudaEventDestroy(e);
  for (cudaStream_t s : sv->streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  cudaMemPoolDestroy(sv->pool);
  delete sv;
}

int shg_server_submit(shg_server* sv, const shg_request* r, uint64_t* ticket) {
  if (!sv || !ticket) return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  size_t in_e = 0, out_e = 0, bytes = 0;
  int st = validate(r, &in_e, &out_e, &bytes);
  if (st) return st;
  if (bytes > sv->cfg.hbm_budget_bytes)
    return shg::set_error(SHG_RESOURCE_EXHAUSTED,
                          "request needs more device memory than the server's budget");
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    if (sv->stopping) return shg::set_error(SHG_FAILED_PRECONDITION, "server is stopping");
    Req q;
    q.r = *r;
    q.in_elems = in_e;
    q.out_elems = out_e;
    q.bytes = bytes;
    q.t_submit = Clock::now();
    *ticket = sv->reqs.size();
    sv->reqs.push_back(std::move(q));
    sv->pending.push_back(*ticket);
    ++sv->stats.submitted;
  }
  sv->cv_work.notify_one();
  return SHG_OK;
}

int shg_server_poll(shg_server* sv, uint64_t ticket, int* done) {
  if (!sv || !done) return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(sv->mu);
  if (ticket >= sv->reqs.size()) return shg::set_error(SHG_INVALID_ARGUMENT, "unknown ticket");
  *done = sv->reqs[ticket].done ? 1 : 0;
  return *done ? sv->reqs[ticket].status : SHG_OK;
}

int shg_server_wait(shg_server* sv, uint64_t ticket, int64_t timeout_us) {
  if (!sv) return shg::set_error(SHG_INVALID_ARGUMENT, "null server");
  std::unique_lock<std::mutex> lock(sv->mu);
  if (ticket >= sv->reqs.size()) return shg::set_error(SHG_INVALID_ARGUMENT, "unknown ticket");
  const bool ok = sv->cv_done.wait_for(lock, std::chrono::microseconds(std::max<int64_t>(0, timeout_us)),
                                       [&] { return sv->reqs[ticket].done; });
  if (!ok) return shg::set_error(SHG_DEADLINE_EXCEEDED, "request still running");
  return sv->reqs[ticket].status;
}

int shg_server_latency(shg_server* sv, uint64_t ticket, double* admit_us, double* launch_us,
                       double* done_us) {
  if (!sv || !admit_us || !launch_us || !done_us)
    return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(sv->mu);
  if (ticket >= sv->reqs.size()) return shg::set_error(SHG_INVALID_ARGUMENT, "unknown ticket");
  const Req& q = sv->reqs[ticket];
  if (!q.done) return shg::set_error(SHG_FAILED_PRECONDITION, "request not finished");
  *admit_us = us_between(q.t_submit, q.t_admit);
  *launch_us = us_between(q.t_submit, q.t_launch);
  *done_us = us_between(q.t_submit, q.t_done);
  return SHG_OK;
}

int shg_server_get_stats(shg_server* sv, shg_server_stats* out) {
  if (!sv || !out) return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(sv->mu);
  *out = sv->stats;
  out->mean_batch = sv->stats.batches ? (double)sv->batched_requests / sv->stats.batches : 0;
  return SHG_OK;
}

int shg_server_replay(shg_server* sv, const shg_request* reqs, const double* arrival_us,
                      int count, uint64_t* tickets) {
  if (!sv || (count > 0 && (!reqs || !arrival_us || !tickets)) || count < 0)
    return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  const Clock::time_point t0 = Clock::now();
  for (int i = 0; i < count; ++i) {
    const Clock::time_point at =
        t0 + std::chrono::duration_cast<Clock::duration>(
                 std::chrono::duration<double, std::micro>(arrival_us[i]));
    for (;;) {
      const Clock::time_point now = Clock::now();
      if (now >= at) break;
      if (at - now > std::chrono::microseconds(200))
        std::this_thread::sleep_for(at - now - std::chrono::microseconds(100));
    }
    const int st = shg_server_submit(sv, &reqs[i], &tickets[i]);
    if (st) return st;
  }
  return SHG_OK;
}

}  // extern "C"
