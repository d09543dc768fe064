// Uneven-batch executor and autotuner (include/shell_gpu_batch.h).
//
// Host-side orchestration over the batched C ABI entry points: operations
// are grouped by (context, kind, key, shape), each group's operands are
// gathered into contiguous scratch by one kernel, the group runs through one
// batched call with its tuned settings, and one kernel scatters the results.
// Groups of different contexts run on different internal streams, forked
// from and joined back into the caller's stream with events, so small groups
// of different ring degrees overlap on the GPU; groups of one context share
// a stream (they share the context's scratch).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/shell_gpu.h"
#include "../../include/shell_gpu_batch.h"
#include "../../include/shell_gpu_runtime.h"
#include "kernels.cuh"

namespace {

constexpr int kStreams = 4;

struct Op {
  int kind;
  shg_context* ctx;
  const shg_key* key;
  uint64_t* out;
  const uint64_t* a;
  const uint64_t* b;
  int ncomp, L;
  uint64_t t;
  std::vector<uint64_t> ql_inv;
};

struct GroupKey {
  shg_context* ctx;
  int kind;
  const shg_key* key;
  int ncomp, L;
  uint64_t t;
  std::vector<uint64_t> ql_inv;
  bool operator<(const GroupKey& o) const {
    return std::tie(ctx, kind, key, ncomp, L, t, ql_inv) <
           std::tie(o.ctx, o.kind, o.key, o.ncomp, o.L, o.t, o.ql_inv);
  }
};

struct Group {
  GroupKey gk;
  std::vector<int> ops;
  int log_n = 0, dim = 0, stream = 0;
  size_t in_elems = 0, out_elems = 0;  // per operation (a and b each; result)
  bool a_contig = false, b_contig = false, out_contig = false;
  size_t tab_a = 0, tab_b = 0, tab_out = 0;  // offsets into the pointer table
  size_t arena_a = 0, arena_b = 0, arena_out = 0;  // offsets into the arena
  int count() const { return (int)ops.size(); }
};

struct Tuning {
  int chunk = 0, four_step_min = 13, ks_fused = 1;
  double ms = 0;
};
using TuneKey = std::tuple<int, int, int, int, int>;  // log_n, L, dim, kind, bucket

std::mutex g_tune_mu;
std::map<TuneKey, Tuning> g_tune;

int bucket(int count) {
  int b = 1;
  while (b < count) b <<= 1;
  return b;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int cuda_error(cudaError_t e, const char* what) {
  return shg::set_error(SHG_INTERNAL, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SHG_BCUDA(call)                                  \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_error(_e, #call); \
  } while (0)

}  // namespace

struct shg_batch {
  std::vector<Op> ops;
  std::vector<Group> groups;
  bool planned = false;
  uint64_t* arena[kStreams] = {};
  size_t arena_elems[kStreams] = {};
  void** d_tables = nullptr;
  cudaStream_t streams[kStreams] = {};
  cudaEvent_t fork = nullptr, join[kStreams] = {};

  void release_plan() {
    if (planned) cudaDeviceSynchronize();
    for (int i = 0; i < kStreams; ++i) {
      cudaFree(arena[i]);
      arena[i] = nullptr;
      arena_elems[i] = 0;
    }
    cudaFree(d_tables);
    d_tables = nullptr;
    groups.clear();
    planned = false;
  }
};

namespace {

int tuning_key_of(const Group& g, TuneKey* k) {
  *k = TuneKey{g.log_n, g.gk.L, g.dim, g.gk.kind, bucket(g.count())};
  return 0;
}

// Applies the table's entry for g (if any) to its context; returns the
// previous settings in *saved.
int apply_tuning(const Group& g, Tuning* saved, bool* applied) {
  *applied = false;
  int st = shg_context_get_tuning(g.gk.ctx, &saved->chunk, &saved->four_step_min,
                                  &saved->ks_fused);
  if (st) return st;
  TuneKey k;
  tuning_key_of(g, &k);
  Tuning t;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(k);
    if (it == g_tune.end()) return SHG_OK;
    t = it->second;
  }
  if ((st = shg_context_set_chunk(g.gk.ctx, t.chunk))) return st;
  if ((st = shg_context_set_four_step_min(g.gk.ctx, t.four_step_min))) return st;
  if ((st = shg_context_set_ks_fused(g.gk.ctx, t.ks_fused))) return st;
  *applied = true;
  return SHG_OK;
}

int restore_tuning(const Group& g, const Tuning& saved) {
  int st = shg_context_set_chunk(g.gk.ctx, saved.chunk);
  if (!st) st = shg_context_set_four_step_min(g.gk.ctx, saved.four_step_min);
  if (!st) st = shg_context_set_ks_fused(g.gk.ctx, saved.ks_fused);
  return st;
}

int plan(shg_batch* b) {
  b->release_plan();
  std::map<GroupKey, int> index;
  std::map<shg_context*, int> ctx_stream;
  for (int i = 0; i < (int)b->ops.size(); ++i) {
    const Op& op = b->ops[i];
    GroupKey gk{op.ctx, op.kind, op.key, op.ncomp, op.L, op.t, op.ql_inv};
    auto it = index.find(gk);
    if (it == index.end()) {
      it = index.emplace(gk, (int)b->groups.size()).first;
      Group g;
      g.gk = gk;
      g.log_n = shg_context_log_n(op.ctx);
      g.dim = op.key ? shg_key_dimension(op.key) : 0;
      auto cs = ctx_stream.find(op.ctx);
      if (cs == ctx_stream.end())
        cs = ctx_stream.emplace(op.ctx, (int)ctx_stream.size() % kStreams).first;
      g.stream = cs->second;
      const size_t n = (size_t)1 << g.log_n;
      if (op.kind == SHG_OP_MODREDUCE) {
        g.in_elems = (size_t)op.ncomp * op.L * n;
        g.out_elems = (size_t)op.ncomp * (op.L - 1) * n;
      } else {
        g.in_elems = 2 * (size_t)op.L * n;
        g.out_elems = 2 * (size_t)op.L * n;
      }
      b->groups.push_back(std::move(g));
    }
    b->groups[it->second].ops.push_back(i);
  }
  // Contiguity, arena regions (per stream; groups of a stream run in turn)
  // and pointer tables.
  std::vector<void*> tables;
  for (Group& g : b->groups) {
    const Op& o0 = b->ops[g.ops[0]];
    g.a_contig = g.b_contig = g.out_contig = true;
    for (int j = 0; j < g.count(); ++j) {
      const Op& o = b->ops[g.ops[j]];
      g.a_contig &= o.a == o0.a + j * g.in_elems;
      if (g.gk.kind == SHG_OP_MUL_RELIN) g.b_contig &= o.b == o0.b + j * g.in_elems;
      g.out_contig &= o.out == o0.out + j * g.out_elems;
    }
    size_t need = 0;
    auto add_table = [&](size_t* off, auto getter) {
      *off = tables.size();
      for (int j = 0; j < g.count(); ++j) tables.push_back((void*)getter(b->ops[g.ops[j]]));
    };
    if (!g.a_contig) {
      g.arena_a = need;
      need += g.count() * g.in_elems;
      add_table(&g.tab_a, [](const Op& o) { return o.a; });
    }
    if (g.gk.kind == SHG_OP_MUL_RELIN && !g.b_contig) {
      g.arena_b = need;
      need += g.count() * g.in_elems;
      add_table(&g.tab_b, [](const Op& o) { return o.b; });
    }
    if (!g.out_contig) {
      g.arena_out = need;
      need += g.count() * g.out_elems;
      add_table(&g.tab_out, [](const Op& o) { return o.out; });
    }
    b->arena_elems[g.stream] = std::max(b->arena_elems[g.stream], need);
  }
  for (int i = 0; i < kStreams; ++i) {
    if (b->arena_elems[i] == 0) continue;
    cudaError_t e = cudaMalloc(&b->arena[i], b->arena_elems[i] * sizeof(uint64_t));
    if (e != cudaSuccess) {
      cudaGetLastError();
      b->release_plan();
      return shg::set_error(SHG_RESOURCE_EXHAUSTED,
                            std::string("batch scratch: ") + cudaGetErrorString(e));
    }
  }
  if (!tables.empty()) {
    SHG_BCUDA(cudaMalloc(&b->d_tables, tables.size() * sizeof(void*)));
    SHG_BCUDA(cudaMemcpy(b->d_tables, tables.data(), tables.size() * sizeof(void*),
                         cudaMemcpyHostToDevice));
  }
  for (int i = 0; i < kStreams; ++i) {
    if (!b->streams[i]) SHG_BCUDA(cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking));
    if (!b->join[i]) SHG_BCUDA(cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming));
  }
  if (!b->fork) SHG_BCUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  b->planned = true;
  return SHG_OK;
}

// Operand pointers of group g in contiguous form (arena or the caller's).
struct GroupBufs {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* out;
};

GroupBufs bufs_of(const shg_batch* b, const Group& g) {
  const Op& o0 = b->ops[g.ops[0]];
  uint64_t* ar = b->arena[g.stream];
  return GroupBufs{g.a_contig ? o0.a : ar + g.arena_a,
                   g.gk.kind != SHG_OP_MUL_RELIN ? nullptr
                                                  : (g.b_contig ? o0.b : ar + g.arena_b),
                   g.out_contig ? o0.out : ar + g.arena_out};
}

void gather(const shg_batch* b, const Group& g, const GroupBufs& gb, cudaStream_t s) {
  if (!g.a_contig)
    shg::launch_gather(const_cast<uint64_t*>(gb.a),
                       reinterpret_cast<const uint64_t* const*>(b->d_tables + g.tab_a),
                       g.in_elems, g.count(), s);
  if (g.gk.kind == SHG_OP_MUL_RELIN && !g.b_contig)
    shg::launch_gather(const_cast<uint64_t*>(gb.b),
                       reinterpret_cast<const uint64_t* const*>(b->d_tables + g.tab_b),
                       g.in_elems, g.count(), s);
}

void scatter(const shg_batch* b, const Group& g, const GroupBufs& gb, cudaStream_t s) {
  if (!g.out_contig)
    shg::launch_scatter(reinterpret_cast<uint64_t* const*>(b->d_tables + g.tab_out), gb.out,
                        g.out_elems, g.count(), s);
}

int run_op(const Group& g, const GroupBufs& gb, cudaStream_t s) {
  switch (g.gk.kind) {
    case SHG_OP_MUL_RELIN:
      return shg_bgv_mul_relin(g.gk.ctx, g.gk.key, gb.out, gb.a, gb.b, g.count(), s);
    case SHG_OP_ROTATE:
      return shg_bgv_rotate(g.gk.ctx, g.gk.key, gb.out, gb.a, g.count(), s);
    default:
      return shg_poly_modreduce_lsb(g.gk.ctx, gb.out, gb.a, g.gk.t, g.gk.ql_inv.data(), 1,
                                    g.count() * g.gk.ncomp, g.gk.L, s);
  }
}

int add_op(shg_batch* b, Op op) {
  if (!b) return shg::set_error(SHG_INVALID_ARGUMENT, "null batch");
  if (!op.ctx) return shg::set_error(SHG_INVALID_ARGUMENT, "null context");
  for (const void* p : {(const void*)op.out, (const void*)op.a})
    if (!p || !aligned16(p))
      return shg::set_error(SHG_INVALID_ARGUMENT, "buffers must be non-null and 16-byte aligned");
  if (op.kind == SHG_OP_MUL_RELIN && (!op.b || !aligned16(op.b)))
    return shg::set_error(SHG_INVALID_ARGUMENT, "buffers must be non-null and 16-byte aligned");
  if (op.out == op.a || (op.b && op.out == op.b))
    return shg::set_error(SHG_INVALID_ARGUMENT, "`out` must not alias an input");
  b->ops.push_back(std::move(op));
  b->planned = false;
  return SHG_OK;
}

int check_key(shg_context* ctx, const shg_key* key, bool relin) {
  if (!key) return shg::set_error(SHG_INVALID_ARGUMENT, "null key");
  if (shg_key_context(key) != ctx)
    return shg::set_error(SHG_INVALID_ARGUMENT, "key belongs to another context");
  if (relin != (shg_key_power(key) == 1))
    return shg::set_error(SHG_INVALID_ARGUMENT,
                          relin ? "Relinearization key can only apply to a ciphertext of power 1."
                                : "rotation needs a Galois key (power != 1)");
  return SHG_OK;
}

}  // namespace

extern "C" {

int shg_batch_create(shg_batch** out) {
  if (!out) return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  *out = new shg_batch();
  return SHG_OK;
}

void shg_batch_destroy(shg_batch* b) {
  if (!b) return;
  b->release_plan();
  for (int i = 0; i < kStreams; ++i) {
    if (b->streams[i]) cudaStreamDestroy(b->streams[i]);
    if (b->join[i]) cudaEventDestroy(b->join[i]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  delete b;
}

int shg_batch_clear(shg_batch* b) {
  if (!b) return shg::set_error(SHG_INVALID_ARGUMENT, "null batch");
  b->release_plan();
  b->ops.clear();
  return SHG_OK;
}

int shg_batch_size(const shg_batch* b) { return b ? (int)b->ops.size() : 0; }
int shg_batch_num_groups(const shg_batch* b) {
  return b && b->planned ? (int)b->groups.size() : 0;
}

int shg_batch_add_mul_relin(shg_batch* b, shg_context* ctx, const shg_key* key, uint64_t* out,
                            const uint64_t* a, const uint64_t* bb) {
  int st = check_key(ctx, key, true);
  if (st) return st;
  return add_op(b, Op{SHG_OP_MUL_RELIN, ctx, key, out, a, bb, 2, shg_key_num_limbs(key), 0, {}});
}

int shg_batch_add_rotate(shg_batch* b, shg_context* ctx, const shg_key* key, uint64_t* out,
                         const uint64_t* ct) {
  int st = check_key(ctx, key, false);
  if (st) return st;
  return add_op(b, Op{SHG_OP_ROTATE, ctx, key, out, ct, nullptr, 2, shg_key_num_limbs(key), 0, {}});
}

int shg_batch_add_modreduce(shg_batch* b, shg_context* ctx, uint64_t* out, const uint64_t* in,
                            int num_components, int num_limbs, uint64_t t,
                            const uint64_t* ql_inv) {
  if (!ctx) return shg::set_error(SHG_INVALID_ARGUMENT, "null context");
  if (num_components <= 0)
    return shg::set_error(SHG_INVALID_ARGUMENT, "`num_components` must be positive.");
  if (num_limbs <= 1 || num_limbs > shg_context_num_moduli(ctx))
    return shg::set_error(
        SHG_FAILED_PRECONDITION,
        "Cannot perform ModReduce with insufficient number of prime moduli.");
  if (!ql_inv)
    return shg::set_error(SHG_INVALID_ARGUMENT,
                          "`ql_inv` must be defined with respect to " +
                              std::to_string(num_limbs - 1) + " moduli.");
  if (t == 0) return shg::set_error(SHG_INVALID_ARGUMENT, "`t` must be positive.");
  return add_op(b, Op{SHG_OP_MODREDUCE, ctx, nullptr, out, in, nullptr, num_components,
                      num_limbs, t, std::vector<uint64_t>(ql_inv, ql_inv + num_limbs - 1)});
}

int shg_batch_run(shg_batch* b, shg_stream stream) {
  if (!b) return shg::set_error(SHG_INVALID_ARGUMENT, "null batch");
  if (b->ops.empty()) return SHG_OK;
  int st;
  if (!b->planned && (st = plan(b))) return st;
  cudaStream_t user = (cudaStream_t)stream;
  SHG_BCUDA(cudaEventRecord(b->fork, user));
  bool used[kStreams] = {};
  for (const Group& g : b->groups) used[g.stream] = true;
  for (int i = 0; i < kStreams; ++i)
    if (used[i]) SHG_BCUDA(cudaStreamWaitEvent(b->streams[i], b->fork, 0));
  for (const Group& g : b->groups) {
    cudaStream_t s = b->streams[g.stream];
    const GroupBufs gb = bufs_of(b, g);
    gather(b, g, gb, s);
    Tuning saved;
    bool applied = false;
    if ((st = apply_tuning(g, &saved, &applied))) return st;
    st = run_op(g, gb, s);
    if (applied) {
      const int st2 = restore_tuning(g, saved);
      if (!st) st = st2;
    }
    if (st) return st;
    scatter(b, g, gb, s);
  }
  for (int i = 0; i < kStreams; ++i) {
    if (!used[i]) continue;
    SHG_BCUDA(cudaEventRecord(b->join[i], b->streams[i]));
    SHG_BCUDA(cudaStreamWaitEvent(user, b->join[i], 0));
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "batch run");
  return SHG_OK;
}

int shg_batch_autotune(shg_batch* b, int reps, shg_stream stream) {
  if (!b) return shg::set_error(SHG_INVALID_ARGUMENT, "null batch");
  if (reps < 1) return shg::set_error(SHG_INVALID_ARGUMENT, "`reps` must be positive.");
  if (b->ops.empty()) return SHG_OK;
  int st;
  if (!b->planned && (st = plan(b))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  SHG_BCUDA(cudaEventCreate(&e0));
  SHG_BCUDA(cudaEventCreate(&e1));
  std::map<TuneKey, bool> done;  // groups that share a table entry are tuned once
  for (const Group& g : b->groups) {
    TuneKey gkey;
    tuning_key_of(g, &gkey);
    if (done.count(gkey)) continue;
    done[gkey] = true;
    const GroupBufs gb = bufs_of(b, g);
    gather(b, g, gb, s);
    Tuning saved;
    if ((st = shg_context_get_tuning(g.gk.ctx, &saved.chunk, &saved.four_step_min,
                                     &saved.ks_fused)))
      break;
    auto time_cfg = [&](Tuning& c) -> int {
      int r = shg_context_set_chunk(g.gk.ctx, c.chunk);
      if (!r) r = shg_context_set_four_step_min(g.gk.ctx, c.four_step_min);
      if (!r) r = shg_context_set_ks_fused(g.gk.ctx, c.ks_fused);
      if (!r) r = run_op(g, gb, s);  // warm-up (sizes scratch)
      if (r) return r;
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_error(cudaGetLastError(), "tune");
      cudaEventRecord(e0, s);
      for (int i = 0; i < reps && !r; ++i) r = run_op(g, gb, s);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) return cuda_error(cudaGetLastError(), "tune");
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      c.ms = ms / reps;
      return r;
    };
    Tuning best = saved;
    if ((st = time_cfg(best))) break;
    auto consider = [&](Tuning c) -> int {
      const int r = time_cfg(c);
      if (!r && c.ms < best.ms) best = c;
      return r;
    };
    // Transform organisation: one CTA per limb or the four-step kernels.
    if (g.log_n >= 12 && g.log_n <= 14) {
      Tuning c = best;
      c.four_step_min = best.four_step_min <= g.log_n ? 16 : g.log_n;
      if ((st = consider(c))) break;
    }
    const bool four_step = g.log_n >= best.four_step_min || g.log_n > 14;
    if (g.gk.kind != SHG_OP_MODREDUCE) {
      if (four_step && g.log_n >= 12) {
        Tuning c = best;
        c.ks_fused = 1 - best.ks_fused;
        if ((st = consider(c))) break;
      }
      for (int ch : {4, 8, 16, 32}) {
        if (ch > std::max(4, g.count()) || ch == best.chunk) continue;
        Tuning c = best;
        c.chunk = ch;
        if ((st = consider(c))) break;
      }
      if (st) break;
    }
    if ((st = restore_tuning(g, saved))) break;
    TuneKey k;
    tuning_key_of(g, &k);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[k] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

int shg_tuning_clear(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.clear();
  return SHG_OK;
}

int shg_tuning_size(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  return (int)g_tune.size();
}

int shg_tuning_save(const char* path) {
  if (!path) return shg::set_error(SHG_INVALID_ARGUMENT, "null path");
  std::ofstream f(path);
  if (!f) return shg::set_error(SHG_INVALID_ARGUMENT, std::string("cannot write ") + path);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (const auto& kv : g_tune) {
    const auto& k = kv.first;
    const Tuning& t = kv.second;
    f << std::get<0>(k) << ' ' << std::get<1>(k) << ' ' << std::get<2>(k) << ' '
      << std::get<3>(k) << ' ' << std::get<4>(k) << ' ' << t.chunk << ' '
      << t.four_step_min << ' ' << t.ks_fused << ' ' << t.ms << '\n';
  }
  return f ? SHG_OK : shg::set_error(SHG_INTERNAL, "write failed");
}

int shg_tuning_load(const char* path) {
  if (!path) return shg::set_error(SHG_INVALID_ARGUMENT, "null path");
  std::ifstream f(path);
  if (!f) return shg::set_error(SHG_INVALID_ARGUMENT, std::string("cannot read ") + path);
  std::map<TuneKey, Tuning> loaded;
  std::string line;
  int lineno = 0;
  while (std::getline(f, line)) {
    ++lineno;
    if (line.empty()) continue;
    std::istringstream is(line);
    int log_n, L, dim, kind, bkt;
    Tuning t;
    if (!(is >> log_n >> L >> dim >> kind >> bkt >> t.chunk >> t.four_step_min >> t.ks_fused >>
          t.ms) ||
        log_n < 1 || L < 1 || kind < 0 || kind > 2 || t.chunk < 0 || t.four_step_min < 12 ||
        t.four_step_min > 16 || (t.ks_fused != 0 && t.ks_fused != 1))
      return shg::set_error(SHG_INVALID_ARGUMENT,
                            "malformed tuning line " + std::to_string(lineno));
    loaded[TuneKey{log_n, L, dim, kind, bkt}] = t;
  }
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (const auto& kv : loaded) g_tune[kv.first] = kv.second;
  return SHG_OK;
}

int shg_tuning_lookup(int log_n, int num_limbs, int dimension, int kind, int count, int* chunk,
                      int* four_step_min, int* ks_fused) {
  if (!chunk || !four_step_min || !ks_fused)
    return shg::set_error(SHG_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(TuneKey{log_n, num_limbs, dimension, kind, bucket(count)});
  if (it == g_tune.end()) return shg::set_error(SHG_FAILED_PRECONDITION, "no tuning entry");
  *chunk = it->second.chunk;
  *four_step_min = it->second.four_step_min;
  *ks_fused = it->second.ks_fused;
  return SHG_OK;
}

}  // extern "C"
