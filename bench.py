#!/usr/bin/env python3
"""Benchmark: RNS BGV ct x ct multiply + relinearization on one GB300.

Workload (the reference's ct-mult+relin configuration): ring degree n = 2^14,
six 45-bit NTT primes (the largest below 2^45 that are 1 mod 2^15), t = 65537,
gadget base 2^20 (dimension 18), 1024 seeded ciphertext pairs per step.

One step = RnsBgvCiphertext::operator* + RnsRelinKey::ApplyTo on all 1024
pairs.  `value` is the batched path (shg_bgv_mul_relin, replayed from a CUDA
graph) with inputs resident in HBM; `e2e` is the same call fed from pinned
host buffers with the host->device and device->host copies inside the timed
region; `plain` is the one-call-per-op drop-in path (shg_ct_tensor +
shg_relin_apply per ciphertext).  Every path is bit-exact with the CPU
reference (tests/test_gpu_parity.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "shell-encryption_gb300")
sys.path.insert(0, PKG)

LOG_N = 14
QS = [35184371138561, 35184370941953, 35184370352129, 35184370155521,
      35184369893377, 35184368877569]
T_PLAIN = 65537
LOG_BS = [20] * 6
METRIC = "RNS ct-mult+relin/sec (batched vs plain, same GPU, bit-exact); p50/p99 ms"
UNIT = "ct-mult+relin/s"
# DRAM bytes (read + write) per ciphertext of each kernel scope, from ncu
# captures of the same kernels (dram__bytes_read.sum + dram__bytes_write.sum
# of one 16-ciphertext launch); None where not captured.
TRAFFIC_PER_CT = {
    "ks_rows": (300.8e6 + 20.6e6) / 16,     # k4_ks_rows_warp
    "digit_cols": (12.7e6 + 169.2e6) / 16,  # k4_digit_cols_all
}
# What bounds those kernels instead: the FMA-heavy pipe (the IMAD family,
# every 32 x 32-bit partial product of the 64-bit modular arithmetic), from
# the same ncu capture (sm__pipe_fmaheavy_cycles_active, one 16-ciphertext
# launch).
MULPIPE_BUSY = {
    "ks_rows": 0.772,     # k4_ks_rows_warp
    "digit_cols": 0.761,  # k4_digit_cols_all
}
# Kernel scopes the library times (shg_profile_query) in one ct-mult+relin
# step; the four-step key switch runs digit_cols + ks_rows, the unfused one
# digit_ntt + ks_inner.
SCOPES = ("tensor_intt", "digit_cols", "ks_rows", "digit_ntt", "ks_inner")


def scope_model(name, n, L, k, cts):
    """(algorithmic DRAM bytes, butterflies) of one launch over `cts` ciphertexts.

    Bytes count each operand once: tensor_intt reads both inputs and writes
    (c0, c1) and the plain c2 (7 polys); the digit kernels read c2 and write
    the k digit transforms; the inner-product kernels read the digit
    transforms, the base and write the result (k + 4 polys) plus the key once.
    """
    poly = L * n * 8
    bfly_ntt = n // 2 * (n.bit_length() - 1)
    if name == "tensor_intt":
        return 7 * poly * cts, L * bfly_ntt * cts
    if name == "digit_ntt":
        return (1 + k) * poly * cts, k * L * bfly_ntt * cts
    if name == "digit_cols":
        return (1 + k) * poly * cts, k * L * (n // 2) * (n.bit_length() - 1 - 7) * cts
    if name == "ks_rows":
        return (k + 4) * poly * cts + 2 * k * poly, k * L * (n // 2) * 7 * cts
    if name == "ks_inner":
        return (k + 4) * poly * cts + 2 * k * poly, 0
    raise KeyError(name)


def config(batch):
    return {
        "workload": "bgv-ct-mult-relin n=2^14 L=6x45-bit t=65537 gadget 2^20 (k=18)",
        "log_n": LOG_N, "num_limbs": len(QS), "log_q": 45, "gadget_log_base": 20,
        "gadget_dim": 18, "batch": batch,
        "l2": "inputs larger than L2 (each step reads 3.2 GB of ciphertexts)",
        "parallelism": "replicas",
    }


def splitmix_limbs(seed, count, qs, n):
    """Seeded uniform residues [count][len(qs)][n] (splitmix64 stream)."""
    L = len(qs)
    with np.errstate(over="ignore"):
        idx = np.arange(1, count * L * n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z.reshape(count, L, n) % np.array(qs, np.uint64).reshape(1, L, 1))


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # plumbing only: barrier and max-reduce
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def host_link_ms(h2d_bytes, d2h_bytes, rates):
    """Fastest time (ms) for one step's copies on the host link, from probed
    rates (GB/s: "h2d" and "d2h" one way, "duplex" [h2d, d2h] both ways at
    once): both directions run side by side at the both-ways rates until the
    shorter one is done, and the rest of the longer one runs alone at its
    one-way rate."""
    up, down = rates["duplex"]
    t_in, t_out = h2d_bytes / (up * 1e6), d2h_bytes / (down * 1e6)
    t_both = min(t_in, t_out)
    if t_in >= t_out:
        return t_both + (h2d_bytes - up * 1e6 * t_both) / (rates["h2d"] * 1e6)
    return t_both + (d2h_bytes - down * 1e6 * t_both) / (rates["d2h"] * 1e6)


def warm_link(step, sync, min_calls, seconds=1.0):
    """Untimed warm-up of a host-buffer leg: at least `min_calls` calls and at
    least `seconds` of them.  After a second or two without host-link traffic
    (device-only work, or idle) the first copies run at about 10 GB/s for some
    0.3 s before the link returns to its steady 211 / 193 GB/s (measured on
    the GB300 machines), so a few calls alone can leave the timing on the slow
    start."""
    t0 = time.perf_counter()
    i = 0
    while i < min_calls or time.perf_counter() - t0 < seconds:
        step()
        sync()
        i += 1


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons in the background."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(seconds, threads, seed=7):
    """The reference's CPU path (oracle restatement of ct x ct +
    relinearization) on `threads` host threads, one ciphertext pair per
    thread per round, repeated for about `seconds`: returns (ops/s, ops, s)."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    n = 1 << LOG_N
    rns = O.Rns(LOG_N, QS)
    k = rns.gadget_dim(LOG_BS)
    kb = splitmix_limbs(seed + 2, k, QS, n)
    ka = splitmix_limbs(seed + 3, k, QS, n)
    a = splitmix_limbs(seed, 2 * threads, QS, n).reshape(threads, 2, len(QS), n)
    b = splitmix_limbs(seed + 1, 2 * threads, QS, n).reshape(threads, 2, len(QS), n)
    ops = 0
    t0 = time.perf_counter()
    while True:
        rns.mul_relin_batch(a, b, kb, ka, LOG_BS, threads=threads)
        ops += threads
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return ops / dt, ops, dt


def run_reference(args, world, rank, dist):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per_step = []
    ops_total = 0
    for i in range(args.warmup + args.steps):
        rate, ops, dt = cpu_reference(2.0, threads, seed=100 + i)
        if i >= args.warmup:
            per_step.append(dt)
            ops_total += ops
    total = sum(per_step)
    value = ops_total / total
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": dict(config(threads), batch=threads),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: about 2 s of ct-mult+relin at n=2^14, L=6, "
                                   f"one ciphertext pair per host thread per round",
                         "single_thread_ms_per_op": 1e3 / cpu_reference(1.0, 1, seed=99)[0]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# PIR workload: oblivious expansion + database absorb (n = 2^12, one 60-bit
# prime, 10 levels, gadget base 2^8, 256 queries, 2^10-item database).
# ---------------------------------------------------------------------------

PIR_LOG_N, PIR_Q, PIR_LEVELS, PIR_LOG_B = 12, 1152921504606830593, 10, 8
PIR_QUERIES, PIR_ITEMS, PIR_LOG_T = 256, 1024, 16
PIR_METRIC = "PIR oblivious expansion + absorb queries/sec (n=2^12, 10 levels, 2^10 items)"
PIR_UNIT = "queries/s"
PIR_SCOPES = ("monomials", "ntt_fwd", "intt_export", "digit_ntt", "ks_inner", "digit_cols",
              "ks_rows", "expand_combine", "absorb_sum")


def pir_config(queries):
    return {
        "workload": "pir-expand-absorb n=2^12 q=60-bit gadget 2^8 (dim 8) 10 levels, "
                    "2^10-item database",
        "log_n": PIR_LOG_N, "log_q": 60, "levels": PIR_LEVELS, "gadget_log_base": PIR_LOG_B,
        "gadget_dim": 8, "queries": queries, "db_items": PIR_ITEMS,
        "l2": "expanded ciphertexts per step (16 GiB) exceed L2",
        "parallelism": "replicas",
    }


def pir_scope_model(name, n, dim, members, queries, levels):
    """(algorithmic DRAM bytes, butterflies) of one whole step of a scope:
    members = key switches (every non-root node of every query's tree)."""
    poly = n * 8
    bfly = n // 2 * (n.bit_length() - 1)
    if name == "monomials":
        return levels * poly, 0
    if name == "ntt_fwd":
        return 2 * levels * poly, levels * bfly
    if name == "intt_export":
        return 2 * poly * members, bfly * members
    if name == "digit_ntt":
        return (1 + dim) * poly * members, dim * bfly * members
    if name == "digit_cols":
        return (1 + dim) * poly * members, dim * (n // 2) * (n.bit_length() - 1 - 7) * members
    if name == "ks_rows":
        return (dim + 3) * poly * members, dim * (n // 2) * 7 * members
    if name == "ks_inner":
        return (dim + 3) * poly * members, 0
    if name == "expand_combine":
        return 8 * poly * members, 0
    if name == "absorb_sum":
        return (PIR_ITEMS * 2 + 2) * poly * queries + PIR_ITEMS * poly, 0
    raise KeyError(name)


def pir_keys_db_queries(seed, n, queries):
    dim = -(-60 // PIR_LOG_B)
    keys = np.stack([np.stack([splitmix_limbs(seed + 10 * j + c, dim, [PIR_Q], n).reshape(dim, n)
                               for c in (0, 1)]) for j in range(PIR_LEVELS)])
    with np.errstate(over="ignore"):
        db_plain = (splitmix_limbs(seed + 999, PIR_ITEMS, [1 << 62], n).reshape(PIR_ITEMS, n)
                    & np.uint64((1 << PIR_LOG_T) - 1))
    q = splitmix_limbs(seed + 555, 2 * queries, [PIR_Q], n).reshape(queries, 2, n)
    return dim, keys, db_plain, q


def cpu_pir(seconds, threads, seed=7):
    """The reference's CPU path for one PIR query (oracle restatement of
    GaloisKeysObliviousExpander::ObliviousExpand + FusedAbsorbAddInPlace),
    one query per host thread per round, for about `seconds`."""
    import concurrent.futures
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    n = 1 << PIR_LOG_N
    p = O.Prime(PIR_Q, PIR_LOG_N)
    dim, keys, db_plain, q = pir_keys_db_queries(seed, n, threads)
    db = np.stack([p.ntt_fwd(p.import_(row)) for row in db_plain])

    def one(i):
        return p.absorb_sum(p.oblivious_expand(PIR_LEVELS, PIR_LOG_B, keys, q[i]), db)

    ops = 0
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        while True:
            list(ex.map(one, range(threads)))
            ops += threads
            dt = time.perf_counter() - t0
            if dt >= seconds:
                break
    return ops / dt, ops, dt


def run_pir_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per_step, ops_total = [], 0
    for i in range(args.warmup + args.steps):
        _, ops, dt = cpu_pir(2.0, threads, seed=100 + i)
        if i >= args.warmup:
            per_step.append(dt)
            ops_total += ops
    total = sum(per_step)
    value = ops_total / total
    print(json.dumps({
        "metric": PIR_METRIC, "value": value, "unit": PIR_UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": pir_config(threads),
        "cpu_baseline": {"value": value, "unit": PIR_UNIT, "cores": threads, "kind": "port",
                         "sample": "each step: about 2 s of whole queries, one per host "
                                   "thread per round"},
        "e2e": {"value": value, "unit": PIR_UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_pir(args, world, rank, local, dist):
    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    n = 1 << PIR_LOG_N
    Qn = args.queries
    ctx = sg.Context(PIR_LOG_N, [PIR_Q], (1 << PIR_LOG_T) + 1)
    # The expansion's key switches (8 digits of one 60-bit prime at n = 2^12)
    # measured 9.6 % faster on the four-step kernels with the fused row phase.
    sg.check(lib.shg_context_set_four_step_min(ctx.h, args.four_step_min or 12))
    if args.ks_unfused:
        sg.check(lib.shg_context_set_ks_fused(ctx.h, 0))
    dim, keys, db_plain, queries = pir_keys_db_queries(3000 + 97 * rank, n, Qn)
    gkeys = [sg.Key(ctx, [PIR_LOG_B], (n >> j) + 1, keys[j, 0], keys[j, 1])
             for j in range(PIR_LEVELS)]
    karr = (ctypes.c_void_p * PIR_LEVELS)(*[k.h for k in gkeys])
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value
    # Database rows: plaintexts in [0, 2^16) imported to Montgomery form
    # (times R^2 mod q through a Montgomery multiply) and put in NTT form.
    d_db = sg.DeviceBuffer.from_array(db_plain)
    r2 = np.array([pow(2, 128, PIR_Q)], np.uint64)
    sg.check(lib.shg_poly_mul_rns_scalar(ctx.h, d_db.ptr, d_db.ptr,
                                         r2.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                         PIR_ITEMS, 1, s))
    sg.check(lib.shg_ntt_forward(ctx.h, d_db.ptr, PIR_ITEMS, 1, s))
    q_bytes = Qn * 2 * n * 8

    def host(nbytes):
        p = ctypes.c_void_p()
        sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    h_q, h_out = host(q_bytes), host(q_bytes)
    np.ctypeslib.as_array((ctypes.c_uint64 * (Qn * 2 * n)).from_address(h_q))[:] = queries.reshape(-1)
    d_q, d_out = sg.DeviceBuffer(q_bytes), sg.DeviceBuffer(q_bytes)
    sg.check(lib.shg_memcpy_h2d(d_q.ptr, h_q, q_bytes, s))

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b, ctypes.byref(ms)))
        return ms.value

    def step_device():
        sg.check(lib.shg_pir_expand_absorb(ctx.h, karr, PIR_LEVELS, d_db.ptr, PIR_ITEMS,
                                           d_out.ptr, d_q.ptr, Qn, s))

    step_device()
    sg.check(lib.shg_stream_synchronize(s))
    n0 = lib.shg_launch_count()
    sg.check(lib.shg_graph_capture_begin(s))
    step_device()
    g = ctypes.c_void_p()
    sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
    graph = g.value
    launches_per_step = lib.shg_launch_count() - n0
    for _ in range(args.warmup):
        sg.check(lib.shg_graph_launch(graph, s))
    sg.check(lib.shg_stream_synchronize(s))
    evs = [ev() for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    sg.check(lib.shg_event_record(evs[0], s))
    for i in range(args.steps):
        sg.check(lib.shg_graph_launch(graph, s))
        sg.check(lib.shg_event_record(evs[i + 1], s))
    sg.check(lib.shg_stream_synchronize(s))
    barrier(dist)
    clk = clocks.stop()
    step_ms = [elapsed(evs[i], evs[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(dist, elapsed(evs[0], evs[-1]))
    ops_all = sum_over_ranks(dist, float(Qn * args.steps))
    value = ops_all / (total_ms / 1e3)

    # End to end: queries in from pinned host memory, results back, per step.
    e2e = None
    if not args.no_e2e:
        def step_e2e():
            sg.check(lib.shg_memcpy_h2d(d_q.ptr, h_q, q_bytes, s))
            step_device()
            sg.check(lib.shg_memcpy_d2h(h_out, d_out.ptr, q_bytes, s))
        warm_link(step_e2e, lambda: sg.check(lib.shg_stream_synchronize(s)),
                  max(3, args.warmup))
        e0, e1 = ev(), ev()
        barrier(dist)
        sg.check(lib.shg_event_record(e0, s))
        for _ in range(args.steps):
            step_e2e()
        sg.check(lib.shg_event_record(e1, s))
        sg.check(lib.shg_stream_synchronize(s))
        e2e_ms = max_over_ranks(dist, elapsed(e0, e1))
        e2e = {"value": ops_all / (e2e_ms / 1e3), "unit": PIR_UNIT,
               "h2d_bytes_per_step": q_bytes, "d2h_bytes_per_step": q_bytes,
               "ms_per_step": e2e_ms / args.steps}

    sg.check(lib.shg_profile_start())
    step_device()
    sg.check(lib.shg_profile_stop())
    prof = {}
    for name in PIR_SCOPES:
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        sg.check(lib.shg_profile_query(name.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        if cnt.value:
            prof[name] = (ms.value, cnt.value)
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    bfly_peak = ctypes.c_double()
    sg.check(lib.shg_measure_butterfly_rate(ctypes.byref(bfly_peak)))
    members = Qn * ((1 << PIR_LEVELS) - 1)
    step_total = sum(v[0] for v in prof.values())
    kernels, bfly_step, bfly_ms = {}, 0.0, 0.0
    for name, (ms, cnt) in prof.items():
        nbytes, bfly = pir_scope_model(name, n, dim, members, Qn, PIR_LEVELS)
        kernels[name] = {"share_of_step": ms / step_total, "launches": cnt,
                         "avg_launch_ms": ms / cnt,
                         "algorithmic_bytes_per_launch": nbytes / cnt,
                         "achieved_gbs": nbytes / (ms / 1e3) / 1e9,
                         "int_frac": (bfly / (ms / 1e3) / bfly_peak.value) if bfly else None}
        if bfly:
            bfly_step += bfly
            bfly_ms += ms
    top = max(prof, key=lambda nm: prof[nm][0])
    tk = kernels[top]
    roofline = {
        "kernel": top, "bound": "hbm", "achieved": tk["achieved_gbs"], "peak": peak,
        "unit": "GB/s", "frac": tk["achieved_gbs"] / peak, "peak_source": peak_src,
        "traffic": None, "algorithmic_bytes_per_launch": tk["algorithmic_bytes_per_launch"],
        "avg_launch_ms": tk["avg_launch_ms"],
        "integer": {"peak_butterflies_per_s": bfly_peak.value,
                    "achieved_butterflies_per_s": bfly_step / (bfly_ms / 1e3),
                    "frac": bfly_step / (bfly_ms / 1e3) / bfly_peak.value},
        "kernels": kernels,
    }
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, ops, dt = cpu_pir(10.0, threads)
        cpu = {"value": rate, "unit": PIR_UNIT, "cores": threads, "kind": "port",
               "sample": f"{ops} queries (expand to 2^10 + absorb) in {dt:.1f} s, "
                         f"one query per host thread per round"}
    lat = sorted(step_ms)
    line = {
        "metric": PIR_METRIC, "value": value, "unit": PIR_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform keys, queries and a 2^16-valued database)",
        "config": pir_config(Qn),
        "expanded_ciphertexts_per_s": value * (1 << PIR_LEVELS),
        "key_switches_per_s": value * ((1 << PIR_LEVELS) - 1),
        "latency_ms": {"step_p50": lat[len(lat) // 2], "step_p99": lat[-1]},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sg.check(lib.shg_graph_destroy(graph))
    for hp in (h_q, h_out):
        lib.shg_host_free(hp)


# ---------------------------------------------------------------------------
# Uneven batch: 4096 instances, n in {2^11..2^15}, 1..12 limbs of 50-bit
# primes, 70% ct-mult+relin / 20% rotation / 10% modulus switch, run through
# the batch executor (autotuned, graph-replayed) vs one call per operation.
# ---------------------------------------------------------------------------

Q50 = [1125899904679937, 1125899903827969, 1125899903500289, 1125899903107073,
       1125899902124033, 1125899901665281, 1125899899174913, 1125899896160257,
       1125899887312897, 1125899886395393, 1125899885740033, 1125899885412353]
UNEVEN_METRIC = "uneven batch ops/sec (n 2^11..2^15, 1..12 limbs; 70% ct-mult+relin, " \
                "20% rotation, 10% ModReduce)"
UNEVEN_UNIT = "ops/s"
UNEVEN_LOG_B = 20


def uneven_instances(count, seed):
    """Seeded instance list: (log_n, limbs, kind, galois exponent j)."""
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(count):
        log_n = rng.randint(11, 15)
        L = rng.randint(1, 12)
        r = rng.random()
        kind = 0 if r < 0.7 else (1 if r < 0.9 else 2)
        while kind == 2 and L == 1:
            L = rng.randint(1, 12)
        out.append((log_n, L, kind, rng.randint(1, 8)))
    return out


def uneven_config(count):
    return {"workload": "uneven-batch n=2^11..2^15 L=1..12 x 50-bit, gadget 2^20, "
                        "70/20/10 ct-mult+relin/rotation/ModReduce, Galois powers 5^j mod 2n, "
                        "j in 1..8",
            "instances": count, "gadget_log_base": UNEVEN_LOG_B,
            "l2": "operands per step exceed L2 by far", "parallelism": "replicas"}


def run_uneven(args, world, rank, local, dist):
    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    inst = uneven_instances(args.instances, 4242 + rank)
    shapes = sorted({(ln, L) for ln, L, _, _ in inst})
    ctxs, relin, galois = {}, {}, {}
    pools = {}
    for ln, L in shapes:
        n = 1 << ln
        if ln not in pools:
            Lmax = max(l2 for l1, l2 in shapes if l1 == ln)
            kmax = 3 * Lmax
            pools[ln] = (splitmix_limbs(9000 + ln, kmax, Q50[:Lmax], n),
                         splitmix_limbs(9100 + ln, kmax, Q50[:Lmax], n))
        pb, pa = pools[ln]
        ctx = sg.Context(ln, Q50[:L])
        ctxs[(ln, L)] = ctx
        k = 3 * L
        kb = np.ascontiguousarray(pb[:k, :L])
        ka = np.ascontiguousarray(pa[:k, :L])
        used = {(kind, j) for l1, l2, kind, j in inst if (l1, l2) == (ln, L)}
        if any(kind == 0 for kind, _ in used):
            relin[(ln, L)] = sg.Key(ctx, [UNEVEN_LOG_B] * L, 1, kb, ka)
        for kind, j in used:
            if kind == 1 and (ln, L, j) not in galois:
                galois[(ln, L, j)] = sg.Key(ctx, [UNEVEN_LOG_B] * L, pow(5, j, 2 * n), kb, ka)
    # Operands: inputs in one region, outputs in another, each instance at a
    # shuffled position (a group's operands are not adjacent).
    import random
    rng = random.Random(77 + rank)
    order = list(range(len(inst)))
    rng.shuffle(order)
    in_off, out_off, pos_in, pos_out = 0, 0, {}, {}
    for i in order:
        ln, L, kind, _ = inst[i]
        ct = 2 * L * (1 << ln) * 8
        pos_in[i] = in_off
        in_off += ct * (2 if kind == 0 else 1)
        pos_out[i] = out_off
        out_off += ct
    d_in, d_out = sg.DeviceBuffer(in_off), sg.DeviceBuffer(out_off)
    for i, (ln, L, kind, _) in enumerate(inst):
        cts = 2 if kind == 0 else 1
        sg.check(lib.shg_poly_fill_uniform(ctxs[(ln, L)].h, d_in.ptr + pos_in[i], 2 * cts, L,
                                           500000 + i, None))
    ql = {key: ctxs[key].ql_inv(key[1] - 1) for key in ctxs if key[1] > 1}
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value
    b = ctypes.c_void_p()
    sg.check(lib.shg_batch_create(ctypes.byref(b)))
    u64p = ctypes.POINTER(ctypes.c_uint64)

    def per_op(i):
        ln, L, kind, j = inst[i]
        ctx = ctxs[(ln, L)]
        a = d_in.ptr + pos_in[i]
        o = d_out.ptr + pos_out[i]
        ct = 2 * L * (1 << ln) * 8
        if kind == 0:
            return lib.shg_bgv_mul_relin(ctx.h, relin[(ln, L)].h, o, a, a + ct, 1, s)
        if kind == 1:
            return lib.shg_bgv_rotate(ctx.h, galois[(ln, L, j)].h, o, a, 1, s)
        return lib.shg_poly_modreduce_lsb(ctx.h, o, a, 65537, ql[(ln, L)].ctypes.data_as(u64p),
                                          1, 2, L, s)

    for i, (ln, L, kind, j) in enumerate(inst):
        ctx = ctxs[(ln, L)]
        a = d_in.ptr + pos_in[i]
        o = d_out.ptr + pos_out[i]
        ct = 2 * L * (1 << ln) * 8
        if kind == 0:
            sg.check(lib.shg_batch_add_mul_relin(b, ctx.h, relin[(ln, L)].h, o, a, a + ct))
        elif kind == 1:
            sg.check(lib.shg_batch_add_rotate(b, ctx.h, galois[(ln, L, j)].h, o, a))
        else:
            sg.check(lib.shg_batch_add_modreduce(b, ctx.h, o, a, 2, L, 65537,
                                                 ql[(ln, L)].ctypes.data_as(u64p)))

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b2):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b2, ctypes.byref(ms)))
        return ms.value

    # Plain: one call per operation (also the reference result).
    for i in range(len(inst)):
        sg.check(per_op(i))
    sg.check(lib.shg_stream_synchronize(s))
    e0, e1 = ev(), ev()
    sg.check(lib.shg_event_record(e0, s))
    for i in range(len(inst)):
        sg.check(per_op(i))
    sg.check(lib.shg_event_record(e1, s))
    sg.check(lib.shg_stream_synchronize(s))
    plain_ms = elapsed(e0, e1)
    ref_out = np.empty(out_off // 8, np.uint64)
    sg.check(lib.shg_memcpy_d2h(ref_out.ctypes.data, d_out.ptr, out_off, s))
    sg.check(lib.shg_memset_device(d_out.ptr, 0, out_off, s))

    # Batched: plan + autotune (untimed), capture, replay.
    sg.check(lib.shg_batch_run(b, s))
    sg.check(lib.shg_stream_synchronize(s))
    t0 = time.perf_counter()
    if not args.no_autotune:
        sg.check(lib.shg_batch_autotune(b, 2, s))
    tune_s = time.perf_counter() - t0
    sg.check(lib.shg_batch_run(b, s))
    sg.check(lib.shg_stream_synchronize(s))
    n0 = lib.shg_launch_count()
    sg.check(lib.shg_graph_capture_begin(s))
    sg.check(lib.shg_batch_run(b, s))
    g = ctypes.c_void_p()
    sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
    graph = g.value
    launches_per_step = lib.shg_launch_count() - n0
    for _ in range(args.warmup):
        sg.check(lib.shg_graph_launch(graph, s))
    sg.check(lib.shg_stream_synchronize(s))
    evs = [ev() for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    sg.check(lib.shg_event_record(evs[0], s))
    for i in range(args.steps):
        sg.check(lib.shg_graph_launch(graph, s))
        sg.check(lib.shg_event_record(evs[i + 1], s))
    sg.check(lib.shg_stream_synchronize(s))
    barrier(dist)
    clk = clocks.stop()
    total_ms = max_over_ranks(dist, elapsed(evs[0], evs[-1]))
    ops_all = sum_over_ranks(dist, float(len(inst) * args.steps))
    value = ops_all / (total_ms / 1e3)
    got = np.empty(out_off // 8, np.uint64)
    sg.check(lib.shg_memcpy_d2h(got.ctypes.data, d_out.ptr, out_off, s))
    sg.check(lib.shg_stream_synchronize(s))
    bit_exact = bool(np.array_equal(got, ref_out))

    e2e = None
    if not args.no_e2e:
        def host(nbytes):
            p = ctypes.c_void_p()
            sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
            return p.value
        h_in, h_out = host(in_off), host(out_off)
        sg.check(lib.shg_memcpy_d2h(h_in, d_in.ptr, in_off, s))
        sg.check(lib.shg_stream_synchronize(s))

        def step_e2e():
            sg.check(lib.shg_memcpy_h2d(d_in.ptr, h_in, in_off, s))
            sg.check(lib.shg_graph_launch(graph, s))
            sg.check(lib.shg_memcpy_d2h(h_out, d_out.ptr, out_off, s))
        warm_link(step_e2e, lambda: sg.check(lib.shg_stream_synchronize(s)),
                  max(3, args.warmup))
        x0, x1 = ev(), ev()
        barrier(dist)
        sg.check(lib.shg_event_record(x0, s))
        for _ in range(args.steps):
            step_e2e()
        sg.check(lib.shg_event_record(x1, s))
        sg.check(lib.shg_stream_synchronize(s))
        e2e_ms = max_over_ranks(dist, elapsed(x0, x1))
        e2e = {"value": ops_all / (e2e_ms / 1e3), "unit": UNEVEN_UNIT,
               "h2d_bytes_per_step": in_off, "d2h_bytes_per_step": out_off,
               "ms_per_step": e2e_ms / args.steps}
        lib.shg_host_free(h_in)
        lib.shg_host_free(h_out)
    kinds = [x[2] for x in inst]
    line = {
        "metric": UNEVEN_METRIC, "value": value, "unit": UNEVEN_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded instances, uniform residues, keys from seeded pools)",
        "config": uneven_config(len(inst)),
        "mix": {"ct_mult_relin": kinds.count(0), "rotation": kinds.count(1),
                "modreduce": kinds.count(2), "contexts": len(ctxs),
                "galois_keys": len(galois), "groups": lib.shg_batch_num_groups(b)},
        "plain": {"value": len(inst) / (plain_ms / 1e3), "unit": UNEVEN_UNIT,
                  "path": "one per-op C ABI call per instance"},
        "batched_over_plain": (value / world) / (len(inst) / (plain_ms / 1e3)),
        "bit_exact_batched_vs_plain": bit_exact,
        "autotune": {"seconds": tune_s, "entries": lib.shg_tuning_size(),
                     "enabled": not args.no_autotune},
        "e2e": e2e, "gpu_launches": int(launches_per_step * args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sg.check(lib.shg_graph_destroy(graph))
    lib.shg_batch_destroy(b)


# ---------------------------------------------------------------------------
# Serving: Poisson arrivals from 64 clients with resident keys; parameter sets
# (n, limbs) in {(2^12, 2), (2^13, 3), (2^14, 6), (2^15, 12)} of 50-bit primes;
# 70% ct-mult+relin, 20% rotation, 10% PIR expand+absorb; served with
# continuous batching vs one call per request.
# ---------------------------------------------------------------------------

SERVE_PARAMS = [(12, 2), (13, 3), (14, 6), (15, 12)]
SERVE_METRIC = "served requests/sec (continuous batching, Poisson arrivals; p50/p99/p999 ms)"
SERVE_UNIT = "req/s"


def serve_config(clients, rates, seconds):
    return {"workload": "serving: Poisson arrivals, 64 clients, (n, limbs) in "
                        "{(2^12,2),(2^13,3),(2^14,6),(2^15,12)} x 50-bit, 70% ct-mult+relin, "
                        "20% rotation, 10% PIR expand+absorb (n=2^12, 10 levels)",
            "clients": clients, "rates_req_s": rates, "arrival_seconds": seconds,
            "parallelism": "replicas"}


def run_serve(args, world, rank, local, dist):
    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    rates = [int(r) for r in args.rates.split(",")]
    clients = args.clients
    ctxs, keys = {}, {}
    for ln, L in SERVE_PARAMS:
        n = 1 << ln
        ctx = sg.Context(ln, Q50[:L])
        ctxs[(ln, L)] = ctx
        k = 3 * L
        kb = splitmix_limbs(9300 + ln, k, Q50[:L], n)
        ka = splitmix_limbs(9400 + ln, k, Q50[:L], n)
        for c in range(clients):
            keys[(c, ln, L, 0)] = sg.Key(ctx, [UNEVEN_LOG_B] * L, 1, kb, ka)
            keys[(c, ln, L, 1)] = sg.Key(ctx, [UNEVEN_LOG_B] * L, 5, kb, ka)
    # PIR: one context, a shared database, per-client expansion keys.
    pn = 1 << PIR_LOG_N
    pctx = sg.Context(PIR_LOG_N, [PIR_Q], (1 << PIR_LOG_T) + 1)
    sg.check(lib.shg_context_set_four_step_min(pctx.h, 12))  # as in the pir workload
    dim, pkeys, db_plain, _ = pir_keys_db_queries(3000, pn, 1)
    d_db = sg.DeviceBuffer.from_array(db_plain)
    r2 = np.array([pow(2, 128, PIR_Q)], np.uint64)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    sg.check(lib.shg_poly_mul_rns_scalar(pctx.h, d_db.ptr, d_db.ptr, r2.ctypes.data_as(u64p),
                                         PIR_ITEMS, 1, None))
    sg.check(lib.shg_ntt_forward(pctx.h, d_db.ptr, PIR_ITEMS, 1, None))
    pir_keys, pir_arr = {}, {}
    for c in range(clients):
        pir_keys[c] = [sg.Key(pctx, [PIR_LOG_B], (pn >> j) + 1, pkeys[j, 0], pkeys[j, 1])
                       for j in range(PIR_LEVELS)]
        pir_arr[c] = (ctypes.c_void_p * PIR_LEVELS)(*[kk.h for kk in pir_keys[c]])

    def host(nbytes):
        p = ctypes.c_void_p()
        sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    # Pinned host operands: two input ciphertexts per parameter set (read
    # only, shared) and a ring of output slots per parameter set.
    RING = 64
    bufs = {}
    for ln, L in SERVE_PARAMS:
        ct = 2 * L * (1 << ln) * 8
        a, b = host(ct), host(ct)
        for hp, seed in ((a, 11), (b, 12)):
            view = np.ctypeslib.as_array((ctypes.c_uint64 * (ct // 8)).from_address(hp))
            view[:] = splitmix_limbs(seed + ln, 2, Q50[:L], 1 << ln).reshape(-1)
        bufs[(ln, L)] = (a, b, [host(ct) for _ in range(RING)])
    pq = host(2 * pn * 8)
    np.ctypeslib.as_array((ctypes.c_uint64 * (2 * pn)).from_address(pq))[:] = \
        splitmix_limbs(555, 2, [PIR_Q], pn).reshape(-1)
    pouts = [host(2 * pn * 8) for _ in range(RING)]

    def requests(rate, seed):
        rng = np.random.default_rng(seed)
        count = max(1, int(rate * args.seconds))
        gaps = rng.exponential(1e6 / rate, count)
        arrival = np.cumsum(gaps) - gaps[0]
        arr = (sg.Request * count)()
        kinds = np.zeros(count, np.int32)
        for i in range(count):
            c = int(rng.integers(clients))
            r = rng.random()
            kind = 0 if r < 0.7 else (1 if r < 0.9 else 2)
            kinds[i] = kind
            q = arr[i]
            if kind == 2:
                q.kind, q.ctx, q.keys, q.levels = 2, pctx.h, pir_arr[c], PIR_LEVELS
                q.db, q.num_items, q.in_a, q.out = d_db.ptr, PIR_ITEMS, pq, pouts[i % RING]
                continue
            ln, L = SERVE_PARAMS[int(rng.integers(len(SERVE_PARAMS)))]
            a, b, outs = bufs[(ln, L)]
            q.kind, q.ctx, q.key = kind, ctxs[(ln, L)].h, keys[(c, ln, L, kind)].h
            q.in_a, q.in_b, q.out = a, b, outs[i % RING]
        return arr, (ctypes.c_double * count)(*arrival.tolist()), kinds

    def serve(rate, max_batch, streams, seed):
        cfg = sg.ServerConfig(args.hbm_budget_gb << 30, max_batch, args.max_wait_us, streams)
        sv = ctypes.c_void_p()
        sg.check(lib.shg_server_create(ctypes.byref(cfg), ctypes.byref(sv)))
        reqs, arrival, kinds = requests(rate, seed)
        count = len(reqs)
        tickets = (ctypes.c_uint64 * count)()
        t0 = time.perf_counter()
        sg.check(lib.shg_server_replay(sv, reqs, arrival, count, tickets))
        for i in range(count):
            sg.check(lib.shg_server_wait(sv, tickets[i], 600_000_000))
        wall = time.perf_counter() - t0
        lat = np.empty(count)
        a_, l_, d_ = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        end = 0.0
        for i in range(count):
            sg.check(lib.shg_server_latency(sv, tickets[i], ctypes.byref(a_), ctypes.byref(l_),
                                            ctypes.byref(d_)))
            lat[i] = d_.value
            end = max(end, arrival[i] + d_.value)
        st = sg.ServerStats()
        sg.check(lib.shg_server_get_stats(sv, ctypes.byref(st)))
        lib.shg_server_destroy(sv)
        ms = lat / 1e3

        def pct(p):
            return float(np.percentile(ms, p))
        res = {"offered_req_s": rate, "requests": count,
               "throughput_req_s": count / (end / 1e6), "wall_s": wall,
               "p50_ms": pct(50), "p99_ms": pct(99), "p999_ms": pct(99.9),
               "by_kind_p50_ms": {k: float(np.percentile(ms[kinds == i], 50))
                                  for i, k in enumerate(["ct_mult_relin", "rotation", "pir"])
                                  if np.any(kinds == i)},
               "mean_batch": st.mean_batch, "batches": st.batches,
               "peak_gb_in_flight": st.peak_bytes_in_flight / 2**30,
               "admission_waits": st.admission_waits, "failed": st.failed}
        return res

    serve(1000, 16, args.streams, 1)  # warm-up: scratch, pools, code paths
    sweep, plain = [], []
    for i, rate in enumerate(rates):
        sweep.append(serve(rate, args.max_batch, args.streams, 100 + i))
        plain.append(serve(rate, 1, 1, 100 + i))
    clk = {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled for the serving sweep"]}
    top = sweep[-1]
    line = {
        "metric": SERVE_METRIC, "value": top["throughput_req_s"], "unit": SERVE_UNIT,
        "n_gpus": world, "steps": len(rates), "warmup": 1,
        "ms_per_step": 1e3 * top["wall_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded Poisson arrivals, uniform ciphertexts, pooled key material)",
        "config": serve_config(clients, rates, args.seconds),
        "latency_ms": {"p50": top["p50_ms"], "p99": top["p99_ms"], "p999": top["p999_ms"]},
        "sweep": sweep, "plain_per_request": plain,
        "served_over_plain_at_top_rate": top["throughput_req_s"] / plain[-1]["throughput_req_s"],
        "e2e": {"value": top["throughput_req_s"], "unit": SERVE_UNIT,
                "note": "requests carry host buffers; copies in and out are inside every "
                        "request's latency"},
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Encryption: RnsRlweSecretKey::EncryptPolynomialBgv with the randomness drawn
# on the device from SHELL's ChaCha PRNG (one 32-byte seed per ciphertext),
# n = 2^14, the six 45-bit primes, variance 8, 1024 ciphertexts per step.
# ---------------------------------------------------------------------------

ENC_METRIC = "BGV encryptions/sec (EncryptPolynomialBgv, ChaCha sampling on the device, " \
             "bit-exact)"
ENC_UNIT = "encryptions/s"
ENC_VARIANCE = 8
ENC_SCOPES = ("sample_uniform_error", "bgv_encrypt_ntt", "error_lift", "ntt_fwd",
              "bgv_enc_combine")


def enc_config(count):
    return {"workload": "bgv-encrypt n=2^14 6x45-bit primes t=65537 variance 8",
            "log_n": LOG_N, "log_q": 45, "limbs": len(QS), "variance": ENC_VARIANCE,
            "ciphertexts": count, "l2": "plaintexts and ciphertexts per step (2.4 GB) exceed L2",
            "parallelism": "replicas"}


def enc_scope_model(name, n, L, cts):
    """(algorithmic DRAM bytes, ChaCha keystream bytes) of one step of a scope."""
    poly = L * n * 8
    if name == "sample_uniform_error":
        # c1 out plus the int32 error coefficients; keystream: the uniform
        # words plus 4 bytes per error coefficient at variance 8
        return (poly + n * 4) * cts, (L * n * 8 + n * 4) * cts
    if name == "bgv_encrypt_ntt":
        # error in, plaintext and c1 in, c0 out (the transform scratch stays in L2)
        return (n * 4 + 3 * poly) * cts, 0
    if name == "error_lift":
        return (n * 4 + poly) * cts, 0
    if name == "ntt_fwd":
        return 2 * poly * cts, 0
    if name == "bgv_enc_combine":
        return 4 * poly * cts, 0
    raise KeyError(name)


def cpu_encrypt(seconds, threads, seed=7):
    """The reference's CPU encryption (oracle restatement of
    EncryptPolynomialBgv with the ChaCha PRNG), one ciphertext per host thread
    per round, for about `seconds`."""
    import concurrent.futures
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    n = 1 << LOG_N
    L = len(QS)
    rns = O.Rns(LOG_N, QS)
    key = splitmix_limbs(seed, 1, QS, n).reshape(L, n)
    m = splitmix_limbs(seed + 1, threads, QS, n).reshape(threads, L, n)

    def one(i):
        return rns.encrypt_bgv(T_PLAIN, ENC_VARIANCE, key, m[i], bytes([i % 256] * 32))

    ops = 0
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        while True:
            list(ex.map(one, range(threads)))
            ops += threads
            dt = time.perf_counter() - t0
            if dt >= seconds:
                break
    return ops / dt, ops, dt


def run_encrypt_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per_step, ops_total = [], 0
    for i in range(args.warmup + args.steps):
        _, ops, dt = cpu_encrypt(2.0, threads, seed=100 + i)
        if i >= args.warmup:
            per_step.append(dt)
            ops_total += ops
    total = sum(per_step)
    value = ops_total / total
    print(json.dumps({
        "metric": ENC_METRIC, "value": value, "unit": ENC_UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": enc_config(threads),
        "cpu_baseline": {"value": value, "unit": ENC_UNIT, "cores": threads, "kind": "port",
                         "sample": "each step: about 2 s of whole encryptions, one per host "
                                   "thread per round"},
        "e2e": {"value": value, "unit": ENC_UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_encrypt(args, world, rank, local, dist):
    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    n = 1 << LOG_N
    L = len(QS)
    B = args.batch
    ctx = sg.Context(LOG_N, QS, T_PLAIN)
    if args.four_step_min:
        sg.check(lib.shg_context_set_four_step_min(ctx.h, args.four_step_min))
    if args.chunk:
        sg.check(lib.shg_context_set_chunk(ctx.h, args.chunk))
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value
    key = splitmix_limbs(4000 + rank, 1, QS, n).reshape(L, n)
    d_key = sg.DeviceBuffer.from_array(key)
    m_bytes, ct_bytes, seed_bytes = B * L * n * 8, B * 2 * L * n * 8, B * 32

    def host(nbytes):
        p = ctypes.c_void_p()
        sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    h_m, h_out, h_seeds = host(m_bytes), host(ct_bytes), host(seed_bytes)
    np.ctypeslib.as_array((ctypes.c_uint64 * (B * L * n)).from_address(h_m))[:] = \
        splitmix_limbs(4100 + rank, B, QS, n).reshape(-1)
    np.ctypeslib.as_array((ctypes.c_uint8 * seed_bytes).from_address(h_seeds))[:] = \
        np.frombuffer(splitmix_limbs(4200 + rank, B * 4, [1 << 62], 1).tobytes(), np.uint8)
    d_m, d_out, d_seeds = (sg.DeviceBuffer(m_bytes), sg.DeviceBuffer(ct_bytes),
                           sg.DeviceBuffer(seed_bytes))
    sg.check(lib.shg_memcpy_h2d(d_m.ptr, h_m, m_bytes, s))
    sg.check(lib.shg_memcpy_h2d(d_seeds.ptr, h_seeds, seed_bytes, s))

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b, ctypes.byref(ms)))
        return ms.value

    def step_device():
        sg.check(lib.shg_bgv_encrypt(ctx.h, d_out.ptr, d_key.ptr, d_m.ptr, d_seeds.ptr, L, B,
                                     ENC_VARIANCE, s))

    step_device()
    sg.check(lib.shg_stream_synchronize(s))
    n0 = lib.shg_launch_count()
    sg.check(lib.shg_graph_capture_begin(s))
    step_device()
    g = ctypes.c_void_p()
    sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
    graph = g.value
    launches_per_step = lib.shg_launch_count() - n0
    for _ in range(args.warmup):
        sg.check(lib.shg_graph_launch(graph, s))
    sg.check(lib.shg_stream_synchronize(s))
    evs = [ev() for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    sg.check(lib.shg_event_record(evs[0], s))
    for i in range(args.steps):
        sg.check(lib.shg_graph_launch(graph, s))
        sg.check(lib.shg_event_record(evs[i + 1], s))
    sg.check(lib.shg_stream_synchronize(s))
    barrier(dist)
    clk = clocks.stop()
    step_ms = [elapsed(evs[i], evs[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(dist, elapsed(evs[0], evs[-1]))
    ops_all = sum_over_ranks(dist, float(B * args.steps))
    value = ops_all / (total_ms / 1e3)

    # End to end: plaintexts and seeds in from pinned host memory, ciphertexts
    # back, per step.
    e2e = None
    if not args.no_e2e:
        def step_e2e():
            sg.check(lib.shg_memcpy_h2d(d_m.ptr, h_m, m_bytes, s))
            sg.check(lib.shg_memcpy_h2d(d_seeds.ptr, h_seeds, seed_bytes, s))
            step_device()
            sg.check(lib.shg_memcpy_d2h(h_out, d_out.ptr, ct_bytes, s))
        warm_link(step_e2e, lambda: sg.check(lib.shg_stream_synchronize(s)),
                  max(3, args.warmup))
        e0, e1 = ev(), ev()
        barrier(dist)
        sg.check(lib.shg_event_record(e0, s))
        for _ in range(args.steps):
            step_e2e()
        sg.check(lib.shg_event_record(e1, s))
        sg.check(lib.shg_stream_synchronize(s))
        e2e_ms = max_over_ranks(dist, elapsed(e0, e1))
        e2e = {"value": ops_all / (e2e_ms / 1e3), "unit": ENC_UNIT,
               "h2d_bytes_per_step": m_bytes + seed_bytes, "d2h_bytes_per_step": ct_bytes,
               "ms_per_step": e2e_ms / args.steps}

    sg.check(lib.shg_profile_start())
    step_device()
    sg.check(lib.shg_profile_stop())
    prof = {}
    for name in ENC_SCOPES:
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        sg.check(lib.shg_profile_query(name.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        if cnt.value:
            prof[name] = (ms.value, cnt.value)
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    step_total = sum(v[0] for v in prof.values())
    kernels = {}
    for name, (ms, cnt) in prof.items():
        nbytes, ks = enc_scope_model(name, n, L, B)
        kernels[name] = {"share_of_step": ms / step_total, "launches": cnt,
                         "avg_launch_ms": ms / cnt,
                         "algorithmic_bytes_per_launch": nbytes / cnt,
                         "achieved_gbs": nbytes / (ms / 1e3) / 1e9,
                         "keystream_gbs": (ks / (ms / 1e3) / 1e9) if ks else None}
    top = max(prof, key=lambda nm: prof[nm][0])
    tk = kernels[top]
    roofline = {
        "kernel": top, "bound": "hbm", "achieved": tk["achieved_gbs"], "peak": peak,
        "unit": "GB/s", "frac": tk["achieved_gbs"] / peak, "peak_source": peak_src,
        "traffic": None, "algorithmic_bytes_per_launch": tk["algorithmic_bytes_per_launch"],
        "avg_launch_ms": tk["avg_launch_ms"], "kernels": kernels,
        "step_bytes_min": 3 * L * n * 8 * B,
        "step_frac_of_hbm": 3 * L * n * 8 * B / (total_ms / args.steps / 1e3) / 1e9 / peak,
    }
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, ops, dt = cpu_encrypt(10.0, threads)
        cpu = {"value": rate, "unit": ENC_UNIT, "cores": threads, "kind": "port",
               "sample": f"{ops} encryptions in {dt:.1f} s, one per host thread per round"}
    lat = sorted(step_ms)
    line = {
        "metric": ENC_METRIC, "value": value, "unit": ENC_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform key, plaintexts and PRNG seeds)",
        "config": enc_config(B),
        "latency_ms": {"step_p50": lat[len(lat) // 2], "step_p99": lat[-1]},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sg.check(lib.shg_graph_destroy(graph))
    for hp in (h_m, h_out, h_seeds):
        lib.shg_host_free(hp)


# ---------------------------------------------------------------------------
# BFV: RnsBfvCiphertext::operator* (Kim et al. tensor with basis extension),
# n = 2^14, six 45-bit main and seven 45-bit auxiliary primes, 1024 pairs.
# ---------------------------------------------------------------------------

BFV_METRIC = "RNS BFV ct*ct/sec (RnsBfvCiphertext::Mul, bit-exact)"
BFV_UNIT = "bfv-mul/s"
P45_AUX = [35184368320513, 35184368025601, 35184367828993, 35184367337473, 35184366911489,
           35184366551041, 35184366223361]
BFV_SCOPES = ("ntt_inv", "ntt_fwd", "switch_basis", "tensor", "lin2")


def bfv_config(count):
    return {"workload": "bfv-mul n=2^14 6x45-bit main + 7x45-bit aux primes t=65537",
            "log_n": LOG_N, "log_q": 45, "limbs": len(QS), "aux_limbs": len(P45_AUX),
            "pairs": count, "l2": "inputs and outputs per step (8 GB) exceed L2",
            "parallelism": "replicas"}


def bfv_scope_model(name, n, Lm, K, pairs):
    """Algorithmic DRAM bytes of one step of a scope (limb = n * 8 bytes)."""
    limb = n * 8
    per = {"ntt_inv": 2 * (4 * Lm + 3 * K), "ntt_fwd": 2 * (2 * K + 2 * Lm + 2 * K + 3 * Lm),
           "switch_basis": 9 * (Lm + K), "tensor": 7 * Lm + 7 * K, "lin2": 9 * Lm}[name]
    return per * limb * pairs


def cpu_bfv(seconds, threads, seed=7):
    """The reference's CPU RnsBfvCiphertext::Mul (oracle restatement), one pair
    per host thread per round, for about `seconds`."""
    import concurrent.futures
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    n = 1 << LOG_N
    L, K = len(QS), len(P45_AUX)
    rns = O.Rns(LOG_N, QS + P45_AUX)
    aux = list(range(L, L + K))
    a = splitmix_limbs(seed, 2 * threads, QS, n).reshape(threads, 2, L, n)
    b = splitmix_limbs(seed + 1, 2 * threads, QS, n).reshape(threads, 2, L, n)

    def one(i):
        return rns.bfv_mul(L, aux, T_PLAIN, a[i], b[i])

    ops = 0
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        while True:
            list(ex.map(one, range(threads)))
            ops += threads
            dt = time.perf_counter() - t0
            if dt >= seconds:
                break
    return ops / dt, ops, dt


def run_bfv_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per_step, ops_total = [], 0
    for i in range(args.warmup + args.steps):
        _, ops, dt = cpu_bfv(2.0, threads, seed=100 + i)
        if i >= args.warmup:
            per_step.append(dt)
            ops_total += ops
    total = sum(per_step)
    value = ops_total / total
    print(json.dumps({
        "metric": BFV_METRIC, "value": value, "unit": BFV_UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": bfv_config(threads),
        "cpu_baseline": {"value": value, "unit": BFV_UNIT, "cores": threads, "kind": "port",
                         "sample": "each step: about 2 s of whole BFV products, one per host "
                                   "thread per round"},
        "e2e": {"value": value, "unit": BFV_UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_bfv(args, world, rank, local, dist):
    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    n = 1 << LOG_N
    L, K = len(QS), len(P45_AUX)
    B = args.batch
    ctx = sg.Context(LOG_N, QS, T_PLAIN, ps=P45_AUX)
    if args.four_step_min:
        sg.check(lib.shg_context_set_four_step_min(ctx.h, args.four_step_min))
    if args.chunk:
        sg.check(lib.shg_context_set_chunk(ctx.h, args.chunk))
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value
    in_bytes, out_bytes = B * 2 * L * n * 8, B * 3 * L * n * 8

    def host(nbytes):
        p = ctypes.c_void_p()
        sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    h_a, h_b, h_out = host(in_bytes), host(in_bytes), host(out_bytes)
    for hp, seed in ((h_a, 5100 + rank), (h_b, 5200 + rank)):
        np.ctypeslib.as_array((ctypes.c_uint64 * (B * 2 * L * n)).from_address(hp))[:] = \
            splitmix_limbs(seed, 2 * B, QS, n).reshape(-1)
    d_a, d_b, d_out = (sg.DeviceBuffer(in_bytes), sg.DeviceBuffer(in_bytes),
                       sg.DeviceBuffer(out_bytes))
    sg.check(lib.shg_memcpy_h2d(d_a.ptr, h_a, in_bytes, s))
    sg.check(lib.shg_memcpy_h2d(d_b.ptr, h_b, in_bytes, s))

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b, ctypes.byref(ms)))
        return ms.value

    def step_device():
        sg.check(lib.shg_bfv_mul(ctx.h, d_out.ptr, d_a.ptr, d_b.ptr, B, L, s))

    step_device()
    sg.check(lib.shg_stream_synchronize(s))
    n0 = lib.shg_launch_count()
    sg.check(lib.shg_graph_capture_begin(s))
    step_device()
    g = ctypes.c_void_p()
    sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
    graph = g.value
    launches_per_step = lib.shg_launch_count() - n0
    for _ in range(args.warmup):
        sg.check(lib.shg_graph_launch(graph, s))
    sg.check(lib.shg_stream_synchronize(s))
    evs = [ev() for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    sg.check(lib.shg_event_record(evs[0], s))
    for i in range(args.steps):
        sg.check(lib.shg_graph_launch(graph, s))
        sg.check(lib.shg_event_record(evs[i + 1], s))
    sg.check(lib.shg_stream_synchronize(s))
    barrier(dist)
    clk = clocks.stop()
    step_ms = [elapsed(evs[i], evs[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(dist, elapsed(evs[0], evs[-1]))
    ops_all = sum_over_ranks(dist, float(B * args.steps))
    value = ops_all / (total_ms / 1e3)

    e2e = None
    if not args.no_e2e:
        def step_e2e():
            sg.check(lib.shg_memcpy_h2d(d_a.ptr, h_a, in_bytes, s))
            sg.check(lib.shg_memcpy_h2d(d_b.ptr, h_b, in_bytes, s))
            step_device()
            sg.check(lib.shg_memcpy_d2h(h_out, d_out.ptr, out_bytes, s))
        warm_link(step_e2e, lambda: sg.check(lib.shg_stream_synchronize(s)),
                  max(3, args.warmup))
        e0, e1 = ev(), ev()
        barrier(dist)
        sg.check(lib.shg_event_record(e0, s))
        for _ in range(args.steps):
            step_e2e()
        sg.check(lib.shg_event_record(e1, s))
        sg.check(lib.shg_stream_synchronize(s))
        e2e_ms = max_over_ranks(dist, elapsed(e0, e1))
        e2e = {"value": ops_all / (e2e_ms / 1e3), "unit": BFV_UNIT,
               "h2d_bytes_per_step": 2 * in_bytes, "d2h_bytes_per_step": out_bytes,
               "ms_per_step": e2e_ms / args.steps}

    sg.check(lib.shg_profile_start())
    step_device()
    sg.check(lib.shg_profile_stop())
    prof = {}
    for name in BFV_SCOPES:
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        sg.check(lib.shg_profile_query(name.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        if cnt.value:
            prof[name] = (ms.value, cnt.value)
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    bfly_peak = ctypes.c_double()
    sg.check(lib.shg_measure_butterfly_rate(ctypes.byref(bfly_peak)))
    step_total = sum(v[0] for v in prof.values())
    kernels = {}
    limb_bfly = n // 2 * LOG_N
    bfly_limbs = {"ntt_inv": 4 * L + 3 * K, "ntt_fwd": 4 * K + 5 * L}
    for name, (ms, cnt) in prof.items():
        nbytes = bfv_scope_model(name, n, L, K, B)
        kernels[name] = {"share_of_step": ms / step_total, "launches": cnt,
                         "avg_launch_ms": ms / cnt,
                         "algorithmic_bytes_per_launch": nbytes / cnt,
                         "achieved_gbs": nbytes / (ms / 1e3) / 1e9}
        if name in bfly_limbs:
            kernels[name]["int_frac"] = (bfly_limbs[name] * limb_bfly * B / (ms / 1e3)
                                         / bfly_peak.value)
    top = max(prof, key=lambda nm: prof[nm][0])
    tk = kernels[top]
    roofline = {
        "kernel": top, "bound": "hbm", "achieved": tk["achieved_gbs"], "peak": peak,
        "unit": "GB/s", "frac": tk["achieved_gbs"] / peak, "peak_source": peak_src,
        "traffic": None, "algorithmic_bytes_per_launch": tk["algorithmic_bytes_per_launch"],
        "avg_launch_ms": tk["avg_launch_ms"], "kernels": kernels,
        "butterfly_peak_per_s": bfly_peak.value,
    }
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, ops, dt = cpu_bfv(10.0, threads)
        cpu = {"value": rate, "unit": BFV_UNIT, "cores": threads, "kind": "port",
               "sample": f"{ops} BFV products in {dt:.1f} s, one per host thread per round"}
    lat = sorted(step_ms)
    line = {
        "metric": BFV_METRIC, "value": value, "unit": BFV_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform ciphertexts)", "config": bfv_config(B),
        "latency_ms": {"step_p50": lat[len(lat) // 2], "step_p99": lat[-1]},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sg.check(lib.shg_graph_destroy(graph))
    for hp in (h_a, h_b, h_out):
        lib.shg_host_free(hp)


# Limb-NTT throughput (the path's forward / inverse transforms on their own):
# 1024 polynomials of six limbs per call (inputs larger than L2 at every
# size).  n = 2^12 and 2^14 use the workload's 45-bit primes (1 mod 2^15);
# n = 2^15 needs primes that are 1 mod 2^16 and takes six 50-bit ones.
NTT_CASES = ((12, QS, "six 45-bit primes"), (14, QS, "six 45-bit primes"),
             (15, [1125899904679937, 1125899903827969, 1125899903500289, 1125899903107073,
                   1125899902124033, 1125899901665281], "six 50-bit primes"))
NTT_POLYS = 1024


def ntt_record(sg, lib, s, ev, elapsed, peak, bfly_peak, reps=10, polys=NTT_POLYS,
               four_step_min=0):
    """Forward and inverse limb-NTTs/s (shg_ntt_forward / shg_ntt_inverse in
    place over NTT_POLYS x 6 limbs), with the HBM fraction at 16 n bytes per
    limb-NTT (each limb read and written once) and the butterfly rate against
    the integer ceiling."""
    out = {}
    for log_n, qs, primes in NTT_CASES:
        n, L = 1 << log_n, len(qs)
        ctx = sg.Context(log_n, qs)
        if four_step_min:
            sg.check(lib.shg_context_set_four_step_min(ctx.h, four_step_min))
        buf = sg.DeviceBuffer(polys * L * n * 8)
        sg.check(lib.shg_poly_fill_uniform(ctx.h, buf.ptr, polys, L, 99, s))
        limbs = polys * L
        rec = {"n": n, "primes": primes, "limb_ntts_per_call": limbs,
               "bytes_per_limb_ntt": 16 * n, "butterflies_per_limb_ntt": n // 2 * log_n}
        for name, fn in (("fwd", lib.shg_ntt_forward), ("inv", lib.shg_ntt_inverse)):
            for _ in range(3):
                sg.check(fn(ctx.h, buf.ptr, polys, L, s))
            e0, e1 = ev(), ev()
            sg.check(lib.shg_event_record(e0, s))
            for _ in range(reps):
                sg.check(fn(ctx.h, buf.ptr, polys, L, s))
            sg.check(lib.shg_event_record(e1, s))
            sg.check(lib.shg_stream_synchronize(s))
            call_s = elapsed(e0, e1) / reps / 1e3
            gbs = 16 * n * limbs / call_s / 1e9
            bps = (n // 2 * log_n) * limbs / call_s
            rec[name] = {"limb_ntts_per_s": limbs / call_s, "ms_per_call": call_s * 1e3,
                         "achieved_gbs": gbs, "hbm_frac": gbs / peak,
                         "butterflies_per_s": bps, "int_frac": bps / bfly_peak}
        buf.free()
        ctx.close()
        out[f"n{n}"] = rec
    out["unit"] = "limb-NTT/s"
    out["peak_gbs"] = peak
    out["peak_butterflies_per_s"] = bfly_peak
    return out


def run_ntt(args, rank):
    """--workload ntt: the limb-NTT record alone (forward and inverse
    transforms at n = 2^12, 2^14, 2^15 over six primes)."""
    import shell_gpu as sg
    lib = sg.lib()
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b, ctypes.byref(ms)))
        return ms.value
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak = float(peaks["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        peak = 6800.0
    bfly = ctypes.c_double()
    sg.check(lib.shg_measure_butterfly_rate(ctypes.byref(bfly)))
    rec = ntt_record(sg, lib, s, ev, elapsed, peak, bfly.value, reps=max(args.steps, 1),
                     polys=args.ntt_polys, four_step_min=args.four_step_min)
    n14 = rec["n16384"]["fwd"]
    if rank == 0:
        print(json.dumps({"metric": "limb-NTT/s (forward, n=2^14, six 45-bit primes)",
                          "value": n14["limb_ntts_per_s"], "unit": "limb-NTT/s",
                          "higher_is_better": True, "dtype": "u64", "data": "synthetic",
                          "config": {"workload": f"{args.ntt_polys} polynomials x 6 limbs"},
                          "ntt": rec}), flush=True)


def other_workloads(args, world, rank, local, dist):
    """Compact runs of the path's other workloads for the default line (so they
    are timed under the same clocks): PIR expand + absorb, BGV encryption with
    on-device sampling, BFV multiplication, the uneven batch (C3: 4096 mixed
    instances, autotuned, against one call per instance) -- each its own
    workload function with 3 warm-up and 3 timed steps, device-resident
    inputs, no CPU leg and no host-copy leg -- and serving (C5) at its
    saturating offered rate of 50 k requests/s for one second of arrivals.
    Their full lines come from --workload."""
    import contextlib
    import io
    out = {}
    for wl, runner in (("pir", run_pir), ("encrypt", run_encrypt), ("bfv-mul", run_bfv),
                       ("uneven", run_uneven), ("serve", run_serve)):
        a = argparse.Namespace(**vars(args))
        a.workload, a.steps, a.warmup = wl, 3, 3
        a.rates = "50000"  # serving: the saturating rate only
        a.no_cpu_baseline, a.no_e2e = True, True
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            runner(a, world, rank, local, dist)
        lines = [ln for ln in buf.getvalue().splitlines() if ln.startswith("{")]
        if not lines:
            continue
        d = json.loads(lines[-1])
        rec = {k: d.get(k) for k in ("metric", "value", "unit", "ms_per_step")}
        rec["workload"] = (d.get("config") or {}).get("workload")
        if d.get("roofline"):
            rec["roofline_frac"] = d["roofline"].get("frac")
        if wl == "serve" and d.get("sweep"):
            top = d["sweep"][-1]
            rec.update({k: top.get(k) for k in ("offered_req_s", "throughput_req_s", "p50_ms",
                                                 "p99_ms", "mean_batch")})
            rec["served_over_plain"] = d.get("served_over_plain_at_top_rate")
        for k in ("batched_over_plain", "bit_exact_batched_vs_plain"):
            if k in d:
                rec[k] = d[k]
        if d.get("plain"):
            rec["plain"] = d["plain"].get("value")
        out[wl] = rec
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--plain-ops", type=int, default=256)
    ap.add_argument("--chunk", type=int, default=0, help="ciphertexts per internal chunk")
    ap.add_argument("--four-step-min", type=int, default=0,
                    help="log n from which NTTs use the four-step kernels (default 14)")
    ap.add_argument("--ks-unfused", action="store_true",
                    help="separate digit row phase and key inner product kernels")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--rates", default="1000,5000,20000,50000")
    ap.add_argument("--seconds", type=float, default=1.0, help="arrival window per rate")
    ap.add_argument("--clients", type=int, default=64)
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--max-wait-us", type=int, default=500)
    ap.add_argument("--streams", type=int, default=4)
    ap.add_argument("--host-piece", type=int, default=0,
                    help="e2e host pipeline: ciphertexts per piece (0: library default)")
    ap.add_argument("--host-slots", type=int, default=0,
                    help="e2e host pipeline: staging slots in flight (0: library default)")
    ap.add_argument("--host-ramp", type=int, default=-1,
                    help="e2e host pipeline: piece ramp (-1: library default)")
    ap.add_argument("--hbm-budget-gb", type=int, default=32)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", default="ct-mult-relin",
                    choices=["ct-mult-relin", "pir", "uneven", "serve", "encrypt", "bfv-mul",
                             "ntt"],
                    help="ct-mult-relin: RNS BGV ct x ct + relinearization (n=2^14, 6 primes); "
                         "pir: oblivious expansion + database absorb (n=2^12, one prime); "
                         "uneven: 4096 mixed instances through the batch executor; "
                         "encrypt: EncryptPolynomialBgv with on-device ChaCha sampling; "
                         "bfv-mul: RnsBfvCiphertext ct x ct with basis extension; "
                         "ntt: the forward / inverse limb-NTT record alone")
    ap.add_argument("--queries", type=int, default=PIR_QUERIES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ntt", action="store_true", help="skip the limb-NTT throughput record")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the compact PIR / encryption / BFV records of the default line")
    ap.add_argument("--ntt-polys", type=int, default=NTT_POLYS,
                    help="polynomials (of six limbs) per transform call in the NTT record")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gpu" else args.warmup

    world, rank, local, dist = dist_setup(args)
    if args.workload == "ntt":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": "limb-NTT/s",
                                  "unavailable": "timed only for the ct-mult-relin and pir "
                                                 "workloads"}), flush=True)
        else:
            run_ntt(args, rank)
        return
    if args.workload == "serve":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": SERVE_METRIC,
                                  "unavailable": "timed only for the ct-mult-relin and pir "
                                                 "workloads"}), flush=True)
        else:
            run_serve(args, world, rank, local, dist)
        return
    if args.workload == "uneven":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": UNEVEN_METRIC,
                                  "unavailable": "timed only for the ct-mult-relin and pir "
                                                 "workloads"}), flush=True)
        else:
            run_uneven(args, world, rank, local, dist)
        return
    if args.workload == "bfv-mul":
        if args.impl == "reference":
            run_bfv_reference(args, world, rank)
        else:
            run_bfv(args, world, rank, local, dist)
        return
    if args.workload == "encrypt":
        if args.impl == "reference":
            run_encrypt_reference(args, world, rank)
        else:
            run_encrypt(args, world, rank, local, dist)
        return
    if args.workload == "pir":
        if args.impl == "reference":
            run_pir_reference(args, world, rank)
        else:
            run_pir(args, world, rank, local, dist)
        return
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        return

    import shell_gpu as sg
    lib = sg.lib()
    sg.check(lib.shg_set_device(local))
    n = 1 << LOG_N
    L = len(QS)
    B = args.batch
    ct_elems = 2 * L * n
    ct_bytes = ct_elems * 8

    ctx = sg.Context(LOG_N, QS, T_PLAIN)
    if args.chunk:
        sg.check(lib.shg_context_set_chunk(ctx.h, args.chunk))
    if args.four_step_min:
        sg.check(lib.shg_context_set_four_step_min(ctx.h, args.four_step_min))
    if args.ks_unfused:
        sg.check(lib.shg_context_set_ks_fused(ctx.h, 0))
    if args.host_piece or args.host_slots:
        sg.check(lib.shg_context_set_host_pipeline(ctx.h, args.host_piece or 32,
                                                   args.host_slots or 4))
    if args.host_ramp >= 0:
        sg.check(lib.shg_context_set_host_ramp(ctx.h, args.host_ramp))
    k = 18
    kb = splitmix_limbs(1000 + rank, k, QS, n)
    ka = splitmix_limbs(2000 + rank, k, QS, n)
    key = sg.Key(ctx, LOG_BS, 1, kb, ka)

    # Pinned host inputs (also the e2e source) and device copies.
    def host(nbytes):
        p = ctypes.c_void_p()
        sg.check(lib.shg_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    h_a, h_b, h_out = host(B * ct_bytes), host(B * ct_bytes), host(B * ct_bytes)
    for hp, seed in ((h_a, 11 + 97 * rank), (h_b, 13 + 97 * rank)):
        view = np.ctypeslib.as_array((ctypes.c_uint64 * (B * ct_elems)).from_address(hp))
        for c0 in range(0, B, 64):
            c1 = min(B, c0 + 64)
            view[c0 * ct_elems:c1 * ct_elems] = splitmix_limbs(
                seed * 1000003 + c0, 2 * (c1 - c0), QS, n).reshape(-1)
    d_a, d_b, d_out = (sg.DeviceBuffer(B * ct_bytes) for _ in range(3))
    s = ctypes.c_void_p()
    sg.check(lib.shg_stream_create(ctypes.byref(s)))
    s = s.value
    sg.check(lib.shg_memcpy_h2d(d_a.ptr, h_a, B * ct_bytes, s))
    sg.check(lib.shg_memcpy_h2d(d_b.ptr, h_b, B * ct_bytes, s))
    sg.check(lib.shg_stream_synchronize(s))

    def ev():
        e = ctypes.c_void_p()
        sg.check(lib.shg_event_create(ctypes.byref(e)))
        return e.value

    def elapsed(a, b):
        ms = ctypes.c_float()
        sg.check(lib.shg_event_elapsed_ms(a, b, ctypes.byref(ms)))
        return ms.value

    def step_device():
        sg.check(lib.shg_bgv_mul_relin(ctx.h, key.h, d_out.ptr, d_a.ptr, d_b.ptr, B, s))

    # Warm up (allocates scratch), then capture one step into a graph.
    step_device()
    sg.check(lib.shg_stream_synchronize(s))
    n0 = lib.shg_launch_count()
    sg.check(lib.shg_graph_capture_begin(s))
    step_device()
    g = ctypes.c_void_p()
    sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
    graph = g.value
    launches_per_step = lib.shg_launch_count() - n0
    for _ in range(args.warmup):
        sg.check(lib.shg_graph_launch(graph, s))
    sg.check(lib.shg_stream_synchronize(s))

    evs = [ev() for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(dist)
    sg.check(lib.shg_device_synchronize())
    sg.check(lib.shg_event_record(evs[0], s))
    for i in range(args.steps):
        sg.check(lib.shg_graph_launch(graph, s))
        sg.check(lib.shg_event_record(evs[i + 1], s))
    sg.check(lib.shg_stream_synchronize(s))
    sg.check(lib.shg_device_synchronize())
    barrier(dist)
    clk = clocks.stop()
    step_ms = [elapsed(evs[i], evs[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(dist, elapsed(evs[0], evs[-1]))
    ops_all = sum_over_ranks(dist, float(B * args.steps))
    value = ops_all / (total_ms / 1e3)

    # Bit-exactness check of the timed graph's output against the plain
    # one-call-per-op path, which recomputes the first min(plain ops, 64)
    # ciphertexts (the parity tests cover the oracle side).
    check_cts = max(1, min(args.plain_ops, B, 64))
    out_graph = np.empty(ct_elems * check_cts, np.uint64)
    sg.check(lib.shg_memcpy_d2h(out_graph.ctypes.data, d_out.ptr, out_graph.nbytes, s))
    sg.check(lib.shg_stream_synchronize(s))

    def link_probe():
        """Host-link bandwidth now (GB/s): 1.6 GB pinned->device, device->
        pinned, and both at once on two streams."""
        nb = B * ct_bytes
        s2 = ctypes.c_void_p()
        sg.check(lib.shg_stream_create(ctypes.byref(s2)))
        a0, a1, b0, b1 = ev(), ev(), ev(), ev()
        rates = {}
        for name, h2d, d2h in (("h2d", True, False), ("d2h", False, True), ("duplex", True, True)):
            sg.check(lib.shg_device_synchronize())
            sg.check(lib.shg_event_record(a0, s))
            sg.check(lib.shg_event_record(b0, s2.value))
            if h2d:
                sg.check(lib.shg_memcpy_h2d(d_a.ptr, h_a, nb, s))
            if d2h:
                sg.check(lib.shg_memcpy_d2h(h_out, d_out.ptr, nb, s2.value))
            sg.check(lib.shg_event_record(a1, s))
            sg.check(lib.shg_event_record(b1, s2.value))
            sg.check(lib.shg_device_synchronize())
            if name == "duplex":
                rates[name] = [nb / elapsed(a0, a1) / 1e6, nb / elapsed(b0, b1) / 1e6]
            else:
                rates[name] = nb / elapsed(*((a0, a1) if h2d else (b0, b1))) / 1e6
        sg.check(lib.shg_stream_destroy(s2.value))
        return rates

    # End to end: pinned host buffers in, result back to the host, per step.
    e2e = None
    if not args.no_e2e:
        def step_e2e():
            # The host-buffer entry point: pinned inputs in, results back in
            # host memory, copies pipelined against compute inside the call.
            sg.check(lib.shg_bgv_mul_relin_host(ctx.h, key.h, h_out, h_a, h_b, B, s))
        # Warm-up calls first: the first large host copies after the device-only
        # phase run at a fraction of the link's rate (probes there read 10-20
        # GB/s against 211), so the probe and the timing come after them.
        warm_link(step_e2e, lambda: sg.check(lib.shg_stream_synchronize(s)), max(3, args.warmup))
        link_before = link_probe()
        # one more untimed call after the probe, so the timing starts from the
        # pipeline's steady state (the first step after a probe has read slow)
        step_e2e()
        sg.check(lib.shg_stream_synchronize(s))
        xev = [ev() for _ in range(args.steps + 1)]
        barrier(dist)
        sg.check(lib.shg_event_record(xev[0], s))
        for i in range(args.steps):
            step_e2e()
            sg.check(lib.shg_event_record(xev[i + 1], s))
        sg.check(lib.shg_stream_synchronize(s))
        barrier(dist)
        e2e_ms = max_over_ranks(dist, elapsed(xev[0], xev[-1]))
        e2e_step_ms = [round(elapsed(xev[i], xev[i + 1]), 3) for i in range(args.steps)]
        link_after = link_probe()
        # The step's copies alone at the probed rates: the host link bounds
        # the step when this exceeds the device step.
        h2d_ms = 2 * B * ct_bytes / (max(link_before["duplex"][0], link_after["duplex"][0]) * 1e6)
        # the link's capacity: the better of the two probes, rate by rate
        best = {"h2d": max(link_before["h2d"], link_after["h2d"]),
                "d2h": max(link_before["d2h"], link_after["d2h"]),
                "duplex": [max(a, b) for a, b in zip(link_before["duplex"],
                                                     link_after["duplex"])]}
        link_ms = host_link_ms(2 * B * ct_bytes, B * ct_bytes, best)
        bound_ms = max(link_ms, total_ms / args.steps)
        e2e = {"value": ops_all / (e2e_ms / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": 2 * B * ct_bytes, "d2h_bytes_per_step": B * ct_bytes,
               "ms_per_step": e2e_ms / args.steps, "step_ms": e2e_step_ms,
               "link": {"unit": "GB/s", "before": link_before, "after": link_after,
                        "h2d_ms_per_step_at_duplex_rate": h2d_ms,
                        "link_ms_per_step": link_ms,
                        "device_ms_per_step": total_ms / args.steps},
               "roofline": {"bound": "host link" if link_ms >= total_ms / args.steps
                            else "device", "bound_ms_per_step": bound_ms,
                            "frac": bound_ms / (e2e_ms / args.steps)}}

    # End to end in the wire format: host ciphertexts serialized as the
    # reference serializes them (log q-bit packed limbs), packed bytes over the
    # host link, (de)serialization on the device.
    e2e_wire = None
    if not args.no_e2e:
        pb = lib.shg_poly_serialized_bytes(ctx.h, L)
        wct = 2 * pb
        hw_a, hw_b, hw_out = host(B * wct), host(B * wct), host(B * wct)
        dw = sg.DeviceBuffer(B * wct)
        for dsrc, hdst in ((d_a, hw_a), (d_b, hw_b)):
            sg.check(lib.shg_poly_serialize(ctx.h, dw.ptr, dsrc.ptr, 2 * B, L, s))
            sg.check(lib.shg_memcpy_d2h(hdst, dw.ptr, B * wct, s))
        sg.check(lib.shg_stream_synchronize(s))
        dw.free()

        def step_wire():
            sg.check(lib.shg_bgv_mul_relin_host_serialized(ctx.h, key.h, hw_out, hw_a, hw_b, B,
                                                           s))
        warm_link(step_wire, lambda: sg.check(lib.shg_stream_synchronize(s)), max(3, args.warmup))
        w0, w1 = ev(), ev()
        barrier(dist)
        sg.check(lib.shg_event_record(w0, s))
        for _ in range(args.steps):
            step_wire()
        sg.check(lib.shg_event_record(w1, s))
        sg.check(lib.shg_stream_synchronize(s))
        barrier(dist)
        wire_ms = max_over_ranks(dist, elapsed(w0, w1))
        e2e_wire = {"value": ops_all / (wire_ms / 1e3), "unit": UNIT,
                    "h2d_bytes_per_step": 2 * B * wct, "d2h_bytes_per_step": B * wct,
                    "ms_per_step": wire_ms / args.steps,
                    "format": "SHELL serialization (MontgomeryInt::SerializeVector per limb)"}
        for hp in (hw_a, hw_b, hw_out):
            lib.shg_host_free(hp)

    # Plain drop-in path: one ct_tensor + one relin_apply call per ciphertext.
    P = min(args.plain_ops, B)
    d_ct3 = sg.DeviceBuffer(P * 3 * L * n * 8)
    op_evs = [ev() for _ in range(P + 1)]

    def plain(record):
        for i in range(P):
            sg.check(lib.shg_ct_tensor(ctx.h, d_ct3.ptr + i * 3 * L * n * 8,
                                       d_a.ptr + i * ct_bytes, d_b.ptr + i * ct_bytes, 1, L, s))
            sg.check(lib.shg_relin_apply(ctx.h, key.h, d_out.ptr + i * ct_bytes,
                                         d_ct3.ptr + i * 3 * L * n * 8, 1, s))
            if record:
                sg.check(lib.shg_event_record(op_evs[i + 1], s))
    plain(False)
    sg.check(lib.shg_stream_synchronize(s))
    sg.check(lib.shg_event_record(op_evs[0], s))
    plain(True)
    sg.check(lib.shg_stream_synchronize(s))
    op_ms = [elapsed(op_evs[i], op_evs[i + 1]) for i in range(P)]
    plain_total = elapsed(op_evs[0], op_evs[-1])
    plain_rate = P / (plain_total / 1e3)
    # plain outputs must equal the batched ones (same inputs, same key)
    out_plain = np.empty(ct_elems * check_cts, np.uint64)
    sg.check(lib.shg_memcpy_d2h(out_plain.ctypes.data, d_out.ptr, out_plain.nbytes, s))
    sg.check(lib.shg_stream_synchronize(s))
    bit_exact = bool(np.array_equal(out_graph, out_plain))

    # Dominant kernel timing (live CUDA events on the launch stream) for the
    # roofline: one more batched step with per-launch events, its chunks on
    # one stream so the kernels' event intervals do not overlap.
    sg.check(lib.shg_context_set_ks_lanes(ctx.h, 1))
    sg.check(lib.shg_profile_start())
    step_device()
    sg.check(lib.shg_profile_stop())
    sg.check(lib.shg_context_set_ks_lanes(ctx.h, 2))
    prof = {}
    for name in SCOPES:
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        sg.check(lib.shg_profile_query(name.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        if cnt.value:
            prof[name] = (ms.value, cnt.value)
    if not prof:
        raise RuntimeError("no kernel launch was timed in the profiled step")
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    bfly_peak = ctypes.c_double()
    sg.check(lib.shg_measure_butterfly_rate(ctypes.byref(bfly_peak)))
    step_total = sum(v[0] for v in prof.values())
    kernels = {}
    bfly_step, bfly_ms = 0.0, 0.0
    for name, (ms, cnt) in prof.items():
        nbytes, bfly = scope_model(name, n, L, k, B / cnt)
        launch_s = ms / cnt / 1e3
        kernels[name] = {
            "share_of_step": ms / step_total, "launches": cnt, "avg_launch_ms": ms / cnt,
            "algorithmic_bytes_per_launch": nbytes, "achieved_gbs": nbytes / launch_s / 1e9,
            "butterflies_per_launch": bfly,
            "int_frac": (bfly / launch_s / bfly_peak.value) if bfly else None,
        }
        if bfly:
            bfly_step += bfly * cnt
            bfly_ms += ms
    top = max(prof, key=lambda nm: prof[nm][0])
    tk = kernels[top]
    traffic = (TRAFFIC_PER_CT[top] * B / prof[top][1]) if top in TRAFFIC_PER_CT else None
    roofline = {
        "kernel": top, "bound": "hbm", "achieved": tk["achieved_gbs"], "peak": peak,
        "unit": "GB/s", "frac": tk["achieved_gbs"] / peak, "peak_source": peak_src,
        "traffic": traffic,
        "algorithmic_bytes_per_launch": tk["algorithmic_bytes_per_launch"],
        "avg_launch_ms": tk["avg_launch_ms"],
        "multiply_pipe": {"busy_frac": MULPIPE_BUSY.get(top),
                          "source": "ncu sm__pipe_fmaheavy_cycles_active of one 16-ciphertext "
                                    "launch: the kernel is bound by 64-bit integer multiply "
                                    "throughput, not HBM"} if top in MULPIPE_BUSY else None,
        # The transforms are bound by 64-bit integer multiply issue, not HBM:
        # butterflies/s of the NTT-bearing kernels against the live probe.
        "integer": {"peak_butterflies_per_s": bfly_peak.value,
                    "achieved_butterflies_per_s": bfly_step / (bfly_ms / 1e3),
                    "frac": bfly_step / (bfly_ms / 1e3) / bfly_peak.value,
                    "peak_source": "shg_measure_butterfly_rate (register-only lazy butterflies)"},
        "kernels": kernels,
    }

    ntt = None if args.no_ntt else ntt_record(sg, lib, s, ev, elapsed, peak, bfly_peak.value,
                                              polys=args.ntt_polys)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, ops, dt = cpu_reference(10.0, threads)
        rate1, _, _ = cpu_reference(1.0, 1)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ops} ct-mult+relin ops at n=2^14, L=6 in {dt:.1f} s "
                         f"(one ciphertext pair per host thread per round)",
               "single_thread_ms_per_op": 1e3 / rate1}

    lat = sorted(step_ms)
    oplat = sorted(op_ms)

    def pct(v, p):
        return v[min(len(v) - 1, int(round(p / 100 * (len(v) - 1))))]

    others = None
    if world == 1 and not args.no_others:
        others = other_workloads(args, world, rank, local, dist)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform residues, splitmix64)", "config": config(B),
        "latency_ms": {"batched_step_p50": pct(lat, 50), "batched_step_p99": pct(lat, 99),
                       "plain_op_p50": pct(oplat, 50), "plain_op_p99": pct(oplat, 99)},
        "plain": {"value": plain_rate, "unit": UNIT, "ops": P,
                  "path": "shg_ct_tensor + shg_relin_apply per ciphertext"},
        "batched_over_plain": value / world / plain_rate,
        "bit_exact_batched_vs_plain": bit_exact, "bit_exact_checked_cts": check_cts,
        "e2e": e2e, "e2e_wire": e2e_wire, "roofline": roofline, "ntt": ntt,
        "other_workloads": others, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sg.check(lib.shg_graph_destroy(graph))
    for hp in (h_a, h_b, h_out):
        lib.shg_host_free(hp)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
