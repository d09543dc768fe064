"""Serving loop with continuous batching (include/shell_gpu_serve.h).

Requests of several clients (own keys), parameter sets and operations are
submitted concurrently; every result must be identical to the same request
served alone, and to the oracle.  A tight HBM budget must hold the admitted
footprint under it while everything still completes; waits are bounded.
"""
import ctypes
import threading

import numpy as np
import pytest

from conftest import Q50, Q60

LOG_B = 20
PARAMS = [(11, 2), (12, 3), (14, 2)]
PIR = dict(log_n=9, levels=4, log_b=8, items=12)


def _server(sg, budget=1 << 30, max_batch=16, max_wait_us=200, streams=3):
    cfg = sg.ServerConfig(budget, max_batch, max_wait_us, streams)
    h = ctypes.c_void_p()
    sg.check(sg.lib().shg_server_create(ctypes.byref(cfg), ctypes.byref(h)))
    return h


def _setup(sg, oracle):
    clients = []
    for c in range(2):
        env = {}
        for log_n, L in PARAMS:
            qs, n = Q50[:L], 1 << log_n
            ctx = sg.Context(log_n, qs)
            rns = oracle.Rns(log_n, qs)
            k = rns.gadget_dim([LOG_B] * L)
            kb = oracle.uniform_limbs(100 * c + log_n, qs, n, k)
            ka = oracle.uniform_limbs(100 * c + log_n + 50, qs, n, k)
            env[(log_n, L)] = dict(ctx=ctx, rns=rns, qs=qs, n=n, kb=kb, ka=ka,
                                   relin=sg.Key(ctx, [LOG_B] * L, 1, kb, ka),
                                   galois=sg.Key(ctx, [LOG_B] * L, 5, kb, ka))
        # PIR context for this client
        n = 1 << PIR["log_n"]
        p = oracle.Prime(Q60, PIR["log_n"])
        dim = p.gadget_size(PIR["log_b"])
        keys = oracle.uniform_limbs(700 + c, [Q60], n, PIR["levels"] * 2 * dim).reshape(
            PIR["levels"], 2, dim, n)
        db = oracle.uniform_limbs(800 + c, [Q60], n, PIR["items"]).reshape(PIR["items"], n)
        pctx = sg.Context(PIR["log_n"], [Q60])
        gkeys = [sg.Key(pctx, [PIR["log_b"]], (n >> j) + 1, keys[j, 0], keys[j, 1])
                 for j in range(PIR["levels"])]
        karr = (ctypes.c_void_p * PIR["levels"])(*[k.h for k in gkeys])
        env["pir"] = dict(ctx=pctx, p=p, keys=keys, gkeys=gkeys, karr=karr, db=db,
                          d_db=sg.DeviceBuffer.from_array(db), n=n)
        clients.append(env)
    return clients


def _requests(sg, oracle, clients, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        c = int(rng.integers(len(clients)))
        env = clients[c]
        kind = int(rng.choice([0, 0, 0, 1, 2]))
        if kind == 2:
            e = env["pir"]
            a = oracle.uniform_limbs(5000 + i, [Q60], e["n"], 2).reshape(2, e["n"])
            out = np.zeros_like(a)
            r = sg.Request(kind=2, ctx=e["ctx"].h, key=None, keys=e["karr"],
                           levels=PIR["levels"], db=e["d_db"].ptr, num_items=PIR["items"],
                           in_a=a.ctypes.data, in_b=None, out=out.ctypes.data)
            reqs.append(dict(client=c, kind=2, a=a, out=out, req=r))
            continue
        shape = PARAMS[int(rng.integers(len(PARAMS)))]
        e = env[shape]
        a = oracle.uniform_limbs(6000 + i, e["qs"], e["n"], 2)
        b = oracle.uniform_limbs(7000 + i, e["qs"], e["n"], 2)
        out = np.zeros_like(a)
        key = e["relin"] if kind == 0 else e["galois"]
        r = sg.Request(kind=kind, ctx=e["ctx"].h, key=key.h, keys=None, levels=0, db=None,
                       num_items=0, in_a=a.ctypes.data, in_b=b.ctypes.data,
                       out=out.ctypes.data)
        reqs.append(dict(client=c, kind=kind, shape=shape, a=a, b=b, out=out, req=r))
    return reqs


def _oracle_result(clients, q):
    env = clients[q["client"]]
    if q["kind"] == 2:
        e = env["pir"]
        exp = e["p"].oblivious_expand(PIR["levels"], PIR["log_b"], e["keys"], q["a"])
        return e["p"].absorb_sum(exp[:PIR["items"]], e["db"])
    e = env[q["shape"]]
    rns, L = e["rns"], q["shape"][1]
    if q["kind"] == 0:
        return rns.relin(rns.tensor(q["a"], q["b"]), e["kb"], e["ka"], [LOG_B] * L)
    sub = np.stack([rns.substitute(q["a"][c], 5) for c in range(2)])
    return rns.galois(sub, e["kb"], e["ka"], [LOG_B] * L)


@pytest.mark.gpu
def test_each_result_is_the_same_alone_and_in_the_mix(sg, oracle):
    lib = sg.lib()
    clients = _setup(sg, oracle)
    reqs = _requests(sg, oracle, clients, 48, seed=3)
    sv = _server(sg)
    try:
        # In the mix: three submitting threads at once.
        tickets = [None] * len(reqs)

        def submit(idx):
            for i in idx:
                t = ctypes.c_uint64()
                sg.check(lib.shg_server_submit(sv, ctypes.byref(reqs[i]["req"]), ctypes.byref(t)))
                tickets[i] = t.value

        threads = [threading.Thread(target=submit, args=(range(k, len(reqs), 3),))
                   for k in range(3)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        for t in tickets:
            sg.check(lib.shg_server_wait(sv, t, 60_000_000))
        mixed = [q["out"].copy() for q in reqs]
        st = sg.ServerStats()
        sg.check(lib.shg_server_get_stats(sv, ctypes.byref(st)))
        assert st.completed == len(reqs) and st.failed == 0
        assert st.batches < len(reqs)  # some requests shared a launch
        # Alone: one request at a time.
        for q in reqs:
            q["out"][:] = 0
            t = ctypes.c_uint64()
            sg.check(lib.shg_server_submit(sv, ctypes.byref(q["req"]), ctypes.byref(t)))
            sg.check(lib.shg_server_wait(sv, t.value, 60_000_000))
        for q, m in zip(reqs, mixed):
            assert np.array_equal(q["out"], m)
        for q in reqs[:10]:
            assert np.array_equal(q["out"], _oracle_result(clients, q))
        adm, lau, done = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        sg.check(lib.shg_server_latency(sv, tickets[0], ctypes.byref(adm), ctypes.byref(lau),
                                        ctypes.byref(done)))
        assert 0 <= adm.value <= lau.value <= done.value
    finally:
        lib.shg_server_destroy(sv)


@pytest.mark.gpu
def test_admission_keeps_footprint_under_budget(sg, oracle):
    lib = sg.lib()
    clients = _setup(sg, oracle)
    reqs = [q for q in _requests(sg, oracle, clients, 40, seed=5) if q["kind"] == 0]
    biggest = max(q["a"].nbytes * 3 for q in reqs)
    budget = 2 * biggest
    sv = _server(sg, budget=budget, max_batch=4)
    try:
        tickets = []
        for q in reqs:
            t = ctypes.c_uint64()
            sg.check(lib.shg_server_submit(sv, ctypes.byref(q["req"]), ctypes.byref(t)))
            tickets.append(t.value)
        for t in tickets:
            sg.check(lib.shg_server_wait(sv, t, 60_000_000))
        st = sg.ServerStats()
        sg.check(lib.shg_server_get_stats(sv, ctypes.byref(st)))
        assert st.completed == len(reqs)
        assert st.peak_bytes_in_flight <= budget
        assert st.admission_waits > 0
        for q in reqs[:5]:
            assert np.array_equal(q["out"], _oracle_result(clients, q))
        # A request larger than the whole budget is refused up front.
        big = sv  # same server
        e = clients[0][(14, 2)]
        a = np.zeros((2, 2, 1 << 14), np.uint64)
        small = _server(sg, budget=a.nbytes, max_batch=1)
        try:
            r = sg.Request(kind=0, ctx=e["ctx"].h, key=e["relin"].h, keys=None, levels=0,
                           db=None, num_items=0, in_a=a.ctypes.data, in_b=a.ctypes.data,
                           out=a.ctypes.data)
            t = ctypes.c_uint64()
            assert lib.shg_server_submit(small, ctypes.byref(r), ctypes.byref(t)) == 8
        finally:
            lib.shg_server_destroy(small)
        del big
    finally:
        lib.shg_server_destroy(sv)


@pytest.mark.gpu
def test_wait_is_bounded(sg, oracle):
    lib = sg.lib()
    log_n, L = 15, 4
    qs, n = Q50[:L], 1 << log_n
    ctx = sg.Context(log_n, qs)
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim([LOG_B] * L)
    key = sg.Key(ctx, [LOG_B] * L, 1, oracle.uniform_limbs(1, qs, n, k),
                 oracle.uniform_limbs(2, qs, n, k))
    a = oracle.uniform_limbs(3, qs, n, 2)
    out = np.zeros_like(a)
    sv = _server(sg)
    try:
        r = sg.Request(kind=0, ctx=ctx.h, key=key.h, keys=None, levels=0, db=None, num_items=0,
                       in_a=a.ctypes.data, in_b=a.ctypes.data, out=out.ctypes.data)
        t = ctypes.c_uint64()
        sg.check(lib.shg_server_submit(sv, ctypes.byref(r), ctypes.byref(t)))
        assert lib.shg_server_wait(sv, t.value, 0) == 4  # DEADLINE_EXCEEDED
        sg.check(lib.shg_server_wait(sv, t.value, 60_000_000))
        done = ctypes.c_int()
        assert lib.shg_server_poll(sv, t.value, ctypes.byref(done)) == 0 and done.value == 1
        assert lib.shg_server_wait(sv, 12345, 0) == 3  # unknown ticket
    finally:
        lib.shg_server_destroy(sv)


def test_server_config_is_validated_before_device_work(sg):
    lib = sg.lib()
    h = ctypes.c_void_p()
    for cfg in [sg.ServerConfig(0, 8, 100, 2), sg.ServerConfig(1 << 20, 0, 100, 2),
                sg.ServerConfig(1 << 20, 8, -1, 2), sg.ServerConfig(1 << 20, 8, 100, 0)]:
        assert lib.shg_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 3
        assert b"bad server configuration" in lib.shg_last_error()
