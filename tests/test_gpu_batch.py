"""Uneven-batch executor (include/shell_gpu_batch.h) on the GPU.

A batch mixes ct-mult+relin, rotations and modulus switches over contexts of
different ring degree and limb count, with operands scattered through one
device arena in shuffled order.  Every result must equal the one-call-per-op
entry points (themselves pinned to the oracle in test_gpu_parity.py) and,
for a sample, the oracle directly; the same holds after CUDA-graph capture
and replay and after autotuning.
"""
import ctypes
import random

import numpy as np
import pytest

from conftest import Q50

pytestmark = pytest.mark.gpu

SHAPES = [(11, 2), (12, 3), (13, 1), (14, 2), (15, 2)]  # (log_n, limbs)
LOG_B = 20


class Arena:
    """One device allocation handing out 256-byte aligned blocks."""

    def __init__(self, sg, nbytes):
        self.buf = sg.DeviceBuffer(nbytes)
        self.off = 0

    def take(self, nbytes):
        p = self.buf.ptr + self.off
        self.off += (nbytes + 255) // 256 * 256
        assert self.off <= self.buf.nbytes
        return p


def _fill(sg, ctx, ptr, count, L, seed):
    sg.check(sg.lib().shg_poly_fill_uniform(ctx.h, ptr, count, L, seed, None))


def _download(sg, ptr, shape):
    out = np.empty(shape, np.uint64)
    sg.check(sg.lib().shg_memcpy_d2h(out.ctypes.data, ptr, out.nbytes, None))
    sg.check(sg.lib().shg_stream_synchronize(None))
    return out


def _build(sg, oracle, n_ops, seed):
    lib = sg.lib()
    rng = random.Random(seed)
    envs = {}
    for log_n, L in SHAPES:
        qs = Q50[:L]
        ctx = sg.Context(log_n, qs)
        n = 1 << log_n
        rns = oracle.Rns(log_n, qs)
        k = rns.gadget_dim([LOG_B] * L)
        kb = oracle.uniform_limbs(1000 + log_n, qs, n, k)
        ka = oracle.uniform_limbs(2000 + log_n, qs, n, k)
        relin = sg.Key(ctx, [LOG_B] * L, 1, kb, ka)
        galois = {p: sg.Key(ctx, [LOG_B] * L, p, kb, ka) for p in (5, 25)}
        envs[(log_n, L)] = dict(ctx=ctx, qs=qs, n=n, rns=rns, kb=kb, ka=ka, relin=relin,
                                galois=galois, ql_inv=ctx.ql_inv(L - 1) if L > 1 else None)
    ops = []
    for i in range(n_ops):
        log_n, L = rng.choice(SHAPES)
        r = rng.random()
        kind = 0 if r < 0.7 else (1 if r < 0.9 else 2)
        if kind == 2 and L == 1:
            kind = 0
        ops.append(dict(kind=kind, shape=(log_n, L), seed=10_000 + i,
                        power=rng.choice((5, 25))))
    total = 0
    for o in ops:
        n, L = 1 << o["shape"][0], o["shape"][1]
        total += 4 * 2 * L * n * 8 + 1024
    arena = Arena(sg, total)
    order = list(range(len(ops)))
    rng.shuffle(order)  # operands of one group end up far apart
    for i in order:
        o = ops[i]
        env = envs[o["shape"]]
        L, n = o["shape"][1], env["n"]
        ct_bytes = 2 * L * n * 8
        o["a"] = arena.take(ct_bytes)
        o["b"] = arena.take(ct_bytes)
        o["out"] = arena.take(ct_bytes)
        o["ref"] = arena.take(ct_bytes)
        _fill(sg, env["ctx"], o["a"], 2, L, o["seed"])
        _fill(sg, env["ctx"], o["b"], 2, L, o["seed"] + 1)
    sg.check(lib.shg_stream_synchronize(None))
    return envs, ops, arena


def _reference_calls(sg, envs, ops):
    """One call per operation through the per-op entry points."""
    lib = sg.lib()
    for o in ops:
        env = envs[o["shape"]]
        L = o["shape"][1]
        if o["kind"] == 0:
            sg.check(lib.shg_bgv_mul_relin(env["ctx"].h, env["relin"].h, o["ref"], o["a"], o["b"],
                                           1, None))
        elif o["kind"] == 1:
            sg.check(lib.shg_bgv_rotate(env["ctx"].h, env["galois"][o["power"]].h, o["ref"],
                                        o["a"], 1, None))
        else:
            sg.check(lib.shg_poly_modreduce_lsb(env["ctx"].h, o["ref"], o["a"], 65537,
                                                env["ql_inv"].ctypes.data_as(sg._u64p), 1, 2, L,
                                                None))
    sg.check(lib.shg_stream_synchronize(None))


def _queue(sg, envs, ops):
    lib = sg.lib()
    b = ctypes.c_void_p()
    sg.check(lib.shg_batch_create(ctypes.byref(b)))
    for o in ops:
        env = envs[o["shape"]]
        L = o["shape"][1]
        if o["kind"] == 0:
            sg.check(lib.shg_batch_add_mul_relin(b, env["ctx"].h, env["relin"].h, o["out"],
                                                 o["a"], o["b"]))
        elif o["kind"] == 1:
            sg.check(lib.shg_batch_add_rotate(b, env["ctx"].h, env["galois"][o["power"]].h,
                                              o["out"], o["a"]))
        else:
            sg.check(lib.shg_batch_add_modreduce(b, env["ctx"].h, o["out"], o["a"], 2, L, 65537,
                                                 env["ql_inv"].ctypes.data_as(sg._u64p)))
    return b


def _out_shape(o):
    log_n, L = o["shape"]
    return (2, L - 1 if o["kind"] == 2 else L, 1 << log_n)


def _check_all(sg, ops):
    for o in ops:
        shp = _out_shape(o)
        got = _download(sg, o["out"], shp)
        want = _download(sg, o["ref"], shp)
        assert np.array_equal(got, want), (o["kind"], o["shape"])


def test_fill_uniform_matches_oracle_generator(sg, oracle):
    qs, log_n = Q50[:3], 10
    ctx = sg.Context(log_n, qs)
    buf = sg.DeviceBuffer(2 * 3 * (1 << log_n) * 8)
    _fill(sg, ctx, buf.ptr, 2, 3, 12345)
    got = buf.download((2, 3, 1 << log_n))
    assert np.array_equal(got, oracle.uniform_limbs(12345, qs, 1 << log_n, 2))


def test_uneven_batch_equals_per_op_calls_and_oracle(sg, oracle):
    lib = sg.lib()
    envs, ops, arena = _build(sg, oracle, 60, seed=7)
    _reference_calls(sg, envs, ops)
    b = _queue(sg, envs, ops)
    try:
        assert lib.shg_batch_size(b) == len(ops)
        sg.check(lib.shg_batch_run(b, None))
        sg.check(lib.shg_stream_synchronize(None))
        assert lib.shg_batch_num_groups(b) > 5
        _check_all(sg, ops)
        # A sample straight against the oracle.
        for o in ops[:6]:
            env = envs[o["shape"]]
            L, n, rns = o["shape"][1], env["n"], env["rns"]
            a = _download(sg, o["a"], (2, L, n))
            if o["kind"] == 0:
                bb = _download(sg, o["b"], (2, L, n))
                want = rns.relin(rns.tensor(a, bb), env["kb"], env["ka"], [LOG_B] * L)
            elif o["kind"] == 1:
                sub = np.stack([rns.substitute(a[c], o["power"]) for c in range(2)])
                want = rns.galois(sub, env["kb"], env["ka"], [LOG_B] * L)
            else:
                want = np.stack([rns.modreduce_lsb(a[c], 65537, True) for c in range(2)])
            assert np.array_equal(_download(sg, o["out"], want.shape), want)

        # Captured and replayed: same results.
        for o in ops:
            sg.check(lib.shg_memset_device(o["out"], 0, 2 * o["shape"][1] * 8 << o["shape"][0],
                                           None))
        s = ctypes.c_void_p()
        sg.check(lib.shg_stream_create(ctypes.byref(s)))
        sg.check(lib.shg_graph_capture_begin(s))
        sg.check(lib.shg_batch_run(b, s))
        g = ctypes.c_void_p()
        sg.check(lib.shg_graph_capture_end(s, ctypes.byref(g)))
        sg.check(lib.shg_graph_launch(g, s))
        sg.check(lib.shg_stream_synchronize(s))
        _check_all(sg, ops)
        sg.check(lib.shg_graph_destroy(g))

        # Autotuned settings: still identical.
        sg.check(lib.shg_tuning_clear())
        sg.check(lib.shg_batch_autotune(b, 1, None))
        assert lib.shg_tuning_size() > 0
        sg.check(lib.shg_batch_run(b, None))
        sg.check(lib.shg_stream_synchronize(None))
        _check_all(sg, ops)
        sg.check(lib.shg_stream_destroy(s))
    finally:
        lib.shg_batch_destroy(b)
        sg.check(lib.shg_tuning_clear())


def test_contiguous_group_runs_in_place(sg, oracle):
    """Operands laid out back to back skip the gather and scatter."""
    lib = sg.lib()
    log_n, L, count = 12, 2, 5
    qs, n = Q50[:L], 1 << log_n
    ctx = sg.Context(log_n, qs)
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim([LOG_B] * L)
    kb, ka = oracle.uniform_limbs(5, qs, n, k), oracle.uniform_limbs(6, qs, n, k)
    key = sg.Key(ctx, [LOG_B] * L, 1, kb, ka)
    ct = 2 * L * n * 8
    a, bb, out, ref = (sg.DeviceBuffer(count * ct) for _ in range(4))
    _fill(sg, ctx, a.ptr, 2 * count, L, 1)
    _fill(sg, ctx, bb.ptr, 2 * count, L, 2)
    sg.check(lib.shg_bgv_mul_relin(ctx.h, key.h, ref.ptr, a.ptr, bb.ptr, count, None))
    b = ctypes.c_void_p()
    sg.check(lib.shg_batch_create(ctypes.byref(b)))
    try:
        for i in range(count):
            sg.check(lib.shg_batch_add_mul_relin(b, ctx.h, key.h, out.ptr + i * ct,
                                                 a.ptr + i * ct, bb.ptr + i * ct))
        sg.check(lib.shg_batch_run(b, None))
        sg.check(lib.shg_stream_synchronize(None))
        assert lib.shg_batch_num_groups(b) == 1
        shape = (count, 2, L, n)
        assert np.array_equal(out.download(shape), ref.download(shape))
        # aliasing and wrong key kinds are rejected
        with pytest.raises(sg.ShgError, match="alias"):
            sg.check(lib.shg_batch_add_mul_relin(b, ctx.h, key.h, a.ptr, a.ptr, bb.ptr))
        with pytest.raises(sg.ShgError, match="Galois key"):
            sg.check(lib.shg_batch_add_rotate(b, ctx.h, key.h, out.ptr, a.ptr))
    finally:
        lib.shg_batch_destroy(b)
