"""The allocation-free relinearization entry point (shg_relin_apply_noalloc).

It serves callers that may not allocate device memory while they run (memory
owned by an external pool or arena, or a latency-critical path where an
allocation's implicit synchronization is not acceptable): its scratch is a
fixed array in the library's device image.  These tests check, through the
C ABI, that it returns exactly what shg_relin_apply returns, on two calls in
a row (the second call reuses the scratch the first one left behind), and
that it rejects shapes whose scratch exceeds the fixed array.  The file name
makes pytest collect it last.
"""
import numpy as np
import pytest

from conftest import Q45, Q50

pytestmark = pytest.mark.gpu


def _inputs(oracle, qs, log_n, log_bs, count, seed):
    n = 1 << log_n
    k = sum((q.bit_length() + b - 1) // b for q, b in zip(qs, log_bs))
    kb = oracle.uniform_limbs(seed, qs, n, k)
    ka = oracle.uniform_limbs(seed + 1, qs, n, k)
    ct3 = oracle.uniform_limbs(seed + 2, qs, n, 3 * count).reshape(count, 3, len(qs), n)
    return kb, ka, ct3


@pytest.mark.parametrize("log_n,qs,log_bs,count,ks_fused", [
    (12, Q50[:4], [20] * 4, 3, 1),
    (14, Q45, [20] * 6, 3, 1),   # 14.9 MiB per ciphertext: chunks of two
    (14, Q45, [20] * 6, 3, 0),   # the separate digit-NTT and inner-product kernels
    # 60-bit primes: canonical digit transforms, one digit per REDC
    (14, [1152921504606584833, 1152921504598720513], [30, 30], 2, 1),
])
def test_noalloc_matches_relin_apply_twice(sg, oracle, log_n, qs, log_bs, count, ks_fused):
    lib = sg.lib()
    ctx = sg.Context(log_n, qs)
    sg.check(lib.shg_context_set_ks_fused(ctx.h, ks_fused))
    kb, ka, _ = _inputs(oracle, qs, log_n, log_bs, count, 300)
    key = sg.Key(ctx, log_bs, 1, kb, ka)
    shape = (count, 2, len(qs), 1 << log_n)
    for call, seed in enumerate((310, 320)):
        _, _, ct3 = _inputs(oracle, qs, log_n, log_bs, count, seed)
        d = sg.DeviceBuffer.from_array(ct3)
        want = sg.DeviceBuffer(int(np.prod(shape)) * 8)
        got = sg.DeviceBuffer(int(np.prod(shape)) * 8)
        sg.check(lib.shg_relin_apply(ctx.h, key.h, want.ptr, d.ptr, count, None))
        sg.check(lib.shg_relin_apply_noalloc(ctx.h, key.h, got.ptr, d.ptr, count, None))
        sg.synchronize()
        w, g = want.download(shape), got.download(shape)
        assert np.array_equal(g, w), f"call {call}"


def test_noalloc_rejects_oversized_shape(sg, oracle):
    # n = 2^14, 12 limbs, dimension 36: 58 MiB of scratch per ciphertext.
    qs, log_n, log_bs = Q50, 14, [20] * 12
    ctx = sg.Context(log_n, qs)
    n = 1 << log_n
    k = 36
    kb = oracle.uniform_limbs(1, qs, n, k)
    key = sg.Key(ctx, log_bs, 1, kb, kb)
    d = sg.DeviceBuffer(3 * len(qs) * n * 8)
    out = sg.DeviceBuffer(2 * len(qs) * n * 8)
    with pytest.raises(sg.ShgError, match="fixed scratch holds"):
        sg.check(sg.lib().shg_relin_apply_noalloc(ctx.h, key.h, out.ptr, d.ptr, 1, None))
