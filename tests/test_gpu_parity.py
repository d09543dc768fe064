"""GPU parity tests: every entry point of include/shell_gpu.h against the CPU
oracle (a restatement of google/shell-encryption's algorithms, pinned to the
reference by tests/golden), bit for bit, on seeded inputs.

Mirrors the reference's own tests: NTT round trip and delta -> constant
(dft_transformations_test.cc:84-140), NTT product == negacyclic schoolbook
(polynomial_test.cc:310-337), Substitute (polynomial_test.cc:487-505), RNS
pointwise ops (rns/rns_polynomial_test.cc:618-1110), ModReduceLsb
(rns/rns_polynomial_test.cc:1150-1450), key switching
(rns/rns_relinearization_key_test.cc, rns/rns_galois_key_test.cc) and
oblivious expansion (oblivious_expand_test.cc:219-259).
"""
import numpy as np
import pytest

from conftest import P58, Q45, Q50, Q59, Q60

pytestmark = pytest.mark.gpu


def _run(sg, fn, *args):
    sg.check(fn(*args))
    sg.synchronize()


def _dev(sg, arr):
    return sg.DeviceBuffer.from_array(arr)


# --------------------------------------------------------------------------
# Context parameters
# --------------------------------------------------------------------------

@pytest.mark.parametrize("q,log_n", [(Q45[0], 14), (Q50[3], 11), (Q59, 12), (Q60, 12),
                                     (Q45[5], 3), (Q50[0], 1)])
def test_context_tables_match_reference(sg, oracle, q, log_n):
    ctx = sg.Context(log_n, [q])
    p = oracle.Prime(q, log_n)
    info_gpu = ctx.prime_info(0)
    info_ref = p.info()
    assert [int(x) for x in info_gpu] == [info_ref[k] for k in
                                          ["q", "log_q", "inv_modulus", "r_mod_q",
                                           "r_mod_q_barrett", "inv_r", "inv_r_barrett",
                                           "barrett_num", "psi", "n_inv"]]
    f_gpu, i_gpu = ctx.ntt_tables(0)
    f_ref, i_ref = p.tables()
    assert np.array_equal(f_gpu, f_ref)
    assert np.array_equal(i_gpu, i_ref)


def test_context_validation(sg):
    with pytest.raises(sg.ShgError, match="less than 2\\^62"):
        sg.Context(4, [1 << 62 | 1])
    with pytest.raises(sg.ShgError, match="should be odd"):
        sg.Context(4, [1 << 40])
    with pytest.raises(sg.ShgError, match="not 1 mod 2n"):
        sg.Context(14, [Q59])  # 2^13 | q-1 only
    with pytest.raises(sg.ShgError, match="plaintext_modulus"):
        sg.Context(4, [Q45[0]], t=0)
    with pytest.raises(sg.ShgError, match="must be positive"):
        sg.Context(0, [Q45[0]])


# --------------------------------------------------------------------------
# NTT
# --------------------------------------------------------------------------

NTT_CASES = [(log_n, qs) for log_n in range(1, 15) for qs in ([Q45[0], Q45[1]],)] + [
    (12, [Q59]), (12, [Q60]), (11, Q50[:4]), (13, Q50[:3]), (14, Q45), (15, Q50[:2]),
    (15, [Q50[5]])]


@pytest.mark.parametrize("log_n,four_step_min", [(12, 12), (12, 16), (13, 13), (13, 16),
                                                   (14, 14), (14, 15)])
def test_ntt_both_kernels(sg, oracle, log_n, four_step_min):
    """n = 2^12 .. 2^14 run either on the one-CTA-per-limb kernels or on the
    two-phase four-step kernels (the threshold picks); every fused operation
    is exact on both: NTT round trip, ct-mult+relin, rotation, ModReduceLsb."""
    qs, n = Q45[:3], 1 << log_n
    x = oracle.uniform_limbs(77, qs, n, 2)
    rns = oracle.Rns(log_n, qs)
    ctx = sg.Context(log_n, qs)
    lib = sg.lib()
    sg.check(lib.shg_context_set_four_step_min(ctx.h, four_step_min))
    d = _dev(sg, x)
    _run(sg, lib.shg_ntt_forward, ctx.h, d.ptr, 2, 3, None)
    assert np.array_equal(d.download(x.shape), np.stack([rns.ntt_fwd(x[i]) for i in range(2)]))
    _run(sg, lib.shg_ntt_inverse, ctx.h, d.ptr, 2, 3, None)
    assert np.array_equal(d.download(x.shape), x)
    k = rns.gadget_dim([20] * 3)
    kb, ka = oracle.uniform_limbs(78, qs, n, k), oracle.uniform_limbs(79, qs, n, k)
    a, b = _ct_pair(oracle, qs, n, 2, 80)
    want = np.stack([rns.relin(rns.tensor(a[i], b[i]), kb, ka, [20] * 3) for i in range(2)])
    key = sg.Key(ctx, [20] * 3, 1, kb, ka)
    da, db, out = _dev(sg, a), _dev(sg, b), sg.DeviceBuffer(a.nbytes)
    _run(sg, lib.shg_bgv_mul_relin, ctx.h, key.h, out.ptr, da.ptr, db.ptr, 2, None)
    assert np.array_equal(out.download(want.shape), want)
    power = 5
    gkey = sg.Key(ctx, [20] * 3, power, kb, ka)
    sub = np.stack([np.stack([rns.substitute(a[i, c], power) for c in range(2)])
                    for i in range(2)])
    want_rot = np.stack([rns.galois(sub[i], kb, ka, [20] * 3) for i in range(2)])
    _run(sg, lib.shg_bgv_rotate, ctx.h, gkey.h, out.ptr, da.ptr, 2, None)
    assert np.array_equal(out.download(want_rot.shape), want_rot)
    ql_inv = ctx.ql_inv(2)
    want_mr = np.stack([rns.modreduce_lsb(a[i, c], 65537, True) for i in range(2)
                        for c in range(2)])
    mr = sg.DeviceBuffer(want_mr.nbytes)
    _run(sg, lib.shg_poly_modreduce_lsb, ctx.h, mr.ptr, da.ptr, 65537,
         ql_inv.ctypes.data_as(sg._u64p), 1, 4, 3, None)
    assert np.array_equal(mr.download(want_mr.shape), want_mr)


@pytest.mark.parametrize("log_n,qs", NTT_CASES)
def test_ntt_forward_inverse(sg, oracle, log_n, qs):
    n = 1 << log_n
    count = 3
    x = oracle.uniform_limbs(100 + log_n, qs, n, count)
    rns = oracle.Rns(log_n, qs)
    want = np.stack([rns.ntt_fwd(x[i]) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    d = _dev(sg, x)
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, d.ptr, count, len(qs), None)
    got = d.download(x.shape)
    assert np.array_equal(got, want)
    _run(sg, sg.lib().shg_ntt_inverse, ctx.h, d.ptr, count, len(qs), None)
    assert np.array_equal(d.download(x.shape), x)
    # inverse alone vs oracle on fresh data
    y = oracle.uniform_limbs(200 + log_n, qs, n, count)
    want_inv = np.stack([rns.ntt_inv(y[i]) for i in range(count)])
    d2 = _dev(sg, y)
    _run(sg, sg.lib().shg_ntt_inverse, ctx.h, d2.ptr, count, len(qs), None)
    assert np.array_equal(d2.download(y.shape), want_inv)


def test_ntt_delta_is_constant(sg, oracle):
    """dft_transformations_test.cc:84-110: NTT(delta) is a constant vector."""
    q, log_n = Q50[0], 13
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    one = p.import_(np.array([1], np.uint64))[0]
    x = np.zeros((1, 1, n), np.uint64)
    x[0, 0, 0] = one
    ctx = sg.Context(log_n, [q])
    d = _dev(sg, x)
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, d.ptr, 1, 1, None)
    got = d.download(x.shape)
    assert np.all(got == one)


def test_ntt_product_is_negacyclic_schoolbook(sg, oracle):
    """polynomial_test.cc:310-337."""
    q, log_n = Q59, 6
    n = 1 << log_n
    rng = np.random.default_rng(5)
    a = rng.integers(0, q, n, dtype=np.uint64)
    b = rng.integers(0, q, n, dtype=np.uint64)
    p = oracle.Prime(q, log_n)
    ctx = sg.Context(log_n, [q])
    da = _dev(sg, p.import_(a).reshape(1, 1, n))
    db = _dev(sg, p.import_(b).reshape(1, 1, n))
    lib = sg.lib()
    for d in (da, db):
        _run(sg, lib.shg_ntt_forward, ctx.h, d.ptr, 1, 1, None)
    _run(sg, lib.shg_poly_mul, ctx.h, da.ptr, da.ptr, db.ptr, 1, 1, None)
    _run(sg, lib.shg_ntt_inverse, ctx.h, da.ptr, 1, 1, None)
    got = [int(v) for v in p.export(da.download((n,)))]
    ai, bi = [int(v) for v in a], [int(v) for v in b]
    ref = [0] * n
    for i in range(n):
        for j in range(n):
            k = i + j
            if k >= n:
                ref[k - n] -= ai[i] * bi[j]
            else:
                ref[k] += ai[i] * bi[j]
    assert got == [r % q for r in ref]


# --------------------------------------------------------------------------
# Pointwise ops
# --------------------------------------------------------------------------

@pytest.mark.parametrize("log_n,qs", [(4, Q45[:2]), (12, Q50[:5]), (14, Q45)])
def test_pointwise_ops(sg, oracle, log_n, qs):
    n = 1 << log_n
    count, L = 2, len(qs)
    a = oracle.uniform_limbs(7, qs, n, count)
    b = oracle.uniform_limbs(8, qs, n, count)
    a[0, 0, :4] = 0  # negation of zero yields q in the reference
    c = oracle.uniform_limbs(9, qs, n, count)
    rns = oracle.Rns(log_n, qs)
    P = rns.primes
    ctx = sg.Context(log_n, qs)
    lib = sg.lib()
    da, db, dc = _dev(sg, a), _dev(sg, b), _dev(sg, c)
    out = sg.DeviceBuffer(a.nbytes)

    def per_limb(fn):
        return np.stack([np.stack([fn(P[l], i, l) for l in range(L)]) for i in range(count)])

    cases = {
        "add": (lib.shg_poly_add, (out.ptr, da.ptr, db.ptr),
                per_limb(lambda p, i, l: p.add(a[i, l], b[i, l]))),
        "sub": (lib.shg_poly_sub, (out.ptr, da.ptr, db.ptr),
                per_limb(lambda p, i, l: p.sub(a[i, l], b[i, l]))),
        "mul": (lib.shg_poly_mul, (out.ptr, da.ptr, db.ptr),
                per_limb(lambda p, i, l: p.mul(a[i, l], b[i, l]))),
    }
    for name, (fn, args, want) in cases.items():
        _run(sg, fn, ctx.h, *args, count, L, None)
        assert np.array_equal(out.download(a.shape), want), name
    _run(sg, lib.shg_poly_neg, ctx.h, out.ptr, da.ptr, count, L, None)
    want = per_limb(lambda p, i, l: p.neg(a[i, l]))
    got = out.download(a.shape)
    assert np.array_equal(got, want)
    assert int(got[0, 0, 0]) == qs[0]
    # neg output (holding q) fed back into add / mul stays exact
    _run(sg, lib.shg_poly_add, ctx.h, out.ptr, out.ptr, out.ptr, count, L, None)
    want2 = per_limb(lambda p, i, l: p.add(want[i, l], want[i, l]))
    assert np.array_equal(out.download(a.shape), want2)
    # fma: c += a*b
    _run(sg, lib.shg_poly_fma, ctx.h, dc.ptr, da.ptr, db.ptr, count, L, None)
    want = per_limb(lambda p, i, l: p.fma(c[i, l], a[i, l], b[i, l]))
    assert np.array_equal(dc.download(a.shape), want)
    # RNS scalar (Montgomery) and integer scalar
    sc = np.array([P[l].import_(np.array([12345 + l], np.uint64))[0] for l in range(L)],
                  np.uint64)
    _run(sg, lib.shg_poly_mul_rns_scalar, ctx.h, out.ptr, da.ptr, sc.ctypes.data_as(
        __import__("ctypes").POINTER(__import__("ctypes").c_uint64)), count, L, None)
    want = per_limb(lambda p, i, l: p.mul_scalar(a[i, l], sc[l]))
    assert np.array_equal(out.download(a.shape), want)
    _run(sg, lib.shg_poly_mul_integer, ctx.h, out.ptr, da.ptr, 65537, count, L, None)
    want = per_limb(lambda p, i, l: p.mul_scalar(a[i, l], p.import_(np.array([65537],
                                                                              np.uint64))[0]))
    assert np.array_equal(out.download(a.shape), want)


# --------------------------------------------------------------------------
# Substitute
# --------------------------------------------------------------------------

@pytest.mark.parametrize("log_n,power", [(3, 3), (6, 5), (10, 1023), (12, 4097), (14, 5),
                                         (14, 2 * 16384 - 1), (13, 1), (15, 5)])
def test_substitute(sg, oracle, log_n, power):
    qs = Q45[:3] if log_n < 15 else Q50[:3]
    n = 1 << log_n
    x = oracle.uniform_limbs(31, qs, n, 2)
    rns = oracle.Rns(log_n, qs)
    want = np.stack([rns.substitute(x[i], power) for i in range(2)])
    ctx = sg.Context(log_n, qs)
    d, out = _dev(sg, x), sg.DeviceBuffer(x.nbytes)
    _run(sg, sg.lib().shg_poly_substitute, ctx.h, out.ptr, d.ptr, power, 2, len(qs), None)
    assert np.array_equal(out.download(x.shape), want)


def test_substitute_validation(sg):
    ctx = sg.Context(4, [Q45[0]])
    d, out = sg.DeviceBuffer(16 * 8), sg.DeviceBuffer(16 * 8)
    for bad in (2, -1, 32, 33):
        with pytest.raises(sg.ShgError, match="Substitution power"):
            sg.check(sg.lib().shg_poly_substitute(ctx.h, out.ptr, d.ptr, bad, 1, 1, None))


# --------------------------------------------------------------------------
# Ciphertext tensor, key switching
# --------------------------------------------------------------------------

def _ct_pair(oracle, qs, n, count, seed):
    a = oracle.uniform_limbs(seed, qs, n, 2 * count).reshape(count, 2, len(qs), n)
    b = oracle.uniform_limbs(seed + 1, qs, n, 2 * count).reshape(count, 2, len(qs), n)
    return a, b


@pytest.mark.parametrize("log_n,qs", [(5, Q45[:2]), (12, Q50[:4]), (14, Q45), (15, Q50[:2])])
def test_tensor(sg, oracle, log_n, qs):
    n, count = 1 << log_n, 2
    a, b = _ct_pair(oracle, qs, n, count, 40)
    rns = oracle.Rns(log_n, qs)
    want = np.stack([rns.tensor(a[i], b[i]) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    da, db = _dev(sg, a), _dev(sg, b)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_ct_tensor, ctx.h, out.ptr, da.ptr, db.ptr, count, len(qs), None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.parametrize("log_n,qs,log_bs", [
    (4, Q45[:2], [20, 20]), (10, Q45, [20] * 6), (11, Q50[:2], [50, 16]),
    (12, Q50[:3], [7, 13, 62]), (14, Q45[:3], [20, 20, 20])])
def test_gadget_decompose(sg, oracle, log_n, qs, log_bs):
    n, L, count = 1 << log_n, len(qs), 2
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    a = oracle.uniform_limbs(45, qs, n, count).reshape(count, L, n)
    want = np.stack([rns.decompose(a[i], log_bs) for i in range(count)])
    assert want.shape == (count, k, L, n)
    ctx = sg.Context(log_n, qs)
    lib = sg.lib()
    lb = np.array(log_bs, np.int32)
    d = _dev(sg, a)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, lib.shg_gadget_decompose, ctx.h, L, lb.ctypes.data_as(sg._ip), out.ptr, d.ptr,
         count, None)
    assert np.array_equal(out.download(want.shape), want)


KS_CASES = [
    (4, Q45[:2], [20, 20]),
    (10, Q45[:3], [20, 20, 20]),
    (12, Q50[:4], [20, 20, 20, 20]),
    (11, Q50[:2], [50, 16]),        # a full-width digit exercises the balanced lift
    (14, Q45, [20] * 6),           # the ct-mult+relin workload's parameters
    (15, Q50[:3], [20] * 3),
    (15, Q50[:2], [50, 16]),
    (14, Q45[:2], [2, 2]),          # 46 digits: one row per CTA, partial last warp
    (14, Q45[:2], [1, 1]),          # 90 digits: too many for one CTA, unfused path
    (14, P58[:2], [10, 10]),        # primes just below 2^58: lazy digits, 2 per REDC
    (11, P58[:2], [10, 10]),        # the same in the CTA-resident path
    (14, Q45[:4], [6] * 4),         # 32 digits: 512 threads, the 8-value row kernel's most
    (14, [1152921504606584833, 1152921504598720513], [30, 30]),  # 60-bit: canonical digits
]


@pytest.mark.parametrize("ks_fused", [1, 0])
@pytest.mark.parametrize("log_n,qs,log_bs", KS_CASES)
def test_relin_plain_and_fused(sg, oracle, log_n, qs, log_bs, ks_fused):
    if log_n < 13 and not ks_fused:
        pytest.skip("below the four-step threshold (n < 2^13) the key switch has one path; "
                    "ks_fused chooses between the four-step row kernels")
    n, L = 1 << log_n, len(qs)
    count = 2
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    kb = oracle.uniform_limbs(50, qs, n, k)
    ka = oracle.uniform_limbs(51, qs, n, k)
    a, b = _ct_pair(oracle, qs, n, count, 52)
    ct3 = np.stack([rns.tensor(a[i], b[i]) for i in range(count)])
    want = np.stack([rns.relin(ct3[i], kb, ka, log_bs) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    lib = sg.lib()
    sg.check(lib.shg_context_set_ks_fused(ctx.h, ks_fused))
    key = sg.Key(ctx, log_bs, 1, kb, ka)
    assert key.dimension == k
    d3 = _dev(sg, ct3)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, lib.shg_relin_apply, ctx.h, key.h, out.ptr, d3.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want)
    da, db = _dev(sg, a), _dev(sg, b)
    out2 = sg.DeviceBuffer(want.nbytes)
    _run(sg, lib.shg_bgv_mul_relin, ctx.h, key.h, out2.ptr, da.ptr, db.ptr, count, None)
    assert np.array_equal(out2.download(want.shape), want)


def test_relin_odd_batch(sg, oracle):
    """Three ciphertexts at n = 2^14 through the fused key switch."""
    log_n, qs, log_bs, count = 14, Q45[:3], [20] * 3, 3
    n = 1 << log_n
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    kb = oracle.uniform_limbs(53, qs, n, k)
    ka = oracle.uniform_limbs(54, qs, n, k)
    a, b = _ct_pair(oracle, qs, n, count, 55)
    want = np.stack([rns.relin(rns.tensor(a[i], b[i]), kb, ka, log_bs) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    key = sg.Key(ctx, log_bs, 1, kb, ka)
    da, db = _dev(sg, a), _dev(sg, b)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_bgv_mul_relin, ctx.h, key.h, out.ptr, da.ptr, db.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.parametrize("log_n,qs,log_bs,power", [
    (4, Q45[:2], [20, 20], 5), (12, Q50[:3], [20, 20, 20], 5 ** 3 % 8192),
    (13, Q50[:2], [50, 50], 8191), (14, Q45, [20] * 6, 5), (15, Q50[:2], [20, 20], 25)])
@pytest.mark.parametrize("ks_fused", [1, 0])
def test_galois_and_rotate(sg, oracle, log_n, qs, log_bs, power, ks_fused):
    if log_n < 13 and not ks_fused:
        pytest.skip("below the four-step threshold (n < 2^13) the key switch has one path; "
                    "ks_fused chooses between the four-step row kernels")
    n, L, count = 1 << log_n, len(qs), 2
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    kb = oracle.uniform_limbs(60, qs, n, k)
    ka = oracle.uniform_limbs(61, qs, n, k)
    ct = oracle.uniform_limbs(62, qs, n, 2 * count).reshape(count, 2, L, n)
    want = np.stack([rns.galois(ct[i], kb, ka, log_bs) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    lib = sg.lib()
    sg.check(lib.shg_context_set_ks_fused(ctx.h, ks_fused))
    key = sg.Key(ctx, log_bs, power, kb, ka)
    d = _dev(sg, ct)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, lib.shg_galois_apply, ctx.h, key.h, out.ptr, d.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want)
    # rotate = Substitute(power) then Galois key switch
    sub = np.stack([np.stack([rns.substitute(ct[i, c], power) for c in range(2)])
                    for i in range(count)])
    want_rot = np.stack([rns.galois(sub[i], kb, ka, log_bs) for i in range(count)])
    _run(sg, lib.shg_bgv_rotate, ctx.h, key.h, out.ptr, d.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want_rot)


def test_relin_rejects_galois_key(sg, oracle):
    qs, log_n = Q45[:2], 4
    n = 1 << log_n
    kb = oracle.uniform_limbs(1, qs, n, 6)
    ctx = sg.Context(log_n, qs)
    key = sg.Key(ctx, [20, 20], 5, kb, kb)
    d = sg.DeviceBuffer(3 * 2 * n * 8)
    out = sg.DeviceBuffer(2 * 2 * n * 8)
    with pytest.raises(sg.ShgError, match="power 1"):
        sg.check(sg.lib().shg_relin_apply(ctx.h, key.h, out.ptr, d.ptr, 1, None))


# --------------------------------------------------------------------------
# ModReduceLsb
# --------------------------------------------------------------------------

@pytest.mark.parametrize("log_n,qs,is_ntt", [(4, Q45[:2], 1), (12, Q50[:5], 1),
                                             (14, Q45, 1), (10, Q50[:4], 0), (14, Q45, 0),
                                             (15, Q50[:3], 1), (15, Q50[:3], 0),
                                             (14, P58, 1)])
def test_modreduce_lsb(sg, oracle, log_n, qs, is_ntt):
    n, L, count, t = 1 << log_n, len(qs), 3, 65537
    x = oracle.uniform_limbs(70, qs, n, count)
    rns = oracle.Rns(log_n, qs)
    want = np.stack([rns.modreduce_lsb(x[i], t, bool(is_ntt)) for i in range(count)])
    ctx = sg.Context(log_n, qs, t)
    ql_inv = ctx.ql_inv(L - 1)
    assert np.array_equal(ql_inv, rns.ql_inv(L - 1))
    d = _dev(sg, x)
    out = sg.DeviceBuffer(want.nbytes)
    import ctypes
    _run(sg, sg.lib().shg_poly_modreduce_lsb, ctx.h, out.ptr, d.ptr, t,
         ql_inv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), is_ntt, count, L, None)
    assert np.array_equal(out.download(want.shape), want)


# --------------------------------------------------------------------------
# Single-modulus key switching, oblivious expansion, absorb
# --------------------------------------------------------------------------

@pytest.mark.parametrize("q,log_n,log_b", [(Q60, 7, 10), (Q60, 12, 8), (Q59, 9, 16)])
def test_single_modulus_galois(sg, oracle, q, log_n, log_b):
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    dim = p.gadget_size(log_b)
    k0 = oracle.uniform_limbs(80, [q], n, dim).reshape(dim, n)
    k1 = oracle.uniform_limbs(81, [q], n, dim).reshape(dim, n)
    ct = oracle.uniform_limbs(82, [q], n, 2).reshape(2, n)
    want = p.galois_apply(log_b, ct, k0, k1)
    ctx = sg.Context(log_n, [q])
    key = sg.Key(ctx, [log_b], (n >> 1) + 1, k0, k1)
    d = _dev(sg, ct)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_galois_apply, ctx.h, key.h, out.ptr, d.ptr, 1, None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.parametrize("q,log_n,levels,log_b,count", [(Q60, 7, 3, 10, 2), (Q60, 8, 8, 8, 1),
                                                        (Q60, 12, 4, 8, 2)])
def test_oblivious_expand(sg, oracle, q, log_n, levels, log_b, count):
    import ctypes
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    dim = p.gadget_size(log_b)
    keys = oracle.uniform_limbs(90, [q], n, levels * 2 * dim).reshape(levels, 2, dim, n)
    cts = oracle.uniform_limbs(91, [q], n, 2 * count).reshape(count, 2, n)
    want = np.stack([p.oblivious_expand(levels, log_b, keys, cts[i]) for i in range(count)])
    ctx = sg.Context(log_n, [q])
    gkeys = [sg.Key(ctx, [log_b], (n >> j) + 1, keys[j, 0], keys[j, 1]) for j in range(levels)]
    arr = (ctypes.c_void_p * levels)(*[k.h for k in gkeys])
    d = _dev(sg, cts)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_oblivious_expand, ctx.h, arr, levels, out.ptr, d.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want)


def test_absorb_sum(sg, oracle):
    q, log_n, items, count = Q60, 10, 37, 2
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    cts = oracle.uniform_limbs(95, [q], n, count * items * 2).reshape(count, items, 2, n)
    db = oracle.uniform_limbs(96, [q], n, items).reshape(items, n)
    want = np.stack([p.absorb_sum(cts[i], db) for i in range(count)])
    ctx = sg.Context(log_n, [q])
    dc, dd = _dev(sg, cts), _dev(sg, db)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_absorb_sum, ctx.h, out.ptr, dc.ptr, dd.ptr, items, count, None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.parametrize("log_n,levels,log_b,items,count", [
    (7, 3, 10, 8, 3), (9, 5, 8, 27, 2), (12, 4, 8, 16, 33), (12, 10, 8, 1024, 17)])
def test_pir_expand_absorb(sg, oracle, log_n, levels, log_b, items, count):
    """Expansion to `items` ciphertexts then the database absorb-sum, in one
    call.  At n=2^12 with 10 levels (the PIR workload's shape) a query's
    expansion is 64 MiB, so 17 queries take two groups of the 1 GiB scratch."""
    import ctypes
    q, n = Q60, 1 << log_n
    p = oracle.Prime(q, log_n)
    dim = p.gadget_size(log_b)
    keys = oracle.uniform_limbs(97, [q], n, levels * 2 * dim).reshape(levels, 2, dim, n)
    cts = oracle.uniform_limbs(98, [q], n, 2 * count).reshape(count, 2, n)
    db = oracle.uniform_limbs(99, [q], n, items).reshape(items, n)
    want = np.stack([p.absorb_sum(p.oblivious_expand(levels, log_b, keys, cts[i])[:items], db)
                     for i in range(count)])
    ctx = sg.Context(log_n, [q])
    gkeys = [sg.Key(ctx, [log_b], (n >> j) + 1, keys[j, 0], keys[j, 1]) for j in range(levels)]
    arr = (ctypes.c_void_p * levels)(*[k.h for k in gkeys])
    dc, dd = _dev(sg, cts), _dev(sg, db)
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_pir_expand_absorb, ctx.h, arr, levels, dd.ptr, items, out.ptr,
         dc.ptr, count, None)
    assert np.array_equal(out.download(want.shape), want)
    with pytest.raises(sg.ShgError, match="Output length must be at most"):
        sg.check(sg.lib().shg_pir_expand_absorb(ctx.h, arr, levels, dd.ptr, (1 << levels) + 1,
                                                out.ptr, dc.ptr, count, None))


@pytest.mark.parametrize("log_n,qs,log_bs,ks_fused", [
    (12, Q50[:3], [20] * 3, 1), (14, Q45, [20] * 6, 1), (14, Q45, [20] * 6, 0),
    (13, Q50[:2], [50, 16], 1)])
def test_multikey_batches_equal_per_key_calls(sg, oracle, log_n, qs, log_bs, ks_fused):
    """Members with their own keys (one per client) in one batch: identical to
    one call per key, for ct-mult+relin and rotation."""
    import ctypes
    lib = sg.lib()
    n, L, count = 1 << log_n, len(qs), 5
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    ctx = sg.Context(log_n, qs)
    sg.check(lib.shg_context_set_ks_fused(ctx.h, ks_fused))
    if log_n < 14:
        sg.check(lib.shg_context_set_four_step_min(ctx.h, log_n))  # four-step at small n too
    mats = [(oracle.uniform_limbs(300 + i, qs, n, k), oracle.uniform_limbs(400 + i, qs, n, k))
            for i in range(3)]
    relin = [sg.Key(ctx, log_bs, 1, kb, ka) for kb, ka in mats]
    galois = [sg.Key(ctx, log_bs, 5, kb, ka) for kb, ka in mats]
    pick = [0, 2, 1, 2, 0]
    a, b = _ct_pair(oracle, qs, n, count, 500)
    da, db = _dev(sg, a), _dev(sg, b)
    want = sg.DeviceBuffer(a.nbytes)
    got = sg.DeviceBuffer(a.nbytes)
    ct = 2 * L * n * 8
    for i, kidx in enumerate(pick):
        sg.check(lib.shg_bgv_mul_relin(ctx.h, relin[kidx].h, want.ptr + i * ct, da.ptr + i * ct,
                                       db.ptr + i * ct, 1, None))
    arr = (ctypes.c_void_p * count)(*[relin[kidx].h for kidx in pick])
    _run(sg, lib.shg_bgv_mul_relin_multikey, ctx.h, arr, got.ptr, da.ptr, db.ptr, count, None)
    assert np.array_equal(got.download(a.shape), want.download(a.shape))
    # first member against the oracle as well
    w0 = rns.relin(rns.tensor(a[0], b[0]), mats[pick[0]][0], mats[pick[0]][1], log_bs)
    assert np.array_equal(got.download(a.shape)[0], w0)
    for i, kidx in enumerate(pick):
        sg.check(lib.shg_bgv_rotate(ctx.h, galois[kidx].h, want.ptr + i * ct, da.ptr + i * ct,
                                    1, None))
    arr = (ctypes.c_void_p * count)(*[galois[kidx].h for kidx in pick])
    _run(sg, lib.shg_bgv_rotate_multikey, ctx.h, arr, got.ptr, da.ptr, count, None)
    assert np.array_equal(got.download(a.shape), want.download(a.shape))
    # keys of different powers cannot share a batch
    bad = (ctypes.c_void_p * 2)(relin[0].h, galois[1].h)
    with pytest.raises(sg.ShgError, match="share"):
        sg.check(lib.shg_bgv_rotate_multikey(ctx.h, bad, got.ptr, da.ptr, 2, None))


def test_pir_multikey_equals_per_query_calls(sg, oracle):
    import ctypes
    lib = sg.lib()
    q, log_n, levels, log_b, items, count = Q60, 9, 5, 8, 20, 4
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    dim = p.gadget_size(log_b)
    ctx = sg.Context(log_n, [q])
    clients = []
    for c in range(3):
        keys = oracle.uniform_limbs(600 + c, [q], n, levels * 2 * dim).reshape(levels, 2, dim, n)
        clients.append((keys, [sg.Key(ctx, [log_b], (n >> j) + 1, keys[j, 0], keys[j, 1])
                               for j in range(levels)]))
    pick = [1, 0, 2, 1]
    cts = oracle.uniform_limbs(700, [q], n, 2 * count).reshape(count, 2, n)
    db = oracle.uniform_limbs(701, [q], n, items).reshape(items, n)
    dc, dd = _dev(sg, cts), _dev(sg, db)
    flat = [clients[c][1][j].h for c in pick for j in range(levels)]
    arr = (ctypes.c_void_p * len(flat))(*flat)
    out = sg.DeviceBuffer(count * 2 * n * 8)
    _run(sg, lib.shg_pir_expand_absorb_multikey, ctx.h, arr, levels, dd.ptr, items, out.ptr,
         dc.ptr, count, None)
    got = out.download((count, 2, n))
    for i, c in enumerate(pick):
        keys = clients[c][0]
        want = p.absorb_sum(p.oblivious_expand(levels, log_b, keys, cts[i])[:items], db)
        assert np.array_equal(got[i], want)


def _cbd(rng, n, variance=8):
    """Centred binomial samples of the given variance (sample_error.h:43-100's
    distribution; drawn here with numpy, the device path never samples)."""
    k = 2 * variance
    bits = rng.integers(0, 2, size=(n, 2 * k))
    return bits[:, :k].sum(1) - bits[:, k:].sum(1)


def test_symmetric_rlwe_flow(sg, oracle):
    """The single-modulus flow: encrypt 64 messages, NTT round trip, ct + ct,
    ct * ct, decrypt -- bit-exact with the oracle and decrypting to m1 + m2 and
    the negacyclic product m1 * m2 mod t."""
    lib = sg.lib()
    q, log_n, t, count = Q59, 12, 65537, 64
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    rng = np.random.default_rng(2024)

    def mont(v):
        return p.import_(np.array([int(x) % q for x in v], dtype=np.uint64))

    s = p.ntt_fwd(mont(_cbd(rng, n)))
    msgs = rng.integers(0, t, size=(count, n))
    m = np.stack([p.ntt_fwd(mont(msgs[i])) for i in range(count)])
    a = oracle.uniform_limbs(31, [q], n, count).reshape(count, n)
    e = np.stack([mont(_cbd(rng, n)) for _ in range(count)])
    want = np.stack([p.sym_encrypt(t, s, a[i], e[i], m[i]) for i in range(count)])
    ctx = sg.Context(log_n, [q], t)
    ds, da, de, dm = (_dev(sg, x) for x in (s, a, e, m))
    ct = sg.DeviceBuffer(want.nbytes)
    _run(sg, lib.shg_symmetric_encrypt, ctx.h, ct.ptr, ds.ptr, da.ptr, de.ptr, dm.ptr, count,
         None)
    assert np.array_equal(ct.download(want.shape), want)
    # NTT round trip of every component
    _run(sg, lib.shg_ntt_inverse, ctx.h, ct.ptr, 2 * count, 1, None)
    _run(sg, lib.shg_ntt_forward, ctx.h, ct.ptr, 2 * count, 1, None)
    assert np.array_equal(ct.download(want.shape), want)
    half = count // 2
    cts = ct.download(want.shape)
    lo, hi = _dev(sg, cts[:half]), _dev(sg, cts[half:])
    # ct + ct
    summ = sg.DeviceBuffer(half * 2 * n * 8)
    _run(sg, lib.shg_poly_add, ctx.h, summ.ptr, lo.ptr, hi.ptr, 2 * half, 1, None)
    # ct * ct (3 components)
    prod = sg.DeviceBuffer(half * 3 * n * 8)
    _run(sg, lib.shg_ct_tensor, ctx.h, prod.ptr, lo.ptr, hi.ptr, half, 1, None)
    # decrypt everything
    dec = sg.DeviceBuffer(count * n * 8)
    _run(sg, lib.shg_symmetric_decrypt, ctx.h, dec.ptr, ds.ptr, ct.ptr, 2, count, None)
    got = dec.download((count, n))
    assert np.array_equal(got, np.stack([p.sym_decrypt(t, s, want[i]) for i in range(count)]))
    assert np.array_equal(got.astype(np.int64), msgs)
    _run(sg, lib.shg_symmetric_decrypt, ctx.h, dec.ptr, ds.ptr, summ.ptr, 2, half, None)
    got = dec.download((half, n)).astype(np.int64)
    assert np.array_equal(got, (msgs[:half] + msgs[half:]) % t)
    _run(sg, lib.shg_symmetric_decrypt, ctx.h, dec.ptr, ds.ptr, prod.ptr, 3, half, None)
    got = dec.download((half, n))
    prods = prod.download((half, 3, n))
    for i in (0, 1, half - 1):
        assert np.array_equal(got[i], p.sym_decrypt(t, s, prods[i]))
        full = np.convolve(msgs[i], msgs[half + i])  # length 2n - 1
        neg = full[:n].copy()
        neg[: n - 1] -= full[n:]
        assert np.array_equal(got[i].astype(np.int64), neg % t)
    with pytest.raises(sg.ShgError, match="one-prime"):
        ctx2 = sg.Context(log_n, Q50[:2], t)
        sg.check(lib.shg_symmetric_decrypt(ctx2.h, dec.ptr, ds.ptr, ct.ptr, 2, 1, None))


@pytest.mark.parametrize("log_n,qs", [(3, Q45[:2]), (6, [65537]), (10, Q50[:3]),
                                      (14, Q45), (12, [Q59, Q60])])
def test_serialize_deserialize(sg, oracle, log_n, qs):
    """The wire format (MontgomeryInt::SerializeVector per limb): device
    streams equal the oracle's (pinned to the reference by the golden
    streams); deserializing gives the values back."""
    lib = sg.lib()
    n, L, count = 1 << log_n, len(qs), 3
    x = oracle.uniform_limbs(910 + log_n, qs, n, count)
    want = np.concatenate([oracle.Prime(q, log_n).serialize(x[c, l])
                           for c in range(count) for l, q in enumerate(qs)])
    ctx = sg.Context(log_n, qs)
    per_poly = lib.shg_poly_serialized_bytes(ctx.h, L)
    assert per_poly * count == want.size
    d = _dev(sg, x)
    buf = sg.DeviceBuffer(want.size + 16)
    _run(sg, lib.shg_poly_serialize, ctx.h, buf.ptr, d.ptr, count, L, None)
    got = np.empty(want.size, np.uint8)
    sg.check(lib.shg_memcpy_d2h(got.ctypes.data, buf.ptr, got.nbytes, None))
    sg.synchronize()
    assert np.array_equal(got, want)
    back = sg.DeviceBuffer(x.nbytes)
    sg.check(lib.shg_memcpy_h2d(buf.ptr, want.ctypes.data, want.nbytes, None))
    _run(sg, lib.shg_poly_deserialize, ctx.h, back.ptr, buf.ptr, count, L, None)
    assert np.array_equal(back.download(x.shape), x)


@pytest.mark.parametrize("piece,slots,ramp,wire", [(2, 2, 0, True), (64, 4, 0, True),
                                                   (8, 3, 3, True), (8, 3, 3, False),
                                                   (4, 2, 2, False)])
def test_mul_relin_host_pipeline(sg, oracle, piece, slots, ramp, wire):
    """Host ciphertexts in, host results out, through the piece pipeline
    (fixed pieces, or ramped: 1, 2, 4 ... ciphertexts at both ends), in the
    wire format (serialized like the reference) or as limbs: equals the
    oracle's ct-mult+relin."""
    lib = sg.lib()
    log_n, qs, log_bs = 12, Q50[:3], [20] * 3
    count = 13 if ramp else 5
    n, L = 1 << log_n, len(qs)
    rns = oracle.Rns(log_n, qs)
    k = rns.gadget_dim(log_bs)
    kb, ka = oracle.uniform_limbs(21, qs, n, k), oracle.uniform_limbs(22, qs, n, k)
    a, b = _ct_pair(oracle, qs, n, count, 23)
    primes = [oracle.Prime(q, log_n) for q in qs]

    def ser(x):
        return np.concatenate([primes[l].serialize(x[c, comp, l]) for c in range(x.shape[0])
                               for comp in range(2) for l in range(L)])

    want = np.stack([rns.relin(rns.tensor(a[i], b[i]), kb, ka, log_bs) for i in range(count)])
    ctx = sg.Context(log_n, qs)
    sg.check(lib.shg_context_set_host_pipeline(ctx.h, piece, slots))
    sg.check(lib.shg_context_set_host_ramp(ctx.h, ramp))
    key = sg.Key(ctx, log_bs, 1, kb, ka)
    if wire:
        sa, sb = ser(a), ser(b)
        out = np.zeros_like(sa)
        _run(sg, lib.shg_bgv_mul_relin_host_serialized, ctx.h, key.h, out.ctypes.data,
             sa.ctypes.data, sb.ctypes.data, count, None)
        assert np.array_equal(out, ser(want))
    else:
        a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
        out = np.zeros_like(a)
        _run(sg, lib.shg_bgv_mul_relin_host, ctx.h, key.h, out.ctypes.data, a.ctypes.data,
             b.ctypes.data, count, None)
        assert np.array_equal(out, want)


def test_host_ramp_rejects_out_of_range(sg):
    ctx = sg.Context(12, Q50[:3])
    assert sg.lib().shg_context_set_host_ramp(ctx.h, -1) != 0
    assert sg.lib().shg_context_set_host_ramp(ctx.h, 17) != 0


# --------------------------------------------------------------------------
# On-device sampling (ChaCha PRNG) and EncryptPolynomialBgv
# --------------------------------------------------------------------------

def _seeds(count, salt):
    return np.array([[(i * 31 + c * 17 + salt) % 256 for i in range(32)]
                     for c in range(count)], np.uint8)


def _seed_buf(sg, seeds):
    return sg.DeviceBuffer.from_array(np.frombuffer(seeds.tobytes(), np.uint64))


@pytest.mark.parametrize("log_n,qs,variance,count", [
    (5, [Q45[0]], 1, 3),
    (10, [Q45[0], 65537], 8, 4),        # 65537: about half the candidates rejected
    (12, Q50[:3], 3, 2),
    (13, Q45[:2], 256, 2),
    (14, Q45, 8, 2),
    (15, [Q50[0]], 33, 1),
])
def test_sample_uniform_error(sg, oracle, log_n, qs, variance, count):
    """RnsPolynomial::SampleUniform + SampleError from SingleThreadChaChaPrng,
    one stream per seed, bit-exact with the oracle."""
    lib = sg.lib()
    L, n = len(qs), 1 << log_n
    seeds = _seeds(count, log_n)
    rns = oracle.Rns(log_n, qs)
    want = [rns.sample_uniform_error(L, variance, seeds[c].tobytes()) for c in range(count)]
    ctx = sg.Context(log_n, qs)
    da, de = sg.DeviceBuffer(count * L * n * 8), sg.DeviceBuffer(count * L * n * 8)
    ds = _seed_buf(sg, seeds)
    _run(sg, lib.shg_sample_uniform_error, ctx.h, da.ptr, de.ptr, ds.ptr, L, count, variance,
         None)
    a, e = da.download((count, L, n)), de.download((count, L, n))
    for c in range(count):
        assert np.array_equal(a[c], want[c][0]), c
        assert np.array_equal(e[c], want[c][1]), c


@pytest.mark.parametrize("log_n,qs,count,four_step_min,chunk", [
    (6, Q45[:2], 5, 13, 0),
    (11, [Q59], 3, 13, 0),
    (12, Q50[:3], 4, 12, 0),    # four-step tail at 2^12
    (12, Q50[:3], 4, 13, 0),
    (13, Q45[:4], 3, 13, 0),
    (14, Q45, 45, 13, 16),      # three transform chunks
    (14, Q45, 20, 15, 8),       # CTA-resident transforms, three chunks
    (15, Q50[:2], 2, 13, 0),
    (14, P58[:2], 2, 13, 0),     # lazily reduced error transform just below 2^58
])
def test_bgv_encrypt(sg, oracle, log_n, qs, count, four_step_min, chunk):
    """RnsRlweSecretKey::EncryptPolynomialBgv with on-device sampling,
    bit-exact with the oracle for every ciphertext."""
    lib = sg.lib()
    L, n, t, variance = len(qs), 1 << log_n, 65537, 8
    key = oracle.uniform_limbs(400 + log_n, qs, n).reshape(L, n)
    m = oracle.uniform_limbs(500 + log_n, qs, n, count).reshape(count, L, n)
    seeds = _seeds(count, 3 * log_n)
    rns = oracle.Rns(log_n, qs)
    ctx = sg.Context(log_n, qs, t)
    sg.check(lib.shg_context_set_four_step_min(ctx.h, four_step_min))
    sg.check(lib.shg_context_set_chunk(ctx.h, chunk))
    dk, dm, ds = _dev(sg, key), _dev(sg, m), _seed_buf(sg, seeds)
    out = sg.DeviceBuffer(count * 2 * L * n * 8)
    _run(sg, lib.shg_bgv_encrypt, ctx.h, out.ptr, dk.ptr, dm.ptr, ds.ptr, L, count, variance,
         None)
    got = out.download((count, 2, L, n))
    for c in sorted({0, 1, count // 2, count - 2, count - 1}):
        want = rns.encrypt_bgv(t, variance, key, m[c], seeds[c].tobytes())
        assert np.array_equal(got[c], want), c


def test_bgv_encrypt_decrypts(sg, oracle):
    """c0 + c1 * s = e * t + m: the error part is small and divisible by t
    (the secret-key encryption identity of rns_secret_key_test.cc)."""
    lib = sg.lib()
    log_n, qs, t, variance, count = 12, Q50[:2], 65537, 8, 3
    L, n = len(qs), 1 << log_n
    rns = oracle.Rns(log_n, qs)
    p0 = oracle.Prime(qs[0], log_n)
    key = oracle.uniform_limbs(77, qs, n).reshape(L, n)
    m = oracle.uniform_limbs(78, qs, n, count).reshape(count, L, n)
    ctx = sg.Context(log_n, qs, t)
    seeds = _seeds(count, 1)
    dk, dm, ds = _dev(sg, key), _dev(sg, m), _seed_buf(sg, seeds)
    out = sg.DeviceBuffer(count * 2 * L * n * 8)
    _run(sg, lib.shg_bgv_encrypt, ctx.h, out.ptr, dk.ptr, dm.ptr, ds.ptr, L, count, variance,
         None)
    got = out.download((count, 2, L, n))
    for c in range(count):
        # limb 0: c0 + c1 * s - m = e * t, with |e| <= 2 * variance
        x = p0.add(got[c, 0, 0], p0.mul(got[c, 1, 0], key[0]))
        x = p0.sub(x, m[c, 0])
        v = p0.export(p0.ntt_inv(x)).astype(object)
        q = qs[0]
        s = [int(y) - q if int(y) > q // 2 else int(y) for y in v]
        assert all(y % t == 0 and abs(y // t) <= 2 * variance for y in s)


def test_sampling_validation(sg):
    lib = sg.lib()
    ctx = sg.Context(10, Q45[:2], 65537)
    buf = sg.DeviceBuffer(2 * 2 * 1024 * 8)
    seeds = sg.DeviceBuffer(64)
    for var, msg in [(0, "must be positive"), (257, "must be at most 256")]:
        with pytest.raises(sg.ShgError, match=msg):
            sg.check(lib.shg_sample_uniform_error(ctx.h, buf.ptr, buf.ptr, seeds.ptr, 2, 1, var,
                                                  None))
        with pytest.raises(sg.ShgError, match=msg):
            sg.check(lib.shg_bgv_encrypt(ctx.h, buf.ptr, buf.ptr, buf.ptr, seeds.ptr, 2, 1, var,
                                         None))
    with pytest.raises(sg.ShgError, match="RNS moduli"):
        sg.check(lib.shg_bgv_encrypt(ctx.h, buf.ptr, buf.ptr, buf.ptr, seeds.ptr, 3, 1, 8, None))
    sg.check(lib.shg_bgv_encrypt(ctx.h, buf.ptr, buf.ptr, buf.ptr, seeds.ptr, 2, 0, 8, None))


# --------------------------------------------------------------------------
# RNS basis conversion and BFV (auxiliary primes)
# --------------------------------------------------------------------------

P45 = [35184368320513, 35184368025601, 35184367828993, 35184367337473, 35184366911489,
       35184366551041, 35184366223361]
P50 = [1125899884625921, 1125899884167169, 1125899884036097]
# Primes just below 2^62 and 2^61 (1 mod 2^12): four 62-bit sources overflow
# one 128-bit accumulation, so the conversion reduces twice per value.
Q62 = [4611686018427322369, 4611686018427289601, 4611686018427277313, 4611686018427228161]
P61 = [2305843009213616129, 2305843009213554689, 2305843009213501441]


@pytest.mark.parametrize("log_n,qs,ps,level", [
    (10, Q45, P45, 5),
    (12, Q45, P45, 2),          # a lower level: main prefix q_0..q_2
    (13, Q50[:3], P50[:2], 2),
    (14, Q45, P45, 5),
    (11, Q50[:10], P50, 9),     # ten source limbs
    (11, Q62, P61, 3),          # 62-bit sources
])
def test_switch_rns_basis(sg, oracle, log_n, qs, ps, level):
    """SwitchRnsBasis both ways, ScaleAndSwitchRnsBasis and ApproxSwitchRnsBasis
    (both forms, balanced and not) on 3 polynomials, bit-exact."""
    lib = sg.lib()
    n, K, m = 1 << log_n, len(ps), level + 1
    rns = oracle.Rns(log_n, qs + ps)
    main, aux = list(range(m)), list(range(len(qs), len(qs) + K))
    x = oracle.uniform_limbs(600 + log_n, qs[:m], n, 3).reshape(3, m, n)
    y = oracle.uniform_limbs(700 + log_n, ps, n, 3).reshape(3, K, n)
    ctx = sg.Context(log_n, qs, 65537, ps=ps)
    dx, dy = _dev(sg, x), _dev(sg, y)
    out = sg.DeviceBuffer(3 * max(m, K) * n * 8)
    _run(sg, lib.shg_poly_switch_rns_basis, ctx.h, out.ptr, dx.ptr, 0, m, 3, None)
    assert np.array_equal(out.download((3, K, n)),
                          np.stack([rns.switch_basis(main, aux, x[c]) for c in range(3)]))
    _run(sg, lib.shg_poly_switch_rns_basis, ctx.h, out.ptr, dy.ptr, 1, m, 3, None)
    assert np.array_equal(out.download((3, m, n)),
                          np.stack([rns.switch_basis(aux, main, y[c]) for c in range(3)]))
    _run(sg, lib.shg_poly_scale_switch_rns_basis, ctx.h, out.ptr, dx.ptr, m, 3, None)
    assert np.array_equal(out.download((3, K, n)),
                          np.stack([rns.switch_basis(main, aux, x[c], scale=True)
                                    for c in range(3)]))
    for is_ntt in (0, 1):
        for bal in (0, 1):
            _run(sg, lib.shg_poly_approx_switch_rns_basis, ctx.h, out.ptr, dy.ptr, 1, m, is_ntt,
                 bal, 3, None)
            assert np.array_equal(out.download((3, m, n)),
                                  np.stack([rns.approx_switch_basis(aux, main, y[c], is_ntt, bal)
                                            for c in range(3)]))
            _run(sg, lib.shg_poly_approx_switch_rns_basis, ctx.h, out.ptr, dx.ptr, 0, m, is_ntt,
                 bal, 3, None)
            assert np.array_equal(out.download((3, K, n)),
                                  np.stack([rns.approx_switch_basis(main, aux, x[c], is_ntt, bal)
                                            for c in range(3)]))


def test_switch_rns_basis_rounding_ties(sg, oracle):
    """Coefficients whose sum_i v_i / q_i sits within 2^-32 of a half integer
    take the exact double-precision route; built by hand from the CRT."""
    lib = sg.lib()
    log_n, qs, ps = 10, Q45[:3], P45[:2]
    n = 1 << log_n
    rns = oracle.Rns(log_n, qs + ps)
    p0 = [oracle.Prime(q, log_n) for q in qs]
    # v_0 / q_0 + v_1 / q_1 + v_2 / q_2 ~ 1.5 with v_0 = (q_0 - 1) / 2 etc.
    rng = np.random.default_rng(3)
    x = np.zeros((3, n), dtype=object)
    for k in range(n):
        v = [(qs[0] - 1) // 2 + int(rng.integers(-2, 3)), qs[1] // 2, qs[2] // 2 + int(rng.integers(0, 2))]
        for i in range(3):
            x[i, k] = v[i]
    # x holds the scaled values s_i; undo the (Q/q_i)^-1 factor so the kernel's s_i are them
    xin = np.empty((3, n), np.uint64)
    for i, q in enumerate(qs):
        qhat = 1
        for j, qj in enumerate(qs):
            if j != i:
                qhat = qhat * qj % q
        vals = np.array([int(v) * qhat % q for v in x[i]], np.uint64)
        xin[i] = p0[i].import_(vals)
    want = rns.switch_basis([0, 1, 2], [3, 4], xin)
    ctx = sg.Context(log_n, qs, 65537, ps=ps)
    d, out = _dev(sg, xin), sg.DeviceBuffer(2 * n * 8)
    _run(sg, lib.shg_poly_switch_rns_basis, ctx.h, out.ptr, d.ptr, 0, 3, 1, None)
    assert np.array_equal(out.download((2, n)), want)


@pytest.mark.parametrize("log_n,qs,ps,count,chunk", [
    (11, [8589905921, 8589852673, 8589844481], [1073692673, 1073668097], 3, 0),
    (13, Q45[:4], P45[:5], 2, 0),
    (14, Q45, P45, 5, 2),       # three chunks
    (15, Q50[:2], P50[:2], 1, 0),   # the largest ring
])
def test_bfv_mul_and_absorb(sg, oracle, log_n, qs, ps, count, chunk):
    """RnsBfvCiphertext::operator* and AbsorbInPlace, bit-exact per ciphertext."""
    lib = sg.lib()
    n, L, K, t = 1 << log_n, len(qs), len(ps), 65537
    rns = oracle.Rns(log_n, qs + ps)
    aux = list(range(L, L + K))
    a = oracle.uniform_limbs(800 + log_n, qs, n, 2 * count).reshape(count, 2, L, n)
    b = oracle.uniform_limbs(900 + log_n, qs, n, 2 * count).reshape(count, 2, L, n)
    pt = oracle.uniform_limbs(950 + log_n, qs, n).reshape(L, n)
    ctx = sg.Context(log_n, qs, t, ps=ps)
    sg.check(lib.shg_context_set_chunk(ctx.h, chunk))
    da, db, dp = _dev(sg, a), _dev(sg, b), _dev(sg, pt)
    out = sg.DeviceBuffer(count * 3 * L * n * 8)
    _run(sg, lib.shg_bfv_mul, ctx.h, out.ptr, da.ptr, db.ptr, count, L, None)
    got = out.download((count, 3, L, n))
    for c in sorted({0, count // 2, count - 1}):
        assert np.array_equal(got[c], rns.bfv_mul(L, aux, t, a[c], b[c])), c
    _run(sg, lib.shg_bfv_absorb, ctx.h, out.ptr, da.ptr, dp.ptr, 2, count, L, None)
    got = out.download((count, 2, L, n))
    for c in sorted({0, count - 1}):
        assert np.array_equal(got[c], rns.bfv_absorb(L, aux, t, a[c], pt)), c


def test_bfv_mul_below_top_level(sg, oracle):
    """shg_bfv_mul / shg_bfv_absorb on a three-limb ciphertext of a four-prime
    context (the CRT tables of every level are built), against the oracle's
    general restatement."""
    lib = sg.lib()
    log_n, qs, ps, t, count = 13, Q45[:4], P45[:5], 65537, 2
    n, Lm, K = 1 << log_n, 3, len(ps)
    rns = oracle.Rns(log_n, qs + ps)
    aux = list(range(len(qs), len(qs) + K))
    a = oracle.uniform_limbs(990, qs[:Lm], n, 2 * count).reshape(count, 2, Lm, n)
    b = oracle.uniform_limbs(991, qs[:Lm], n, 2 * count).reshape(count, 2, Lm, n)
    pt = oracle.uniform_limbs(992, qs[:Lm], n).reshape(Lm, n)
    ctx = sg.Context(log_n, qs, t, ps=ps)
    da, db, dp = _dev(sg, a), _dev(sg, b), _dev(sg, pt)
    out = sg.DeviceBuffer(count * 3 * Lm * n * 8)
    _run(sg, lib.shg_bfv_mul, ctx.h, out.ptr, da.ptr, db.ptr, count, Lm, None)
    got = out.download((count, 3, Lm, n))
    for c in range(count):
        assert np.array_equal(got[c], rns.bfv_mul(Lm, aux, t, a[c], b[c])), c
    _run(sg, lib.shg_bfv_absorb, ctx.h, out.ptr, da.ptr, dp.ptr, 2, count, Lm, None)
    got = out.download((count, 2, Lm, n))
    assert np.array_equal(got[1], rns.bfv_absorb(Lm, aux, t, a[1], pt))


def test_bfv_validation(sg):
    lib = sg.lib()
    ctx = sg.Context(10, Q45[:2], 65537)
    buf = sg.DeviceBuffer(4 * 2 * 1024 * 8)
    with pytest.raises(sg.ShgError, match="no auxiliary prime moduli"):
        sg.check(lib.shg_bfv_mul(ctx.h, buf.ptr, buf.ptr, buf.ptr, 1, 2, None))
    with pytest.raises(sg.ShgError, match="distinct"):
        sg.Context(10, Q45[:2], 65537, ps=[Q45[1]])
    ctx = sg.Context(10, Q45[:2], 65537, ps=P45[:1])
    assert lib.shg_context_num_aux_moduli(ctx.h) == 1
    with pytest.raises(sg.ShgError, match="direction"):
        sg.check(lib.shg_poly_switch_rns_basis(ctx.h, buf.ptr, buf.ptr, 2, 2, 1, None))
    with pytest.raises(sg.ShgError, match="RNS moduli"):
        sg.check(lib.shg_bfv_mul(ctx.h, buf.ptr, buf.ptr, buf.ptr, 1, 3, None))
    # empty batches are no-ops, like the reference's loops over zero ciphertexts
    sg.check(lib.shg_bfv_mul(ctx.h, buf.ptr, buf.ptr, buf.ptr, 0, 2, None))
    sg.check(lib.shg_bfv_absorb(ctx.h, buf.ptr, buf.ptr, buf.ptr, 2, 0, 2, None))
    sg.check(lib.shg_poly_switch_rns_basis(ctx.h, buf.ptr, buf.ptr, 0, 2, 0, None))
